"""Batched GPU GMN solver (mipt_gb300_gmn_solve) against the reference's
known answers and the FP64 oracle (oracle/gmn.py).

Tolerances: certified duality gap 1e-6 (FP32 and FP64 iterations); GMN within
2e-6 of the oracle; known answers within the reference tests' tolerances."""
import numpy as np
import pytest

from oracle import gmn as ogmn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg():
    from mipt_gb300 import build
    build.build()
    import mipt_gb300
    return mipt_gb300


def random_states(count, seed):
    """Pure random 3-qubit states mixed with white noise, GHZ/W mixtures."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        kind = i % 3
        if kind == 0:
            v = rng.normal(size=8) + 1j * rng.normal(size=8)
            v /= np.linalg.norm(v)
            base = np.outer(v, v.conj())
        elif kind == 1:
            a = rng.uniform()
            base = a * ogmn.ghz() + (1 - a) * ogmn.w_state()
        else:
            base = ogmn.product()
        w = rng.uniform()
        out.append((1 - w) * base + w * np.eye(8) / 8)
    return np.array(out)


KNOWN = [(ogmn.ghz(), 0.5, 1e-4), (ogmn.w_state(), 0.4428, 1e-3), (ogmn.bell_ab(), 0.0, 1e-4),
         (ogmn.product(), 0.0, 1e-4), (ogmn.ghz_white_noise(0.40), 0.0, 1e-4),
         (ogmn.ghz_white_noise(0.50), 0.0625, 1e-3)]


@pytest.mark.parametrize("fp64", [False, True])
def test_known_answers(mg, fp64):
    rho = np.array([k[0] for k in KNOWN])
    r = mg.gmn_solve(rho, fp64=fp64)
    assert np.all(r["iters"] > 0), r["iters"]
    for (_, want, tol), got in zip(KNOWN, r["gmn"]):
        assert abs(got - want) <= tol, (want, got)
    assert abs(r["gmn"][1] - 0.4714) > 0.01


@pytest.mark.parametrize("fp64", [False, True])
def test_iterates_match_the_oracle(mg, fp64):
    """The GPU runs the oracle's ADMM iteration: after the same number of
    iterations W, Q_1..3, Z_1..3 agree (FP64 1e-9, FP32 1e-4 on entries)."""
    rho = random_states(12, 3)
    k = 200
    r = mg.gmn_solve(rho, fp64=fp64, max_iter=k, check_every=k, gap_tol=1e-15, feas_tol=1e-15, want_solution=True)
    for i in range(len(rho)):
        o = ogmn.solve(rho[i], max_iter=k, check_every=k, gap_tol=1e-15)
        want = np.array([o["W"]] + o["Q"] + o["Z"])
        if abs(o["gap"]) <= 1e-15 and o["infeas"] <= 1e-15:
            continue  # the oracle stopped before k on an exact solution
        np.testing.assert_allclose(r["solution"][i], want, rtol=0, atol=1e-9 if fp64 else 1e-4)


@pytest.mark.parametrize("fp64", [False, True])
def test_certified_bounds_bracket_the_oracle(mg, fp64):
    """Every state gets certified bounds [gmn - gap/2, gmn + gap/2] (dual and
    primal values); they contain the oracle's long-run value. GHZ/W/product
    mixtures certify to 1e-6; generic entangled states converge sublinearly
    (ADMM on a degenerate SDP) and report the gap they reached."""
    rho = random_states(48, 7)
    r = mg.gmn_solve(rho, fp64=fp64, gap_tol=1e-6, max_iter=3000)
    kinds = np.arange(len(rho)) % 3
    assert np.all(r["iters"][kinds > 0] > 0)
    assert np.all(np.abs(r["gap"][kinds > 0]) <= 1e-6)
    for i in range(0, len(rho), 4):
        o = ogmn.solve(rho[i], gap_tol=1e-7, max_iter=20000)
        lo, hi = r["gmn"][i] - abs(r["gap"][i]) / 2, r["gmn"][i] + abs(r["gap"][i]) / 2
        slack = 2e-6 + abs(o["gap"])
        assert lo - slack <= o["gmn"] <= hi + slack, (i, lo, hi, o["gmn"], o["gap"])


def test_warm_start_from_the_solution(mg):
    rho = random_states(36, 11)
    rho = rho[np.arange(len(rho)) % 3 > 0]  # mixtures that certify
    cold = mg.gmn_solve(rho, fp64=True, gap_tol=1e-8, feas_tol=1e-8, want_solution=True)
    assert np.all(cold["iters"] > 0)
    warm = mg.gmn_solve(rho, warm_start=cold["solution"], gap_tol=1e-6)
    assert np.all(warm["iters"] > 0)
    assert np.all(warm["iters"] <= np.maximum(10, cold["iters"] // 2))
    np.testing.assert_allclose(warm["gmn"], cold["gmn"], rtol=0, atol=2e-6)


def test_cut_negativities_match_oracle(mg):
    """Single-qubit-cut negativities (gmn.exe's prefilter) against the FP64
    oracle, and the textbook values for GHZ, W, |000> and Bell(12) x |0>."""
    states = np.concatenate([random_states(60, 11), [ogmn.ghz(), ogmn.w_state(), ogmn.product(), ogmn.bell_ab()]])
    got = mg.cut_negativities(states)
    want = np.array([ogmn.cut_negativities(r) for r in states])
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-10)
    np.testing.assert_allclose(got[-4:], [[0.5] * 3, [np.sqrt(2) / 3] * 3, [0.0] * 3, [0.0, 0.5, 0.5]], atol=1e-12)


def _sanitized(rho):
    """The Hermitisation gmn.exe applies (cpp/apps/gmn.cpp:127-212)."""
    r = np.array(rho, complex)
    for i in range(8):
        r[i, i] = complex(r[i, i].real if np.isfinite(r[i, i].real) else 0.0, 0.0)
    for i in range(8):
        for j in range(i + 1, 8):
            a, b = r[i, j], r[j, i]
            fa, fb = np.isfinite(a), np.isfinite(b)
            v = 0.5 * (a + np.conj(b)) if fa and fb else (a if fa else (np.conj(b) if fb else 0.0))
            r[i, j], r[j, i] = v, np.conj(v)
    return r


@pytest.mark.parametrize("mode", [1, 0])
def test_gmn_exe_rows_match_oracle(mg, tmp_path, mode):
    """gmn.exe end to end: rho3.bin in, "p,gmn,bipneg" rows out, in record
    and subsystem order, against the oracle (GMN to its certified gap,
    bipartite negativity to 1e-10), the prefilter (rows with a separable cut
    are exactly 0), the sanitisation of non-finite entries, the per-p limit
    and the metadata sidecar."""
    import os
    import subprocess
    from mipt_gb300 import rho3file
    exe = os.path.join(os.path.dirname(mg.__file__), "_build", "gmn.exe")
    ph = np.zeros(8, complex)
    ph[0], ph[7] = 1 / np.sqrt(2), np.exp(1j) / np.sqrt(2)
    bad = ogmn.ghz().astype(complex)
    bad[1, 2] = np.nan
    bad[0, 7] = 0.5 + 0.1j
    recs = [[ogmn.ghz_white_noise(0.3), ogmn.product()], [ogmn.w_state(), ogmn.bell_ab()],
            [ogmn.ghz_white_noise(0.6), ogmn.pure(ph)], [ogmn.ghz_white_noise(0.9), bad],
            [ogmn.ghz(), ogmn.product()], [ogmn.w_state(), ogmn.ghz_white_noise(0.5)]]
    p = [0.1, 0.1, 0.2, 0.2, 0.3, 0.3]
    rho3file.write(tmp_path / "rho3.bin", np.array(recs), p=p, p_index=[0, 0, 1, 1, 2, 2],
                   realization=[0, 1, 0, 1, 0, 1], total_qubits=12, periods=4, realizations=2)
    env = dict(os.environ, MIPT_GB300_GMN_GAP="1e-8")
    r = subprocess.run([exe, str(mode), "rho3.bin", "out.csv"], cwd=tmp_path, capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = (tmp_path / "out.csv").read_text().splitlines()
    assert lines[0] == "p,gmn,bipneg" and len(lines) == 13
    rows = np.array([[float(x) for x in ln.split(",")] for ln in lines[1:]])
    mats = [_sanitized(m) for rec in recs for m in rec]
    if mode == 0:
        mats = [m.real.astype(complex) for m in mats]
    np.testing.assert_array_equal(rows[:, 0], np.repeat(p, 2))
    for k, m in enumerate(mats):
        neg = ogmn.cut_negativities(m).min()
        assert abs(rows[k, 2] - neg) < 1e-10, (k, rows[k], neg)
        if neg <= 1e-10:
            assert rows[k, 1] == 0.0, (k, rows[k])
        else:
            want = ogmn.solve(m, gap_tol=1e-10)["gmn"]
            assert abs(rows[k, 1] - want) < 2e-6, (k, rows[k], want)
    # GHZ + white noise closed form (7p - 3) / 8 and the complex phase.
    assert abs(rows[4, 1] - 0.15) < 2e-6 and abs(rows[6, 1] - 0.4125) < 2e-6
    assert abs(rows[5, 1] - (0.5 if mode == 1 else 0.5 * np.cos(1.0))) < 2e-6
    assert ("Warning: replaced 1 non-finite" in r.stderr)
    assert (mode == 0) == ("real-only mode evaluates Re(rho)" in r.stderr)
    meta = (tmp_path / "out_meta.csv").read_text().splitlines()
    assert meta[0].startswith("N,spatial_dimension,grid_x,grid_y,periods,realizations,resolution,p_min,p_max")
    assert meta[1].startswith("12,1,12,1,4,2,3,0.10000000000000001,0.29999999999999999,3,2,6,")
    assert meta[1].endswith(f'"gmn.exe {"complex" if mode == 1 else "real-only"}","rho3.bin"')
    # limit_per_p = 1: the first record of every p.
    r = subprocess.run([exe, str(mode), "rho3.bin", "lim.csv", "1"], cwd=tmp_path, capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lim = (tmp_path / "lim.csv").read_text().splitlines()[1:]
    assert lim == [lines[1 + k] for k in (0, 1, 4, 5, 8, 9)]
    assert "records skipped by limit_per_p: 3" in r.stdout
