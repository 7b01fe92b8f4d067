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
