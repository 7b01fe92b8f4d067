"""The drop-in executables on the GPU against the FP64 oracle: mipt.exe's
rho3.bin records and sim_tmi.exe's p,tmi rows for the same trajectory seeds
(mipt_gb300_trajectory_seed(MIPT_GB300_SEED, p_index * realizations + r)).

Tolerances: FP64 path 1e-10 on rho3 entries and TMI; FP32 path 2e-5 on rho3
entries and 1e-5 on TMI (sums of 7 entropies)."""
import os
import subprocess

import numpy as np
import pytest

from mipt_gb300 import rho3file

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SEED = 20261203


@pytest.fixture(scope="module")
def exes():
    from mipt_gb300 import build
    build.build()
    out = os.path.join(ROOT, "mipt_gb300", "_build")
    return os.path.join(out, "mipt.exe"), os.path.join(out, "sim_tmi.exe")


@pytest.fixture(scope="module")
def orc():
    from oracle import pyoracle
    return pyoracle


def run(args, cwd, fp64, extra=None):
    env = dict(os.environ, MIPT_GB300_SEED=str(SEED), MIPT_GB300_FP64="1" if fp64 else "0", MIPT_GB300_BATCH="3")
    env.update(extra or {})
    r = subprocess.run(args, cwd=cwd, capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


@pytest.mark.parametrize("fp64", [True, False])
def test_mipt_exe_rho3_matches_oracle(exes, orc, tmp_path, fp64):
    mipt, _ = exes
    n, periods, R, res = 10, 3, 4, 2
    run([mipt, "1", str(n), str(periods), str(R), str(res), "0.1", "0.3", "1"], tmp_path, fp64)
    meta, rec = rho3file.read(tmp_path / "rho3.bin")
    assert meta["record_count"] == R * res
    subs = meta["subsystem_qubits"].astype(np.int32)
    ps = np.linspace(0.1, 0.3, res)
    for k in range(R * res):
        pi, r = int(rec["p_index"][k]), int(rec["realization"][k])
        seed = orc.trajectory_seed(SEED, pi * R + r)
        psi = orc.run_trajectory(seed, n, periods, ps[pi], closed=True, want_state=True)["psi"]
        want = orc.rho3(psi, subs).reshape(n, 8, 8, 2)
        want = want[..., 0] + 1j * want[..., 1]
        np.testing.assert_allclose(rec["rho"][k], want, rtol=0, atol=1e-10 if fp64 else 2e-5)


@pytest.mark.parametrize("fp64,order", [(True, 1), (False, 1), (False, 2)])
def test_sim_tmi_exe_matches_oracle(exes, orc, tmp_path, fp64, order):
    _, tmi = exes
    n, periods, R, res = 12, 3, 4, 2
    run([tmi, str(n), str(periods), str(R), str(res), "0.1", "0.3", "1", "1", "out.csv"], tmp_path, fp64,
        {"SIM_TMI_ENTROPY_ORDER": str(order)})
    lines = (tmp_path / "out.csv").read_text().splitlines()
    assert lines[0] == "p,tmi"
    rows = [tuple(float(x) for x in line.split(",")) for line in lines[1:]]
    cycles = n // 4
    assert len(rows) == R * res * cycles
    ps = np.linspace(0.1, 0.3, res)
    tol = 1e-10 if fp64 else 1e-5
    i = 0
    for pi in range(res):
        for r in range(R):
            seed = orc.trajectory_seed(SEED, pi * R + r)
            psi = orc.run_trajectory(seed, n, periods, ps[pi], closed=True, want_state=True)["psi"]
            for c in range(cycles):
                p, got = rows[i]
                i += 1
                assert p == ps[pi]
                assert abs(got - orc.tmi(psi, c, order)) < tol, (pi, r, c, got)


def test_sim_tmi_exe_resumes_to_the_same_file(exes, tmp_path):
    """Interrupt after the first p group (simulated by truncating the finished
    file mid-circuit), re-issue the command: the resumed file is identical."""
    _, tmi = exes
    args = [tmi, "8", "2", "3", "2", "0.1", "0.3", "1", "1"]
    run(args, tmp_path, True)
    path = tmp_path / "csv" / "tmi" / "haarc" / "tmi_haarc_n_8_real_3_0.1_0.3_res_2.csv"
    full = path.read_text()
    lines = full.splitlines(keepends=True)
    path.write_text("".join(lines[:1 + 3 * 2 + 1]))  # first p group + half a circuit
    r = run(args, tmp_path, True)
    assert "RESUMED" in r.stderr
    assert path.read_text() == full


def _entropy_rows(path):
    lines = path.read_text().splitlines()
    head = lines[0].split(",")
    rows = []
    for ln in lines[1:]:
        cells = ln.replace('"Random Haar Unitary"', "haar").split(",")
        rows.append({h: (float(c) if h != "circuit_name" else c) for h, c in zip(head, cells)})
    return head, rows


def test_entropy_exe_matches_oracle(orc, tmp_path):
    """entropy.exe (FP64 path) against the oracle's final states for the same
    trajectory seeds: per L_A the S1 / S2 (natural log) of the N cyclic
    blocks, averaged over translations, then mean / sample stddev / stderr
    over trajectories (cpp/include/mipt/entropy.hpp:580-636)."""
    exe = os.path.join(ROOT, "mipt_gb300", "_build", "entropy.exe")
    n, periods, p, R = 8, 3, 0.3, 5
    run([exe, str(n), str(periods), str(p), str(R), "1", "e.csv"], tmp_path, True, {"MIPT_GB300_BATCH": "2"})
    head, rows = _entropy_rows(tmp_path / "e.csv")
    assert len(rows) == n // 2 - 1
    per = {k: ([], []) for k in range(2, n // 2 + 1)}
    for r in range(R):
        psi = orc.run_trajectory(orc.trajectory_seed(SEED, r), n, periods, p, closed=True, want_state=True)["psi"]
        for kept in per:
            s1 = s2 = 0.0
            for c in range(n):
                rho = orc.rdm(psi, [(c + j) % n for j in range(kept)])
                w = np.linalg.eigvalsh(rho)
                w = w[w > 1e-15]
                s1 += -np.sum(w * np.log(w)) / n
                s2 += -np.log(np.sum(np.abs(rho) ** 2)) / n
            per[kept][0].append(s1)
            per[kept][1].append(s2)
    for row in rows:
        kept = int(row["L_A"])
        assert (row["N"], row["periods"], row["requested_realizations"], row["completed_realizations"]) == (n, periods, R, R)
        assert row["p"] == p and row["circ_type"] == 1 and row["subsystems_per_realization"] == n
        x = n / np.pi * np.sin(np.pi * kept / n)
        assert abs(row["x"] - x) < 1e-14 and abs(row["ln_x"] - np.log(x)) < 1e-14
        for name, vals in (("S1", per[kept][0]), ("S2", per[kept][1])):
            v = np.array(vals)
            assert abs(row[name + "_mean"] - v.mean()) < 1e-9, (kept, name)
            assert abs(row[name + "_stddev"] - v.std(ddof=1)) < 1e-9, (kept, name)
            assert abs(row[name + "_stderr"] - v.std(ddof=1) / np.sqrt(R)) < 1e-9, (kept, name)


def test_entropy_exe_fermion_rppu_matches_oracle(orc, tmp_path):
    """entropy.exe with circ_type 2: the cyclic-block entropies of FermionRPPU
    trajectories from fermionic partial traces, and fermionic_trace = 1."""
    exe = os.path.join(ROOT, "mipt_gb300", "_build", "entropy.exe")
    n, periods, p, R = 8, 2, 0.3, 3
    run([exe, str(n), str(periods), str(p), str(R), "2", "e.csv"], tmp_path, True, {"MIPT_GB300_BATCH": "2"})
    _, rows = _entropy_rows(tmp_path / "e.csv")
    per = {k: ([], []) for k in range(2, n // 2 + 1)}
    for r in range(R):
        psi = orc.run_rppu_trajectory(int(orc.trajectory_seed(SEED, r)), n, periods, p, orc.RPPU_JW)["psi"]
        for kept in per:
            s1 = s2 = 0.0
            for c in range(n):
                rho = orc.rdm(psi, [(c + j) % n for j in range(kept)], True)
                w = np.linalg.eigvalsh(rho)
                w = w[w > 1e-15]
                s1 += -np.sum(w * np.log(w)) / n
                s2 += -np.log(np.sum(np.abs(rho) ** 2)) / n
            per[kept][0].append(s1)
            per[kept][1].append(s2)
    for row in rows:
        kept = int(row["L_A"])
        assert row["circ_type"] == 2 and row["fermionic_trace"] == 1
        for name, vals in (("S1", per[kept][0]), ("S2", per[kept][1])):
            assert abs(row[name + "_mean"] - np.mean(vals)) < 1e-9, (kept, name)


def test_entropy_exe_resumes_its_checkpoint(tmp_path):
    """A 2-trajectory checkpoint re-labelled as part of a 5-trajectory run and
    resumed gives the same file as an uninterrupted 5-trajectory run (up to
    the rounding of restoring the accumulators from mean and stddev); with
    MIPT_ENTROPY_S1_MAX_LA=2 the larger blocks report NaN S1."""
    exe = os.path.join(ROOT, "mipt_gb300", "_build", "entropy.exe")
    base = ["8", "2", "0.2"]
    run([exe] + base + ["2", "1", "part.csv"], tmp_path, True)
    text = (tmp_path / "part.csv").read_text().splitlines()
    relabel = [text[0]] + [ln.replace("8,2,0.20000000000000001,2,", "8,2,0.20000000000000001,5,", 1) for ln in text[1:]]
    (tmp_path / "resumed.csv").write_text("\n".join(relabel) + "\n")
    r = run([exe] + base + ["5", "1", "resumed.csv"], tmp_path, True)
    assert "Resuming from resumed.csv: 2/5" in r.stdout
    run([exe] + base + ["5", "1", "full.csv"], tmp_path, True)
    _, a = _entropy_rows(tmp_path / "resumed.csv")
    _, b = _entropy_rows(tmp_path / "full.csv")
    for ra, rb in zip(a, b):
        for k, v in ra.items():
            if isinstance(v, float):
                assert abs(v - rb[k]) <= 1e-12 * max(1.0, abs(rb[k])), (k, v, rb[k])
    run([exe] + base + ["2", "1", "s1cap.csv"], tmp_path, True, {"MIPT_ENTROPY_S1_MAX_LA": "2"})
    _, c = _entropy_rows(tmp_path / "s1cap.csv")
    assert np.isfinite(c[0]["S1_mean"]) and all(np.isnan(row["S1_mean"]) for row in c[1:])


@pytest.mark.parametrize("circuit", [2, 4])
def test_sim_tmi_exe_rppu_matches_oracle(exes, orc, tmp_path, circuit):
    """sim_tmi.exe on the parity-preserving gate sets: TMI of the cyclic
    quarters from fermionic (circ_type 2) or qubit (4) partial traces of the
    oracle's RPPU trajectories."""
    _, tmi = exes
    n, periods, R, res = 8, 2, 3, 2
    run([tmi, str(n), str(periods), str(R), str(res), "0.1", "0.3", str(circuit), "1", "out.csv"], tmp_path, True)
    rows = [tuple(float(x) for x in line.split(",")) for line in (tmp_path / "out.csv").read_text().splitlines()[1:]]
    cycles, q = n // 4, n // 4
    assert len(rows) == R * res * cycles
    ps = np.linspace(0.1, 0.3, res)
    fermion = circuit == 2
    boundary = orc.RPPU_JW if fermion else orc.RPPU_QUBIT

    def S(psi, modes):
        return orc.entropy(orc.rdm(psi, [m % n for m in modes], fermion), 1)

    i = 0
    for pi in range(res):
        for r in range(R):
            seed = orc.trajectory_seed(SEED, pi * R + r)
            psi = orc.run_rppu_trajectory(int(seed), n, periods, ps[pi], boundary, encoded=True)["psi"]
            for c in range(cycles):
                A, B, C, D = ([c + j * q + k for k in range(q)] for j in range(4))
                want = S(psi, A) + S(psi, B) + S(psi, C) + S(psi, D) - S(psi, A + B) - S(psi, A + C) - S(psi, B + C)
                p, got = rows[i]
                i += 1
                assert abs(got - want) < 1e-10, (pi, r, c, got, want)
