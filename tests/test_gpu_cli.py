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
