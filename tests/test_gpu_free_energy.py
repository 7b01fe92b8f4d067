"""The free-energy path on the GPU against the FP64 oracle: the batch with
workspace-seeded draws, random initial states and an observation schedule,
then free_energy.exe end to end and across a resume.

Tolerances: FP64 path 1e-9 on layer surprisals (natural log), 1e-10 on the
half-chain S1 (bits); FP32 path 2e-5 and 1e-5. Measured-site counts exact."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SEED = 4242


@pytest.fixture(scope="module")
def mg():
    import mipt_gb300
    from mipt_gb300 import build
    build.build()
    return mipt_gb300


@pytest.fixture(scope="module")
def orc():
    from oracle import pyoracle
    return pyoracle


def schedule(n, T, max_t, stride):
    return [t for t in range(T + 1) if t == 0 or (t <= max_t and (t % stride == 0 or t == max_t))]


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("init_kind", [0, 1])
def test_batch_free_energy_trajectories_match_oracle(mg, orc, fp64, init_kind):
    n, p, count = 8, 0.3, 3
    T = 28 * n
    steps = schedule(n, T, 2 * n, 3)
    b = mg.Batch(n, T // 2, count, closed=True, fp64=fp64, observables=mg.OBS_SVN_HALF)
    b.set_observation_steps(steps)
    ts = [orc.fe_trajectory_seed(SEED, i) for i in range(count)]
    sectors = b.set_initial_states([orc.fe_initial_seed(t) for t in ts], init_kind)
    b.prepare_workspace([orc.fe_workspace_seed(t) for t in ts], p)
    b.execute()
    got = b.fetch()
    assert list(sectors) == [-1] * count
    tol_s, tol_e = (1e-9, 1e-10) if fp64 else (2e-5, 1e-5)
    for i in range(count):
        want = orc.fe_trajectory(ts[i], n, p, init_kind, fp32_init=not fp64, entropy_max_t=2 * n, entropy_stride=3)
        counts = np.array([bin(int(m)).count("1") for m in got["measured"][i]])
        np.testing.assert_array_equal(counts, want["measured"])
        np.testing.assert_allclose(got["surprisal"][i], want["surprisal"], rtol=0, atol=tol_s)
        np.testing.assert_allclose(got["obs"][i, :, 0], want["s_half"][steps], rtol=0, atol=tol_e)
        assert np.all(np.isnan(np.delete(want["s_half"], steps)))


def test_initial_state_upload_and_schedule_edges(mg, orc):
    """A host-given initial state, an observation at t = 0 only, and the
    default |0...0> for a trajectory without one, in one execute."""
    n = 6
    b = mg.Batch(n, 2, 2, closed=True, fp64=True, observables=mg.OBS_SVN_HALF)
    b.set_observation_steps([0, 4])
    psi, _ = orc.fe_initial_state(99, n, 1)
    b.set_initial_state(0, psi)
    b.prepare_workspace([5, 6], 0.0)
    b.execute()
    got = b.fetch()
    want0 = orc.entropy(orc.rdm(psi, list(range(n // 2))), 1)
    assert abs(got["obs"][0, 0, 0] - want0) < 1e-10
    assert abs(got["obs"][1, 0, 0]) < 1e-12  # |0...0>
    # No measurements at p = 0: zero surprisal throughout.
    assert np.all(got["surprisal"] == 0)
    # The uploaded state was consumed: the next execute starts from |0...0>.
    b.prepare_workspace([5, 6], 0.0)
    b.execute()
    assert abs(b.fetch()["obs"][0, 0, 0]) < 1e-12
    with pytest.raises(mg.MiptError):
        b.set_observation_steps([3, 2])
    with pytest.raises(mg.MiptError):
        b.set_observation_steps([0, 5])


@pytest.fixture(scope="module")
def fe_exe():
    from mipt_gb300 import build
    build.build()
    return os.path.join(ROOT, "mipt_gb300", "_build", "free_energy.exe")


def run_fe(exe, args, cwd, extra=None):
    env = dict(os.environ, MIPT_FREE_ENERGY_SEED=str(SEED), MIPT_GB300_FP64="1", MIPT_GB300_BATCH="2",
               MIPT_FREE_ENERGY_ENTROPY_STRIDE="2")
    env.update(extra or {})
    r = subprocess.run([exe] + args, cwd=cwd, capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def read_csv(path):
    import csv
    with open(path) as f:
        return list(csv.DictReader(f))


def test_free_energy_exe_matches_oracle(fe_exe, orc, tmp_path):
    n, p, R, init = 6, 0.25, 5, 1
    run_fe(fe_exe, [str(n), str(p), str(R), "1", str(init)], tmp_path)
    stem = tmp_path / f"free_energy_haar_n_{n}_p_0.25_init_{init}_reals_{R}"
    rows = read_csv(f"{stem}_samples.csv")
    series = read_csv(f"{stem}_timeseries.csv")
    T, eq = 28 * n, 4 * n
    assert len(rows) == R and len(series) == T + 1
    F = np.zeros((R, T + 1))
    S = np.full((R, T + 1), np.nan)
    for t, row in enumerate(rows):
        ts = orc.fe_trajectory_seed(SEED, t)
        want = orc.fe_trajectory(ts, n, p, init, entropy_max_t=2 * n, entropy_stride=2)
        assert int(row["trajectory"]) == t and int(row["trajectory_seed"]) == ts and row["parity_sector"] == "-1"
        assert row["circuit_name"] == "Random Haar Unitary"
        assert int(row["measurements_total"]) == want["measured"].sum()
        assert int(row["measurements_production"]) == want["measured"][eq:].sum()
        F[t, 1:] = np.cumsum(want["surprisal"])
        S[t] = want["s_half"]
        prod = np.cumsum(want["surprisal"][eq:])
        slope = np.polyfit(np.arange(1, T - eq + 1), prod, 1)[0]
        for key, value in [("F_total", F[t, -1]), ("F_production", prod[-1]),
                           ("production_rate_endpoint", prod[-1] / (T - eq)), ("production_slope", slope),
                           ("free_energy_density_tilde", slope / n)]:
            assert abs(float(row[key]) - value) < 1e-9, (key, row[key], value)
    for t, row in enumerate(series):
        assert int(row["t"]) == t and int(row["completed_realizations"]) == R
        assert row["phase"] == ("initial" if t == 0 else ("equilibration" if t <= eq else "production"))
        assert abs(float(row["F_mean"]) - F[:, t].mean()) < 1e-9
        if t > 0:
            assert abs(float(row["F_stddev"]) - F[:, t].std(ddof=1)) < 1e-9
            assert abs(float(row["F_over_tL_mean"]) - (F[:, t] / (t * n)).mean()) < 1e-9
        sampled = not np.isnan(S[0, t])
        assert int(row["S_half_count"]) == (R if sampled else 0)
        if sampled:
            assert abs(float(row["S_half_mean"]) - S[:, t].mean()) < 1e-10
        else:
            assert row["S_half_mean"] == "nan"


def test_free_energy_exe_resume_continues_the_run(fe_exe, tmp_path):
    """A run stopped after 3 of 5 trajectories, with a half-written samples
    row, resumes to the same rows and aggregates as an uninterrupted run."""
    n, p, init = 6, 0.2, 0
    full, part = tmp_path / "full", tmp_path / "part"
    full.mkdir()
    part.mkdir()
    run_fe(fe_exe, [str(n), str(p), "5", "1", str(init)], full)
    run_fe(fe_exe, [str(n), str(p), "3", "1", str(init)], part)
    stem3, stem5 = f"free_energy_haar_n_{n}_p_0.2_init_{init}_reals_3", f"free_energy_haar_n_{n}_p_0.2_init_{init}_reals_5"
    samples = (part / f"{stem3}_samples.csv").read_text()
    (part / f"{stem5}_samples.csv").write_text(samples + f"{n},0.20000000000000001,1,\"Random")
    lines = (part / f"{stem3}_timeseries.csv").read_text().splitlines()
    fixed = [lines[0]]
    for line in lines[1:]:
        cells = line.split(",")
        cells[5] = "5"  # requested_realizations (the circuit name holds no comma)
        fixed.append(",".join(cells))
    (part / f"{stem5}_timeseries.csv").write_text("\n".join(fixed) + "\n")
    r = run_fe(fe_exe, [str(n), str(p), "5", "1", str(init)], part, {"MIPT_FREE_ENERGY_SEED": "1"})
    assert "Resuming from" in r.stdout and "3/5 trajectories already recorded, seed stream recovered" in r.stdout
    assert "Dropping" in r.stdout and "Ignoring MIPT_FREE_ENERGY_SEED=1" in r.stdout
    a, b = read_csv(full / f"{stem5}_samples.csv"), read_csv(part / f"{stem5}_samples.csv")
    assert len(a) == len(b) == 5
    for x, y in zip(a, b):
        assert x["trajectory_seed"] == y["trajectory_seed"] and x["measurements_total"] == y["measurements_total"]
        for key in ("F_total", "F_production", "production_slope"):
            assert abs(float(x[key]) - float(y[key])) < 1e-12
    sa, sb = read_csv(full / f"{stem5}_timeseries.csv"), read_csv(part / f"{stem5}_timeseries.csv")
    for x, y in zip(sa, sb):
        assert x["completed_realizations"] == y["completed_realizations"] == "5"
        assert x["S_half_count"] == y["S_half_count"]
        for key in ("F_mean", "F_stddev", "S_half_mean", "S_half_stddev"):
            if x[key] == "nan":
                assert y[key] == "nan"
            else:
                assert abs(float(x[key]) - float(y[key])) <= 1e-12 * max(1.0, abs(float(x[key])))
