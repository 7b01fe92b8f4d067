"""RPPU / qRPPU trajectories on the GPU batch against the FP64 oracle: the
reference's parity-preserving gate draw with its random extra even layer, the
fermionic closure string (FermionRPPU) or the direct closure bond (qRPPU), the
parity-sector engine's measurement order (site n-1 as its own chunk), and the
fermionic or qubit partial trace of the final observables.

Tolerances: FP64 path 1e-9 on layer surprisals, 1e-10 on S_vN and rho3
entries; FP32 path 2e-5 on surprisals and rho3 entries, 1e-5 on S_vN.
Measurement outcomes bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("circuit", [2, 4])
def test_rppu_batch_matches_oracle(mg, orc, fp64, circuit):
    n, periods, p, count = 10, 3, 0.35, 5
    fermion = circuit == 2
    seeds = [mg.trajectory_seed(2026, i) for i in range(count)]
    b = mg.Batch(n, periods, count, fp64=fp64, observables=mg.OBS_SVN_HALF, rho3=True, fermion_trace=fermion,
                 circuit=circuit)
    got = b.run(seeds, p)
    assert got["surprisal"].shape == (count, 2 * periods + 1)
    boundary = orc.RPPU_JW if fermion else orc.RPPU_QUBIT
    subs = [[s, (s + 1) % n, (s + 2) % n] for s in range(n)]
    tol_s, tol_e, tol_r = (1e-9, 1e-10, 1e-10) if fp64 else (2e-5, 1e-5, 2e-5)
    extra_seen = set()
    for i, sd in enumerate(seeds):
        want = orc.run_rppu_trajectory(int(sd), n, periods, p, boundary, encoded=True)
        draw = orc.rppu_draw(int(sd), n, periods, p, boundary)
        T = want["layers"]
        extra_seen.add(T)
        for t in range(T):
            sites = draw["sites"][t, : draw["sites_per_layer"][t]]
            mask = sum(int(o) << int(s) for s, o in zip(sites, want["outcomes"][t][: len(sites)]))
            assert int(got["outcomes"][i, t]) == mask, (i, t)
            assert int(got["measured"][i, t]) == sum(1 << int(s) for s in sites)
        np.testing.assert_allclose(got["surprisal"][i, :T], want["surprisal"], rtol=0, atol=tol_s)
        assert np.all(got["surprisal"][i, T:] == 0) and np.all(got["measured"][i, T:] == 0)
        psi = want["psi"]
        s_half = orc.entropy(orc.rdm(psi, list(range(n // 2)), fermion), 1)
        assert abs(got["obs"][i, 0, 0] - s_half) < tol_e
        r3 = orc.rho3(psi, np.array(subs, np.int32), fermion).reshape(-1)
        np.testing.assert_allclose(got["rho3"][i].reshape(-1), r3, rtol=0, atol=tol_r)
    assert extra_seen == {2 * periods, 2 * periods + 1}  # both extra-layer cases covered


def test_rppu_without_encoded_chunking(mg, orc):
    """split_last = 0 (the reference's MIPT_CUSV_PARITY=0 path): site n-1 joins
    the ordinary ascending chunks."""
    n, periods, p = 8, 2, 0.6
    seeds = [mg.trajectory_seed(7, i) for i in range(3)]
    b = mg.Batch(n, periods, 3, fp64=True, circuit=4, split_last=False)
    got = b.run(seeds, p)
    for i, sd in enumerate(seeds):
        want = orc.run_rppu_trajectory(int(sd), n, periods, p, orc.RPPU_QUBIT, encoded=False)
        np.testing.assert_allclose(got["surprisal"][i, : want["layers"]], want["surprisal"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("circuit,init_kind", [(2, 1), (4, 0)])
def test_rppu_free_energy_trajectories_match_oracle(mg, orc, circuit, init_kind):
    """The free-energy protocol on the parity-preserving gate sets: fixed-parity
    random initial states, workspace-seeded RPPU layers, plain chunking, S1
    with the gate set's partial trace."""
    n, p, count = 8, 0.3, 3
    T = 28 * n
    steps = list(range(0, 2 * n + 1, 4))
    b = mg.Batch(n, T // 2, count, fp64=True, observables=mg.OBS_SVN_HALF, fermion_trace=circuit == 2,
                 circuit=circuit, split_last=False)
    b.set_observation_steps(steps)
    ts = [orc.fe_trajectory_seed(99, i) for i in range(count)]
    sectors = b.set_initial_states([orc.fe_initial_seed(t) for t in ts], init_kind, fixed_parity=True)
    b.prepare_workspace([orc.fe_workspace_seed(t) for t in ts], p)
    b.execute()
    got = b.fetch()
    for i in range(count):
        want = orc.fe_trajectory(ts[i], n, p, init_kind, entropy_max_t=2 * n, entropy_stride=4, circuit=circuit)
        assert sectors[i] == want["parity"] and sectors[i] in (0, 1)
        counts = np.array([bin(int(m)).count("1") for m in got["measured"][i][:T]])
        np.testing.assert_array_equal(counts, want["measured"])
        np.testing.assert_allclose(got["surprisal"][i, :T], want["surprisal"], rtol=0, atol=1e-9)
        assert got["surprisal"][i, T] == 0
        np.testing.assert_allclose(got["obs"][i, :, 0], want["s_half"][steps], rtol=0, atol=1e-10)


@pytest.mark.parametrize("circuit", [2, 4])
def test_mipt_exe_rppu_rho3_matches_oracle(mg, orc, tmp_path, circuit):
    """mipt.exe with circ_type 2 / 4: rho3.bin records against the oracle's
    trajectories (fermionic partial trace for 2)."""
    import os
    import subprocess
    from mipt_gb300 import rho3file
    exe = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "mipt_gb300", "_build",
                       "mipt.exe")
    n, periods, R, res, seed = 8, 2, 3, 2, 515
    env = dict(os.environ, MIPT_GB300_SEED=str(seed), MIPT_GB300_FP64="1", MIPT_GB300_BATCH="4")
    r = subprocess.run([exe, "1", str(n), str(periods), str(R), str(res), "0.2", "0.4", str(circuit)], cwd=tmp_path,
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    meta, rec = rho3file.read(tmp_path / "rho3.bin")
    subs = meta["subsystem_qubits"].astype(np.int32)
    ps = np.linspace(0.2, 0.4, res)
    boundary = orc.RPPU_JW if circuit == 2 else orc.RPPU_QUBIT
    for k in range(R * res):
        pi, rr = int(rec["p_index"][k]), int(rec["realization"][k])
        sd = orc.trajectory_seed(seed, pi * R + rr)
        psi = orc.run_rppu_trajectory(int(sd), n, periods, ps[pi], boundary, encoded=True)["psi"]
        want = orc.rho3(psi, subs, circuit == 2).reshape(n, 8, 8, 2)
        np.testing.assert_allclose(rec["rho"][k], want[..., 0] + 1j * want[..., 1], rtol=0, atol=1e-10)


def test_fermion_closure_fold_matches_string_passes(mg, orc):
    """FermionRPPU's closure string folded into the closure gate (parity sector
    known from the initial-state draw) against the same trajectories run with
    the string as two diagonal passes (the same amplitudes uploaded raw, sector
    unknown); and the caller-ordering check."""
    n, periods, p, count = 10, 3, 0.3, 4
    ts = [orc.fe_trajectory_seed(5, i) for i in range(count)]
    init = [orc.fe_initial_seed(t) for t in ts]
    ws = [orc.fe_workspace_seed(t) for t in ts]
    runs = []
    for raw in (False, True):
        b = mg.Batch(n, periods, count, fp64=True, observables=mg.OBS_SVN_HALF, fermion_trace=True, circuit=2,
                     split_last=False)
        if raw:
            for i, sd in enumerate(init):
                psi, _ = mg.draw_initial_state(sd, n, 1, fixed_parity=True, fp64=True)
                b.set_initial_state(i, psi)
        else:
            sectors = b.set_initial_states(init, 1, fixed_parity=True)
            assert set(sectors) <= {0, 1}
        b.prepare_workspace(ws, p)
        b.execute()
        runs.append(b.fetch())
    np.testing.assert_array_equal(runs[0]["outcomes"], runs[1]["outcomes"])
    np.testing.assert_allclose(runs[0]["surprisal"], runs[1]["surprisal"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(runs[0]["obs"], runs[1]["obs"], rtol=0, atol=1e-12)
    # Initial states set after the closure gates were folded for |0...0>.
    b = mg.Batch(n, periods, count, fp64=True, circuit=2)
    b.prepare_workspace(ws, p)
    sectors = b.set_initial_states(init, 1, fixed_parity=True)
    if any(s == 1 for s in sectors):
        with pytest.raises(mg.MiptError):
            b.execute()
