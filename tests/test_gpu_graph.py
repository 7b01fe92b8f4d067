"""CUDA-graph execution of batches, and mixed chain lengths as one graph.

* Batch.execute_graph: the first call runs normally and captures a graph,
  later calls replay it. Replays with new seeds (the same structure) must
  give bit-identical results to a normal execute of the same trajectories,
  including per-layer observables, extra regions and rho3 blocks (whose job
  tables the graph copies from pinned staging on every replay).
* A structure change (fewer trajectories) re-captures and stays correct.
* BatchGroup: batches of L = 16, 18, 20, 22 (the mixed-length workload's
  chain lengths) as the branches of one graph, against the CPU FP64 oracle:
  outcomes bit-exact, final states and final half-chain S_2 to the FP32
  path's bounds; and per-layer S_2 of short chains (L = 8, 10, 12) against
  the oracle at every layer.
"""
import numpy as np
import pytest

from tests.gpu_util import mask_of

pytestmark = pytest.mark.gpu

P_GRID = np.linspace(0.05, 0.35, 16)


@pytest.fixture(scope="module")
def mg():
    from mipt_gb300 import build
    build.build()
    import mipt_gb300
    return mipt_gb300


@pytest.fixture(scope="module")
def orc():
    from oracle import pyoracle
    return pyoracle


def oracle_masks(orc, seed, n, periods, p, outcomes):
    d = orc.haar_draw(int(seed), n, periods, p, True, 16)
    oc = np.zeros(2 * periods, np.uint64)
    for t in range(2 * periods):
        s = d["sites"][t, : d["sites_per_layer"][t]]
        oc[t] = mask_of(s, outcomes[t, : len(s)])
    return oc


def make_batch(mg, n, periods, count):
    b = mg.Batch(n, periods, capacity=count, fp64=False, observables=mg.OBS_S2_HALF | mg.OBS_TMI_S2,
                 observe_every=1, rho3=True)
    b.add_region([0, 3, 5, 9], 1)
    b.add_region(list(range(4, 12)), 2)
    return b


def fetch_all(b):
    r = b.fetch()
    r["regions"] = b.fetch_regions()
    r["tmi"] = b.fetch_tmi(2)
    return r


def test_graph_replay_matches_normal_execute(mg):
    n, periods, count = 16, 3, 8
    ps = P_GRID[np.arange(count) % 16]
    g = make_batch(mg, n, periods, count)
    ref = make_batch(mg, n, periods, count)
    for step in range(4):
        seeds = [mg.trajectory_seed(500 + step, i) for i in range(count)]
        g.prepare(seeds, ps)
        g.execute_graph()
        got = fetch_all(g)
        ref.prepare(seeds, ps)
        ref.execute()
        want = fetch_all(ref)
        for key in ("measured", "outcomes", "surprisal", "obs", "rho3", "regions", "tmi"):
            np.testing.assert_array_equal(got[key], want[key], err_msg=f"step {step}: {key}")
    # A structure change (fewer trajectories) captures a new graph.
    seeds = [mg.trajectory_seed(600, i) for i in range(count // 2)]
    for _ in range(2):
        g.prepare(seeds, ps[: count // 2])
        g.execute_graph()
        got = fetch_all(g)
        ref.prepare(seeds, ps[: count // 2])
        ref.execute()
        want = fetch_all(ref)
        for key in ("outcomes", "obs", "regions"):
            np.testing.assert_array_equal(got[key], want[key])


def test_mixed_lengths_one_graph_against_oracle(mg, orc):
    lengths, per = [16, 18, 20, 22], 2
    batches, seeds, ps = [], {}, {}
    for L in lengths:
        batches.append(mg.Batch(L, L, capacity=per, fp64=False, observables=mg.OBS_S2_HALF))
        seeds[L] = [mg.trajectory_seed(2, 1000 * L + i) for i in range(per)]
        ps[L] = P_GRID[[L % 16, (L + 7) % 16]]
    group = mg.BatchGroup(batches)
    for rep in range(2):  # capture, then replay
        for L, b in zip(lengths, batches):
            b.prepare(seeds[L], ps[L])
        group.execute()
        for L, b in zip(lengths, batches):
            got = b.fetch()
            e = mg.Engine(fp64=False)
            for i in range(per):
                r = orc.run_trajectory(int(seeds[L][i]), L, L, float(ps[L][i]), True, 16, want_state=True)
                np.testing.assert_array_equal(got["outcomes"][i],
                                              oracle_masks(orc, seeds[L][i], L, L, float(ps[L][i]), r["outcomes"]))
                e.adopt(b.state_ptr(i), L)
                assert np.linalg.norm(e.state() - r["psi"]) < 1e-4
                m = r["psi"].reshape(-1, 1 << (L // 2))
                s2 = -np.log2(np.sum(np.abs(m.conj().T @ m) ** 2))
                assert abs(got["obs"][i, 0, 1] - s2) < 1e-5, (L, i, got["obs"][i, 0, 1], s2)
    group.close()


def test_mixed_lengths_per_layer_against_oracle(mg, orc):
    lengths, per, periods = [8, 10, 12], 3, 3
    batches, seeds = [], {}
    for L in lengths:
        batches.append(mg.Batch(L, periods, capacity=per, fp64=False, observables=mg.OBS_S2_HALF, observe_every=1))
        seeds[L] = [mg.trajectory_seed(8, 100 * L + i) for i in range(per)]
    group = mg.BatchGroup(batches)
    p = 0.25
    for rep in range(2):
        for L, b in zip(lengths, batches):
            b.prepare(seeds[L], p)
        group.execute()
        for L, b in zip(lengths, batches):
            got = b.fetch()
            for i in range(per):
                r = orc.run_trajectory(int(seeds[L][i]), L, periods, p, True, 16, orc.OBS_S2, 1)
                np.testing.assert_array_equal(got["outcomes"][i],
                                              oracle_masks(orc, seeds[L][i], L, periods, p, r["outcomes"]))
                np.testing.assert_allclose(got["obs"][i][:, 1], r["obs"][:, 1], rtol=0, atol=1e-5)
    group.close()
