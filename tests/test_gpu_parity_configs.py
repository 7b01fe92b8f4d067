"""GPU parity of the benchmarked workloads against the CPU FP64 oracle.

* The L=24 headline workload at full depth: periodic Haar brickwork, 48
  layers, FP32 states, p from the bench's grid. The GPU batch runs free
  (no outcome replay): measurement locations and outcomes must equal the
  oracle's bit for bit, the final state must match the oracle's FP64 state,
  and the final half-chain S_2 must match the oracle state's within 1e-5.
* Config 0 in full: all 200 trajectories of the L=12 open chain, p=0.2,
  24 layers, master seed 0, FP64, with half-chain S_vN, S_2 and both TMIs
  after every layer, against the oracle at 1e-10 and outcomes bit-exact.
* Config 3's lattice (4 x 7, L=28, FP32, p=0.15) for two layers: final
  amplitudes, the half-system S_2 and three rho3 blocks against the oracle.

Tolerances: FP64 1e-10 on entropies/TMI, 1e-12 per amplitude (x10 after a
whole trajectory); FP32 1e-5 on entropies, 2e-5 on rho3 entries, and the
L2 distance of final states below 2e-4 (48 layers of FP32 rounding).
"""
from concurrent.futures import ThreadPoolExecutor

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


def masks(draw, outcomes, layers):
    meas = np.zeros(layers, np.uint64)
    oc = np.zeros(layers, np.uint64)
    for t in range(layers):
        s = draw["sites"][t, : draw["sites_per_layer"][t]]
        meas[t] = mask_of(s, [1] * len(s))
        oc[t] = mask_of(s, outcomes[t, : len(s)])
    return meas, oc


def purity_low_cut(psi, k):
    """Tr(rho^2) of qubits 0..k-1: with index = env * 2^k + kept, rho's Gram
    partner M^H M (2^k x 2^k) has the same Frobenius norm as rho."""
    m = psi.reshape(-1, 1 << k)
    g = m.conj().T @ m
    return float(np.sum(np.abs(g) ** 2))


def test_headline_L24_full_depth_free_running(mg, orc):
    n, periods = 24, 24
    layers = 2 * periods
    idx = [0, 9, 15]
    seeds = [mg.trajectory_seed(0, i) for i in idx]
    ps = np.array([P_GRID[i % 16] for i in idx])
    b = mg.Batch(n, periods, capacity=len(seeds), fp64=False, observables=mg.OBS_S2_HALF)
    got = b.run(seeds, ps)
    with ThreadPoolExecutor(len(seeds)) as ex:
        refs = list(ex.map(lambda a: orc.run_trajectory(int(a[0]), n, periods, float(a[1]), True, 16,
                                                        want_state=True), zip(seeds, ps)))
    e = mg.Engine(fp64=False)
    s2s = []
    for i, (s, p, r) in enumerate(zip(seeds, ps, refs)):
        d = orc.haar_draw(int(s), n, periods, float(p), True, 16)
        meas, oc = masks(d, r["outcomes"], layers)
        np.testing.assert_array_equal(got["measured"][i], meas)
        np.testing.assert_array_equal(got["outcomes"][i], oc)
        np.testing.assert_allclose(got["surprisal"][i], r["surprisal"], rtol=0, atol=1e-5)
        e.adopt(b.state_ptr(i), n)
        psi = e.state()
        dist = float(np.linalg.norm(psi - r["psi"]))
        assert dist < 2e-4, (i, dist)
        s2 = -np.log2(purity_low_cut(r["psi"], n // 2))
        assert abs(got["obs"][i, 0, 1] - s2) < 1e-5, (i, got["obs"][i, 0, 1], s2)
        s2s.append(s2)
    # Entangled final states (volume law at p = 0.05), not product states.
    assert min(s2s) > 0.1 and max(s2s) > 2.0, s2s


def test_config0_all_200_trajectories(mg, orc):
    n, periods, p, closed = 12, 12, 0.2, False
    layers = 2 * periods
    seeds = [mg.trajectory_seed(0, i) for i in range(200)]
    b = mg.Batch(n, periods, capacity=len(seeds), closed=closed, fp64=True, observables=15, observe_every=1)
    got = b.run(seeds, p)
    with ThreadPoolExecutor(orc.max_threads()) as ex:
        refs = list(ex.map(lambda s: orc.run_trajectory(int(s), n, periods, p, closed, 16, 15, 1,
                                                        want_state=True), seeds))
    e = mg.Engine(fp64=True)
    for i, (s, r) in enumerate(zip(seeds, refs)):
        d = orc.haar_draw(int(s), n, periods, p, closed, 16)
        meas, oc = masks(d, r["outcomes"], layers)
        np.testing.assert_array_equal(got["measured"][i], meas)
        np.testing.assert_array_equal(got["outcomes"][i], oc)
        np.testing.assert_allclose(got["surprisal"][i], r["surprisal"], rtol=0, atol=1e-10)
        np.testing.assert_allclose(got["obs"][i], r["obs"], rtol=0, atol=1e-10, err_msg=f"trajectory {i}")
        e.adopt(b.state_ptr(i), n)
        np.testing.assert_allclose(e.state(), r["psi"], rtol=0, atol=1e-11)


def test_config3_lattice_L28_two_layers(mg, orc):
    X, Y, p = 4, 7, 0.15
    n, layers = X * Y, 2
    seed = mg.trajectory_seed(3, 0)
    triples = [[0, 1, 2], [0, 4, 8], [5, 6, 9]]
    b = mg.Batch(n, 1, capacity=1, fp64=False, observables=mg.OBS_S2_HALF, observe_every=1, rho3=True,
                 lattice=(X, Y))
    b.set_rho3_subsystems(triples)
    got = b.run([seed], p)
    r3 = b.fetch_rho3_points()[0]
    e = mg.Engine(fp64=False)
    e.adopt(b.state_ptr(0), n)
    psi_gpu = e.state()
    b.close()
    r = orc.run_lattice_trajectory(int(seed), X, Y, layers, p)
    d = orc.haar_lattice_draw(int(seed), X, Y, layers, p)
    meas, oc = masks(d, r["outcomes"], layers)
    np.testing.assert_array_equal(got["measured"][0], meas)
    np.testing.assert_array_equal(got["outcomes"][0], oc)
    dist = float(np.linalg.norm(psi_gpu - r["psi"]))
    assert dist < 2e-5, dist
    del psi_gpu
    np.testing.assert_allclose(r3[-1].ravel(), orc.rho3(r["psi"], triples), rtol=0, atol=2e-5)
    # Half-system S_2 of the oracle's state: the 16384 x 16384 Gram partner
    # in FP64 (a library GEMM on the device, as the checker only).
    import torch
    m = torch.from_numpy(r["psi"].reshape(1 << 14, 1 << 14)).to("cuda")
    g = m.conj().T @ m
    s2 = -np.log2(float((g.abs() ** 2).sum()))
    del m, g
    torch.cuda.empty_cache()
    assert abs(got["obs"][0, -1, 1] - s2) < 1e-5, (got["obs"][0, -1, 1], s2)
