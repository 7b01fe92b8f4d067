"""GPU parity: the CUDA path, called through the C ABI, against the CPU FP64
oracle (oracle/) and the reference's golden fixtures (tests/golden/).

Tolerances: FP64 path 1e-10 on entropies/TMI and 1e-12 on amplitudes;
FP32 path 1e-5 on entropies (the |dS| bound of the FP32 method) and 2e-5 on
amplitudes. Measurement locations and outcomes are compared bit-exactly.
"""
import os

import numpy as np
import pytest

from tests.gpu_util import haar_layer, mask_of, random_state, sites_of

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = np.load(os.path.join(ROOT, "tests", "golden", "ref_fixtures.npz"))

TOL_S = {True: 1e-10, False: 1e-5}
TOL_PSI = {True: 1e-12, False: 2e-5}


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


def device_state(mg, psi, fp64):
    e = mg.Engine(fp64=fp64)
    e.set_state(psi)
    return e


# --------------------------------------------------------------- engine
@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("n,start", [(6, 0), (10, 1), (17, 0), (20, 1), (20, 0)])
def test_apply_bonds(mg, orc, fp64, n, start):
    psi = random_state(n, 100 + n)
    pairs, mats = haar_layer(n if n % 2 == 0 else n - 1, 7 + n, start=0)
    if start == 1:
        d = orc.haar_draw(9 + n, n - (n % 2), 1, 0.0, True)
        g = d["gates_per_layer"][1]
        pairs = d["gate_q"][1, :g]
        mats = d["gate_m"][1, :g, 0::2] + 1j * d["gate_m"][1, :g, 1::2]
    e = device_state(mg, psi, fp64)
    e.apply_bonds(pairs, mats)
    want = psi.copy()
    for (a, b), m in zip(pairs, mats):
        want = orc.apply_bond(want, int(a), int(b), m.reshape(4, 4))
    np.testing.assert_allclose(e.state(), want, rtol=0, atol=TOL_PSI[fp64])


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("n,sites,chunk", [(8, [1, 3, 4, 7], 16), (10, [0, 2, 3, 5, 6, 9], 2),
                                           (16, [0, 5, 9, 12, 15], 16), (20, list(range(0, 20, 2)), 4)])
def test_measure_layer(mg, orc, fp64, n, sites, chunk):
    psi = random_state(n, 300 + n)
    nch = (len(sites) + chunk - 1) // chunk
    rng = np.random.default_rng(n)
    for trial in range(3):
        u = rng.uniform(size=nch)
        e = device_state(mg, psi, fp64)
        out, sp = e.measure_layer(sites, u, chunk)
        want_psi, want_out, want_sp = orc.measure_layer(psi, sites, u, chunk)
        np.testing.assert_array_equal(out, want_out)
        assert abs(sp - want_sp) < (1e-12 if fp64 else 1e-5)
        np.testing.assert_allclose(e.state(), want_psi, rtol=0, atol=TOL_PSI[fp64] * 4)
        # forced replay of the same outcomes
        e2 = device_state(mg, psi, fp64)
        out2, sp2 = e2.measure_layer(sites, u, chunk, forced=want_out)
        np.testing.assert_array_equal(out2, want_out)
        assert abs(sp2 - want_sp) < (1e-12 if fp64 else 1e-5)


# --------------------------------------------- reference-compatible ops
@pytest.mark.parametrize("fp64", [True, False])
def test_rdm_and_entropies_match_reference(mg, fp64):
    for k, (n, ferm, s1, s2) in enumerate(GOLD["rdm_params"]):
        n = int(n)
        psi = GOLD[f"rdm{k}_psi"].view(np.complex128)
        kept = GOLD[f"rdm{k}_kept"]
        want = GOLD[f"rdm{k}_rho"].view(np.complex128).reshape(1 << len(kept), -1)
        e = device_state(mg, psi, fp64)
        rho = mg.rdm_subsystem(e.data, n, kept, bool(ferm), fp64)
        np.testing.assert_allclose(rho, want, rtol=0, atol=1e-12 if fp64 else 2e-6)
        assert abs(mg.entropy_svd(e.data, n, kept, bool(ferm), fp64) - s1) < (1e-10 if fp64 else 5e-5)
        assert abs(mg.renyi2(e.data, n, kept, bool(ferm), fp64) - s2) < (1e-11 if fp64 else 5e-6)


@pytest.mark.parametrize("fp64", [True, False])
def test_product_state_renyi2_is_exactly_zero(mg, fp64):
    psi = np.zeros(1 << 10, np.complex128)
    psi[0b1011001101] = 1.0
    e = device_state(mg, psi, fp64)
    assert mg.renyi2(e.data, 10, [0, 1, 2, 3, 4], False, fp64) == 0.0
    assert mg.entropy_svd(e.data, 10, [0, 1, 2, 3, 4], False, fp64) == 0.0


@pytest.mark.parametrize("fp64", [True, False])
def test_rho3_matches_reference(mg, fp64):
    for k in range(4):
        psi = GOLD[f"rho3_{k}_psi"].view(np.complex128)
        n = int(np.log2(psi.size))
        subs = GOLD[f"rho3_{k}_subs"]
        ferm = bool(GOLD[f"rho3_{k}_ferm"][0])
        e = device_state(mg, psi, fp64)
        got = mg.rho3_subsystems(e.data, n, subs, ferm, fp64)
        np.testing.assert_allclose(got, GOLD[f"rho3_{k}_out"], rtol=0, atol=1e-13 if fp64 else 2e-6)


@pytest.mark.parametrize("fp64", [True, False])
def test_measure_collapse_matches_reference(mg, fp64):
    state = None
    for i, (n, q, u, outcome, cp, _sp) in enumerate(GOLD["mc_params"]):
        psi = GOLD[f"mc{i}_in"].view(np.complex128)
        e = device_state(mg, psi, fp64)
        o, p = mg.measure_collapse(e.data, int(n), int(q), float(u), fp64)
        assert o == int(outcome)
        assert abs(p - cp) < (1e-13 if fp64 else 1e-6)
        np.testing.assert_allclose(e.state(), GOLD[f"mc{i}_out"].view(np.complex128), rtol=0,
                                   atol=1e-14 if fp64 else 1e-6)


def test_measure_collapse_rejects_bad_uniform(mg):
    e = device_state(mg, random_state(4, 1), True)
    with pytest.raises(mg.MiptError):
        mg.measure_collapse(e.data, 4, 1, 1.0, True)


# ------------------------------------------------------ whole trajectories
def oracle_batch(orc, seeds, n, periods, p, closed, chunk=16, obs_flags=0, observe_every=0, forced=None):
    outs = []
    for i, s in enumerate(seeds):
        f = None if forced is None else forced[i]
        outs.append(orc.run_trajectory(int(s), n, periods, p, closed, chunk, obs_flags, observe_every,
                                       forced=f, want_state=True))
    return outs


def oracle_masks(orc, seed, n, periods, p, closed, chunk, out):
    d = orc.haar_draw(int(seed), n, periods, p, closed, chunk)
    T = 2 * periods
    meas = np.zeros(T, np.uint64)
    oc = np.zeros(T, np.uint64)
    for t in range(T):
        s = d["sites"][t, : d["sites_per_layer"][t]]
        meas[t] = mask_of(s, [1] * len(s))
        oc[t] = mask_of(s, out["outcomes"][t, : len(s)])
    return meas, oc


def forced_rows(orc, seeds, n, periods, p, closed, chunk, outs):
    rows = []
    for s, o in zip(seeds, outs):
        d = orc.haar_draw(int(s), n, periods, p, closed, chunk)
        rows.append(o["outcomes"])
    return rows


@pytest.mark.parametrize("fp64", [True, False])
def test_plain_method_trajectories(mg, orc, fp64):
    """Open chain L=12, p=0.2, 24 layers, per-layer S_vN, S_2, TMI (the
    plain-method configuration), against the oracle."""
    n, periods, p, closed = 12, 12, 0.2, False
    seeds = [orc.trajectory_seed(0, i) for i in range(4)]
    ref = oracle_batch(orc, seeds, n, periods, p, closed, obs_flags=15, observe_every=1)
    b = mg.Batch(n, periods, capacity=len(seeds), closed=closed, fp64=fp64, observables=15, observe_every=1)
    forced = None
    if not fp64:
        forced = np.array([oracle_masks(orc, s, n, periods, p, closed, 16, r)[1] for s, r in zip(seeds, ref)])
    got = b.run(seeds, p, forced=forced)
    for i, (s, r) in enumerate(zip(seeds, ref)):
        meas, oc = oracle_masks(orc, s, n, periods, p, closed, 16, r)
        np.testing.assert_array_equal(got["measured"][i], meas)
        np.testing.assert_array_equal(got["outcomes"][i], oc)
        np.testing.assert_allclose(got["surprisal"][i], r["surprisal"], rtol=0, atol=1e-10 if fp64 else 1e-5)
        np.testing.assert_allclose(got["obs"][i], r["obs"], rtol=0, atol=TOL_S[fp64])
        e = mg.Engine(fp64=fp64)
        e.adopt(b.state_ptr(i), n)
        np.testing.assert_allclose(e.state(), r["psi"], rtol=0, atol=TOL_PSI[fp64] * 10)


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("n,periods,p,chunk,tile", [(8, 3, 1.0, 3, 0), (8, 2, 0.0, 16, 0), (16, 2, 0.3, 16, 12),
                                                    (20, 2, 0.35, 16, 0), (18, 2, 1.0, 16, 0), (20, 1, 0.5, 5, 13)])
def test_batch_edge_cases(mg, orc, fp64, n, periods, p, chunk, tile):
    """Multi-chunk layers, p = 0 and p = 1, several tiled passes per layer,
    measured sites outside the tile (fused and stand-alone histograms)."""
    closed = True
    seeds = [orc.trajectory_seed(123, i) for i in range(2)]
    ref = oracle_batch(orc, seeds, n, periods, p, closed, chunk)
    b = mg.Batch(n, periods, capacity=len(seeds), closed=closed, fp64=fp64, chunk_bits=chunk, tile_qubits=tile)
    forced = None
    if not fp64:
        forced = np.array([oracle_masks(orc, s, n, periods, p, closed, chunk, r)[1] for s, r in zip(seeds, ref)])
    got = b.run(seeds, p, forced=forced)
    for i, (s, r) in enumerate(zip(seeds, ref)):
        meas, oc = oracle_masks(orc, s, n, periods, p, closed, chunk, r)
        np.testing.assert_array_equal(got["measured"][i], meas)
        np.testing.assert_array_equal(got["outcomes"][i], oc)
        np.testing.assert_allclose(got["surprisal"][i], r["surprisal"], rtol=0, atol=1e-9 if fp64 else 1e-4)
        e = mg.Engine(fp64=fp64)
        e.adopt(b.state_ptr(i), n)
        np.testing.assert_allclose(e.state(), r["psi"], rtol=0, atol=TOL_PSI[fp64] * 10)


def test_fp32_free_running_matches_fp64(mg, orc):
    """Without replay, the FP32 path samples the same outcomes as the FP64
    oracle (boundary flips are measure-zero) and its entropies agree."""
    n, periods, p = 12, 6, 0.25
    seeds = [orc.trajectory_seed(7, i) for i in range(6)]
    ref = oracle_batch(orc, seeds, n, periods, p, True, obs_flags=15, observe_every=2)
    b = mg.Batch(n, periods, capacity=len(seeds), fp64=False, observables=15, observe_every=2)
    got = b.run(seeds, p)
    for i, (s, r) in enumerate(zip(seeds, ref)):
        _, oc = oracle_masks(orc, s, n, periods, p, True, 16, r)
        np.testing.assert_array_equal(got["outcomes"][i], oc)
        np.testing.assert_allclose(got["obs"][i], r["obs"][1::2], rtol=0, atol=1e-5)


def test_full_size_chain_L24(mg, orc):
    """L=24 (the metric's chain length), FP32, two layers: final state against
    the FP64 oracle, unit norm, half-chain S_2 against the oracle's RDM."""
    n, periods, p = 24, 1, 0.2
    seed = orc.trajectory_seed(2024, 0)
    r = orc.run_trajectory(int(seed), n, periods, p, True, 16, want_state=True)
    _, oc = oracle_masks(orc, seed, n, periods, p, True, 16, r)
    b = mg.Batch(n, periods, capacity=1, fp64=False, observables=2, rho3=True)
    got = b.run([seed], p, forced=oc[None, :])
    e = mg.Engine(fp64=False)
    e.adopt(b.state_ptr(0), n)
    psi = e.state()
    assert abs(np.vdot(psi, psi).real - 1.0) < 1e-5
    np.testing.assert_allclose(psi, r["psi"], rtol=0, atol=1e-5)
    rho = orc.rdm(r["psi"], list(range(12)))
    s2 = -np.log2(np.sum(np.abs(rho) ** 2))
    assert abs(got["obs"][0, 0, 1] - s2) < 1e-5
    subs = np.array([[s, (s + 1) % n, (s + 2) % n] for s in range(n)])
    np.testing.assert_allclose(got["rho3"][0].ravel(), orc.rho3(r["psi"], subs), rtol=0, atol=2e-6)


@pytest.mark.parametrize("n,kept,ferm", [(14, list(range(7)), False), (16, list(range(8)), False),
                                         (18, [17, 3, 9, 0, 12, 5, 8, 1, 14], True), (20, list(range(10, 20)), False),
                                         (16, [15, 14, 13, 12, 11, 10, 9, 8], True), (18, list(range(9)), True),
                                         (12, list(range(8)), False), (20, list(range(12)), False),
                                         (17, [1, 0, 2, 3, 4, 5, 6, 7], False)])
def test_tensor_core_renyi2(mg, orc, n, kept, ferm):
    """FP32 Renyi-2 through the tcgen05 3xTF32 Gram (cuts with >= 128 rows)
    against the FP64 oracle's RDM purity. Every kept set up to 14 modes
    (contiguous, gathered, reversed, fermionic) goes through the pre-split
    operand rows, whose row split gathers the kept modes and applies the
    fermionic signs."""
    psi = random_state(n, 77 + n)
    e = device_state(mg, psi, False)
    got = mg.renyi2(e.data, n, kept, ferm, False)
    rho = orc.rdm(psi, kept, ferm)
    want = -np.log2(np.sum(np.abs(rho) ** 2))
    assert abs(got - want) < 1e-5, (got, want)


def test_fp32_region_svn_large_state(mg):
    """S_vN of 8-qubit regions of L=20 FP32 states (rho summed exactly in
    FP64, measured sites left out) against the FP64 path on the same
    measurement outcomes (|dS| within the FP32 path's 1e-5)."""
    n, periods, p = 20, 3, 0.25
    seeds = [mg.trajectory_seed(20, i) for i in range(2)]
    regions = [list(range(8)), list(range(6, 14)), [0, 3, 5, 9, 12, 15, 17, 19]]
    runs = {}
    for fp64 in (True, False):
        b = mg.Batch(n, periods, capacity=len(seeds), fp64=fp64, observe_every=1)
        for r in regions:
            b.add_region(r, 1)
        got = b.run(seeds, p, forced=None if fp64 else runs[True][1])
        runs[fp64] = (b.fetch_regions(), got["outcomes"])
    np.testing.assert_array_equal(runs[False][1], runs[True][1])
    assert runs[True][0].max() > 1.0  # entangled regions, not only product states
    np.testing.assert_allclose(runs[False][0], runs[True][0], rtol=0, atol=1e-5)


@pytest.mark.parametrize("fp64", [True, False])
def test_large_spectrum_svn_batched_eigensolver(mg, orc, fp64):
    """S_vN of 8- and 9-qubit regions (256 x 256 and 512 x 512 spectra, the
    batched FP64 eigensolver) for several trajectories at once, against the
    oracle's RDM eigenvalues of the same final states."""
    n, periods, p = 18, 2, 0.15
    seeds = [mg.trajectory_seed(31, i) for i in range(3)]
    b = mg.Batch(n, periods, capacity=len(seeds), fp64=fp64)
    regions = [list(range(8)), list(range(9)), [0, 2, 4, 6, 8, 10, 12, 14]]
    for r in regions:
        b.add_region(r, 1)
    b.run(seeds, p)
    got = b.fetch_regions()
    for i, sd in enumerate(seeds):
        psi = orc.run_trajectory(int(sd), n, periods, p, closed=True, want_state=True)["psi"]
        for g, r in enumerate(regions):
            want = orc.entropy(orc.rdm(psi, r), 1)
            assert abs(got[i, 0, g] - want) < (1e-10 if fp64 else 1e-5), (i, r, got[i, 0, g], want)
