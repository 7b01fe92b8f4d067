"""2-D four-colour Haar brickwork on the GPU (config 3 geometry).

Small lattice (3 x 4) against the FP64 oracle at every observation point:
measurement outcomes bit-exact, half-system S_vN / S_2, extra regions and
three-site RDMs (FP64 1e-10; FP32 1e-5 on entropies, 2e-5 on rho3 entries).
Config-3 size (4 x 7, L = 28, FP32, 2 GiB state) through size-independent
properties: Schmidt symmetry of the half-system S_2 (qubits 0..13 by the TMA
operand path vs 14..27 by the gathered one), S_2 <= S_vN on the same region,
unit-trace Hermitian PSD rho3 blocks, outcomes consistent with the draw."""
import numpy as np
import pytest

from tests.gpu_util import mask_of

pytestmark = pytest.mark.gpu


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


def oracle_masks(orc, seed, X, Y, layers, p, outcomes):
    d = orc.haar_lattice_draw(int(seed), X, Y, layers, p)
    meas = np.zeros(layers, np.uint64)
    oc = np.zeros(layers, np.uint64)
    for t in range(layers):
        s = d["sites"][t, : d["sites_per_layer"][t]]
        meas[t] = mask_of(s, [1] * len(s))
        oc[t] = mask_of(s, outcomes[t, : len(s)])
    return meas, oc


def entropy(orc, psi, modes, order):
    return orc.entropy(orc.rdm(psi, modes), order)


@pytest.mark.parametrize("fp64", [True, False])
def test_small_lattice_against_oracle(mg, orc, fp64):
    X, Y, periods, p, every = 3, 4, 4, 0.3, 2
    n, layers = X * Y, 2 * periods
    seeds = [orc.trajectory_seed(3, i) for i in range(4)]
    refs = [orc.run_lattice_trajectory(int(s), X, Y, layers, p, observe_every=every) for s in seeds]
    forced = None
    if not fp64:  # replay the oracle's outcomes so FP32 states stay comparable
        forced = np.array([oracle_masks(orc, s, X, Y, layers, p, r["outcomes"])[1] for s, r in zip(seeds, refs)])
    b = mg.Batch(n, periods, capacity=len(seeds), fp64=fp64, observables=mg.OBS_SVN_HALF | mg.OBS_S2_HALF,
                 observe_every=every, rho3=True, lattice=(X, Y))
    regions = [([0, 1, 3, 4], 1), ([0, 3, 6, 9, 1], 2), (list(range(6, 12)), 1)]
    for modes, order in regions:
        b.add_region(modes, order)
    triples = [[0, 1, 2], [0, 3, 6], [4, 5, 7]]
    b.set_rho3_subsystems(triples)
    got = b.run(seeds, p, forced=forced)
    reg = b.fetch_regions()
    r3 = b.fetch_rho3_points()
    tol = 1e-10 if fp64 else 1e-5
    for i, (s, r) in enumerate(zip(seeds, refs)):
        meas, oc = oracle_masks(orc, s, X, Y, layers, p, r["outcomes"])
        np.testing.assert_array_equal(got["measured"][i], meas)
        np.testing.assert_array_equal(got["outcomes"][i], oc)
        for pt, psi in enumerate(r["states"]):
            half = list(range(n // 2))
            assert abs(got["obs"][i, pt, 0] - entropy(orc, psi, half, 1)) < tol
            assert abs(got["obs"][i, pt, 1] - entropy(orc, psi, half, 2)) < tol
            for g, (modes, order) in enumerate(regions):
                assert abs(reg[i, pt, g] - entropy(orc, psi, modes, order)) < tol, (i, pt, g)
            np.testing.assert_allclose(r3[i, pt].ravel(), orc.rho3(psi, triples), rtol=0,
                                       atol=1e-10 if fp64 else 2e-5)
        np.testing.assert_allclose(got["rho3"][i].ravel(), orc.rho3(r["psi"], triples), rtol=0,
                                   atol=1e-10 if fp64 else 2e-5)


def test_config3_size_lattice_properties(mg, orc):
    """4 x 7 lattice, L = 28 (2 GiB FP32 state), p = 0.15, 6 layers observed
    every layer."""
    X, Y, periods, p = 4, 7, 3, 0.15
    n, layers = X * Y, 2 * periods
    b = mg.Batch(n, periods, capacity=1, fp64=False, observables=mg.OBS_S2_HALF, observe_every=1, rho3=True,
                 lattice=(X, Y))
    comp = b.add_region(list(range(14, 28)), 2)     # complement of the half system
    rows = b.add_region(list(range(8)), 1)          # two rows, S_vN (<= 10 qubits)
    rows2 = b.add_region(list(range(8)), 2)
    b.set_rho3_subsystems([[0, 1, 2], [0, 4, 8], [5, 6, 9]])
    seed = orc.trajectory_seed(28, 0)
    got = b.run([seed], p)
    reg = b.fetch_regions()[0]
    r3 = b.fetch_rho3_points()[0]
    d = mg.draw_haar_lattice(seed, X, Y, layers, p)
    np.testing.assert_array_equal(got["measured"][0], d["measured"])
    assert np.all((got["outcomes"][0] & ~got["measured"][0]) == 0)
    for t in range(layers):
        s2 = got["obs"][0, t, 1]
        assert 0.0 <= s2 <= 14.0
        assert abs(s2 - reg[t, comp]) < 1e-5, (t, s2, reg[t, comp])
        # S_2 <= S_vN, within the FP32 path's 1e-5 (the 8-qubit region's S_2
        # comes from a tensor-core purity over 2^20 environment columns).
        assert -1e-9 <= reg[t, rows2] <= reg[t, rows] + 1e-5
        for blk in r3[t]:
            rho = (blk[0::2] + 1j * blk[1::2]).reshape(8, 8)
            assert abs(np.trace(rho).real - 1.0) < 1e-5
            np.testing.assert_allclose(rho, rho.conj().T, rtol=0, atol=1e-6)
            assert np.linalg.eigvalsh(rho).min() > -1e-6
    assert got["obs"][0, -1, 1] > 0.5  # entanglement has grown
