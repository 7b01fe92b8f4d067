"""Half-size parity-sector states for the RPPU / qRPPU gate sets.

With every initial state in a definite parity sector and site n-1 measured
as its own chunk (the reference's encoded engine,
cpp/include/mipt/cusv/parity.hpp:170-252, cpp/include/mipt/cusv/engine.hpp:372-477),
the batch stores 2^(n-1) amplitudes per trajectory: bonds on (q, n-1) become
parity-selected 2x2 gates on q, site n-1 is measured through the parity of
the stored bits, and observables read an expanded copy.

Checks: the same trajectories with full 2^n states (full_state=1) give
identical outcomes, surprisals and observables (FP64 1e-10, FP32 1e-5 on
entropies and 2e-5 on amplitudes and rho3 entries), for both gate sets, both
parity sectors (random fixed-parity product initial states), sizes that run
on the shared-memory and the register-round pass kernels, and the CPU FP64
oracle's default-initial-state trajectories (outcomes bit-exact).
"""
import numpy as np
import pytest

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


def run(mg, n, periods, p, seeds, circuit, fp64, full_state, init_seeds=None):
    b = mg.Batch(n, periods, len(seeds), fp64=fp64, observables=mg.OBS_SVN_HALF | mg.OBS_S2_HALF,
                 observe_every=2, rho3=True, fermion_trace=circuit == 2, circuit=circuit, full_state=full_state)
    b.add_region([0, 3, n - 1], 1)
    sectors = None
    if init_seeds is not None:
        sectors = b.set_initial_states(init_seeds, 0, fixed_parity=True)
    b.prepare(seeds, p)
    encoded = b.parity_encoded
    b.execute()
    got = b.fetch()
    got["regions"] = b.fetch_regions()
    e = mg.Engine(fp64=fp64)
    got["psi"] = []
    for i in range(len(seeds)):
        e.adopt(b.state_ptr(i), n)
        got["psi"].append(e.state())
    return got, encoded, sectors


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("circuit", [2, 4])
@pytest.mark.parametrize("n", [10, 16])
def test_encoded_matches_full_state(mg, orc, fp64, circuit, n):
    periods, p, count = 3, 0.3, 6
    seeds = [mg.trajectory_seed(77 + n, i) for i in range(count)]
    init = [orc.fe_initial_seed(orc.fe_trajectory_seed(5, i)) for i in range(count)]
    enc, used_enc, sectors = run(mg, n, periods, p, seeds, circuit, fp64, False, init)
    full, used_full, _ = run(mg, n, periods, p, seeds, circuit, fp64, True, init)
    assert used_enc and not used_full
    assert set(sectors) == {0, 1}, sectors  # both parity sectors covered
    tol = 1e-10 if fp64 else 1e-5
    np.testing.assert_array_equal(enc["measured"], full["measured"])
    np.testing.assert_array_equal(enc["outcomes"], full["outcomes"])
    np.testing.assert_allclose(enc["surprisal"], full["surprisal"], rtol=0, atol=tol)
    np.testing.assert_allclose(enc["obs"], full["obs"], rtol=0, atol=tol)
    np.testing.assert_allclose(enc["regions"], full["regions"], rtol=0, atol=tol)
    np.testing.assert_allclose(enc["rho3"], full["rho3"], rtol=0, atol=1e-10 if fp64 else 2e-5)
    for a, b in zip(enc["psi"], full["psi"]):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-12 if fp64 else 2e-5)


@pytest.mark.parametrize("circuit", [2, 4])
def test_encoded_L20_against_oracle(mg, orc, circuit):
    """L=20 FP32 (register-round passes with the parity-selected gate slot,
    sparse first passes) against the oracle's encoded-engine trajectories."""
    n, periods, p, count = 20, 3, 0.25, 3
    fermion = circuit == 2
    seeds = [mg.trajectory_seed(4040, i) for i in range(count)]
    b = mg.Batch(n, periods, count, fp64=False, observables=mg.OBS_SVN_HALF, rho3=True, fermion_trace=fermion,
                 circuit=circuit)
    got = b.run(seeds, p)
    assert b.parity_encoded
    boundary = orc.RPPU_JW if fermion else orc.RPPU_QUBIT
    e = mg.Engine(fp64=False)
    for i, sd in enumerate(seeds):
        want = orc.run_rppu_trajectory(int(sd), n, periods, p, boundary, encoded=True)
        draw = orc.rppu_draw(int(sd), n, periods, p, boundary)
        for t in range(want["layers"]):
            sites = draw["sites"][t, : draw["sites_per_layer"][t]]
            mask = sum(int(o) << int(s) for s, o in zip(sites, want["outcomes"][t][: len(sites)]))
            assert int(got["outcomes"][i, t]) == mask, (i, t)
        e.adopt(b.state_ptr(i), n)
        assert np.linalg.norm(e.state() - want["psi"]) < 1e-4
        s_half = orc.entropy(orc.rdm(want["psi"], list(range(n // 2)), fermion), 1)
        assert abs(got["obs"][i, 0, 0] - s_half) < 1e-5
