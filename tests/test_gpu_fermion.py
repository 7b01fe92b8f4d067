"""GPU parity of the free-fermion (Majorana covariance) path against the FP64
covariance oracle (oracle/oracle.cpp, itself cross-checked against a
Jordan-Wigner state-vector simulation in tests/test_ff_oracle.py).

FP32 evolution with FP64 denominators, re-purification and eigensolves:
entropies and TMI within 1e-5 bits; outcomes bit-exact. FP64 evolution (the
plain method): entropies and TMI within 1e-10 bits, Gamma within 1e-11,
outcomes bit-exact without replay."""
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


@pytest.mark.parametrize("N,depth,p,closed,every", [(16, 40, 0.2, True, 8), (12, 30, 0.3, False, 0),
                                                    (8, 20, 1.0, True, 4), (20, 24, 0.0, True, 12)])
def test_forced_replay_matches_oracle(mg, orc, N, depth, p, closed, every):
    seeds = [orc.trajectory_seed(3, i) for i in range(3)]
    blocks = [1, N // 4, N // 2, N - 1]
    refs = [orc.ff_trajectory(int(s), N, depth, p, closed, blocks=blocks) for s in seeds]
    forced = np.array([r["outcomes"] for r in refs])
    got = mg.ff_run(seeds, p, N, depth, closed, repurify_every=every, blocks=blocks, tmi=(N % 4 == 0),
                    forced=forced, want_gamma=True)
    for i, r in enumerate(refs):
        np.testing.assert_array_equal(got["outcomes"][i], r["outcomes"])
        np.testing.assert_allclose(got["probs"][i], r["probs"], rtol=0, atol=2e-5)
        np.testing.assert_allclose(got["gamma"][i], r["gamma"], rtol=0, atol=5e-5)
        np.testing.assert_allclose(got["s_blocks"][i], r["s_blocks"], rtol=0, atol=1e-5)
        if N % 4 == 0:
            assert abs(got["tmi"][i] - r["tmi"]) < 1e-5


def test_free_running_outcomes_match_oracle(mg, orc):
    N, depth, p = 16, 32, 0.25
    seeds = [orc.trajectory_seed(9, i) for i in range(6)]
    got = mg.ff_run(seeds, p, N, depth, True, repurify_every=16, blocks=[8])
    for i, s in enumerate(seeds):
        r = orc.ff_trajectory(int(s), N, depth, p, True, blocks=[8])
        np.testing.assert_array_equal(got["outcomes"][i], r["outcomes"])
        assert abs(got["s_blocks"][i, 0] - r["s_blocks"][0]) < 1e-5


def test_config_size_N128(mg, orc):
    """N=128 modes (256 Majoranas), depth 256, p=0.2: the free-fermion
    configuration's size, one trajectory replayed against the oracle."""
    N, depth, p = 128, 256, 0.2
    seed = orc.trajectory_seed(42, 0)
    r = orc.ff_trajectory(int(seed), N, depth, p, True, blocks=[16, 32, 64])
    got = mg.ff_run([seed], p, N, depth, True, repurify_every=64, blocks=[16, 32, 64], forced=r["outcomes"][None],
                    want_gamma=True)
    np.testing.assert_allclose(got["s_blocks"][0], r["s_blocks"], rtol=0, atol=1e-5)
    assert abs(got["tmi"][0] - r["tmi"]) < 1e-5
    G = got["gamma"][0]
    np.testing.assert_allclose(G @ G, -np.eye(2 * N), atol=1e-9)


@pytest.mark.parametrize("N,depth,p,closed,every", [(16, 40, 0.2, True, 8), (12, 30, 0.3, False, 0),
                                                    (20, 24, 0.1, True, 12)])
def test_fp64_free_running_matches_oracle(mg, orc, N, depth, p, closed, every):
    seeds = [orc.trajectory_seed(13, i) for i in range(3)]
    blocks = [1, N // 4, N // 2, N - 1]
    got = mg.ff_run(seeds, p, N, depth, closed, repurify_every=every, blocks=blocks, tmi=(N % 4 == 0),
                    want_gamma=True, fp64=True)
    for i, s in enumerate(seeds):
        r = orc.ff_trajectory(int(s), N, depth, p, closed, repurify_every=every, blocks=blocks)
        np.testing.assert_array_equal(got["outcomes"][i], r["outcomes"])
        np.testing.assert_allclose(got["probs"][i], r["probs"], rtol=0, atol=1e-12)
        np.testing.assert_allclose(got["gamma"][i], r["gamma"], rtol=0, atol=1e-11)
        np.testing.assert_allclose(got["s_blocks"][i], r["s_blocks"], rtol=0, atol=1e-10)
        if N % 4 == 0:
            assert abs(got["tmi"][i] - r["tmi"]) < 1e-10


def test_fp64_config_size_N128(mg, orc):
    """N=128, depth 256, p=0.2 in FP64 (the free-fermion configuration as
    specified), free running, against the oracle at 1e-10."""
    N, depth, p = 128, 256, 0.2
    seed = orc.trajectory_seed(43, 0)
    blocks = [16, 32, 64]
    r = orc.ff_trajectory(int(seed), N, depth, p, True, repurify_every=64, blocks=blocks)
    got = mg.ff_run([seed], p, N, depth, True, repurify_every=64, blocks=blocks, want_gamma=True, fp64=True)
    np.testing.assert_array_equal(got["outcomes"][0], r["outcomes"])
    np.testing.assert_allclose(got["s_blocks"][0], r["s_blocks"], rtol=0, atol=1e-10)
    assert abs(got["tmi"][0] - r["tmi"]) < 1e-10
    np.testing.assert_allclose(got["gamma"][0], r["gamma"], rtol=0, atol=1e-11)


def test_bad_arguments(mg):
    with pytest.raises(mg.MiptError):
        mg.ff_run([1], 0.2, 7, 4)
