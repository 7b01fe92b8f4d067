"""Entropies of freshly measured states with the measured sites taken out
of rho = M M^H first: after a projective measurement the state is
|outcome> (x) phi on the measured sites, so only the rows and columns of M
whose measured bits equal the outcome are non-zero (a 2^kq x 2^eq block).

* S_2 of FP32 states through the pre-split tensor-core Gram. High
  measurement rates push the reduced block below one 128-row tile (kq < 7)
  and below one 16-column chunk (eq < 4); both are padded with zeros.
  Checked per layer against the CPU FP64 oracle: outcomes bit-exact, S_2 to
  1e-5 (the FP32 path's bound).
* S_vN and the von Neumann TMI of FP64 and FP32 states through the SIMT Gram
  and the Householder eigensolver, which runs on the reduced rows only:
  FP64 to 1e-10, FP32 to 1e-5."""
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


@pytest.mark.parametrize("n,p", [(14, 0.3), (16, 0.5), (16, 0.9), (18, 0.15)])
def test_per_layer_s2_of_measured_states(mg, n, p):
    from oracle import pyoracle as orc
    periods, count = 3, 4
    seeds = [mg.trajectory_seed(31, 100 * n + i) for i in range(count)]
    b = mg.Batch(n, periods, capacity=count, fp64=False, observables=mg.OBS_S2_HALF, observe_every=1)
    got = b.run(seeds, p)
    for i, s in enumerate(seeds):
        r = orc.run_trajectory(int(s), n, periods, p, True, 16, orc.OBS_S2, 1)
        d = orc.haar_draw(int(s), n, periods, p, True, 16)
        for t in range(2 * periods):
            sites = d["sites"][t, : d["sites_per_layer"][t]]
            assert got["outcomes"][i][t] == mask_of(sites, r["outcomes"][t, : len(sites)])
        np.testing.assert_allclose(got["obs"][i][:, 1], r["obs"][:, 1], rtol=0, atol=1e-5,
                                   err_msg=f"n={n} p={p} trajectory {i}")


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("n,p,periods,count", [(16, 0.35, 2, 3), (20, 0.2, 1, 2)])
def test_per_layer_svn_and_tmi_of_measured_states(mg, fp64, n, p, periods, count):
    """Half-chain S_vN (256- and 1024-row spectra: the Householder eigensolver
    on the reduced rows only) and the von Neumann TMI after every layer,
    against the oracle: FP64 1e-10, FP32 1e-5."""
    from oracle import pyoracle as orc
    flags = mg.OBS_SVN_HALF | mg.OBS_TMI_VN
    seeds = [mg.trajectory_seed(37, 100 * n + i) for i in range(count)]
    b = mg.Batch(n, periods, capacity=count, fp64=fp64, observables=flags, observe_every=1)
    got = b.run(seeds, p)
    tol = 1e-10 if fp64 else 1e-5
    for i, s in enumerate(seeds):
        r = orc.run_trajectory(int(s), n, periods, p, True, 16, orc.OBS_SVN | orc.OBS_TMI1, 1)
        for col in (0, 2):
            np.testing.assert_allclose(got["obs"][i][:, col], r["obs"][:, col], rtol=0, atol=tol,
                                       err_msg=f"n={n} p={p} fp64={fp64} trajectory {i} column {col}")
