"""Bounded device waits report a status instead of hanging.

The FP32 layer pass waits on an mbarrier for each TMA tile load, with a
bounded number of polls. mipt_gb300_test_withhold_tile_loads makes the next
pass launch skip its first CTA's first load, so that wait runs out: the CTA
sets the error flag and returns with no copy in flight, and the batch's
fetch reports MIPT_GB300_E_INTERNAL (the reference's failure contract is a
status code, cpp/src/cuda/tmi_cuda_svd.cu:203-215). Nothing faults or traps,
and the next execute on the same device must run normally and match the
oracle (FP32 1e-5 on entropies, outcomes bit-exact).
"""
import time

import numpy as np
import pytest

from tests.gpu_util import mask_of

pytestmark = pytest.mark.gpu

E_INTERNAL = 9004


@pytest.fixture(scope="module")
def mg():
    from mipt_gb300 import build
    build.build()
    import mipt_gb300
    return mipt_gb300


def oracle_outcomes(orc, seed, n, periods, p, r):
    d = orc.haar_draw(int(seed), n, periods, p, True, 16)
    oc = np.zeros(2 * periods, np.uint64)
    for t in range(2 * periods):
        s = d["sites"][t, : d["sites_per_layer"][t]]
        oc[t] = mask_of(s, r["outcomes"][t, : len(s)])
    return oc


def test_withheld_tile_load_reports_internal_error_then_recovers(mg):
    from oracle import pyoracle as orc
    n, periods, p = 20, 1, 0.25
    seeds = [mg.trajectory_seed(77, i) for i in range(2)]
    b = mg.Batch(n, periods, capacity=len(seeds), fp64=False, observables=mg.OBS_S2_HALF)
    b.run(seeds, p)  # kernels loaded, plans cached
    assert mg.lib().mipt_gb300_test_withhold_tile_loads(1) == 0
    t0 = time.perf_counter()
    with pytest.raises(mg.MiptError) as ei:
        b.run(seeds, p)
    elapsed = time.perf_counter() - t0
    assert ei.value.status == E_INTERNAL, ei.value
    assert "tile load wait timed out" in str(ei.value)
    assert elapsed < 10.0, elapsed
    # The hook applied to one launch only; the next execute is normal.
    got = b.run(seeds, p)
    for i, s in enumerate(seeds):
        r = orc.run_trajectory(int(s), n, periods, p, True, 16, mg.OBS_S2_HALF, 0, want_state=True)
        np.testing.assert_array_equal(got["outcomes"][i], oracle_outcomes(orc, s, n, periods, p, r))
        rho = orc.rdm(r["psi"], list(range(n // 2)))
        want = -np.log2(np.sum(np.abs(rho) ** 2))
        assert abs(got["obs"][i, 0, 1] - want) < 1e-5
