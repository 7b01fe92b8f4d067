"""The non-default kernel paths selected by environment switches give the same
results as the defaults: per-thread tile loads instead of TMA tensor loads
(MIPT_GB300_TILE_TMA=0), one CTA per tile instead of a persistent grid
(MIPT_GB300_PERSISTENT_PASS=0), gathered instead of pre-split tensor-core Gram
operands (MIPT_GB300_TC_PRESPLIT=0), a live tile autotune instead of the
measured table (MIPT_GB300_AUTOTUNE=1). The switches are read once per process,
so each variant runs in a child process on the same seeds. Tolerances: state
amplitudes 1e-6 (the FP32 path's rounding); entropies 1e-5, the FP32 entropy
bound (the gathered Gram keeps the measured sites' zero rows and columns that
the pre-split path leaves out, so its FP32 sums run in another order)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import mipt_gb300 as mg
n, periods, p = 20, 3, 0.25
seeds = [mg.trajectory_seed(91, i) for i in range(3)]
b = mg.Batch(n, periods, capacity=3, fp64=False, observables=mg.OBS_S2_HALF, observe_every=1)
got = b.run(seeds, p)
e = mg.Engine(fp64=False)
e.adopt(b.state_ptr(1), n)
psi = e.state()
s2 = [mg.renyi2(b.state_ptr(i), n, list(range(10)), False, False) for i in range(3)]
print(json.dumps(dict(outcomes=got["outcomes"].tolist(), obs=np.nan_to_num(got["obs"]).tolist(),
                      psi_re=psi.real[:4096].tolist(), psi_im=psi.imag[:4096].tolist(), s2=s2)))
"""


def child(env):
    e = dict(os.environ)
    e.update(env)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, env=e, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.fixture(scope="module")
def default_run():
    from mipt_gb300 import build
    build.build()
    return child({})


@pytest.mark.parametrize("env", [{"MIPT_GB300_TILE_TMA": "0"}, {"MIPT_GB300_PERSISTENT_PASS": "0"},
                                 {"MIPT_GB300_TC_PRESPLIT": "0"}, {"MIPT_GB300_AUTOTUNE": "1"}])
def test_switch_gives_the_same_trajectories(default_run, env):
    alt = child(env)
    assert alt["outcomes"] == default_run["outcomes"]
    np.testing.assert_allclose(alt["psi_re"], default_run["psi_re"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(alt["psi_im"], default_run["psi_im"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(alt["obs"], default_run["obs"], rtol=0, atol=1e-5)
    np.testing.assert_allclose(alt["s2"], default_run["s2"], rtol=0, atol=1e-6)


def test_autotune_reports_every_candidate():
    """mipt_gb300_autotune_tile times the default tile and the two below it."""
    import mipt_gb300 as mg
    best, ms = mg.autotune_tile(16, fp64=False, trajectories=64)
    assert set(ms) == {12, 13, 14} and best in ms and all(t > 0 for t in ms.values())
    assert ms[best] == min(ms.values())
    best, ms = mg.autotune_tile(12, fp64=True, trajectories=4)
    assert set(ms) == {11, 12} and best in ms  # FP64 candidates 11..13, capped at n
    best, ms = mg.autotune_tile(10, fp64=False, trajectories=4)
    assert set(ms) == {10} and best == 10  # every FP32 candidate is capped at n
