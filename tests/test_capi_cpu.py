"""CPU checks of the C-ABI library: it loads, exports every symbol the header
declares, and its host sampler reproduces the reference's random record."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = np.load(os.path.join(ROOT, "tests", "golden", "ref_fixtures.npz"))


@pytest.fixture(scope="module")
def mg():
    from mipt_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()
    import mipt_gb300
    mipt_gb300.lib()
    return mipt_gb300


def header_symbols():
    text = open(os.path.join(ROOT, "include", "mipt_gb300.h")).read()
    return sorted(set(re.findall(r"\b(mipt_(?:cuda|gb300)_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(mg):
    lib = mg.lib()
    names = header_symbols()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_seeding_matches_reference(mg):
    for s, want in zip(GOLD["splitmix_in"], GOLD["splitmix_out"]):
        assert mg.splitmix64(int(s)) == int(want)
    for row, m in zip(GOLD["trajseed_out"], (0, 1, 0xDEADBEEF)):
        assert [mg.trajectory_seed(m, i) for i in range(5)] == [int(x) for x in row]


@pytest.mark.parametrize("k", range(len(GOLD["draw_params"])))
def test_host_sampler_matches_reference(mg, k):
    seed, n, periods, p, closed, chunk = GOLD["draw_params"][k]
    n, periods, chunk = int(n), int(periods), int(chunk)
    d = mg.draw_haar(int(seed), n, periods, float(p), bool(closed), chunk)
    np.testing.assert_array_equal(d["gates_per_layer"], GOLD[f"draw{k}_gates_per_layer"])
    np.testing.assert_array_equal(d["bond_q"], GOLD[f"draw{k}_gate_q"])
    np.testing.assert_allclose(d["bond_u"], GOLD[f"draw{k}_gate_m"], rtol=0, atol=1e-12)
    sites = GOLD[f"draw{k}_sites"]
    spl = GOLD[f"draw{k}_sites_per_layer"]
    for t in range(2 * periods):
        want = 0
        for s in sites[t, : spl[t]]:
            want |= 1 << int(s)
        assert int(d["measured"][t]) == want
    np.testing.assert_array_equal(d["uniforms"], GOLD[f"draw{k}_uniforms"])


def test_bad_arguments_fail_loudly(mg):
    with pytest.raises(mg.MiptError):
        mg.draw_haar(1, 7, 2, 0.2)  # odd chain


@pytest.mark.parametrize("k", range(len(GOLD["feinit_params"])))
def test_initial_state_draw_matches_reference(mg, k):
    seed, n, kind, fixed, parity = (int(x) for x in GOLD["feinit_params"][k])
    psi, sector = mg.draw_initial_state(seed, n, kind, bool(fixed), fp64=True)
    np.testing.assert_array_equal(psi, GOLD[f"feinit{k}_amps"].view(np.complex128))
    assert sector == (parity if parity < 2**63 else -1)
    # The FP32 draw rounds where an FP32 state stores: the oracle does the same.
    from oracle import pyoracle as orc
    psi32, _ = mg.draw_initial_state(seed, n, kind, bool(fixed), fp64=False)
    want32, _ = orc.fe_initial_state(seed, n, kind, bool(fixed), fp32=True)
    np.testing.assert_array_equal(psi32, want32)


@pytest.mark.parametrize("k", range(len(GOLD["fedraw_params"])))
def test_workspace_sampler_matches_reference(mg, k):
    seed, n, layers, p, chunk = GOLD["fedraw_params"][k]
    n, layers, chunk = int(n), int(layers), int(chunk)
    d = mg.draw_haar_workspace(int(seed), n, layers, float(p), chunk)
    np.testing.assert_array_equal(d["gates_per_layer"], GOLD[f"fedraw{k}_gates_per_layer"])
    np.testing.assert_array_equal(d["bond_q"], GOLD[f"fedraw{k}_gate_q"])
    np.testing.assert_allclose(d["bond_u"], GOLD[f"fedraw{k}_gate_m"], rtol=0, atol=1e-12)
    sites, spl = GOLD[f"fedraw{k}_sites"], GOLD[f"fedraw{k}_sites_per_layer"]
    for t in range(layers):
        assert int(d["measured"][t]) == sum(1 << int(s) for s in sites[t, : spl[t]])
    np.testing.assert_array_equal(d["uniforms"], GOLD[f"fedraw{k}_uniforms"])


@pytest.mark.parametrize("seed,n,workspace", [(3, 6, False), (4, 8, False), (11, 10, False), (0x1234, 8, True)])
def test_rppu_sampler_matches_oracle(mg, seed, n, workspace):
    """The batch's RPPU draw against the oracle's (itself pinned to the
    reference): the same bonds and matrices in the plan's order (closure bond
    last, stored for the qubit order (n-1, 0)), the same measured sites, an
    identity extra layer when none was drawn, and one uniform per chunk with
    site n-1 measured alone."""
    from oracle import pyoracle as orc
    periods, p, cb = 3, 0.45, 3
    d = mg.draw_rppu(seed, n, periods, p, chunk_bits=cb, split_last=True, workspace=workspace)
    o = orc.rppu_draw(seed, n, 2 * periods if workspace else periods, p, orc.RPPU_QUBIT, workspace)
    swap = [0, 2, 1, 3]
    k = 0
    n_uniforms = 0
    for t in range(2 * periods + 1):
        bonds = {tuple(int(x) for x in d["bond_q"][t, j]): d["bond_u"][t, j].view(np.complex128).reshape(4, 4)
                 for j in range(n // 2)}
        if t >= o["layers"]:
            assert all(np.array_equal(m, np.eye(4)) for m in bonds.values()) and int(d["measured"][t]) == 0
            continue
        for _ in range(o["ops_per_layer"][t]):
            kind, q0, q1 = (int(x) for x in o["meta"][k])
            m = o["m"][k].view(np.complex128).reshape(4, 4)
            k += 1
            if (q0, q1) == (0, n - 1):
                got = bonds[(n - 1, 0)][np.ix_(swap, swap)]
            else:
                got = bonds[(q0, q1)]
            np.testing.assert_array_equal(got, m)
        sites = o["sites"][t, : o["sites_per_layer"][t]]
        assert int(d["measured"][t]) == sum(1 << int(s) for s in sites)
        plain = len(sites) - (1 if n - 1 in sites else 0)
        n_uniforms += -(-plain // cb) + (1 if n - 1 in sites else 0)
    assert len(d["uniforms"]) == n_uniforms


def test_batch_rejects_unsupported_circuits_before_device_work(mg):
    """Gate-set checks of mipt_gb300_batch_create come before any device call:
    MMS / RFGS, and RPPU off the closed 1-D ring, fail with an invalid-argument
    status on any machine."""
    for kwargs, msg in [(dict(circuit=3), "circuit must be"), (dict(circuit=2, closed=False), "closed 1-D ring"),
                        (dict(circuit=4, lattice=(2, 4)), "closed 1-D ring")]:
        with pytest.raises(mg.MiptError) as e:
            mg.Batch(8, 2, 1, **kwargs)
        assert msg in str(e.value), (kwargs, str(e.value))
