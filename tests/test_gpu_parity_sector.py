"""Jordan-Wigner string and parity-sector passes (mipt_cuda_jw_string_*,
mipt_cuda_parity_*), and the host-state rho3 variants, through the C ABI
against numpy restatements of the reference semantics
(cpp/include/mipt/cuda/cusv_diag.hpp, cusv_parity.hpp, rho_reduce.hpp:78-126).

Tolerances: FP64 1e-12, FP32 2e-6 on amplitudes and weights."""
import ctypes

import numpy as np
import pytest

from tests.gpu_util import random_state

pytestmark = pytest.mark.gpu
TOL = {True: 1e-12, False: 2e-6}


@pytest.fixture(scope="module")
def mg():
    from mipt_gb300 import build
    build.build()
    import mipt_gb300
    L = mipt_gb300.lib()
    vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    for sfx in ("f32", "f64"):
        getattr(L, f"mipt_cuda_jw_string_{sfx}").argtypes = [vp, ci, ci, ctypes.c_uint64]
        getattr(L, f"mipt_cuda_parity_gate_{sfx}").argtypes = [vp, ci, ci, vp, vp]
        getattr(L, f"mipt_cuda_parity_abs2_{sfx}").argtypes = [vp, ci, vp]
        getattr(L, f"mipt_cuda_parity_collapse_{sfx}").argtypes = [vp, ci, ci, cd]
        getattr(L, f"mipt_cuda_parity_expand_{sfx}").argtypes = [vp, ci]
        for mid in ("", "fermion_"):
            getattr(L, f"mipt_cuda_rho3_subsystems_complex_host_{mid}{sfx}").argtypes = [vp, ci, vp, ci, vp]
    L.mipt_cuda_cusv_diag_last_error.restype = ctypes.c_char_p
    L.mipt_cuda_cusv_parity_last_error.restype = ctypes.c_char_p
    return mipt_gb300


def sfx(fp64):
    return "f64" if fp64 else "f32"


def parity(x):
    return np.array([bin(int(v)).count("1") & 1 for v in np.atleast_1d(x)])


def device(mg, psi, fp64):
    e = mg.Engine(fp64=fp64)
    e.set_state(psi)
    return e




@pytest.mark.parametrize("fp64", [True, False])
def test_jw_string(mg, fp64):
    n, control, mask = 11, 3, 0b10110010001
    psi = random_state(n, 5)
    e = device(mg, psi, fp64)
    assert getattr(mg.lib(), f"mipt_cuda_jw_string_{sfx(fp64)}")(e.data, n, control, mask) == 0
    idx = np.arange(1 << n)
    flip = ((idx >> control) & 1).astype(bool) & (parity(idx & mask) == 1)
    want = np.where(flip, -psi, psi)
    np.testing.assert_allclose(e.state(), want, rtol=0, atol=TOL[fp64])
    assert getattr(mg.lib(), f"mipt_cuda_jw_string_{sfx(fp64)}")(e.data, n, n, mask) == -1
    assert b"Invalid JW-string argument" in mg.lib().mipt_cuda_cusv_diag_last_error()


def even_parity_state(n, seed):
    psi = random_state(n, seed)
    psi[parity(np.arange(1 << n)) == 1] = 0
    return psi / np.linalg.norm(psi)


def encode(full, n):
    e = np.arange(1 << (n - 1))
    enc = np.zeros(1 << n, complex)  # encoded state in the low half of a 2^n buffer
    enc[: 1 << (n - 1)] = full[e | (parity(e) << (n - 1))]
    return enc


def random_parity_gate(seed):
    rng = np.random.default_rng(seed)
    def u2():
        q, _ = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
        return q
    return u2(), u2()  # even block on (b_t, b_top) in {00, 11}, odd block on {01, 10}, indexed by b_t


def apply_full(full, n, t, even, odd):
    """The two-mode parity-preserving gate on (t, n-1) in the full space."""
    out = full.copy()
    top = n - 1
    for i in range(1 << n):
        if (i >> t) & 1 or (i >> top) & 1:
            continue
        i00, i10, i01, i11 = i, i | 1 << t, i | 1 << top, i | 1 << t | 1 << top
        a, b = full[i00], full[i11]
        out[i00], out[i11] = even[0, 0] * a + even[0, 1] * b, even[1, 0] * a + even[1, 1] * b
        a, b = full[i01], full[i10]  # b_t = 0, then b_t = 1
        out[i01], out[i10] = odd[0, 0] * a + odd[0, 1] * b, odd[1, 0] * a + odd[1, 1] * b
    return out


def ri(m):
    return np.ascontiguousarray(np.stack([m.real, m.imag], -1).reshape(-1))


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("t", [0, 4, 8])
def test_parity_gate_and_expand(mg, fp64, t):
    n = 10
    full = even_parity_state(n, 11 + t)
    even, odd = random_parity_gate(t)
    want = apply_full(full, n, t, even, odd)
    e = device(mg, encode(full, n), fp64)
    ev, od = ri(even), ri(odd)
    L = mg.lib()
    assert getattr(L, f"mipt_cuda_parity_gate_{sfx(fp64)}")(e.data, n - 1, t, ev.ctypes.data, od.ctypes.data) == 0
    assert getattr(L, f"mipt_cuda_parity_expand_{sfx(fp64)}")(e.data, n) == 0
    np.testing.assert_allclose(e.state(), want, rtol=0, atol=10 * TOL[fp64])


@pytest.mark.parametrize("fp64", [True, False])
def test_parity_abs2_and_collapse(mg, fp64):
    n = 12
    enc = random_state(n - 1, 3)
    buf = np.zeros(1 << n, complex)
    buf[: 1 << (n - 1)] = enc
    e = device(mg, buf, fp64)
    L = mg.lib()
    w = np.zeros(2)
    assert getattr(L, f"mipt_cuda_parity_abs2_{sfx(fp64)}")(e.data, n - 1, w.ctypes.data) == 0
    par = parity(np.arange(1 << (n - 1)))
    want = np.array([np.sum(np.abs(enc[par == 0]) ** 2), np.sum(np.abs(enc[par == 1]) ** 2)])
    np.testing.assert_allclose(w, want, rtol=0, atol=TOL[fp64])
    assert getattr(L, f"mipt_cuda_parity_collapse_{sfx(fp64)}")(e.data, n - 1, 1, w[1]) == 0
    got = e.state()[: 1 << (n - 1)]
    np.testing.assert_allclose(got, np.where(par == 1, enc / np.sqrt(w[1]), 0), rtol=0, atol=10 * TOL[fp64])
    w2 = np.zeros(2)
    assert getattr(L, f"mipt_cuda_parity_abs2_{sfx(fp64)}")(e.data, n - 1, w2.ctypes.data) == 0
    assert abs(w2[0]) == 0.0 and abs(w2[1] - 1.0) < 10 * TOL[fp64]
    assert getattr(L, f"mipt_cuda_parity_collapse_{sfx(fp64)}")(e.data, n - 1, 2, 1.0) == -1
    assert getattr(L, f"mipt_cuda_parity_collapse_{sfx(fp64)}")(e.data, n - 1, 0, 0.0) == -1
    assert b"Invalid parity-collapse argument" in L.mipt_cuda_cusv_parity_last_error()


@pytest.mark.parametrize("fp64", [True, False])
def test_host_rho3_variants_match_device(mg, fp64):
    n = 9
    psi = random_state(n, 21)
    subs = np.array([[s, (s + 1) % n, (s + 3) % n] for s in range(n)], np.int32)
    e = device(mg, psi, fp64)
    host = np.ascontiguousarray(np.stack([psi.real, psi.imag], -1).astype(np.float64 if fp64 else np.float32))
    for fermion in (False, True):
        dev = mg.rho3_subsystems(e.data, n, subs, fermion, fp64)
        out = np.zeros(128 * n)
        mid = "fermion_" if fermion else ""
        fn = getattr(mg.lib(), f"mipt_cuda_rho3_subsystems_complex_host_{mid}{sfx(fp64)}")
        assert fn(host.ctypes.data, n, subs.ctypes.data, n, out.ctypes.data) == 0
        np.testing.assert_array_equal(out, dev)
