"""Allocation-free FP32 Renyi-2 (mipt_gb300_renyi2_f32_noalloc) against the
allocating entry point (mipt_cuda_renyi2_f32), both through the C ABI, and
against the CPU FP64 oracle (the state's reduced density matrix and its
Renyi-2 entropy, computed on the host from the same amplitudes).

Tolerance: 1e-5 bits, the FP32 path's entropy bound. Each case calls the
allocation-free entry point twice in a row; both results must agree with
the allocating entry point and the oracle, and with each other exactly
(every reduction runs in a fixed order). Free device memory is read around
the second and third calls: after the first call has loaded the kernels,
a call changes it by nothing. The file name sorts last so that the module
also runs after every other test in the same process; it needs no state
from them and passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from tests.gpu_util import random_state

pytestmark = pytest.mark.gpu

TOL = 1e-5
E_INVALID = 9001


@pytest.fixture(scope="module")
def mg():
    from mipt_gb300 import build
    build.build()
    import mipt_gb300
    fn = mipt_gb300.lib().mipt_gb300_renyi2_f32_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return mipt_gb300


def call_noalloc(mg, ptr, n, kept, ferm):
    kept = np.ascontiguousarray(kept, np.int32)
    out = np.full(1, np.nan)
    rc = mg.lib().mipt_gb300_renyi2_f32_noalloc(ptr, n, kept.ctypes.data, len(kept), int(ferm), out.ctypes.data)
    return rc, float(out[0])


def noalloc(mg, ptr, n, kept, ferm):
    rc, s = call_noalloc(mg, ptr, n, kept, ferm)
    assert rc == 0, mg.lib().mipt_gb300_last_error().decode(errors="replace")
    return s


def fp32_state(mg, psi):
    e = mg.Engine(fp64=False)
    e.set_state(psi)
    return e


CASES = [
    (10, [0, 1, 2, 3, 4], False),
    (12, [11, 3, 7], True),
    (14, [2], False),
    (16, list(range(8)), False),
    (18, [17, 3, 9, 0, 12, 5, 8, 1, 14], True),
    (20, list(range(10, 20)), False),
    (20, list(range(3, 17)), False),
    (22, [0, 5, 10, 15, 20, 21, 1, 2, 3, 4, 6, 7], True),
]


def oracle_renyi2(psi, kept, ferm):
    from oracle import pyoracle as orc
    # The device state holds FP32 amplitudes: the oracle reads the same ones.
    psi32 = psi.astype(np.complex64).astype(np.complex128)
    return orc.entropy(orc.rdm(psi32, kept, ferm), 2)


def free_device_bytes():
    free = ctypes.c_size_t()
    total = ctypes.c_size_t()
    rt = ctypes.CDLL("libcudart.so.13")
    rt.cudaMemGetInfo.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("n,kept,ferm", CASES)
def test_noalloc_matches_allocating_entry_point(mg, n, kept, ferm):
    psi = random_state(n, 1000 + n)
    e = fp32_state(mg, psi)
    want = mg.renyi2(e.data, n, kept, ferm, False)
    first = noalloc(mg, e.data, n, kept, ferm)
    second = noalloc(mg, e.data, n, kept, ferm)
    assert abs(first - want) < TOL, (first, want)
    assert abs(second - want) < TOL, (second, want)
    assert first == second
    if n <= 20:
        ref = oracle_renyi2(psi, kept, ferm)
        assert abs(first - ref) < TOL, (first, ref)


def test_noalloc_changes_no_device_memory(mg):
    """After the first call, calls leave the device's free memory unchanged."""
    n, kept = 18, list(range(3, 17))
    e = fp32_state(mg, random_state(n, 99))
    noalloc(mg, e.data, n, kept, False)  # first call: kernels load here
    before = free_device_bytes()
    a = noalloc(mg, e.data, n, kept, False)
    b = noalloc(mg, e.data, n, [1, 4, 9], True)
    after = free_device_bytes()
    assert before == after, (before, after)
    assert np.isfinite(a) and np.isfinite(b)


def test_noalloc_interleaved_sizes(mg):
    """Back-to-back calls of different sizes reuse the one static array."""
    n = 18
    e = fp32_state(mg, random_state(n, 4242))
    big, small = list(range(14)), [5, 9, 13]
    want_big = mg.renyi2(e.data, n, big, False, False)
    want_small = mg.renyi2(e.data, n, small, True, False)
    got = [noalloc(mg, e.data, n, big, False), noalloc(mg, e.data, n, small, True),
           noalloc(mg, e.data, n, big, False), noalloc(mg, e.data, n, small, True)]
    assert abs(got[0] - want_big) < TOL and abs(got[2] - want_big) < TOL
    assert abs(got[1] - want_small) < TOL and abs(got[3] - want_small) < TOL
    assert got[0] == got[2] and got[1] == got[3]


def test_noalloc_product_state_and_empty_cut(mg):
    n = 10
    psi = np.zeros(1 << n, np.complex128)
    psi[0b1011001101] = 1.0
    e = fp32_state(mg, psi)
    assert noalloc(mg, e.data, n, [0, 1, 2, 3, 4], False) == 0.0
    assert noalloc(mg, e.data, n, [], False) == 0.0


def test_noalloc_rejects_oversize_request(mg):
    n = 16
    e = fp32_state(mg, random_state(n, 7))
    rc, _ = call_noalloc(mg, e.data, n, list(range(15)), False)
    assert rc == E_INVALID
    msg = mg.lib().mipt_gb300_last_error().decode(errors="replace")
    assert "14 kept modes" in msg and "512 KiB" in msg
    # The rejection leaves the entry point usable.
    want = mg.renyi2(e.data, n, list(range(14)), False, False)
    assert abs(noalloc(mg, e.data, n, list(range(14)), False) - want) < TOL
