"""Hand-written FP64 eigensolver (eigen.cu) behind the von Neumann entropy of
spectra above 64 x 64: Householder tridiagonalisation, one CTA per matrix,
then implicit QL, one thread per matrix.

Checked through the C ABI against the CPU oracle's reduced density matrix,
whose spectrum numpy's LAPACK eigensolver gives: FP64 states to 1e-10 bits
(the FP64 path's bound), FP32 states to 1e-5, at d = 128, 256, 512 and
1024, one matrix per call and many per batched call; plus known answers
(a Bell pair gives exactly 1 bit, a maximally entangled block its qubit
count, a product state 0).
"""
import numpy as np
import pytest

from tests.gpu_util import random_state

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


def svn_of(rho):
    w = np.linalg.eigvalsh(rho)
    w = w[w > 1e-15]
    s = float(-np.sum(w * np.log2(w)))
    return 0.0 if abs(s) < 1e-12 else s


def device_state(mg, psi, fp64):
    e = mg.Engine(fp64=fp64)
    e.set_state(psi)
    return e


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("n,kept", [(14, list(range(7))), (16, [1, 3, 5, 7, 9, 11, 13, 15]),
                                    (18, list(range(9, 18))), (20, list(range(10)))])
def test_single_matrix_entropy(mg, orc, fp64, n, kept):
    psi = random_state(n, 500 + n)
    e = device_state(mg, psi, fp64)
    got = mg.entropy_svd(e.data, n, kept, False, fp64)
    src = psi if fp64 else psi.astype(np.complex64).astype(np.complex128)
    want = svn_of(orc.rdm(src, kept))
    assert abs(got - want) < (1e-10 if fp64 else 1e-5), (got, want)


def test_batched_regions_against_oracle(mg, orc):
    """Many 128 x 128 and 1024 x 1024 spectra in one batched call (FP64
    trajectories of an L=20 chain, two layers)."""
    n, periods, p = 20, 1, 0.1
    seeds = [mg.trajectory_seed(41, i) for i in range(3)]
    b = mg.Batch(n, periods, capacity=len(seeds), fp64=True)
    regions = [list(range(7)), list(range(5, 15)), [0, 2, 4, 6, 8, 10, 12]]
    for r in regions:
        b.add_region(r, 1)
    b.run(seeds, p)
    got = b.fetch_regions()
    for i, sd in enumerate(seeds):
        psi = orc.run_trajectory(int(sd), n, periods, p, closed=True, want_state=True)["psi"]
        for g, r in enumerate(regions):
            want = svn_of(orc.rdm(psi, r))
            assert abs(got[i, 0, g] - want) < 1e-10, (i, r, got[i, 0, g], want)


@pytest.mark.parametrize("fp64", [True, False])
def test_known_spectra(mg, fp64):
    n = 16
    # An FP32 state stores 1/sqrt(2) with a relative error of about 1e-8.
    tol = 1e-12 if fp64 else 1e-6
    # Bell pair on qubits (0, 9), everything else |0>: one bit across any
    # cut that separates 0 from 9; the rest of the 256 x 256 spectrum is 0.
    psi = np.zeros(1 << n, np.complex128)
    psi[0] = psi[(1 << 0) | (1 << 9)] = 1 / np.sqrt(2)
    e = device_state(mg, psi, fp64)
    assert abs(mg.entropy_svd(e.data, n, list(range(8)), False, fp64) - 1.0) < tol
    # Product state: exactly 0.
    psi = np.zeros(1 << n, np.complex128)
    psi[0b1011001110001101] = 1.0
    e = device_state(mg, psi, fp64)
    assert mg.entropy_svd(e.data, n, list(range(9)), False, fp64) == 0.0
    # Qubits 0..6 maximally entangled with 7..13: S = 7 bits.
    psi = np.zeros(1 << n, np.complex128)
    for a in range(128):
        psi[a | (a << 7)] = 1 / np.sqrt(128)
    e = device_state(mg, psi, fp64)
    assert abs(mg.entropy_svd(e.data, n, list(range(7)), False, fp64) - 7.0) < (1e-10 if fp64 else 1e-5)
