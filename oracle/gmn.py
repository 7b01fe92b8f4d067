"""CPU FP64 oracle for the genuine multipartite negativity (GMN) of a
three-qubit state (test infrastructure only: used by tests/ and as the CPU
baseline of the GMN bench, never by the product).

The SDP is the reference's monotone, fully decomposable witness
(cpp/src/analysis/gmn_mosek.c:14-40, python/gmn.py:236-358):

    minimise  Re Tr(rho W)
    over      W, Q_m  (8x8 Hermitian; m = 1, 2, 3 the bipartition masks)
    s.t.      0 <= Q_m <= I,   0 <= W - PT_m(Q_m) <= I,

and GMN = -min, set to 0 at or below 1e-8 (python/gmn.py:347-351). PT_m is
the partial transpose on the index bits of mask m: entry (r, c) comes from
(r & ~m | c & m, c & ~m | r & m) (gmn_mosek.c:152-160). The reference solves it
with MOSEK's interior point method, a closed dependency absent here; this
oracle solves the same SDP by ADMM in FP64 to a certified duality gap, and is
pinned to the reference's known answers (cpp/tests/gmn_solver_tests.cpp:83-205).

ADMM (scaled form, penalty sigma) on the split U_m = Q_m, V_m = W - T_m Q_m
with U_m, V_m in the box C = {0 <= X <= I}:
    x-step (closed form, T_m self-adjoint and an involution):
        a_m = U_m - Yh_m,  b_m = V_m - Zh_m,
        W   = (sum_m (T_m a_m + b_m) - 2 rho / sigma) / 3,
        Q_m = (a_m + T_m (W - b_m)) / 2;
    z-step: U_m = P_C(Q_m + Yh_m), V_m = P_C(W - T_m Q_m + Zh_m);
    dual:   Yh_m += Q_m - U_m,  Zh_m += W - T_m Q_m - V_m.
Dual certificate: with Z_m = sigma Zh_m shifted onto sum_m Z_m = -rho,
    d(Z) = -sum_m [Tr (T_m Z_m)_+ + Tr (Z_m)_+]  <=  min  <=  Re Tr(rho W)
for any feasible W; the gap is Re Tr(rho W) - d(Z) with W's infeasibility
reported beside it.
"""
import numpy as np

MASKS = (1, 2, 3)
ZERO_TOL = 1e-8

_PT_INDEX = {}


def pt_index(mask, d=8):
    """Flat gather index of the partial transpose on `mask`."""
    if (mask, d) not in _PT_INDEX:
        idx = np.zeros((d, d), np.int64)
        for r in range(d):
            for c in range(d):
                sr = (r & ~mask) | (c & mask)
                sc = (c & ~mask) | (r & mask)
                idx[r, c] = sr * d + sc
        _PT_INDEX[(mask, d)] = idx
    return _PT_INDEX[(mask, d)]


def pt(x, mask):
    return x.reshape(-1)[pt_index(mask, x.shape[0])]


def proj_box(x):
    """Projection onto {0 <= X <= I}: eigenvalues clipped to [0, 1]."""
    w, v = np.linalg.eigh(0.5 * (x + x.conj().T))
    return (v * np.clip(w, 0.0, 1.0)) @ v.conj().T


def dual_value(rho, Z):
    shift = (sum(Z) + rho) / len(Z)
    Z = [z - shift for z in Z]
    d = 0.0
    for m, z in zip(MASKS, Z):
        for x in (pt(z, m), z):
            w = np.linalg.eigvalsh(0.5 * (x + x.conj().T))
            d -= np.sum(w[w > 0])
    return d


def infeasibility(W, Q):
    e = 0.0
    for m, q in zip(MASKS, Q):
        for x in (q, W - pt(q, m)):
            w = np.linalg.eigvalsh(0.5 * (x + x.conj().T))
            e = max(e, -w[0], w[-1] - 1.0)
    return e


def solve(rho, sigma=0.1, gap_tol=1e-9, max_iter=200000, check_every=10, state=None):
    """FP64 ADMM. Returns dict(gmn, primal, dual, gap, infeas, iters, W, Q, Z)."""
    rho = np.asarray(rho, np.complex128)
    rho = 0.5 * (rho + rho.conj().T)
    d = rho.shape[0]
    if state is None:
        U = [np.zeros((d, d), complex) for _ in MASKS]
        V = [np.zeros((d, d), complex) for _ in MASKS]
        Yh = [np.zeros((d, d), complex) for _ in MASKS]
        Zh = [np.zeros((d, d), complex) for _ in MASKS]
    else:
        U, V, Yh, Zh = (list(x) for x in state)
    it = 0
    while True:
        a = [u - y for u, y in zip(U, Yh)]
        b = [v - z for v, z in zip(V, Zh)]
        W = (sum(pt(am, m) + bm for m, am, bm in zip(MASKS, a, b)) - 2.0 * rho / sigma) / 3.0
        Q = [0.5 * (am + pt(W - bm, m)) for m, am, bm in zip(MASKS, a, b)]
        X1 = [q + y for q, y in zip(Q, Yh)]
        X2 = [W - pt(q, m) + z for m, q, z in zip(MASKS, Q, Zh)]
        U = [proj_box(x) for x in X1]
        V = [proj_box(x) for x in X2]
        Yh = [x - u for x, u in zip(X1, U)]
        Zh = [x - v for x, v in zip(X2, V)]
        it += 1
        if it % check_every == 0 or it >= max_iter:
            primal = float(np.real(np.trace(rho @ W)))
            dual = dual_value(rho, [sigma * z for z in Zh])
            gap = primal - dual
            infeas = infeasibility(W, Q)
            if (abs(gap) <= gap_tol and infeas <= gap_tol) or it >= max_iter:
                break
    value = -0.5 * (primal + dual)
    return dict(gmn=value if value > ZERO_TOL else 0.0, primal=primal, dual=dual, gap=gap, infeas=infeas, iters=it,
                W=W, Q=Q, Z=[sigma * z for z in Zh], state=(U, V, Yh, Zh))


def cut_negativities(rho):
    """Negativity (||rho^{T_m}||_1 - 1) / 2 of the three single-qubit cuts
    (partial transpose on index bit m), values in (-1e-10, 0) set to 0: the
    reference's cut_negativity (cpp/include/mipt/analysis/cut_negativity.hpp:139-200,
    qubit case); gmn.exe's prefilter is their minimum
    (cpp/src/analysis/fgmn.cpp:972-986, cpp/apps/gmn.cpp:413-424)."""
    rho = np.asarray(rho, np.complex128)
    out = np.zeros(3)
    for m in range(3):
        w = np.linalg.eigvalsh(pt(rho, 1 << m))
        n = 0.5 * (np.sum(np.abs(w)) - 1.0)
        out[m] = 0.0 if -1e-10 < n < 0.0 else n
    return out


# --------------------------------------------------------- reference states
def pure(amplitudes):
    v = np.asarray(amplitudes, complex)
    return np.outer(v, v.conj())


def ghz():
    v = np.zeros(8, complex)
    v[0] = v[7] = 1 / np.sqrt(2)
    return pure(v)


def w_state():
    v = np.zeros(8, complex)
    v[1] = v[2] = v[4] = 1 / np.sqrt(3)
    return pure(v)


def bell_ab():
    v = np.zeros(8, complex)
    v[0] = v[6] = 1 / np.sqrt(2)
    return pure(v)


def product():
    v = np.zeros(8, complex)
    v[0] = 1
    return pure(v)


def ghz_white_noise(p):
    return p * ghz() + (1 - p) * np.eye(8) / 8
