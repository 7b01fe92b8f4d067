"""The free-fermion (Majorana covariance) oracle against an independent
Jordan-Wigner state-vector simulation of the same circuit (small N): the
covariance, the measurement probabilities and the block entropies / TMI
(fermionic trace of the state-vector oracle) must agree."""
import numpy as np
import pytest

from oracle import pyoracle as orc

scipy_linalg = pytest.importorskip("scipy.linalg")

X = np.array([[0, 1], [1, 0]], complex)
Y = np.array([[0, -1j], [1j, 0]])
Z = np.diag([1.0, -1.0]).astype(complex)
I2 = np.eye(2, dtype=complex)


def op_on(N, ops):
    """Tensor product with qubit q = bit q of the index (qubit 0 rightmost)."""
    out = np.array([[1.0 + 0j]])
    for q in reversed(range(N)):
        out = np.kron(out, ops.get(q, I2))
    return out


def majoranas(N):
    g = []
    for j in range(N):
        string = {q: Z for q in range(j)}
        g.append(op_on(N, {**string, j: Y}))  # i g_{2j} g_{2j+1} = Z_j
        g.append(op_on(N, {**string, j: X}))
    return g


def covariance(psi, g):
    M = len(g)
    G = np.zeros((M, M))
    for a in range(M):
        for b in range(M):
            if a != b:
                G[a, b] = np.real(1j * np.vdot(psi, g[a] @ (g[b] @ psi)))
    return G


def gaussian_unitary(O, gs):
    """U with U^dag g_a U = sum_c O_ac g_c on the four Majoranas gs."""
    A = np.real(scipy_linalg.logm(O))
    H = sum(A[c, d] * gs[c] @ gs[d] for c in range(4) for d in range(4)) / 4.0
    for sign in (1.0, -1.0):
        U = scipy_linalg.expm(sign * H)
        ok = all(np.allclose(U.conj().T @ gs[a] @ U, sum(O[a, c] * gs[c] for c in range(4)), atol=1e-9)
                 for a in range(4))
        if ok:
            return U
    raise AssertionError("no Gaussian unitary found for the rotation")


@pytest.mark.parametrize("N,depth,p,seed", [(4, 6, 0.3, 1), (6, 8, 0.25, 7), (4, 4, 1.0, 3), (6, 5, 0.0, 11)])
def test_covariance_matches_state_vector(N, depth, p, seed):
    closed = False  # the ring-closing gate carries a Jordan-Wigner string on qubits
    ref = orc.ff_trajectory(seed, N, depth, p, closed, blocks=list(range(1, N + 1)))
    d = orc.ff_draw(seed, N, depth, p, closed)
    g = majoranas(N)
    psi = np.zeros(1 << N, complex)
    psi[0] = 1.0
    for t in range(depth):
        for i in range(d["gates_per_layer"][t]):
            m = d["gate_mode"][t, i]
            m2 = (m + 1) % N
            O = d["rot"][t, i].reshape(4, 4)
            U = gaussian_unitary(O, [g[2 * m], g[2 * m + 1], g[2 * m2], g[2 * m2 + 1]])
            psi = U @ psi
        for i in range(d["sites_per_layer"][t]):
            j = d["sites"][t, i]
            s = ref["outcomes"][t, i]
            P = op_on(N, {j: Z})
            p_s = np.real(np.vdot(psi, (np.eye(1 << N) + s * P) @ psi)) / 2
            assert abs(p_s - ref["probs"][t, i]) < 1e-10
            psi = (psi + s * (P @ psi)) / 2
            psi /= np.linalg.norm(psi)
    np.testing.assert_allclose(covariance(psi, g), ref["gamma"], atol=1e-10)
    # entropies of blocks [0, l): qubit and fermionic reduced states coincide
    for l, s in zip(range(1, N + 1), ref["s_blocks"]):
        rho = orc.rdm(psi, list(range(l)), fermion=True)
        assert abs(orc.entropy(rho, 1) - s) < 1e-9
    if N % 4 == 0:
        b = N // 4
        A, B, C, D = [list(range(k * b, (k + 1) * b)) for k in range(4)]
        S = lambda m: orc.entropy(orc.rdm(psi, m, fermion=True), 1)
        tmi = S(A) + S(B) + S(C) + S(D) - S(A + B) - S(A + C) - S(B + C)
        assert abs(tmi - ref["tmi"]) < 1e-9


def test_covariance_stays_pure_and_repurification_is_harmless():
    a = orc.ff_trajectory(5, 16, 40, 0.2, True)
    b = orc.ff_trajectory(5, 16, 40, 0.2, True, repurify_every=8)
    G = a["gamma"]
    np.testing.assert_allclose(G @ G, -np.eye(32), atol=1e-10)
    np.testing.assert_allclose(a["gamma"], b["gamma"], atol=1e-10)
    np.testing.assert_array_equal(a["outcomes"], b["outcomes"])
