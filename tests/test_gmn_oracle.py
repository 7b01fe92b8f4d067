"""The FP64 GMN oracle (oracle/gmn.py) against the reference's known answers
(cpp/tests/gmn_solver_tests.cpp:83-205): GHZ 0.5, W 0.4428 (and not the
bipartite 0.4714), Bell(AB) x |0> and |000> 0, GHZ + white noise 0 at
p = 0.40 and 0.0625 at p = 0.50 (threshold 3/7). Tolerances as there."""
import numpy as np
import pytest

from oracle import gmn


@pytest.mark.parametrize("name,rho,want,tol", [
    ("GHZ", gmn.ghz(), 0.5, 1e-4),
    ("W", gmn.w_state(), 0.4428, 1e-3),
    ("Bell(AB) x |0>", gmn.bell_ab(), 0.0, 1e-4),
    ("|000>", gmn.product(), 0.0, 1e-4),
    ("GHZ+noise p=0.40", gmn.ghz_white_noise(0.40), 0.0, 1e-4),
    ("GHZ+noise p=0.50", gmn.ghz_white_noise(0.50), 0.0625, 1e-3),
])
def test_known_answers(name, rho, want, tol):
    r = gmn.solve(rho, gap_tol=1e-9)
    assert abs(r["gmn"] - want) <= tol, (name, r["gmn"])
    assert abs(r["gap"]) <= 1e-8 and r["infeas"] <= 1e-8


def test_w_is_not_the_bipartite_negativity():
    assert abs(gmn.solve(gmn.w_state())["gmn"] - 0.4714) > 0.01


def test_white_noise_closed_form():
    """GMN of p|GHZ><GHZ| + (1-p) I/8 is max(0, (7p - 3) / 8)."""
    for p in (0.3, 0.45, 0.6, 0.8, 1.0):
        assert abs(gmn.solve(gmn.ghz_white_noise(p), gap_tol=1e-10)["gmn"] - max(0.0, (7 * p - 3) / 8)) < 1e-7


def test_dual_bound_and_partial_transpose():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
    for m in (1, 2, 3):
        assert np.allclose(gmn.pt(gmn.pt(x, m), m), x)  # involution
        y = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
        assert np.isclose(np.trace(gmn.pt(x, m) @ y.conj().T), np.trace(x @ gmn.pt(y, m).conj().T))  # self-adjoint
    rho = gmn.ghz_white_noise(0.7)
    r = gmn.solve(rho, gap_tol=1e-10)
    # the certificate is a lower bound of the optimum for any dual point
    assert gmn.dual_value(rho, [0.5 * z for z in r["Z"]] ) <= r["primal"] + 1e-12
