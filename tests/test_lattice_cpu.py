"""2-D four-colour brickwork (config 3 geometry): the product's lattice bonds
and draws against the oracle's independent restatement, and both against a
literal restatement of the reference's loops (python/mipt.py:244-311) on the
square lattices where those loops are well defined. No GPU needed."""
import numpy as np
import pytest

import mipt_gb300 as mg
from oracle import pyoracle as orc


def reference_loops(s, colour):
    """python/mipt.py:244-311 for an s x s lattice (x == y == s), one colour."""
    x = y = s
    out = []
    if colour == 0 or colour == 1:
        for i in range(y):
            if i % 2 == colour:
                for j in range(0, x, 2):
                    out.append((i * x + j, i * x + j + 1))
            else:
                out.append((i * x, i * x + x - 1))
                for j in range(1, x - 1, 2):
                    out.append((i * x + j, i * x + j + 1))
    else:
        for i in range(x):
            if i % 2 == colour - 2:
                for j in range(0, y, 2):
                    out.append((j * y + i, ((j + 1) * y) % (x * y) + i))
            else:
                out.append((i, (y - 1) * y + i))
                for j in range(1, y - 1, 2):
                    out.append((j * y + i, (j + 1) * y + i))
    return out


@pytest.mark.parametrize("s", [2, 4, 6])
@pytest.mark.parametrize("colour", range(4))
def test_square_lattice_matches_reference_loops(s, colour):
    want = reference_loops(s, colour)
    assert [tuple(b) for b in mg.lattice_bonds(s, s, colour)] == want
    assert [tuple(b) for b in orc.lattice_bonds(s, s, colour)] == want


@pytest.mark.parametrize("X,Y", [(4, 7), (7, 4), (3, 4), (4, 6), (5, 5), (2, 3)])
def test_rectangular_lattices_product_equals_oracle(X, Y):
    n = X * Y
    for colour in range(4):
        a = mg.lattice_bonds(X, Y, colour)
        np.testing.assert_array_equal(a, orc.lattice_bonds(X, Y, colour))
        used = a.ravel()
        assert len(set(used.tolist())) == len(used)  # every site at most once
        for q0, q1 in a:  # nearest neighbours on the torus, in the colour's direction
            r0, c0, r1, c1 = q0 // X, q0 % X, q1 // X, q1 % X
            if colour < 2:
                assert r0 == r1 and (c1 - c0) % X in (1, X - 1)
            else:
                assert c0 == c1 and (r1 - r0) % Y in (1, Y - 1)


@pytest.mark.parametrize("X,Y,p", [(4, 7, 0.15), (3, 4, 0.3), (4, 4, 1.0)])
def test_lattice_draw_product_equals_oracle(X, Y, p):
    layers = 9
    for seed in (1, 12345):
        a = mg.draw_haar_lattice(seed, X, Y, layers, p)
        b = orc.haar_lattice_draw(seed, X, Y, layers, p)
        np.testing.assert_array_equal(a["gates_per_layer"], b["gates_per_layer"])
        for t in range(layers):
            g = a["gates_per_layer"][t]
            np.testing.assert_array_equal(a["bond_q"][t, :g], b["gate_q"][t, :g])
            np.testing.assert_allclose(a["bond_u"][t, :g], b["gate_m"][t, :g], rtol=0, atol=1e-13)
            sites = [q for q in range(X * Y) if (int(a["measured"][t]) >> q) & 1]
            assert sites == b["sites"][t, : b["sites_per_layer"][t]].tolist()
        np.testing.assert_array_equal(a["uniforms"], b["uniforms"])
