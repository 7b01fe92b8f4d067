"""Helpers for the GPU parity tests."""
import numpy as np


def random_state(n, seed):
    rng = np.random.default_rng(seed)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return psi / np.linalg.norm(psi)


def haar_layer(n, seed, start=0, closed=True):
    """Bond pairs and Haar 4x4 matrices of one brickwork layer (oracle draw)."""
    from oracle import pyoracle as orc
    d = orc.haar_draw(seed, n, 1, 0.0, closed)
    t = start
    g = d["gates_per_layer"][t]
    pairs = d["gate_q"][t, :g]
    mats = d["gate_m"][t, :g, 0::2] + 1j * d["gate_m"][t, :g, 1::2]
    return pairs, mats


def sites_of(mask, n):
    return [q for q in range(n) if (int(mask) >> q) & 1]


def mask_of(sites, values):
    m = 0
    for s, v in zip(sites, values):
        if v:
            m |= 1 << int(s)
    return m
