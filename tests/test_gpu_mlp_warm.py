"""The learned warm start of the GMN solver: the GPU perceptron's gradients
against the FP64 CPU reference (oracle/mlp.py, same BF16-rounded weights),
training on solver-generated pairs, and what the trained network gains over
the cold start: ADMM iterations to a certified duality gap of 1e-6 on held-out
states, with the same GMN values.

Tolerances: loss 1e-4 relative, gradients 1e-3 relative to the largest
entry of each layer block (FP32 accumulation), GMN 2e-6."""
import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg():
    from mipt_gb300 import build
    build.build()
    import mipt_gb300
    return mipt_gb300


@pytest.mark.parametrize("dims", [(64, 32, 48, 20), (64, 256, 256, 448)])
def test_gradients_match_cpu_reference(mg, dims):
    from mipt_gb300 import gmn_warm
    net = gmn_warm.MLP(dims, seed=3)
    rng = np.random.default_rng(5)
    p = net.params()
    p[:] = rng.normal(scale=0.2, size=p.size).astype(np.float32)
    net.set_params(p)
    x = rng.normal(size=(37, dims[0])).astype(np.float32)
    t = rng.normal(size=(37, dims[-1])).astype(np.float32)
    loss, g = net.loss_grad(x, t)
    want_loss, want_g = omlp.loss_grad(p, dims, x, t)
    assert abs(loss - want_loss) <= 1e-4 * abs(want_loss)
    o = 0
    for i in range(len(dims) - 1):
        for n in (dims[i] * dims[i + 1], dims[i + 1]):
            a, b = g[o:o + n], want_g[o:o + n]
            assert np.max(np.abs(a - b)) <= 1e-3 * np.max(np.abs(b)) + 1e-7, (i, n)
            o += n
    # forward agrees with the reference's output too
    y = net.forward(x)
    layers = omlp.unpack(p, dims)
    h = x.astype(np.float64)
    for li, (W, b) in enumerate(layers):
        h = h @ omlp.bf16(W).T + b
        if li + 1 < len(layers):
            h = np.maximum(h, 0)
    np.testing.assert_allclose(y, h, rtol=0, atol=1e-4 * np.max(np.abs(h)))


def test_warm_start_on_held_out_states(mg):
    """Train on solver-generated pairs from trajectory rho3 blocks and GHZ/W/
    product mixtures, then warm-start held-out states of each class.

    Checked for both warm starts (the network's prediction, and the solved
    training state nearest to each new state): every warm-started state that
    certifies has the cold-start GMN value (2e-6). The nearest solved state
    must keep the certified fraction (within 0.02) and gain at least 1.5x in
    iterations on held-out mixtures (about 2x measured). The network's
    predictions are too coarse for this ADMM (its duals need about 0.3 %
    accuracy to pay off): it costs iterations (about 0.5-0.6x measured) and
    some certifications within the iteration limit, so those are reported,
    not asserted."""
    from mipt_gb300 import gmn_warm
    sigma = gmn_warm.WARM_SIGMA
    train = np.concatenate([gmn_warm.trajectory_states(256, 21), gmn_warm.mixtures(20000, 1)])
    held = {"trajectory": gmn_warm.trajectory_states(24, 22), "mixture": gmn_warm.mixtures(400, 2)}
    x, t, _ = gmn_warm.solve_pairs(train, gap_tol=1e-6, max_iter=3000, sigma=sigma)
    assert len(x) > 0.8 * len(train)
    model = gmn_warm.WarmStartModel(seed=0)
    first, last = model.fit(x, t)
    assert last < 0.25 * first, (first, last)
    nearest = gmn_warm.NearestSolved(x, t)
    kw = dict(gap_tol=1e-6, max_iter=3000, check_every=5, sigma=sigma)
    gains = {}
    for cls, rho in held.items():
        cold = mg.gmn_solve(rho, **kw)
        for name, guess in (("network", model.predict(rho)), ("nearest", nearest.predict(rho))):
            warm = mg.gmn_solve(rho, warm_start=guess, **kw)
            c_ok, w_ok = cold["iters"] > 0, warm["iters"] > 0
            ok = c_ok & w_ok
            gain = cold["iters"][ok].mean() / warm["iters"][ok].mean()
            gains[(cls, name)] = gain
            print(f"{cls:10s} {name:8s} certified cold {c_ok.mean():.3f} warm {w_ok.mean():.3f}; iterations "
                  f"{cold['iters'][ok].mean():.1f} -> {warm['iters'][ok].mean():.1f} (x{gain:.2f}, {ok.sum()} states)")
            if name == "nearest":
                assert w_ok.mean() >= c_ok.mean() - 0.02, (cls, name)
            np.testing.assert_allclose(warm["gmn"][ok], cold["gmn"][ok], rtol=0, atol=2e-6)
    assert gains[("mixture", "nearest")] >= 1.5, gains
