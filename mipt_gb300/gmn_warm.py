"""Learned warm start of the batched GMN solver (no reference counterpart).

A multilayer perceptron (64 -> 256 -> 256 -> 448, ReLU, BF16 weights with
FP32 accumulation) maps the 64 real parameters of a three-qubit density
matrix to the ADMM state the cold-start solver converges to: W, Q_1..3 and
the duals Z_1..3 (7 Hermitian 8x8 matrices, 64 real parameters each). The
network is trained and evaluated on the GPU by the library's own kernels
(mipt_gb300_mlp_*); the cold-start solver (mipt_gb300_gmn_solve without a
warm start) generates the training pairs and certifies every warm-started
solution, so a poor prediction costs iterations, never correctness.
"""
import ctypes

import numpy as np

from . import _check, _p, gmn_solve, lib

DIMS = (64, 256, 256, 448)
# ADMM penalty the warm start is trained and used at: the solver's scaled
# duals Z / sigma grow as 1 / sigma, and so do errors in predicted duals, so a
# warm start made at the cold-start default (0.1) is 10x less accurate.
WARM_SIGMA = 1.0
_IU = np.triu_indices(8, 1)


def features(rho):
    """[N, 8, 8] Hermitian -> [N, 64]: diagonal, Re and Im of the strict upper triangle."""
    rho = np.asarray(rho, np.complex128).reshape(-1, 8, 8)
    d = np.real(np.diagonal(rho, axis1=1, axis2=2))
    u = rho[:, _IU[0], _IU[1]]
    return np.ascontiguousarray(np.concatenate([d, u.real, u.imag], axis=1), np.float32)


def from_features(f):
    f = np.asarray(f, np.float64).reshape(-1, 64)
    m = np.zeros((len(f), 8, 8), complex)
    m[:, np.arange(8), np.arange(8)] = f[:, :8]
    u = f[:, 8:36] + 1j * f[:, 36:64]
    m[:, _IU[0], _IU[1]] = u
    m[:, _IU[1], _IU[0]] = u.conj()
    return m


def targets(solution):
    """[N, 7, 8, 8] (W, Q_1..3, Z_1..3) -> [N, 448]."""
    s = np.asarray(solution).reshape(-1, 8, 8)
    return np.ascontiguousarray(features(s).reshape(-1, 7 * 64))


def from_targets(t):
    return from_features(np.asarray(t).reshape(-1, 64)).reshape(-1, 7, 8, 8)


class MLP:
    """The GPU multilayer perceptron (C ABI mipt_gb300_mlp_*)."""

    def __init__(self, dims=DIMS, seed=0):
        L = lib()
        L.mipt_gb300_mlp_create.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p]
        L.mipt_gb300_mlp_destroy.argtypes = [ctypes.c_void_p]
        L.mipt_gb300_mlp_param_count.argtypes = [ctypes.c_void_p]
        L.mipt_gb300_mlp_param_count.restype = ctypes.c_longlong
        L.mipt_gb300_mlp_get_params.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.mipt_gb300_mlp_set_params.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.mipt_gb300_mlp_forward.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.mipt_gb300_mlp_loss_grad.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 2
        L.mipt_gb300_mlp_train.argtypes = ([ctypes.c_void_p] * 3 + [ctypes.c_int] * 3 +
                                           [ctypes.c_float, ctypes.c_uint64, ctypes.c_void_p])
        self.dims = tuple(int(d) for d in dims)
        d = np.array(self.dims, np.int32)
        h = ctypes.c_void_p()
        _check(L.mipt_gb300_mlp_create(_p(d), len(d), seed, ctypes.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            lib().mipt_gb300_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nparams(self):
        return int(lib().mipt_gb300_mlp_param_count(self._h))

    def params(self):
        out = np.zeros(self.nparams, np.float32)
        _check(lib().mipt_gb300_mlp_get_params(self._h, _p(out)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparams
        _check(lib().mipt_gb300_mlp_set_params(self._h, _p(p)))

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((len(x), self.dims[-1]), np.float32)
        _check(lib().mipt_gb300_mlp_forward(self._h, _p(x), len(x), _p(y)))
        return y

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = ctypes.c_double()
        g = np.zeros(self.nparams, np.float32)
        _check(lib().mipt_gb300_mlp_loss_grad(self._h, _p(x), _p(t), len(x), ctypes.byref(loss), _p(g)))
        return loss.value, g

    def train(self, x, t, epochs=20, batch=256, lr=1e-3, seed=0):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = ctypes.c_double()
        _check(lib().mipt_gb300_mlp_train(self._h, _p(x), _p(t), len(x), epochs, batch, lr, seed,
                                          ctypes.byref(loss)))
        return loss.value


def warm_start(mlp, rho):
    """Predicted (W, Q_1..3, Z_1..3) for each state (raw network, no scaling)."""
    return from_targets(mlp.forward(features(rho)))


class WarmStartModel:
    """The network with its input/target standardisation: trained on
    (features, solver targets) pairs standardised per dimension, predictions
    mapped back to solver state."""

    def __init__(self, seed=0, dims=DIMS):
        self.net = MLP(dims, seed)
        self.stats = None

    def fit(self, x, t, schedule=((60, 1e-3), (60, 3e-4), (60, 1e-4)), batch=512, seed=0):
        xm, xs = x.mean(0), x.std(0) + 1e-6
        tm, ts = t.mean(0), t.std(0) + 1e-6
        self.stats = (xm, xs, tm, ts)
        xn, tn = (x - xm) / xs, (t - tm) / ts
        first = self.net.loss_grad(xn[:1024], tn[:1024])[0]
        for i, (epochs, lr) in enumerate(schedule):
            self.net.train(xn, tn, epochs=epochs, batch=batch, lr=lr, seed=seed + i)
        return first, self.net.loss_grad(xn[:1024], tn[:1024])[0]

    def predict(self, rho):
        xm, xs, tm, ts = self.stats
        y = self.net.forward((features(rho) - xm) / xs)
        return from_targets(y * ts + tm)

    def save(self, path):
        xm, xs, tm, ts = self.stats
        np.savez(path, params=self.net.params(), dims=np.array(self.net.dims), xm=xm, xs=xs, tm=tm, ts=ts)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        m = cls(dims=tuple(int(v) for v in d["dims"]))
        m.net.set_params(d["params"])
        m.stats = (d["xm"], d["xs"], d["tm"], d["ts"])
        return m


class NearestSolved:
    """Warm start from the solved training state nearest to each new state (in
    the 64 real parameters of rho): the ADMM state the cold-start solver
    reached for it. A non-parametric counterpart of WarmStartModel over the
    same solver-generated pairs; the solver still certifies every result."""

    def __init__(self, x, t, chunk=4096):
        self.x = np.ascontiguousarray(x, np.float64)
        self.t = np.ascontiguousarray(t, np.float32)
        self.x2 = np.sum(self.x ** 2, axis=1)
        self.chunk = chunk

    def predict(self, rho):
        f = features(rho).astype(np.float64)
        out = np.empty((len(f), self.t.shape[1]), np.float32)
        for a in range(0, len(f), self.chunk):
            q = f[a:a + self.chunk]
            d2 = self.x2[None, :] - 2.0 * (q @ self.x.T)
            out[a:a + len(q)] = self.t[np.argmin(d2, axis=1)]
        return from_targets(out)


# ------------------------------------------------------------ config-4 data
def trajectory_states(count, seed, n=16, periods=16):
    """rho3 blocks of the final states of `count` Haar trajectories (L = n
    periodic ring, FP32 states, p uniform in [0.05, 0.35]): n blocks each,
    the trajectory half of the GMN workload."""
    from . import Batch, trajectory_seed
    rng = np.random.default_rng(seed)
    b = Batch(n, periods, capacity=count, fp64=False, rho3=True)
    seeds = np.array([trajectory_seed(seed, i) for i in range(count)], np.uint64)
    r = b.run(seeds, rng.uniform(0.05, 0.35, size=count))
    b.close()
    x = r["rho3"].reshape(-1, 128)
    return (x[:, 0::2] + 1j * x[:, 1::2]).reshape(-1, 8, 8)


def mixtures(count, seed):
    """Seeded GHZ / W / product states and random two-state mixtures of them,
    with white noise of weight U[0, 1] (the synthetic half of the GMN workload)."""
    rng = np.random.default_rng(seed)
    g = np.zeros(8, complex)
    g[0] = g[7] = 1 / np.sqrt(2)
    w = np.zeros(8, complex)
    w[1] = w[2] = w[4] = 1 / np.sqrt(3)
    base = [np.outer(g, g.conj()), np.outer(w, w.conj())]
    out = np.zeros((count, 8, 8), complex)
    for i in range(count):
        kind = rng.integers(3)
        if kind < 2:
            a = rng.uniform()
            rho = a * base[kind] + (1 - a) * base[1 - kind]
        else:
            # random product state
            v = np.ones(1, complex)
            for _ in range(3):
                q = rng.normal(size=2) + 1j * rng.normal(size=2)
                v = np.kron(q / np.linalg.norm(q), v)
            rho = np.outer(v, v.conj())
        nw = rng.uniform()
        out[i] = (1 - nw) * rho + nw * np.eye(8) / 8
    return out


def solve_pairs(rho, **kw):
    """Cold-start solutions as training targets; keeps certified states only."""
    r = gmn_solve(rho, want_solution=True, **kw)
    ok = r["iters"] > 0
    return features(rho[ok]), targets(r["solution"][ok]), r
