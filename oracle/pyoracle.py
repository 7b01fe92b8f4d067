"""ctypes binding for the CPU FP64 oracle (oracle/oracle.cpp).

Test infrastructure: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline and reference legs, always as the checker or as the
timed CPU baseline.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build():
    subprocess.check_call([os.path.join(HERE, "build_oracle.sh")])


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = ctypes.CDLL(LIB_PATH)
    vp, ci, cd, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint64
    L.orc_splitmix64.restype = u64
    L.orc_splitmix64.argtypes = [u64]
    L.orc_trajectory_seed.restype = u64
    L.orc_trajectory_seed.argtypes = [u64, u64]
    L.orc_haar_draw.argtypes = [u64, ci, ci, cd, ci, ci] + [vp] * 7
    L.orc_apply_bond.argtypes = [vp, ci, ci, ci, vp]
    L.orc_measure_layer.argtypes = [vp, ci, vp, ci, ci, vp, vp, vp, vp]
    L.orc_measure_collapse.argtypes = [vp, ci, ci, cd, vp, vp]
    L.orc_rdm.argtypes = [vp, ci, vp, ci, ci, vp]
    L.orc_entropy_hermitian.restype = cd
    L.orc_entropy_hermitian.argtypes = [vp, ci, ci]
    L.orc_eigvalsh.argtypes = [vp, ci, vp]
    L.orc_tmi.restype = cd
    L.orc_tmi.argtypes = [vp, ci, ci, ci]
    L.orc_rho3.argtypes = [vp, ci, vp, ci, ci, vp]
    L.orc_run_haar_trajectory.argtypes = [u64, ci, ci, cd, ci, ci, ci, ci, vp, vp, vp, vp, vp]
    L.orc_run_batch.argtypes = [u64, ci, ci, ci, ci, cd, ci, ci, ci, vp, vp, ci]
    L.orc_max_threads.restype = ci
    L.orc_fe_initial_state.argtypes = [u64, ci, ci, ci, ci, vp, vp]
    L.orc_fe_draw.argtypes = [ctypes.c_uint32, ci, ci, cd, ci] + [vp] * 7
    L.orc_fe_trajectory.argtypes = [u64, ci, cd, ci, ci, ci, ci, ci, vp, vp, vp, vp]
    L.orc_fe_batch.argtypes = [u64, ci, ci, ci, cd, ci, ci, vp, ci]
    L.orc_rppu_draw.argtypes = [u64, ci, ci, cd, ci, ci] + [vp] * 5
    L.orc_fe_trajectory_circuit.argtypes = [u64, ci, cd, ci, ci, ci, ci, ci, ci, vp, vp, vp, vp]
    L.orc_run_rppu_trajectory.argtypes = [u64, ci, ci, cd, ci, ci, ci, vp, vp, vp]
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data


def trajectory_seed(master, index):
    return lib().orc_trajectory_seed(master, index)


def haar_draw(seed, n, periods, p, closed=True, chunk_bits=16):
    """Returns dict(gates_per_layer, gate_q, gate_m[complex L x n/2 x 4 x 4],
    sites_per_layer, sites, uniforms)."""
    L, mg = 2 * periods, n // 2
    gpl = np.zeros(L, np.int32)
    gq = np.zeros((L, mg, 2), np.int32)
    gm = np.zeros((L, mg, 32))
    spl = np.zeros(L, np.int32)
    sites = np.full((L, n), -1, np.int32)
    uni = np.zeros(L * n + 1)
    nu = np.zeros(1, np.int32)
    rc = lib().orc_haar_draw(seed, n, periods, p, int(closed), chunk_bits,
                             *[_p(a) for a in (gpl, gq, gm, spl, sites, uni, nu)])
    if rc:
        raise RuntimeError("orc_haar_draw failed")
    return dict(gates_per_layer=gpl, gate_q=gq, gate_m=gm, sites_per_layer=spl, sites=sites,
                uniforms=uni[: nu[0]].copy())


def measure_collapse(psi, q, u):
    psi = np.ascontiguousarray(psi, np.complex128).copy()
    n = int(np.log2(psi.size))
    oc = np.zeros(1, np.int32)
    cp = np.zeros(1)
    if lib().orc_measure_collapse(_p(psi), n, q, u, _p(oc), _p(cp)):
        raise RuntimeError("orc_measure_collapse failed")
    return psi, int(oc[0]), float(cp[0])


def rdm(psi, kept, fermion=False):
    psi = np.ascontiguousarray(psi, np.complex128)
    n = int(np.log2(psi.size))
    kk = np.ascontiguousarray(kept, np.int32)
    d = 1 << len(kept)
    rho = np.zeros((d, d), np.complex128)
    if lib().orc_rdm(_p(psi), n, _p(kk), len(kept), int(fermion), _p(rho)):
        raise RuntimeError("orc_rdm failed")
    return rho


def entropy(rho, order=1):
    rho = np.ascontiguousarray(rho, np.complex128)
    return lib().orc_entropy_hermitian(_p(rho), rho.shape[0], order)


def eigvalsh(rho):
    rho = np.ascontiguousarray(rho, np.complex128)
    w = np.zeros(rho.shape[0])
    lib().orc_eigvalsh(_p(rho), rho.shape[0], _p(w))
    return w


def tmi(psi, offset=0, order=1):
    psi = np.ascontiguousarray(psi, np.complex128)
    return lib().orc_tmi(_p(psi), int(np.log2(psi.size)), offset, order)


def rho3(psi, subs, fermion=False):
    psi = np.ascontiguousarray(psi, np.complex128)
    subs = np.ascontiguousarray(subs, np.int32)
    out = np.zeros(128 * len(subs))
    if lib().orc_rho3(_p(psi), int(np.log2(psi.size)), _p(subs), len(subs), int(fermion), _p(out)):
        raise RuntimeError("orc_rho3 failed")
    return out


def apply_bond(psi, q0, q1, U):
    psi = np.ascontiguousarray(psi, np.complex128).copy()
    U = np.ascontiguousarray(U, np.complex128)
    lib().orc_apply_bond(_p(psi), int(np.log2(psi.size)), q0, q1, _p(U))
    return psi


def measure_layer(psi, sites, uniforms, chunk_bits=16, forced=None):
    psi = np.ascontiguousarray(psi, np.complex128).copy()
    s = np.ascontiguousarray(sites, np.int32)
    u = np.ascontiguousarray(uniforms, np.float64)
    f = None if forced is None else np.ascontiguousarray(forced, np.int32)
    oc = np.zeros(max(1, len(sites)), np.int32)
    sp = np.zeros(1)
    if lib().orc_measure_layer(_p(psi), int(np.log2(psi.size)), _p(s), len(sites), chunk_bits, _p(u), _p(f),
                               _p(oc), _p(sp)):
        raise RuntimeError("orc_measure_layer failed")
    return psi, oc[: len(sites)].copy(), float(sp[0])


OBS_SVN, OBS_S2, OBS_TMI1, OBS_TMI2 = 1, 2, 4, 8


def run_trajectory(seed, n, periods, p, closed=True, chunk_bits=16, obs_flags=0, observe_every=0,
                   forced=None, want_state=False):
    T = 2 * periods
    outcomes = np.full((T, n), -1, np.int32)
    surprisal = np.zeros(T)
    obs = np.full((T, 4), np.nan)
    f = None if forced is None else np.ascontiguousarray(forced, np.int32)
    psi = np.zeros(1 << n, np.complex128) if want_state else None
    rc = lib().orc_run_haar_trajectory(seed, n, periods, p, int(closed), chunk_bits, obs_flags, observe_every,
                                       _p(f), _p(outcomes), _p(surprisal), _p(obs), _p(psi))
    if rc:
        raise RuntimeError("orc_run_haar_trajectory failed")
    return dict(outcomes=outcomes, surprisal=surprisal, obs=obs, psi=psi)


def run_batch(master, first, count, n, periods, p, closed=True, chunk_bits=16, obs_flags=OBS_S2, threads=0):
    s2 = np.zeros(count)
    sp = np.zeros(count)
    if lib().orc_run_batch(master, first, count, n, periods, p, int(closed), chunk_bits, obs_flags, _p(s2), _p(sp),
                           threads):
        raise RuntimeError("orc_run_batch failed")
    return s2, sp


def max_threads():
    return lib().orc_max_threads()


# ------------------------------------------------------------ free fermions
def _ff_bind():
    L = lib()
    if getattr(L, "_ff_bound", False):
        return L
    vp, ci, cd, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint64
    L.orc_ff_trajectory.argtypes = [u64, ci, ci, cd, ci, ci, vp, vp, vp, vp, vp, ci, vp, vp]
    L.orc_ff_draw.argtypes = [u64, ci, ci, cd, ci, vp, vp, vp, vp, vp, vp]
    L.orc_ff_block_entropy.restype = cd
    L.orc_ff_block_entropy.argtypes = [vp, ci, vp, ci]
    L._ff_bound = True
    return L


def ff_trajectory(seed, N, depth, p, closed=True, repurify_every=0, forced=None, blocks=(), want_gamma=True):
    L = _ff_bind()
    outcomes = np.zeros((depth, N), np.int32)
    probs = np.zeros((depth, N))
    gamma = np.zeros((2 * N, 2 * N)) if want_gamma else None
    bl = np.ascontiguousarray(blocks, np.int32)
    sb = np.zeros(max(1, len(bl)))
    tmi = np.zeros(1)
    f = None if forced is None else np.ascontiguousarray(forced, np.int32)
    if L.orc_ff_trajectory(seed, N, depth, p, int(closed), repurify_every, _p(f), _p(outcomes), _p(probs),
                           _p(gamma), _p(bl), len(bl), _p(sb), _p(tmi) if N % 4 == 0 else None):
        raise RuntimeError("orc_ff_trajectory failed")
    return dict(outcomes=outcomes, probs=probs, gamma=gamma, s_blocks=sb[: len(bl)], tmi=float(tmi[0]))


def ff_draw(seed, N, depth, p, closed=True):
    L = _ff_bind()
    mg = N // 2 + 1
    gpl = np.zeros(depth, np.int32)
    gm = np.zeros((depth, mg), np.int32)
    rot = np.zeros((depth, mg, 16))
    spl = np.zeros(depth, np.int32)
    sites = np.full((depth, N), -1, np.int32)
    uni = np.zeros(depth * N + 1)
    if L.orc_ff_draw(seed, N, depth, p, int(closed), _p(gpl), _p(gm), _p(rot), _p(spl), _p(sites), _p(uni)):
        raise RuntimeError("orc_ff_draw failed")
    return dict(gates_per_layer=gpl, gate_mode=gm, rot=rot, sites_per_layer=spl, sites=sites, uniforms=uni)


def ff_block_entropy(gamma, modes):
    L = _ff_bind()
    g = np.ascontiguousarray(gamma, np.float64)
    m = np.ascontiguousarray(modes, np.int32)
    return L.orc_ff_block_entropy(_p(g), g.shape[0] // 2, _p(m), len(m))


# ------------------------------------------------------------ 2-D lattices
def _lattice_bind():
    L = lib()
    if getattr(L, "_lattice_bound", False):
        return L
    vp, ci, cd, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint64
    L.orc_lattice_bonds.argtypes = [ci, ci, ci, vp]
    L.orc_lattice_bonds.restype = ci
    L.orc_haar_lattice_draw.argtypes = [u64, ci, ci, ci, cd, ci, vp, vp, vp, vp, vp, vp, vp]
    L.orc_haar_lattice_draw.restype = ci
    L.orc_run_lattice_trajectory.argtypes = [u64, ci, ci, ci, cd, ci, vp, vp, vp, ci, vp, vp]
    L.orc_run_lattice_trajectory.restype = ci
    L._lattice_bound = True
    return L


def lattice_bonds(X, Y, colour):
    L = _lattice_bind()
    pairs = np.zeros(X * Y, np.int32)
    c = L.orc_lattice_bonds(X, Y, colour, _p(pairs))
    return pairs[: 2 * c].reshape(-1, 2)


def haar_lattice_draw(seed, X, Y, layers, p, chunk_bits=16):
    L = _lattice_bind()
    n, mg = X * Y, (X * Y) // 2
    gpl = np.zeros(layers, np.int32)
    gq = np.zeros((layers, mg, 2), np.int32)
    gm = np.zeros((layers, mg, 32))
    spl = np.zeros(layers, np.int32)
    sites = np.full((layers, n), -1, np.int32)
    uni = np.zeros(layers * n)
    nu = np.zeros(1, np.int32)
    if L.orc_haar_lattice_draw(seed, X, Y, layers, p, chunk_bits, _p(gpl), _p(gq), _p(gm), _p(spl), _p(sites),
                               _p(uni), _p(nu)):
        raise RuntimeError("orc_haar_lattice_draw failed")
    return dict(gates_per_layer=gpl, gate_q=gq, gate_m=gm, sites_per_layer=spl, sites=sites,
                uniforms=uni[: int(nu[0])])


def run_lattice_trajectory(seed, X, Y, layers, p, chunk_bits=16, forced=None, observe_every=0):
    L = _lattice_bind()
    n = X * Y
    outcomes = np.full((layers, n), -1, np.int32)
    surprisal = np.zeros(layers)
    points = layers // observe_every if observe_every > 0 else 0
    states = np.zeros((max(points, 1), 1 << n), np.complex128)
    psi = np.zeros(1 << n, np.complex128)
    f = None if forced is None else np.ascontiguousarray(forced, np.int32)
    if L.orc_run_lattice_trajectory(seed, X, Y, layers, p, chunk_bits, _p(f), _p(outcomes), _p(surprisal),
                                    observe_every, _p(states) if points else None, _p(psi)):
        raise RuntimeError("orc_run_lattice_trajectory failed")
    return dict(outcomes=outcomes, surprisal=surprisal, states=states[:points], psi=psi)


# ------------------------------------------------------------ free energy
FE_CIRCUIT_SALT = 0x4349524355495455
FE_INITIAL_SALT = 0x494E495449414C53


def fe_trajectory_seed(master, index):
    """trajectory_seed = splitmix64(master ^ index) (the free-energy stream)."""
    return lib().orc_splitmix64((master ^ index) & 0xFFFFFFFFFFFFFFFF)


def fe_workspace_seed(trajectory_seed):
    return lib().orc_splitmix64(trajectory_seed ^ FE_CIRCUIT_SALT) & 0xFFFFFFFF


def fe_initial_seed(trajectory_seed):
    return lib().orc_splitmix64(trajectory_seed ^ FE_INITIAL_SALT)


def fe_initial_state(seed, n, kind, fixed_parity=False, fp32=False):
    ri = np.zeros(2 << n)
    par = np.zeros(1, np.int32)
    if lib().orc_fe_initial_state(seed, n, kind, int(fixed_parity), int(fp32), _p(ri), _p(par)):
        raise RuntimeError("orc_fe_initial_state failed")
    return ri.view(np.complex128), int(par[0])


def fe_draw(seed32, n, layers, p, chunk_bits=16):
    mg = n // 2
    gpl = np.zeros(layers, np.int32)
    gq = np.zeros((layers, mg, 2), np.int32)
    gm = np.zeros((layers, mg, 32))
    spl = np.zeros(layers, np.int32)
    sites = np.full((layers, n), -1, np.int32)
    uni = np.zeros(layers * n + 1)
    nu = np.zeros(1, np.int32)
    if lib().orc_fe_draw(seed32, n, layers, p, chunk_bits, *[_p(a) for a in (gpl, gq, gm, spl, sites, uni, nu)]):
        raise RuntimeError("orc_fe_draw failed")
    return dict(gates_per_layer=gpl, gate_q=gq, gate_m=gm, sites_per_layer=spl, sites=sites,
                uniforms=uni[: nu[0]].copy())


def fe_trajectory(trajectory_seed, n, p, init_kind, fp32_init=False, chunk_bits=16, entropy_max_t=None,
                  entropy_stride=1, circuit=1):
    """One free-energy trajectory (28n timesteps) of gate set `circuit` (1 Haar,
    2 FermionRPPU, 4 qRPPU): surprisal[T], measured counts[T], half-chain S1
    bits [T+1] (NaN where not sampled), parity sector."""
    T = 28 * n
    if entropy_max_t is None:
        entropy_max_t = 2 * n
    sp = np.zeros(T)
    mc = np.zeros(T, np.int32)
    sh = np.zeros(T + 1)
    par = np.zeros(1, np.int32)
    if lib().orc_fe_trajectory_circuit(trajectory_seed, n, p, circuit, init_kind, int(fp32_init), chunk_bits,
                                       entropy_max_t, entropy_stride, _p(sp), _p(mc), _p(sh), _p(par)):
        raise RuntimeError("orc_fe_trajectory failed")
    return dict(surprisal=sp, measured=mc, s_half=sh, parity=int(par[0]))


def fe_batch(master, first, count, n, p, init_kind, chunk_bits=16, threads=0):
    """F_total of trajectories first..first+count-1 on host threads (CPU baseline)."""
    out = np.zeros(count)
    if lib().orc_fe_batch(master, first, count, n, p, init_kind, chunk_bits, _p(out), threads):
        raise RuntimeError("orc_fe_batch failed")
    return out


# ------------------------------------------------------------ RPPU / qRPPU
RPPU_FSWAP, RPPU_JW, RPPU_QUBIT = 0, 1, 2


def rppu_draw(seed, n, periods, p, boundary, workspace=False):
    """Ops of each layer in application order: (kinds[k], q0[k], q1[k],
    matrices[k] 4x4 complex), ops per layer, sites per layer, sites."""
    T = periods if workspace else 2 * periods + 1
    oc = np.zeros(T, np.int32)
    meta = np.zeros((T * 4 * n, 3), np.int32)
    m = np.zeros((T * 4 * n, 32))
    spl = np.zeros(T, np.int32)
    sites = np.full((T, n), -1, np.int32)
    t = lib().orc_rppu_draw(seed, n, periods, p, boundary, int(workspace), _p(oc), _p(meta), _p(m), _p(spl),
                            _p(sites))
    if t < 0:
        raise RuntimeError("orc_rppu_draw failed")
    k = int(oc[:t].sum())
    return dict(layers=t, ops_per_layer=oc[:t], meta=meta[:k], m=m[:k], sites_per_layer=spl[:t], sites=sites[:t])


def run_rppu_trajectory(seed, n, periods, p, boundary, encoded=True, chunk_bits=16):
    """One RPPU trajectory from |0...0> on the Circuit1D streams."""
    T = 2 * periods + 1
    sp = np.zeros(T)
    oc = np.full((T, n), -1, np.int32)
    psi = np.zeros(1 << n, np.complex128)
    t = lib().orc_run_rppu_trajectory(seed, n, periods, p, boundary, int(encoded), chunk_bits, _p(sp), _p(oc),
                                      _p(psi))
    if t < 0:
        raise RuntimeError("orc_run_rppu_trajectory failed")
    return dict(layers=t, surprisal=sp[:t], outcomes=oc[:t], psi=psi)
