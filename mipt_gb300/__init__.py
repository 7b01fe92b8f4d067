"""GB300-native monitored-circuit trajectory path (Python host side).

Everything here calls the C ABI of ``mipt_gb300/_build/libmipt_gb300.so``
(declared in ``include/mipt_gb300.h``) through ctypes. There is no CPU or
eager fallback: if the library is missing, importing the bindings raises.

The functions mirror the reference's operator interface for this path
(cpp/include/mipt/cuda/*.hpp and the cuStateVec Engine of
cpp/include/mipt/cusv/engine.hpp in the reference project): same names,
argument meaning and error behaviour (nonzero status -> exception carrying
the library's message).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmipt_gb300.so")

OBS_SVN_HALF, OBS_S2_HALF, OBS_TMI_VN, OBS_TMI_S2 = 1, 2, 4, 8

_lib = None


class MiptError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"mipt_gb300 status {status}: {message}")
        self.status = status


class FFConfig(ctypes.Structure):
    _fields_ = [("n_modes", ctypes.c_int), ("depth", ctypes.c_int), ("closed", ctypes.c_int),
                ("repurify_every", ctypes.c_int), ("n_blocks", ctypes.c_int),
                ("block_len", ctypes.POINTER(ctypes.c_int)), ("host_threads", ctypes.c_int), ("fp64", ctypes.c_int)]


class BatchConfig(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int) for name in (
        "n_qubits", "periods", "closed", "fp64", "chunk_bits", "observables", "observe_every", "rho3",
        "fermion_trace", "host_threads", "tile_qubits", "tmi_cycles", "lattice_x", "lattice_y", "circuit",
        "split_last", "full_state")]


def lib():
    """Load the compiled library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m mipt_gb300.build`")
    L = ctypes.CDLL(LIB_PATH)
    vp, ci, cd, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint64
    L.mipt_gb300_last_error.restype = ctypes.c_char_p
    L.mipt_gb300_version.restype = ctypes.c_char_p
    L.mipt_cuda_measure_collapse_last_error.restype = ctypes.c_char_p
    for name in ("mipt_cuda_rdm_subsystem", "mipt_cuda_entropy_svd", "mipt_cuda_renyi2"):
        for suffix in ("_f32", "_f64"):
            getattr(L, name + suffix).argtypes = [vp, ci, vp, ci, ci, vp]
    for mid in ("", "fermion_"):
        for suffix in ("f32", "f64"):
            getattr(L, f"mipt_cuda_rho3_subsystems_complex_{mid}{suffix}").argtypes = [vp, ci, vp, ci, vp]
    for suffix in ("f32", "f64"):
        getattr(L, f"mipt_cuda_rho3_subsystems_complex_both_{suffix}").argtypes = [vp, ci, vp, ci, vp, vp]
        getattr(L, f"mipt_cuda_measure_collapse_{suffix}").argtypes = [vp, ci, ci, cd, vp, vp]
    L.mipt_gb300_engine_create.argtypes = [ci, ctypes.POINTER(vp)]
    L.mipt_gb300_engine_destroy.argtypes = [vp]
    L.mipt_gb300_engine_destroy.restype = None
    L.mipt_gb300_engine_reset.argtypes = [vp, ci]
    L.mipt_gb300_engine_adopt.argtypes = [vp, vp, ci]
    L.mipt_gb300_engine_data.argtypes = [vp]
    L.mipt_gb300_engine_data.restype = vp
    L.mipt_gb300_engine_set_from_host.argtypes = [vp, vp, ci]
    L.mipt_gb300_engine_to_host.argtypes = [vp, vp]
    L.mipt_gb300_engine_apply_bonds.argtypes = [vp, vp, ci, vp]
    L.mipt_gb300_engine_measure_layer.argtypes = [vp, vp, ci, ci, vp, vp, vp, vp]
    L.mipt_gb300_batch_create.argtypes = [ctypes.POINTER(BatchConfig), ci, ctypes.POINTER(vp)]
    L.mipt_gb300_batch_destroy.argtypes = [vp]
    L.mipt_gb300_batch_destroy.restype = None
    L.mipt_gb300_batch_prepare_haar.argtypes = [vp, vp, vp, ci, vp]
    L.mipt_gb300_batch_prepare_haar_workspace.argtypes = [vp, vp, vp, ci]
    L.mipt_gb300_batch_set_initial_states.argtypes = [vp, vp, ci, ci, ci, vp]
    L.mipt_gb300_batch_set_initial_state.argtypes = [vp, ci, vp]
    L.mipt_gb300_batch_set_observation_steps.argtypes = [vp, vp, ci]
    L.mipt_gb300_draw_initial_state.argtypes = [u64, ci, ci, ci, ci, vp, vp]
    L.mipt_gb300_draw_haar_workspace.argtypes = [ctypes.c_uint32, ci, ci, cd, ci, vp, vp, vp, vp, vp, vp]
    L.mipt_gb300_draw_rppu.argtypes = [u64, ci, ci, cd, ci, ci, ci, vp, vp, vp, vp, vp, vp]
    L.mipt_gb300_batch_execute.argtypes = [vp, vp]
    L.mipt_gb300_batch_fetch.argtypes = [vp, vp, vp, vp, vp, vp]
    L.mipt_gb300_batch_fetch_tmi.argtypes = [vp, ci, vp]
    L.mipt_gb300_batch_add_region.argtypes = [vp, vp, ci, ci, vp]
    L.mipt_gb300_batch_fetch_regions.argtypes = [vp, vp]
    L.mipt_gb300_batch_set_rho3_subsystems.argtypes = [vp, vp, ci]
    L.mipt_gb300_batch_rho3_subsystem_count.argtypes = [vp]
    L.mipt_gb300_batch_fetch_rho3_points.argtypes = [vp, vp]
    L.mipt_gb300_lattice_bonds.argtypes = [ci, ci, ci, vp, vp]
    L.mipt_gb300_gmn_solve.argtypes = [vp, vp, ci, vp, vp, vp, vp, vp]
    L.mipt_gb300_gmn_solve_sigma.argtypes = [vp, vp, ci, vp, vp, vp, vp, vp, vp]
    L.mipt_gb300_cut_negativities.argtypes = [vp, ci, vp]
    L.mipt_gb300_autotune_tile.argtypes = [ci, ci, ci, ci, ci, ci, vp, vp, vp, vp]
    L.mipt_gb300_draw_haar_lattice.argtypes = [u64, ci, ci, ci, cd, ci, vp, vp, vp, vp, vp, vp]
    L.mipt_gb300_batch_run_haar.argtypes = [vp, vp, vp, ci, vp, vp, vp, vp, vp, vp]
    L.mipt_gb300_batch_state.argtypes = [vp, ci]
    L.mipt_gb300_batch_state.restype = vp
    L.mipt_gb300_batch_launches.argtypes = [vp]
    L.mipt_gb300_batch_parity_encoded.argtypes = [vp]
    L.mipt_gb300_batch_launches.restype = ctypes.c_longlong
    L.mipt_gb300_batch_set_profiling.argtypes = [vp, ci]
    L.mipt_gb300_batch_kernel_stats.argtypes = [vp, vp, vp]
    L.mipt_gb300_splitmix64.argtypes = [u64]
    L.mipt_gb300_splitmix64.restype = u64
    L.mipt_gb300_trajectory_seed.argtypes = [u64, u64]
    L.mipt_gb300_trajectory_seed.restype = u64
    L.mipt_gb300_draw_haar.argtypes = [u64, ci, ci, cd, ci, ci, vp, vp, vp, vp, vp, vp]
    L.mipt_gb300_ff_run.argtypes = [ctypes.POINTER(FFConfig), vp, vp, ci, vp, vp, vp, vp, vp, vp]
    L.mipt_gb300_batch_execute_graph.argtypes = [vp, vp]
    L.mipt_gb300_batch_group_create.argtypes = [vp, ci, ctypes.POINTER(vp)]
    L.mipt_gb300_batch_group_execute.argtypes = [vp, vp]
    L.mipt_gb300_batch_group_destroy.argtypes = [vp]
    L.mipt_gb300_batch_group_destroy.restype = None
    L.mipt_gb300_test_withhold_tile_loads.argtypes = [ci]
    _lib = L
    return L


def _check(status):
    if status != 0:
        raise MiptError(status, lib().mipt_gb300_last_error().decode(errors="replace"))


def _p(a):
    return None if a is None else a.ctypes.data


def _dtype_suffix(fp64):
    return "f64" if fp64 else "f32"


# ----------------------------------------------------------------- seeding
def splitmix64(v):
    return lib().mipt_gb300_splitmix64(v)


def trajectory_seed(master, index):
    return lib().mipt_gb300_trajectory_seed(master, index)


def draw_initial_state(seed, n, kind, fixed_parity=False, fp64=True):
    """The free-energy protocol's random initial state (complex amplitudes, parity sector)."""
    ri = np.zeros(2 << n)
    par = ctypes.c_int()
    _check(lib().mipt_gb300_draw_initial_state(seed, n, int(kind), int(fixed_parity), int(fp64), _p(ri),
                                               ctypes.byref(par)))
    return ri.view(np.complex128), par.value


def draw_haar(seed, n, periods, p, closed=True, chunk_bits=16):
    """Host draw of one Haar trajectory (no GPU): the reference's random record."""
    L = 2 * periods
    gpl = np.zeros(L, np.int32)
    bq = np.zeros((L, n // 2, 2), np.int32)
    bu = np.zeros((L, n // 2, 32))
    meas = np.zeros(L, np.uint64)
    uni = np.zeros(L * n + 1)
    nu = np.zeros(1, np.int32)
    _check(lib().mipt_gb300_draw_haar(seed, n, periods, p, int(closed), chunk_bits, _p(gpl), _p(bq), _p(bu),
                                      _p(meas), _p(uni), _p(nu)))
    return dict(gates_per_layer=gpl, bond_q=bq, bond_u=bu, measured=meas, uniforms=uni[: nu[0]].copy())


def draw_haar_workspace(seed32, n, layers, p, chunk_bits=16):
    """Host draw of one free-energy trajectory's layers (probed-workspace streams)."""
    gpl = np.zeros(layers, np.int32)
    bq = np.zeros((layers, n // 2, 2), np.int32)
    bu = np.zeros((layers, n // 2, 32))
    meas = np.zeros(layers, np.uint64)
    uni = np.zeros(layers * n + 1)
    nu = np.zeros(1, np.int32)
    _check(lib().mipt_gb300_draw_haar_workspace(seed32, n, layers, p, chunk_bits, _p(gpl), _p(bq), _p(bu),
                                                _p(meas), _p(uni), _p(nu)))
    return dict(gates_per_layer=gpl, bond_q=bq, bond_u=bu, measured=meas, uniforms=uni[: nu[0]].copy())


def draw_rppu(seed, n, periods, p, chunk_bits=16, split_last=True, workspace=False):
    """Host draw of one RPPU / qRPPU trajectory as the batch runs it (2*periods + 1 layers)."""
    L = 2 * periods + 1
    gpl = np.zeros(L, np.int32)
    bq = np.zeros((L, n // 2, 2), np.int32)
    bu = np.zeros((L, n // 2, 32))
    meas = np.zeros(L, np.uint64)
    uni = np.zeros(L * n + L)
    nu = np.zeros(1, np.int32)
    _check(lib().mipt_gb300_draw_rppu(seed, n, periods, p, chunk_bits, int(split_last), int(workspace), _p(gpl),
                                      _p(bq), _p(bu), _p(meas), _p(uni), _p(nu)))
    return dict(gates_per_layer=gpl, bond_q=bq, bond_u=bu, measured=meas, uniforms=uni[: nu[0]].copy())


# -------------------------------------------------- reference-compatible ops
def rdm_subsystem(state_ptr, n, kept, fermion_trace=False, fp64=True):
    """mipt_cuda_rdm_subsystem_*: RDM of `kept` from a device state pointer."""
    kept = np.ascontiguousarray(kept, np.int32)
    d = 1 << len(kept)
    out = np.zeros((d, d), np.complex128)
    fn = getattr(lib(), "mipt_cuda_rdm_subsystem_" + _dtype_suffix(fp64))
    _check(fn(state_ptr, n, _p(kept), len(kept), int(fermion_trace), _p(out)))
    return out


def entropy_svd(state_ptr, n, kept, fermion_trace=False, fp64=True):
    kept = np.ascontiguousarray(kept, np.int32)
    out = np.zeros(1)
    fn = getattr(lib(), "mipt_cuda_entropy_svd_" + _dtype_suffix(fp64))
    _check(fn(state_ptr, n, _p(kept), len(kept), int(fermion_trace), _p(out)))
    return float(out[0])


def renyi2(state_ptr, n, kept, fermion_trace=False, fp64=True):
    kept = np.ascontiguousarray(kept, np.int32)
    out = np.zeros(1)
    fn = getattr(lib(), "mipt_cuda_renyi2_" + _dtype_suffix(fp64))
    _check(fn(state_ptr, n, _p(kept), len(kept), int(fermion_trace), _p(out)))
    return float(out[0])


def rho3_subsystems(state_ptr, n, subsystems, fermion_trace=False, fp64=True):
    subs = np.ascontiguousarray(subsystems, np.int32).reshape(-1, 3)
    out = np.zeros(128 * len(subs))
    mid = "fermion_" if fermion_trace else ""
    fn = getattr(lib(), f"mipt_cuda_rho3_subsystems_complex_{mid}{_dtype_suffix(fp64)}")
    _check(fn(state_ptr, n, _p(subs), len(subs), _p(out)))
    return out


def measure_collapse(state_ptr, n, qubit, uniform_01, fp64=True):
    outcome = np.zeros(1, np.int32)
    prob = np.zeros(1)
    fn = getattr(lib(), "mipt_cuda_measure_collapse_" + _dtype_suffix(fp64))
    status = fn(state_ptr, n, qubit, uniform_01, _p(outcome), _p(prob))
    if status != 0:
        raise MiptError(status, lib().mipt_cuda_measure_collapse_last_error().decode(errors="replace"))
    return int(outcome[0]), float(prob[0])


# ------------------------------------------------------------------ engine
class Engine:
    """One state vector, layer by layer (the reference's cuStateVec Engine)."""

    def __init__(self, fp64=True):
        h = ctypes.c_void_p()
        _check(lib().mipt_gb300_engine_create(int(fp64), ctypes.byref(h)))
        self._h = h
        self.fp64 = fp64
        self.n = 0

    def close(self):
        if self._h:
            lib().mipt_gb300_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self, n):
        _check(lib().mipt_gb300_engine_reset(self._h, n))
        self.n = n

    def adopt(self, ptr, n):
        _check(lib().mipt_gb300_engine_adopt(self._h, ptr, n))
        self.n = n

    @property
    def data(self):
        return lib().mipt_gb300_engine_data(self._h)

    def set_state(self, psi):
        psi = np.ascontiguousarray(psi, np.complex128)
        n = int(np.log2(psi.size))
        _check(lib().mipt_gb300_engine_set_from_host(self._h, _p(psi), n))
        self.n = n

    def state(self):
        out = np.zeros(1 << self.n, np.complex128)
        _check(lib().mipt_gb300_engine_to_host(self._h, _p(out)))
        return out

    def apply_bonds(self, pairs, matrices):
        pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        m = np.ascontiguousarray(np.asarray(matrices, np.complex128).reshape(len(pairs), 16))
        _check(lib().mipt_gb300_engine_apply_bonds(self._h, _p(pairs), len(pairs), _p(m)))

    def measure_layer(self, sites, uniforms, chunk_bits=16, forced=None):
        sites = np.ascontiguousarray(sites, np.int32)
        u = np.ascontiguousarray(uniforms, np.float64)
        f = None if forced is None else np.ascontiguousarray(forced, np.int32)
        out = np.zeros(max(1, len(sites)), np.int32)
        sp = np.zeros(1)
        _check(lib().mipt_gb300_engine_measure_layer(self._h, _p(sites), len(sites), chunk_bits, _p(u), _p(f),
                                                     _p(out), _p(sp)))
        return out[: len(sites)].copy(), float(sp[0])


# ------------------------------------------------------------------- batch
class Batch:
    """Many Haar trajectories of one chain length, run as one device schedule."""

    def __init__(self, n, periods, capacity, closed=True, fp64=False, chunk_bits=16, observables=0,
                 observe_every=0, rho3=False, fermion_trace=False, host_threads=0, tile_qubits=0, tmi_cycles=0,
                 lattice=None, circuit=1, split_last=True, full_state=False):
        lx, ly = lattice if lattice is not None else (0, 0)
        cfg = BatchConfig(n, periods, int(closed), int(fp64), chunk_bits, observables, observe_every, int(rho3),
                          int(fermion_trace), host_threads, tile_qubits, tmi_cycles, lx, ly, int(circuit),
                          int(split_last), int(full_state))
        self.regions = 0
        self.tmi_cycles = max(1, tmi_cycles)
        h = ctypes.c_void_p()
        _check(lib().mipt_gb300_batch_create(ctypes.byref(cfg), capacity, ctypes.byref(h)))
        self._h = h
        self.n, self.periods = n, periods
        self.layers = 2 * periods + (1 if circuit in (2, 4) else 0)
        self.observe_every = observe_every
        self.points = (self.layers // observe_every) if observe_every > 0 else 1
        self.rho3 = rho3
        self.count = 0

    def close(self):
        if self._h:
            lib().mipt_gb300_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def prepare_workspace(self, workspace_seeds, p):
        """Free-energy draw: layers from the probed workspace streams of each 32-bit seed."""
        seeds = np.ascontiguousarray(workspace_seeds, np.uint32)
        p = np.ascontiguousarray(np.broadcast_to(np.asarray(p, np.float64), seeds.shape))
        _check(lib().mipt_gb300_batch_prepare_haar_workspace(self._h, _p(seeds), _p(p), len(seeds)))
        self.count = len(seeds)

    def set_initial_states(self, seeds, kind, fixed_parity=False):
        """Random initial states (kind 0 product, 1 Haar) for the next execute; returns parity sectors."""
        seeds = np.ascontiguousarray(seeds, np.uint64)
        sectors = np.zeros(len(seeds), np.int32)
        _check(lib().mipt_gb300_batch_set_initial_states(self._h, _p(seeds), int(kind), int(fixed_parity),
                                                          len(seeds), _p(sectors)))
        return sectors

    def set_initial_state(self, index, psi):
        ri = np.ascontiguousarray(np.asarray(psi, np.complex128)).view(np.float64)
        _check(lib().mipt_gb300_batch_set_initial_state(self._h, int(index), _p(ri)))

    def set_observation_steps(self, steps):
        """Observe after each listed number of layers (0 = the initial state)."""
        steps = np.ascontiguousarray(steps, np.int32)
        _check(lib().mipt_gb300_batch_set_observation_steps(self._h, _p(steps), len(steps)))
        self.points = len(steps) if len(steps) else ((self.layers // self.observe_every)
                                                     if self.observe_every > 0 else 1)

    def prepare(self, seeds, p, forced=None):
        seeds = np.ascontiguousarray(seeds, np.uint64)
        p = np.ascontiguousarray(np.broadcast_to(np.asarray(p, np.float64), seeds.shape))
        f = None if forced is None else np.ascontiguousarray(forced, np.uint64)
        _check(lib().mipt_gb300_batch_prepare_haar(self._h, _p(seeds), _p(p), len(seeds), _p(f)))
        self.count = len(seeds)

    def execute(self, stream=None):
        _check(lib().mipt_gb300_batch_execute(self._h, stream))

    def execute_graph(self, stream=None):
        """execute() through a captured CUDA graph (one launch once captured)."""
        _check(lib().mipt_gb300_batch_execute_graph(self._h, stream))

    def fetch(self):
        c, T = self.count, self.layers
        measured = np.zeros((c, T), np.uint64)
        outcomes = np.zeros((c, T), np.uint64)
        surprisal = np.zeros((c, T))
        obs = np.zeros((c, self.points, 4))
        rho3 = np.zeros((c, self.rho3_count, 128)) if self.rho3 else None
        _check(lib().mipt_gb300_batch_fetch(self._h, _p(measured), _p(outcomes), _p(surprisal), _p(obs), _p(rho3)))
        return dict(measured=measured, outcomes=outcomes, surprisal=surprisal, obs=obs, rho3=rho3)

    @property
    def rho3_count(self):
        return lib().mipt_gb300_batch_rho3_subsystem_count(self._h)

    def add_region(self, modes, order=1):
        """Entropy (order 1: von Neumann, 2: Renyi-2) of `modes` at every observation point."""
        modes = np.ascontiguousarray(modes, np.int32)
        rid = ctypes.c_int()
        _check(lib().mipt_gb300_batch_add_region(self._h, _p(modes), len(modes), int(order), ctypes.byref(rid)))
        self.regions += 1
        return rid.value

    def fetch_regions(self):
        out = np.zeros((self.count, self.points, self.regions))
        _check(lib().mipt_gb300_batch_fetch_regions(self._h, _p(out)))
        return out

    def set_rho3_subsystems(self, triples):
        t = np.ascontiguousarray(triples, np.int32).reshape(-1, 3)
        _check(lib().mipt_gb300_batch_set_rho3_subsystems(self._h, _p(t), len(t)))

    def fetch_rho3_points(self):
        out = np.zeros((self.count, self.points, self.rho3_count, 128))
        _check(lib().mipt_gb300_batch_fetch_rho3_points(self._h, _p(out)))
        return out

    def fetch_tmi(self, order=1):
        """TMI at every cyclic offset: [count][points][tmi_cycles]."""
        out = np.zeros((self.count, self.points, self.tmi_cycles))
        _check(lib().mipt_gb300_batch_fetch_tmi(self._h, int(order), _p(out)))
        return out

    def run(self, seeds, p, forced=None):
        self.prepare(seeds, p, forced)
        self.execute()
        return self.fetch()

    def state_ptr(self, i):
        return lib().mipt_gb300_batch_state(self._h, i)

    @property
    def launches(self):
        return lib().mipt_gb300_batch_launches(self._h)

    @property
    def parity_encoded(self):
        """Whether the prepared trajectories run on half-size parity-sector states."""
        return bool(lib().mipt_gb300_batch_parity_encoded(self._h))


    def set_profiling(self, enable=True):
        _check(lib().mipt_gb300_batch_set_profiling(self._h, int(enable)))

    KERNEL_KINDS = ("pass", "hist", "measure", "observables", "other")

    def kernel_stats(self):
        ms = np.zeros(5)
        n = np.zeros(5, np.int64)
        _check(lib().mipt_gb300_batch_kernel_stats(self._h, _p(ms), _p(n)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.KERNEL_KINDS)}


class BatchGroup:
    """Batches executed as the parallel branches of one CUDA graph."""

    def __init__(self, batches):
        self.batches = list(batches)
        arr = (ctypes.c_void_p * len(self.batches))(*[b._h.value for b in self.batches])
        h = ctypes.c_void_p()
        _check(lib().mipt_gb300_batch_group_create(arr, len(self.batches), ctypes.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            lib().mipt_gb300_batch_group_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def execute(self, stream=None):
        _check(lib().mipt_gb300_batch_group_execute(self._h, stream))


class GmnConfig(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int), ("check_every", ctypes.c_int), ("gap_tol", ctypes.c_double),
                ("feas_tol", ctypes.c_double), ("sigma", ctypes.c_double), ("fp64", ctypes.c_int)]


def rho_to_ri(rho):
    """[..., 8, 8] complex -> [..., 128] row-major (re, im) doubles."""
    rho = np.asarray(rho, np.complex128)
    return np.ascontiguousarray(np.stack([rho.real, rho.imag], -1).reshape(rho.shape[:-2] + (128,)))


def ri_to_rho(ri):
    ri = np.asarray(ri, np.float64)
    return (ri[..., 0::2] + 1j * ri[..., 1::2]).reshape(ri.shape[:-1] + (8, 8))


def gmn_solve(rho, warm_start=None, max_iter=20000, check_every=10, gap_tol=1e-6, feas_tol=1e-6, sigma=0.0,
              fp64=False, want_solution=False):
    """GMN of three-qubit states rho[N, 8, 8] by the batched GPU ADMM.
    warm_start: [N, 7, 8, 8] (W, Q_1..3, Z_1..3) or None. sigma: the ADMM
    penalty, a scalar (0: the library default, 0.1) or one per state."""
    r = rho_to_ri(np.asarray(rho).reshape(-1, 8, 8))
    n = len(r)
    per_state = np.ndim(sigma) > 0
    cfg = GmnConfig(max_iter, check_every, gap_tol, feas_tol, 0.0 if per_state else float(sigma), int(fp64))
    ws = None
    if warm_start is not None:
        ws = np.ascontiguousarray(rho_to_ri(np.asarray(warm_start).reshape(n, 7, 8, 8)), np.float32)
    g = np.zeros(n)
    gap = np.zeros(n)
    it = np.zeros(n, np.int32)
    sol = np.zeros((n, 7, 128)) if want_solution else None
    if per_state:
        sg = np.ascontiguousarray(np.broadcast_to(np.asarray(sigma, np.float64), (n,)))
        _check(lib().mipt_gb300_gmn_solve_sigma(ctypes.byref(cfg), _p(r), n, _p(sg), _p(ws), _p(g), _p(gap), _p(it),
                                                _p(sol)))
    else:
        _check(lib().mipt_gb300_gmn_solve(ctypes.byref(cfg), _p(r), n, _p(ws), _p(g), _p(gap), _p(it), _p(sol)))
    out = dict(gmn=g, gap=gap, iters=it)
    if want_solution:
        out["solution"] = ri_to_rho(sol)
    return out


def autotune_tile(n, fp64=False, closed=True, lattice=None, trajectories=4):
    """Times every candidate pass-tile size for this geometry (passes only)
    and returns (best_tile, {tile: ms per cycle of all layer colours})."""
    lx, ly = lattice if lattice else (0, 1)
    best = ctypes.c_int()
    cand = np.zeros(3, np.int32)
    ms = np.zeros(3)
    cnt = ctypes.c_int()
    _check(lib().mipt_gb300_autotune_tile(n, int(fp64), int(closed), lx, ly, trajectories, ctypes.byref(best),
                                          _p(cand), _p(ms), ctypes.byref(cnt)))
    return best.value, {int(c): float(t) for c, t in zip(cand[: cnt.value], ms[: cnt.value])}


def cut_negativities(rho):
    """Negativity of the three single-qubit cuts of states rho[N, 8, 8] (FP64
    on the GPU); the minimum is gmn.exe's bipartite-negativity prefilter."""
    r = rho_to_ri(np.asarray(rho).reshape(-1, 8, 8))
    out = np.zeros((len(r), 3))
    _check(lib().mipt_gb300_cut_negativities(_p(r), len(r), _p(out)))
    return out


def lattice_bonds(x, y, colour):
    """Bond list (pairs) of colour 0..3 of the x by y lattice brickwork."""
    pairs = np.zeros(x * y + 2, np.int32)
    cnt = ctypes.c_int()
    _check(lib().mipt_gb300_lattice_bonds(x, y, colour, _p(pairs), ctypes.byref(cnt)))
    return pairs[: 2 * cnt.value].reshape(-1, 2)


def draw_haar_lattice(seed, x, y, layers, p, chunk_bits=16):
    """One 2-D Haar trajectory as the batch draws it."""
    n, mb = x * y, (x * y) // 2
    gpl = np.zeros(layers, np.int32)
    bq = np.zeros((layers, mb, 2), np.int32)
    bu = np.zeros((layers, mb, 32))
    meas = np.zeros(layers, np.uint64)
    uni = np.zeros(layers * n)
    nu = ctypes.c_int()
    _check(lib().mipt_gb300_draw_haar_lattice(seed, x, y, layers, p, chunk_bits, _p(gpl), _p(bq), _p(bu), _p(meas),
                                               _p(uni), ctypes.byref(nu)))
    return dict(gates_per_layer=gpl, bond_q=bq, bond_u=bu, measured=meas, uniforms=uni[: nu.value])


def outcomes_to_mask(sites, outcomes):
    """Bit mask (bit q = outcome of site q) from per-site outcomes."""
    m = 0
    for s, o in zip(sites, outcomes):
        if s >= 0 and o:
            m |= 1 << int(s)
    return m


# ----------------------------------------------------------- free fermions
def ff_run(seeds, p, n_modes, depth, closed=True, repurify_every=64, blocks=(), tmi=True, forced=None,
           want_gamma=False, host_threads=0, fp64=False):
    """Monitored free-fermion trajectories on the Majorana covariance matrix
    (fp64: Gamma evolves in FP64, the plain method)."""
    seeds = np.ascontiguousarray(seeds, np.uint64)
    c = len(seeds)
    p = np.ascontiguousarray(np.broadcast_to(np.asarray(p, np.float64), seeds.shape))
    bl = np.ascontiguousarray(blocks, np.int32)
    cfg = FFConfig(n_modes, depth, int(closed), repurify_every, len(bl),
                   bl.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if len(bl) else None, host_threads, int(fp64))
    outcomes = np.zeros((c, depth, n_modes), np.int32)
    probs = np.zeros((c, depth, n_modes))
    gamma = np.zeros((c, 2 * n_modes, 2 * n_modes)) if want_gamma else None
    sb = np.zeros((c, max(1, len(bl))))
    t = np.zeros(c) if tmi else None
    f = None if forced is None else np.ascontiguousarray(forced, np.int32)
    _check(lib().mipt_gb300_ff_run(ctypes.byref(cfg), _p(seeds), _p(p), c, _p(f), _p(outcomes), _p(probs),
                                   _p(gamma), _p(sb), _p(t)))
    return dict(outcomes=outcomes, probs=probs, gamma=gamma, s_blocks=sb[:, : len(bl)], tmi=t)
