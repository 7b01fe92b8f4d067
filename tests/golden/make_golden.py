"""Generate tests/golden/ref_fixtures.npz from the reference's own host code.

Runs in the development container only: it loads oracle/_ref/libmipt_ref.so,
which oracle/ref/build_ref.sh compiles from the reference checkout's headers
(the reference's samplers -- Haar, probed-workspace and RPPU/qRPPU layer draws
and the free-energy initial states --, bond-matrix builders, measurement
primitive, reduced-density and entropy code, the rho3.bin writer and the
checkpoint readers of free_energy.exe, entropy.exe and sim_tmi.exe). The
fixtures it writes are what the CPU oracle and the product are pinned to on
machines without the reference.

    python tests/golden/make_golden.py
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libmipt_ref.so")

# (seed, n, periods, p, closed, chunk_bits): covers open and closed chains,
# p = 0 and p = 1 (the sampler's two short-cuts), chunk splitting, and the
# the chain lengths of the measured workloads.
DRAWS = [
    (0, 12, 12, 0.2, 0, 16),
    (1, 12, 3, 0.2, 1, 16),
    (123, 24, 2, 0.35, 1, 16),
    (5, 22, 2, 1.0, 1, 16),
    (9, 8, 5, 0.0, 1, 4),
    (77, 20, 2, 0.9, 1, 3),
    (2024, 16, 3, 0.15, 1, 16),
    (31337, 4, 4, 0.5, 1, 16),
]


def xorshift_state(n, seed):
    """Dense random state in the style of the reference's GPU RDM tests:
    xorshift64 uniforms, Box-Muller normals, normalised."""
    state = seed & 0xFFFFFFFFFFFFFFFF
    mask = 0xFFFFFFFFFFFFFFFF

    def uniform():
        nonlocal state
        state ^= (state << 13) & mask
        state ^= state >> 7
        state ^= (state << 17) & mask
        return (state >> 11) * (1.0 / 9007199254740992.0)

    def normal():
        u1 = max(1.0e-12, uniform())
        u2 = uniform()
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(6.283185307179586 * u2)

    dim = 1 << n
    psi = np.empty(dim, np.complex128)
    for i in range(dim):
        re = normal()
        im = normal()
        psi[i] = re + 1j * im
    return psi / np.linalg.norm(psi)


def entropy_checkpoint_cases():
    """entropy.exe result CSVs (its checkpoint) in the reference's layout, with
    the run each is resumed by: (text, n, periods, p, requested, circ_type,
    largest S1 block of the run)."""
    head = ("N,periods,p,requested_realizations,completed_realizations,circ_type,circuit_name,fermionic_trace,L_A,"
            "x,ln_x,S1_mean,S1_stddev,S1_stderr,S2_mean,S2_stddev,S2_stderr,subsystems_per_realization,"
            "total_subsystems")
    legacy = ("N,periods,p,requested_realizations,completed_realizations,circ_type,circuit_name,fermionic_trace,L_A,"
              "x,ln_x,S2_mean,S2_stddev,S2_stderr,subsystems_per_realization,total_subsystems")

    def rows(n, periods, p, requested, done, s1_upto, edit=None, old=False):
        out = [legacy if old else head]
        for kept in range(2, n // 2 + 1):
            x = float((n / np.pi) * np.sin(np.pi * kept / n))
            sd = 0.25
            se = float(sd / np.sqrt(done)) if done > 1 else 0.0
            if edit == kept:
                se *= 1.5
            s1 = f"{0.5 * kept!r},{sd!r},{se!r}" if kept <= s1_upto else "nan,nan,nan"
            s2 = f"{0.4 * kept!r},{sd!r},{se!r}"
            mid = s2 if old else f"{s1},{s2}"
            out.append(f'{n},{periods},{p!r},{requested},{done},1,"Random Haar Unitary",0,{kept},{x!r},'
                       f'{float(np.log(x))!r},{mid},{n},{n * done}')
        return "\n".join(out) + "\n"

    return [
        (rows(8, 2, 0.1, 5, 2, 4), 8, 2, 0.1, 5, 1, 4),
        (rows(8, 2, 0.1, 5, 5, 4), 8, 2, 0.1, 5, 1, 4),
        (rows(8, 2, 0.1, 5, 2, 4), 8, 2, 0.1, 5, 1, 3),
        (rows(8, 2, 0.1, 5, 3, 4, edit=3), 8, 2, 0.1, 5, 1, 4),
        (rows(8, 2, 0.1, 5, 2, 4, old=True), 8, 2, 0.1, 5, 1, 4),
        (rows(8, 2, 0.1, 5, 2, 4), 10, 2, 0.1, 5, 1, 5),
        (rows(8, 2, 0.1, 5, 2, 4), 8, 2, 0.2, 5, 1, 4),
        (rows(8, 2, 0.1, 5, 2, 2), 8, 2, 0.1, 5, 1, 2),
    ]


def tmi_checkpoint_cases():
    """sim_tmi.exe `p,tmi` CSVs with the run resuming them: (file name, text,
    n, realizations, resolution, p_min, p_max, all_cycles). The file names
    follow the generated csv/tmi/<tag>/ naming or deliberately not."""
    def p_text(v):
        return format(float(v), ".17g")

    def body(ps, per_p, extra=(), header="p,tmi"):
        lines = [header]
        for pv, count in zip(ps, per_p):
            lines += [f"{p_text(pv)},{0.01 * i!r}" for i in range(count)]
        lines += list(extra)
        return "\n".join(lines) + "\n"

    ps = np.linspace(0.1, 0.3, 2)
    nm = "tmi_haar_n_8_real_3_0.1_0.3_res_2.csv"
    nmc = "tmi_haarc_n_8_real_3_0.1_0.3_res_2.csv"
    return [
        (nm, body(ps, [3, 3]), 8, 3, 2, 0.1, 0.3, 0),
        (nm, body(ps, [3, 1]), 8, 3, 2, 0.1, 0.3, 0),
        (nmc, body(ps, [6, 3]), 8, 3, 2, 0.1, 0.3, 1),
        (nm, body(ps, [3], extra=[f"{p_text(0.25)},0.5"]), 8, 3, 2, 0.1, 0.3, 0),
        (nm, body(ps, [2], header="p,TMI"), 8, 3, 2, 0.1, 0.3, 0),
        ("tmi_haar_n_12_real_3_0.1_0.3_res_2.csv", body(ps, [1]), 8, 3, 2, 0.1, 0.3, 0),
        ("my_tmi.csv", body(ps, [3, 2]), 8, 3, 2, 0.1, 0.3, 0),
    ]


def fe_checkpoint_cases(lib):
    """free_energy.exe checkpoint pairs (samples CSV, time-series CSV, run
    parameters) in the reference's layout: a clean one, a killed flush, a
    lagging aggregate, and three the reference refuses."""
    sm = lib.ref_splitmix64
    H_S = ("N,p,circ_type,circuit_name,init_state,trajectory,parity_sector,trajectory_seed,equil_timesteps,"
           "production_timesteps,total_timesteps,measurements_total,measurements_production,F_total,F_production,"
           "production_rate_endpoint,production_slope,free_energy_density_tilde")
    H_T = ("N,p,circ_type,circuit_name,init_state,requested_realizations,completed_realizations,t,t_over_L,phase,"
           "F_mean,F_stddev,F_stderr,F_over_tL_mean,F_over_tL_stddev,F_over_tL_stderr,S_half_mean,S_half_stddev,"
           "S_half_stderr,S_half_count")
    name = '"Random Haar Unitary"'

    def samples(n, p, init, master, count, skip=None):
        rows = [H_S]
        for t in range(count):
            if t == skip:
                continue
            ts = sm((master ^ t) & 0xFFFFFFFFFFFFFFFF)
            rows.append(f"{n},{p!r},1,{name},{init},{t},-1,{ts},{4 * n},{24 * n},{28 * n},10,8,1.5,1.25,0.1,0.1,0.0125")
        return "\n".join(rows) + "\n"

    def series(n, p, init, requested, completed, max_t):
        rows = [H_T]
        for t in range(28 * n + 1):
            phase = "initial" if t == 0 else ("equilibration" if t <= 4 * n else "production")
            sc = completed if t <= max_t else 0
            st = "0.5,0.1,0.05" if sc else "nan,nan,nan"
            f = "0,0,0" if t == 0 else "0.25,0.01,0.005"
            ftl = "nan,nan,nan" if t == 0 else "0.01,0.001,0.0005"
            rows.append(f"{n},{p!r},1,{name},{init},{requested},{completed},{t},{t / n!r},{phase},{f},{ftl},{st},{sc}")
        return "\n".join(rows) + "\n"

    n, p, R = 6, 0.2, 6
    return [
        (samples(n, p, 0, 991, 3), series(n, p, 0, R, 3, 12), (n, p, 0, R, 12, 1)),
        (samples(n, p, 0, 5, 4) + f"{n},0.2,1,\"Ran", series(n, p, 0, R, 4, 12), (n, p, 0, R, 12, 1)),
        (samples(n, p, 1, 2**64 - 7, 3), series(n, p, 1, R, 2, 12), (n, p, 1, R, 12, 1)),
        (samples(n, p, 0, 42, 3, skip=1), series(n, p, 0, R, 2, 12), (n, p, 0, R, 12, 1)),
        (samples(n, p, 0, 42, 3), series(n, p, 0, R, 3, 12), (n, p, 0, R, 7, 1)),
        (samples(n, p, 1, 42, 3), series(n, p, 1, R, 3, 12), (n, p, 0, R, 12, 1)),
    ]


def main():
    if not os.path.exists(LIB):
        subprocess.check_call([os.path.join(ROOT, "oracle", "ref", "build_ref.sh")])
    lib = ctypes.CDLL(LIB)
    vp = ctypes.c_void_p
    lib.ref_haar_draw.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_int, ctypes.c_int] + [vp] * 7
    lib.ref_trajectory_seed.restype = ctypes.c_uint64
    lib.ref_trajectory_seed.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
    lib.ref_splitmix64.restype = ctypes.c_uint64
    lib.ref_splitmix64.argtypes = [ctypes.c_uint64]
    lib.ref_measure_collapse.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, vp, vp, vp]
    lib.ref_rdm_from_state.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, vp]
    lib.ref_entropy_hermitian.restype = ctypes.c_double
    lib.ref_entropy_hermitian.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    lib.ref_renyi2_from_purity.restype = ctypes.c_double
    lib.ref_renyi2_from_purity.argtypes = [ctypes.c_double]
    lib.ref_rho3_from_state.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, vp]

    out = {}
    # --- seeding -----------------------------------------------------------
    seeds_in = np.array([0, 1, 2, 12345, 2**63 + 7, 2**64 - 1], np.uint64)
    out["splitmix_in"] = seeds_in
    out["splitmix_out"] = np.array([lib.ref_splitmix64(int(s)) for s in seeds_in], np.uint64)
    out["trajseed_out"] = np.array([[lib.ref_trajectory_seed(m, i) for i in range(5)]
                                    for m in (0, 1, 0xDEADBEEF)], np.uint64)

    # --- Haar trajectory draws ---------------------------------------------
    out["draw_params"] = np.array([d for d in DRAWS], np.float64)
    for k, (seed, n, periods, p, closed, chunk) in enumerate(DRAWS):
        L, mg = 2 * periods, n // 2
        gpl = np.zeros(L, np.int32)
        gq = np.zeros((L, mg, 2), np.int32)
        gm = np.zeros((L, mg, 32))
        spl = np.zeros(L, np.int32)
        sites = np.full((L, n), -1, np.int32)
        uni = np.zeros(L * n + 1)
        nu = np.zeros(1, np.int32)
        rc = lib.ref_haar_draw(seed, n, periods, p, closed, chunk,
                               *[a.ctypes.data for a in (gpl, gq, gm, spl, sites, uni, nu)])
        assert rc == 0
        out[f"draw{k}_gates_per_layer"] = gpl
        out[f"draw{k}_gate_q"] = gq
        out[f"draw{k}_gate_m"] = gm
        out[f"draw{k}_sites_per_layer"] = spl
        out[f"draw{k}_sites"] = sites
        out[f"draw{k}_uniforms"] = uni[: nu[0]].copy()

    # --- sequential measurement (reference known answer + random states) ---
    cases = []
    psi = np.array([1, 2, 3, 4], np.complex128)
    cases.append((psi, 2, 0, 0.5))
    cases.append((None, 2, 1, 0.9))  # continues from the collapsed state above
    for k, (n, q, u) in enumerate([(6, 2, 0.3), (8, 7, 0.99), (5, 0, 0.01), (7, 4, 0.5)]):
        cases.append((xorshift_state(n, 0x1234 + k), n, q, u))
    states_in, states_out, meas = [], [], []
    prev = None
    for psi, n, q, u in cases:
        if psi is None:
            psi = prev
        buf = np.ascontiguousarray(psi.astype(np.complex128)).view(np.float64).copy()
        states_in.append(buf.copy())
        oc = np.zeros(1, np.int32)
        cp = np.zeros(1)
        sp = np.zeros(1)
        rc = lib.ref_measure_collapse(buf.ctypes.data, n, q, u, oc.ctypes.data, cp.ctypes.data, sp.ctypes.data)
        assert rc == 0
        states_out.append(buf.copy())
        prev = buf.view(np.complex128).copy()
        meas.append((n, q, u, oc[0], cp[0], sp[0]))
    for i, (a, b) in enumerate(zip(states_in, states_out)):
        out[f"mc{i}_in"] = a
        out[f"mc{i}_out"] = b
    out["mc_params"] = np.array(meas, np.float64)

    # --- RDMs and entropies on dense random states --------------------------
    rdm_cases = [
        (6, [0, 1, 2], 0), (6, [4, 1], 1), (7, [6, 0, 3], 1), (8, [0, 1, 2, 3], 0),
        (8, [2, 5, 7, 0], 1), (9, [8, 0, 1], 0), (10, [0, 1, 2, 3, 4], 0), (10, [9, 3, 5, 1, 7], 1),
        (12, [0, 1, 2, 3, 4, 5], 0), (12, [6, 7, 8, 0, 1, 2], 0),
    ]
    ent = []
    for k, (n, kept, ferm) in enumerate(rdm_cases):
        psi = xorshift_state(n, 0xABCDEF0123456789 + n + len(kept))
        ri = np.ascontiguousarray(psi).view(np.float64)
        d = 1 << len(kept)
        kk = np.array(kept, np.int32)
        rho = np.zeros(2 * d * d)
        assert lib.ref_rdm_from_state(ri.ctypes.data, n, kk.ctypes.data, len(kept), ferm, rho.ctypes.data) == 0
        s1 = lib.ref_entropy_hermitian(rho.ctypes.data, d, 1)
        s2 = lib.ref_entropy_hermitian(rho.ctypes.data, d, 2)
        out[f"rdm{k}_psi"] = ri.copy()
        out[f"rdm{k}_kept"] = kk
        out[f"rdm{k}_rho"] = rho
        ent.append((n, ferm, s1, s2))
    out["rdm_params"] = np.array(ent, np.float64)

    # --- closed-form entropies (maximally mixed, pure, rank 2) --------------
    closed_forms = []
    for d in (2, 4, 8, 64):
        rho = np.eye(d, dtype=np.complex128) / d
        ri = np.ascontiguousarray(rho).view(np.float64)
        closed_forms.append((d, 0, lib.ref_entropy_hermitian(ri.ctypes.data, d, 1),
                             lib.ref_entropy_hermitian(ri.ctypes.data, d, 2)))
    rho = np.zeros((4, 4), np.complex128)
    rho[0, 0] = 1.0
    ri = np.ascontiguousarray(rho).view(np.float64)
    closed_forms.append((4, 1, lib.ref_entropy_hermitian(ri.ctypes.data, 4, 1),
                         lib.ref_entropy_hermitian(ri.ctypes.data, 4, 2)))
    rho = np.diag([0.3, 0.7, 0.0, 0.0]).astype(np.complex128)
    ri = np.ascontiguousarray(rho).view(np.float64)
    closed_forms.append((4, 2, lib.ref_entropy_hermitian(ri.ctypes.data, 4, 1),
                         lib.ref_entropy_hermitian(ri.ctypes.data, 4, 2)))
    out["closed_forms"] = np.array(closed_forms, np.float64)
    out["renyi2_purity_in"] = np.array([1.0, 1.0 + 1e-15, 0.5, 0.25, 0.0, -1.0, 0.999999999999])
    out["renyi2_purity_out"] = np.array([lib.ref_renyi2_from_purity(float(x)) for x in out["renyi2_purity_in"]])

    # --- three-site RDMs on the periodic ring --------------------------------
    for k, (n, ferm) in enumerate([(6, 0), (6, 1), (8, 1), (5, 0)]):
        psi = xorshift_state(n, 0x5151 + 7 * k)
        ri = np.ascontiguousarray(psi).view(np.float64)
        subs = np.array([[s, (s + 1) % n, (s + 2) % n] for s in range(n)], np.int32)
        rho3 = np.zeros(128 * n)
        assert lib.ref_rho3_from_state(ri.ctypes.data, n, subs.ctypes.data, n, ferm, rho3.ctypes.data) == 0
        out[f"rho3_{k}_psi"] = ri.copy()
        out[f"rho3_{k}_subs"] = subs
        out[f"rho3_{k}_ferm"] = np.array([ferm])
        out[f"rho3_{k}_out"] = rho3

    # --- free-energy protocol: initial states and workspace draws -----------
    lib.ref_fe_initial_state.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp]
    lib.ref_fe_draw.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                ctypes.c_int] + [vp] * 7
    fe_init = []
    for k, (seed, n, kind, fixed) in enumerate([(11, 6, 0, 0), (12, 6, 1, 0), (13, 7, 0, 1), (14, 6, 1, 1),
                                                (2**64 - 3, 10, 0, 0), (99, 10, 1, 0)]):
        amps = np.zeros(2 << n)
        par = np.zeros(1, np.int32)
        assert lib.ref_fe_initial_state(seed, n, kind, fixed, amps.ctypes.data, par.ctypes.data) == 0
        out[f"feinit{k}_amps"] = amps
        fe_init.append((seed, n, kind, fixed, par[0]))
    out["feinit_params"] = np.array(fe_init, np.uint64)
    FE_DRAWS = [(0x12345678, 6, 12, 0.3, 16), (7, 8, 10, 1.0, 3), (0xFFFFFFFF, 10, 6, 0.1, 16), (1, 4, 8, 0.0, 16)]
    out["fedraw_params"] = np.array(FE_DRAWS, np.float64)
    for k, (seed, n, layers, p, chunk) in enumerate(FE_DRAWS):
        mg = n // 2
        gpl = np.zeros(layers, np.int32)
        gq = np.zeros((layers, mg, 2), np.int32)
        gm = np.zeros((layers, mg, 32))
        spl = np.zeros(layers, np.int32)
        sites = np.full((layers, n), -1, np.int32)
        uni = np.zeros(layers * n + 1)
        nu = np.zeros(1, np.int32)
        assert lib.ref_fe_draw(seed, n, layers, p, chunk,
                               *[a.ctypes.data for a in (gpl, gq, gm, spl, sites, uni, nu)]) == 0
        out[f"fedraw{k}_gates_per_layer"] = gpl
        out[f"fedraw{k}_gate_q"] = gq
        out[f"fedraw{k}_gate_m"] = gm
        out[f"fedraw{k}_sites_per_layer"] = spl
        out[f"fedraw{k}_sites"] = sites
        out[f"fedraw{k}_uniforms"] = uni[: nu[0]].copy()

    # --- RPPU / qRPPU layer draws (ops as the engine receives them) -----------
    lib.ref_rppu_draw.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_int] + [vp] * 5
    lib.ref_rppu_draw.restype = ctypes.c_int
    # (seed, n, periods-or-layers, p, boundary 0 FSWAP / 1 JW / 2 qubit, workspace)
    RPPU_DRAWS = [(3, 6, 3, 0.3, 1, 0), (4, 8, 2, 0.5, 0, 0), (5, 10, 2, 1.0, 2, 0), (6, 4, 4, 0.0, 1, 0),
                  (0xABCDEF12, 6, 7, 0.25, 1, 1), (77, 8, 5, 0.4, 2, 1)]
    out["rppu_params"] = np.array(RPPU_DRAWS, np.float64)
    for k, (seed, n, periods, p, boundary, ws) in enumerate(RPPU_DRAWS):
        T = periods if ws else 2 * periods + 1
        oc = np.zeros(T, np.int32)
        meta = np.zeros((T * 4 * n, 3), np.int32)
        m = np.zeros((T * 4 * n, 32))
        spl = np.zeros(T, np.int32)
        sites = np.full((T, n), -1, np.int32)
        t = lib.ref_rppu_draw(seed, n, periods, p, boundary, ws,
                              *[a.ctypes.data for a in (oc, meta, m, spl, sites)])
        assert t > 0
        kk = int(oc[:t].sum())
        out[f"rppu{k}_ops_per_layer"] = oc[:t].copy()
        out[f"rppu{k}_meta"] = meta[:kk].copy()
        out[f"rppu{k}_m"] = m[:kk].copy()
        out[f"rppu{k}_sites_per_layer"] = spl[:t].copy()
        out[f"rppu{k}_sites"] = sites[:t].copy()

    # --- rho3.bin files written by the reference's DensityMatrixWriter -------
    lib.ref_rho3_write.argtypes = [ctypes.c_char_p, vp, ctypes.c_uint64, ctypes.c_double, ctypes.c_double] + [vp] * 5
    import tempfile
    rng = np.random.default_rng(31)
    # (spatial, total, kept, periods, realizations, resolution, grid_x, grid_y, subsystems), records
    RHO3_FILES = [((1, 5, 3, 4, 1, 2, 5, 1, 5), 2), ((2, 6, 3, 3, 2, 1, 2, 3, 4), 3), ((1, 4, 2, 1, 1, 1, 4, 1, 2), 1)]
    for k, (dims, nrec) in enumerate(RHO3_FILES):
        dims_a = np.array(dims, np.uint32)
        S, K = dims[8], dims[2]
        subs = np.concatenate([rng.permutation(dims[1])[:K] for _ in range(S)]).astype(np.uint32)
        pidx = rng.integers(0, 3, size=nrec).astype(np.uint32)
        real = rng.integers(0, 9, size=nrec).astype(np.uint32)
        ps = rng.uniform(0, 1, size=nrec)
        payload = rng.standard_normal(nrec * S * 2 * (1 << K) ** 2)
        with tempfile.TemporaryDirectory() as tmp:
            path = os.path.join(tmp, "rho3.bin")
            assert lib.ref_rho3_write(path.encode(), dims_a.ctypes.data, nrec, 0.125, 0.875, subs.ctypes.data,
                                      pidx.ctypes.data, real.ctypes.data, ps.ctypes.data, payload.ctypes.data) == 0
            with open(path, "rb") as f:
                out[f"rho3file{k}_bytes"] = np.frombuffer(f.read(), np.uint8).copy()
        out[f"rho3file{k}_dims"] = dims_a
        out[f"rho3file{k}_subs"] = subs
        out[f"rho3file{k}_pidx"] = pidx
        out[f"rho3file{k}_real"] = real
        out[f"rho3file{k}_p"] = ps
        out[f"rho3file{k}_payload"] = payload

    # --- sim_tmi.exe checkpoints through the reference's own reader ----------
    lib.ref_tmi_resume.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int,
                                   vp, ctypes.c_char_p, ctypes.c_int]
    rows_t = []
    with tempfile.TemporaryDirectory() as tmp:
        for k, (name, text, n, R, res, pmin, pmax, allc) in enumerate(tmi_checkpoint_cases()):
            path = os.path.join(tmp, name)
            with open(path, "w") as f:
                f.write(text)
            cycles = n // 4 if allc else 1
            tag = "haarc" if allc else "haar"
            expected = f"csv/tmi/{tag}/tmi_{tag}_n_{n}_real_{R}_{pmin:g}_{pmax:g}_res_{res}.csv"
            texts = [format(float(v), ".17g").encode() for v in np.linspace(pmin, pmax, res)]
            arr = (ctypes.c_char_p * len(texts))(*texts)
            res_out = np.zeros(7, np.int64)
            msg = ctypes.create_string_buffer(1024)
            rc = lib.ref_tmi_resume(path.encode(), expected.encode(), R, cycles, ctypes.cast(arr, vp), len(texts),
                                    res_out.ctypes.data, msg, 1024)
            out[f"tmick{k}_name"] = np.array(name)
            out[f"tmick{k}_text"] = np.array(text)
            out[f"tmick{k}_message"] = np.array(msg.value.decode().replace(tmp + os.sep, ""))
            rows_t.append([n, R, res, pmin, pmax, allc, rc, *res_out.tolist()])
    out["tmick_params"] = np.array(rows_t, np.float64)

    # --- entropy.exe checkpoints through the reference's own reader ----------
    lib.ref_entropy_resume.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_long,
                                       ctypes.c_int, ctypes.c_int, vp, ctypes.c_char_p, ctypes.c_int]
    rows_e = []
    with tempfile.TemporaryDirectory() as tmp:
        for k, (text, n, periods, p, requested, circ, s1max) in enumerate(entropy_checkpoint_cases()):
            path = os.path.join(tmp, f"e{k}.csv")
            with open(path, "w") as f:
                f.write(text)
            done = np.zeros(1, np.int64)
            msg = ctypes.create_string_buffer(1024)
            rc = lib.ref_entropy_resume(path.encode(), n, periods, p, requested, circ, s1max, done.ctypes.data, msg,
                                        1024)
            out[f"entck{k}_text"] = np.array(text)
            out[f"entck{k}_message"] = np.array(msg.value.decode().replace(tmp + os.sep, ""))
            rows_e.append([n, periods, p, requested, circ, s1max, rc, int(done[0])])
    out["entck_params"] = np.array(rows_e, np.float64)

    # --- free_energy.exe checkpoints through the reference's own readers ----
    lib.ref_fe_resume.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp,
                                  ctypes.c_char_p, ctypes.c_int]
    import tempfile
    cases = fe_checkpoint_cases(lib)
    rows = []
    with tempfile.TemporaryDirectory() as tmp:
        for k, (samples, series, prm) in enumerate(cases):
            sp, tp = os.path.join(tmp, f"s{k}.csv"), os.path.join(tmp, f"t{k}.csv")
            with open(sp, "w") as f:
                f.write(samples)
            with open(tp, "w") as f:
                f.write(series)
            res = np.zeros(4, np.int64)
            master = np.zeros(1, np.uint64)
            msg = ctypes.create_string_buffer(1024)
            n, p, init, R, max_t, stride = prm
            rc = lib.ref_fe_resume(sp.encode(), tp.encode(), n, p, 1, init, R, 1, max_t, stride,
                                   res.ctypes.data, master.ctypes.data, msg, 1024)
            out[f"feck{k}_samples"] = np.array(samples)
            out[f"feck{k}_series"] = np.array(series)
            out[f"feck{k}_message"] = np.array(msg.value.decode().replace(tmp + os.sep, ""))
            rows.append([n, p, init, R, max_t, stride, rc, *res.tolist(), float(master[0])])
            out[f"feck{k}_master"] = master.copy()
    out["feck_params"] = np.array(rows, np.float64)

    path = os.path.join(HERE, "ref_fixtures.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.1f} KiB, {len(out)} arrays)")


if __name__ == "__main__":
    sys.exit(main())
