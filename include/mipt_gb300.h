/*
 * mipt_gb300 -- C ABI of the GB300-native monitored-circuit trajectory path.
 *
 * Conventions shared by every entry point:
 *   - return 0 on success, nonzero on failure (a cudaError_t value, or
 *     MIPT_GB300_E_* below); mipt_gb300_last_error() describes the failure
 *     of the calling thread's last call;
 *   - device state vectors are borrowed, never freed, and hold 2^n
 *     interleaved complex amplitudes (float2 for *_f32, double2 for *_f64),
 *     qubit q = bit q of the amplitude index;
 *   - host output buffers are caller-owned; density matrices are row-major
 *     (re, im) pairs;
 *   - calls without a stream argument are synchronous to the host.
 *
 * The mipt_cuda_* functions keep the names, arguments and meaning of the
 * reference's C ABI (paths inside the reference project are cited per
 * function); a caller linked against the reference's CUDA objects can link
 * this library instead.
 */
#ifndef MIPT_GB300_H
#define MIPT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MIPT_GB300_E_INVALID 9001  /* bad argument */
#define MIPT_GB300_E_NUMERIC 9002  /* zero-norm state / no outcome with weight */
#define MIPT_GB300_E_NODEVICE 9003 /* no CUDA device */
#define MIPT_GB300_E_INTERNAL 9004

const char *mipt_gb300_last_error(void);
const char *mipt_gb300_version(void);

/* ------------------------------------------------------------------ RDMs */

/* Reduced density matrix of the retained modes (row index bit k <-> mode
 * host_kept_modes[k]); fermion_trace != 0 applies the Jordan-Wigner sign of
 * moving the kept modes ahead of the environment.
 * Replaces cpp/include/mipt/cuda/tmi_cuda_rdm.hpp:20-34. */
int mipt_cuda_rdm_subsystem_f64(const void *device_state_vector, int n_qubits, const int *host_kept_modes,
                                int kept_count, int fermion_trace, double *host_rho_ri_row_major);
int mipt_cuda_rdm_subsystem_f32(const void *device_state_vector, int n_qubits, const int *host_kept_modes,
                                int kept_count, int fermion_trace, double *host_rho_ri_row_major);

/* Von Neumann entropy (bits) of the same subsystem.
 * Replaces cpp/include/mipt/cuda/tmi_cuda_svd.hpp:58-72. */
int mipt_cuda_entropy_svd_f64(const void *device_state_vector, int n_qubits, const int *host_kept_modes,
                              int kept_count, int fermion_trace, double *entropy_out);
int mipt_cuda_entropy_svd_f32(const void *device_state_vector, int n_qubits, const int *host_kept_modes,
                              int kept_count, int fermion_trace, double *entropy_out);

/* Renyi-2 entropy S_2 = -log2 Tr(rho^2) (bits), from the Gram matrix only.
 * Replaces cpp/include/mipt/cuda/tmi_cuda_svd.hpp:84-98. */
int mipt_cuda_renyi2_f64(const void *device_state_vector, int n_qubits, const int *host_kept_modes,
                         int kept_count, int fermion_trace, double *entropy_out);
int mipt_cuda_renyi2_f32(const void *device_state_vector, int n_qubits, const int *host_kept_modes,
                         int kept_count, int fermion_trace, double *entropy_out);

/* mipt_cuda_renyi2_f32 without any device allocation. No reference
 * counterpart. Scratch is a static 512 KiB array per device, so
 * kept_count <= 14; larger requests return MIPT_GB300_E_INVALID. Every call
 * (with the caller's device current) looks up the array's address in the
 * current context. No call may be made during a stream capture: each call
 * copies synchronously and clears on the legacy default stream. The array is
 * shared by all calls on a device: calls that overlap on the GPU race, so
 * callers serialise them. */
int mipt_gb300_renyi2_f32_noalloc(const void *device_state_vector, int n_qubits, const int *host_kept_modes,
                                  int kept_count, int fermion_trace, double *entropy_out);

/* Three-site reduced density matrices, 128 doubles per subsystem;
 * host_subsystems is a flat int[3*subsystem_count].
 * Replaces cpp/include/mipt/cuda/rho_reduce.hpp:22-126. */
int mipt_cuda_rho3_subsystems_complex_f64(const void *device_state_vector, int n_qubits, const int *host_subsystems,
                                          int subsystem_count, double *host_rho_ri_row_major);
int mipt_cuda_rho3_subsystems_complex_f32(const void *device_state_vector, int n_qubits, const int *host_subsystems,
                                          int subsystem_count, double *host_rho_ri_row_major);
int mipt_cuda_rho3_subsystems_complex_fermion_f64(const void *device_state_vector, int n_qubits,
                                                  const int *host_subsystems, int subsystem_count,
                                                  double *host_rho_ri_row_major);
int mipt_cuda_rho3_subsystems_complex_fermion_f32(const void *device_state_vector, int n_qubits,
                                                  const int *host_subsystems, int subsystem_count,
                                                  double *host_rho_ri_row_major);
int mipt_cuda_rho3_subsystems_complex_both_f64(const void *device_state_vector, int n_qubits,
                                               const int *host_subsystems, int subsystem_count,
                                               double *host_rho_ri_row_major, double *host_fermion_rho_ri_row_major);
int mipt_cuda_rho3_subsystems_complex_both_f32(const void *device_state_vector, int n_qubits,
                                               const int *host_subsystems, int subsystem_count,
                                               double *host_rho_ri_row_major, double *host_fermion_rho_ri_row_major);

/* Host-resident state vectors: copied to a reusable device buffer of the
 * calling thread, then the same reduction.
 * Replaces cpp/include/mipt/cuda/rho_reduce.hpp:78-126. */
int mipt_cuda_rho3_subsystems_complex_host_f64(const void *host_state_vector, int n_qubits,
                                               const int *host_subsystems, int subsystem_count,
                                               double *host_rho_ri_row_major);
int mipt_cuda_rho3_subsystems_complex_host_f32(const void *host_state_vector, int n_qubits,
                                               const int *host_subsystems, int subsystem_count,
                                               double *host_rho_ri_row_major);
int mipt_cuda_rho3_subsystems_complex_host_fermion_f64(const void *host_state_vector, int n_qubits,
                                                       const int *host_subsystems, int subsystem_count,
                                                       double *host_rho_ri_row_major);
int mipt_cuda_rho3_subsystems_complex_host_fermion_f32(const void *host_state_vector, int n_qubits,
                                                       const int *host_subsystems, int subsystem_count,
                                                       double *host_rho_ri_row_major);
int mipt_cuda_rho3_subsystems_complex_host_both_f64(const void *host_state_vector, int n_qubits,
                                                    const int *host_subsystems, int subsystem_count,
                                                    double *host_rho_ri_row_major,
                                                    double *host_fermion_rho_ri_row_major);
int mipt_cuda_rho3_subsystems_complex_host_both_f32(const void *host_state_vector, int n_qubits,
                                                    const int *host_subsystems, int subsystem_count,
                                                    double *host_rho_ri_row_major,
                                                    double *host_fermion_rho_ri_row_major);

/* --------------------------------------------- diagonal and parity passes */

/* Periodic-boundary Jordan-Wigner chain as one diagonal pass: amplitude *= -1
 * where bit control_qubit is set and popcount(index & string_mask) is odd.
 * Invalid arguments return -1. Asynchronous on the default stream.
 * Replaces cpp/include/mipt/cuda/cusv_diag.hpp:10-20. */
int mipt_cuda_jw_string_f32(void *device_state_vector, int n_qubits, int control_qubit, uint64_t string_mask);
int mipt_cuda_jw_string_f64(void *device_state_vector, int n_qubits, int control_qubit, uint64_t string_mask);
const char *mipt_cuda_cusv_diag_last_error(void);

/* Parity-sector encoding: an encoded index e (encoded_qubits = n-1 bits)
 * stands for the even-parity basis state whose bit n-1 is parity(e).
 * gate: 2x2 on bit `target` of every pair, `even_ri` where parity(e with the
 * target bit cleared) is 0, `odd_ri` where it is 1 (8 doubles each: row-major
 * (re, im) M00 M01 M10 M11). abs2: {even, odd} weights, fixed-order sums
 * (synchronous). collapse: keep parity(e) == outcome, scale 1/sqrt(weight).
 * expand: the encoded state in the low half of a 2^full_qubits buffer becomes
 * the full state in place. Invalid arguments return -1; other calls are
 * asynchronous on the default stream.
 * Replaces cpp/include/mipt/cuda/cusv_parity.hpp:23-60. */
int mipt_cuda_parity_gate_f32(void *device_state_vector, int encoded_qubits, int target, const double *even_ri,
                              const double *odd_ri);
int mipt_cuda_parity_gate_f64(void *device_state_vector, int encoded_qubits, int target, const double *even_ri,
                              const double *odd_ri);
int mipt_cuda_parity_abs2_f32(const void *device_state_vector, int encoded_qubits, double *host_weights);
int mipt_cuda_parity_abs2_f64(const void *device_state_vector, int encoded_qubits, double *host_weights);
int mipt_cuda_parity_collapse_f32(void *device_state_vector, int encoded_qubits, int outcome, double weight);
int mipt_cuda_parity_collapse_f64(void *device_state_vector, int encoded_qubits, int outcome, double weight);
int mipt_cuda_parity_expand_f32(void *device_state_vector, int full_qubits);
int mipt_cuda_parity_expand_f64(void *device_state_vector, int full_qubits);
const char *mipt_cuda_cusv_parity_last_error(void);

/* ----------------------------------------------------------- measurement */

/* Sequential single-site Born measurement with collapse; the collapse is
 * normalised by the raw branch weight. uniform_01 in [0,1).
 * Replaces cpp/include/mipt/cuda/free_energy_measure.hpp:13-29. */
int mipt_cuda_measure_collapse_f32(void *device_state_vector, int n_qubits, int measured_qubit, double uniform_01,
                                   int *outcome, double *realized_probability);
int mipt_cuda_measure_collapse_f64(void *device_state_vector, int n_qubits, int measured_qubit, double uniform_01,
                                   int *outcome, double *realized_probability);
const char *mipt_cuda_measure_collapse_last_error(void);

/* ---------------------------------------------------------------- engine */

/* One state vector driven layer by layer: the C form of the reference's
 * cuStateVec Engine (cpp/include/mipt/cusv/engine.hpp:100-582). */
typedef struct mipt_gb300_engine mipt_gb300_engine;

int mipt_gb300_engine_create(int fp64, mipt_gb300_engine **out);
void mipt_gb300_engine_destroy(mipt_gb300_engine *engine);
/* Allocate (if needed) and set |0...0>.                   engine.hpp:143-155 */
int mipt_gb300_engine_reset(mipt_gb300_engine *engine, int n_qubits);
/* Operate on a caller-owned device buffer (never freed).  engine.hpp:131-140 */
int mipt_gb300_engine_adopt(mipt_gb300_engine *engine, void *device_state_vector, int n_qubits);
void *mipt_gb300_engine_data(mipt_gb300_engine *engine);
int mipt_gb300_engine_set_from_host(mipt_gb300_engine *engine, const double *host_state_ri, int n_qubits);
int mipt_gb300_engine_to_host(mipt_gb300_engine *engine, double *host_state_ri);
/* Apply a layer of pairwise-disjoint two-qubit gates: bond j acts on qubits
 * (pairs[2j], pairs[2j+1]) with the row-major 4x4 complex matrix
 * matrices_ri[32j .. 32j+32) whose index bit 0 is pairs[2j].
 *                                                           engine.hpp:236-288 */
int mipt_gb300_engine_apply_bonds(mipt_gb300_engine *engine, const int *pairs, int bond_count,
                                  const double *matrices_ri);
/* Joint Born measurement of the ascending site list in chunks of chunk_bits
 * sites, one uniform per chunk; forced_outcomes (nullable, one per site)
 * replays a recorded outcome. Writes outcomes[i] for sites[i] and the
 * layer surprisal -log P.                                   engine.hpp:293-368 */
int mipt_gb300_engine_measure_layer(mipt_gb300_engine *engine, const int *sites, int site_count, int chunk_bits,
                                    const double *uniforms, const int *forced_outcomes, int *outcomes,
                                    double *surprisal);

/* ------------------------------------------------------ batched trajectories */

/* Per-layer or final observables of a batch (flags). */
#define MIPT_GB300_OBS_SVN_HALF 1  /* half-chain von Neumann entropy (bits) */
#define MIPT_GB300_OBS_S2_HALF 2   /* half-chain Renyi-2 entropy (bits) */
#define MIPT_GB300_OBS_TMI_VN 4    /* TMI of contiguous quarters, von Neumann */
#define MIPT_GB300_OBS_TMI_S2 8    /* TMI of contiguous quarters, Renyi-2 */

typedef struct mipt_gb300_batch_config
{
    int n_qubits;      /* even, 4..30 */
    int periods;       /* layers = 2 * periods */
    int closed;        /* 1: odd layers close the ring with bond (n-1, 0) */
    int fp64;          /* 0: FP32 state vectors (FP64 probabilities), 1: FP64 */
    int chunk_bits;    /* joint-measurement chunk, 1..20 (reference default 16) */
    int observables;   /* MIPT_GB300_OBS_* */
    int observe_every; /* evaluate observables after every k-th layer; 0 = final state only */
    int rho3;          /* 1: final three-site RDMs of the n ring triples */
    int fermion_trace; /* trace convention for RDMs / rho3 */
    int host_threads;  /* host sampler threads, 0 = all */
    int tile_qubits;   /* local qubits per pass tile, 0 = default */
    int tmi_cycles;    /* TMI quarters at cyclic offsets 0..tmi_cycles-1 (0 or 1: offset 0 only;
                          at most n/4) -- cpp/include/mipt/tmi/compute.hpp:89-113 */
    int lattice_x;     /* lattice_y > 1: 2-D four-colour brickwork on a lattice_x x lattice_y torus */
    int lattice_y;     /* (n_qubits = x * y, qubit = row * x + column; closed is ignored) */
    int circuit;       /* gate set, the reference's circ_type: 0 or 1 Haar brickwork; 2 FermionRPPU,
                          4 qRPPU (closed 1-D ring; layers = 2 * periods + 1, the last one the
                          reference's random extra even layer or an identity layer) --
                          cpp/include/mipt/circuits/rppu_layer.hpp:167-300 */
    int split_last;    /* RPPU: measure site n-1 as its own chunk after the others, as the
                          reference's parity-sector engine does (its default; MIPT_CUSV_PARITY=0
                          there is split_last = 0) -- cpp/include/mipt/cusv/engine.hpp:415-458 */
    int full_state;    /* RPPU with split_last: 0 keeps the reference's parity-sector encoding, 2^(n-1)
                          stored amplitudes per trajectory when every initial state has a definite parity
                          (cpp/include/mipt/cusv/parity.hpp:170-252); 1 always keeps the full 2^n state */
} mipt_gb300_batch_config;

typedef struct mipt_gb300_batch mipt_gb300_batch;

int mipt_gb300_batch_create(const mipt_gb300_batch_config *config, int capacity, mipt_gb300_batch **out);

/* Tile-shape autotuner (no reference counterpart). Times one cycle of every
 * layer colour of the geometry (passes only, fixed gates) on `trajectories`
 * scratch states for each candidate local-qubit count per pass tile (the
 * default, 14 FP32 / 13 FP64, and the two below it where they fit) and writes
 * the fastest to *best_tile; candidates[i] and ms_per_cycle[i] (nullable, at
 * least 3 entries) receive the timings, *candidate_count their number. A batch
 * created with tile_qubits = 0 takes its tile from a table measured this way
 * on GB300 (mipt_gb300/tune_tiles.py), or tunes live with MIPT_GB300_AUTOTUNE=1. */
int mipt_gb300_autotune_tile(int n_qubits, int fp64, int closed, int lattice_x, int lattice_y, int trajectories,
                             int *best_tile, int *candidates, double *ms_per_cycle, int *candidate_count);
void mipt_gb300_batch_destroy(mipt_gb300_batch *batch);

/* 1 if the prepared trajectories run on half-size parity-sector states (see
 * full_state in mipt_gb300_batch_config), else 0. */
int mipt_gb300_batch_parity_encoded(const mipt_gb300_batch *batch);

/* Test hook for the bounded device waits (no reference counterpart; the
 * reference's failure contract is its status ladder, cpp/src/cuda/tmi_cuda_svd.cu:203-215).
 * The next `count` FP32 pass launches that load tiles by TMA do not issue the
 * first tile load of their first CTA. That CTA's wait for the tile gives up
 * after well under a second, it returns without leaving a copy in flight,
 * and the batch's fetch reports MIPT_GB300_E_INTERNAL ("tile load wait timed
 * out"). The device stays usable: the next execute runs normally. */
int mipt_gb300_test_withhold_tile_loads(int count);

/* Draw `count` trajectories (trajectory i from seeds[i] with measurement
 * rate p[i]) on host threads exactly as the reference's HaarCircuit1D
 * (cpp/include/mipt/circuit.hpp:129-140,415-439) -- or, for circuit 2/4, its
 * RppuCircuit1D / QrppuCircuit1D (circuit.hpp:445-560) -- draws them, and
 * upload gates, measurement sites and uniforms. forced_outcomes (nullable,
 * [count][layers] bit masks) replays recorded outcomes. */
int mipt_gb300_batch_prepare_haar(mipt_gb300_batch *batch, const uint64_t *seeds, const double *p, int count,
                                  const uint64_t *forced_outcomes);
/* Free-energy protocol (cpp/apps/free_energy.cpp:460-533): the same Haar
 * brickwork, `2 * periods` layers drawn from the probed circuit workspace's
 * streams (cpp/include/mipt/probed.hpp:103-108,196-206) -- layer stream
 * mt19937(seed), measurement stream mt19937(seed ^ 0x9e3779b9) -- for the
 * 32-bit workspace seed of each trajectory. */
int mipt_gb300_batch_prepare_haar_workspace(mipt_gb300_batch *batch, const uint32_t *workspace_seeds,
                                            const double *p, int count);
/* Initial states for the next execute instead of |0...0>: trajectory i from
 * the reference's random initial-state draw (cpp/include/mipt/free_energy.hpp:
 * 125-222; kind 0 random product, 1 random Haar; fixed_parity for the
 * parity-preserving circuits) with an mt19937_64 seeded by seeds[i], drawn on
 * host threads; parity_sectors[i] (nullable) gets the sector or -1. Or one
 * trajectory from host amplitudes (host_ri[2^n][2]). Consumed by the next
 * mipt_gb300_batch_execute; other trajectories start from |0...0>. */
int mipt_gb300_batch_set_initial_states(mipt_gb300_batch *batch, const uint64_t *seeds, int kind, int fixed_parity,
                                        int count, int *parity_sectors);
int mipt_gb300_batch_set_initial_state(mipt_gb300_batch *batch, int index, const double *host_ri);
/* The same initial-state draw on the host: host_ri[2^n][2], amplitudes
 * rounded as an FP32 (fp64 = 0) or FP64 state stores them. */
int mipt_gb300_draw_initial_state(uint64_t seed, int n_qubits, int kind, int fixed_parity, int fp64,
                                  double *host_ri, int *parity_sector);
/* Observation schedule replacing observe_every: observables (and rho3 blocks
 * per point) after steps[i] layers, steps increasing in 0..layers, 0 = the
 * initial state; points = count (count = 0 restores observe_every). */
int mipt_gb300_batch_set_observation_steps(mipt_gb300_batch *batch, const int *steps, int count);
/* Run every layer of the prepared batch on the device, asynchronously on
 * `stream` (a cudaStream_t; NULL = default stream). */
int mipt_gb300_batch_execute(mipt_gb300_batch *batch, void *stream);
/* mipt_gb300_batch_execute through a CUDA graph (no reference counterpart;
 * the reference runs trajectories one at a time,
 * cpp/include/mipt/tmi/runner.hpp:269-378). The first call, and any call
 * after the batch's structure changed (trajectory count, which layers measure
 * and in how many chunks, forced outcomes, observation schedule, regions),
 * runs a normal execute and then captures a second one on a private stream;
 * later calls replay the captured graph with one launch. Batches whose initial
 * states were uploaded, or with profiling on, run a normal execute. */
int mipt_gb300_batch_execute_graph(mipt_gb300_batch *batch, void *stream);

/* Several batches (for example one per chain length of a mixed-length
 * workload) executed as the parallel branches of one CUDA graph, replayed
 * with one launch per call under the same rules as
 * mipt_gb300_batch_execute_graph. Results are fetched per batch. The group
 * does not own its batches; destroy it before them. */
typedef struct mipt_gb300_batch_group mipt_gb300_batch_group;
int mipt_gb300_batch_group_create(mipt_gb300_batch *const *batches, int count, mipt_gb300_batch_group **out);
int mipt_gb300_batch_group_execute(mipt_gb300_batch_group *group, void *stream);
void mipt_gb300_batch_group_destroy(mipt_gb300_batch_group *group);
/* Wait for the batch and copy results to host (each pointer nullable):
 *   measured[count][layers], outcomes[count][layers]  site bit masks
 *   surprisal[count][layers]                          -log P per layer
 *   obs[count][points][4]  (S_vN half, S_2 half, TMI vN, TMI S2; NaN where
 *                          not requested), points = layers/observe_every or 1
 *   rho3[count][n][128]                               final three-site RDMs */
int mipt_gb300_batch_fetch(mipt_gb300_batch *batch, uint64_t *measured, uint64_t *outcomes, double *surprisal,
                           double *obs, double *rho3);
/* prepare + execute + fetch in one synchronous call. */
/* Extra observable regions, evaluated at every observation point: the
 * entropy of order 1 (von Neumann) or 2 (Renyi-2) of the kept modes
 * modes[0..k). Add before mipt_gb300_batch_prepare_haar; *region_id gets the
 * region's column in mipt_gb300_batch_fetch_regions's out[count][points][regions]. */
int mipt_gb300_batch_add_region(mipt_gb300_batch *batch, const int *modes, int k, int order, int *region_id);
int mipt_gb300_batch_fetch_regions(mipt_gb300_batch *batch, double *out);
/* Three-site subsystems of the rho3 output (default: the n ring triples in
 * 1-D, the horizontal then vertical lattice triples in 2-D,
 * cpp/include/mipt/rdm.hpp:92-127). With observe_every > 0 the blocks are also
 * evaluated at every observation point: mipt_gb300_batch_fetch_rho3_points
 * writes out[count][points][subsystems][128]. */
int mipt_gb300_batch_set_rho3_subsystems(mipt_gb300_batch *batch, const int *triples, int subsystem_count);
int mipt_gb300_batch_rho3_subsystem_count(mipt_gb300_batch *batch);
int mipt_gb300_batch_fetch_rho3_points(mipt_gb300_batch *batch, double *out);

/* The bond list of colour 0..3 of the x by y lattice brickwork (pairs[2*count]) */
int mipt_gb300_lattice_bonds(int x, int y, int colour, int *pairs, int *count);
/* One 2-D Haar trajectory as the batch draws it (layer t uses colour t % 4):
 * outputs as mipt_gb300_draw_haar with `layers` layers. */
int mipt_gb300_draw_haar_lattice(uint64_t seed, int x, int y, int layers, double p, int chunk_bits,
                                 int *gates_per_layer, int *bond_q, double *bond_u, uint64_t *measured,
                                 double *uniforms, int *n_uniforms);

/* TMI at every cyclic offset, after mipt_gb300_batch_execute:
 * tmi[count][points][tmi_cycles] (order 1: von Neumann, 2: Renyi-2; the
 * batch must have been created with the matching MIPT_GB300_OBS_TMI_* flag).
 * Offset c uses A = [c, c+n/4), B, C, D the following quarters (mod n). */
int mipt_gb300_batch_fetch_tmi(mipt_gb300_batch *batch, int order, double *tmi);
int mipt_gb300_batch_run_haar(mipt_gb300_batch *batch, const uint64_t *seeds, const double *p, int count,
                              const uint64_t *forced_outcomes, uint64_t *measured, uint64_t *outcomes,
                              double *surprisal, double *obs, double *rho3);
/* Device pointer of trajectory i's state vector after execute. */
void *mipt_gb300_batch_state(mipt_gb300_batch *batch, int index);
/* Number of kernel launches the last execute enqueued. */
long long mipt_gb300_batch_launches(mipt_gb300_batch *batch);
/* Bracket each launch category of execute with CUDA events on its stream;
 * mipt_gb300_batch_kernel_stats then reports, for the last fetched execute,
 * device milliseconds and bracket counts per category:
 *   [0] layer passes (gates + fused histograms)  [1] stand-alone histograms
 *   [2] outcome sampling                          [3] observables
 *   [4] initialisation and final collapse */
int mipt_gb300_batch_set_profiling(mipt_gb300_batch *batch, int enable);
int mipt_gb300_batch_kernel_stats(mipt_gb300_batch *batch, double *ms, long long *launches);

/* ------------------------------------------------- GMN of three-qubit states */

/* Genuine multipartite negativity of rho3 blocks: the reference's monotone
 * witness SDP (cpp/src/analysis/gmn_mosek.c:14-40, python/gmn.py:236-358),
 *     min Re Tr(rho W)  s.t.  0 <= Q_m <= I, 0 <= W - PT_m(Q_m) <= I, m = 1..3,
 * GMN = -min (0 at or below 1e-8), solved for all `count` states at once by
 * ADMM on the GPU (FP32, or FP64 with fp64 = 1) with FP64 certificates: a
 * state is done when the primal value and a dual bound differ by at most
 * gap_tol and the box constraints are violated by at most feas_tol. */
typedef struct mipt_gb300_gmn_config
{
    int max_iter;    /* ADMM iterations per state at most */
    int check_every; /* iterations between FP64 certificates */
    double gap_tol;  /* duality gap, e.g. 1e-6 */
    double feas_tol; /* eigenvalue violation of the box constraints */
    double sigma;    /* ADMM penalty (0: 0.1) */
    int fp64;        /* 1: FP64 iterations */
} mipt_gb300_gmn_config;

/* rho: [count][128] row-major (re, im) 8x8 blocks (the rho3.bin payload
 * layout). warm_start (nullable): [count][7][128] floats, row-major (re, im)
 * W, Q_1..3, Z_1..3 (Z_m the duals of the W - PT_m(Q_m) constraints).
 * Outputs (nullable): gmn[count], gap[count] (at the last certificate),
 * iterations[count] (negative: max_iter reached without a certificate),
 * solution[count][7][128] (W, Q_1..3, Z_1..3, same layout). */
int mipt_gb300_gmn_solve(const mipt_gb300_gmn_config *config, const double *rho, int count,
                         const float *warm_start, double *gmn, double *gap, int *iterations, double *solution);
/* As mipt_gb300_gmn_solve with a per-state ADMM penalty sigma[count] (> 0). */
int mipt_gb300_gmn_solve_sigma(const mipt_gb300_gmn_config *config, const double *rho, int count,
                               const double *sigma, const float *warm_start, double *gmn, double *gap,
                               int *iterations, double *solution);

/* Negativity of the three single-qubit cuts of each 8x8 state (the
 * bipartite-negativity prefilter of the reference's gmn.exe,
 * cpp/apps/gmn.cpp:413-424, compute_min_bipartite_negativity_8x8_cpp
 * cpp/src/analysis/fgmn.cpp:1443-1453 over cut_negativity
 * cpp/include/mipt/analysis/cut_negativity.hpp:139-200): negativity[3 * i + m]
 * = (||rho_i^{T_m}||_1 - 1) / 2 for the partial transpose on qubit m (index
 * bit m), values in (-1e-10, 0) set to 0. FP64 Jacobi on the GPU.
 * rho: [count][128] as for mipt_gb300_gmn_solve. */
int mipt_gb300_cut_negativities(const double *rho, int count, double *negativity);

/* Learned warm start: a multilayer perceptron (dims[0] inputs, ReLU between
 * layers, linear output) trained and evaluated on the GPU by the library's
 * own kernels. Weights are FP32 master copies (Adam) and BF16 copies that
 * every product reads with FP32 accumulation. Parameters are laid out layer
 * by layer: W_l (dims[l+1] x dims[l], row-major), then b_l. No reference
 * counterpart (the reference has no learned component). */
typedef struct mipt_gb300_mlp mipt_gb300_mlp;
int mipt_gb300_mlp_create(const int *dims, int n_dims, uint64_t seed, mipt_gb300_mlp **out);
void mipt_gb300_mlp_destroy(mipt_gb300_mlp *mlp);
long long mipt_gb300_mlp_param_count(const mipt_gb300_mlp *mlp);
int mipt_gb300_mlp_get_params(mipt_gb300_mlp *mlp, float *params);
int mipt_gb300_mlp_set_params(mipt_gb300_mlp *mlp, const float *params);
/* y[n][dims.back()] from x[n][dims[0]] (host arrays). */
int mipt_gb300_mlp_forward(mipt_gb300_mlp *mlp, const float *x, int n, float *y);
/* Mean squared error of the n rows and its gradient w.r.t. every parameter. */
int mipt_gb300_mlp_loss_grad(mipt_gb300_mlp *mlp, const float *x, const float *target, int n, double *loss,
                             float *grad);
/* Adam epochs over the n rows in shuffled batches; final_loss = the MSE of
 * the last batch of the last epoch. */
int mipt_gb300_mlp_train(mipt_gb300_mlp *mlp, const float *x, const float *target, int n, int epochs, int batch,
                         float learning_rate, uint64_t shuffle_seed, double *final_loss);

/* ------------------------------------------ free fermions (covariance) */

/* Monitored free-fermion circuit on the Majorana covariance matrix of N
 * modes (no counterpart in the reference, which simulates fermionic circuits
 * only as Jordan-Wigner state vectors): layer t applies Haar SO(4) rotations
 * to the four Majoranas of mode pairs (m, m+1 mod N), m = t%2, t%2+2, ...,
 * then measures each mode's parity i g_{2j} g_{2j+1} with probability p.
 * Same seed streams as the Haar path. */
typedef struct mipt_gb300_ff_config
{
    int n_modes;          /* even, 4..128 */
    int depth;            /* layers */
    int closed;           /* 1: odd layers close the ring with modes (N-1, 0) */
    int repurify_every;   /* FP64 re-purification every k layers (0: final only) */
    int n_blocks;         /* entropies of the mode blocks [0, block_len[i]) */
    const int *block_len;
    int host_threads;     /* sampler threads, 0 = all */
    int fp64;             /* 1: Gamma evolves in FP64 (the plain method); 0: FP32 with FP64
                           * denominators, re-purification and eigensolves */
} mipt_gb300_ff_config;

/* Runs `count` trajectories (seeds[i], rate p[i]). forced (nullable,
 * [count][depth][N], +-1 for the i-th measured mode of a layer) replays
 * outcomes. Outputs (nullable): outcomes/probs [count][depth][N] (+-1 and the
 * realised probability per measured mode, 0 padding), gamma_out
 * [count][2N][2N] final covariance (FP64, re-purified), s_blocks
 * [count][n_blocks] and tmi [count] (contiguous quarters), in bits. */
int mipt_gb300_ff_run(const mipt_gb300_ff_config *config, const uint64_t *seeds, const double *p, int count,
                      const int *forced, int *outcomes, double *probs, double *gamma_out, double *s_blocks,
                      double *tmi);

/* Host-side seeding helpers (the reference's splitmix64 streams,
 * cpp/include/mipt/types.hpp:262-273). */
uint64_t mipt_gb300_splitmix64(uint64_t value);
uint64_t mipt_gb300_trajectory_seed(uint64_t master, uint64_t index);

/* Draw one Haar trajectory on the host (no GPU needed): gates_per_layer[L],
 * bond_q[L][n/2][2], bond_u[L][n/2][32] (row-major 4x4, re/im), measured[L]
 * site masks, uniforms[] one per measurement chunk (n_uniforms returned). */
int mipt_gb300_draw_haar(uint64_t seed, int n_qubits, int periods, double p, int closed, int chunk_bits,
                         int *gates_per_layer, int *bond_q, double *bond_u, uint64_t *measured, double *uniforms,
                         int *n_uniforms);

/* One RPPU / qRPPU trajectory as the batch draws it (circuit 2 or 4; the
 * draw is the same, the batch adds the fermionic closure string for 2):
 * 2*periods + 1 layers in the plan's bond order (odd layers end with the
 * closure bond (n-1, 0)); a missing extra even layer is identity gates.
 * workspace = 1: the probed workspace's streams from the low 32 bits of seed,
 * 2*periods layers and an identity last layer. Outputs as mipt_gb300_draw_haar. */
int mipt_gb300_draw_rppu(uint64_t seed, int n_qubits, int periods, double p, int chunk_bits, int split_last,
                         int workspace, int *gates_per_layer, int *bond_q, double *bond_u, uint64_t *measured,
                         double *uniforms, int *n_uniforms);
/* The free-energy workspace draw of one trajectory on the host (closed ring,
 * `layers` layers; outputs as mipt_gb300_draw_haar). */
int mipt_gb300_draw_haar_workspace(uint32_t seed, int n_qubits, int layers, double p, int chunk_bits,
                                   int *gates_per_layer, int *bond_q, double *bond_u, uint64_t *measured,
                                   double *uniforms, int *n_uniforms);

#ifdef __cplusplus
}
#endif

#endif /* MIPT_GB300_H */
