// State-vector engine for batches of monitored-circuit trajectories.
//
// Layout in HBM: trajectory b's state is the contiguous array
// states[b * 2^n .. (b+1) * 2^n) of interleaved complex amplitudes (float2 for
// the FP32 path, double2 for FP64); qubit q is bit q of the amplitude index
// (the little-endian convention of the reference, cpp/include/mipt/cusv/matrix.hpp:5-13).
//
// One brickwork layer is applied in one or more tiled passes. A pass loads a
// tile of 2^k amplitudes whose local qubits hold every bond the pass applies,
// applies those bonds in shared memory and stores the tile back, so each pass
// is one read and one write of the state. The last pass of a layer also
// accumulates the Born histogram of the layer's measured sites; the measured
// outcome is sampled on the device and the collapse is applied while the next
// pass loads its tiles, so a measurement costs no extra sweep of the state.
#pragma once

#include "common.cuh"

#include <cuda_runtime.h>
#include <vector>

namespace mg
{

struct Bond
{
    int q0, q1; // matrix index bit 0 <-> q0, bit 1 <-> q1; q1 = -1: parity-selected 2x2 gate on q0
};

// One register round of a pass: every thread holds 2^rb amplitudes whose
// register-index bit i is local tile bit reg[i]; thread-index bit i is local
// bit tid[i] (the first five, one per residue mod 5, are the warp lanes).
// slot[s] >= 0 applies pass gate slot[s] on register bits (2s, 2s+1).
struct Round
{
    std::int8_t reg[6];
    std::int8_t tid[10];
    std::int16_t slot[3];
};

constexpr int kMaxRounds = 8;

// Register round of the two-CTA cluster kernel: the 2^14-amplitude tile is
// split between the two CTAs of a cluster by tile bit x (CTA rank = bit x);
// each thread holds 32 amplitudes (register bits reg[0..5)), thread-index bit
// i is tile bit tid[i]. slot[s] >= 0 applies pass gate slot[s] on register
// bits (2s, 2s+1).
struct ClusterRound
{
    std::int8_t reg[6];
    std::int8_t tid[8];
    std::int8_t x;
    std::int16_t slot[3];
};

// TMA view of a pass's tiles: dimension d of the tensor map covers global
// index bits [lo[d], lo[d] + bits[d]) of the batch of states (the last one
// also the trajectory bits above bit n); local runs are whole box dimensions.
struct TileTma
{
    int rank;
    int lo[5];
    int bits[5];
};

struct PassPlan
{
    PassGeom geom;
    PassGates gates;
    int rounds; // 0: tile too small for register rounds (shared-memory kernel)
    int rb;     // register bits per thread
    Round round[kMaxRounds];
    int cluster_rounds; // > 0: FP32 two-CTA cluster schedule available
    int cluster_rb;     // register bits per thread of that schedule
    ClusterRound cround[kMaxRounds];
    PassGeom hgeom; // histogram geometry of one CTA's half tile (cluster kernel)
};

// Splits one layer's bonds into tiled passes of at most kmax local qubits
// with at least cmin contiguous low qubits per tile (for coalescing), and
// schedules each pass's bonds into register rounds of rb register bits.
std::vector<PassPlan> plan_layer(int n, const std::vector<Bond> &bonds, int kmax, int cmin, int rb);

// Geometry of the per-tile histogram partials a pass writes when it fuses
// the layer's Born histogram (a half tile for the cluster kernel).
const PassGeom &fused_hist_geometry(const PassPlan &p, bool fp32);

// Register bits per thread of the register-round pass kernel (FP32: 6 by
// default, MIPT_GB300_RB=5 for 32 amplitudes per thread; FP64: 5).
int fp32_register_bits();
template <typename Real> inline int register_bits() { return sizeof(Real) == 4 ? fp32_register_bits() : 5; }

// Tile geometry used for a stand-alone histogram of the sites in `chunk`:
// low contiguous qubits, then as many unmeasured qubits as fit, so that few
// measured sites are tile-local.
__host__ __device__ void histogram_geometry(int n, int kmax, int cmin, std::uint64_t chunk, PassGeom &g);

// Device scratch needed per trajectory for histogram partials.
constexpr std::size_t kHistScratch = std::size_t{1} << 20; // doubles
constexpr int kMaxChunks = 8;

// Per-(trajectory, layer) measurement record on the device.
struct LayerMeas
{
    std::uint64_t chunk[kMaxChunks]; // measured sites of each chunk (bit = qubit)
    double uniform[kMaxChunks];
    int nchunks;
    int pad;
};

struct LayerResult
{
    std::uint64_t outcome;   // bit q = measured value of site q (0 where unmeasured)
    double surprisal;        // -log P(joint outcome of the layer)
    double prob[kMaxChunks]; // branch / total of each chunk
};

template <typename Real>
struct EngineLaunch
{
    Cx<Real> *states;
    std::uint64_t dim;
    int batch;
};

// Kernel launchers (engine.cu).
template <typename Real>
cudaError_t launch_init_zero(Cx<Real> *states, std::uint64_t dim, int batch, cudaStream_t s);

// collapse_in (if any) is applied as the tiles load: amplitudes whose bits on
// mask & col_keep differ from value become zero, the others are scaled by the
// collapse's scale (col_scaled) or kept as they are. sparse: the pass visits
// only the tiles that agree with collapse_in's outcome on the pass's
// non-local measured bits (the others are zero before and after the pass and
// are left untouched in memory); the layer's next pass must then load with
// col_keep = those non-local qubits and col_scaled = 0. Needs a register-round
// plan (sparse_pass_supported) and no fused histogram. parity_mode: the states
// are parity-sector states (collapses may carry a parity condition, the plan
// may hold parity-selected gates); it selects the kernel variant built for
// them.
template <typename Real>
cudaError_t launch_pass(Cx<Real> *states, int batch, const PassPlan &plan, const Cx<Real> *layer_gates,
                        std::size_t gate_stride, const Collapse *collapse_in, std::size_t collapse_stride,
                        const LayerMeas *meas, std::size_t meas_stride, double *partials, int fuse_hist,
                        int *err, cudaStream_t s, std::uint64_t col_keep = ~0ull, int col_scaled = 1,
                        int sparse = 0, int parity_mode = 0);

// Test hook: the next `count` TMA-fed pass launches do not issue CTA 0's
// first tile load; its bounded wait (well under a second) runs out, the CTA
// sets bit 8 of the error flag and returns. No load is left in flight.
void set_withheld_tile_loads(int count);

// Whether launch_pass accepts sparse / residual-collapse arguments for this
// plan and batch size.
bool sparse_pass_supported(const PassPlan &plan, bool fp32, int batch);

// Non-local qubits of a pass (mask).
inline std::uint64_t nonlocal_mask(const PassGeom &g)
{
    std::uint64_t m = 0;
    for (int i = 0; i < g.n_nl; ++i) m |= 1ull << g.nl[i];
    return m;
}

template <typename Real>
cudaError_t launch_hist(const Cx<Real> *states, int batch, int n, int kmax, int cmin, int chunk_index,
                        const Collapse *collapse_in, std::size_t collapse_stride, const LayerMeas *meas,
                        std::size_t meas_stride, double *partials, bool direct, cudaStream_t s,
                        const signed char *sector = nullptr);

// Samples (or replays) the outcome of chunk `chunk_index` from the partial
// histograms, writes the combined collapse of the layer and the outcome.
// Parity-sector states (n stored qubits): a chunk at bit n is the chain's top
// qubit; sector[b] (0 or 1) is trajectory b's total parity, its outcome lands
// at bit n of the outcome mask and its collapse is a parity condition.
cudaError_t launch_measure(int batch, int n, const PassGeom *fused_geom, int kmax, int cmin, int chunk_index,
                           const LayerMeas *meas, std::size_t meas_stride, const double *partials,
                           double *bins_scratch, std::size_t bins_stride, const std::uint64_t *forced,
                           std::size_t forced_stride,
                           Collapse *collapse_out, std::size_t collapse_stride, LayerResult *result,
                           std::size_t result_stride, int *error_flag, cudaStream_t s,
                           const signed char *sector = nullptr);

template <typename Real>
cudaError_t launch_collapse(Cx<Real> *states, std::uint64_t dim, int batch, const Collapse *collapse,
                            std::size_t collapse_stride, cudaStream_t s);

// Host helper: local positions of `chunk` within geometry g.
int local_measured_count(const PassGeom &g, std::uint64_t chunk);

} // namespace mg
