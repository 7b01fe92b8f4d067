// Reduced density matrices, purities, entropies and three-site blocks of
// batched state vectors.
#pragma once

#include "common.cuh"

#include <cuda_runtime.h>
#include <vector>

namespace mg
{

// One reduced-density-matrix request: rho = M M^H over the retained modes
// kept[0..k) (row index bit i <-> kept[i]); the environment is the
// complement in ascending mode order (the reference's Schmidt layout,
// cpp/include/mipt/cuda/schmidt_gram.cuh:13-19). With `fermion`, M[r][e]
// changes sign once per occupied environment mode below each occupied kept
// mode (schmidt_gram.cuh:196-249).
struct GramJob
{
    int traj;
    int k;
    int fermion;
    int rows_fastest; // kept set contains qubit 0 -> gather along rows
    std::int8_t kept[32];
    std::int8_t env[32];
    std::uint64_t below[32];
};

GramJob make_gram_job(int traj, int n, const int *kept, int k, bool fermion);

constexpr int kGramTile = 64;

// Number of lower-triangle 64x64 tiles of a d x d matrix.
inline int gram_tiles(int k)
{
    const int t = (k >= 6) ? (1 << (k - 6)) : 1;
    return t * (t + 1) / 2;
}

// rho for every job (all jobs share k): full FP64 d x d Hermitian matrices
// written to rho_out[job][d][d] (row-major complex). With a pending collapse,
// non-fermionic jobs leave out the sites it measured (the state is a product
// on them, so the spectrum and purity are those of the reduced matrix): rho
// then holds that 2^k' x 2^k' matrix in its leading rows and columns, zeros
// elsewhere, and dims_out[job] (nullable) receives 2^k'.
template <typename Real>
cudaError_t gram_rho(const Cx<Real> *states, int n, const GramJob *d_jobs, int njobs, int k,
                     const Collapse *collapse, std::size_t collapse_stride, double *rho_out, void *scratch,
                     std::size_t scratch_bytes, cudaStream_t s, int *dims_out = nullptr);

// Purity Tr(rho^2) of every job without materialising rho.
template <typename Real>
cudaError_t gram_purity(const Cx<Real> *states, int n, const GramJob *d_jobs, int njobs, int k,
                        const Collapse *collapse, std::size_t collapse_stride, double *purity_out, void *scratch,
                        std::size_t scratch_bytes, cudaStream_t s);

std::size_t gram_scratch_bytes(int n, int k, int njobs, bool rho);

// Purity of FP32 states with FP64 accumulation and no environment split:
// one block per lower-triangle tile writes its partial into
// scratch[job][tile] (gram_tiles(k) doubles per job, each written once),
// then a fixed-order row sum writes purity_out[job].
cudaError_t gram_purity_f64acc(const Cx<float> *states, int n, const GramJob *d_jobs, int njobs, int k,
                               double *purity_out, void *scratch, std::size_t scratch_bytes, cudaStream_t s);

// Purity through the tensor-core (tcgen05, 3xTF32) Gram, FP32 states only;
// needs 7 <= k <= 16 and n - k >= 4. err receives bit 4 if a pipeline wait
// timed out (the kernel then returns without a result). tma_traj_count > 0
// asserts that every job keeps modes 0..k-1 in order and that `states` holds
// tma_traj_count state vectors; the operands then arrive by TMA.
bool gram_tc_supported(int n, int k);
std::size_t gram_tc_scratch_bytes(int k, int njobs);
// With tma_traj_count > 0, k <= gram_tc_presplit_max_k() and a `rows` buffer of at least
// gram_tc_rows_bytes_per_job(n) bytes (16-byte aligned), the operands are
// first split into TF32 hi/lo rows (jobs in groups that fit the buffer) and
// the Gram streams them by TMA alone; MIPT_GB300_TC_PRESPLIT=0 turns that off.
bool gram_tc_presplit_enabled();
int gram_tc_presplit_max_k(); // largest k for the pre-split path (MIPT_GB300_TC_PRESPLIT_MAX_K, default 14)
std::size_t gram_tc_rows_bytes_per_job(int n);
cudaError_t gram_purity_tc(const Cx<float> *states, int n, const GramJob *d_jobs, int njobs, int k,
                           const Collapse *collapse, std::size_t collapse_stride, double *purity_out, void *scratch,
                           std::size_t scratch_bytes, int *err, cudaStream_t s, int tma_traj_count = 0,
                           void *rows = nullptr, std::size_t rows_bytes = 0);

// Purity of full matrices rho[job][d][d].
cudaError_t purity_of(const double *rho, int d, int njobs, double *purity_out, cudaStream_t s);

// Von Neumann entropies (bits) of Hermitian matrices rho[job][d][d] for
// d <= 64, by a parallel-order complex Jacobi eigensolver in FP64.
cudaError_t jacobi_entropy(const double *rho, int d, int njobs, double *entropy_out, double *eig_out,
                           cudaStream_t s);

// Von Neumann entropies (bits) of Hermitian matrices rho[job][d][d]
// (destroyed) for 2 <= d <= 4096: FP64 Householder tridiagonalisation (one
// CTA per matrix, or, with fewer matrices than resident CTAs, several CTAs
// per matrix in a cooperative launch), then implicit QL, one thread per
// matrix (eigen.cu).
// eig_out (nullable) receives each matrix's eigenvalues (unordered);
// scratch holds hermitian_eig_scratch_doubles(d, njobs) doubles. A QL
// iteration limit that runs out sets bit 1 of *err and writes NaN; a timed-out
// barrier between the CTAs of one matrix sets bit 2.
// dims (nullable): the rows of each matrix that hold data (the rest of
// its d x d block is zero); the reduction and QL then run on those only.
std::size_t hermitian_eig_scratch_doubles(int d, int njobs);
cudaError_t hermitian_eig_entropy(double *rho, int d, int njobs, double *entropy_out, double *eig_out,
                                  double *scratch, int *err, cudaStream_t s, const int *dims = nullptr);

// Three-site RDMs of every trajectory, for `count` triples subs[3*i..].
// out[traj][i][8][8] complex row-major. fermion selects the fermionic trace
// of the reference's three-site sweep (cpp/src/cuda/rho_reduce.cu:49-110).
template <typename Real>
cudaError_t rho3_sweep(const Cx<Real> *states, int n, int batch, const int *d_subs, int count, int fermion,
                       const Collapse *collapse, std::size_t collapse_stride, double *out, void *scratch,
                       std::size_t scratch_bytes, cudaStream_t s);
std::size_t rho3_scratch_bytes(int n, int batch, int count);

// S_2 = -log2(purity) with the reference's clamps (purity >= 1 -> 0,
// |S| < 1e-12 -> 0; cpp/include/mipt/tmi/linalg.hpp:134-141,201-208).
__host__ __device__ inline double renyi2_from_purity(double purity)
{
    if (!(purity > 0.0) || purity >= 1.0) return 0.0;
    const double s = -log2(purity);
    return (s < 1e-12 && s > -1e-12) ? 0.0 : s;
}

} // namespace mg
