// Diagonal Jordan-Wigner sign pass and the parity-sector passes of the
// state-vector engine: the reference's C ABI of cpp/include/mipt/cuda/
// cusv_diag.hpp and cusv_parity.hpp (paths inside the reference project).
//
// Semantics kept from the reference:
//   jw_string: amplitude *= -1 where bit `control` is set and
//     popcount(index & mask) is odd (cusv_diag.hpp:3-9); mask 0 is a no-op.
//   parity sector: an encoded index e of n-1 bits stands for the even-parity
//     basis state with b_{n-1} = parity(e) (cusv_parity.hpp:3-18).
//   parity_gate: on every pair (i0, i0 | 1<<target) with bit `target` of i0
//     clear, the 2x2 `even` (parity(i0) = 0) or `odd` (parity(i0) = 1)
//     matrix, row-major (re, im) M00 M01 M10 M11 (cusv_parity.hpp:25-35).
//   parity_abs2: {sum |a_e|^2 over even parity(e), over odd}, summed in a
//     fixed order (cusv_parity.hpp:37-43).
//   parity_collapse: keep parity(e) == outcome, scale by 1/sqrt(weight).
//   parity_expand: in place, e -> e | 2^(n-1) when parity(e) is odd.
// Invalid arguments return -1 with a message in the *_last_error string;
// launch failures return the cudaError_t. Passes other than abs2 run
// asynchronously on the default stream, as the reference's do.
//
// All passes are HBM-bound streams: consecutive threads own consecutive
// amplitudes (or pairs), grids are sized in multiples of the 152 SMs.
#include "mipt_gb300.h"

#include "common.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

namespace
{
using mg::Cx;

thread_local char g_diag_error[256] = {0};
thread_local char g_parity_error[256] = {0};

constexpr int kThreads = 256;
constexpr int kReduceBlocks = 152 * 4;

int grid_for(std::uint64_t work)
{
    const std::uint64_t need = (work + kThreads - 1) / kThreads;
    const std::uint64_t cap = 152ull * 32;
    return static_cast<int>(need < 1 ? 1 : (need < cap ? need : cap));
}

int launch_status(char *buf, const char *what)
{
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return 0;
    std::snprintf(buf, 256, "%s failed: %s", what, cudaGetErrorString(e));
    return static_cast<int>(e);
}

__device__ __forceinline__ bool odd_parity(std::uint64_t x) { return (__popcll(x) & 1) != 0; }

template <typename Real>
__global__ void k_jw_string(Cx<Real> *__restrict__ psi, std::uint64_t dim, std::uint64_t control, std::uint64_t mask)
{
    const std::uint64_t stride = static_cast<std::uint64_t>(gridDim.x) * blockDim.x;
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < dim; i += stride)
        if ((i & control) && odd_parity(i & mask))
        {
            Cx<Real> v = psi[i];
            v.re = -v.re;
            v.im = -v.im;
            psi[i] = v;
        }
}

template <typename Real> struct Mat2
{
    Real v[16]; // even M00..M11 (re, im), then odd
};

template <typename Real>
__global__ void k_parity_gate(Cx<Real> *__restrict__ psi, std::uint64_t pairs, int target, Mat2<Real> g)
{
    const std::uint64_t stride = static_cast<std::uint64_t>(gridDim.x) * blockDim.x;
    const std::uint64_t low = (1ull << target) - 1ull;
    for (std::uint64_t p = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; p < pairs; p += stride)
    {
        const std::uint64_t i0 = ((p & ~low) << 1) | (p & low);
        const std::uint64_t i1 = i0 | (1ull << target);
        const Real *m = g.v + (odd_parity(i0) ? 8 : 0);
        const Cx<Real> a = psi[i0], b = psi[i1];
        Cx<Real> x, y;
        x.re = m[0] * a.re - m[1] * a.im + m[2] * b.re - m[3] * b.im;
        x.im = m[0] * a.im + m[1] * a.re + m[2] * b.im + m[3] * b.re;
        y.re = m[4] * a.re - m[5] * a.im + m[6] * b.re - m[7] * b.im;
        y.im = m[4] * a.im + m[5] * a.re + m[6] * b.im + m[7] * b.re;
        psi[i0] = x;
        psi[i1] = y;
    }
}

// Per-block {even, odd} partials in FP64 (FP32 squares are exact in FP64),
// grid-stride order and a fixed shared-memory tree.
template <typename Real>
__global__ void k_parity_abs2(const Cx<Real> *__restrict__ psi, std::uint64_t dim, double *__restrict__ part)
{
    __shared__ double se[kThreads], so[kThreads];
    double e = 0.0, o = 0.0;
    const std::uint64_t stride = static_cast<std::uint64_t>(gridDim.x) * blockDim.x;
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < dim; i += stride)
    {
        const Cx<Real> v = psi[i];
        const double w = static_cast<double>(v.re) * v.re + static_cast<double>(v.im) * v.im;
        if (odd_parity(i))
            o += w;
        else
            e += w;
    }
    se[threadIdx.x] = e;
    so[threadIdx.x] = o;
    __syncthreads();
    for (int k = kThreads / 2; k > 0; k /= 2)
    {
        if (threadIdx.x < k)
        {
            se[threadIdx.x] += se[threadIdx.x + k];
            so[threadIdx.x] += so[threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        part[2 * blockIdx.x] = se[0];
        part[2 * blockIdx.x + 1] = so[0];
    }
}

__global__ void k_sum_pairs(const double *__restrict__ part, int blocks, double *__restrict__ out)
{
    __shared__ double se[kThreads], so[kThreads];
    double e = 0.0, o = 0.0;
    for (int b = threadIdx.x; b < blocks; b += blockDim.x)
    {
        e += part[2 * b];
        o += part[2 * b + 1];
    }
    se[threadIdx.x] = e;
    so[threadIdx.x] = o;
    __syncthreads();
    for (int k = kThreads / 2; k > 0; k /= 2)
    {
        if (threadIdx.x < k)
        {
            se[threadIdx.x] += se[threadIdx.x + k];
            so[threadIdx.x] += so[threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        out[0] = se[0];
        out[1] = so[0];
    }
}

template <typename Real>
__global__ void k_parity_collapse(Cx<Real> *__restrict__ psi, std::uint64_t dim, int outcome, Real scale)
{
    const std::uint64_t stride = static_cast<std::uint64_t>(gridDim.x) * blockDim.x;
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < dim; i += stride)
    {
        Cx<Real> v = psi[i];
        const bool keep = static_cast<int>(odd_parity(i)) == outcome;
        v.re = keep ? v.re * scale : Real(0);
        v.im = keep ? v.im * scale : Real(0);
        psi[i] = v;
    }
}

template <typename Real> __global__ void k_parity_expand(Cx<Real> *__restrict__ psi, std::uint64_t half)
{
    const std::uint64_t stride = static_cast<std::uint64_t>(gridDim.x) * blockDim.x;
    for (std::uint64_t e = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; e < half; e += stride)
    {
        const Cx<Real> v = psi[e];
        const Cx<Real> z{Real(0), Real(0)};
        if (odd_parity(e))
        {
            psi[e | half] = v;
            psi[e] = z;
        }
        else
        {
            psi[e | half] = z;
        }
    }
}

bool bad_state(const void *state, int qubits)
{
    if (state == nullptr || qubits < 1 || qubits > 62)
    {
        std::snprintf(g_parity_error, sizeof(g_parity_error), "Invalid parity-sector argument.");
        return true;
    }
    return false;
}

template <typename Real> int jw_string(void *state, int n, int control, std::uint64_t mask)
{
    g_diag_error[0] = '\0';
    if (state == nullptr || n < 1 || n >= 63 || control < 0 || control >= n)
    {
        std::snprintf(g_diag_error, sizeof(g_diag_error), "Invalid JW-string argument.");
        return -1;
    }
    if (mask == 0) return 0;
    const std::uint64_t dim = 1ull << n;
    k_jw_string<Real><<<grid_for(dim), kThreads>>>(static_cast<Cx<Real> *>(state), dim, 1ull << control, mask);
    return launch_status(g_diag_error, "JW-string kernel launch");
}

template <typename Real> int parity_gate(void *state, int nq, int target, const double *even, const double *odd)
{
    g_parity_error[0] = '\0';
    if (bad_state(state, nq) || !even || !odd || target < 0 || target >= nq)
    {
        std::snprintf(g_parity_error, sizeof(g_parity_error), "Invalid parity-gate argument.");
        return -1;
    }
    Mat2<Real> g;
    for (int k = 0; k < 8; ++k)
    {
        g.v[k] = static_cast<Real>(even[k]);
        g.v[8 + k] = static_cast<Real>(odd[k]);
    }
    const std::uint64_t pairs = 1ull << (nq - 1);
    k_parity_gate<Real><<<grid_for(pairs), kThreads>>>(static_cast<Cx<Real> *>(state), pairs, target, g);
    return launch_status(g_parity_error, "parity-gate kernel launch");
}

// Partials of the calling thread (the reference keeps one per host thread).
double *abs2_scratch(cudaError_t &e)
{
    static thread_local double *buf = nullptr;
    e = cudaSuccess;
    if (!buf) e = cudaMalloc(&buf, sizeof(double) * (2 * kReduceBlocks + 2));
    return e == cudaSuccess ? buf : nullptr;
}

template <typename Real> int parity_abs2(const void *state, int nq, double *weights)
{
    g_parity_error[0] = '\0';
    if (bad_state(state, nq) || weights == nullptr) return -1;
    cudaError_t e;
    double *part = abs2_scratch(e);
    if (!part)
    {
        std::snprintf(g_parity_error, sizeof(g_parity_error), "cudaMalloc(parity partials) failed: %s",
                      cudaGetErrorString(e));
        return static_cast<int>(e);
    }
    const std::uint64_t dim = 1ull << nq;
    const int blocks = static_cast<int>(std::min<std::uint64_t>(kReduceBlocks, (dim + kThreads - 1) / kThreads));
    k_parity_abs2<Real><<<blocks, kThreads>>>(static_cast<const Cx<Real> *>(state), dim, part);
    if (const int rc = launch_status(g_parity_error, "parity-abs2 kernel launch")) return rc;
    k_sum_pairs<<<1, kThreads>>>(part, blocks, part + 2 * kReduceBlocks);
    if (const int rc = launch_status(g_parity_error, "parity-abs2 finalize launch")) return rc;
    e = cudaMemcpy(weights, part + 2 * kReduceBlocks, 2 * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
    {
        std::snprintf(g_parity_error, sizeof(g_parity_error), "cudaMemcpy(parity weights) failed: %s",
                      cudaGetErrorString(e));
        return static_cast<int>(e);
    }
    return 0;
}

template <typename Real> int parity_collapse(void *state, int nq, int outcome, double weight)
{
    g_parity_error[0] = '\0';
    if (bad_state(state, nq) || (outcome != 0 && outcome != 1) || !(weight > 0.0))
    {
        std::snprintf(g_parity_error, sizeof(g_parity_error), "Invalid parity-collapse argument.");
        return -1;
    }
    const std::uint64_t dim = 1ull << nq;
    k_parity_collapse<Real><<<grid_for(dim), kThreads>>>(static_cast<Cx<Real> *>(state), dim, outcome,
                                                         static_cast<Real>(1.0 / std::sqrt(weight)));
    return launch_status(g_parity_error, "parity-collapse kernel launch");
}

template <typename Real> int parity_expand(void *state, int n)
{
    g_parity_error[0] = '\0';
    if (bad_state(state, n) || n < 2)
    {
        std::snprintf(g_parity_error, sizeof(g_parity_error), "Invalid parity-expand argument.");
        return -1;
    }
    const std::uint64_t half = 1ull << (n - 1);
    k_parity_expand<Real><<<grid_for(half), kThreads>>>(static_cast<Cx<Real> *>(state), half);
    return launch_status(g_parity_error, "parity-expand kernel launch");
}
} // namespace

extern "C" {
int mipt_cuda_jw_string_f32(void *s, int n, int control, std::uint64_t mask)
{
    return jw_string<float>(s, n, control, mask);
}
int mipt_cuda_jw_string_f64(void *s, int n, int control, std::uint64_t mask)
{
    return jw_string<double>(s, n, control, mask);
}
const char *mipt_cuda_cusv_diag_last_error(void) { return g_diag_error; }

int mipt_cuda_parity_gate_f32(void *s, int nq, int t, const double *e, const double *o)
{
    return parity_gate<float>(s, nq, t, e, o);
}
int mipt_cuda_parity_gate_f64(void *s, int nq, int t, const double *e, const double *o)
{
    return parity_gate<double>(s, nq, t, e, o);
}
int mipt_cuda_parity_abs2_f32(const void *s, int nq, double *w) { return parity_abs2<float>(s, nq, w); }
int mipt_cuda_parity_abs2_f64(const void *s, int nq, double *w) { return parity_abs2<double>(s, nq, w); }
int mipt_cuda_parity_collapse_f32(void *s, int nq, int outcome, double weight)
{
    return parity_collapse<float>(s, nq, outcome, weight);
}
int mipt_cuda_parity_collapse_f64(void *s, int nq, int outcome, double weight)
{
    return parity_collapse<double>(s, nq, outcome, weight);
}
int mipt_cuda_parity_expand_f32(void *s, int n) { return parity_expand<float>(s, n); }
int mipt_cuda_parity_expand_f64(void *s, int n) { return parity_expand<double>(s, n); }
const char *mipt_cuda_cusv_parity_last_error(void) { return g_parity_error; }
}
