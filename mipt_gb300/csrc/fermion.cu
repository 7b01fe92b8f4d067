// Free-fermion (Gaussian) monitored circuits on the Majorana covariance
// matrix Gamma (2N x 2N, real antisymmetric, Gamma^2 = -1 for pure states).
//
// The reference simulates fermionic circuits only as Jordan-Wigner state
// vectors (cpp/include/mipt/circuits/rppu_layer.hpp, cpp/include/mipt/cusv/parity.hpp
// in the reference project); this path works on Gamma directly:
//   gate on modes (m, m+1 mod N): Haar SO(4) rotation O of their four
//     Majoranas, Gamma <- O Gamma O^T
//   parity measurement of mode j (Majoranas a = 2j, b = 2j+1): outcome s = +1
//     with probability (1 + Gamma_ab)/2, then for k, l outside {a, b}
//     Gamma_kl += (Gamma_kb Gamma_la - Gamma_ka Gamma_lb) / (Gamma_ab + s),
//     rows/columns a, b cleared and Gamma_ab = s
//   re-purification: Gamma <- Gamma (3 + Gamma^2) / 2 (Newton-Schulz step)
//   entropy of modes M: eigenvalues nu^2 of -Gamma_M^2 (each twice),
//     S = sum over pairs of H2((1 + nu)/2), in bits.
//
// Precision: the layer evolution runs in FP32 with Gamma held as a packed upper
// triangle in shared memory by one persistent block per trajectory (FP64 only
// for the measurement denominator and probability). Between evolution
// segments, and before the entropies, Gamma is re-purified in FP64 by batched
// FP64 GEMMs; the block eigensolves are FP64 Jacobi.
#include "mipt_gb300.h"

#include "common.cuh"
#include "sampler.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace mg
{
int api_fail(int code, const std::string &what);
int api_cuda_fail(cudaError_t e, const char *what);
} // namespace mg

namespace mg
{
namespace
{
constexpr int FF_THREADS = 512;

__device__ __forceinline__ int tri_index(int k, int l, int M) { return k * M - (k * (k + 1)) / 2 + (l - k - 1); }

template <typename Real>
__device__ __forceinline__ Real tri_get(const Real *T, int i, int j, int M)
{
    if (i == j) return Real(0);
    return i < j ? T[tri_index(i, j, M)] : -T[tri_index(j, i, M)];
}

template <typename Real>
__device__ __forceinline__ void tri_set(Real *T, int i, int j, int M, Real v)
{
    if (i < j)
        T[tri_index(i, j, M)] = v;
    else if (i > j)
        T[tri_index(j, i, M)] = -v;
}

__device__ __forceinline__ float fmaR(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmaR(double a, double b, double c) { return fma(a, b, c); }

// Runs layers [t0, t1) for one trajectory per block. Gamma (full matrix in
// global memory) is loaded into a packed upper triangle and written back at
// the end. FP32: the triangle lives in shared memory. FP64: it does not fit
// there at N = 128 (261 KB), so it lives in the trajectory's slice of
// tri_global (L2-resident while the block runs); the work is the same.
//   rot    [traj][depth][G][16]    row-major rotation of group g
//   groups [2][G][4]               Majorana indices of group g (by layer parity)
//   mcount [traj][depth], mmode/unif/forced/outc/prob [traj][depth][N]
template <typename Real>
__global__ void __launch_bounds__(FF_THREADS)
    k_ff_evolve(int N, int depth, int G, int t0, int t1, const Real *__restrict__ rot,
                const unsigned char *__restrict__ groups, const int *__restrict__ mcount,
                const unsigned char *__restrict__ mmode, const double *__restrict__ unif,
                const signed char *__restrict__ forced, signed char *__restrict__ outc, double *__restrict__ prob,
                Real *__restrict__ gamma, Real *__restrict__ tri_global)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = 2 * N;
    const int P = M * (M - 1) / 2;
    Real *sm = reinterpret_cast<Real *>(smem_raw);
    Real *T = tri_global ? tri_global + static_cast<std::size_t>(blockIdx.x) * P : sm;
    Real *Ucol = tri_global ? sm : sm + P;
    Real *Vcol = Ucol + M;
    Real *R = Vcol + M;
    unsigned char *grp = reinterpret_cast<unsigned char *>(R + G * 16);
    __shared__ Real s_sign, s_coef;

    const int traj = blockIdx.x;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int warp = tid >> 5, lane = tid & 31, nwarps = nthr >> 5;
    Real *Gm = gamma + static_cast<std::size_t>(traj) * M * M;

    for (int k = warp; k < M; k += nwarps)
        for (int l = k + 1 + lane; l < M; l += 32) T[tri_index(k, l, M)] = Gm[k * M + l];
    __syncthreads();

    for (int t = t0; t < t1; ++t)
    {
        const std::size_t lt = static_cast<std::size_t>(traj) * depth + t;
        for (int i = tid; i < G * 16; i += nthr) R[i] = rot[lt * G * 16 + i];
        for (int i = tid; i < G * 4; i += nthr) grp[i] = groups[(t & 1) * G * 4 + i];
        __syncthreads();

        // Gamma_{g_a g_b} <- O_a Gamma_{g_a g_b} O_b^T for every pair of groups a <= b.
        const int nbp = G * (G + 1) / 2;
        for (int bp = tid; bp < nbp; bp += nthr)
        {
            int b = static_cast<int>((sqrtf(8.f * bp + 1.f) - 1.f) * 0.5f);
            while ((b + 1) * (b + 2) / 2 <= bp) ++b;
            while (b * (b + 1) / 2 > bp) --b;
            const int a = bp - b * (b + 1) / 2;
            int ia[4], ib[4];
            for (int r = 0; r < 4; ++r)
            {
                ia[r] = grp[a * 4 + r];
                ib[r] = grp[b * 4 + r];
            }
            Real X[4][4], Y[4][4];
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) X[r][c] = tri_get(T, ia[r], ib[c], M);
            const Real *Oa = R + a * 16, *Ob = R + b * 16;
            // Y = Oa X Ob^T
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c)
                {
                    Real acc = Real(0);
                    for (int k = 0; k < 4; ++k)
                    {
                        Real xo = Real(0);
                        for (int l = 0; l < 4; ++l) xo = fmaR(X[k][l], Ob[c * 4 + l], xo);
                        acc = fmaR(Oa[r * 4 + k], xo, acc);
                    }
                    Y[r][c] = acc;
                }
            if (a == b)
            {
                for (int r = 0; r < 4; ++r)
                    for (int c = r + 1; c < 4; ++c) tri_set(T, ia[r], ia[c], M, Y[r][c]);
            }
            else
            {
                for (int r = 0; r < 4; ++r)
                    for (int c = 0; c < 4; ++c) tri_set(T, ia[r], ib[c], M, Y[r][c]);
            }
        }
        __syncthreads();

        const int mc = mcount[lt];
        for (int i = 0; i < mc; ++i)
        {
            const int j = mmode[lt * N + i];
            const int a = 2 * j, b = a + 1;
            for (int k = tid; k < M; k += nthr)
            {
                Ucol[k] = tri_get(T, k, a, M);
                Vcol[k] = tri_get(T, k, b, M);
            }
            if (tid == 0)
            {
                // FP64 probability and denominator.
                const double g = static_cast<double>(tri_get(T, a, b, M));
                const double pplus = fmin(fmax((1.0 + g) * 0.5, 0.0), 1.0);
                int s;
                if (forced)
                    s = forced[lt * N + i] > 0 ? 1 : -1;
                else
                    s = unif[lt * N + i] < pplus ? 1 : -1;
                const double pr = s > 0 ? pplus : 1.0 - pplus;
                const double den = g + static_cast<double>(s);
                s_sign = static_cast<Real>(s);
                s_coef = (den != 0.0) ? static_cast<Real>(1.0 / den) : Real(0);
                outc[lt * N + i] = static_cast<signed char>(s);
                prob[lt * N + i] = pr;
            }
            __syncthreads();
            const Real coef = s_coef;
            for (int k = warp; k < M; k += nwarps)
            {
                if (k == a || k == b) continue;
                const Real uk = Ucol[k], vk = Vcol[k];
                for (int l = k + 1 + lane; l < M; l += 32)
                {
                    if (l == a || l == b) continue;
                    Real &x = T[tri_index(k, l, M)];
                    x = fmaR(coef, fmaR(vk, Ucol[l], -uk * Vcol[l]), x);
                }
            }
            __syncthreads();
            for (int k = tid; k < M; k += nthr)
            {
                if (k != a) tri_set(T, k, a, M, Real(0));
                if (k != b) tri_set(T, k, b, M, Real(0));
            }
            __syncthreads();
            if (tid == 0) tri_set(T, a, b, M, s_sign);
            __syncthreads();
        }
    }

    for (int e = tid; e < M * M; e += nthr)
    {
        const int i = e / M, jj = e % M;
        Gm[e] = tri_get(T, i, jj, M);
    }
}

// Batched FP64 C = alpha * A B + beta * D over square M x M matrices.
constexpr int GT = 64;
__global__ void __launch_bounds__(256) k_dgemm(int M, const double *__restrict__ A, const double *__restrict__ B,
                                               const double *__restrict__ D, double *__restrict__ C, double alpha,
                                               double beta)
{
    __shared__ double As[16][GT + 1], Bs[16][GT + 1];
    const std::size_t off = static_cast<std::size_t>(blockIdx.z) * M * M;
    const int r0 = blockIdx.y * GT, c0 = blockIdx.x * GT;
    const int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < M; k0 += 16)
    {
        for (int i = tid; i < 16 * GT; i += 256)
        {
            const int kk = i / GT, rr = i % GT;
            As[kk][rr] = (r0 + rr < M && k0 + kk < M) ? A[off + static_cast<std::size_t>(r0 + rr) * M + k0 + kk] : 0.0;
            Bs[kk][rr] = (c0 + rr < M && k0 + kk < M) ? B[off + static_cast<std::size_t>(k0 + kk) * M + c0 + rr] : 0.0;
        }
        __syncthreads();
        for (int kk = 0; kk < 16; ++kk)
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(As[kk][ty * 4 + i], Bs[kk][tx * 4 + j], acc[i][j]);
        __syncthreads();
    }
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
        {
            const int r = r0 + ty * 4 + i, c = c0 + tx * 4 + j;
            if (r < M && c < M)
            {
                const std::size_t e = off + static_cast<std::size_t>(r) * M + c;
                C[e] = alpha * acc[i][j] + (D ? beta * D[e] : 0.0);
            }
        }
}

__global__ void k_f32_to_f64(const float *a, double *b, std::size_t n)
{
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x)
        b[i] = a[i];
}

// Antisymmetrise in FP64, then round to the FP32 working copy.
__global__ void k_antisym(int M, double *g64, float *g32, std::size_t count)
{
    const std::size_t per = static_cast<std::size_t>(M) * M;
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < count * per;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x)
    {
        const std::size_t b = i / per, e = i % per;
        const int r = static_cast<int>(e / M), c = static_cast<int>(e % M);
        if (r > c) continue;
        const std::size_t o = b * per;
        const double v = (r == c) ? 0.0 : 0.5 * (g64[o + e] - g64[o + static_cast<std::size_t>(c) * M + r]);
        g64[o + e] = v;
        g64[o + static_cast<std::size_t>(c) * M + r] = -v;
        if (g32)
        {
            g32[o + e] = static_cast<float>(v);
            g32[o + static_cast<std::size_t>(c) * M + r] = static_cast<float>(-v);
        }
    }
}

// Entropy (bits) of a set of modes (mask over N <= 128 modes) from the FP64
// covariance: S = -Gamma_M^2 assembled in shared memory, parallel-order real
// Jacobi, S = 1/2 sum_i H2((1 + sqrt(mu_i))/2).
struct FFEntJob
{
    int traj;
    int pad;
    std::uint64_t mask[2];
};

__global__ void __launch_bounds__(256) k_ff_entropy(int N, const double *__restrict__ g64,
                                                    const FFEntJob *__restrict__ jobs, double *__restrict__ out)
{
    extern __shared__ double Sm[];
    __shared__ int maj[256];
    __shared__ int s_d;
    __shared__ double rc[128], rs[128];
    __shared__ int rp[128], rq[128];
    __shared__ double red[256];
    __shared__ int done;
    const FFEntJob J = jobs[blockIdx.x];
    const int M = 2 * N;
    const int tid = threadIdx.x, T = blockDim.x;
    if (tid == 0)
    {
        int d = 0;
        for (int m = 0; m < N; ++m)
            if ((J.mask[m >> 6] >> (m & 63)) & 1ull)
            {
                maj[d++] = 2 * m;
                maj[d++] = 2 * m + 1;
            }
        s_d = d;
    }
    __syncthreads();
    const int d = s_d;
    const int ld = d + 1;
    if (d == 0)
    {
        if (tid == 0) out[blockIdx.x] = 0.0;
        return;
    }
    const double *G = g64 + static_cast<std::size_t>(J.traj) * M * M;
    // S = Gamma_M^T Gamma_M
    for (int e = tid; e < d * d; e += T)
    {
        const int p = e / d, q = e % d;
        double acc = 0.0;
        for (int r = 0; r < d; ++r) acc = fma(G[maj[r] * M + maj[p]], G[maj[r] * M + maj[q]], acc);
        Sm[p * ld + q] = acc;
    }
    __syncthreads();
    const int half = d / 2;
    for (int sweep = 0; sweep < 40; ++sweep)
    {
        double off = 0.0, dg = 0.0;
        for (int e = tid; e < d * d; e += T)
        {
            const int p = e / d, q = e % d;
            const double v = Sm[p * ld + q];
            if (p != q)
                off += v * v;
            else
                dg += v * v;
        }
        red[tid] = off;
        __syncthreads();
        for (int w = T / 2; w > 0; w /= 2)
        {
            if (tid < w) red[tid] += red[tid + w];
            __syncthreads();
        }
        const double offs = red[0];
        __syncthreads();
        red[tid] = dg;
        __syncthreads();
        for (int w = T / 2; w > 0; w /= 2)
        {
            if (tid < w) red[tid] += red[tid + w];
            __syncthreads();
        }
        if (tid == 0) done = (offs <= 1e-30 * red[0]) || offs == 0.0;
        __syncthreads();
        if (done) break;
        for (int round = 0; round < d - 1; ++round)
        {
            if (tid < half)
            {
                int p, q;
                if (tid == 0)
                {
                    p = round;
                    q = d - 1;
                }
                else
                {
                    p = (round + tid) % (d - 1);
                    q = (round - tid + d - 1) % (d - 1);
                }
                if (p > q)
                {
                    const int t = p;
                    p = q;
                    q = t;
                }
                const double apq = Sm[p * ld + q];
                double c = 1.0, s = 0.0;
                if (fabs(apq) > 1e-300)
                {
                    const double th = (Sm[q * ld + q] - Sm[p * ld + p]) / (2.0 * apq);
                    const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(1.0 + th * th));
                    c = 1.0 / sqrt(1.0 + t * t);
                    s = t * c;
                }
                rp[tid] = p;
                rq[tid] = q;
                rc[tid] = c;
                rs[tid] = s;
            }
            __syncthreads();
            for (int w = tid; w < half * d; w += T)
            {
                const int pi = w / d, k = w % d;
                const int p = rp[pi], q = rq[pi];
                const double c = rc[pi], s = rs[pi];
                const double akp = Sm[k * ld + p], akq = Sm[k * ld + q];
                Sm[k * ld + p] = c * akp - s * akq;
                Sm[k * ld + q] = s * akp + c * akq;
            }
            __syncthreads();
            for (int w = tid; w < half * d; w += T)
            {
                const int pi = w / d, k = w % d;
                const int p = rp[pi], q = rq[pi];
                const double c = rc[pi], s = rs[pi];
                const double apk = Sm[p * ld + k], aqk = Sm[q * ld + k];
                Sm[p * ld + k] = c * apk - s * aqk;
                Sm[q * ld + k] = s * apk + c * aqk;
            }
            __syncthreads();
            if (tid < half)
            {
                Sm[rp[tid] * ld + rq[tid]] = 0.0;
                Sm[rq[tid] * ld + rp[tid]] = 0.0;
            }
            __syncthreads();
        }
    }
    if (tid == 0)
    {
        double s = 0.0;
        for (int i = 0; i < d; ++i)
        {
            const double nu = sqrt(fmin(fmax(Sm[i * ld + i], 0.0), 1.0));
            const double x = 0.5 * (1.0 + nu);
            double h = 0.0;
            if (x > 1e-15) h -= x * log2(x);
            if (1.0 - x > 1e-15) h -= (1.0 - x) * log2(1.0 - x);
            s += 0.5 * h;
        }
        out[blockIdx.x] = fabs(s) < 1e-12 ? 0.0 : s;
    }
}

struct Dev
{
    void *p = nullptr;
    ~Dev()
    {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(std::size_t bytes) { return cudaMalloc(&p, std::max<std::size_t>(bytes, 256)); }
    template <typename T> T *as() { return static_cast<T *>(p); }
};

#define FF_CUDA(x)                                                                                               \
    do                                                                                                           \
    {                                                                                                            \
        cudaError_t e_ = (x);                                                                                    \
        if (e_ != cudaSuccess) return api_cuda_fail(e_, #x);                                                     \
    } while (0)

// Two FP64 Newton-Schulz steps on count matrices (g64 in place), then
// antisymmetrise and refresh the FP32 copy.
int purify(int M, int count, double *g64, double *tmp, double *tmp2, float *g32)
{
    dim3 grid((M + GT - 1) / GT, (M + GT - 1) / GT, count);
    for (int it = 0; it < 2; ++it)
    {
        k_dgemm<<<grid, 256>>>(M, g64, g64, nullptr, tmp, 1.0, 0.0);      // tmp = G G
        k_dgemm<<<grid, 256>>>(M, g64, tmp, g64, tmp2, 0.5, 1.5);         // tmp2 = (G tmp)/2 + 3G/2
        FF_CUDA(cudaGetLastError());
        FF_CUDA(cudaMemcpyAsync(g64, tmp2, sizeof(double) * M * M * count, cudaMemcpyDeviceToDevice));
    }
    k_antisym<<<std::min<std::size_t>((static_cast<std::size_t>(count) * M * M + 255) / 256, 4096), 256>>>(
        M, g64, g32, count);
    FF_CUDA(cudaGetLastError());
    return 0;
}
} // namespace
} // namespace mg

using namespace mg;

extern "C" int mipt_gb300_ff_run(const mipt_gb300_ff_config *cfg, const std::uint64_t *seeds, const double *p,
                                 int count, const int *forced, int *outcomes, double *probs, double *gamma_out,
                                 double *s_blocks, double *tmi)
{
    if (!cfg || !seeds || !p || count <= 0) return api_fail(MIPT_GB300_E_INVALID, "bad free-fermion arguments");
    const int N = cfg->n_modes, depth = cfg->depth;
    if (N < 4 || N > 128 || (N % 2) != 0 || depth < 1)
        return api_fail(MIPT_GB300_E_INVALID, "free-fermion chains need even 4 <= N <= 128 and depth >= 1");
    if (tmi && (N % 4) != 0) return api_fail(MIPT_GB300_E_INVALID, "TMI needs N divisible by 4");
    for (int i = 0; i < cfg->n_blocks; ++i)
        if (!cfg->block_len || cfg->block_len[i] < 0 || cfg->block_len[i] > N)
            return api_fail(MIPT_GB300_E_INVALID, "block lengths must be in [0, N]");
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return api_fail(MIPT_GB300_E_NODEVICE, "no CUDA device");

    std::vector<FermionDraw> draws;
    try
    {
        draw_fermion_batch(seeds, p, count, N, depth, cfg->closed != 0, draws, cfg->host_threads);
    }
    catch (const std::exception &e)
    {
        return api_fail(MIPT_GB300_E_INVALID, e.what());
    }
    const int M = 2 * N, G = N / 2;
    const std::size_t C = count, D = depth;
    const bool fp64 = cfg->fp64 != 0;
    std::vector<double> h_rot(C * D * G * 16, 0.0);
    std::vector<int> h_mc(C * D);
    std::vector<unsigned char> h_mm(C * D * N);
    std::vector<double> h_u(C * D * N);
    std::vector<signed char> h_forced(forced ? C * D * N : 0);
    for (std::size_t b = 0; b < C; ++b)
    {
        const FermionDraw &d = draws[b];
        for (int t = 0; t < depth; ++t)
        {
            double *dst = &h_rot[((b * D + t) * G) * 16];
            const int gc = d.gate_count[t];
            for (int g = 0; g < gc; ++g)
                for (int e = 0; e < 16; ++e) dst[g * 16 + e] = d.rot[(static_cast<std::size_t>(t) * d.max_gates + g) * 16 + e];
            for (int g = gc; g < G; ++g)
                for (int e = 0; e < 16; ++e) dst[g * 16 + e] = (e % 5 == 0) ? 1.0 : 0.0;
            h_mc[b * D + t] = d.meas_count[t];
            for (int i = 0; i < d.meas_count[t]; ++i)
            {
                h_mm[(b * D + t) * N + i] = static_cast<unsigned char>(d.meas_mode[static_cast<std::size_t>(t) * N + i]);
                h_u[(b * D + t) * N + i] = d.uniform[static_cast<std::size_t>(t) * N + i];
                if (forced) h_forced[(b * D + t) * N + i] = static_cast<signed char>(forced[(b * D + t) * N + i] > 0 ? 1 : -1);
            }
        }
    }
    // Group tables: even layers pair modes (2g, 2g+1); odd layers (2g+1, 2g+2),
    // the last one closing the ring or, on an open chain, an identity group of
    // the two end modes.
    std::vector<unsigned char> h_grp(2 * G * 4);
    for (int g = 0; g < G; ++g)
    {
        for (int r = 0; r < 4; ++r) h_grp[(0 * G + g) * 4 + r] = static_cast<unsigned char>(4 * g + r);
        const int m = 2 * g + 1;
        if (m < N - 1 || cfg->closed)
        {
            const int m2 = (m + 1) % N;
            const int idx[4] = {2 * m, 2 * m + 1, 2 * m2, 2 * m2 + 1};
            for (int r = 0; r < 4; ++r) h_grp[(G + g) * 4 + r] = static_cast<unsigned char>(idx[r]);
        }
        else
        {
            const int idx[4] = {0, 1, M - 2, M - 1};
            for (int r = 0; r < 4; ++r) h_grp[(G + g) * 4 + r] = static_cast<unsigned char>(idx[r]);
        }
    }

    Dev d_rot, d_grp, d_mc, d_mm, d_u, d_f, d_oc, d_pr, d_g32, d_g64, d_t1, d_t2, d_tri, d_jobs, d_ent;
    const std::size_t rot_elem = fp64 ? sizeof(double) : sizeof(float);
    FF_CUDA(d_rot.alloc(rot_elem * h_rot.size()));
    FF_CUDA(d_grp.alloc(h_grp.size()));
    FF_CUDA(d_mc.alloc(sizeof(int) * h_mc.size()));
    FF_CUDA(d_mm.alloc(h_mm.size()));
    FF_CUDA(d_u.alloc(sizeof(double) * h_u.size()));
    if (forced) FF_CUDA(d_f.alloc(h_forced.size()));
    FF_CUDA(d_oc.alloc(C * D * N));
    FF_CUDA(d_pr.alloc(sizeof(double) * C * D * N));
    if (!fp64) FF_CUDA(d_g32.alloc(sizeof(float) * C * M * M));
    FF_CUDA(d_g64.alloc(sizeof(double) * C * M * M));
    if (fp64) FF_CUDA(d_tri.alloc(sizeof(double) * C * (static_cast<std::size_t>(M) * (M - 1) / 2)));
    FF_CUDA(d_t1.alloc(sizeof(double) * C * M * M));
    FF_CUDA(d_t2.alloc(sizeof(double) * C * M * M));
    if (fp64)
        FF_CUDA(cudaMemcpy(d_rot.p, h_rot.data(), sizeof(double) * h_rot.size(), cudaMemcpyHostToDevice));
    else
    {
        std::vector<float> r32(h_rot.begin(), h_rot.end());
        FF_CUDA(cudaMemcpy(d_rot.p, r32.data(), sizeof(float) * r32.size(), cudaMemcpyHostToDevice));
    }
    FF_CUDA(cudaMemcpy(d_grp.p, h_grp.data(), h_grp.size(), cudaMemcpyHostToDevice));
    FF_CUDA(cudaMemcpy(d_mc.p, h_mc.data(), sizeof(int) * h_mc.size(), cudaMemcpyHostToDevice));
    FF_CUDA(cudaMemcpy(d_mm.p, h_mm.data(), h_mm.size(), cudaMemcpyHostToDevice));
    FF_CUDA(cudaMemcpy(d_u.p, h_u.data(), sizeof(double) * h_u.size(), cudaMemcpyHostToDevice));
    if (forced) FF_CUDA(cudaMemcpy(d_f.p, h_forced.data(), h_forced.size(), cudaMemcpyHostToDevice));
    FF_CUDA(cudaMemset(d_oc.p, 0, C * D * N));
    FF_CUDA(cudaMemset(d_pr.p, 0, sizeof(double) * C * D * N));
    {
        std::vector<double> g0(static_cast<std::size_t>(M) * M, 0.0);
        for (int j = 0; j < N; ++j)
        {
            g0[(2 * j) * M + 2 * j + 1] = 1.0;
            g0[(2 * j + 1) * M + 2 * j] = -1.0;
        }
        std::vector<float> g0f(g0.begin(), g0.end());
        for (std::size_t b = 0; b < C; ++b)
        {
            if (fp64)
                FF_CUDA(cudaMemcpy(d_g64.as<double>() + b * M * M, g0.data(), sizeof(double) * M * M,
                                   cudaMemcpyHostToDevice));
            else
                FF_CUDA(cudaMemcpy(d_g32.as<float>() + b * M * M, g0f.data(), sizeof(float) * M * M,
                                   cudaMemcpyHostToDevice));
        }
    }
    // Shared memory: the packed triangle (FP32 only), two columns, the
    // rotations and the group table.
    const std::size_t tri_bytes = rot_elem * (static_cast<std::size_t>(M) * (M - 1) / 2);
    const std::size_t smem = (fp64 ? 0 : tri_bytes) + rot_elem * (2 * M + G * 16) + G * 4 + 16;
    if (fp64)
        FF_CUDA(cudaFuncSetAttribute(k_ff_evolve<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
    else
        FF_CUDA(cudaFuncSetAttribute(k_ff_evolve<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
    const int seg = cfg->repurify_every > 0 ? cfg->repurify_every : depth;
    const int cvt_blocks = static_cast<int>(std::min<std::size_t>((C * M * M + 255) / 256, 4096));
    for (int t0 = 0; t0 < depth; t0 += seg)
    {
        const int t1 = std::min(depth, t0 + seg);
        if (fp64)
            k_ff_evolve<double><<<count, FF_THREADS, smem>>>(
                N, depth, G, t0, t1, d_rot.as<double>(), d_grp.as<unsigned char>(), d_mc.as<int>(),
                d_mm.as<unsigned char>(), d_u.as<double>(), forced ? d_f.as<signed char>() : nullptr,
                d_oc.as<signed char>(), d_pr.as<double>(), d_g64.as<double>(), d_tri.as<double>());
        else
            k_ff_evolve<float><<<count, FF_THREADS, smem>>>(
                N, depth, G, t0, t1, d_rot.as<float>(), d_grp.as<unsigned char>(), d_mc.as<int>(),
                d_mm.as<unsigned char>(), d_u.as<double>(), forced ? d_f.as<signed char>() : nullptr,
                d_oc.as<signed char>(), d_pr.as<double>(), d_g32.as<float>(), nullptr);
        FF_CUDA(cudaGetLastError());
        // FP64 re-purification between segments (and of the final state).
        if (!fp64)
        {
            k_f32_to_f64<<<cvt_blocks, 256>>>(d_g32.as<float>(), d_g64.as<double>(), C * M * M);
            FF_CUDA(cudaGetLastError());
        }
        const int rc = purify(M, count, d_g64.as<double>(), d_t1.as<double>(), d_t2.as<double>(),
                              fp64 ? nullptr : d_g32.as<float>());
        if (rc) return rc;
    }
    // Entropy jobs: blocks [0, len) (the shorter side of the cut, the state is
    // pure) and the seven TMI subsets of contiguous quarters.
    std::vector<FFEntJob> jobs;
    auto mask_of = [&](int a, int len) {
        FFEntJob j{};
        for (int i = 0; i < len; ++i)
        {
            const int m = (a + i) % N;
            j.mask[m >> 6] |= 1ull << (m & 63);
        }
        return j;
    };
    const int nb = cfg->n_blocks;
    const int per = nb + (tmi ? 7 : 0);
    for (int b = 0; b < count; ++b)
    {
        for (int i = 0; i < nb; ++i)
        {
            const int len = cfg->block_len[i];
            FFEntJob j = (len <= N - len) ? mask_of(0, len) : mask_of(len, N - len);
            j.traj = b;
            jobs.push_back(j);
        }
        if (tmi)
        {
            const int q = N / 4;
            FFEntJob A = mask_of(0, q), B = mask_of(q, q), Cq = mask_of(2 * q, q), Dq = mask_of(3 * q, q);
            auto uni = [](FFEntJob x, const FFEntJob &y) {
                x.mask[0] |= y.mask[0];
                x.mask[1] |= y.mask[1];
                return x;
            };
            FFEntJob set[7] = {A, B, Cq, Dq, uni(A, B), uni(A, Cq), uni(B, Cq)};
            for (auto &j : set)
            {
                j.traj = b;
                jobs.push_back(j);
            }
        }
    }
    std::vector<double> ent(jobs.size(), 0.0);
    if (!jobs.empty())
    {
        FF_CUDA(d_jobs.alloc(sizeof(FFEntJob) * jobs.size()));
        FF_CUDA(d_ent.alloc(sizeof(double) * jobs.size()));
        FF_CUDA(cudaMemcpy(d_jobs.p, jobs.data(), sizeof(FFEntJob) * jobs.size(), cudaMemcpyHostToDevice));
        int dmax = 0;
        for (const auto &j : jobs) dmax = std::max(dmax, 2 * (__builtin_popcountll(j.mask[0]) + __builtin_popcountll(j.mask[1])));
        if (dmax > 128) return api_fail(MIPT_GB300_E_INVALID, "entropy blocks above 64 modes are not supported");
        const std::size_t esm = sizeof(double) * std::max(1, dmax) * (std::max(1, dmax) + 1);
        FF_CUDA(cudaFuncSetAttribute(k_ff_entropy, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(esm)));
        k_ff_entropy<<<static_cast<int>(jobs.size()), 256, esm>>>(N, d_g64.as<double>(), d_jobs.as<FFEntJob>(),
                                                                  d_ent.as<double>());
        FF_CUDA(cudaGetLastError());
        FF_CUDA(cudaMemcpy(ent.data(), d_ent.p, sizeof(double) * ent.size(), cudaMemcpyDeviceToHost));
    }
    FF_CUDA(cudaDeviceSynchronize());
    if (outcomes)
    {
        std::vector<signed char> oc(C * D * N);
        FF_CUDA(cudaMemcpy(oc.data(), d_oc.p, oc.size(), cudaMemcpyDeviceToHost));
        for (std::size_t i = 0; i < oc.size(); ++i) outcomes[i] = oc[i];
    }
    if (probs) FF_CUDA(cudaMemcpy(probs, d_pr.p, sizeof(double) * C * D * N, cudaMemcpyDeviceToHost));
    if (gamma_out) FF_CUDA(cudaMemcpy(gamma_out, d_g64.p, sizeof(double) * C * M * M, cudaMemcpyDeviceToHost));
    for (int b = 0; b < count; ++b)
    {
        for (int i = 0; i < nb && s_blocks; ++i) s_blocks[static_cast<std::size_t>(b) * nb + i] = ent[b * per + i];
        if (tmi)
        {
            const double *e = &ent[b * per + nb];
            tmi[b] = e[0] + e[1] + e[2] + e[3] - e[4] - e[5] - e[6];
        }
    }
    return 0;
}
