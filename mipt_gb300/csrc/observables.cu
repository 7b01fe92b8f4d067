// Reduced density matrices of batched state vectors.
//
// rho_A = M M^H, where M is the Schmidt matrix of the kept modes, is the one
// dense contraction of the path. This file holds the SIMT formulation: the
// Schmidt gather is fused into the operand loads (no M is materialised), the
// pending measurement collapse and the fermionic signs are applied while
// loading, only lower-triangle tiles are computed, and the purity can be
// reduced straight from the tiles without writing rho.
//
// Reference behaviour reproduced (paths inside the reference project):
//   Schmidt layout and fermionic masks  cpp/include/mipt/cuda/schmidt_gram.cuh:13-19,196-315
//   Gram + mirror of the lower triangle cpp/include/mipt/cuda/schmidt_gram.cuh:327-445
//   purity reduction in FP64            cpp/src/cuda/tmi_cuda_svd.cu:124-155
//   entropy in bits, eigenvalue cut     cpp/include/mipt/tmi/linalg.hpp:125-141
//   three-site sweep signs              cpp/src/cuda/rho_reduce.cu:36-110
#include "observables.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <type_traits>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

namespace mg
{

GramJob make_gram_job(int traj, int n, const int *kept, int k, bool fermion)
{
    if (k < 0 || k > n || k > 16) throw std::invalid_argument("kept-mode count out of range");
    GramJob j{};
    j.traj = traj;
    j.k = k;
    j.fermion = fermion ? 1 : 0;
    std::uint64_t used = 0;
    for (int i = 0; i < k; ++i)
    {
        if (kept[i] < 0 || kept[i] >= n || ((used >> kept[i]) & 1ull))
            throw std::invalid_argument("kept modes must be distinct and in range");
        used |= 1ull << kept[i];
        j.kept[i] = static_cast<std::int8_t>(kept[i]);
    }
    int e = 0;
    for (int q = 0; q < n; ++q)
        if (!((used >> q) & 1ull)) j.env[e++] = static_cast<std::int8_t>(q);
    for (int i = 0; i < k; ++i)
    {
        std::uint64_t m = 0;
        for (int b = 0; b < e; ++b)
            if (j.env[b] < kept[i]) m |= 1ull << b;
        j.below[i] = m;
    }
    j.rows_fastest = (used & 1ull) ? 1 : 0;
    return j;
}

namespace
{
// MIPT_GB300_MEASURED_COMPACT=0 keeps the sites a pending collapse measures
// in the Gram (see CompactJob and k_gram).
bool measured_compact_enabled()
{
    static const bool on = [] {
        const char *v = std::getenv("MIPT_GB300_MEASURED_COMPACT");
        return !(v && v[0] == '0');
    }();
    return on;
}

// MIPT_GB300_RHO_SUMS=fp64 sums the rho of FP32 states exactly in FP64
// instead of in compensated FP32 runs.
bool compensated_rho_sums()
{
    static const bool on = [] {
        const char *v = std::getenv("MIPT_GB300_RHO_SUMS");
        return !(v && std::strcmp(v, "fp64") == 0);
    }();
    return on;
}

constexpr int TM = kGramTile;
constexpr int TK = 32;
constexpr int kGramThreads = 256;

// K-step of the Gram tile: 32 environment columns for FP32 operands, 16 for
// FP64 (keeps both operand tiles within the 48 KB static shared memory).
template <typename Real> struct GramK
{
    static constexpr int TK = sizeof(Real) == 4 ? 32 : 16;
    static constexpr int BITS = sizeof(Real) == 4 ? 5 : 4;
};

__device__ __forceinline__ void tile_coords(int id, int &tr, int &tc)
{
    int r = static_cast<int>((sqrt(8.0 * id + 1.0) - 1.0) * 0.5);
    while ((r + 1) * (r + 2) / 2 <= id) ++r;
    while (r * (r + 1) / 2 > id) --r;
    tr = r;
    tc = id - r * (r + 1) / 2;
}

// check: apply the collapse's mask test; scale: its renormalisation (also
// for reduced jobs, whose addresses all pass the test).
template <typename Real>
__device__ __forceinline__ Cx<Real> gather(const Cx<Real> *__restrict__ psi, std::uint64_t addr, const Collapse &cl,
                                           bool check, bool scale, bool negate)
{
    Cx<Real> v = psi[addr];
    if (check && (addr & cl.mask) != cl.value) return Cx<Real>{Real(0), Real(0)};
    if (scale)
    {
        const Real sc = static_cast<Real>(cl.scale);
        v.re *= sc;
        v.im *= sc;
    }
    if (negate)
    {
        v.re = -v.re;
        v.im = -v.im;
    }
    return v;
}

// mode 0: write split partials of rho (full tile) to part_out;
// mode 1: reduce the tile's contribution to Tr(rho^2) into pur_out.
// Acc is the type of the totals: FP64 whenever rho is materialised (its
// small eigenvalues feed -lambda log lambda, so accumulation rounding must
// stay below the state's own second-order error), the operand type for the
// purity-only mode. With kMixed (FP32 states, FP64 totals) the products are
// summed in FP32 runs before each run joins the FP64 totals: FP32
// throughput instead of GB300's FP64 rate. Plain runs of 64 (the
// allocation-free purity) have a relative rounding of about 5e-7, which
// moves a purity by as little but is too coarse for rho's small
// eigenvalues; materialised rho of FP32 states uses compensated runs
// (kComp), of FP64 states exact FP64 sums.
// One step of a compensated dot product (Ogita, Rump and Oishi, "Accurate sum
// and dot product", 2005, Dot2): s += x * y in FP32, with the exact rounding
// errors of the product (TwoProduct by FMA) and of the sum (Knuth's TwoSum)
// added to c. The _rn intrinsics keep the product and the additions from being
// contracted into FMAs, which the error-free transformations rely on.
__device__ __forceinline__ void comp_fma(float x, float y, float &s, float &c)
{
    const float p = __fmul_rn(x, y);
    const float ep = fmaf(x, y, -p);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float es = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    c = __fadd_rn(c, __fadd_rn(ep, es));
    s = t;
}

template <typename Real, typename Acc, bool kMixed = false, bool kComp = false>
__global__ void __launch_bounds__(kGramThreads)
    k_gram(const Cx<Real> *__restrict__ states, int n, const GramJob *__restrict__ jobs,
           const Collapse *__restrict__ col, std::size_t col_stride, int splits, std::uint64_t kchunk, int mode,
           Acc *__restrict__ part_out, double *__restrict__ pur_out, int compact, int *__restrict__ dims_out)
{
    constexpr int TK = GramK<Real>::TK;
    constexpr int KB = GramK<Real>::BITS;
    __shared__ GramJob J;
    __shared__ Cx<Real> As[TK][TM + 1];
    __shared__ Cx<Real> Bs[TK][TM + 1];
    __shared__ std::uint64_t roffA[TM], roffB[TM], crossA[TM], crossB[TM], elo[TK];
    __shared__ double red[kGramThreads / 32];
    __shared__ std::uint64_t s_fixed;
    __shared__ int s_reduced, s_nenv, s_check;

    const int tid = threadIdx.x;
    const int job = blockIdx.z;
    const bool has_col = col != nullptr;
    if (tid == 0)
    {
        J = jobs[job];
        // Reduced job (compact): the sites the pending collapse measured
        // leave the kept and environment lists and their outcome bits join
        // every address. The state is |outcome> (x) phi on them, so rho is
        // phi's reduced matrix on the kept modes left, padded with zero
        // rows and columns (the same spectrum and purity); fermionic jobs
        // keep every mode.
        s_fixed = 0;
        s_reduced = 0;
        s_nenv = n - J.k;
        s_check = has_col ? 1 : 0;
        if (compact && !J.fermion)
        {
            Collapse c0{0, 0, 1.0, 0};
            if (has_col) c0 = col[J.traj * col_stride];
            const std::uint64_t drop = c0.parity == 0 ? c0.mask : 0ull;
            const int kf = J.k;
            int a = 0, e = 0;
            for (int i = 0; i < kf; ++i)
                if (!((drop >> J.kept[i]) & 1ull)) J.kept[a++] = J.kept[i];
            for (int i = 0; i < n - kf; ++i)
                if (!((drop >> J.env[i]) & 1ull)) J.env[e++] = J.env[i];
            // The smaller side: M M^H and M^H M have the same non-zero
            // spectrum (the pure state's Schmidt values), so the Gram runs over
            // the environment when it has fewer modes left.
            const bool swap = e < a;
            if (swap)
            {
                std::int8_t t[32];
                for (int i = 0; i < a; ++i) t[i] = J.kept[i];
                for (int i = 0; i < e; ++i) J.kept[i] = J.env[i];
                for (int i = 0; i < a; ++i) J.env[i] = t[i];
                const int x = a;
                a = e;
                e = x;
            }
            if (drop != 0ull || swap)
            {
                J.k = a;
                J.rows_fastest = (a > 0 && J.kept[0] == 0) ? 1 : 0;
                s_nenv = e;
                s_fixed = c0.value & drop;
                s_reduced = 1;
                if (drop != 0ull) s_check = 0;
            }
        }
        if (dims_out != nullptr && blockIdx.x == 0 && blockIdx.y == 0) dims_out[job] = 1 << J.k;
    }
    __syncthreads();
    const int D = 1 << jobs[job].k; // rows of the output matrix
    const int k = J.k;
    const int d = 1 << k; // rows with data
    int tr, tc;
    tile_coords(blockIdx.x, tr, tc);
    const int r0 = tr * TM, c0 = tc * TM;
    const int nenv = s_nenv;
    const std::uint64_t E = 1ull << nenv;
    // A reduced job spreads its (smaller) environment evenly over the same
    // splits, in multiples of TK columns.
    std::uint64_t kc = kchunk;
    if (s_reduced)
    {
        kc = (E + splits - 1) / splits;
        kc = (kc + TK - 1) / TK * TK;
    }
    const std::uint64_t ebeg = static_cast<std::uint64_t>(blockIdx.y) * kc;
    const std::uint64_t eend = ebeg + kc < E ? ebeg + kc : E;
    if (r0 >= d)
    {
        // Rows past the reduced block: this tile of rho is zero.
        if (mode == 0)
        {
            Acc *out = part_out + (static_cast<std::size_t>(job) * splits + blockIdx.y) * static_cast<std::size_t>(D) * D * 2;
            for (int i = tid; i < TM * TM; i += kGramThreads)
            {
                const int r = r0 + i / TM, c = c0 + i % TM;
                if (r < D && c < D && r >= c)
                {
                    out[(static_cast<std::size_t>(r) * D + c) * 2] = Acc(0);
                    out[(static_cast<std::size_t>(r) * D + c) * 2 + 1] = Acc(0);
                }
            }
        }
        else if (tid == 0)
            pur_out[static_cast<std::size_t>(job) * gridDim.x + blockIdx.x] = 0.0;
        return;
    }

    if (tid < TM)
    {
        const int r = r0 + tid, c = c0 + tid;
        std::uint64_t oa = 0, ob = 0, xa = 0, xb = 0;
        if (r < d)
            for (int i = 0; i < k; ++i)
                if ((r >> i) & 1)
                {
                    oa |= 1ull << J.kept[i];
                    xa ^= J.below[i];
                }
        if (c < d)
            for (int i = 0; i < k; ++i)
                if ((c >> i) & 1)
                {
                    ob |= 1ull << J.kept[i];
                    xb ^= J.below[i];
                }
        roffA[tid] = oa;
        roffB[tid] = ob;
        crossA[tid] = J.fermion ? xa : 0ull;
        crossB[tid] = J.fermion ? xb : 0ull;
    }
    else if (tid < TM + TK)
    {
        const int i = tid - TM;
        const int nb = nenv < KB ? nenv : KB;
        std::uint64_t o = 0;
        for (int b = 0; b < nb; ++b)
            if ((i >> b) & 1) o |= 1ull << J.env[b];
        elo[i] = o;
    }
    Collapse cl{0, 0, 1.0, 0};
    if (has_col) cl = col[J.traj * col_stride];
    const bool check = s_check != 0;
    const std::uint64_t fixed = s_fixed;
    __syncthreads();

    const Cx<Real> *psi = states + (static_cast<std::size_t>(J.traj) << n);
    const int ty = tid / 16, tx = tid % 16;
    // kMixed: products summed in FP32 runs of 2 * TK = 64 environment
    // columns, each run added to the FP64 totals (the reference's
    // mixed-precision sweep, cpp/include/mipt/cuda/reduce_sweep.cuh:59-96);
    // otherwise the products go straight into Acc.
    // kComp (with kMixed): each FP32 run is a compensated dot product (its
    // rounding errors carried in a second FP32 accumulator), accurate as if
    // computed in twice the working precision, so runs can be 8 chunks (256
    // columns) long: FP64-quality rho entries at the FP32 rate (ten FP32
    // operations per product; GB300 runs FP32 about 64x faster than FP64).
    static_assert(!kMixed || (sizeof(Real) == 4 && sizeof(Acc) == 8), "mixed runs: FP32 states, FP64 totals");
    static_assert(!kComp || kMixed, "compensated runs are FP32 runs");
    using Run = typename std::conditional<kMixed, float, Acc>::type;
    constexpr int kRunChunks = kComp ? 8 : 2;
    Acc accr[4][4], acci[4][4];
    Run runr[4][4], runi[4][4];
    Run cmpr[kComp ? 4 : 1][kComp ? 4 : 1], cmpi[kComp ? 4 : 1][kComp ? 4 : 1];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            accr[i][j] = acci[i][j] = Acc(0);
            runr[i][j] = runi[i][j] = Run(0);
            if constexpr (kComp) cmpr[i][j] = cmpi[i][j] = Run(0);
        }
    int run_chunks = 0;

    for (std::uint64_t e0 = ebeg; e0 < eend; e0 += TK)
    {
        std::uint64_t ehi = fixed;
        for (int b = KB; b < nenv; ++b)
            if ((e0 >> b) & 1ull) ehi |= 1ull << J.env[b];
        for (int idx = tid; idx < TM * TK; idx += kGramThreads)
        {
            int i, kk;
            if (J.rows_fastest)
            {
                i = idx % TM;
                kk = idx / TM;
            }
            else
            {
                kk = idx % TK;
                i = idx / TK;
            }
            const std::uint64_t e = e0 + kk;
            Cx<Real> va{Real(0), Real(0)}, vb{Real(0), Real(0)};
            if (e < eend)
            {
                const std::uint64_t eo = ehi | elo[kk];
                if (r0 + i < d)
                    va = gather(psi, eo | roffA[i], cl, check, has_col, (__popcll(e & crossA[i]) & 1) != 0);
                if (c0 + i < d)
                    vb = gather(psi, eo | roffB[i], cl, check, has_col, (__popcll(e & crossB[i]) & 1) != 0);
            }
            As[kk][i] = va;
            Bs[kk][i] = vb;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < TK; ++kk)
        {
            Cx<Real> a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
            {
                a[i] = As[kk][ty * 4 + i];
                b[i] = Bs[kk][tx * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                {
                    // a * conj(b)
                    if constexpr (kComp)
                    {
                        comp_fma(a[i].re, b[j].re, runr[i][j], cmpr[i][j]);
                        comp_fma(a[i].im, b[j].im, runr[i][j], cmpr[i][j]);
                        comp_fma(a[i].im, b[j].re, runi[i][j], cmpi[i][j]);
                        comp_fma(-a[i].re, b[j].im, runi[i][j], cmpi[i][j]);
                    }
                    else
                    {
                        runr[i][j] = fma(Run(a[i].re), Run(b[j].re), runr[i][j]);
                        runr[i][j] = fma(Run(a[i].im), Run(b[j].im), runr[i][j]);
                        runi[i][j] = fma(Run(a[i].im), Run(b[j].re), runi[i][j]);
                        runi[i][j] = fma(-Run(a[i].re), Run(b[j].im), runi[i][j]);
                    }
                }
        }
        if constexpr (kMixed)
        {
            if (++run_chunks == kRunChunks || e0 + TK >= eend)
            {
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                    {
                        if constexpr (kComp)
                        {
                            accr[i][j] += static_cast<Acc>(runr[i][j]) + static_cast<Acc>(cmpr[i][j]);
                            acci[i][j] += static_cast<Acc>(runi[i][j]) + static_cast<Acc>(cmpi[i][j]);
                            cmpr[i][j] = cmpi[i][j] = Run(0);
                        }
                        else
                        {
                            accr[i][j] += static_cast<Acc>(runr[i][j]);
                            acci[i][j] += static_cast<Acc>(runi[i][j]);
                        }
                        runr[i][j] = runi[i][j] = Run(0);
                    }
                run_chunks = 0;
            }
        }
        __syncthreads();
    }
    if constexpr (!kMixed)
    {
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
            {
                accr[i][j] = runr[i][j];
                acci[i][j] = runi[i][j];
            }
    }

    if (mode == 0)
    {
        // Rows and columns past d (a reduced job) are zero and written as such.
        Acc *out = part_out + (static_cast<std::size_t>(job) * splits + blockIdx.y) * static_cast<std::size_t>(D) * D * 2;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
            {
                const int r = r0 + ty * 4 + i, c = c0 + tx * 4 + j;
                if (r < D && c < D && r >= c)
                {
                    out[(static_cast<std::size_t>(r) * D + c) * 2] = accr[i][j];
                    out[(static_cast<std::size_t>(r) * D + c) * 2 + 1] = acci[i][j];
                }
            }
    }
    else
    {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
            {
                const int r = r0 + ty * 4 + i, c = c0 + tx * 4 + j;
                if (r < d && c < d && r >= c)
                {
                    const double w = (r == c) ? 1.0 : 2.0;
                    const double re = static_cast<double>(accr[i][j]), im = static_cast<double>(acci[i][j]);
                    s += w * (re * re + im * im);
                }
            }
        for (int off = 16; off > 0; off /= 2) s += __shfl_down_sync(0xffffffffu, s, off);
        if ((tid & 31) == 0) red[tid >> 5] = s;
        __syncthreads();
        if (tid == 0)
        {
            double t = 0.0;
            for (int w = 0; w < kGramThreads / 32; ++w) t += red[w];
            pur_out[static_cast<std::size_t>(job) * gridDim.x + blockIdx.x] = t;
        }
    }
}

__global__ void k_gram_finalize(const double *__restrict__ part, int d, int splits, int njobs, double *__restrict__ rho)
{
    const std::uint64_t per = static_cast<std::uint64_t>(d) * d;
    const std::uint64_t total = per * njobs;
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<std::uint64_t>(gridDim.x) * blockDim.x)
    {
        const std::uint64_t job = i / per, rc = i % per;
        const int r = static_cast<int>(rc / d), c = static_cast<int>(rc % d);
        if (r < c) continue;
        double sr = 0.0, si = 0.0;
        for (int z = 0; z < splits; ++z)
        {
            const double *p = part + ((job * splits + z) * per + rc) * 2;
            sr += static_cast<double>(p[0]);
            si += static_cast<double>(p[1]);
        }
        double *o = rho + job * per * 2;
        if (r == c)
        {
            o[rc * 2] = sr;
            o[rc * 2 + 1] = 0.0;
        }
        else
        {
            o[(static_cast<std::uint64_t>(r) * d + c) * 2] = sr;
            o[(static_cast<std::uint64_t>(r) * d + c) * 2 + 1] = si;
            o[(static_cast<std::uint64_t>(c) * d + r) * 2] = sr;
            o[(static_cast<std::uint64_t>(c) * d + r) * 2 + 1] = -si;
        }
    }
}

__global__ void k_sum_rows(const double *__restrict__ in, int per, double *__restrict__ out)
{
    // out[job] = sum of in[job][0..per) in a fixed order (one block per job).
    __shared__ double red[256];
    const double *p = in + static_cast<std::size_t>(blockIdx.x) * per;
    double s = 0.0;
    for (int i = threadIdx.x; i < per; i += blockDim.x) s += p[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w /= 2)
    {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

__global__ void k_purity(const double *__restrict__ rho, int d, double *__restrict__ out)
{
    __shared__ double red[256];
    const std::uint64_t per = static_cast<std::uint64_t>(d) * d;
    const double *p = rho + blockIdx.x * per * 2;
    double s = 0.0;
    for (std::uint64_t i = threadIdx.x; i < per; i += blockDim.x) s += p[2 * i] * p[2 * i] + p[2 * i + 1] * p[2 * i + 1];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w /= 2)
    {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// Parallel-order (round-robin) cyclic Jacobi for one Hermitian d x d matrix
// per block, d <= 64, in FP64 shared memory.
__global__ void __launch_bounds__(256) k_jacobi(const double *__restrict__ rho, int d, double *__restrict__ ent,
                                                double *__restrict__ eig)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *A = reinterpret_cast<double2 *>(smem_raw); // d x (d+1)
    __shared__ double rc[32], rs[32];
    __shared__ double2 rph[32];
    __shared__ int rp[32], rq[32];
    __shared__ double red[256];
    __shared__ int done;
    const int ld = d + 1;
    const int tid = threadIdx.x, T = blockDim.x;
    const double *src = rho + static_cast<std::size_t>(blockIdx.x) * d * d * 2;
    for (int i = tid; i < d * d; i += T)
    {
        const int r = i / d, c = i % d;
        A[r * ld + c] = make_double2(src[2 * i], src[2 * i + 1]);
    }
    __syncthreads();
    // Hermitise: average with the conjugate transpose.
    for (int i = tid; i < d * d; i += T)
    {
        const int r = i / d, c = i % d;
        if (r < c)
        {
            const double2 a = A[r * ld + c], b = A[c * ld + r];
            const double2 h = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
            A[r * ld + c] = h;
            A[c * ld + r] = make_double2(h.x, -h.y);
        }
        else if (r == c)
        {
            A[r * ld + c].y = 0.0;
        }
    }
    __syncthreads();
    const int half = d / 2;
    for (int sweep = 0; sweep < 40 && d > 1; ++sweep)
    {
        double off = 0.0, dg = 0.0;
        for (int i = tid; i < d * d; i += T)
        {
            const int r = i / d, c = i % d;
            const double2 a = A[r * ld + c];
            if (r != c)
                off += a.x * a.x + a.y * a.y;
            else
                dg += a.x * a.x;
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
                const double2 apq = A[p * ld + q];
                const double mag = sqrt(apq.x * apq.x + apq.y * apq.y);
                double c = 1.0, s = 0.0;
                double2 ph = make_double2(1.0, 0.0);
                if (mag > 1e-300)
                {
                    const double app = A[p * ld + p].x, aqq = A[q * ld + q].x;
                    const double th = (aqq - app) / (2.0 * mag);
                    const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(1.0 + th * th));
                    c = 1.0 / sqrt(1.0 + t * t);
                    s = t * c;
                    ph = make_double2(apq.x / mag, apq.y / mag);
                }
                rp[tid] = p;
                rq[tid] = q;
                rc[tid] = c;
                rs[tid] = s;
                rph[tid] = ph;
            }
            __syncthreads();
            // A <- A J (columns p, q of every pair)
            for (int w = tid; w < half * d; w += T)
            {
                const int pi = w / d, kr = w % d;
                const int p = rp[pi], q = rq[pi];
                const double c = rc[pi], s = rs[pi];
                const double2 ph = rph[pi];
                const double2 akp = A[kr * ld + p], akq = A[kr * ld + q];
                // s*conj(ph)*akq and s*ph*akp
                const double2 t1 = make_double2(s * (ph.x * akq.x + ph.y * akq.y), s * (ph.x * akq.y - ph.y * akq.x));
                const double2 t2 = make_double2(s * (ph.x * akp.x - ph.y * akp.y), s * (ph.x * akp.y + ph.y * akp.x));
                A[kr * ld + p] = make_double2(c * akp.x - t1.x, c * akp.y - t1.y);
                A[kr * ld + q] = make_double2(t2.x + c * akq.x, t2.y + c * akq.y);
            }
            __syncthreads();
            // A <- J^H A (rows p, q of every pair)
            for (int w = tid; w < half * d; w += T)
            {
                const int pi = w / d, kc = w % d;
                const int p = rp[pi], q = rq[pi];
                const double c = rc[pi], s = rs[pi];
                const double2 ph = rph[pi];
                const double2 apk = A[p * ld + kc], aqk = A[q * ld + kc];
                // s*ph*aqk and s*conj(ph)*apk
                const double2 t1 = make_double2(s * (ph.x * aqk.x - ph.y * aqk.y), s * (ph.x * aqk.y + ph.y * aqk.x));
                const double2 t2 = make_double2(s * (ph.x * apk.x + ph.y * apk.y), s * (ph.x * apk.y - ph.y * apk.x));
                A[p * ld + kc] = make_double2(c * apk.x - t1.x, c * apk.y - t1.y);
                A[q * ld + kc] = make_double2(t2.x + c * aqk.x, t2.y + c * aqk.y);
            }
            __syncthreads();
            if (tid < half)
            {
                const int p = rp[tid], q = rq[tid];
                A[p * ld + q] = make_double2(0.0, 0.0);
                A[q * ld + p] = make_double2(0.0, 0.0);
            }
            __syncthreads();
        }
    }
    if (tid == 0)
    {
        double s = 0.0;
        for (int i = 0; i < d; ++i)
        {
            const double l = A[i * ld + i].x;
            if (eig) eig[static_cast<std::size_t>(blockIdx.x) * d + i] = l;
            if (l > 1e-15) s -= l * log2(l);
        }
        ent[blockIdx.x] = (fabs(s) < 1e-12) ? 0.0 : s;
    }
}

// ------------------------------------------------------------- three sites
constexpr int R3_THREADS = 256;

template <typename Real>
__global__ void __launch_bounds__(R3_THREADS)
    k_rho3(const Cx<Real> *__restrict__ states, int n, const int *__restrict__ subs, int fermion,
           const Collapse *__restrict__ col, std::size_t col_stride, int chunks, double *__restrict__ part)
{
    __shared__ std::uint64_t lo_tab[256];
    __shared__ std::uint64_t off[8], cross[8];
    __shared__ int isign[8];
    __shared__ std::int8_t env[64];
    __shared__ double red[R3_THREADS / 32][72];
    const int tid = threadIdx.x;
    const int tri = blockIdx.y, traj = blockIdx.z;
    const int q[3] = {subs[3 * tri], subs[3 * tri + 1], subs[3 * tri + 2]};
    const int nenv = n - 3;
    if (tid == 0)
    {
        int e = 0;
        for (int b = 0; b < n; ++b)
            if (b != q[0] && b != q[1] && b != q[2]) env[e++] = static_cast<std::int8_t>(b);
    }
    __syncthreads();
    if (tid < 256)
    {
        const int nb = nenv < 8 ? nenv : 8;
        std::uint64_t o = 0;
        for (int b = 0; b < nb; ++b)
            if ((tid >> b) & 1) o |= 1ull << env[b];
        lo_tab[tid] = o;
    }
    if (tid < 8)
    {
        std::uint64_t o = 0, x = 0;
        int par = 0;
        for (int i = 0; i < 3; ++i)
            if ((tid >> i) & 1)
            {
                o |= 1ull << q[i];
                for (int b = 0; b < nenv; ++b)
                    if (env[b] < q[i]) x ^= 1ull << b;
                for (int j = i + 1; j < 3; ++j)
                    if (((tid >> j) & 1) && q[i] > q[j]) par ^= 1;
            }
        off[tid] = o;
        cross[tid] = fermion ? x : 0ull;
        isign[tid] = (fermion && par) ? -1 : 1;
    }
    Collapse cl{0, 0, 1.0, 0};
    const bool has_col = col != nullptr;
    if (has_col) cl = col[traj * col_stride];
    __syncthreads();

    const Cx<Real> *psi = states + (static_cast<std::size_t>(traj) << n);
    const std::uint64_t E = 1ull << nenv;
    const std::uint64_t per = (E + chunks - 1) / chunks;
    const std::uint64_t beg = blockIdx.x * per, end = beg + per < E ? beg + per : E;
    Real ar[36], ai[36];
#pragma unroll
    for (int i = 0; i < 36; ++i) ar[i] = ai[i] = Real(0);
    const Real sc = static_cast<Real>(cl.scale);
    for (std::uint64_t e = beg + tid; e < end; e += R3_THREADS)
    {
        std::uint64_t hi = 0;
        for (int b = 8; b < nenv; ++b)
            if ((e >> b) & 1ull) hi |= 1ull << env[b];
        const std::uint64_t eo = hi | lo_tab[e & 255];
        Cx<Real> v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r)
        {
            const std::uint64_t a = eo | off[r];
            Cx<Real> x = psi[a];
            if (has_col)
            {
                if ((a & cl.mask) != cl.value)
                    x = Cx<Real>{Real(0), Real(0)};
                else
                {
                    x.re *= sc;
                    x.im *= sc;
                }
            }
            const int sg = ((__popcll(e & cross[r]) & 1) ? -1 : 1) * isign[r];
            if (sg < 0)
            {
                x.re = -x.re;
                x.im = -x.im;
            }
            v[r] = x;
        }
        int t = 0;
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c <= r; ++c, ++t)
            {
                ar[t] = fma(v[r].re, v[c].re, ar[t]);
                ar[t] = fma(v[r].im, v[c].im, ar[t]);
                ai[t] = fma(v[r].im, v[c].re, ai[t]);
                ai[t] = fma(-v[r].re, v[c].im, ai[t]);
            }
    }
    const int warp = tid >> 5, lane = tid & 31;
#pragma unroll
    for (int t = 0; t < 36; ++t)
    {
        double x = static_cast<double>(ar[t]), y = static_cast<double>(ai[t]);
        for (int o = 16; o > 0; o /= 2)
        {
            x += __shfl_down_sync(0xffffffffu, x, o);
            y += __shfl_down_sync(0xffffffffu, y, o);
        }
        if (lane == 0)
        {
            red[warp][2 * t] = x;
            red[warp][2 * t + 1] = y;
        }
    }
    __syncthreads();
    if (tid < 72)
    {
        double s = 0.0;
        for (int w = 0; w < R3_THREADS / 32; ++w) s += red[w][tid];
        part[((static_cast<std::size_t>(traj) * gridDim.y + tri) * chunks + blockIdx.x) * 72 + tid] = s;
    }
}

__global__ void k_rho3_finalize(const double *__restrict__ part, int chunks, int total_triples, double *__restrict__ out)
{
    const int id = blockIdx.x;
    if (id >= total_triples) return;
    const int t = threadIdx.x;
    if (t >= 36) return;
    double sr = 0.0, si = 0.0;
    for (int c = 0; c < chunks; ++c)
    {
        sr += part[(static_cast<std::size_t>(id) * chunks + c) * 72 + 2 * t];
        si += part[(static_cast<std::size_t>(id) * chunks + c) * 72 + 2 * t + 1];
    }
    int r = 0;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    const int c = t - r * (r + 1) / 2;
    double *o = out + static_cast<std::size_t>(id) * 128;
    o[(r * 8 + c) * 2] = sr;
    o[(r * 8 + c) * 2 + 1] = (r == c) ? 0.0 : si;
    if (r != c)
    {
        o[(c * 8 + r) * 2] = sr;
        o[(c * 8 + r) * 2 + 1] = -si;
    }
}

int gram_splits(int n, int k, int njobs, bool rho)
{
    if (!rho) return 1;
    const std::uint64_t E = 1ull << (n - k);
    const int tiles = gram_tiles(k) * njobs;
    int splits = 1;
    while (tiles * splits < 2 * 152 && E / (2ull * splits) >= static_cast<std::uint64_t>(TK) * 8) splits *= 2;
    return splits;
}
} // namespace

std::size_t gram_scratch_bytes(int n, int k, int njobs, bool rho)
{
    if (!rho) return sizeof(double) * static_cast<std::size_t>(gram_tiles(k)) * njobs;
    const int splits = gram_splits(n, k, njobs, true);
    return sizeof(double) * 2 * static_cast<std::size_t>(splits) * njobs * (std::size_t{1} << (2 * k));
}

template <typename Real>
cudaError_t gram_rho(const Cx<Real> *states, int n, const GramJob *d_jobs, int njobs, int k,
                     const Collapse *collapse, std::size_t collapse_stride, double *rho_out, void *scratch,
                     std::size_t scratch_bytes, cudaStream_t s, int *dims_out)
{
    if (njobs <= 0) return cudaSuccess;
    const int splits = gram_splits(n, k, njobs, true);
    const std::size_t need = sizeof(double) * 2 * static_cast<std::size_t>(splits) * njobs * (std::size_t{1} << (2 * k));
    if (need > scratch_bytes) return cudaErrorInvalidValue;
    const std::uint64_t E = 1ull << (n - k);
    const std::uint64_t kchunk = (E + splits - 1) / splits;
    dim3 grid(gram_tiles(k), splits, njobs);
    const int compact = measured_compact_enabled() ? 1 : 0;
    // rho feeds -lambda log lambda: plain FP32 runs of 64 products left
    // about 5e-7 relative error in its entries, which moved the S_vN of
    // near-pure reduced states by up to 2e-5 at n = 20. FP32 states sum in
    // compensated FP32 runs (FP64-quality entries at the FP32 rate), FP64
    // states exactly in FP64.
    // Compensated runs (rho entries to about 1e-13 of their scale) for tall
    // Grams (environment >= 64x the kept dimension), where the Gram's work
    // dominates; exact FP64 sums otherwise: their entries are cleaner, and the
    // QL sweeps, which dominate square Grams, resolve fewer noise-level
    // eigenvalues (half-chain spectra of L = 16 and 18: 1.7x faster QL).
    bool comp = false;
    if constexpr (sizeof(Real) == 4) comp = compensated_rho_sums() && n - k >= k + 6;
    if (comp)
    {
        if constexpr (sizeof(Real) == 4)
            k_gram<Real, double, true, true><<<grid, kGramThreads, 0, s>>>(
                states, n, d_jobs, collapse, collapse_stride, splits, kchunk, 0, static_cast<double *>(scratch),
                nullptr, compact, dims_out);
    }
    else
        k_gram<Real, double><<<grid, kGramThreads, 0, s>>>(states, n, d_jobs, collapse, collapse_stride, splits,
                                                           kchunk, 0, static_cast<double *>(scratch), nullptr,
                                                           compact, dims_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int d = 1 << k;
    const std::uint64_t total = static_cast<std::uint64_t>(d) * d * njobs;
    const int blocks = static_cast<int>(std::min<std::uint64_t>((total + 255) / 256, 152ull * 16));
    k_gram_finalize<<<blocks, 256, 0, s>>>(static_cast<const double *>(scratch), d, splits, njobs, rho_out);
    return cudaGetLastError();
}

template <typename Real>
cudaError_t gram_purity(const Cx<Real> *states, int n, const GramJob *d_jobs, int njobs, int k,
                        const Collapse *collapse, std::size_t collapse_stride, double *purity_out, void *scratch,
                        std::size_t scratch_bytes, cudaStream_t s)
{
    if (njobs <= 0) return cudaSuccess;
    const int tiles = gram_tiles(k);
    if (sizeof(double) * static_cast<std::size_t>(tiles) * njobs > scratch_bytes) return cudaErrorInvalidValue;
    const std::uint64_t E = 1ull << (n - k);
    dim3 grid(tiles, 1, njobs);
    k_gram<Real, Real><<<grid, kGramThreads, 0, s>>>(states, n, d_jobs, collapse, collapse_stride, 1, E, 1, nullptr,
                                                     static_cast<double *>(scratch),
                                                     measured_compact_enabled() ? 1 : 0, nullptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_sum_rows<<<njobs, 256, 0, s>>>(static_cast<const double *>(scratch), tiles, purity_out);
    return cudaGetLastError();
}

cudaError_t gram_purity_f64acc(const Cx<float> *states, int n, const GramJob *d_jobs, int njobs, int k,
                               double *purity_out, void *scratch, std::size_t scratch_bytes, cudaStream_t s)
{
    if (njobs <= 0) return cudaSuccess;
    const int tiles = gram_tiles(k);
    if (sizeof(double) * static_cast<std::size_t>(tiles) * njobs > scratch_bytes) return cudaErrorInvalidValue;
    const std::uint64_t E = 1ull << (n - k);
    dim3 grid(tiles, 1, njobs);
    // From n = 20 the products run in FP32 runs of 64 into FP64 totals (the
    // purity needs no more); below that every product is summed in FP64.
    if (n >= 20)
        k_gram<float, double, true><<<grid, kGramThreads, 0, s>>>(states, n, d_jobs, nullptr, 0, 1, E, 1, nullptr,
                                                                  static_cast<double *>(scratch), 0, nullptr);
    else
        k_gram<float, double><<<grid, kGramThreads, 0, s>>>(states, n, d_jobs, nullptr, 0, 1, E, 1, nullptr,
                                                            static_cast<double *>(scratch), 0, nullptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_sum_rows<<<njobs, 256, 0, s>>>(static_cast<const double *>(scratch), tiles, purity_out);
    return cudaGetLastError();
}

cudaError_t purity_of(const double *rho, int d, int njobs, double *purity_out, cudaStream_t s)
{
    if (njobs <= 0) return cudaSuccess;
    k_purity<<<njobs, 256, 0, s>>>(rho, d, purity_out);
    return cudaGetLastError();
}

cudaError_t jacobi_entropy(const double *rho, int d, int njobs, double *entropy_out, double *eig_out, cudaStream_t s)
{
    if (njobs <= 0) return cudaSuccess;
    if (d > 64) return cudaErrorInvalidValue;
    const std::size_t smem = sizeof(double2) * d * (d + 1);
    cudaError_t e = cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    k_jacobi<<<njobs, 256, smem, s>>>(rho, d, entropy_out, eig_out);
    return cudaGetLastError();
}

std::size_t rho3_scratch_bytes(int n, int batch, int count)
{
    const std::uint64_t E = 1ull << (n - 3);
    int chunks = static_cast<int>(std::min<std::uint64_t>(std::max<std::uint64_t>(1, E / (R3_THREADS * 16)), 256));
    return sizeof(double) * 72 * static_cast<std::size_t>(chunks) * count * batch;
}

template <typename Real>
cudaError_t rho3_sweep(const Cx<Real> *states, int n, int batch, const int *d_subs, int count, int fermion,
                       const Collapse *collapse, std::size_t collapse_stride, double *out, void *scratch,
                       std::size_t scratch_bytes, cudaStream_t s)
{
    if (count <= 0 || batch <= 0) return cudaSuccess;
    const std::uint64_t E = 1ull << (n - 3);
    int chunks = static_cast<int>(std::min<std::uint64_t>(std::max<std::uint64_t>(1, E / (R3_THREADS * 16)), 256));
    if (rho3_scratch_bytes(n, batch, count) > scratch_bytes) return cudaErrorInvalidValue;
    dim3 grid(chunks, count, batch);
    k_rho3<Real><<<grid, R3_THREADS, 0, s>>>(states, n, d_subs, fermion, collapse, collapse_stride, chunks,
                                             static_cast<double *>(scratch));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_rho3_finalize<<<count * batch, 64, 0, s>>>(static_cast<const double *>(scratch), chunks, count * batch, out);
    return cudaGetLastError();
}


// ===================================================================
// Tensor-core Gram (tcgen05, FP32 states): purity Tr(rho^2) of
// rho = M M^H without materialising rho.
//
// One real GEMM per 128x64 block of rho: D[128 x 128] = X_r [128 x K] *
// [X_c ; Y_c]^T, where row i of X holds the Schmidt row as interleaved
// (re, im) reals and Y holds (-im, re): D[:, :64] = Re rho, D[:, 64:] = Im rho.
// Operands are split into TF32 hi/lo parts and D accumulates
// hi*hi + hi*lo + lo*hi in FP32 tensor memory (3xTF32). Producer warps gather
// the Schmidt rows straight from the state (pending collapse and fermionic
// signs applied), split them and write the 128B-swizzled K-major layout the
// MMA descriptors describe; one thread issues tcgen05.mma. The producers
// issue all of a chunk's loads together, one chunk ahead of its stores, and
// also drain D from tensor memory into FP32 registers between segments.
namespace
{
constexpr int TCM = 128;                 // rows of a rho block (A rows)
constexpr int TCC = 64;                  // columns of a rho block (complex B rows)
constexpr int TCN = 2 * TCC;             // X rows + Y rows = D columns
constexpr int TC_PWARPS = 8;             // producer warps (they also drain and reduce D)
constexpr int TC_THREADS = (TC_PWARPS + 1) * 32;
constexpr int TC_DCOLS = TCN / (TC_PWARPS / 4);                 // D columns drained per producer thread
constexpr int TC_ITEMS = (TCM + TCC) * 8 / (TC_PWARPS * 32);   // gathered items per thread per chunk
static_assert(TC_DCOLS % 32 == 0 && TC_ITEMS * TC_PWARPS * 32 == (TCM + TCC) * 8, "producer split");
constexpr int TC_A_BYTES = TCM * 128;    // one operand half (hi or lo) of A: 16 KB
constexpr int TC_B_BYTES = TCN * 128;    // one operand half of [X ; Y]: 16 KB
constexpr int TC_STAGE = 2 * TC_A_BYTES + 2 * TC_B_BYTES;
constexpr int TC_STAGES = 2;             // operand stages (split hi/lo, MMA layout)
constexpr int TC_ELEMS = 2 * TC_ITEMS;   // amplitudes a producer thread gathers per chunk
constexpr int TC_RAW_BYTES = TC_ELEMS * TC_PWARPS * 32 * 8;     // one chunk of raw amplitudes: 24 KB
constexpr int TC_RING = 3;               // raw chunks in flight (cp.async ring)
constexpr int TC_TMEM_BUFS = 4;          // accumulation buffers (segments in flight)
constexpr int TC_TMEM_COLS = TC_TMEM_BUFS * TCN;
static_assert(TC_ELEMS * 2 <= 32 && TC_TMEM_COLS <= 512, "chunk codes or tensor memory overflow");
constexpr std::size_t TC_SMEM =
    static_cast<std::size_t>(TC_STAGES) * TC_STAGE + static_cast<std::size_t>(TC_RING) * TC_RAW_BYTES + 1024;
constexpr long long TC_SPIN = 1ll << 24;

__device__ __forceinline__ std::uint32_t sm_addr(const void *p)
{
    return static_cast<std::uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(std::uint64_t *bar, std::uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sm_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(std::uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(sm_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try(std::uint64_t *bar, std::uint32_t parity)
{
    std::uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(sm_addr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Limit of one bounded mbarrier wait of the tensor-core Gram.
constexpr std::uint64_t TC_WAIT_NS = 2000000000ull;

// Bounded wait: gives up after 2 s (or TC_SPIN polls), raises the error flag
// and the block-wide abort flag (so every later wait returns at once).
__device__ __forceinline__ bool mbar_wait(std::uint64_t *bar, std::uint32_t parity, volatile int *abort_flag,
                                          int *err)
{
    if (mbar_try(bar, parity)) return true;
    const std::uint64_t t0 = device_ns();
    for (long long i = 0; i < TC_SPIN; ++i)
    {
        if (*abort_flag) return false;
        if (mbar_try(bar, parity)) return true;
        if ((i & 15) == 15 && device_ns() - t0 > TC_WAIT_NS) break;
    }
    *abort_flag = 1;
    atomicOr(err, 4);
    return false;
}

// Bounded wait that ignores the abort flag: used on the way out to let this
// block's own bulk copies land before it exits.
__device__ __forceinline__ void mbar_settle(std::uint64_t *bar, std::uint32_t parity)
{
    const std::uint64_t t0 = device_ns();
    for (long long i = 0; i < TC_SPIN; ++i)
    {
        if (mbar_try(bar, parity)) return;
        if ((i & 15) == 15 && device_ns() - t0 > TC_WAIT_NS) return;
    }
}

// 3xTF32 split with integer ops: hi = x rounded to the nearest TF32 value
// (ties away from zero: half a TF32 ulp added to the magnitude bits, the low
// 13 mantissa bits cleared), lo = x - hi, exact in FP32 (|lo| <= 2^-11 |x|).
// The tensor core reads lo with TF32 precision, an error <= 2^-22 |x|.
__device__ __forceinline__ void tf32_split(float x, float &hi, float &lo)
{
    hi = __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
    lo = x - hi;
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ std::uint64_t sw128_desc(std::uint32_t saddr)
{
    return static_cast<std::uint64_t>((saddr >> 4) & 0x3FFFu) | (1ull << 16) | (64ull << 32) | (1ull << 46) |
           (2ull << 61);
}

// Instruction descriptor: D = F32, A = B = TF32, both K-major, N = TCN, M = 128.
constexpr std::uint32_t kTcIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((TCN >> 3) << 17) | ((TCM >> 4) << 24);

// Chunks (of 32 real K) accumulated in one tensor-memory buffer before the
// producer warps drain it into registers: the tensor core's FP32 accumulation
// carries a relative bias of order 2^-23 per accumulation step, so long
// in-TMEM sums drift (measured: linear in K); short segments bound it.
constexpr int TC_SEG = 2;

// kTma: every job keeps modes 0..k-1 in order, so the Schmidt matrix of
// trajectory t is the plain [E][d] block of the state buffer; `tmap` views
// the buffer as a 2-D array (d amplitudes per row, E * trajectories rows) and
// the raw chunks arrive by TMA instead of per-amplitude cp.async gathers.
template <bool kTma>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_gram_tc(const Cx<float> *__restrict__ states, int n, const GramJob *__restrict__ jobs,
              const Collapse *__restrict__ col, std::size_t col_stride, double *__restrict__ pur_out,
              int *__restrict__ err, const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ __align__(1024) unsigned char tc_raw[];
    __shared__ GramJob J;
    __shared__ __align__(8) std::uint64_t full_bar[TC_STAGES], empty_bar[TC_STAGES], seg_bar[TC_TMEM_BUFS],
        drained_bar[TC_TMEM_BUFS], raw_bar[TC_RING];
    __shared__ std::uint32_t tmem_base;
    __shared__ std::uint64_t roffA[TCM], roffB[TCC], crossA[TCM], crossB[TCC], elo[16];
    __shared__ double red[TC_PWARPS];
    __shared__ volatile int abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const std::uint32_t raw_s = sm_addr(tc_raw);
    unsigned char *smem = tc_raw + ((1024u - (raw_s & 1023u)) & 1023u);
    const int job = blockIdx.z;
    int tr, tc;
    tile_coords(blockIdx.x, tr, tc);

    if (tid == 0)
    {
        J = jobs[job];
        for (int st = 0; st < TC_STAGES; ++st)
        {
            mbar_init(&full_bar[st], TC_PWARPS);
            mbar_init(&empty_bar[st], 1);
        }
        for (int b = 0; b < TC_TMEM_BUFS; ++b)
        {
            mbar_init(&seg_bar[b], 1);
            mbar_init(&drained_bar[b], TC_PWARPS);
        }
        for (int b = 0; b < TC_RING; ++b) mbar_init(&raw_bar[b], 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == TC_PWARPS)
    {
        // TC_TMEM_BUFS accumulation buffers of TCN columns.
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sm_addr(&tmem_base)),
                     "n"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    const int k = J.k;
    const int nenv = n - k;
    // Block (tr, tc) of the 128-row lower triangle is split into two 64-column halves.
    const int r0 = tr * TCM, c0 = tc * TCM + static_cast<int>(blockIdx.y) * TCC;
    if (tid < TCM)
    {
        std::uint64_t oa = 0, ob = 0, xa = 0, xb = 0;
        const int r = r0 + tid, c = c0 + tid;
        for (int i = 0; i < k; ++i)
        {
            if ((r >> i) & 1)
            {
                oa |= 1ull << J.kept[i];
                xa ^= J.below[i];
            }
            if ((c >> i) & 1)
            {
                ob |= 1ull << J.kept[i];
                xb ^= J.below[i];
            }
        }
        roffA[tid] = oa;
        crossA[tid] = J.fermion ? xa : 0ull;
        if (tid < TCC)
        {
            roffB[tid] = ob;
            crossB[tid] = J.fermion ? xb : 0ull;
        }
    }
    else if (tid < TCM + 16)
    {
        const int i = tid - TCM;
        std::uint64_t o = 0;
        for (int b = 0; b < 4; ++b)
            if ((i >> b) & 1) o |= 1ull << J.env[b];
        elo[i] = o;
    }
    Collapse cl{0, 0, 1.0, 0};
    const bool has_col = col != nullptr;
    if (has_col) cl = col[J.traj * col_stride];
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    const std::uint32_t tmem = tmem_base;
    const Cx<float> *psi = states + (static_cast<std::size_t>(J.traj) << n);
    const int nchunks = 1 << (nenv - 4); // 16 complex environment columns per stage
    const int nseg = (nchunks + TC_SEG - 1) / TC_SEG;

    if (warp < TC_PWARPS)
    {
        // Warp w drains TMEM lanes 32*(w%4).. and buffer columns
        // TC_DCOLS*(w/4)..; the running sums stay in registers for the whole
        // K loop.
        float acc[TC_DCOLS];
#pragma unroll
        for (int i = 0; i < TC_DCOLS; ++i) acc[i] = 0.f;
        const std::uint32_t lane_base = static_cast<std::uint32_t>((warp & 3) * 32) << 16;
        const int col_base = (warp >> 2) * TC_DCOLS;
        int next_drain = 0;
        auto drain = [&](int seg) {
            const int buf = seg % TC_TMEM_BUFS;
            if (!mbar_wait(&seg_bar[buf], (seg / TC_TMEM_BUFS) & 1, &abort_flag, err)) return;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int cb = 0; cb < TC_DCOLS / 32; ++cb)
            {
                std::uint32_t v[32];
                const std::uint32_t taddr = tmem + lane_base + buf * TCN + col_base + cb * 32;
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                      "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                      "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int i = 0; i < 32; ++i) acc[cb * 32 + i] += __uint_as_float(v[i]);
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&drained_bar[buf]);
        };
        // Item j of this thread: operand row `row` of A (which = 0) or of the
        // column block (which = 1), environment columns 2q, 2q+1 of the chunk.
        auto item_coords = [&](int j, int &which, int &row, int &q) {
            const int item = tid + j * TC_PWARPS * 32;
            which = item >= TCM * 8;
            const int rem = which ? item - TCM * 8 : item;
            const int rows = which ? TCC : TCM;
            if (J.rows_fastest)
            {
                row = rem & (rows - 1);
                q = which ? (rem >> 6) : (rem >> 7);
            }
            else
            {
                q = rem & 7;
                row = rem >> 3;
            }
        };
        // Raw amplitudes travel global -> shared with cp.async into a ring of
        // TC_RING chunk slots; amplitude e of thread t sits at
        // slot[(e * threads + t) * 8], and each thread converts only what it
        // copied itself. The returned code holds 2 bits per amplitude:
        // bit 0 = kept by the pending collapse, bit 1 = fermionic sign.
        unsigned char *raw = smem + TC_STAGES * TC_STAGE;
        const std::uint32_t raw_s0 = sm_addr(raw);
        auto issue_chunk = [&](int chunk) -> std::uint32_t {
            std::uint32_t code = 0;
            if (!kTma && chunk < nchunks)
            {
                const std::uint64_t e0 = static_cast<std::uint64_t>(chunk) << 4;
                std::uint64_t ehi = 0;
                for (int b = 4; b < nenv; ++b)
                    if ((e0 >> b) & 1ull) ehi |= 1ull << J.env[b];
                const std::uint32_t slot = raw_s0 + (chunk % TC_RING) * TC_RAW_BYTES;
#pragma unroll
                for (int j = 0; j < TC_ITEMS; ++j)
                {
                    int which, row, q;
                    item_coords(j, which, row, q);
                    const std::uint64_t ro = which ? roffB[row] : roffA[row];
                    const std::uint64_t cx = which ? crossB[row] : crossA[row];
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                    {
                        const int el = 2 * j + h;
                        const std::uint64_t addr = ehi | elo[2 * q + h] | ro;
                        const bool keep = !has_col || (addr & cl.mask) == cl.value;
                        const bool neg = (__popcll((e0 + 2 * q + h) & cx) & 1) != 0;
                        if (keep)
                            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                                             slot + static_cast<std::uint32_t>((el * TC_PWARPS * 32 + tid) * 8)),
                                         "l"(psi + addr)
                                         : "memory");
                        code |= (keep ? 1u : 0u) << (2 * el);
                        code |= (neg ? 2u : 0u) << (2 * el);
                    }
                }
            }
            if (!kTma) asm volatile("cp.async.commit_group;" ::: "memory");
            return code;
        };
        // TMA mode: thread 0 loads chunk `chunk` into its ring slot as three
        // 64-row boxes (A rows r0.., r0+64.., column-block rows c0..), each
        // laid out [16 environment columns][64 rows]. The slot last held
        // chunk - TC_RING, which every warp has converted once the full
        // barrier of that chunk completed.
        const int traj_row0 = J.traj << nenv;
        int tma_issued = 0; // chunks thread 0 has issued (TMA mode)
        auto issue_tma = [&](int chunk) {
            if (!kTma || tid != 0 || chunk >= nchunks) return;
            if (chunk >= TC_RING && !mbar_wait(&full_bar[(chunk - TC_RING) % TC_STAGES],
                                               ((chunk - TC_RING) / TC_STAGES) & 1, &abort_flag, err))
                return;
            const int slot = chunk % TC_RING;
            const std::uint32_t bar = sm_addr(&raw_bar[slot]);
            const std::uint32_t dst = raw_s0 + slot * TC_RAW_BYTES;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(TC_RAW_BYTES)
                         : "memory");
            const int y = traj_row0 + (chunk << 4);
            const int xs[3] = {r0, r0 + 64, c0};
#pragma unroll
            for (int b = 0; b < 3; ++b)
                asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
                             "%3}], [%4];" ::"r"(dst + b * 8192),
                             "l"(reinterpret_cast<std::uint64_t>(&tmap)), "r"(xs[b]), "r"(y), "r"(bar)
                             : "memory");
            tma_issued = chunk + 1;
        };
        // TMA mode keep flags of the pending collapse: per row (fixed per
        // thread) and per environment column (one ballot per chunk).
        std::uint32_t row_keep = 0;
        const std::uint64_t low_mask = (1ull << k) - 1ull;
        if (kTma)
            for (int j = 0; j < TC_ITEMS; ++j)
            {
                int which, row, q;
                item_coords(j, which, row, q);
                const std::uint64_t r = static_cast<std::uint64_t>(which ? c0 + row : r0 + row);
                if (!has_col || (r & cl.mask) == (cl.value & low_mask)) row_keep |= 1u << j;
            }
        const float scale = has_col ? static_cast<float>(cl.scale) : 1.0f;
        std::uint32_t code0 = issue_chunk(0);
        std::uint32_t code1 = issue_chunk(1);
        issue_tma(0);
        issue_tma(1);
        int converted = 0;
        for (int chunk = 0; chunk < nchunks; ++chunk)
        {
            const std::uint32_t code2 = issue_chunk(chunk + 2);
            if constexpr (kTma)
            {
                if (!mbar_wait(&raw_bar[chunk % TC_RING], (chunk / TC_RING) & 1, &abort_flag, err)) break;
                std::uint32_t env_keep = 0xffffu;
                if (has_col)
                {
                    const std::uint64_t e = (static_cast<std::uint64_t>(chunk) << 4) + (lane & 15);
                    env_keep = __ballot_sync(0xffffffffu, ((e << k) & cl.mask) == (cl.value & ~low_mask)) & 0xffffu;
                }
                code0 = 0;
#pragma unroll
                for (int j = 0; j < TC_ITEMS; ++j)
                {
                    int which, row, q;
                    item_coords(j, which, row, q);
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        if (((row_keep >> j) & 1u) && ((env_keep >> (2 * q + h)) & 1u)) code0 |= 1u << (2 * (2 * j + h));
                }
            }
            else
            {
                asm volatile("cp.async.wait_group %0;" ::"n"(TC_RING - 1) : "memory");
            }
            const int st = chunk % TC_STAGES;
            if (chunk >= TC_STAGES &&
                !mbar_wait(&empty_bar[st], ((chunk / TC_STAGES) - 1) & 1, &abort_flag, err))
                break;
            unsigned char *stage = smem + st * TC_STAGE;
            unsigned char *Ahi = stage, *Alo = stage + TC_A_BYTES;
            unsigned char *Bhi = stage + 2 * TC_A_BYTES, *Blo = Bhi + TC_B_BYTES;
            const unsigned char *slot = raw + (chunk % TC_RING) * TC_RAW_BYTES;
#pragma unroll
            for (int j = 0; j < TC_ITEMS; ++j)
            {
                int which, row, q;
                item_coords(j, which, row, q);
                Cx<float> v[2];
#pragma unroll
                for (int h = 0; h < 2; ++h)
                {
                    const int el = 2 * j + h;
                    const std::uint32_t cd = (code0 >> (2 * el)) & 3u;
                    const int raw_off = !kTma ? (el * TC_PWARPS * 32 + tid) * 8
                                        : which ? 2 * 8192 + ((2 * q + h) * 64 + row) * 8
                                                : (row >> 6) * 8192 + ((2 * q + h) * 64 + (row & 63)) * 8;
                    const float2 x = *reinterpret_cast<const float2 *>(slot + raw_off);
                    const float f = (cd & 2u) ? -scale : scale;
                    v[h].re = (cd & 1u) ? x.x * f : 0.0f;
                    v[h].im = (cd & 1u) ? x.y * f : 0.0f;
                }
                // X row (re, im, re, im) and, for the column block, the Y row
                // (-im, re, -im, re): the split commutes with negation and
                // permutation, so Y reuses X's hi/lo.
                float4 h, l;
                tf32_split(v[0].re, h.x, l.x);
                tf32_split(v[0].im, h.y, l.y);
                tf32_split(v[1].re, h.z, l.z);
                tf32_split(v[1].im, h.w, l.w);
                auto put = [&](unsigned char *hi_buf, unsigned char *lo_buf, int rr, float4 hv, float4 lv) {
                    const int off = (rr >> 3) * 1024 + (rr & 7) * 128 + ((q ^ (rr & 7)) << 4);
                    *reinterpret_cast<float4 *>(hi_buf + off) = hv;
                    *reinterpret_cast<float4 *>(lo_buf + off) = lv;
                };
                if (!which)
                {
                    put(Ahi, Alo, row, h, l);
                }
                else
                {
                    put(Bhi, Blo, row, h, l);
                    put(Bhi, Blo, TCC + row, make_float4(-h.y, h.x, -h.w, h.z), make_float4(-l.y, l.x, -l.w, l.z));
                }
            }
            // Make the generic-proxy stores visible to the tensor core.
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&full_bar[st]);
            // Drain segment s once the first chunk of segment s+TC_TMEM_BUFS-1
            // is queued: by then its MMAs finished long ago.
            if (chunk >= (next_drain + TC_TMEM_BUFS - 1) * TC_SEG && next_drain < nseg) drain(next_drain++);
            issue_tma(chunk + 2);
            converted = chunk + 1;
            code0 = code1;
            code1 = code2;
        }
        if (!kTma) asm volatile("cp.async.wait_all;" ::: "memory");
        // After an abort, let the chunks thread 0 issued but nobody consumed land.
        for (int c = converted; c < tma_issued; ++c) mbar_settle(&raw_bar[c % TC_RING], (c / TC_RING) & 1);
        while (next_drain < nseg) drain(next_drain++);

        // Weighted squares of this thread's row: buffer columns below TCC
        // hold Re rho, the rest Im rho, both for rho columns c0 + (col % TCC).
        const int r = r0 + (warp & 3) * 32 + lane;
        double sum = 0.0;
        if (!abort_flag)
        {
#pragma unroll
            for (int i = 0; i < TC_DCOLS; ++i)
            {
                const int c = c0 + ((col_base + i) & (TCC - 1));
                const double w = (r > c) ? 2.0 : ((r == c) ? 1.0 : 0.0);
                const double x = static_cast<double>(acc[i]);
                sum += w * x * x;
            }
        }
        for (int off = 16; off > 0; off /= 2) sum += __shfl_down_sync(0xffffffffu, sum, off);
        if (lane == 0) red[warp] = sum;
    }
    else if (lane == 0)
    {
        for (int chunk = 0; chunk < nchunks; ++chunk)
        {
            const int st = chunk % TC_STAGES;
            const int seg = chunk / TC_SEG;
            const int buf = seg % TC_TMEM_BUFS;
            if (chunk % TC_SEG == 0 && seg >= TC_TMEM_BUFS &&
                !mbar_wait(&drained_bar[buf], ((seg / TC_TMEM_BUFS) - 1) & 1, &abort_flag, err))
                break;
            if (!mbar_wait(&full_bar[st], (chunk / TC_STAGES) & 1, &abort_flag, err)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const std::uint32_t dt = tmem + buf * TCN;
            const std::uint32_t base = sm_addr(smem + st * TC_STAGE);
            const std::uint32_t Ahi = base, Alo = base + TC_A_BYTES;
            const std::uint32_t Bhi = base + 2 * TC_A_BYTES, Blo = Bhi + TC_B_BYTES;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
            {
                const std::uint32_t koff = ks * 32;
                const std::uint64_t ah = sw128_desc(Ahi + koff), al = sw128_desc(Alo + koff);
                const std::uint64_t bh = sw128_desc(Bhi + koff), bl = sw128_desc(Blo + koff);
                const std::uint32_t acc0 = ((chunk % TC_SEG) | ks) ? 1u : 0u;
                asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                             " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(dt),
                             "l"(ah), "l"(bh), "r"(kTcIdesc), "r"(acc0)
                             : "memory");
                asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                             " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(dt),
                             "l"(ah), "l"(bl), "r"(kTcIdesc), "r"(1u)
                             : "memory");
                asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                             " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(dt),
                             "l"(al), "l"(bh), "r"(kTcIdesc), "r"(1u)
                             : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             sm_addr(&empty_bar[st]))
                         : "memory");
            if (chunk % TC_SEG == TC_SEG - 1 || chunk == nchunks - 1)
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 sm_addr(&seg_bar[buf]))
                             : "memory");
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0)
    {
        double t = 0.0;
        for (int w = 0; w < TC_PWARPS; ++w) t += red[w];
        pur_out[(static_cast<std::size_t>(job) * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = t;
    }
    if (warp == TC_PWARPS)
    {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TC_TMEM_COLS)
                     : "memory");
    }
}

// ------------------------------------------------- pre-split operand rows
// For cuts that keep modes 0..k-1 (the Schmidt matrix of a trajectory is the
// plain [E][d] block of its state), the 3xTF32 operands are built once per
// observation by k_tf32_rows instead of once per (row block, column block)
// pair inside the Gram: operand row (job j, chunk c, kept index a), at row
// index (j * nchunks + c) * d + a, holds the 16 environment columns
// e = 16c..16c+15 as 32 floats [Re psi(a, e) .. | Im psi(a, e) ..], TF32 hi
// parts in rows [0, R) and lo parts in rows [R, 2R). The Gram then only
// streams 128-byte rows into 128B-swizzled K-major stages by TMA.
constexpr int TP_C = 128;                                 // complex columns of a rho block (B rows)
constexpr int TP_N = 2 * TP_C;                            // TMEM columns per buffer: Re, then Im
constexpr int TP_BUFS = 2;                                // accumulation buffers (512 TMEM columns)
constexpr int TP_DCOLS = TP_N / (TC_PWARPS / 4);          // D columns drained per thread
constexpr int TP_STAGES = 3;
constexpr int TP_A_BYTES = TCM * 128;                     // hi or lo half of A: 16 KB
constexpr int TP_B_BYTES = TP_C * 128;                    // hi or lo half of B: 16 KB
constexpr int TP_STAGE = 2 * TP_A_BYTES + 2 * TP_B_BYTES; // 64 KB
constexpr std::size_t TP_SMEM = static_cast<std::size_t>(TP_STAGES) * TP_STAGE + 1024;
constexpr int TP_THREADS = (TC_PWARPS + 2) * 32;          // drain warps, MMA warp, TMA warp
static_assert(TP_BUFS * TP_N <= 512 && TP_DCOLS % 32 == 0, "tensor memory or drain split");
// D = F32, A = B = TF32, K-major, N = TP_C (the Re or Im half of the block), M = 128;
// bit 13 negates A.
constexpr std::uint32_t kTpIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((TP_C >> 3) << 17) | ((TCM >> 4) << 24);
constexpr std::uint32_t kTpIdescNegA = kTpIdesc | (1u << 13);

// Geometry of one pre-split Gram job after the sites its trajectory's
// pending collapse measures are taken out. After a projective measurement the
// state is a product |outcome> (x) phi on the measured sites, so rho of the
// kept modes has the spectrum of phi's reduced matrix on the kept modes left:
// M keeps only the rows and columns whose measured bits equal the outcome
// (every other entry is zero), so Tr(rho^2) = ||M' M'^H||_F^2 with M' the
// 2^kq x 2^eq block of them. Fermionic jobs are not reduced (their sign
// factors depend on every mode).
struct CompactJob
{
    std::uint64_t fixed; // the measured sites' outcome bits
    std::uint64_t mask, value; // collapse test still to apply (unreduced jobs)
    float scale;
    int kq, eq; // kept and environment modes left
    std::int8_t kpos[16]; // their global positions, ascending
    std::int8_t epos[32];
};

// One thread per job: the reduced geometry of each pre-split Gram job.
__global__ void k_compact_jobs(const GramJob *__restrict__ jobs, int njobs, int n, int k,
                               const Collapse *__restrict__ col, std::size_t col_stride, int compact,
                               CompactJob *__restrict__ out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= njobs) return;
    const GramJob &J = jobs[j];
    Collapse cl{0, 0, 1.0, 0};
    if (col != nullptr) cl = col[J.traj * col_stride];
    CompactJob c{};
    c.scale = static_cast<float>(cl.scale);
    const bool reduce = compact && !J.fermion && cl.parity == 0;
    std::uint64_t drop = reduce ? cl.mask : 0ull;
    c.fixed = reduce ? (cl.value & cl.mask) : 0ull;
    c.mask = reduce ? 0ull : cl.mask;
    c.value = reduce ? 0ull : cl.value;
    int kq = 0, eq = 0;
    for (int i = 0; i < k; ++i)
        if (!((drop >> J.kept[i]) & 1ull)) c.kpos[kq++] = J.kept[i];
    for (int i = 0; i < n - k; ++i)
        if (!((drop >> J.env[i]) & 1ull)) c.epos[eq++] = J.env[i];
    // The smaller side (same purity from M^H M), when the kept modes left
    // fit the operand rows' chunks of environment columns (kq <= n - k).
    if (compact && !J.fermion && eq < kq && kq <= n - k)
    {
        std::int8_t t[16];
        for (int i = 0; i < kq; ++i) t[i] = c.kpos[i];
        for (int i = 0; i < eq; ++i) c.kpos[i] = c.epos[i];
        for (int i = 0; i < kq; ++i) c.epos[i] = t[i];
        const int x = kq;
        kq = eq;
        eq = x;
    }
    c.kq = kq;
    c.eq = eq;
    out[j] = c;
}

// Operand rows and chunks of a reduced job the Gram reads: rows below
// max(2^kq, 128) (one whole 128-row block), chunks of 16 environment
// columns below max(2^eq / 16, 1).
__host__ __device__ __forceinline__ std::uint32_t compact_rows(int kq) { return kq >= 7 ? (1u << kq) : 128u; }
__host__ __device__ __forceinline__ int compact_chunks(int eq) { return eq >= 4 ? (1 << (eq - 4)) : 1; }

// One thread per operand row: 16 environment columns of job j's reduced
// matrix (pending collapse applied; fermionic signs for fermionic jobs;
// columns past 2^eq and rows past 2^kq are zero), split into TF32 hi/lo.
// Rows and chunks the Gram does not read are skipped.
__global__ void k_tf32_rows(const Cx<float> *__restrict__ states, int n, int k, const GramJob *__restrict__ jobs,
                            const CompactJob *__restrict__ cjobs, int njobs, float4 *__restrict__ rows,
                            std::uint64_t lo_rows)
{
    const std::uint64_t d = 1ull << k;
    const int cbits = n - k - 4;
    const std::uint64_t total = (static_cast<std::uint64_t>(njobs) << cbits) << k;
    for (std::uint64_t idx = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; idx < total;
         idx += static_cast<std::uint64_t>(gridDim.x) * blockDim.x)
    {
        const std::uint64_t a = idx & (d - 1);
        const std::uint64_t c = (idx >> k) & ((1ull << cbits) - 1);
        const int j = static_cast<int>(idx >> (k + cbits));
        const CompactJob &C = cjobs[j];
        if (a >= compact_rows(C.kq) || c >= static_cast<std::uint64_t>(compact_chunks(C.eq))) continue;
        float re[16], im[16];
        if (a >= (1ull << C.kq))
        {
#pragma unroll
            for (int i = 0; i < 16; ++i) re[i] = im[i] = 0.f;
        }
        else
        {
            const GramJob &J = jobs[j];
            const Cx<float> *psi = states + (static_cast<std::size_t>(J.traj) << n);
            std::uint64_t base = C.fixed, cross = 0;
            for (int b = 0; b < C.kq; ++b)
                if ((a >> b) & 1ull)
                {
                    base |= 1ull << C.kpos[b];
                    cross ^= J.below[b]; // fermionic jobs are never reduced: kpos = kept
                }
            if (!J.fermion) cross = 0;
            for (int b = 4; b < C.eq; ++b)
                if ((c >> (b - 4)) & 1ull) base |= 1ull << C.epos[b];
            std::uint64_t low[4] = {0, 0, 0, 0};
            for (int b = 0; b < 4 && b < C.eq; ++b) low[b] = 1ull << C.epos[b];
            const int ncols = C.eq >= 4 ? 16 : (1 << C.eq);
#pragma unroll
            for (int i = 0; i < 16; ++i)
            {
                const std::uint64_t gi = base | ((i & 1) ? low[0] : 0ull) | ((i & 2) ? low[1] : 0ull) |
                                         ((i & 4) ? low[2] : 0ull) | ((i & 8) ? low[3] : 0ull);
                Cx<float> v{0.f, 0.f};
                if (i < ncols) v = psi[gi];
                const bool keep = i < ncols && (gi & C.mask) == C.value;
                // Fermionic sign: one flip per occupied environment mode
                // below each occupied kept mode (environment index 16c + i).
                const float sg = (__popcll(((c << 4) | static_cast<std::uint64_t>(i)) & cross) & 1) ? -C.scale : C.scale;
                re[i] = keep ? v.re * sg : 0.f;
                im[i] = keep ? v.im * sg : 0.f;
            }
        }
        float4 *hi = rows + idx * 8, *lo = rows + (idx + lo_rows) * 8;
#pragma unroll
        for (int q = 0; q < 8; ++q)
        {
            const float *src = q < 4 ? re + 4 * q : im + 4 * (q - 4);
            float4 h, l;
            tf32_split(src[0], h.x, l.x);
            tf32_split(src[1], h.y, l.y);
            tf32_split(src[2], h.z, l.z);
            tf32_split(src[3], h.w, l.w);
            hi[q] = h;
            lo[q] = l;
        }
    }
}

__device__ __forceinline__ void tp_mma(std::uint32_t d, std::uint64_t a, std::uint64_t b, std::uint32_t idesc,
                                       std::uint32_t acc)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d),
                 "l"(a), "l"(b), "r"(idesc), "r"(acc)
                 : "memory");
}

// Purity partials of one 128 x 128 block of rho for job job0 + blockIdx.z
// from the pre-split rows of the group's job blockIdx.z (tmap: 2-D FP32 view,
// 32 floats per row, box 32 x 64, 128-byte swizzle). Warp TC_PWARPS issues the
// MMAs (Re rho = Re.Re + Im.Im into TMEM columns [0, 128), Im rho = Im.Re -
// Re.Im into [128, 256) of a buffer, each term as 3 TF32 products, N = 128),
// warp TC_PWARPS + 1 the TMA loads (8 boxes per 64 KB stage), and warps
// 0..TC_PWARPS-1 drain the two TMEM buffers into FP32 registers and reduce the
// weighted squares as k_gram_tc does. Every wait is bounded (bit 4 of *err).
__global__ void __launch_bounds__(TP_THREADS, 1)
    k_gram_tc_pre(int n, int k, int job0, double *__restrict__ pur_out, int *__restrict__ err, std::uint32_t lo_rows,
                  const __grid_constant__ CUtensorMap tmap, const CompactJob *__restrict__ cjobs)
{
    extern __shared__ __align__(1024) unsigned char tp_raw[];
    __shared__ __align__(8) std::uint64_t full_bar[TP_STAGES], empty_bar[TP_STAGES], seg_bar[TP_BUFS],
        drained_bar[TP_BUFS];
    __shared__ std::uint32_t tmem_base;
    __shared__ double red[TC_PWARPS];
    __shared__ volatile int abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const std::uint32_t raw_s = sm_addr(tp_raw);
    unsigned char *smem = tp_raw + ((1024u - (raw_s & 1023u)) & 1023u);
    const int job = blockIdx.z;
    int tr, tc;
    tile_coords(blockIdx.x, tr, tc);
    // A block past the job's reduced rows holds zeros only.
    const CompactJob &C = cjobs[job];
    if (static_cast<std::uint32_t>(tr * TCM) >= compact_rows(C.kq))
    {
        if (tid == 0) pur_out[static_cast<std::size_t>(job0 + job) * gridDim.x + blockIdx.x] = 0.0;
        return;
    }
    if (tid == 0)
    {
        for (int st = 0; st < TP_STAGES; ++st)
        {
            mbar_init(&full_bar[st], 1);
            mbar_init(&empty_bar[st], 1);
        }
        for (int b = 0; b < TP_BUFS; ++b)
        {
            mbar_init(&seg_bar[b], 1);
            mbar_init(&drained_bar[b], TC_PWARPS);
        }
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == TC_PWARPS)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sm_addr(&tmem_base)),
                     "n"(TP_BUFS * TP_N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const std::uint32_t tmem = tmem_base;
    const int r0 = tr * TCM, c0 = tc * TCM;
    const int row_chunks = 1 << (n - k - 4); // chunks per job in the row buffer
    const int nchunks = compact_chunks(C.eq); // chunks streamed
    const int nseg = (nchunks + TC_SEG - 1) / TC_SEG;

    if (warp < TC_PWARPS)
    {
        float acc[TP_DCOLS];
#pragma unroll
        for (int i = 0; i < TP_DCOLS; ++i) acc[i] = 0.f;
        const std::uint32_t lane_base = static_cast<std::uint32_t>((warp & 3) * 32) << 16;
        const int col_base = (warp >> 2) * TP_DCOLS;
        for (int seg = 0; seg < nseg && !abort_flag; ++seg)
        {
            const int buf = seg % TP_BUFS;
            if (!mbar_wait(&seg_bar[buf], (seg / TP_BUFS) & 1, &abort_flag, err)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int cb = 0; cb < TP_DCOLS / 32; ++cb)
            {
                std::uint32_t v[32];
                const std::uint32_t taddr = tmem + lane_base + buf * TP_N + col_base + cb * 32;
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                      "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                      "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int i = 0; i < 32; ++i) acc[cb * 32 + i] += __uint_as_float(v[i]);
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&drained_bar[buf]);
        }
        const int r = r0 + (warp & 3) * 32 + lane;
        double sum = 0.0;
        if (!abort_flag)
        {
#pragma unroll
            for (int i = 0; i < TP_DCOLS; ++i)
            {
                const int c = c0 + ((col_base + i) & (TP_C - 1));
                const double w = (r > c) ? 2.0 : ((r == c) ? 1.0 : 0.0);
                const double x = static_cast<double>(acc[i]);
                sum += w * x * x;
            }
        }
        for (int off = 16; off > 0; off /= 2) sum += __shfl_down_sync(0xffffffffu, sum, off);
        if (lane == 0) red[warp] = sum;
    }
    else if (warp == TC_PWARPS && lane == 0)
    {
        for (int chunk = 0; chunk < nchunks; ++chunk)
        {
            const int st = chunk % TP_STAGES;
            const int seg = chunk / TC_SEG;
            const int buf = seg % TP_BUFS;
            if (chunk % TC_SEG == 0 && seg >= TP_BUFS &&
                !mbar_wait(&drained_bar[buf], ((seg / TP_BUFS) - 1) & 1, &abort_flag, err))
                break;
            if (!mbar_wait(&full_bar[st], (chunk / TP_STAGES) & 1, &abort_flag, err)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const std::uint32_t base = sm_addr(smem + st * TP_STAGE);
            const std::uint32_t Ahi = base, Alo = base + TP_A_BYTES;
            const std::uint32_t Bhi = base + 2 * TP_A_BYTES, Blo = Bhi + TP_B_BYTES;
            const std::uint32_t dre = tmem + buf * TP_N, dim = dre + TP_C;
            const bool first = chunk % TC_SEG == 0;
            // Re rho: 32 real K (16 Re then 16 Im) in four K = 8 steps.
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
            {
                const std::uint32_t ko = ks * 32;
                tp_mma(dre, sw128_desc(Ahi + ko), sw128_desc(Bhi + ko), kTpIdesc, (first && ks == 0) ? 0u : 1u);
                tp_mma(dre, sw128_desc(Ahi + ko), sw128_desc(Blo + ko), kTpIdesc, 1u);
                tp_mma(dre, sw128_desc(Alo + ko), sw128_desc(Bhi + ko), kTpIdesc, 1u);
            }
            // Im rho = Im(A).Re(B) - Re(A).Im(B).
#pragma unroll
            for (int ps = 0; ps < 4; ++ps)
            {
                const std::uint32_t ka = (ps < 2 ? 64u : 0u) + (ps & 1) * 32u;
                const std::uint32_t kb = (ps < 2 ? 0u : 64u) + (ps & 1) * 32u;
                const std::uint32_t id = ps < 2 ? kTpIdesc : kTpIdescNegA;
                tp_mma(dim, sw128_desc(Ahi + ka), sw128_desc(Bhi + kb), id, (first && ps == 0) ? 0u : 1u);
                tp_mma(dim, sw128_desc(Ahi + ka), sw128_desc(Blo + kb), id, 1u);
                tp_mma(dim, sw128_desc(Alo + ka), sw128_desc(Bhi + kb), id, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             sm_addr(&empty_bar[st]))
                         : "memory");
            if (chunk % TC_SEG == TC_SEG - 1 || chunk == nchunks - 1)
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 sm_addr(&seg_bar[buf]))
                             : "memory");
        }
    }
    else if (warp == TC_PWARPS + 1 && lane == 0)
    {
        int issued = 0;
        const std::uint64_t tm = reinterpret_cast<std::uint64_t>(&tmap);
        for (int chunk = 0; chunk < nchunks; ++chunk)
        {
            const int st = chunk % TP_STAGES;
            if (chunk >= TP_STAGES &&
                !mbar_wait(&empty_bar[st], ((chunk / TP_STAGES) - 1) & 1, &abort_flag, err))
                break;
            const std::uint32_t bar = sm_addr(&full_bar[st]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(TP_STAGE)
                         : "memory");
            const std::uint32_t base = sm_addr(smem + st * TP_STAGE);
            const int yb = static_cast<int>((static_cast<std::uint32_t>(job) * row_chunks + chunk) << k);
            const int lo = static_cast<int>(lo_rows);
            const std::uint32_t Bb = base + 2 * TP_A_BYTES;
            const std::uint32_t dst[8] = {base, base + 8192, base + TP_A_BYTES, base + TP_A_BYTES + 8192,
                                          Bb, Bb + 8192, Bb + TP_B_BYTES, Bb + TP_B_BYTES + 8192};
            const int ys[8] = {yb + r0, yb + r0 + 64, lo + yb + r0, lo + yb + r0 + 64,
                               yb + c0, yb + c0 + 64, lo + yb + c0, lo + yb + c0 + 64};
#pragma unroll
            for (int b = 0; b < 8; ++b)
                asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
                             "%3}], [%4];" ::"r"(dst[b]),
                             "l"(tm), "r"(0), "r"(ys[b]), "r"(bar)
                             : "memory");
            issued = chunk + 1;
        }
        // After an abort, let the loads still in flight land.
        for (int c = issued - TP_STAGES > 0 ? issued - TP_STAGES : 0; c < issued; ++c)
            mbar_settle(&full_bar[c % TP_STAGES], (c / TP_STAGES) & 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0)
    {
        double t = 0.0;
        for (int w = 0; w < TC_PWARPS; ++w) t += red[w];
        pur_out[static_cast<std::size_t>(job0 + job) * gridDim.x + blockIdx.x] = t;
    }
    if (warp == TC_PWARPS)
    {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TP_BUFS * TP_N)
                     : "memory");
    }
}
} // namespace

bool gram_tc_supported(int n, int k)
{
    static const bool on = [] {
        const char *v = std::getenv("MIPT_GB300_TC_GRAM");
        return !(v && v[0] == '0');
    }();
    return on && k >= 7 && k <= 16 && (n - k) >= 4;
}

// Lower-triangle 128-row blocks of rho.
int gram_tc_blocks(int k)
{
    const int t = 1 << (k - 7);
    return t * (t + 1) / 2;
}

// CTAs (and purity partials) per job: every block is split into two
// 64-column halves.
int gram_tc_tiles(int k) { return 2 * gram_tc_blocks(k); }

std::size_t gram_tc_scratch_bytes(int k, int njobs)
{
    // Purity partials, then the reduced job table of the pre-split path.
    return sizeof(double) * static_cast<std::size_t>(gram_tc_tiles(k)) * njobs +
           sizeof(CompactJob) * static_cast<std::size_t>(njobs);
}

namespace
{
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}
} // namespace

bool gram_tc_presplit_enabled()
{
    static const bool on = [] {
        const char *v = std::getenv("MIPT_GB300_TC_PRESPLIT");
        return !(v && v[0] == '0');
    }();
    return on;
}

std::size_t gram_tc_rows_bytes_per_job(int n) { return (std::size_t{16}) << n; }

int gram_tc_presplit_max_k()
{
    static const int k = [] {
        const char *v = std::getenv("MIPT_GB300_TC_PRESPLIT_MAX_K");
        return (v && *v) ? std::atoi(v) : 14;
    }();
    return k;
}

cudaError_t gram_purity_tc(const Cx<float> *states, int n, const GramJob *d_jobs, int njobs, int k,
                           const Collapse *collapse, std::size_t collapse_stride, double *purity_out, void *scratch,
                           std::size_t scratch_bytes, int *err, cudaStream_t s, int tma_traj_count, void *rows,
                           std::size_t rows_bytes)
{
    if (njobs <= 0) return cudaSuccess;
    if (!gram_tc_supported(n, k)) return cudaErrorInvalidValue;
    const int tiles = gram_tc_tiles(k);
    if (gram_tc_scratch_bytes(k, njobs) > scratch_bytes) return cudaErrorInvalidValue;
    const std::size_t per_job = gram_tc_rows_bytes_per_job(n);
    // Measured against the gathered path: L = 24 half cut (k = 12) 85 -> 39 ms
    // for 32 states, L = 28 lattice half (k = 14) 1.8x faster per layer; k = 15
    // and 16 stay on the gathered path (not measured).
    if (k <= gram_tc_presplit_max_k() && rows != nullptr && rows_bytes >= per_job && tensor_map_encoder() != nullptr &&
        (reinterpret_cast<std::uintptr_t>(rows) & 15u) == 0)
    {
        // Pre-split operand rows, jobs in groups that fit `rows`.
        const int group = static_cast<int>(std::min<std::size_t>(static_cast<std::size_t>(njobs), rows_bytes / per_job));
        cudaError_t e = cudaFuncSetAttribute(k_gram_tc_pre, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(TP_SMEM));
        if (e != cudaSuccess) return e;
        CompactJob *cjobs = reinterpret_cast<CompactJob *>(static_cast<char *>(scratch) +
                                                           sizeof(double) * static_cast<std::size_t>(gram_tc_tiles(k)) *
                                                               njobs);
        k_compact_jobs<<<(njobs + 127) / 128, 128, 0, s>>>(d_jobs, njobs, n, k, collapse, collapse_stride,
                                                           measured_compact_enabled() ? 1 : 0, cjobs);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        for (int g0 = 0; g0 < njobs; g0 += group)
        {
            const int g = std::min(group, njobs - g0);
            const std::uint64_t lo_rows = static_cast<std::uint64_t>(g) << (n - 4);
            if (2 * lo_rows >= (1ull << 31)) return cudaErrorInvalidValue;
            CUtensorMap map;
            std::memset(&map, 0, sizeof(map));
            const cuuint64_t dims[2] = {32, 2 * lo_rows};
            const cuuint64_t strides[1] = {128};
            const cuuint32_t box[2] = {32, 64};
            const cuuint32_t estr[2] = {1, 1};
            if (tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, rows, dims, strides, box, estr,
                                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                return cudaErrorInvalidValue;
            const std::uint64_t nrows = lo_rows;
            const int blocks = static_cast<int>(std::min<std::uint64_t>((nrows + 255) / 256, 152ull * 8));
            k_tf32_rows<<<blocks, 256, 0, s>>>(states, n, k, d_jobs + g0, cjobs + g0, g,
                                               static_cast<float4 *>(rows), lo_rows);
            e = cudaGetLastError();
            if (e != cudaSuccess) return e;
            dim3 grid(gram_tc_blocks(k), 1, g);
            k_gram_tc_pre<<<grid, TP_THREADS, TP_SMEM, s>>>(n, k, g0, static_cast<double *>(scratch), err,
                                                            static_cast<std::uint32_t>(lo_rows), map, cjobs + g0);
            e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
        k_sum_rows<<<njobs, 256, 0, s>>>(static_cast<const double *>(scratch), gram_tc_blocks(k), purity_out);
        return cudaGetLastError();
    }
    CUtensorMap map;
    std::memset(&map, 0, sizeof(map));
    const std::uint64_t state_rows = static_cast<std::uint64_t>(tma_traj_count) << (n - k);
    bool tma = tma_traj_count > 0 && state_rows < (1ull << 31) && tensor_map_encoder() != nullptr &&
               (reinterpret_cast<std::uintptr_t>(states) & 15u) == 0;
    if (tma)
    {
        const cuuint64_t dims[2] = {1ull << k, state_rows};
        const cuuint64_t strides[1] = {(1ull << k) * sizeof(Cx<float>)};
        const cuuint32_t box[2] = {64, 16};
        const cuuint32_t estr[2] = {1, 1};
        tma = tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<Cx<float> *>(states), dims,
                                   strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    }
    auto kernel = tma ? k_gram_tc<true> : k_gram_tc<false>;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(TC_SMEM));
    if (e != cudaSuccess) return e;
    dim3 grid(gram_tc_blocks(k), 2, njobs);
    kernel<<<grid, TC_THREADS, TC_SMEM, s>>>(states, n, d_jobs, collapse, collapse_stride,
                                             static_cast<double *>(scratch), err, map);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_sum_rows<<<njobs, 256, 0, s>>>(static_cast<const double *>(scratch), tiles, purity_out);
    return cudaGetLastError();
}

#define MG_INST(R)                                                                                               \
    template cudaError_t gram_rho<R>(const Cx<R> *, int, const GramJob *, int, int, const Collapse *, std::size_t, \
                                     double *, void *, std::size_t, cudaStream_t, int *);                        \
    template cudaError_t gram_purity<R>(const Cx<R> *, int, const GramJob *, int, int, const Collapse *,          \
                                        std::size_t, double *, void *, std::size_t, cudaStream_t);               \
    template cudaError_t rho3_sweep<R>(const Cx<R> *, int, int, const int *, int, int, const Collapse *,          \
                                       std::size_t, double *, void *, std::size_t, cudaStream_t);
MG_INST(float)
MG_INST(double)
#undef MG_INST

} // namespace mg
