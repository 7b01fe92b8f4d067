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

#include <algorithm>
#include <cmath>
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

template <typename Real>
__device__ __forceinline__ Cx<Real> gather(const Cx<Real> *__restrict__ psi, std::uint64_t addr, const Collapse &cl,
                                           bool has_col, bool negate)
{
    Cx<Real> v = psi[addr];
    if (has_col)
    {
        if ((addr & cl.mask) != cl.value) return Cx<Real>{Real(0), Real(0)};
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
// Acc is the accumulation type: FP64 whenever rho is materialised (its
// small eigenvalues feed -lambda log lambda, so accumulation rounding must
// stay below the state's own second-order error), the operand type for the
// purity-only mode.
template <typename Real, typename Acc>
__global__ void __launch_bounds__(kGramThreads)
    k_gram(const Cx<Real> *__restrict__ states, int n, const GramJob *__restrict__ jobs,
           const Collapse *__restrict__ col, std::size_t col_stride, int splits, std::uint64_t kchunk, int mode,
           Acc *__restrict__ part_out, double *__restrict__ pur_out)
{
    constexpr int TK = GramK<Real>::TK;
    constexpr int KB = GramK<Real>::BITS;
    __shared__ GramJob J;
    __shared__ Cx<Real> As[TK][TM + 1];
    __shared__ Cx<Real> Bs[TK][TM + 1];
    __shared__ std::uint64_t roffA[TM], roffB[TM], crossA[TM], crossB[TM], elo[TK];
    __shared__ double red[kGramThreads / 32];

    const int tid = threadIdx.x;
    const int job = blockIdx.z;
    if (tid == 0) J = jobs[job];
    __syncthreads();
    const int k = J.k;
    const int d = 1 << k;
    int tr, tc;
    tile_coords(blockIdx.x, tr, tc);
    const int r0 = tr * TM, c0 = tc * TM;
    const int nenv = n - k;
    const std::uint64_t E = 1ull << nenv;
    const std::uint64_t ebeg = static_cast<std::uint64_t>(blockIdx.y) * kchunk;
    const std::uint64_t eend = ebeg + kchunk < E ? ebeg + kchunk : E;

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
    Collapse cl{0, 0, 1.0, 0.0};
    const bool has_col = col != nullptr;
    if (has_col) cl = col[J.traj * col_stride];
    __syncthreads();

    const Cx<Real> *psi = states + (static_cast<std::size_t>(J.traj) << n);
    const int ty = tid / 16, tx = tid % 16;
    Acc accr[4][4], acci[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) accr[i][j] = acci[i][j] = Acc(0);

    for (std::uint64_t e0 = ebeg; e0 < eend; e0 += TK)
    {
        std::uint64_t ehi = 0;
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
                    va = gather(psi, eo | roffA[i], cl, has_col, (__popcll(e & crossA[i]) & 1) != 0);
                if (c0 + i < d)
                    vb = gather(psi, eo | roffB[i], cl, has_col, (__popcll(e & crossB[i]) & 1) != 0);
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
                    // a * conj(b); FP32 x FP32 products are exact in FP64
                    accr[i][j] = fma(Acc(a[i].re), Acc(b[j].re), accr[i][j]);
                    accr[i][j] = fma(Acc(a[i].im), Acc(b[j].im), accr[i][j]);
                    acci[i][j] = fma(Acc(a[i].im), Acc(b[j].re), acci[i][j]);
                    acci[i][j] = fma(-Acc(a[i].re), Acc(b[j].im), acci[i][j]);
                }
        }
        __syncthreads();
    }

    if (mode == 0)
    {
        Acc *out = part_out + (static_cast<std::size_t>(job) * splits + blockIdx.y) * static_cast<std::size_t>(d) * d * 2;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
            {
                const int r = r0 + ty * 4 + i, c = c0 + tx * 4 + j;
                if (r < d && c < d && r >= c)
                {
                    out[(static_cast<std::size_t>(r) * d + c) * 2] = accr[i][j];
                    out[(static_cast<std::size_t>(r) * d + c) * 2 + 1] = acci[i][j];
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
    Collapse cl{0, 0, 1.0, 0.0};
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
                     std::size_t scratch_bytes, cudaStream_t s)
{
    if (njobs <= 0) return cudaSuccess;
    const int splits = gram_splits(n, k, njobs, true);
    const std::size_t need = sizeof(double) * 2 * static_cast<std::size_t>(splits) * njobs * (std::size_t{1} << (2 * k));
    if (need > scratch_bytes) return cudaErrorInvalidValue;
    const std::uint64_t E = 1ull << (n - k);
    const std::uint64_t kchunk = (E + splits - 1) / splits;
    dim3 grid(gram_tiles(k), splits, njobs);
    k_gram<Real, double><<<grid, kGramThreads, 0, s>>>(states, n, d_jobs, collapse, collapse_stride, splits, kchunk,
                                                       0, static_cast<double *>(scratch), nullptr);
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
                                                     static_cast<double *>(scratch));
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

#define MG_INST(R)                                                                                               \
    template cudaError_t gram_rho<R>(const Cx<R> *, int, const GramJob *, int, int, const Collapse *, std::size_t, \
                                     double *, void *, std::size_t, cudaStream_t);                               \
    template cudaError_t gram_purity<R>(const Cx<R> *, int, const GramJob *, int, int, const Collapse *,          \
                                        std::size_t, double *, void *, std::size_t, cudaStream_t);               \
    template cudaError_t rho3_sweep<R>(const Cx<R> *, int, int, const int *, int, int, const Collapse *,          \
                                       std::size_t, double *, void *, std::size_t, cudaStream_t);
MG_INST(float)
MG_INST(double)
#undef MG_INST

} // namespace mg
