// Tiled layer passes, fused Born histograms, on-device outcome sampling and
// deferred collapse for batches of state vectors.
//
// Reference behaviour reproduced (paths inside the reference project):
//   gate application  = custatevecApplyMatrix with a row-major matrix whose
//                       index bit k is targets[k]   cpp/include/mipt/cusv/engine.hpp:236-277,
//                                                   cpp/include/mipt/cusv/matrix.hpp:5-13
//   layer measurement = Engine::measure_layer: chunks of <= chunk_bits sites,
//                       joint histogram, one uniform per chunk, linear CDF
//                       scan, starved-bin fallback to the heaviest bin,
//                       collapse scaled by 1/sqrt(branch)
//                                                   cpp/include/mipt/cusv/engine.hpp:293-368
#include "engine.cuh"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

#include <cooperative_groups.h>
#include <cuda.h>
#include <cudaTypedefs.h>

namespace mg
{

namespace
{
constexpr int kPassThreads = 512;
constexpr int kMeasureThreads = 1024;
constexpr int kSmemBins = 4096;

template <typename Real> struct Acc;
// FP32 amplitudes: per-thread runs of 64 squared magnitudes in FP32,
// promoted to FP64 (the reference's mixed-precision sweep scheme,
// cpp/include/mipt/cuda/reduce_sweep.cuh:59-96).
template <> struct Acc<float>
{
    double total = 0.0;
    float run = 0.f;
    int count = 0;
    __device__ void add(float v)
    {
        run += v;
        if (++count == 64)
        {
            total += static_cast<double>(run);
            run = 0.f;
            count = 0;
        }
    }
    __device__ double value() const { return total + static_cast<double>(run); }
};
template <> struct Acc<double>
{
    double total = 0.0;
    __device__ void add(double v) { total += v; }
    __device__ double value() const { return total; }
};

template <typename Real>
__device__ __forceinline__ Real norm2(Cx<Real> v)
{
    return v.re * v.re + v.im * v.im;
}

// Deterministic histogram of a tile in shared memory over the local bit
// positions lm[0..m_loc): out[bin] = sum of |tile[j]|^2 over j whose bits at
// lm[i] spell bin. Fixed summation order for a given launch shape.
template <typename Real>
__device__ void tile_histogram(const Cx<Real> *tile, int k, const int *lm, int m_loc, double *out, double *red)
{
    const int T = blockDim.x;
    const int tid = threadIdx.x;
    const std::uint64_t nb = 1ull << m_loc;
    const std::uint64_t per_bin = 1ull << (k - m_loc);
    if (nb <= static_cast<std::uint64_t>(T))
    {
        const int G = T / static_cast<int>(nb);
        const std::uint64_t bin = tid / G;
        const int sub = tid % G;
        std::uint64_t fixed = 0;
        for (int i = 0; i < m_loc; ++i) fixed |= ((bin >> i) & 1ull) << lm[i];
        Acc<Real> acc;
        for (std::uint64_t r = sub; r < per_bin; r += G)
        {
            std::uint64_t j = r;
            for (int i = 0; i < m_loc; ++i) j = insert_zero(j, lm[i]);
            acc.add(norm2(tile[j | fixed]));
        }
        double v = acc.value();
        // Tree over the G threads of this bin: shuffles inside a warp, then
        // a fixed-order sum of warp results.
        const int width = G < 32 ? G : 32;
        for (int off = width / 2; off > 0; off /= 2) v += __shfl_down_sync(0xffffffffu, v, off, width);
        if (G <= 32)
        {
            if (sub == 0) out[bin] = v;
        }
        else
        {
            if ((tid & 31) == 0) red[tid >> 5] = v;
            __syncthreads();
            if (sub == 0)
            {
                double s = 0.0;
                for (int w = 0; w < G / 32; ++w) s += red[(tid >> 5) + w];
                out[bin] = s;
            }
        }
    }
    else
    {
        for (std::uint64_t bin = tid; bin < nb; bin += T)
        {
            std::uint64_t fixed = 0;
            for (int i = 0; i < m_loc; ++i) fixed |= ((bin >> i) & 1ull) << lm[i];
            Acc<Real> acc;
            for (std::uint64_t r = 0; r < per_bin; ++r)
            {
                std::uint64_t j = r;
                for (int i = 0; i < m_loc; ++i) j = insert_zero(j, lm[i]);
                acc.add(norm2(tile[j | fixed]));
            }
            out[bin] = acc.value();
        }
    }
}

template <typename Real>
__device__ __forceinline__ Cx<Real> collapse_value(Cx<Real> v, std::uint64_t gidx, const Collapse &cl, Real scale)
{
    if (!collapse_keeps(gidx, cl)) return Cx<Real>{Real(0), Real(0)};
    return Cx<Real>{v.re * scale, v.im * scale};
}

// Bits r of a register index whose bit i is set (r < 64).
__host__ __device__ constexpr std::uint64_t reg_bit_pattern(int i)
{
    return i == 0 ? 0xAAAAAAAAAAAAAAAAull
         : i == 1 ? 0xCCCCCCCCCCCCCCCCull
         : i == 2 ? 0xF0F0F0F0F0F0F0F0ull
         : i == 3 ? 0xFF00FF00FF00FF00ull
         : i == 4 ? 0xFFFF0000FFFF0000ull
                  : 0xFFFFFFFF00000000ull;
}

// Which of a thread's 2^RB register elements a pending collapse keeps, as a
// bit mask over the register index r. Element r has the global index gt | (the
// gr[i] of r's set bits), the gr[i] being single bits outside gt. The mask /
// value test splits into the thread's part (all or nothing) and one pattern
// per register bit in the mask; the parity condition of parity-sector states
// (PAR) is the XOR of the patterns of the register bits it covers.
template <int RB, bool PAR>
__device__ __forceinline__ std::uint64_t collapse_keep_bits(std::uint64_t gt, const std::uint64_t (&gr)[RB],
                                                            const Collapse &cl)
{
    constexpr std::uint64_t full = RB == 6 ? ~0ull : ((1ull << (1 << RB)) - 1ull);
    std::uint64_t rpos = 0;
#pragma unroll
    for (int i = 0; i < RB; ++i) rpos |= gr[i];
    const std::uint64_t mt = cl.mask & ~rpos;
    if ((gt & mt) != (cl.value & mt)) return 0;
    std::uint64_t keep = full;
#pragma unroll
    for (int i = 0; i < RB; ++i)
        if (gr[i] & cl.mask) keep &= (gr[i] & cl.value) ? reg_bit_pattern(i) : ~reg_bit_pattern(i);
    if constexpr (PAR)
    {
        if (cl.parity != 0)
        {
            const std::uint64_t pm = cl.parity & ~kParityBit;
            std::uint64_t odd = 0;
#pragma unroll
            for (int i = 0; i < RB; ++i)
                if (gr[i] & pm) odd ^= reg_bit_pattern(i);
            const bool want_odd = ((cl.parity >> 63) ^ static_cast<std::uint64_t>(__popcll(gt & pm) & 1)) != 0;
            keep &= want_odd ? odd : ~odd;
        }
    }
    return keep & full;
}

// Applies a keep mask and the collapse's renormalisation to the registers.
template <typename Real, int NA>
__device__ __forceinline__ void apply_keep_bits(Cx<Real> (&a)[NA], std::uint64_t keep, Real scale)
{
    constexpr std::uint64_t full = NA == 64 ? ~0ull : ((1ull << NA) - 1ull);
    if (keep == full && scale == Real(1)) return;
#pragma unroll
    for (int r = 0; r < NA; ++r)
    {
        const bool k = (keep >> r) & 1ull;
        a[r] = k ? Cx<Real>{a[r].re * scale, a[r].im * scale} : Cx<Real>{Real(0), Real(0)};
    }
}

// Loads the tile of geometry g with index tix into shared memory, applying a
// pending collapse. seg[s] holds the offset of high segment s.
template <typename Real>
__device__ void load_tile(Cx<Real> *tile, const Cx<Real> *__restrict__ psi, const PassGeom &g, std::uint64_t base,
                          const std::uint32_t *seg, const Collapse &cl, bool has_col)
{
    const std::uint64_t nloc = 1ull << g.k;
    const std::uint64_t cmask = (1ull << g.c) - 1ull;
    const Real scale = static_cast<Real>(cl.scale);
    for (std::uint64_t j = threadIdx.x; j < nloc; j += blockDim.x)
    {
        const std::uint64_t gidx = base | seg[j >> g.c] | (j & cmask);
        Cx<Real> v = psi[gidx];
        if (has_col) v = collapse_value(v, gidx, cl, scale);
        tile[j] = v;
    }
}

template <typename Real>
__global__ void __launch_bounds__(kPassThreads) k_pass(Cx<Real> *__restrict__ states, PassGeom g, PassGates pg,
                                                       const Cx<Real> *__restrict__ gates, std::size_t gate_stride,
                                                       const Collapse *__restrict__ col_in, std::size_t col_stride,
                                                       const LayerMeas *__restrict__ meas, std::size_t meas_stride,
                                                       double *__restrict__ partials, int fuse_hist)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx<Real> *tile = reinterpret_cast<Cx<Real> *>(smem_raw);
    std::uint32_t *seg = reinterpret_cast<std::uint32_t *>(smem_raw + (sizeof(Cx<Real>) << g.k));
    __shared__ Cx<Real> U[kMaxPassGates][16];
    __shared__ double red[kPassThreads / 32];

    const int b = blockIdx.y;
    const std::uint64_t tix = blockIdx.x;
    const std::uint64_t dim = 1ull << g.n;
    Cx<Real> *psi = states + static_cast<std::size_t>(b) * dim;
    const std::uint64_t base = scatter_bits(tix, g.nl, g.n_nl);
    const int h = g.k - g.c;
    for (std::uint32_t s = threadIdx.x; s < (1u << h); s += blockDim.x)
        seg[s] = static_cast<std::uint32_t>(scatter_bits(s, g.pos + g.c, h));
    for (int i = threadIdx.x; i < pg.count * 16; i += blockDim.x)
        U[i / 16][i % 16] = gates[b * gate_stride + static_cast<std::size_t>(pg.gate[i / 16]) * 16 + (i % 16)];
    Collapse cl{0, 0, 1.0, 0};
    const bool has_col = col_in != nullptr;
    if (has_col) cl = col_in[b * col_stride];
    __syncthreads();

    load_tile(tile, psi, g, base, seg, cl, has_col);
    __syncthreads();

    const std::uint64_t groups = 1ull << (g.k - 2);
    const int bpar = __popcll(base) & 1;
    for (int gi = 0; gi < pg.count; ++gi)
    {
        if (pg.kind[gi])
        {
            // Parity-selected 2x2 on local bit la: the block is chosen by the
            // parity of the element's other index bits (tile base + local).
            const int a = pg.la[gi];
            Cx<Real> u[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) u[e] = U[gi][e];
            for (std::uint64_t pr = threadIdx.x; pr < (1ull << (g.k - 1)); pr += blockDim.x)
            {
                const std::uint64_t j0 = insert_zero(pr, a), j1 = j0 | (1ull << a);
                const int o = ((bpar + __popcll(j0)) & 1) * 4;
                const Cx<Real> x0 = tile[j0], x1 = tile[j1];
                tile[j0] = cfma(u[o + 1], x1, cmul(u[o], x0));
                tile[j1] = cfma(u[o + 3], x1, cmul(u[o + 2], x0));
            }
            __syncthreads();
            continue;
        }
        const int a = pg.la[gi], bb = pg.lb[gi];
        const int lo = a < bb ? a : bb, hi = a < bb ? bb : a;
        Cx<Real> u[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) u[e] = U[gi][e];
        const std::uint64_t ma = 1ull << a, mb = 1ull << bb;
        for (std::uint64_t grp = threadIdx.x; grp < groups; grp += blockDim.x)
        {
            const std::uint64_t j0 = insert_zero(insert_zero(grp, lo), hi);
            const std::uint64_t idx[4] = {j0, j0 | ma, j0 | mb, j0 | ma | mb};
            Cx<Real> in[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) in[c] = tile[idx[c]];
#pragma unroll
            for (int r = 0; r < 4; ++r)
            {
                Cx<Real> acc = cmul(u[4 * r], in[0]);
                acc = cfma(u[4 * r + 1], in[1], acc);
                acc = cfma(u[4 * r + 2], in[2], acc);
                acc = cfma(u[4 * r + 3], in[3], acc);
                tile[idx[r]] = acc;
            }
        }
        __syncthreads();
    }

    const std::uint64_t nloc = 1ull << g.k;
    const std::uint64_t cmask = (1ull << g.c) - 1ull;
    for (std::uint64_t j = threadIdx.x; j < nloc; j += blockDim.x)
        psi[base | seg[j >> g.c] | (j & cmask)] = tile[j];

    if (fuse_hist)
    {
        const LayerMeas &M = meas[b * meas_stride];
        if (M.nchunks > 0)
        {
            const std::uint64_t chunk = M.chunk[0];
            int lm[kMaxLocal + 1];
            int m_loc = 0;
            for (int i = 0; i < g.k; ++i)
                if ((chunk >> g.pos[i]) & 1ull) lm[m_loc++] = i;
            double *part = partials + static_cast<std::size_t>(b) * kHistScratch + (tix << m_loc);
            tile_histogram(tile, g.k, lm, m_loc, part, red);
        }
    }
}


// Deterministic histogram over an array of squared magnitudes in shared
// memory (same traversal as tile_histogram).
template <typename T>
__device__ void value_histogram(const T *val, int k, const int *lm, int m_loc, double *out, double *red)
{
    const int T_ = blockDim.x;
    const int tid = threadIdx.x;
    const std::uint64_t nb = 1ull << m_loc;
    const std::uint64_t per_bin = 1ull << (k - m_loc);
    if (nb <= static_cast<std::uint64_t>(T_))
    {
        const int G = T_ / static_cast<int>(nb);
        const std::uint64_t bin = tid / G;
        const int sub = tid % G;
        std::uint64_t fixed = 0;
        for (int i = 0; i < m_loc; ++i) fixed |= ((bin >> i) & 1ull) << lm[i];
        Acc<T> acc;
        for (std::uint64_t r = sub; r < per_bin; r += G)
        {
            std::uint64_t j = r;
            for (int i = 0; i < m_loc; ++i) j = insert_zero(j, lm[i]);
            acc.add(val[j | fixed]);
        }
        double v = acc.value();
        const int width = G < 32 ? G : 32;
        for (int off = width / 2; off > 0; off /= 2) v += __shfl_down_sync(0xffffffffu, v, off, width);
        if (G <= 32)
        {
            if (sub == 0) out[bin] = v;
        }
        else
        {
            if ((tid & 31) == 0) red[tid >> 5] = v;
            __syncthreads();
            if (sub == 0)
            {
                double s = 0.0;
                for (int w = 0; w < G / 32; ++w) s += red[(tid >> 5) + w];
                out[bin] = s;
            }
        }
    }
    else
    {
        for (std::uint64_t bin = tid; bin < nb; bin += T_)
        {
            std::uint64_t fixed = 0;
            for (int i = 0; i < m_loc; ++i) fixed |= ((bin >> i) & 1ull) << lm[i];
            Acc<T> acc;
            for (std::uint64_t r = 0; r < per_bin; ++r)
            {
                std::uint64_t j = r;
                for (int i = 0; i < m_loc; ++i) j = insert_zero(j, lm[i]);
                acc.add(val[j | fixed]);
            }
            out[bin] = acc.value();
        }
    }
}

// Born histogram of an FP32 tile straight from the registers of the pass's
// last round, in a fixed order. Squared magnitudes are folded over the
// unmeasured register bits in registers (pairwise FP32 adds); every thread
// then stores its 2^RB values to S[(warp * 2^RB + r) * L + lane] (L lanes per
// warp; S needs 2^k floats), and the bins are summed from there: bin `bin`
// collects the entries whose measured bits spell it, over all values of the
// unmeasured lane and warp bits, G threads per bin each summing a fixed
// slice and a shuffle tree joining the G partial sums. `mmask` is the measured
// set in tile positions (bin bit i <-> i-th measured position from the
// bottom); out[bin] as in value_histogram. Rounding: pairwise register folds
// and shuffle trees plus sequential runs of at most 2^(TB - log2 G) terms in
// FP32, within the reference's scheme of FP32 runs of 64
// (cpp/include/mipt/cuda/reduce_sweep.cuh:59-96); the per-bin result is
// widened to FP64.
template <int RB>
__device__ void register_histogram(const Cx<float> (&amp)[1 << RB], const Round &Z, int TB, std::uint32_t mmask,
                                   int m_loc, float *S, int *tab, double *out)
{
    constexpr int NA = 1 << RB;
    const int tid = threadIdx.x;
    const int nl = TB < 5 ? TB : 5;
    const int L = 1 << nl;
    const unsigned lanes = TB >= 5 ? 0xffffffffu : ((1u << L) - 1u);
    float p[NA];
#pragma unroll
    for (int r = 0; r < NA; ++r) p[r] = norm2(amp[r]);
    unsigned um_reg = 0;
#pragma unroll
    for (int i = 0; i < RB; ++i)
        if (!((mmask >> Z.reg[i]) & 1u)) um_reg |= 1u << i;
#pragma unroll
    for (int i = 0; i < RB; ++i)
        if ((um_reg >> i) & 1u)
        {
#pragma unroll
            for (int r = 0; r < NA; ++r)
                if (!((r >> i) & 1)) p[r] += p[r | (1 << i)];
        }
    // tab[q], q < k: offset in S of tile position q; tab[16 + t]: offset of
    // the t-th unmeasured thread bit; tab[31]: their count.
    for (int q = tid; q < 16; q += blockDim.x)
    {
        int st = 0;
        for (int j = 0; j < RB; ++j)
            if (Z.reg[j] == q) st = (1 << j) * L;
        for (int j = 0; j < TB; ++j)
            if (Z.tid[j] == q) st = j < nl ? (1 << j) : (1 << (j - nl)) * NA * L;
        tab[q] = st;
    }
    if (tid == 0)
    {
        int uc = 0;
        for (int j = 0; j < TB; ++j)
            if (!((mmask >> Z.tid[j]) & 1u)) tab[16 + uc++] = j < nl ? (1 << j) : (1 << (j - nl)) * NA * L;
        tab[31] = uc;
    }
    __syncthreads(); // the tile buffer is free; tab is ready
    {
        float *row = S + (static_cast<std::size_t>((tid >> 5) * NA) << nl) + (tid & 31);
#pragma unroll
        for (int r = 0; r < NA; ++r) row[r << nl] = p[r];
    }
    __syncthreads();
    const int uc = tab[31];
    const int nbin = 1 << m_loc;
    const int T = blockDim.x;
    const int G = nbin >= T ? 1 : (T / nbin < 32 ? T / nbin : 32);
    const int per = (1 << uc) / G > 0 ? (1 << uc) / G : 1;
    for (int w = tid / G; w < nbin; w += T / G)
    {
        const int sub = tid % G;
        int off = 0;
        {
            std::uint32_t mm = mmask;
            for (int i = 0; i < m_loc; ++i)
            {
                const int q = __ffs(mm) - 1;
                mm &= mm - 1u;
                if ((w >> i) & 1) off += tab[q];
            }
        }
        float s = 0.f;
        // This lane's terms c0 .. c0 + cnt - 1 (cnt is 0 or `per`, a power of
        // two). The offsets of the unmeasured bits are distinct powers of
        // two, so the terms are visited in Gray-code order of their low bits:
        // each step flips one bit of the offset.
        const int c0 = sub * per;
        const int cnt = (1 << uc) - c0 < per ? (1 << uc) - c0 : per;
        if (cnt > 0)
        {
            int o = off;
            for (int t = 0; t < uc; ++t)
                if ((c0 >> t) & 1) o += tab[16 + t];
            for (int i = 0;;)
            {
                s += S[o];
                if (++i >= cnt) break;
                o ^= tab[16 + __ffs(i) - 1];
            }
        }
        for (int d = G >> 1; d > 0; d >>= 1) s += __shfl_down_sync(lanes, s, d, G);
        if (sub == 0) out[w] = static_cast<double>(s);
    }
}

// Position of tile bit p once tile bit x is removed (CTA-local offset).
__device__ __forceinline__ int opos_d(int p, int x) { return p > x ? p - 1 : p; }

// XOR swizzle of one local tile bit: bits >= 5 also flip low bit (p mod 5),
// so any five lanes whose tile bits have distinct residues mod 5 touch
// distinct shared-memory banks. Linear over GF(2): swz(a ^ b) = swz(a) ^ swz(b).
__device__ __forceinline__ std::uint32_t swz1(int p)
{
    return (1u << p) ^ (p >= 5 ? (1u << (p % 5)) : 0u);
}

// Applies a 4x4 gate on register-index bits (2S, 2S+1); matrix index bit 0
// is register bit 2S. All register indices are compile-time constants.
template <int S, typename Real, int NA>
__device__ __forceinline__ void apply_slot(Cx<Real> (&a)[NA], const Cx<Real> *__restrict__ Us)
{
    constexpr int lo = 2 * S;
    Cx<Real> u[16];
#pragma unroll
    for (int e = 0; e < 16; ++e) u[e] = Us[e];
#pragma unroll
    for (int g = 0; g < NA / 4; ++g)
    {
        const int base = ((g >> lo) << (lo + 2)) | (g & ((1 << lo) - 1));
        const Cx<Real> in0 = a[base], in1 = a[base | (1 << lo)], in2 = a[base | (2 << lo)], in3 = a[base | (3 << lo)];
#pragma unroll
        for (int r = 0; r < 4; ++r)
        {
            Cx<Real> acc = cmul(u[4 * r], in0);
            acc = cfma(u[4 * r + 1], in1, acc);
            acc = cfma(u[4 * r + 2], in2, acc);
            acc = cfma(u[4 * r + 3], in3, acc);
            a[base | (r << lo)] = acc;
        }
    }
}


// FP32 variant of apply_slot on Blackwell's packed FP32x2 FMA: for
// acc += u * in, acc = fma2({u.re, u.re}, {in.re, in.im}, acc) then
// acc = fma2({-u.im, u.im}, {in.im, in.re}, acc) -- two packed FMAs per
// complex multiply-add instead of four scalar ones.
template <int S, int NA>
__device__ __forceinline__ void apply_slot_f2(Cx<float> (&a)[NA], const Cx<float> *__restrict__ Us)
{
    constexpr int lo = 2 * S;
    float2 ur[16], ui[16];
#pragma unroll
    for (int e = 0; e < 16; ++e)
    {
        const Cx<float> u = Us[e];
        ur[e] = make_float2(u.re, u.re);
        ui[e] = make_float2(-u.im, u.im);
    }
#pragma unroll
    for (int g = 0; g < NA / 4; ++g)
    {
        const int base = ((g >> lo) << (lo + 2)) | (g & ((1 << lo) - 1));
        float2 in[4], sw[4];
#pragma unroll
        for (int c = 0; c < 4; ++c)
        {
            const Cx<float> v = a[base | (c << lo)];
            in[c] = make_float2(v.re, v.im);
            sw[c] = make_float2(v.im, v.re);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
        {
            float2 acc = __fmul2_rn(ur[4 * r], in[0]);
            acc = __ffma2_rn(ui[4 * r], sw[0], acc);
#pragma unroll
            for (int c = 1; c < 4; ++c)
            {
                acc = __ffma2_rn(ur[4 * r + c], in[c], acc);
                acc = __ffma2_rn(ui[4 * r + c], sw[c], acc);
            }
            a[base | (r << lo)] = Cx<float>{acc.x, acc.y};
        }
    }
}

template <int S, typename Real, int NA>
__device__ __forceinline__ void apply_slot_fast(Cx<Real> (&a)[NA], const Cx<Real> *__restrict__ Us, bool packed)
{
    if constexpr (sizeof(Real) == 4)
    {
        if (packed)
        {
            apply_slot_f2<S>(a, Us);
            return;
        }
    }
    apply_slot<S>(a, Us);
}

// Parity-selected 2x2 gate on register bit 2S of a parity-sector state: the
// pair (r, r | bit 2S) gets Us[0..3] when the parity of the element's other
// index bits is even and Us[4..7] when it is odd. Those bits are the
// thread's (tpar: the parity of the tile base and the thread index, which
// map one to one onto index bits) plus register bits other than 2S (a
// compile-time parity per r).
template <int S, typename Real, int NA>
__device__ __forceinline__ void apply_parity_slot(Cx<Real> (&a)[NA], const Cx<Real> *__restrict__ Us, int tpar)
{
    Cx<Real> A[4], B[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        const Cx<Real> e = Us[i], o = Us[4 + i];
        A[i] = tpar ? o : e; // register parity even
        B[i] = tpar ? e : o; // register parity odd
    }
#pragma unroll
    for (int r = 0; r < NA; ++r)
    {
        if ((r >> (2 * S)) & 1) continue;
        const int r1 = r | (1 << (2 * S));
        int pr = 0;
#pragma unroll
        for (int b = 0; b < 8; ++b) pr ^= (r >> b) & 1;
        const Cx<Real> x0 = a[r], x1 = a[r1];
        if (pr)
        {
            a[r] = cfma(B[1], x1, cmul(B[0], x0));
            a[r1] = cfma(B[3], x1, cmul(B[2], x0));
        }
        else
        {
            a[r] = cfma(A[1], x1, cmul(A[0], x0));
            a[r1] = cfma(A[3], x1, cmul(A[2], x0));
        }
    }
}

__device__ __forceinline__ std::uint32_t smem_u32(const void *p)
{
    return static_cast<std::uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool tile_bar_try(std::uint64_t *bar, std::uint32_t parity)
{
    std::uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Bounded wait for a tile load: gives up after 0.3 s (or 2^22 polls).
__device__ __forceinline__ bool tile_bar_wait(std::uint64_t *bar, std::uint32_t parity)
{
    if (tile_bar_try(bar, parity)) return true;
    const std::uint64_t t0 = device_ns();
    for (int i = 0; i < (1 << 22); ++i)
    {
        if (tile_bar_try(bar, parity)) return true;
        if ((i & 15) == 15 && device_ns() - t0 > 300000000ull) return false;
        if (i >= 32) __nanosleep(64);
    }
    return false;
}

// One thread: fetches the tile whose first amplitude has batch-global index
// gb (trajectory << n | tile base) into `tile` in plain tile order with one
// TMA tensor load. Dimension d of the map covers global index bits [lo[d],
// lo[d] + bits[d]) (the last one also the trajectory index above bit n); its
// coordinate is those bits of gb, 0 on local runs.
__device__ __forceinline__ void tile_tma_load(void *tile, const CUtensorMap *map, const TileTma &t, const PassGeom &g,
                                              std::uint64_t gb, std::uint64_t *bar)
{
    int c[5] = {0, 0, 0, 0, 0};
    for (int d = 0; d < t.rank; ++d)
    {
        const std::uint64_t v = gb >> t.lo[d];
        c[d] = static_cast<int>(d + 1 == t.rank ? v : (v & ((1ull << t.bits[d]) - 1)));
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(static_cast<std::uint32_t>(sizeof(Cx<float>) << g.k))
                 : "memory");
    const std::uint32_t dst = smem_u32(tile), mb = smem_u32(bar);
    const unsigned long long m = reinterpret_cast<unsigned long long>(map);
    switch (t.rank)
    {
    case 1:
        asm volatile("cp.async.bulk.tensor.1d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];"
                     ::"r"(dst), "l"(m), "r"(c[0]), "r"(mb) : "memory");
        break;
    case 2:
        asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                     "[%4];" ::"r"(dst), "l"(m), "r"(c[0]), "r"(c[1]), "r"(mb) : "memory");
        break;
    case 3:
        asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                     "%4}], [%5];" ::"r"(dst), "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(mb) : "memory");
        break;
    case 4:
        asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                     "%4, %5}], [%6];" ::"r"(dst), "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(mb)
                     : "memory");
        break;
    default:
        asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                     "%4, %5, %6}], [%7];" ::"r"(dst), "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]),
                     "r"(mb)
                     : "memory");
        break;
    }
}

// Work items of a pass. Dense: item = trajectory * 2^n_nl + tile. Sparse
// (the first pass of a layer that follows a measurement): a tile whose
// non-local measured bits differ from the outcome is zero once the pending
// collapse is applied, and the pass's gates (all on local qubits) keep it
// zero, so only the 2^(n_nl - m_b) tiles of trajectory b that agree with its
// outcome on its m_b non-local measured bits are items. pref[b] is the first
// item of trajectory b (pref[batch] = the total); the r-th item of b has r's
// bits on the free non-local bits, the outcome on the fixed ones, ascending.
struct ItemSpace
{
    const std::uint32_t *pref;
    std::uint64_t nlq; // non-local qubits of the pass (mask)
};

__device__ __forceinline__ void decode_item(std::uint64_t item, bool sparse, const ItemSpace &sp, const PassGeom &g,
                                            const Collapse *col_in, std::size_t col_stride, int batch, int &b,
                                            std::uint64_t &tix)
{
    if (!sparse)
    {
        b = static_cast<int>(item >> g.n_nl);
        tix = item & ((1ull << g.n_nl) - 1);
        return;
    }
    int lo = 0, hi = batch - 1; // largest b with pref[b] <= item
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (sp.pref[mid] <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    b = lo;
    const Collapse c = col_in[static_cast<std::size_t>(b) * col_stride];
    std::uint64_t r = item - sp.pref[b];
    tix = 0;
    for (int i = 0; i < g.n_nl; ++i)
    {
        const int q = g.nl[i];
        std::uint64_t bit;
        if ((c.mask >> q) & 1ull)
            bit = (c.value >> q) & 1ull;
        else
        {
            bit = r & 1ull;
            r >>= 1;
        }
        tix |= bit << i;
    }
}

// Builds pref[0..batch] of the sparse item space (all threads of the CTA;
// red holds at least 32 words). Returns the item count.
__device__ std::uint32_t build_item_prefix(std::uint32_t *pref, std::uint32_t *red, const PassGeom &g,
                                           std::uint64_t nlq, const Collapse *col_in, std::size_t col_stride,
                                           int batch)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    const int per = (batch + nt - 1) / nt;
    const int b0 = tid * per, b1 = min(batch, b0 + per);
    auto count = [&](int b) {
        const std::uint64_t m = col_in[static_cast<std::size_t>(b) * col_stride].mask & nlq;
        return 1u << (g.n_nl - __popcll(m));
    };
    std::uint32_t sum = 0;
    for (int b = b0; b < b1; ++b) sum += count(b);
    // Exclusive scan of the per-thread sums over the CTA.
    const int lane = tid & 31, warp = tid >> 5;
    std::uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const std::uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) red[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        std::uint32_t w = lane < (nt >> 5) ? red[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const std::uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < (nt >> 5)) red[lane] = w; // inclusive warp totals
    }
    __syncthreads();
    std::uint32_t run = x - sum + (warp > 0 ? red[warp - 1] : 0u);
    for (int b = b0; b < b1; ++b)
    {
        pref[b] = run;
        run += count(b);
    }
    const std::uint32_t total = red[(nt >> 5) - 1];
    if (tid == 0) pref[batch] = total;
    __syncthreads();
    return total;
}

// One tiled pass with register rounds: global -> registers (lanes on the
// contiguous low qubits), gates applied in registers, swizzled shared-memory
// transposes between rounds, registers -> global, optional fused histogram.
// Work items are (trajectory, tile) pairs, item = trajectory * 2^n_nl + tile;
// the CTA at flat index c runs items c, c + C, ... with C the number of CTAs,
// so one launch shape serves both one item per CTA (C = items) and a
// persistent grid. With TMA (FP32, persistent grid) tiles arrive by one TMA
// tensor load each into the shared tile buffer in plain tile order: the load
// of the CTA's next item is issued as soon as the current item's last
// transpose has read the buffer, so it streams under the last gate round, the
// stores and the histogram, whose values then use their own 2^k floats after
// the tile buffer. A load wait that runs out sets bit 8 of *err and ends the
// CTA.
template <typename Real, int RB, bool TMA, bool PAR>
__global__ void __launch_bounds__(RB == 5 && sizeof(Real) == 4 ? 512 : 256)
    k_pass_rounds(Cx<Real> *__restrict__ states, PassPlan P, const Cx<Real> *__restrict__ gates,
                  std::size_t gate_stride, const Collapse *__restrict__ col_in, std::size_t col_stride,
                  const LayerMeas *__restrict__ meas, std::size_t meas_stride, double *__restrict__ partials,
                  int fuse_hist, int packed, int batch, const __grid_constant__ CUtensorMap tmap, TileTma tt,
                  int *err, std::uint64_t col_keep, int col_scaled, int sparse, int withhold_first_load)
{
    constexpr int NA = 1 << RB;
    extern __shared__ __align__(128) unsigned char smem_dyn[];
    // TMA tensor loads need a 128-byte aligned destination; the launch adds
    // 128 bytes of dynamic shared memory for the shift.
    unsigned char *smem_raw = smem_dyn;
    if constexpr (TMA) smem_raw += (128u - (smem_u32(smem_dyn) & 127u)) & 127u;
    Cx<Real> *tile = reinterpret_cast<Cx<Real> *>(smem_raw);
    __shared__ Cx<Real> U[kMaxPassGates][16];
    __shared__ double red[8];

    const PassGeom &g = P.geom;
    const int TB = g.k - RB;
    const int tid = threadIdx.x;
    const bool sp_on = sparse != 0;
    ItemSpace sp{nullptr, 0};
    std::uint64_t items = static_cast<std::uint64_t>(batch) << g.n_nl;
    if (sp_on)
    {
        // The item prefix table follows the tile (and, with TMA, the
        // histogram values) in dynamic shared memory.
        __shared__ std::uint32_t sred[32];
        std::uint32_t *pref = reinterpret_cast<std::uint32_t *>(
            smem_raw + (sizeof(Cx<Real>) << g.k) + (TMA ? (sizeof(float) << g.k) : 0));
        for (int i = 0; i < g.n_nl; ++i) sp.nlq |= 1ull << g.nl[i];
        items = build_item_prefix(pref, sred, g, sp.nlq, col_in, col_stride, batch);
        sp.pref = pref;
    }
    const std::uint64_t step = static_cast<std::uint64_t>(gridDim.x) * gridDim.y;
    const std::uint64_t first = static_cast<std::uint64_t>(blockIdx.y) * gridDim.x + blockIdx.x;
    __shared__ __align__(8) std::uint64_t tile_bar;
    __shared__ int tile_fail;
    std::uint32_t tile_phase = 0;
    // Batch-global index of the first amplitude of an item's tile.
    auto item_base = [&](std::uint64_t it) {
        int bb;
        std::uint64_t tt_;
        decode_item(it, sp_on, sp, g, col_in, col_stride, batch, bb, tt_);
        return (static_cast<std::uint64_t>(bb) << g.n) | scatter_bits(tt_, g.nl, g.n_nl);
    };
    if constexpr (TMA)
    {
        if (tid == 0)
        {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&tile_bar)) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            tile_fail = 0;
        }
        __syncthreads();
        // withhold_first_load (a test hook): CTA 0 does not issue its first
        // tile load, so its bounded wait runs out and the pass reports it.
        const bool withhold = withhold_first_load != 0 && first == 0;
        if (tid == 0 && first < items && !withhold) tile_tma_load(tile, &tmap, tt, g, item_base(first), &tile_bar);
    }
    int cur_b = -1;
    for (std::uint64_t item = first; item < items; item += step)
    {
        int b;
        std::uint64_t tix;
        decode_item(item, sp_on, sp, g, col_in, col_stride, batch, b, tix);
        __syncthreads(); // the previous item's shared-memory reads are complete
        Cx<Real> *psi = states + (static_cast<std::size_t>(b) << g.n);
        const std::uint64_t base = scatter_bits(tix, g.nl, g.n_nl);
        const int tpar = PAR ? ((__popcll(base) + __popc(static_cast<unsigned>(tid))) & 1) : 0;
        if (b != cur_b)
            for (int i = tid; i < P.gates.count * 16; i += blockDim.x)
                U[i / 16][i % 16] = gates[b * gate_stride + static_cast<std::size_t>(P.gates.gate[i / 16]) * 16 + (i % 16)];
        cur_b = b;
        Collapse cl{0, 0, 1.0, 0};
        const bool has_col = col_in != nullptr;
        if (has_col)
        {
            // col_keep < all ones: the residual of a collapse that an earlier
            // pass of the layer applied to every tile it visited; only the
            // bits of the tiles it skipped are left. A parity condition is not
            // (that pass's gates may have changed the stored bits' parity).
            cl = col_in[b * col_stride];
            cl.mask &= col_keep;
            cl.value &= col_keep;
            if (!col_scaled)
            {
                cl.scale = 1.0;
                cl.parity = 0;
            }
        }
        const Real scale = static_cast<Real>(cl.scale);

        const std::uint64_t next = item + step;
        Cx<Real> amp[NA];
        if constexpr (TMA)
        {
            // This item's tile is in the tile buffer in plain tile order.
            if (!tile_bar_wait(&tile_bar, tile_phase)) tile_fail = 1;
            tile_phase ^= 1u;
            const Round &R = P.round[0];
            std::uint64_t gt = base;
            std::uint32_t jt = 0;
            for (int i = 0; i < TB; ++i)
                if ((tid >> i) & 1)
                {
                    gt |= 1ull << g.pos[R.tid[i]];
                    jt |= 1u << R.tid[i];
                }
            std::uint64_t gr[RB];
            std::uint32_t jr[RB];
#pragma unroll
            for (int i = 0; i < RB; ++i)
            {
                gr[i] = 1ull << g.pos[R.reg[i]];
                jr[i] = 1u << R.reg[i];
            }
#pragma unroll
            for (int r = 0; r < NA; ++r)
            {
                std::uint32_t j = jt;
#pragma unroll
                for (int i = 0; i < RB; ++i)
                    if ((r >> i) & 1) j |= jr[i];
                amp[r] = tile[j];
            }
            if (has_col) apply_keep_bits(amp, collapse_keep_bits<RB, PAR>(gt, gr, cl), scale);
        }
        else
        {
            const Round &R = P.round[0];
            std::uint64_t gt = base;
            for (int i = 0; i < TB; ++i)
                if ((tid >> i) & 1) gt |= 1ull << g.pos[R.tid[i]];
            std::uint64_t gr[RB];
#pragma unroll
            for (int i = 0; i < RB; ++i) gr[i] = 1ull << g.pos[R.reg[i]];
#pragma unroll
            for (int r = 0; r < NA; ++r)
            {
                std::uint64_t gi = gt;
#pragma unroll
                for (int i = 0; i < RB; ++i)
                    if ((r >> i) & 1) gi |= gr[i];
                amp[r] = psi[gi];
            }
            if (has_col) apply_keep_bits(amp, collapse_keep_bits<RB, PAR>(gt, gr, cl), scale);
        }
        __syncthreads(); // gate matrices visible; round-0 reads of the tile buffer are done
        if constexpr (TMA)
        {
            if (tile_fail)
            {
                if (tid == 0)
                {
                    atomicOr(err, 8);
                    tile_bar_wait(&tile_bar, tile_phase ^ 1u); // let the load land before leaving
                }
                return;
            }
            if (P.rounds == 1 && next < items && tid == 0) tile_tma_load(tile, &tmap, tt, g, item_base(next), &tile_bar);
        }

        for (int ri = 0; ri < P.rounds; ++ri)
        {
            const Round &R = P.round[ri];
            if (ri > 0)
            {
                const Round &A = P.round[ri - 1];
                std::uint32_t sa = 0, sb = 0;
                for (int i = 0; i < TB; ++i)
                    if ((tid >> i) & 1)
                    {
                        sa ^= swz1(A.tid[i]);
                        sb ^= swz1(R.tid[i]);
                    }
                std::uint32_t ra[RB], rb_[RB];
#pragma unroll
                for (int i = 0; i < RB; ++i)
                {
                    ra[i] = swz1(A.reg[i]);
                    rb_[i] = swz1(R.reg[i]);
                }
                if (ri > 1) __syncthreads(); // previous round's reads are complete
#pragma unroll
                for (int r = 0; r < NA; ++r)
                {
                    std::uint32_t p = sa;
#pragma unroll
                    for (int i = 0; i < RB; ++i)
                        if ((r >> i) & 1) p ^= ra[i];
                    tile[p] = amp[r];
                }
                __syncthreads();
#pragma unroll
                for (int r = 0; r < NA; ++r)
                {
                    std::uint32_t p = sb;
#pragma unroll
                    for (int i = 0; i < RB; ++i)
                        if ((r >> i) & 1) p ^= rb_[i];
                    amp[r] = tile[p];
                }
                if constexpr (TMA)
                {
                    if (ri == P.rounds - 1 && next < items)
                    {
                        __syncthreads(); // the last reads of the tile buffer for this item are done
                        if (tid == 0) tile_tma_load(tile, &tmap, tt, g, item_base(next), &tile_bar);
                    }
                }
            }
            if constexpr (PAR)
            {
                if (R.slot[0] >= 0)
                {
                    if (P.gates.kind[R.slot[0]])
                        apply_parity_slot<0>(amp, U[R.slot[0]], tpar);
                    else
                        apply_slot_fast<0>(amp, U[R.slot[0]], packed != 0);
                }
                if (RB >= 4 && R.slot[1] >= 0)
                {
                    if (P.gates.kind[R.slot[1]])
                        apply_parity_slot<(RB >= 4 ? 1 : 0)>(amp, U[R.slot[1]], tpar);
                    else
                        apply_slot_fast<(RB >= 4 ? 1 : 0)>(amp, U[R.slot[1]], packed != 0);
                }
                if (RB >= 6 && R.slot[2] >= 0)
                {
                    if (P.gates.kind[R.slot[2]])
                        apply_parity_slot<(RB >= 6 ? 2 : 0)>(amp, U[R.slot[2]], tpar);
                    else
                        apply_slot_fast<(RB >= 6 ? 2 : 0)>(amp, U[R.slot[2]], packed != 0);
                }
            }
            else
            {
                if (R.slot[0] >= 0) apply_slot_fast<0>(amp, U[R.slot[0]], packed != 0);
                if (RB >= 4 && R.slot[1] >= 0) apply_slot_fast<(RB >= 4 ? 1 : 0)>(amp, U[R.slot[1]], packed != 0);
                if (RB >= 6 && R.slot[2] >= 0) apply_slot_fast<(RB >= 6 ? 2 : 0)>(amp, U[R.slot[2]], packed != 0);
            }
        }

        const Round &Z = P.round[P.rounds - 1];
        {
            std::uint64_t gt = base;
            for (int i = 0; i < TB; ++i)
                if ((tid >> i) & 1) gt |= 1ull << g.pos[Z.tid[i]];
            std::uint64_t gr[RB];
#pragma unroll
            for (int i = 0; i < RB; ++i) gr[i] = 1ull << g.pos[Z.reg[i]];
#pragma unroll
            for (int r = 0; r < NA; ++r)
            {
                std::uint64_t gi = gt;
#pragma unroll
                for (int i = 0; i < RB; ++i)
                    if ((r >> i) & 1) gi |= gr[i];
                psi[gi] = amp[r];
            }
        }

        if (fuse_hist)
        {
            const LayerMeas &M = meas[b * meas_stride];
            if constexpr (sizeof(Real) == 4)
            {
                if (M.nchunks > 0)
                {
                    const std::uint64_t chunk = M.chunk[0];
                    std::uint32_t mmask = 0;
                    for (int i = 0; i < g.k; ++i)
                        if ((chunk >> g.pos[i]) & 1ull) mmask |= 1u << i;
                    const int m_loc = __popc(mmask);
                    double *part = partials + static_cast<std::size_t>(b) * kHistScratch + (tix << m_loc);
                    float *S = reinterpret_cast<float *>(smem_raw + (TMA ? (sizeof(Cx<float>) << g.k) : 0));
                    __shared__ int tab[32];
                    register_histogram<RB>(amp, Z, TB, mmask, m_loc, S, tab, part);
                }
            }
            else if (M.nchunks > 0)
            {
                __syncthreads(); // the tile buffer is free
                Real *val = reinterpret_cast<Real *>(smem_raw);
                std::uint32_t jt = 0;
                for (int i = 0; i < TB; ++i)
                    if ((tid >> i) & 1) jt |= 1u << Z.tid[i];
#pragma unroll
                for (int r = 0; r < NA; ++r)
                {
                    std::uint32_t j = jt;
#pragma unroll
                    for (int i = 0; i < RB; ++i)
                        if ((r >> i) & 1) j |= 1u << Z.reg[i];
                    val[j] = norm2(amp[r]);
                }
                __syncthreads();
                const std::uint64_t chunk = M.chunk[0];
                int lm[kMaxLocal + 1];
                int m_loc = 0;
                for (int i = 0; i < g.k; ++i)
                    if ((chunk >> g.pos[i]) & 1ull) lm[m_loc++] = i;
                double *part = partials + static_cast<std::size_t>(b) * kHistScratch + (tix << m_loc);
                value_histogram(val, g.k, lm, m_loc, part, red);
            }
        }
    }
}


// One tiled pass of a 2^14-amplitude tile split across the two CTAs of a
// thread-block cluster (tile bit x = CTA rank): 256 threads x 32 amplitudes
// per CTA, 64 KB of shared memory and at most 128 registers per thread, so two
// CTAs fit on an SM and the load, gate and store phases of different CTAs
// overlap. Transposes go through distributed shared memory.
template <int RB>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(1 << (13 - RB), 2)
    k_pass_cluster(Cx<float> *__restrict__ states, PassPlan P, const Cx<float> *__restrict__ gates,
                   std::size_t gate_stride, const Collapse *__restrict__ col_in, std::size_t col_stride,
                   const LayerMeas *__restrict__ meas, std::size_t meas_stride, double *__restrict__ partials,
                   int fuse_hist)
{
    constexpr int NA = 1 << RB, TB = 13 - RB;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx<float> *tile = reinterpret_cast<Cx<float> *>(smem_raw);
    __shared__ Cx<float> U[kMaxPassGates][16];
    __shared__ double red[8];
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned rank = cluster.block_rank();
    Cx<float> *peer = cluster.map_shared_rank(tile, static_cast<int>(rank ^ 1u));

    const PassGeom &g = P.geom;
    const int tid = threadIdx.x;
    const int b = blockIdx.y;
    const std::uint64_t tix = blockIdx.x >> 1;
    Cx<float> *psi = states + (static_cast<std::size_t>(b) << g.n);
    const std::uint64_t base = scatter_bits(tix, g.nl, g.n_nl);
    for (int i = tid; i < P.gates.count * 16; i += blockDim.x)
        U[i / 16][i % 16] = gates[b * gate_stride + static_cast<std::size_t>(P.gates.gate[i / 16]) * 16 + (i % 16)];
    Collapse cl{0, 0, 1.0, 0};
    const bool has_col = col_in != nullptr;
    if (has_col) cl = col_in[b * col_stride];
    const float scale = static_cast<float>(cl.scale);

    // n <= 32: every amplitude index fits in 32 bits.
    const std::uint32_t cmask = static_cast<std::uint32_t>(cl.mask), cval = static_cast<std::uint32_t>(cl.value);
    Cx<float> amp[NA];
    {
        const ClusterRound &R = P.cround[0];
        std::uint32_t gt = static_cast<std::uint32_t>(base) | (rank << g.pos[R.x]);
        for (int i = 0; i < TB; ++i)
            if ((tid >> i) & 1) gt |= 1u << g.pos[R.tid[i]];
        std::uint32_t gr[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) gr[i] = 1u << g.pos[R.reg[i]];
#pragma unroll
        for (int r = 0; r < NA; ++r)
        {
            std::uint32_t gi = gt;
#pragma unroll
            for (int i = 0; i < RB; ++i)
                if ((r >> i) & 1) gi |= gr[i];
            Cx<float> v = psi[gi];
            if (has_col)
            {
                const float f = ((gi & cmask) == cval) ? scale : 0.f;
                v.re *= f;
                v.im *= f;
            }
            amp[r] = v;
        }
    }
    __syncthreads();

    for (int ri = 0; ri < P.cluster_rounds; ++ri)
    {
        const ClusterRound &R = P.cround[ri];
        if (ri > 0)
        {
            const ClusterRound &A = P.cround[ri - 1];
            const int xa = A.x;
            // write: my elements have bit xa == rank, so they are all home here
            std::uint32_t sa = 0;
            for (int i = 0; i < TB; ++i)
                if ((tid >> i) & 1) sa ^= swz1(opos_d(A.tid[i], xa));
            std::uint32_t ra[RB];
#pragma unroll
            for (int i = 0; i < RB; ++i) ra[i] = swz1(opos_d(A.reg[i], xa));
            if (ri > 1) cluster.sync(); // the peer has finished reading my buffer
#pragma unroll
            for (int r = 0; r < NA; ++r)
            {
                std::uint32_t p = sa;
#pragma unroll
                for (int i = 0; i < RB; ++i)
                    if ((r >> i) & 1) p ^= ra[i];
                tile[p] = amp[r];
            }
            cluster.sync();
            // read in the storage coordinates of round A; home CTA = bit xa
            std::uint32_t sb = 0;
            unsigned hb = 0;
            for (int i = 0; i < TB; ++i)
                if ((tid >> i) & 1)
                {
                    if (R.tid[i] == xa)
                        hb ^= 1u;
                    else
                        sb ^= swz1(opos_d(R.tid[i], xa));
                }
            if (rank)
            {
                if (R.x == xa)
                    hb ^= 1u;
                else
                    sb ^= swz1(opos_d(R.x, xa));
            }
            std::uint32_t rbv[RB];
            unsigned rh[RB];
#pragma unroll
            for (int i = 0; i < RB; ++i)
            {
                rh[i] = R.reg[i] == xa ? 1u : 0u;
                rbv[i] = R.reg[i] == xa ? 0u : swz1(opos_d(R.reg[i], xa));
            }
#pragma unroll
            for (int r = 0; r < NA; ++r)
            {
                std::uint32_t p = sb;
                unsigned h = hb;
#pragma unroll
                for (int i = 0; i < RB; ++i)
                    if ((r >> i) & 1)
                    {
                        p ^= rbv[i];
                        h ^= rh[i];
                    }
                amp[r] = (h == rank) ? tile[p] : peer[p];
            }
        }
        if (R.slot[0] >= 0) apply_slot<0>(amp, U[R.slot[0]]);
        if (R.slot[1] >= 0) apply_slot<1>(amp, U[R.slot[1]]);
        if (RB >= 6 && R.slot[2] >= 0) apply_slot<(RB >= 6 ? 2 : 0)>(amp, U[R.slot[2]]);
    }

    const ClusterRound &Z = P.cround[P.cluster_rounds - 1];
    {
        std::uint32_t gt = static_cast<std::uint32_t>(base) | (rank << g.pos[Z.x]);
        for (int i = 0; i < TB; ++i)
            if ((tid >> i) & 1) gt |= 1u << g.pos[Z.tid[i]];
        std::uint32_t gr[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) gr[i] = 1u << g.pos[Z.reg[i]];
#pragma unroll
        for (int r = 0; r < NA; ++r)
        {
            std::uint32_t gi = gt;
#pragma unroll
            for (int i = 0; i < RB; ++i)
                if ((r >> i) & 1) gi |= gr[i];
            psi[gi] = amp[r];
        }
    }

    // The peer may still read my buffer for the last transpose.
    if (P.cluster_rounds > 1) cluster.sync();
    if (fuse_hist)
    {
        const LayerMeas &M = meas[b * meas_stride];
        if (M.nchunks > 0)
        {
            float *val = reinterpret_cast<float *>(smem_raw);
            const int xz = Z.x;
            std::uint32_t jt = 0;
            for (int i = 0; i < TB; ++i)
                if ((tid >> i) & 1) jt |= 1u << opos_d(Z.tid[i], xz);
#pragma unroll
            for (int r = 0; r < NA; ++r)
            {
                std::uint32_t j = jt;
#pragma unroll
                for (int i = 0; i < RB; ++i)
                    if ((r >> i) & 1) j |= 1u << opos_d(Z.reg[i], xz);
                val[j] = norm2(amp[r]);
            }
            __syncthreads();
            const std::uint64_t chunk = M.chunk[0];
            const PassGeom &h = P.hgeom;
            int lm[kMaxLocal + 1];
            int m_loc = 0;
            for (int i = 0; i < h.k; ++i)
                if ((chunk >> h.pos[i]) & 1ull) lm[m_loc++] = i;
            const std::uint64_t t2 = (tix << 1) | rank;
            double *part = partials + static_cast<std::size_t>(b) * kHistScratch + (t2 << m_loc);
            value_histogram(val, h.k, lm, m_loc, part, red);
        }
    }
}

template <typename Real>
__global__ void __launch_bounds__(kPassThreads) k_hist(const Cx<Real> *__restrict__ states, int n, int kmax, int cmin,
                                                       int ci, const Collapse *__restrict__ col_in,
                                                       std::size_t col_stride, const LayerMeas *__restrict__ meas,
                                                       std::size_t meas_stride, double *__restrict__ partials,
                                                       int direct, const signed char *__restrict__ sector)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ PassGeom g;
    __shared__ double red[kPassThreads / 32];
    const int b = blockIdx.y;
    const LayerMeas &M = meas[b * meas_stride];
    if (ci >= M.nchunks) return;
    const std::uint64_t chunk = M.chunk[ci];
    // A chunk at bit n of a parity-sector state (n qubits stored, the top
    // qubit of the chain being the parity of the others and of the
    // trajectory's sector) is that top qubit alone: its two bins sum the
    // amplitudes by parity, over tiles of the geometry of an empty chunk.
    const bool par_chunk = (chunk >> n) != 0ull;
    if (threadIdx.x == 0) histogram_geometry(n, kmax, cmin, par_chunk ? 0ull : chunk, g);
    __syncthreads();
    Cx<Real> *tile = reinterpret_cast<Cx<Real> *>(smem_raw);
    std::uint32_t *seg = reinterpret_cast<std::uint32_t *>(direct ? smem_raw : smem_raw + (sizeof(Cx<Real>) << g.k));
    const std::uint64_t tix = blockIdx.x;
    const std::uint64_t dim = 1ull << n;
    const Cx<Real> *psi = states + static_cast<std::size_t>(b) * dim;
    const std::uint64_t base = scatter_bits(tix, g.nl, g.n_nl);
    const int h = g.k - g.c;
    for (std::uint32_t s = threadIdx.x; s < (1u << h); s += blockDim.x)
        seg[s] = static_cast<std::uint32_t>(scatter_bits(s, g.pos + g.c, h));
    Collapse cl{0, 0, 1.0, 0};
    const bool has_col = col_in != nullptr;
    if (has_col) cl = col_in[b * col_stride];
    __syncthreads();
    if (par_chunk)
    {
        // Tile bins (top qubit 0, 1) in the order of the direct sum below.
        const int P = sector ? sector[b] : 0;
        const std::uint64_t nloc = 1ull << g.k, cmask = (1ull << g.c) - 1ull;
        const Real scale = static_cast<Real>(cl.scale);
        Acc<Real> acc[2];
        for (std::uint64_t r = threadIdx.x; r < nloc; r += blockDim.x)
        {
            const std::uint64_t gidx = base | seg[r >> g.c] | (r & cmask);
            Cx<Real> v = psi[gidx];
            if (has_col) v = collapse_value(v, gidx, cl, scale);
            const int bit = (P + __popcll(gidx)) & 1;
            acc[bit].add(norm2(v));
        }
        double *pp = partials + static_cast<std::size_t>(b) * kHistScratch + (tix << 1);
        for (int bin = 0; bin < 2; ++bin)
        {
            double v = acc[bin].value();
            for (int off = 16; off > 0; off /= 2) v += __shfl_down_sync(0xffffffffu, v, off, 32);
            __syncthreads();
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
            __syncthreads();
            if (threadIdx.x == 0)
            {
                double t = 0.0;
                for (int w = 0; w < static_cast<int>(blockDim.x) / 32; ++w) t += red[w];
                pp[bin] = t;
            }
        }
        return;
    }
    int lm[kMaxLocal + 1];
    int m_loc = 0;
    for (int i = 0; i < g.k; ++i)
        if ((chunk >> g.pos[i]) & 1ull) lm[m_loc++] = i;
    double *part = partials + static_cast<std::size_t>(b) * kHistScratch + (tix << m_loc);
    if (direct)
    {
        // Every measured site is outside the tile (the host checked), so the
        // tile contributes one total: stream it from global memory in the
        // order tile_histogram sums a one-bin tile (thread t takes local
        // indices t, t + T, ...; then the same shuffle and warp tree), without
        // staging it in shared memory.
        const std::uint64_t nloc = 1ull << g.k, cmask = (1ull << g.c) - 1ull;
        const Real scale = static_cast<Real>(cl.scale);
        Acc<Real> acc;
        // Four loads in flight per thread, added in the same order as one at
        // a time; tiles that are not a multiple of four block-widths take the
        // plain loop.
        const std::uint64_t T4 = 4ull * blockDim.x;
        if (nloc % T4 != 0)
            for (std::uint64_t r = threadIdx.x; r < nloc; r += blockDim.x)
            {
                const std::uint64_t gidx = base | seg[r >> g.c] | (r & cmask);
                Cx<Real> v = psi[gidx];
                if (has_col) v = collapse_value(v, gidx, cl, scale);
                acc.add(norm2(v));
            }
        else
        for (std::uint64_t r0 = threadIdx.x; r0 < nloc; r0 += T4)
        {
            Cx<Real> v[4];
            std::uint64_t gi[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
            {
                const std::uint64_t r = r0 + static_cast<std::uint64_t>(u) * blockDim.x;
                gi[u] = base | seg[r >> g.c] | (r & cmask);
                v[u] = psi[gi[u]];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
            {
                if (has_col) v[u] = collapse_value(v[u], gi[u], cl, scale);
                acc.add(norm2(v[u]));
            }
        }
        double v = acc.value();
        for (int off = 16; off > 0; off /= 2) v += __shfl_down_sync(0xffffffffu, v, off, 32);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0)
        {
            double t = 0.0;
            for (int w = 0; w < static_cast<int>(blockDim.x) / 32; ++w) t += red[w];
            part[0] = t;
        }
        return;
    }
    load_tile(tile, psi, g, base, seg, cl, has_col);
    __syncthreads();
    tile_histogram(tile, g.k, lm, m_loc, part, red);
}

// One block per trajectory: gather the chunk's joint histogram from the tile
// partials in a fixed order, sample the outcome exactly as the reference's
// host CDF scan does, and record the collapse.
__global__ void __launch_bounds__(kMeasureThreads)
    k_measure(int n, PassGeom fg, int fused, int kmax, int cmin, int ci, const LayerMeas *__restrict__ meas,
              std::size_t meas_stride, const double *__restrict__ partials, double *__restrict__ bins_scratch,
              std::size_t bins_stride, const std::uint64_t *__restrict__ forced, std::size_t forced_stride, Collapse *__restrict__ col,
              std::size_t col_stride, LayerResult *__restrict__ res, std::size_t res_stride, int *__restrict__ err,
              const signed char *__restrict__ sector)
{
    __shared__ PassGeom g;
    __shared__ double sbins[kSmemBins];
    __shared__ double seg_sum[kMeasureThreads];
    __shared__ int lm_bit[kMaxLocal + 1], hm_pos[kMaxQubits], hm_bit[kMaxQubits];
    __shared__ int s_mloc, s_mhi;
    __shared__ std::uint64_t s_chosen;
    __shared__ double s_branch, s_total;

    const int b = blockIdx.x;
    const LayerMeas &M = meas[b * meas_stride];
    if (ci >= M.nchunks) return;
    const std::uint64_t chunk = M.chunk[ci];
    const int m = __popcll(chunk);
    const int tid = threadIdx.x;
    const int T = blockDim.x;
    // Parity-sector state: a chunk at bit n is the chain's top qubit, whose
    // two bins k_hist wrote per tile as if it were the tile's lowest local bit.
    const bool par_chunk = (chunk >> n) != 0ull;
    if (tid == 0)
    {
        if (par_chunk)
        {
            histogram_geometry(n, kmax, cmin, 0ull, g);
            lm_bit[0] = 0;
            s_mloc = 1;
            s_mhi = 0;
        }
        else
        {
            if (fused)
                g = fg;
            else
                histogram_geometry(n, kmax, cmin, chunk, g);
            int ml = 0, mh = 0;
            for (int i = 0; i < g.k; ++i)
                if ((chunk >> g.pos[i]) & 1ull) lm_bit[ml++] = __popcll(chunk & ((1ull << g.pos[i]) - 1ull));
            for (int i = 0; i < g.n_nl; ++i)
                if ((chunk >> g.nl[i]) & 1ull)
                {
                    hm_pos[mh] = i;
                    hm_bit[mh++] = __popcll(chunk & ((1ull << g.nl[i]) - 1ull));
                }
            s_mloc = ml;
            s_mhi = mh;
        }
    }
    __syncthreads();
    const int m_loc = s_mloc, m_hi = s_mhi;
    const std::uint64_t NB = 1ull << m;
    const std::uint64_t per_bin_tiles = 1ull << (g.n_nl - m_hi);
    const double *part = partials + static_cast<std::size_t>(b) * kHistScratch;
    double *bins = NB <= kSmemBins ? sbins : bins_scratch + static_cast<std::size_t>(b) * bins_stride;

    // With fewer bins than threads, G consecutive lanes (a power of two, at
    // most a warp) share one bin: lane g sums its tiles g, g + G, ... and a
    // fixed shuffle tree joins the G partial sums, so the order is the same
    // on every run.
    const int G = NB >= static_cast<std::uint64_t>(T) ? 1 : static_cast<int>(std::min<std::uint64_t>(32, T / NB));
    const int groups = T / G;
    // The bin's tiles: tile index t = tile-index bits of r deposited into the
    // unmeasured positions (`free`); stepping r by G adds G's deposit there,
    // carried across the measured positions by setting them first.
    std::uint64_t free_bits = (g.n_nl >= 64 ? ~0ull : ((1ull << g.n_nl) - 1ull));
    for (int i = 0; i < m_hi; ++i) free_bits &= ~(1ull << hm_pos[i]);
    auto deposit = [&](std::uint64_t x) {
        std::uint64_t out = 0, f = free_bits;
        for (int i = 0; f != 0ull; ++i)
        {
            const std::uint64_t low = f & (~f + 1ull);
            if ((x >> i) & 1ull) out |= low;
            f &= f - 1ull;
        }
        return out;
    };
    const std::uint64_t t_step = deposit(static_cast<std::uint64_t>(G));
    for (std::uint64_t B = tid / G; B < NB; B += groups)
    {
        const int gl = tid % G;
        std::uint64_t bl = 0, th = 0;
        for (int i = 0; i < m_loc; ++i) bl |= ((B >> lm_bit[i]) & 1ull) << i;
        for (int i = 0; i < m_hi; ++i) th |= ((B >> hm_bit[i]) & 1ull) << hm_pos[i];
        double s = 0.0;
        std::uint64_t t = deposit(static_cast<std::uint64_t>(gl));
        for (std::uint64_t r = gl; r < per_bin_tiles; r += G)
        {
            s += part[((t | th) << m_loc) + bl];
            t = ((t | ~free_bits) + t_step) & free_bits;
        }
        for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
        if (gl == 0) bins[B] = s;
    }
    __syncthreads();

    // Contiguous segments of bins, one per participating thread.
    const std::uint64_t P = NB < static_cast<std::uint64_t>(T) ? NB : static_cast<std::uint64_t>(T);
    const std::uint64_t S = (NB + P - 1) / P;
    if (static_cast<std::uint64_t>(tid) < P)
    {
        double s = 0.0;
        const std::uint64_t lo = tid * S, hi = (tid + 1) * S < NB ? (tid + 1) * S : NB;
        for (std::uint64_t i = lo; i < hi; ++i) s += bins[i];
        seg_sum[tid] = s;
    }
    __syncthreads();
    // Total and CDF search by warp 0: lane l sums segments [l Q, (l+1) Q) in
    // order, a shuffle scan gives each lane's cumulative range, and the first
    // lane whose range passes the draw walks its segments, then the bins of
    // the segment it lands in.
    if (tid < 32)
    {
        const int lane = tid;
        const std::uint64_t Q = (P + 31) / 32;
        const std::uint64_t s0 = lane * Q < P ? lane * Q : P, s1 = (lane + 1) * Q < P ? (lane + 1) * Q : P;
        double partial = 0.0;
        for (std::uint64_t i = s0; i < s1; ++i) partial += seg_sum[i];
        double incl = partial;
        for (int o = 1; o < 32; o <<= 1)
        {
            const double y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        double excl = __shfl_up_sync(0xffffffffu, incl, 1);
        if (lane == 0) excl = 0.0;
        const double total = __shfl_sync(0xffffffffu, incl, 31);
        std::uint64_t chosen = NB - 1;
        const bool bad = !(total > 0.0) || !isfinite(total);
        if (forced != nullptr)
        {
            const std::uint64_t f = forced[b * forced_stride];
            chosen = 0;
            int j = 0;
            for (int q = 0; q < n; ++q)
                if ((chunk >> q) & 1ull) chosen |= ((f >> q) & 1ull) << j++;
            if (par_chunk) chosen = (f >> n) & 1ull;
        }
        else if (!bad)
        {
            const double draw = M.uniform[ci] * total;
            const unsigned past = __ballot_sync(0xffffffffu, s0 < s1 && draw < incl);
            if (past != 0u)
            {
                const int leader = __ffs(past) - 1;
                std::uint64_t pick = NB - 1;
                if (lane == leader)
                {
                    double run = excl;
                    std::uint64_t segi = s1 - 1;
                    for (std::uint64_t i = s0; i < s1; ++i)
                    {
                        if (draw < run + seg_sum[i])
                        {
                            segi = i;
                            break;
                        }
                        run += seg_sum[i];
                    }
                    const std::uint64_t lo = segi * S, hi = (segi + 1) * S < NB ? (segi + 1) * S : NB;
                    pick = hi - 1;
                    for (std::uint64_t i = lo; i < hi; ++i)
                    {
                        run += bins[i];
                        if (draw < run)
                        {
                            pick = i;
                            break;
                        }
                    }
                }
                chosen = __shfl_sync(0xffffffffu, pick, leader);
            }
        }
        if (lane == 0)
        {
            double branch = bins[chosen];
            bool fail = bad;
            if (!bad && !(branch > 0.0) && forced == nullptr)
            {
                // Numerically starved bin: take the heaviest (first on ties).
                std::uint64_t best = 0;
                for (std::uint64_t i = 1; i < NB; ++i)
                    if (bins[i] > bins[best]) best = i;
                chosen = best;
                branch = bins[best];
            }
            if (!(branch > 0.0)) fail = true;
            s_chosen = chosen;
            s_branch = branch;
            s_total = total;
            if (fail) atomicOr(err, 1);
        }
    }
    __syncthreads();
    if (tid == 0)
    {
        const std::uint64_t chosen = s_chosen;
        const double branch = s_branch, total = s_total;
        std::uint64_t val = 0;
        int j = 0;
        for (int q = 0; q < n; ++q)
            if ((chunk >> q) & 1ull) val |= ((chosen >> j++) & 1ull) << q;
        if (par_chunk) val = (chosen & 1ull) << n;
        const bool ok = branch > 0.0 && total > 0.0 && isfinite(total);
        const double scale = ok ? 1.0 / sqrt(branch) : 1.0;
        Collapse &c = col[b * col_stride];
        if (par_chunk)
        {
            // Top qubit = chosen: the stored bits' parity is sector ^ chosen.
            const std::uint64_t want = static_cast<std::uint64_t>(((sector ? sector[b] : 0) ^ chosen) & 1);
            c.parity = ((1ull << n) - 1ull) | (want << 63);
            if (ci == 0)
            {
                c.mask = 0;
                c.value = 0;
                c.scale = scale;
            }
            else
                c.scale *= scale;
        }
        else if (ci == 0)
        {
            c.mask = chunk;
            c.value = val;
            c.scale = scale;
        }
        else
        {
            c.mask |= chunk;
            c.value |= val;
            c.scale *= scale;
        }
        LayerResult &r = res[b * res_stride];
        r.outcome |= val;
        const double pr = ok ? branch / total : 0.0;
        r.prob[ci] = pr;
        r.surprisal += ok ? -log(pr) : 0.0;
    }
}

template <typename Real>
__global__ void k_init_zero(Cx<Real> *states, std::uint64_t dim, std::uint64_t total)
{
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<std::uint64_t>(gridDim.x) * blockDim.x)
        states[i] = Cx<Real>{(i % dim) == 0 ? Real(1) : Real(0), Real(0)};
}

template <typename Real>
__global__ void k_collapse(Cx<Real> *states, std::uint64_t dim, std::uint64_t total, const Collapse *col,
                           std::size_t col_stride)
{
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<std::uint64_t>(gridDim.x) * blockDim.x)
    {
        const Collapse cl = col[(i / dim) * col_stride];
        states[i] = collapse_value(states[i], i % dim, cl, static_cast<Real>(cl.scale));
    }
}

// MIPT_GB300_CLUSTER_PASS=1 selects the two-CTA cluster kernel for FP32
// passes (default: the single-CTA register-round kernel, measured faster).
bool use_cluster_kernel()
{
    static const bool on = [] {
        const char *v = std::getenv("MIPT_GB300_CLUSTER_PASS");
        return v && v[0] == '1';
    }();
    return on;
}

// MIPT_GB300_PACKED_FMA=0 disables the packed FP32x2 gate arithmetic.
bool use_packed_fma()
{
    static const bool on = [] {
        const char *v = std::getenv("MIPT_GB300_PACKED_FMA");
        return !(v && v[0] == '0');
    }();
    return on;
}

// The register-round pass runs on a persistent grid (resident CTAs loop over
// the (trajectory, tile) items; measured 1.5 % faster at L=24 than one CTA per
// item); MIPT_GB300_PERSISTENT_PASS=0 launches one CTA per item instead.
bool use_persistent_pass()
{
    static const bool on = [] {
        const char *v = std::getenv("MIPT_GB300_PERSISTENT_PASS");
        return !(v && v[0] == '0');
    }();
    return on;
}

// Launch grid of a register-round pass: one CTA per (tile, trajectory) item,
// or, in persistent mode, as many CTAs as fit on the device at once.
dim3 pass_grid(const void *fn, int threads, std::size_t smem, dim3 items)
{
    if (!use_persistent_pass()) return items;
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem) != cudaSuccess || per_sm < 1)
    {
        cudaGetLastError();
        return items;
    }
    const std::uint64_t total = static_cast<std::uint64_t>(items.x) * items.y;
    const std::uint64_t resident = static_cast<std::uint64_t>(sms) * per_sm;
    return dim3(static_cast<unsigned>(std::min(total, resident)), 1, 1);
}

int grid_for(std::uint64_t total, int threads)
{
    const std::uint64_t blocks = (total + threads - 1) / threads;
    return static_cast<int>(std::min<std::uint64_t>(blocks, 152ull * 32ull));
}

template <typename Real>
std::size_t pass_smem(int k)
{
    return (sizeof(Cx<Real>) << k) + (sizeof(std::uint32_t) << k);
}

template <typename Real>
cudaError_t ensure_smem_attr(const void *fn, std::size_t bytes)
{
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}
} // namespace

__host__ __device__ void histogram_geometry(int n, int kmax, int cmin, std::uint64_t chunk, PassGeom &g)
{
    const int k = kmax < n ? kmax : n;
    const int c0 = cmin < k ? cmin : k;
    std::uint64_t used = (c0 >= 64) ? ~0ull : ((1ull << c0) - 1ull);
    int cnt = c0;
    for (int q = c0; q < n && cnt < k; ++q)
        if (!((chunk >> q) & 1ull))
        {
            used |= 1ull << q;
            ++cnt;
        }
    for (int q = c0; q < n && cnt < k; ++q)
        if (!((used >> q) & 1ull))
        {
            used |= 1ull << q;
            ++cnt;
        }
    g.n = n;
    g.k = k;
    int a = 0, z = 0;
    for (int q = 0; q < n; ++q)
    {
        if ((used >> q) & 1ull)
            g.pos[a++] = static_cast<std::int8_t>(q);
        else
            g.nl[z++] = static_cast<std::int8_t>(q);
    }
    int c = 0;
    while (c < k && g.pos[c] == c) ++c;
    g.c = c;
    g.n_nl = n - k;
}

int fp32_register_bits()
{
    static const int rb = [] {
        const char *v = std::getenv("MIPT_GB300_RB");
        return (v && v[0] == '5') ? 5 : 6;
    }();
    return rb;
}

const PassGeom &fused_hist_geometry(const PassPlan &p, bool fp32)
{
    return (fp32 && p.cluster_rounds > 0 && use_cluster_kernel()) ? p.hgeom : p.geom;
}

int local_measured_count(const PassGeom &g, std::uint64_t chunk)
{
    int m = 0;
    for (int i = 0; i < g.k; ++i)
        if ((chunk >> g.pos[i]) & 1ull) ++m;
    return m;
}

namespace
{
PassGeom make_geom(int n, std::uint64_t local)
{
    PassGeom g{};
    g.n = n;
    int a = 0, z = 0;
    for (int q = 0; q < n; ++q)
    {
        if ((local >> q) & 1ull)
            g.pos[a++] = static_cast<std::int8_t>(q);
        else
            g.nl[z++] = static_cast<std::int8_t>(q);
    }
    g.k = a;
    g.n_nl = z;
    int c = 0;
    while (c < a && g.pos[c] == c) ++c;
    g.c = c;
    return g;
}

int local_index(const PassGeom &g, int q)
{
    for (int i = 0; i < g.k; ++i)
        if (g.pos[i] == q) return i;
    return -1;
}

// Greedy packing of `todo` bonds into passes that each keep qubits
// 0..cmin-1 local; returns the passes and fills their gate lists.
std::vector<PassPlan> pack(int n, const std::vector<Bond> &bonds, std::vector<int> todo, int kmax, int cmin,
                           std::uint64_t first_local)
{
    std::vector<PassPlan> out;
    std::uint64_t local = first_local;
    bool first = first_local != 0;
    while (!todo.empty())
    {
        if (!first) local = (1ull << std::min(cmin, n)) - 1ull;
        std::vector<int> taken, rest;
        for (int i : todo)
        {
            const std::uint64_t need =
                local | (1ull << bonds[i].q0) | (bonds[i].q1 >= 0 ? (1ull << bonds[i].q1) : 0ull);
            if (__builtin_popcountll(need) <= kmax && (taken.size() < static_cast<std::size_t>(kMaxPassGates)))
            {
                if (first && (need != local))
                {
                    rest.push_back(i);
                    continue;
                }
                local = need;
                taken.push_back(i);
            }
            else
            {
                rest.push_back(i);
            }
        }
        if (taken.empty() && !first) throw std::runtime_error("bond does not fit a pass");
        // Widen the tile with further low qubits (longer contiguous runs).
        for (int q = 0; q < n && __builtin_popcountll(local) < kmax; ++q) local |= 1ull << q;
        PassPlan p{};
        p.geom = make_geom(n, local);
        p.gates.count = static_cast<int>(taken.size());
        std::uint64_t used = 0;
        for (int i : taken)
            used |= (1ull << bonds[i].q0) | (bonds[i].q1 >= 0 ? (1ull << bonds[i].q1) : 0ull);
        for (std::size_t j = 0; j < taken.size(); ++j)
        {
            const Bond &bd = bonds[taken[j]];
            p.gates.gate[j] = static_cast<std::int16_t>(taken[j]);
            p.gates.la[j] = static_cast<std::int8_t>(local_index(p.geom, bd.q0));
            int q1 = bd.q1;
            p.gates.kind[j] = 0;
            if (q1 < 0)
            {
                // Parity gate: pair it with a local qubit no other gate of
                // the pass touches.
                p.gates.kind[j] = 1;
                for (int q = 0; q < n && q1 < 0; ++q)
                    if (((local >> q) & 1ull) && !((used >> q) & 1ull)) q1 = q;
                if (q1 < 0)
                    q1 = bd.q0; // no free partner: the pass runs on the shared-memory kernel
                else
                    used |= 1ull << q1;
            }
            p.gates.lb[j] = static_cast<std::int8_t>(local_index(p.geom, q1));
        }
        if (!taken.empty()) out.push_back(p);
        todo = rest;
        first = false;
    }
    return out;
}
} // namespace


namespace
{
// Lane sets usable for the global load/store rounds: the four lowest tile
// bits (contiguous qubits) plus one bit of residue 4 mod 5.
std::uint32_t io_lanes(int k, std::uint32_t regmask)
{
    const std::uint32_t opts[2] = {0x1Fu, 0x20Fu};
    for (std::uint32_t o : opts)
    {
        if ((o >> k) != 0) continue;
        if ((o & regmask) == 0) return o;
    }
    return 0;
}

// Any five tile bits outside regmask with residues 0..4 mod 5 (one each).
std::uint32_t mid_lanes(int k, std::uint32_t regmask)
{
    std::uint32_t out = 0;
    for (int res = 0; res < 5; ++res)
    {
        int pick = -1;
        for (int p = res; p < k; p += 5)
            if (!((regmask >> p) & 1u))
            {
                pick = p;
                break;
            }
        if (pick < 0) return 0;
        out |= 1u << pick;
    }
    return out;
}

struct RoundSearch
{
    int k, rb, slots, nr;
    std::vector<std::pair<int, int>> bonds;
    std::vector<int> assign;
    std::vector<int> load;
};

bool rounds_feasible(RoundSearch &S, std::vector<std::uint32_t> &lanes)
{
    lanes.assign(S.nr, 0);
    for (int r = 0; r < S.nr; ++r)
    {
        std::uint32_t reg = 0;
        for (std::size_t b = 0; b < S.bonds.size(); ++b)
            if (S.assign[b] == r) reg |= (1u << S.bonds[b].first) | (1u << S.bonds[b].second);
        const bool io = (r == 0 || r == S.nr - 1);
        lanes[r] = io ? io_lanes(S.k, reg) : mid_lanes(S.k, reg);
        if (lanes[r] == 0) return false;
        if (S.nr == 1) lanes[r] = io_lanes(S.k, reg);
    }
    return true;
}

bool rounds_dfs(RoundSearch &S, std::size_t b, std::vector<std::uint32_t> &lanes)
{
    if (b == S.bonds.size()) return rounds_feasible(S, lanes);
    for (int r = 0; r < S.nr; ++r)
    {
        if (S.load[r] >= S.slots) continue;
        S.assign[b] = r;
        ++S.load[r];
        if (rounds_dfs(S, b + 1, lanes)) return true;
        --S.load[r];
    }
    return false;
}

// Schedules a pass's bonds into register rounds; returns false when the tile
// is too small or no schedule fits kMaxRounds.
bool plan_rounds(PassPlan &p, int rb)
{
    const int k = p.geom.k;
    p.rounds = 0;
    p.rb = rb;
    if (k < rb + 5 || k > 15) return false;
    RoundSearch S;
    S.k = k;
    S.rb = rb;
    S.slots = rb / 2;
    for (int i = 0; i < p.gates.count; ++i) S.bonds.push_back({p.gates.la[i], p.gates.lb[i]});
    const int nb = static_cast<int>(S.bonds.size());
    std::vector<std::uint32_t> lanes;
    for (int nr = std::max(1, (nb + S.slots - 1) / S.slots); nr <= kMaxRounds; ++nr)
    {
        S.nr = nr;
        S.assign.assign(nb, -1);
        S.load.assign(nr, 0);
        if (!rounds_dfs(S, 0, lanes)) continue;
        for (int r = 0; r < nr; ++r)
        {
            Round &R = p.round[r];
            std::uint32_t used = lanes[r];
            int slot = 0;
            for (int s = 0; s < 3; ++s) R.slot[s] = -1;
            for (int bI = 0; bI < nb; ++bI)
                if (S.assign[bI] == r)
                {
                    R.reg[2 * slot] = static_cast<std::int8_t>(S.bonds[bI].first);
                    R.reg[2 * slot + 1] = static_cast<std::int8_t>(S.bonds[bI].second);
                    used |= (1u << S.bonds[bI].first) | (1u << S.bonds[bI].second);
                    R.slot[slot] = static_cast<std::int16_t>(bI);
                    ++slot;
                }
            // Fill the remaining register bits with free tile bits.
            for (int i = 2 * slot; i < rb; ++i)
                for (int q = 0; q < k; ++q)
                    if (!((used >> q) & 1u))
                    {
                        R.reg[i] = static_cast<std::int8_t>(q);
                        used |= 1u << q;
                        break;
                    }
            // Lanes ordered by residue, then the warp bits.
            int t = 0;
            for (int res = 0; res < 5; ++res)
                for (int q = res; q < k; q += 5)
                    if ((lanes[r] >> q) & 1u)
                    {
                        R.tid[t++] = static_cast<std::int8_t>(q);
                        break;
                    }
            for (int q = 0; q < k; ++q)
                if (!((used >> q) & 1u)) R.tid[t++] = static_cast<std::int8_t>(q);
            if (t != k - rb) return false;
        }
        p.rounds = nr;
        return true;
    }
    return false;
}
} // namespace

namespace
{
// MIPT_GB300_CLUSTER_RB=5 selects 32 amplitudes per thread (256 threads per
// CTA) for the cluster kernel instead of 64 (128 threads).
int cluster_register_bits()
{
    static const int rb = [] {
        const char *v = std::getenv("MIPT_GB300_CLUSTER_RB");
        return (v && v[0] == '5') ? 5 : 6;
    }();
    return rb;
}

// Position of tile bit p once tile bit x is removed (the CTA-local offset).
inline int opos(int p, int x) { return p > x ? p - 1 : p; }

// Lanes 0..3 must flip the four low shared-memory bank bits (residues
// {0,1,2,3} mod 5 of their offset positions) for conflict-free 8-byte access.
bool lanes_ok(const int *l, int x)
{
    int seen = 0;
    for (int i = 0; i < 4; ++i)
    {
        const int r = opos(l[i], x) % 5;
        if (r > 3 || ((seen >> r) & 1)) return false;
        seen |= 1 << r;
    }
    return true;
}

struct CSearch
{
    int k, nr, rb;
    std::vector<std::pair<int, int>> bonds;
    std::vector<int> assign, load;
    std::vector<ClusterRound> out;
};

// Chooses x and lanes for rounds in order; the read side of round i uses the
// storage coordinates of round i-1's x.
bool cluster_choose(CSearch &S, int r, int prev_x)
{
    if (r == S.nr) return true;
    const int k = S.k;
    std::uint32_t reg = 0;
    std::vector<int> mine;
    for (std::size_t b = 0; b < S.bonds.size(); ++b)
        if (S.assign[b] == r)
        {
            reg |= (1u << S.bonds[b].first) | (1u << S.bonds[b].second);
            mine.push_back(static_cast<int>(b));
        }
    const bool first = r == 0, last = r == S.nr - 1;
    for (int x = k - 1; x >= 0; --x)
    {
        if ((reg >> x) & 1u) continue;
        // candidate lane sets: {0,1,2,3} first, then any four free bits
        std::vector<std::array<int, 4>> cands;
        if (!(reg & 0xFu) && x > 3) cands.push_back({0, 1, 2, 3});
        if (!first && !last)
        {
            std::vector<int> freeb;
            for (int q = 0; q < k; ++q)
                if (!((reg >> q) & 1u) && q != x) freeb.push_back(q);
            const int F = static_cast<int>(freeb.size());
            for (int a = 0; a < F; ++a)
                for (int b2 = a + 1; b2 < F; ++b2)
                    for (int c = b2 + 1; c < F; ++c)
                        for (int d = c + 1; d < F; ++d)
                            cands.push_back({freeb[a], freeb[b2], freeb[c], freeb[d]});
        }
        for (auto l : cands)
        {
            // order lanes so lane i has residue i in the read coordinates
            const int xr = first ? x : prev_x; // read (or load) coordinates
            std::array<int, 4> ord{};
            bool ok = true;
            int seen = 0;
            for (int q : l)
            {
                const int rr = opos(q, xr) % 5;
                if (rr > 3 || ((seen >> rr) & 1)) { ok = false; break; }
                seen |= 1 << rr;
                ord[rr] = q;
            }
            if (!ok) continue;
            if (!first && !lanes_ok(ord.data(), prev_x)) continue;
            if (!last && !lanes_ok(ord.data(), x)) continue;
            if ((first || last) && !(ord[0] == 0 && ord[1] == 1 && ord[2] == 2 && ord[3] == 3)) continue;
            ClusterRound R{};
            int slot = 0;
            R.slot[0] = R.slot[1] = R.slot[2] = -1;
            std::uint32_t used = (1u << x) | (1u << ord[0]) | (1u << ord[1]) | (1u << ord[2]) | (1u << ord[3]);
            for (int b : mine)
            {
                R.reg[2 * slot] = static_cast<std::int8_t>(S.bonds[b].first);
                R.reg[2 * slot + 1] = static_cast<std::int8_t>(S.bonds[b].second);
                used |= (1u << S.bonds[b].first) | (1u << S.bonds[b].second);
                R.slot[slot] = static_cast<std::int16_t>(b);
                ++slot;
            }
            for (int i = 2 * slot; i < S.rb; ++i)
                for (int q = 0; q < k; ++q)
                    if (!((used >> q) & 1u))
                    {
                        R.reg[i] = static_cast<std::int8_t>(q);
                        used |= 1u << q;
                        break;
                    }
            int t = 0;
            for (int i = 0; i < 4; ++i) R.tid[t++] = static_cast<std::int8_t>(ord[i]);
            for (int q = 0; q < k; ++q)
                if (!((used >> q) & 1u)) R.tid[t++] = static_cast<std::int8_t>(q);
            if (t != k - 1 - S.rb) continue;
            R.x = static_cast<std::int8_t>(x);
            S.out[r] = R;
            if (cluster_choose(S, r + 1, x)) return true;
        }
    }
    return false;
}

bool cluster_dfs(CSearch &S, std::size_t b)
{
    if (b == S.bonds.size()) return cluster_choose(S, 0, -1);
    for (int r = 0; r < S.nr; ++r)
    {
        if (S.load[r] >= S.rb / 2) continue;
        S.assign[b] = r;
        ++S.load[r];
        if (cluster_dfs(S, b + 1)) return true;
        --S.load[r];
    }
    return false;
}

bool plan_cluster_rounds(PassPlan &p, int rb)
{
    p.cluster_rounds = 0;
    p.cluster_rb = rb;
    if (p.geom.k != 14) return false;
    CSearch S;
    S.k = 14;
    S.rb = rb;
    for (int i = 0; i < p.gates.count; ++i) S.bonds.push_back({p.gates.la[i], p.gates.lb[i]});
    const int nb = static_cast<int>(S.bonds.size());
    const int slots = rb / 2;
    for (int nr = std::max(1, (nb + slots - 1) / slots); nr <= kMaxRounds; ++nr)
    {
        S.nr = nr;
        S.assign.assign(nb, -1);
        S.load.assign(nr, 0);
        S.out.assign(nr, ClusterRound{});
        if (!cluster_dfs(S, 0)) continue;
        for (int r = 0; r < nr; ++r) p.cround[r] = S.out[r];
        p.cluster_rounds = nr;
        // Histogram geometry of a half tile: the tile bits other than the last
        // round's x are local; tile-index bit 0 is the CTA rank (qubit of x).
        const int xz = p.cround[nr - 1].x;
        PassGeom h{};
        h.n = p.geom.n;
        h.k = 13;
        int a = 0;
        for (int q = 0; q < 14; ++q)
            if (q != xz) h.pos[a++] = p.geom.pos[q];
        h.n_nl = p.geom.n_nl + 1;
        h.nl[0] = p.geom.pos[xz];
        for (int i = 0; i < p.geom.n_nl; ++i) h.nl[i + 1] = p.geom.nl[i];
        int c = 0;
        while (c < 13 && h.pos[c] == c) ++c;
        h.c = c;
        p.hgeom = h;
        return true;
    }
    return false;
}
} // namespace

std::vector<PassPlan> plan_layer(int n, const std::vector<Bond> &bonds, int kmax, int cmin, int rb)
{
    if (n > 32) throw std::invalid_argument("engine supports at most 32 qubits");
    kmax = std::min(kmax, n);
    std::vector<int> all(bonds.size());
    for (std::size_t i = 0; i < bonds.size(); ++i) all[i] = static_cast<int>(i);
    if (bonds.empty())
    {
        PassPlan p{};
        p.geom = make_geom(n, (1ull << kmax) - 1ull);
        p.gates.count = 0;
        plan_rounds(p, rb);
        if (rb >= 5) plan_cluster_rounds(p, cluster_register_bits());
        return {p};
    }
    // Try first tiles made of a low contiguous block, optionally with the top
    // qubit (for a ring-closing bond), and keep the plan with fewest passes.
    std::vector<PassPlan> best;
    for (int c0 = kmax; c0 >= std::max(1, kmax - 3); --c0)
    {
        for (int wrap = 0; wrap < 2; ++wrap)
        {
            std::uint64_t local = (1ull << c0) - 1ull;
            if (wrap)
            {
                if (c0 >= kmax || c0 >= n) continue;
                local |= 1ull << (n - 1);
            }
            auto plan = pack(n, bonds, all, kmax, cmin, local);
            if (best.empty() || plan.size() < best.size()) best = plan;
        }
    }
    for (auto &p : best)
    {
        bool unpaired = false;
        for (int j = 0; j < p.gates.count; ++j) unpaired = unpaired || (p.gates.kind[j] && p.gates.la[j] == p.gates.lb[j]);
        if (unpaired)
        {
            p.rounds = 0;
            p.cluster_rounds = 0;
            continue;
        }
        plan_rounds(p, rb);
        bool parity = false;
        for (int j = 0; j < p.gates.count; ++j) parity = parity || p.gates.kind[j];
        if (rb >= 5 && !parity) plan_cluster_rounds(p, cluster_register_bits());
    }
    return best;
}

template <typename Real>
cudaError_t launch_init_zero(Cx<Real> *states, std::uint64_t dim, int batch, cudaStream_t s)
{
    const std::uint64_t total = dim * static_cast<std::uint64_t>(batch);
    k_init_zero<Real><<<grid_for(total, 256), 256, 0, s>>>(states, dim, total);
    return cudaGetLastError();
}

// MIPT_GB300_TILE_TMA=0 turns the TMA tile loads of FP32 passes off.
bool use_tile_tma()
{
    static const bool on = [] {
        const char *v = std::getenv("MIPT_GB300_TILE_TMA");
        return !(v && v[0] == '0');
    }();
    return on;
}

PFN_cuTensorMapEncodeTiled_v12000 tile_map_encoder()
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

// Tensor map over `batch` FP32 states of 2^n amplitudes whose box is one tile
// of geometry g in plain tile order. The global index bits split into runs of
// local or non-local qubits; local runs longer than 8 bits split into boxes of
// at most 256; the last run also carries the trajectory index. Needs local
// positions in ascending qubit order, a local run at bit 0 (the innermost box
// then spans >= 16 bytes) and at most 5 dimensions; false otherwise.
bool encode_tile_map(CUtensorMap &map, TileTma &t, const Cx<float> *states, int batch, const PassGeom &g)
{
    std::memset(&map, 0, sizeof(map));
    t = TileTma{};
    if (tile_map_encoder() == nullptr || (reinterpret_cast<std::uintptr_t>(states) & 15u) != 0) return false;
    for (int i = 1; i < g.k; ++i)
        if (g.pos[i] <= g.pos[i - 1]) return false;
    bool local[kMaxQubits] = {};
    for (int i = 0; i < g.k; ++i) local[g.pos[i]] = true;
    if (!local[0]) return false;
    int q = 0;
    while (q < g.n)
    {
        int len = 1;
        while (q + len < g.n && local[q + len] == local[q] && (!local[q] || len < 8)) ++len;
        if (t.rank == 5) return false;
        t.lo[t.rank] = q;
        t.bits[t.rank] = len;
        ++t.rank;
        q += len;
    }
    cuuint64_t dims[5], strides[4];
    cuuint32_t box[5], es[5];
    for (int d = 0; d < t.rank; ++d)
    {
        const bool loc = local[t.lo[d]];
        dims[d] = 1ull << t.bits[d];
        if (d + 1 == t.rank) dims[d] *= static_cast<cuuint64_t>(batch);
        box[d] = loc ? (1u << t.bits[d]) : 1u;
        es[d] = 1;
        if (d > 0) strides[d - 1] = (1ull << t.lo[d]) * sizeof(Cx<float>);
    }
    if (dims[t.rank - 1] >= (1ull << 32)) return false;
    return tile_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, static_cast<cuuint32_t>(t.rank),
                              const_cast<Cx<float> *>(states), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Test hook: the next `count` TMA-fed pass launches withhold CTA 0's first
// tile load (set_withheld_tile_loads), so their bounded tile waits run out.
std::atomic<int> g_withheld_loads{0};

int take_withheld_load()
{
    int c = g_withheld_loads.load();
    while (c > 0 && !g_withheld_loads.compare_exchange_weak(c, c - 1)) {}
    return c > 0 ? 1 : 0;
}

// Launches k_pass_rounds<Real, RB, TMA, PAR> on its grid.
template <typename Real, int RB, bool TMA, bool PAR>
cudaError_t launch_rounds(Cx<Real> *states, int batch, const PassPlan &plan, const Cx<Real> *layer_gates,
                          std::size_t gate_stride, const Collapse *collapse_in, std::size_t collapse_stride,
                          const LayerMeas *meas, std::size_t meas_stride, double *partials, int fuse_hist,
                          const CUtensorMap &map, const TileTma &tt, int *err, cudaStream_t s,
                          std::uint64_t col_keep, int col_scaled, int sparse)
{
    const void *fn = reinterpret_cast<const void *>(&k_pass_rounds<Real, RB, TMA, PAR>);
    const std::size_t smem = (sizeof(Cx<Real>) << plan.geom.k) + (TMA ? (sizeof(float) << plan.geom.k) + 128 : 0) +
                             (sparse ? sizeof(std::uint32_t) * (static_cast<std::size_t>(batch) + 1) : 0);
    cudaError_t e = ensure_smem_attr<Real>(fn, smem);
    if (e != cudaSuccess) return e;
    const int threads = 1 << (plan.geom.k - RB);
    const dim3 pgrid = pass_grid(fn, threads, smem, dim3(1u << plan.geom.n_nl, batch));
    k_pass_rounds<Real, RB, TMA, PAR><<<pgrid, threads, smem, s>>>(states, plan, layer_gates, gate_stride, collapse_in,
                                                               collapse_stride, meas, meas_stride, partials,
                                                               fuse_hist, use_packed_fma() ? 1 : 0, batch, map, tt,
                                                               err, col_keep, col_scaled, sparse,
                                                               TMA ? take_withheld_load() : 0);
    return cudaGetLastError();
}


bool sparse_pass_supported(const PassPlan &plan, bool fp32, int batch)
{
    if (plan.rounds <= 0 || plan.geom.n_nl <= 0 || batch < 1) return false;
    if (fp32 && plan.cluster_rounds > 0 && use_cluster_kernel()) return false;
    if (fp32 && plan.rb != 5 && plan.rb != 6) return false;
    if (!fp32 && plan.rb != 5) return false;
    if ((static_cast<std::uint64_t>(batch) << plan.geom.n_nl) >= (1ull << 31)) return false;
    // Tile (+ histogram values and alignment with TMA) + item table.
    const std::size_t base = fp32 ? (sizeof(Cx<float>) << plan.geom.k) + (sizeof(float) << plan.geom.k) + 128
                                  : (sizeof(Cx<double>) << plan.geom.k);
    return base + sizeof(std::uint32_t) * (static_cast<std::size_t>(batch) + 1) <= (200u << 10);
}

template <typename Real>
cudaError_t launch_pass(Cx<Real> *states, int batch, const PassPlan &plan, const Cx<Real> *layer_gates,
                        std::size_t gate_stride, const Collapse *collapse_in, std::size_t collapse_stride,
                        const LayerMeas *meas, std::size_t meas_stride, double *partials, int fuse_hist,
                        int *err, cudaStream_t s, std::uint64_t col_keep, int col_scaled, int sparse,
                        int parity_mode)
{
    dim3 grid(1u << plan.geom.n_nl, batch);
    if ((sparse || col_keep != ~0ull || !col_scaled) && !sparse_pass_supported(plan, sizeof(Real) == 4, batch))
        return cudaErrorInvalidValue;
    if (sparse && (collapse_in == nullptr || fuse_hist)) return cudaErrorInvalidValue;
    if constexpr (sizeof(Real) == 4)
    {
        if (plan.cluster_rounds > 0 && use_cluster_kernel())
        {
            const std::size_t smem = sizeof(Cx<float>) << 13;
            dim3 cgrid(2u << plan.geom.n_nl, batch);
            cudaError_t e;
            if (plan.cluster_rb == 6)
            {
                e = cudaFuncSetAttribute(reinterpret_cast<const void *>(&k_pass_cluster<6>),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
                if (e != cudaSuccess) return e;
                k_pass_cluster<6><<<cgrid, 128, smem, s>>>(states, plan, layer_gates, gate_stride, collapse_in,
                                                           collapse_stride, meas, meas_stride, partials, fuse_hist);
            }
            else
            {
                e = cudaFuncSetAttribute(reinterpret_cast<const void *>(&k_pass_cluster<5>),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
                if (e != cudaSuccess) return e;
                k_pass_cluster<5><<<cgrid, 256, smem, s>>>(states, plan, layer_gates, gate_stride, collapse_in,
                                                           collapse_stride, meas, meas_stride, partials, fuse_hist);
            }
            return cudaGetLastError();
        }
    }
    if (plan.rounds > 0)
    {
#define MG_ROUNDS(RBV, TMAV, PARV)                                                                                    \
    launch_rounds<Real, RBV, TMAV, PARV>(states, batch, plan, layer_gates, gate_stride, collapse_in, collapse_stride, \
                                         meas, meas_stride, partials, fuse_hist, map, tt, err, s, col_keep,            \
                                         col_scaled, sparse)
        CUtensorMap map;
        TileTma tt{};
        std::memset(&map, 0, sizeof(map));
        const bool par = parity_mode != 0;
        if constexpr (sizeof(Real) == 4)
        {
            const bool tma = use_persistent_pass() && use_tile_tma() && err != nullptr &&
                             encode_tile_map(map, tt, states, batch, plan.geom);
            if (plan.rb == 6)
            {
                if (tma) return par ? MG_ROUNDS(6, true, true) : MG_ROUNDS(6, true, false);
                return par ? MG_ROUNDS(6, false, true) : MG_ROUNDS(6, false, false);
            }
            if (plan.rb == 5)
            {
                if (tma) return par ? MG_ROUNDS(5, true, true) : MG_ROUNDS(5, true, false);
                return par ? MG_ROUNDS(5, false, true) : MG_ROUNDS(5, false, false);
            }
            return cudaErrorInvalidValue;
        }
        else
        {
            if (plan.rb != 5) return cudaErrorInvalidValue;
            return par ? MG_ROUNDS(5, false, true) : MG_ROUNDS(5, false, false);
        }
#undef MG_ROUNDS
    }
    const std::size_t smem = pass_smem<Real>(plan.geom.k);
    cudaError_t e = ensure_smem_attr<Real>(reinterpret_cast<const void *>(&k_pass<Real>), smem);
    if (e != cudaSuccess) return e;
    k_pass<Real><<<grid, kPassThreads, smem, s>>>(states, plan.geom, plan.gates, layer_gates, gate_stride,
                                                  collapse_in, collapse_stride, meas, meas_stride, partials,
                                                  fuse_hist);
    return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_hist(const Cx<Real> *states, int batch, int n, int kmax, int cmin, int chunk_index,
                        const Collapse *collapse_in, std::size_t collapse_stride, const LayerMeas *meas,
                        std::size_t meas_stride, double *partials, bool direct, cudaStream_t s,
                        const signed char *sector)
{
    const int k = std::min(kmax, n);
    // Direct (all measured sites outside the tile): only the segment table.
    const std::size_t smem = direct ? (sizeof(std::uint32_t) << std::max(0, k - std::min(cmin, k)))
                                    : pass_smem<Real>(k);
    cudaError_t e = ensure_smem_attr<Real>(reinterpret_cast<const void *>(&k_hist<Real>), smem);
    if (e != cudaSuccess) return e;
    dim3 grid(1u << (n - k), batch);
    k_hist<Real><<<grid, kPassThreads, smem, s>>>(states, n, kmax, cmin, chunk_index, collapse_in, collapse_stride,
                                                  meas, meas_stride, partials, direct ? 1 : 0, sector);
    return cudaGetLastError();
}

cudaError_t launch_measure(int batch, int n, const PassGeom *fused_geom, int kmax, int cmin, int chunk_index,
                           const LayerMeas *meas, std::size_t meas_stride, const double *partials,
                           double *bins_scratch, std::size_t bins_stride, const std::uint64_t *forced,
                           std::size_t forced_stride, Collapse *collapse_out, std::size_t collapse_stride,
                           LayerResult *result, std::size_t result_stride, int *error_flag, cudaStream_t s,
                           const signed char *sector)
{
    PassGeom fg{};
    if (fused_geom) fg = *fused_geom;
    k_measure<<<batch, kMeasureThreads, 0, s>>>(n, fg, fused_geom != nullptr, kmax, cmin, chunk_index, meas,
                                                meas_stride, partials, bins_scratch, bins_stride, forced,
                                                forced_stride,
                                                collapse_out, collapse_stride, result, result_stride, error_flag,
                                                sector);
    return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_collapse(Cx<Real> *states, std::uint64_t dim, int batch, const Collapse *collapse,
                            std::size_t collapse_stride, cudaStream_t s)
{
    const std::uint64_t total = dim * static_cast<std::uint64_t>(batch);
    k_collapse<Real><<<grid_for(total, 256), 256, 0, s>>>(states, dim, total, collapse, collapse_stride);
    return cudaGetLastError();
}

void set_withheld_tile_loads(int count) { g_withheld_loads.store(count > 0 ? count : 0); }

#define MG_INSTANTIATE(R)                                                                                        \
    template cudaError_t launch_init_zero<R>(Cx<R> *, std::uint64_t, int, cudaStream_t);                         \
    template cudaError_t launch_pass<R>(Cx<R> *, int, const PassPlan &, const Cx<R> *, std::size_t,              \
                                        const Collapse *, std::size_t, const LayerMeas *, std::size_t, double *, \
                                        int, int *, cudaStream_t, std::uint64_t, int, int, int);                 \
    template cudaError_t launch_hist<R>(const Cx<R> *, int, int, int, int, int, const Collapse *, std::size_t,   \
                                        const LayerMeas *, std::size_t, double *, bool, cudaStream_t,            \
                                        const signed char *);                                                    \
    template cudaError_t launch_collapse<R>(Cx<R> *, std::uint64_t, int, const Collapse *, std::size_t,          \
                                            cudaStream_t);
MG_INSTANTIATE(float)
MG_INSTANTIATE(double)
#undef MG_INSTANTIATE

} // namespace mg
