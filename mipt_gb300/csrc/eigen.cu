// Batched FP64 eigenvalues of complex Hermitian matrices (reduced density
// matrices), and the von Neumann entropy from them.
//
// Reference behaviour reproduced: the FP64 spectrum of rho_A and
// S_vN = -sum lambda log2 lambda over lambda > 1e-15, |S| < 1e-12 -> 0
// (cpp/src/cuda/tmi_cuda_svd.cu:663-798 with its FP64 retry :458-561, and
// cpp/include/mipt/tmi/linalg.hpp:125-132). The reference gets the spectrum
// from cuSOLVER (heevd / gesvd); here it is computed by two kernels of our
// own, written from the textbook algorithms:
//
//   k_tridiag   one CTA per matrix: Householder reduction of the Hermitian
//               matrix (row-major, interleaved re/im, the lower triangle
//               read and updated) to a real
//               symmetric tridiagonal matrix. Step j reflects the column below
//               the diagonal onto alpha e_1 with H = I - beta v v^H,
//               v = x - alpha e_1, alpha = -phase(x_0) |x|, beta = 2 / |v|^2,
//               and updates the trailing block B <- H B H as
//               B - v w^H - w v^H with p = beta B v, K = beta/2 v^H p,
//               w = p - K v. The off-diagonal |alpha| is kept (a Hermitian
//               tridiagonal matrix with complex off-diagonals is unitarily
//               similar to the real one with their moduli).
//   k_tridiag_ql one thread per matrix: eigenvalues of the tridiagonal matrix
//               by the implicit QL iteration with Wilkinson-type shifts and
//               plane rotations (the tql1/tqli scheme of EISPACK and
//               Numerical Recipes, eigenvalues only), then the entropy.
//
// All reductions run in a fixed order, so results are reproducible.
// FP64 throughout: GB300's FP64 rate bounds the reduction at about 16/3 d^3
// flops per matrix (full matrix-vector product, lower-triangle update).
#include "observables.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

namespace mg
{
namespace
{
constexpr int kTriThreads = 512;
constexpr int kQlMaxIter = 60;

__device__ __forceinline__ double2 cmul_conj(double2 a, double2 b) // a * conj(b)
{
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// Block sum in a fixed order: per-warp shuffle trees, then warp 0 sums the
// warp totals. `red` holds at least 32 doubles. Every thread gets the sum.
__device__ double block_sum(double v, double *red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads(); // red is free (previous readers are done)
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0)
    {
        double t = lane < nw ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

// Barrier among the `parts` CTAs of one matrix (multi-CTA reduction): a
// monotonic arrival counter, so epoch e is complete when it reaches
// (e + 1) * parts. The wait is bounded; a wait that runs out sets bit 2 of
// *err and makes every CTA of the matrix return.
__device__ bool parts_barrier(unsigned *ctr, unsigned parts, unsigned &epoch, int *err, int *s_ok)
{
    __syncthreads();
    if (threadIdx.x == 0)
    {
        int ok = 1;
        __threadfence();
        atomicAdd(ctr, 1u);
        const unsigned target = (epoch + 1) * parts;
        const std::uint64_t t0 = device_ns();
        for (unsigned it = 0; *reinterpret_cast<volatile unsigned *>(ctr) < target; ++it)
        {
            if (it > (1u << 24) || ((it & 15u) == 15u && device_ns() - t0 > 2000000000ull))
            {
                atomicOr(err, 2);
                ok = 0;
                break;
            }
            if (it > 32) __nanosleep(128);
        }
        __threadfence();
        *s_ok = ok;
    }
    ++epoch;
    __syncthreads();
    return *s_ok != 0;
}

// Householder tridiagonalisation. parts == 1: one CTA per matrix. parts > 1
// (cooperative launch, all CTAs resident): CTA `part` of a matrix owns the
// trailing-block rows i with i % parts == part; every CTA computes the
// reflector, |x| and K itself from the same data in the same order (so all
// agree bit for bit), the rows' p = beta B v go through pglob, and two
// barriers per step order the row updates against the next step's reads.
__global__ void __launch_bounds__(kTriThreads)
    k_tridiag(double2 *__restrict__ mats, int d, double *__restrict__ diag, double *__restrict__ off, int parts,
              double2 *__restrict__ pglob, unsigned *__restrict__ bars, int *__restrict__ err,
              const int *__restrict__ dims)
{
    extern __shared__ double2 sh[];
    double2 *v = sh;     // Householder vector (length m)
    double2 *w = sh + d; // p, then w
    __shared__ double red[33];
    __shared__ int s_ok;
    const int mat = blockIdx.x / parts, part = blockIdx.x % parts;
    double2 *a = mats + static_cast<std::size_t>(mat) * d * d;
    double *dg = diag + static_cast<std::size_t>(mat) * d;
    double *of = off + static_cast<std::size_t>(mat) * d;
    double2 *pg = parts > 1 ? pglob + static_cast<std::size_t>(mat) * d : nullptr;
    unsigned *bar = parts > 1 ? bars + mat : nullptr;
    unsigned epoch = 0;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    // Rows that hold data (the rest of the d x d block is zero: their
    // eigenvalues are 0). The row stride stays d.
    const int dm = dims != nullptr ? dims[mat] : d;

    for (int j = 0; j + 1 < dm; ++j)
    {
        const int m = dm - 1 - j, r0 = j + 1;
        __syncthreads(); // the previous step's reads of v[] and w[] are done
        // x = column j below the diagonal (the lower triangle is the valid
        // half of the trailing block).
        double part_sum = 0.0;
        for (int i = tid; i < m; i += nt)
        {
            const double2 x = a[static_cast<std::size_t>(r0 + i) * d + j];
            v[i] = x;
            if (i > 0) part_sum += x.x * x.x + x.y * x.y;
        }
        const double sigma = block_sum(part_sum, red); // also orders the v[] writes
        const double2 x0 = v[0];
        const double ax0 = hypot(x0.x, x0.y);
        const double norm = sqrt(ax0 * ax0 + sigma);
        if (tid == 0 && part == 0)
        {
            dg[j] = a[static_cast<std::size_t>(j) * d + j].x;
            of[j] = norm;
        }
        if (m == 1 || sigma == 0.0) continue; // already tridiagonal in this column (a phase only)
        const double2 ph = ax0 > 0.0 ? make_double2(x0.x / ax0, x0.y / ax0) : make_double2(1.0, 0.0);
        const double beta = 2.0 / ((ax0 + norm) * (ax0 + norm) + sigma);
        __syncthreads(); // every thread has read v[0]
        if (tid == 0) v[0] = make_double2(ph.x * (ax0 + norm), ph.y * (ax0 + norm));
        __syncthreads();
        // p = beta * B v on this CTA's rows, one warp per row. Only the lower
        // triangle of B is kept: row i supplies B_ik for k <= i, column i
        // (conj(B_ki), a strided read) the rest. Four independent accumulator
        // pairs per lane keep the FP64 pipe busy.
        for (int i = part + warp * parts; i < m; i += nw * parts)
        {
            const double2 *row = a + static_cast<std::size_t>(r0 + i) * d + r0;
            const double2 *col = a + static_cast<std::size_t>(r0) * d + r0 + i;
            double sr[4] = {0.0, 0.0, 0.0, 0.0}, si[4] = {0.0, 0.0, 0.0, 0.0};
            auto acc = [&](int kk, double &ar, double &ai) {
                double2 bk;
                if (kk <= i)
                    bk = row[kk];
                else
                {
                    const double2 t = col[static_cast<std::size_t>(kk) * d];
                    bk = make_double2(t.x, -t.y);
                }
                const double2 x = v[kk];
                ar = fma(bk.x, x.x, ar);
                ar = fma(-bk.y, x.y, ar);
                ai = fma(bk.x, x.y, ai);
                ai = fma(bk.y, x.x, ai);
            };
            int k = lane;
            for (; k + 96 < m; k += 128)
            {
#pragma unroll
                for (int u = 0; u < 4; ++u) acc(k + 32 * u, sr[u], si[u]);
            }
#pragma unroll
            for (int u = 0; u < 3; ++u)
                if (k + 32 * u < m) acc(k + 32 * u, sr[u], si[u]);
            double tr = (sr[0] + sr[1]) + (sr[2] + sr[3]);
            double ti = (si[0] + si[1]) + (si[2] + si[3]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
            {
                tr += __shfl_xor_sync(0xffffffffu, tr, o);
                ti += __shfl_xor_sync(0xffffffffu, ti, o);
            }
            if (lane == 0)
            {
                const double2 pv = make_double2(beta * tr, beta * ti);
                if (pg)
                    pg[i] = pv;
                else
                    w[i] = pv;
            }
        }
        if (pg)
        {
            if (!parts_barrier(bar, parts, epoch, err, &s_ok)) return;
            for (int i = tid; i < m; i += nt) w[i] = pg[i];
        }
        __syncthreads();
        // K = beta/2 Re(v^H p) (real for Hermitian B).
        part_sum = 0.0;
        for (int i = tid; i < m; i += nt) part_sum += v[i].x * w[i].x + v[i].y * w[i].y;
        const double K = 0.5 * beta * block_sum(part_sum, red);
        for (int i = tid; i < m; i += nt) w[i] = make_double2(w[i].x - K * v[i].x, w[i].y - K * v[i].y);
        __syncthreads();
        // B <- B - v w^H - w v^H on this CTA's rows of the trailing block's
        // lower triangle: b -= v_i conj(w_k) + w_i conj(v_k), eight FMAs per
        // entry (the diagonal's imaginary parts cancel exactly).
        for (int i = part + warp * parts; i < m; i += nw * parts)
        {
            double2 *row = a + static_cast<std::size_t>(r0 + i) * d + r0;
            const double2 vi = v[i], wi = w[i];
#pragma unroll 4
            for (int k = lane; k <= i; k += 32)
            {
                const double2 wk = w[k], vk = v[k];
                double2 b = row[k];
                b.x = fma(-vi.x, wk.x, b.x);
                b.x = fma(-vi.y, wk.y, b.x);
                b.x = fma(-wi.x, vk.x, b.x);
                b.x = fma(-wi.y, vk.y, b.x);
                b.y = fma(-vi.y, wk.x, b.y);
                b.y = fma(vi.x, wk.y, b.y);
                b.y = fma(-wi.y, vk.x, b.y);
                b.y = fma(wi.x, vk.y, b.y);
                row[k] = b;
            }
        }
        if (pg && !parts_barrier(bar, parts, epoch, err, &s_ok)) return;
    }
    if (tid == 0 && part == 0)
    {
        dg[dm - 1] = a[static_cast<std::size_t>(dm - 1) * d + dm - 1].x;
        of[dm - 1] = 0.0;
        for (int i = dm; i < d; ++i) dg[i] = of[i] = 0.0;
    }
}

// Implicit QL on one symmetric tridiagonal matrix (diagonal dg[0..d), off-
// diagonal of[0..d-1), of[j] coupling j and j+1); eigenvalues overwrite dg.
// Returns false if an eigenvalue needs more than kQlMaxIter sweeps.
__device__ bool tridiag_ql(double *dg, double *of, int d)
{
    // Off-diagonals below eps * |T| count as zero: eigenvalues are then
    // exact to about eps * |T| in absolute terms, far below the entropy's
    // 1e-15 eigenvalue cut-off for a density matrix.
    double anorm = 0.0;
    for (int i = 0; i < d; ++i) anorm = fmax(anorm, fabs(dg[i]) + fabs(of[i]) + (i > 0 ? fabs(of[i - 1]) : 0.0));
    const double tiny = 2.220446049250313e-16 * anorm;
    for (int l = 0; l < d; ++l)
    {
        int iter = 0;
        for (;;)
        {
            int m = l;
            for (; m + 1 < d; ++m)
            {
                const double dd = fabs(dg[m]) + fabs(dg[m + 1]);
                if (fabs(of[m]) <= 2.220446049250313e-16 * dd || fabs(of[m]) <= tiny) break;
            }
            if (m == l) break;
            if (++iter > kQlMaxIter) return false;
            // Shift from the leading 2x2 block's eigenvalue nearer dg[l].
            double g = (dg[l + 1] - dg[l]) / (2.0 * of[l]);
            double r = hypot(g, 1.0);
            g = dg[m] - dg[l] + of[l] / (g + copysign(r, g));
            double s = 1.0, c = 1.0, p = 0.0;
            int i = m - 1;
            bool underflow = false;
            for (; i >= l; --i)
            {
                const double f = s * of[i], b = c * of[i];
                // The entries of a density matrix's tridiagonal form are at
                // most 1 in modulus, so f^2 + g^2 needs no scaling; one
                // reciprocal square root gives r, s and c (a shorter
                // dependent chain than hypot and a division).
                const double t = fma(f, f, g * g);
                if (t == 0.0)
                {
                    of[i + 1] = 0.0;
                    dg[i + 1] -= p;
                    of[m] = 0.0;
                    underflow = true;
                    break;
                }
                const double ir = rsqrt(t);
                r = t * ir;
                of[i + 1] = r;
                s = f * ir;
                c = g * ir;
                g = dg[i + 1] - p;
                r = (dg[i] - g) * s + 2.0 * c * b;
                p = s * r;
                dg[i + 1] = g + p;
                g = c * r - b;
            }
            if (underflow) continue;
            dg[l] -= p;
            of[l] = g;
            of[m] = 0.0;
        }
    }
    return true;
}

__global__ void k_tridiag_ql(double *__restrict__ diag, double *__restrict__ off, int d, int nb,
                             double *__restrict__ entropy, int *__restrict__ err, const int *__restrict__ dims)
{
    const int jb = blockIdx.x * blockDim.x + threadIdx.x;
    if (jb >= nb) return;
    double *dg = diag + static_cast<std::size_t>(jb) * d;
    double *of = off + static_cast<std::size_t>(jb) * d;
    const int dm = dims != nullptr ? dims[jb] : d;
    if (!tridiag_ql(dg, of, dm))
    {
        atomicOr(err, 1);
        entropy[jb] = NAN;
        return;
    }
    double s = 0.0;
    for (int i = 0; i < dm; ++i)
    {
        const double l = dg[i];
        if (l > 1e-15) s -= l * log2(l);
    }
    entropy[jb] = fabs(s) < 1e-12 ? 0.0 : s;
}
} // namespace

std::size_t hermitian_eig_scratch_doubles(int d, int nb)
{
    // diag and off (d each), p vectors (2 d), barrier counters (1 double
    // each, used as unsigned).
    return (4 * static_cast<std::size_t>(d) + 1) * nb;
}

cudaError_t hermitian_eig_entropy(double *rho, int d, int nb, double *entropy_out, double *eig_out, double *scratch,
                                  int *err, cudaStream_t s, const int *dims)
{
    if (nb <= 0) return cudaSuccess;
    if (d < 2 || d > 4096) return cudaErrorInvalidValue;
    double *diag = eig_out ? eig_out : scratch;
    double *off = scratch + static_cast<std::size_t>(d) * nb;
    double2 *pglob = reinterpret_cast<double2 *>(scratch + 2 * static_cast<std::size_t>(d) * nb);
    unsigned *bars = reinterpret_cast<unsigned *>(scratch + 4 * static_cast<std::size_t>(d) * nb);
    const std::size_t smem = 2 * sizeof(double2) * d;
    cudaError_t e = cudaFuncSetAttribute(k_tridiag, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    // Fewer matrices than SMs: spread each matrix over `parts` resident CTAs
    // (cooperative launch), at least 16 trailing rows per CTA.
    int dev = 0, sms = 0, per_sm = 0;
    int parts = 1;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tridiag, kTriThreads, smem) == cudaSuccess &&
        per_sm > 0)
    {
        const int resident = sms * per_sm;
        parts = std::max(1, std::min({resident / nb, d / 16, 64}));
    }
    cudaGetLastError();
    if (parts > 1)
    {
        e = cudaMemsetAsync(bars, 0, sizeof(unsigned) * nb, s);
        if (e != cudaSuccess) return e;
        int dd = d;
        void *args[] = {&rho, &dd, &diag, &off, &parts, &pglob, &bars, &err, &dims};
        e = cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(&k_tridiag), dim3(nb * parts),
                                        dim3(kTriThreads), args, smem, s);
    }
    else
    {
        k_tridiag<<<nb, kTriThreads, smem, s>>>(reinterpret_cast<double2 *>(rho), d, diag, off, 1, nullptr, nullptr,
                                                err, dims);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    // One thread per matrix, spread over every SM: the QL sweep is a serial
    // FP64 chain per matrix, so few threads per SM run it fastest.
    const int sm_count = sms > 0 ? sms : 152;
    const int tpb = std::max(1, std::min(32, (nb + sm_count - 1) / sm_count));
    k_tridiag_ql<<<(nb + tpb - 1) / tpb, tpb, 0, s>>>(diag, off, d, nb, entropy_out, err, dims);
    return cudaGetLastError();
}

} // namespace mg
