// Batched genuine-multipartite-negativity (GMN) SDP of three-qubit states on
// the GPU: first-order ADMM in FP32 (or FP64) with FP64 duality-gap
// certificates.
//
// The SDP is the reference's monotone, fully decomposable witness
// (cpp/src/analysis/gmn_mosek.c:14-40, python/gmn.py:236-358, paths inside the
// reference project):
//     min Re Tr(rho W)  s.t.  0 <= Q_m <= I,  0 <= W - PT_m(Q_m) <= I,
// m = 1, 2, 3 the bipartition masks; GMN = -min, 0 at or below 1e-8
// (python/gmn.py:347-351). PT_m takes entry (r, c) from
// (r & ~m | c & m, c & ~m | r & m) (gmn_mosek.c:152-160). The reference solves
// it with MOSEK's interior point method; here every problem runs ADMM on the
// split U_m = Q_m, V_m = W - PT_m(Q_m) in the box C = {0 <= X <= I}:
//   x-step (closed form; PT_m is self-adjoint and an involution)
//     a = U - Yh, b = V - Zh,  W = (sum_m PT_m(a_m) + b_m - 2 rho / sigma) / 3,
//     Q_m = (a_m + PT_m(W - b_m)) / 2;
//   z-step  U_m = P_C(Q_m + Yh_m),  V_m = P_C(W - PT_m(Q_m) + Zh_m);
//   dual    Yh_m += Q_m - U_m,  Zh_m += W - PT_m(Q_m) - V_m.
// Every check_every iterations an FP64 kernel certifies each problem: with
// Z_m = sigma Zh_m shifted onto sum_m Z_m = -rho,
//     d = -sum_m [Tr (PT_m Z_m)_+ + Tr (Z_m)_+]  <=  min  <=  Re Tr(rho W),
// and a problem is done when |Re Tr(rho W) - d| <= gap_tol and W, Q violate
// the box constraints by at most feas_tol (eigenvalues). Its GMN is
// -(Re Tr(rho W) + d) / 2.
//
// GB300 mapping: P_C needs the spectrum of an 8x8 Hermitian matrix; eight
// lanes share one problem, lane c holding column c, and diagonalise by a
// parallel cyclic Jacobi (round-robin: 4 disjoint rotations per round, 7
// rounds per sweep) with column exchanges by warp shuffles. W and Q are staged
// in shared memory for the partial-transpose gathers; the ADMM state streams
// from global memory. Compute-bound on the FP32 pipes.
#include "mipt_gb300.h"

#include "common.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace mg
{
int api_fail(int code, const std::string &what);
int api_cuda_fail(cudaError_t e, const char *what);
} // namespace mg

using namespace mg;

namespace
{
constexpr int kLanes = 8;
// ADMM penalty when the config gives none: on the config-4 state mix, 0.1
// certifies 95.0 % of states to a 1e-6 gap within 3000 iterations in 118
// iterations on average, against 91.9 % and 136 at 1.0.
constexpr double kDefaultSigma = 0.1;
constexpr int kThreads = 256;
constexpr int kProbPerBlock = kThreads / kLanes;

template <typename Real> struct C2
{
    Real re, im;
};
template <typename Real> __device__ __forceinline__ C2<Real> cadd(C2<Real> a, C2<Real> b) { return {a.re + b.re, a.im + b.im}; }
template <typename Real> __device__ __forceinline__ C2<Real> csub(C2<Real> a, C2<Real> b) { return {a.re - b.re, a.im - b.im}; }
template <typename Real> __device__ __forceinline__ C2<Real> cscale(C2<Real> a, Real s) { return {a.re * s, a.im * s}; }
template <typename Real> __device__ __forceinline__ C2<Real> cmul(C2<Real> a, C2<Real> b)
{
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename Real> __device__ __forceinline__ C2<Real> cconj(C2<Real> a) { return {a.re, -a.im}; }

__host__ __device__ constexpr int rr_partner(int r, int l)
{
    // Round r of the 8-player round robin: (r, 7) and pairs summing to 2r mod 7.
    return l == 7 ? r : (l == r ? 7 : ((2 * r - l) % 7 + 7) % 7);
}

template <typename Real> __device__ __forceinline__ C2<Real> pick(const C2<Real> (&v)[8], int i)
{
    C2<Real> out = v[0];
#pragma unroll
    for (int k = 1; k < 8; ++k)
        if (i == k) out = v[k];
    return out;
}

template <typename Real> __device__ __forceinline__ Real shfl(Real v, int src, unsigned mask)
{
    return __shfl_sync(mask, v, src);
}

// Hermitian 8x8 Jacobi on an 8-lane group: lane c holds column c of A (and,
// with kVec, column c of the eigenvector matrix, starting from I). On return
// A is diagonal to rounding; lane c's eigenvalue is Re A[c][c].
template <typename Real, bool kVec>
__device__ void jacobi8(C2<Real> (&A)[8], C2<Real> (&V)[8], int c, int gbase, unsigned gmask, int sweeps)
{
    for (int sw = 0; sw < sweeps; ++sw)
    {
#pragma unroll
        for (int r = 0; r < 7; ++r)
        {
            const int partner = rr_partner(r, c);
            const Real a_self = pick(A, c).re;
            const Real a_part = shfl(a_self, gbase + partner, gmask);
            // Lane p (= min of the pair) forms the rotation from A[p][p],
            // A[q][q] and A[p][q] = conj(A[q][p]).
            Real cs = 1, sn = 0, er = 1, ei = 0;
            if (c < partner)
            {
                // |b| by hypot (no subnormal squares: e = b / |b| must be a unit
                // phase or the rotation is not unitary); rotations whose
                // off-diagonal is negligible beside the diagonal pair are skipped.
                const C2<Real> b = cconj(pick(A, partner));
                const Real ab = hypot(b.re, b.im);
                const Real eps = sizeof(Real) == 4 ? Real(6e-8) : Real(1.2e-16);
                const Real tiny = sizeof(Real) == 4 ? Real(1e-18) : Real(1e-30);
                if (ab > tiny && ab > eps * (fabs(a_self) + fabs(a_part)))
                {
                    er = b.re / ab;
                    ei = b.im / ab;
                    const Real tau = (a_self - a_part) / (Real(2) * ab);
                    const Real t = (tau >= Real(0) ? Real(1) : Real(-1)) / (fabs(tau) + sqrt(Real(1) + tau * tau));
                    cs = Real(1) / sqrt(Real(1) + t * t);
                    sn = t * cs;
                }
            }
            // Row update with all four rotations of the round (pair k's p is
            // known at compile time), and this lane's own rotation on the way.
            Real mcs = cs, msn = sn, mer = er, mei = ei;
#pragma unroll
            for (int l = 0; l < 8; ++l)
            {
                const int q = rr_partner(r, l);
                if (!(l < q)) continue;
                const Real kcs = shfl(cs, gbase + l, gmask), ksn = shfl(sn, gbase + l, gmask);
                const Real ker = shfl(er, gbase + l, gmask), kei = shfl(ei, gbase + l, gmask);
                if (c == q)
                {
                    mcs = kcs;
                    msn = ksn;
                    mer = ker;
                    mei = kei;
                }
                // G = [[cs, -sn], [conj(e) sn, conj(e) cs]]; rows: G^H A.
                const C2<Real> ce{ker, -kei};
                const C2<Real> g10 = cscale(ce, ksn), g11 = cscale(ce, kcs);
                const C2<Real> rp = A[l], rq = A[q];
                A[l] = cadd(cscale(rp, kcs), cmul(cconj(g10), rq));
                A[q] = cadd(cscale(rp, -ksn), cmul(cconj(g11), rq));
            }
            // Column update: exchange columns with the partner.
            const C2<Real> ce{mer, -mei};
            const C2<Real> g10 = cscale(ce, msn), g11 = cscale(ce, mcs);
            const bool is_p = c < partner;
#pragma unroll
            for (int i = 0; i < 8; ++i)
            {
                C2<Real> o;
                o.re = shfl(A[i].re, gbase + partner, gmask);
                o.im = shfl(A[i].im, gbase + partner, gmask);
                A[i] = is_p ? cadd(cscale(A[i], mcs), cmul(o, g10)) : cadd(cscale(o, -msn), cmul(A[i], g11));
                if (kVec)
                {
                    C2<Real> v;
                    v.re = shfl(V[i].re, gbase + partner, gmask);
                    v.im = shfl(V[i].im, gbase + partner, gmask);
                    V[i] = is_p ? cadd(cscale(V[i], mcs), cmul(v, g10)) : cadd(cscale(v, -msn), cmul(V[i], g11));
                }
            }
        }
    }
}

// X <- P_C(X) (eigenvalues clipped to [0, 1]) for the group's matrix; lane c
// passes and receives column c. The reconstruction V clip(L) V^H rounds
// (r, c) and (c, r) differently, so the result is made exactly Hermitian
// through the group's 64-entry shared scratch: an anti-Hermitian residue
// would otherwise accumulate in the ADMM duals, iteration after iteration.
template <typename Real>
__device__ void project_box(C2<Real> (&X)[8], int c, int gbase, unsigned gmask, C2<Real> *scratch)
{
    C2<Real> V[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) V[i] = C2<Real>{i == c ? Real(1) : Real(0), Real(0)};
    jacobi8<Real, true>(X, V, c, gbase, gmask, sizeof(Real) == 4 ? 6 : 7);
    const Real lam = fmin(fmax(pick(X, c).re, Real(0)), Real(1));
    C2<Real> R[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) R[i] = C2<Real>{0, 0};
#pragma unroll
    for (int k = 0; k < 8; ++k)
    {
        const Real lk = shfl(lam, gbase + k, gmask);
        C2<Real> vk[8];
#pragma unroll
        for (int i = 0; i < 8; ++i)
        {
            vk[i].re = shfl(V[i].re, gbase + k, gmask);
            vk[i].im = shfl(V[i].im, gbase + k, gmask);
        }
        const C2<Real> coef = cscale(cconj(pick(vk, c)), lk);
#pragma unroll
        for (int i = 0; i < 8; ++i) R[i] = cadd(R[i], cmul(vk[i], coef));
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) scratch[c * 8 + i] = R[i];
    __syncwarp(gmask);
#pragma unroll
    for (int i = 0; i < 8; ++i)
    {
        const C2<Real> t = scratch[i * 8 + c]; // R[c][i]
        X[i] = cscale(cadd(R[i], cconj(t)), Real(0.5));
    }
    __syncwarp(gmask);
}

__device__ __forceinline__ int pt_src(int r, int c, int m)
{
    // Column-major flat index (col * 8 + row) of the entry PT_m reads for (r, c).
    const int sr = (r & ~m) | (c & m), sc = (c & ~m) | (r & m);
    return sc * 8 + sr;
}

struct GmnArrays
{
    int count;
    const void *rho;   // [P][64] Real2, column-major
    void *U, *V, *Yh, *Zh; // [P][3][64]
    void *W, *Q;       // [P][64], [P][3][64] (latest x-step)
    const double *sigma;
    const int *done;
    float *res; // FP32 residual of each state's last iteration
};

template <typename Real>
__global__ void __launch_bounds__(kThreads) k_gmn_iterate(GmnArrays a, int iters)
{
    // Per problem: W (64), Q_1..3 (192), projection scratch (64) -- dynamic.
    extern __shared__ __align__(16) unsigned char gmn_smem[];
    auto sW = reinterpret_cast<C2<Real>(*)[64]>(gmn_smem);
    auto sQ = reinterpret_cast<C2<Real>(*)[3][64]>(gmn_smem + sizeof(C2<Real>) * 64 * kProbPerBlock);
    auto sR = reinterpret_cast<C2<Real>(*)[64]>(gmn_smem + sizeof(C2<Real>) * 256 * kProbPerBlock);
    const int g = threadIdx.x / kLanes, c = threadIdx.x % kLanes;
    const int prob = blockIdx.x * kProbPerBlock + g;
    const int lane = threadIdx.x & 31, gbase = lane & ~7;
    const unsigned gmask = 0xFFu << gbase;
    if (prob >= a.count || a.done[prob]) return; // whole 8-lane groups leave together
    const Real sigma = static_cast<Real>(a.sigma[prob]);
    const C2<Real> *rho = static_cast<const C2<Real> *>(a.rho) + static_cast<std::size_t>(prob) * 64;
    C2<Real> *U = static_cast<C2<Real> *>(a.U) + static_cast<std::size_t>(prob) * 192;
    C2<Real> *V = static_cast<C2<Real> *>(a.V) + static_cast<std::size_t>(prob) * 192;
    C2<Real> *Yh = static_cast<C2<Real> *>(a.Yh) + static_cast<std::size_t>(prob) * 192;
    C2<Real> *Zh = static_cast<C2<Real> *>(a.Zh) + static_cast<std::size_t>(prob) * 192;
    C2<Real> *Wg = static_cast<C2<Real> *>(a.W) + static_cast<std::size_t>(prob) * 64;
    C2<Real> *Qg = static_cast<C2<Real> *>(a.Q) + static_cast<std::size_t>(prob) * 192;
    const Real two_over_sigma = Real(2) / sigma;
    // Residual of the launch's last iteration: |dYh|^2 + |dZh|^2 (primal) plus
    // sigma^2 (|dU|^2 + |dV|^2) (dual), over this lane's column.
    float resid = 0.f;
    for (int it = 0; it < iters; ++it)
    {
        const bool last = it + 1 == iters;
        // x-step: W column c.
#pragma unroll
        for (int r = 0; r < 8; ++r)
        {
            C2<Real> w = cscale(rho[c * 8 + r], -two_over_sigma);
#pragma unroll
            for (int m = 1; m <= 3; ++m)
            {
                const int s = pt_src(r, c, m);
                const int o = (m - 1) * 64;
                w = cadd(w, csub(U[o + s], Yh[o + s]));           // PT_m(a_m)
                w = cadd(w, csub(V[o + c * 8 + r], Zh[o + c * 8 + r])); // b_m
            }
            sW[g][c * 8 + r] = cscale(w, Real(1) / Real(3));
        }
        __syncwarp(gmask);
        // Q_m = (a_m + PT_m(W - b_m)) / 2.
#pragma unroll
        for (int m = 1; m <= 3; ++m)
        {
            const int o = (m - 1) * 64;
#pragma unroll
            for (int r = 0; r < 8; ++r)
            {
                const int s = pt_src(r, c, m);
                const C2<Real> am = csub(U[o + c * 8 + r], Yh[o + c * 8 + r]);
                const C2<Real> wb = csub(sW[g][s], csub(V[o + s], Zh[o + s]));
                sQ[g][m - 1][c * 8 + r] = cscale(cadd(am, wb), Real(0.5));
            }
        }
        __syncwarp(gmask);
        // Every lane has read its old U, V, Yh, Zh entries: new values may be written.
#pragma unroll 1
        for (int m = 1; m <= 3; ++m)
        {
            const int o = (m - 1) * 64;
            C2<Real> X[8];
            // U_m = P_C(Q_m + Yh_m); Yh_m += Q_m - U_m.
#pragma unroll
            for (int r = 0; r < 8; ++r) X[r] = cadd(sQ[g][m - 1][c * 8 + r], Yh[o + c * 8 + r]);
            C2<Real> X0[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) X0[r] = X[r];
            project_box(X, c, gbase, gmask, sR[g]);
#pragma unroll
            for (int r = 0; r < 8; ++r)
            {
                if (last)
                {
                    const C2<Real> dy = csub(csub(X0[r], X[r]), Yh[o + c * 8 + r]);
                    const C2<Real> du = csub(X[r], U[o + c * 8 + r]);
                    resid += float(dy.re * dy.re + dy.im * dy.im) +
                             float(sigma * sigma * (du.re * du.re + du.im * du.im));
                }
                U[o + c * 8 + r] = X[r];
                Yh[o + c * 8 + r] = csub(X0[r], X[r]);
            }
            // V_m = P_C(W - PT_m(Q_m) + Zh_m); Zh_m += W - PT_m(Q_m) - V_m.
#pragma unroll
            for (int r = 0; r < 8; ++r)
            {
                X[r] = cadd(csub(sW[g][c * 8 + r], sQ[g][m - 1][pt_src(r, c, m)]), Zh[o + c * 8 + r]);
                X0[r] = X[r];
            }
            project_box(X, c, gbase, gmask, sR[g]);
#pragma unroll
            for (int r = 0; r < 8; ++r)
            {
                if (last)
                {
                    const C2<Real> dz = csub(csub(X0[r], X[r]), Zh[o + c * 8 + r]);
                    const C2<Real> dv = csub(X[r], V[o + c * 8 + r]);
                    resid += float(dz.re * dz.re + dz.im * dz.im) +
                             float(sigma * sigma * (dv.re * dv.re + dv.im * dv.im));
                }
                V[o + c * 8 + r] = X[r];
                Zh[o + c * 8 + r] = csub(X0[r], X[r]);
            }
        }
        __syncwarp(gmask);
    }
#pragma unroll
    for (int r = 0; r < 8; ++r)
    {
        Wg[c * 8 + r] = sW[g][c * 8 + r];
#pragma unroll
        for (int m = 0; m < 3; ++m) Qg[m * 64 + c * 8 + r] = sQ[g][m][c * 8 + r];
    }
    for (int off = 4; off > 0; off /= 2) resid += __shfl_xor_sync(gmask, resid, off);
    if (c == 0) a.res[prob] = sqrtf(resid);
}

// Sum over the 8 lanes of a group.
__device__ __forceinline__ double group_sum(double v, unsigned gmask)
{
    for (int off = 4; off > 0; off /= 2) v += __shfl_xor_sync(gmask, v, off);
    return v;
}
__device__ __forceinline__ double group_max(double v, unsigned gmask)
{
    for (int off = 4; off > 0; off /= 2) v = fmax(v, __shfl_xor_sync(gmask, v, off));
    return v;
}

struct GmnCheck
{
    int count;
    const void *rho; // Real2
    const double2 *rho64;
    const void *W, *Q, *Zh;
    const double *sigma;
    int *done;
    int *iters;
    int iter_now;
    double gap_tol, feas_tol;
    double *primal, *dual, *gap, *infeas, *gmn;
    int *remaining;
    // FP64 certificates are computed for candidates only: states whose FP32
    // residual is at most cand_tol and whose back-off has expired (after a
    // failed candidate check the next one waits 2, then 4 check intervals).
    const float *res;
    float cand_tol;
    int *next_check, *backoff;
    int check_every;
    int force; // certify every remaining state (final pass)
};

// Spectrum of the group's Hermitian matrix (FP64), lane c returns eigenvalue c.
__device__ double eigval8(C2<double> (&A)[8], int c, int gbase, unsigned gmask)
{
    C2<double> V[8];
    jacobi8<double, false>(A, V, c, gbase, gmask, 7);
    return pick(A, c).re;
}

template <typename Real> __global__ void __launch_bounds__(kThreads) k_gmn_check(GmnCheck k)
{
    const int g = threadIdx.x / kLanes, c = threadIdx.x % kLanes;
    const int prob = blockIdx.x * kProbPerBlock + g;
    const int lane = threadIdx.x & 31, gbase = lane & ~7;
    const unsigned gmask = 0xFFu << gbase;
    if (prob >= k.count || k.done[prob]) return;
    if (!k.force && (k.res[prob] > k.cand_tol || k.iter_now < k.next_check[prob]))
    {
        if (c == 0) atomicAdd(k.remaining, 1);
        return;
    }
    const double sigma = k.sigma[prob];
    const double2 *rho = k.rho64 + static_cast<std::size_t>(prob) * 64;
    const C2<Real> *W = static_cast<const C2<Real> *>(k.W) + static_cast<std::size_t>(prob) * 64;
    const C2<Real> *Q = static_cast<const C2<Real> *>(k.Q) + static_cast<std::size_t>(prob) * 192;
    const C2<Real> *Zh = static_cast<const C2<Real> *>(k.Zh) + static_cast<std::size_t>(prob) * 192;
    auto ld = [](const C2<Real> &x) { return C2<double>{static_cast<double>(x.re), static_cast<double>(x.im)}; };
    // Primal Re Tr(rho W) = sum_{r,c} Re(rho[r][c] W[c][r]).
    double p = 0.0;
#pragma unroll
    for (int r = 0; r < 8; ++r)
    {
        const double2 a = rho[c * 8 + r];
        const C2<double> w = ld(W[r * 8 + c]);
        p += a.x * w.re - a.y * w.im;
    }
    p = group_sum(p, gmask);
    // Dual: Z_m = sigma Zh_m - (sigma sum Zh + rho) / 3 at any entry.
    auto zshift = [&](int m, int idx) {
        C2<double> s{rho[idx].x, rho[idx].y};
        for (int mm = 0; mm < 3; ++mm) s = cadd(s, cscale(ld(Zh[mm * 64 + idx]), sigma));
        return csub(cscale(ld(Zh[m * 64 + idx]), sigma), cscale(s, 1.0 / 3.0));
    };
    double d = 0.0, feas = 0.0;
    for (int m = 1; m <= 3; ++m)
    {
        C2<double> A[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) A[r] = zshift(m - 1, c * 8 + r);
        double l = eigval8(A, c, gbase, gmask);
        d -= group_sum(fmax(l, 0.0), gmask);
#pragma unroll
        for (int r = 0; r < 8; ++r) A[r] = zshift(m - 1, pt_src(r, c, m));
        l = eigval8(A, c, gbase, gmask);
        d -= group_sum(fmax(l, 0.0), gmask);
        // Box violations of Q_m and W - PT_m(Q_m).
#pragma unroll
        for (int r = 0; r < 8; ++r) A[r] = ld(Q[(m - 1) * 64 + c * 8 + r]);
        l = eigval8(A, c, gbase, gmask);
        feas = fmax(feas, fmax(-l, l - 1.0));
#pragma unroll
        for (int r = 0; r < 8; ++r) A[r] = csub(ld(W[c * 8 + r]), ld(Q[(m - 1) * 64 + pt_src(r, c, m)]));
        l = eigval8(A, c, gbase, gmask);
        feas = fmax(feas, fmax(-l, l - 1.0));
    }
    feas = group_max(feas, gmask);
    if (c == 0)
    {
        const double gp = p - d;
        k.primal[prob] = p;
        k.dual[prob] = d;
        k.gap[prob] = gp;
        k.infeas[prob] = feas;
        const double v = -0.5 * (p + d);
        k.gmn[prob] = v > 1e-8 ? v : 0.0;
        k.iters[prob] = k.iter_now;
        if (fabs(gp) <= k.gap_tol && feas <= k.feas_tol)
        {
            k.done[prob] = 1;
        }
        else
        {
            atomicAdd(k.remaining, 1);
            const int b = min(2 * max(k.backoff[prob], 1), 4);
            k.backoff[prob] = b;
            k.next_check[prob] = k.iter_now + b * k.check_every;
        }
    }
}

// rho (host layout: row-major re/im, 128 doubles) -> column-major Real2 and
// double2 copies; state zeroed (cold start).
template <typename Real>
__global__ void k_gmn_load(int count, const double *rho_in, C2<Real> *rho, double2 *rho64)
{
    const std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<std::size_t>(count) * 64) return;
    const std::size_t p = i / 64;
    const int e = static_cast<int>(i % 64), col = e / 8, row = e % 8;
    const double *src = rho_in + p * 128 + 2 * (row * 8 + col);
    // Hermitian part, as the reference symmetrises its input (python/gmn.py:276).
    const double *tr = rho_in + p * 128 + 2 * (col * 8 + row);
    const double re = 0.5 * (src[0] + tr[0]), im = 0.5 * (src[1] - tr[1]);
    rho[i] = C2<Real>{static_cast<Real>(re), static_cast<Real>(im)};
    rho64[i] = make_double2(re, im);
}

// Warm start from a solution guess (host layout, 7 matrices per problem:
// W, Q_1..3, Z_1..3): U_m = P_C-free Q_m, V_m = W - PT_m(Q_m),
// Yh_m = PT_m(Z_m) / sigma, Zh_m = Z_m / sigma.
template <typename Real>
__global__ void k_gmn_warm(int count, const float *guess, const double *sigma, C2<Real> *U, C2<Real> *V, C2<Real> *Yh,
                           C2<Real> *Zh)
{
    const std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<std::size_t>(count) * 64) return;
    const std::size_t p = i / 64;
    const int e = static_cast<int>(i % 64), col = e / 8, row = e % 8;
    const float *G = guess + p * 7 * 128;
    const Real inv = static_cast<Real>(1.0 / sigma[p]);
    auto at = [&](int mat, int r, int cc) {
        // Hermitian part of the guess at (r, cc).
        const float *a = G + mat * 128 + 2 * (r * 8 + cc);
        const float *b = G + mat * 128 + 2 * (cc * 8 + r);
        return C2<Real>{static_cast<Real>(0.5f * (a[0] + b[0])), static_cast<Real>(0.5f * (a[1] - b[1]))};
    };
    for (int m = 1; m <= 3; ++m)
    {
        const int sr = (row & ~m) | (col & m), sc = (col & ~m) | (row & m);
        const std::size_t o = p * 192 + (m - 1) * 64 + e;
        U[o] = at(m, row, col);
        V[o] = csub(at(0, row, col), at(m, sr, sc));
        Yh[o] = cscale(at(3 + m, sr, sc), inv);
        Zh[o] = cscale(at(3 + m, row, col), inv);
    }
}

struct DevMem
{
    void *p = nullptr;
    std::size_t bytes = 0;
    ~DevMem()
    {
        if (p) cudaFree(p);
    }
    cudaError_t ensure(std::size_t need)
    {
        if (need <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, need);
        if (e == cudaSuccess) bytes = need;
        return e;
    }
};

#define GMN_CUDA(x)                                                                                              \
    do                                                                                                           \
    {                                                                                                            \
        cudaError_t e_ = (x);                                                                                    \
        if (e_ != cudaSuccess) return api_cuda_fail(e_, #x);                                                     \
    } while (0)

template <typename Real>
int gmn_solve(const mipt_gb300_gmn_config &cfg, const double *h_rho, int count, const float *h_guess, double *h_gmn,
              double *h_gap, int *h_iters, double *h_solution, const double *h_sigma = nullptr)
{
    const std::size_t P = static_cast<std::size_t>(count), M = sizeof(C2<Real>) * 64;
    DevMem rho_in, rho, rho64, U, V, Yh, Zh, W, Q, sig, done, iters, outs, rem, guess, res, nextc, boff;
    GMN_CUDA(rho_in.ensure(P * 128 * sizeof(double)));
    GMN_CUDA(rho.ensure(P * M));
    GMN_CUDA(rho64.ensure(P * 64 * sizeof(double2)));
    for (DevMem *b : {&U, &V, &Yh, &Zh, &Q}) GMN_CUDA(b->ensure(P * 3 * M));
    GMN_CUDA(W.ensure(P * M));
    GMN_CUDA(sig.ensure(P * sizeof(double)));
    GMN_CUDA(done.ensure(P * sizeof(int)));
    GMN_CUDA(iters.ensure(P * sizeof(int)));
    GMN_CUDA(outs.ensure(P * 5 * sizeof(double)));
    GMN_CUDA(rem.ensure(sizeof(int)));
    GMN_CUDA(res.ensure(P * sizeof(float)));
    GMN_CUDA(nextc.ensure(P * sizeof(int)));
    GMN_CUDA(boff.ensure(P * sizeof(int)));
    GMN_CUDA(cudaMemset(nextc.p, 0, P * sizeof(int)));
    GMN_CUDA(cudaMemset(boff.p, 0, P * sizeof(int)));
    GMN_CUDA(cudaMemcpy(rho_in.p, h_rho, P * 128 * sizeof(double), cudaMemcpyHostToDevice));
    const int lb = static_cast<int>((P * 64 + 255) / 256);
    k_gmn_load<Real><<<lb, 256>>>(count, static_cast<const double *>(rho_in.p), static_cast<C2<Real> *>(rho.p),
                                  static_cast<double2 *>(rho64.p));
    std::vector<double> s(P, cfg.sigma > 0 ? cfg.sigma : kDefaultSigma);
    if (h_sigma)
        for (std::size_t i = 0; i < P; ++i) s[i] = h_sigma[i];
    GMN_CUDA(cudaMemcpy(sig.p, s.data(), P * sizeof(double), cudaMemcpyHostToDevice));
    GMN_CUDA(cudaMemset(done.p, 0, P * sizeof(int)));
    GMN_CUDA(cudaMemset(iters.p, 0, P * sizeof(int)));
    for (DevMem *b : {&U, &V, &Yh, &Zh, &Q, &W}) GMN_CUDA(cudaMemset(b->p, 0, b->bytes));
    if (h_guess)
    {
        GMN_CUDA(guess.ensure(P * 7 * 128 * sizeof(float)));
        GMN_CUDA(cudaMemcpy(guess.p, h_guess, P * 7 * 128 * sizeof(float), cudaMemcpyHostToDevice));
        k_gmn_warm<Real><<<lb, 256>>>(count, static_cast<const float *>(guess.p), static_cast<const double *>(sig.p),
                                      static_cast<C2<Real> *>(U.p), static_cast<C2<Real> *>(V.p),
                                      static_cast<C2<Real> *>(Yh.p), static_cast<C2<Real> *>(Zh.p));
    }
    GMN_CUDA(cudaGetLastError());
    GmnArrays a{count, rho.p, U.p, V.p, Yh.p, Zh.p, W.p, Q.p, static_cast<const double *>(sig.p),
                static_cast<const int *>(done.p), static_cast<float *>(res.p)};
    double *o = static_cast<double *>(outs.p);
    GmnCheck k{count, rho.p, static_cast<const double2 *>(rho64.p), W.p, Q.p, Zh.p,
               static_cast<const double *>(sig.p), static_cast<int *>(done.p), static_cast<int *>(iters.p), 0,
               cfg.gap_tol, cfg.feas_tol, o, o + P, o + 2 * P, o + 3 * P, o + 4 * P, static_cast<int *>(rem.p),
               static_cast<const float *>(res.p), static_cast<float>(30.0 * std::max(cfg.gap_tol, cfg.feas_tol)),
               static_cast<int *>(nextc.p), static_cast<int *>(boff.p), std::max(1, cfg.check_every), 0};
    const int blocks = static_cast<int>((P + kProbPerBlock - 1) / kProbPerBlock);
    const int every = std::max(1, cfg.check_every);
    int it = 0;
    const std::size_t smem = sizeof(C2<Real>) * 320 * kProbPerBlock;
    GMN_CUDA(cudaFuncSetAttribute(k_gmn_iterate<Real>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem)));
    while (it < cfg.max_iter)
    {
        const int n = std::min(every, cfg.max_iter - it);
        k_gmn_iterate<Real><<<blocks, kThreads, smem>>>(a, n);
        it += n;
        GMN_CUDA(cudaMemset(rem.p, 0, sizeof(int)));
        k.iter_now = it;
        k_gmn_check<Real><<<blocks, kThreads>>>(k);
        GMN_CUDA(cudaGetLastError());
        int remaining = 0;
        GMN_CUDA(cudaMemcpy(&remaining, rem.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (remaining == 0) break;
        if (it >= cfg.max_iter)
        {
            // Last pass: bounds for every state still uncertified.
            k.force = 1;
            k_gmn_check<Real><<<blocks, kThreads>>>(k);
            GMN_CUDA(cudaGetLastError());
        }
    }
    std::vector<double> hres(P * 5);
    GMN_CUDA(cudaMemcpy(hres.data(), outs.p, hres.size() * sizeof(double), cudaMemcpyDeviceToHost));
    std::vector<int> its(P), dn(P);
    GMN_CUDA(cudaMemcpy(its.data(), iters.p, P * sizeof(int), cudaMemcpyDeviceToHost));
    GMN_CUDA(cudaMemcpy(dn.data(), done.p, P * sizeof(int), cudaMemcpyDeviceToHost));
    for (std::size_t i = 0; i < P; ++i)
    {
        if (h_gmn) h_gmn[i] = hres[4 * P + i];
        if (h_gap) h_gap[i] = hres[2 * P + i];
        if (h_iters) h_iters[i] = dn[i] ? its[i] : -its[i];
    }
    if (h_solution)
    {
        // W, Q_1..3, Z_1..3 in host layout (row-major re/im), Z = sigma Zh.
        std::vector<C2<Real>> w(P * 64), q(P * 192), z(P * 192);
        GMN_CUDA(cudaMemcpy(w.data(), W.p, P * M, cudaMemcpyDeviceToHost));
        GMN_CUDA(cudaMemcpy(q.data(), Q.p, P * 3 * M, cudaMemcpyDeviceToHost));
        GMN_CUDA(cudaMemcpy(z.data(), Zh.p, P * 3 * M, cudaMemcpyDeviceToHost));
        for (std::size_t i = 0; i < P; ++i)
            for (int mat = 0; mat < 7; ++mat)
                for (int row = 0; row < 8; ++row)
                    for (int col = 0; col < 8; ++col)
                    {
                        C2<Real> v = mat == 0 ? w[i * 64 + col * 8 + row]
                                     : mat <= 3 ? q[i * 192 + (mat - 1) * 64 + col * 8 + row]
                                                : z[i * 192 + (mat - 4) * 64 + col * 8 + row];
                        const double sc = mat >= 4 ? s[i] : 1.0;
                        double *dst = h_solution + (i * 7 + mat) * 128 + 2 * (row * 8 + col);
                        dst[0] = sc * static_cast<double>(v.re);
                        dst[1] = sc * static_cast<double>(v.im);
                    }
    }
    return 0;
}
} // namespace

namespace
{
// Negativity of every single-qubit cut of 8x8 states: 8-lane group g handles
// (state g / 3, cut g % 3). Lane c loads column c of the partial transpose on
// qubit m (entry (r, c) from (r & ~mask | c & mask, c & ~mask | r & mask),
// mask = 1 << m), the FP64 Jacobi diagonalises it, and
// N = (sum_c |lambda_c| - 1) / 2, values in (-1e-10, 0) set to 0
// (cpp/include/mipt/analysis/cut_negativity.hpp:139-200).
__global__ void __launch_bounds__(kThreads) k_cut_negativity(int count, const double *__restrict__ rho,
                                                              double *__restrict__ neg)
{
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = tid / kLanes, c = tid % kLanes;
    const int gbase = (threadIdx.x % 32) / kLanes * kLanes;
    const unsigned gmask = 0xffu << gbase;
    const bool live = g < 3 * count;
    const int st = live ? g / 3 : 0, mask = 1 << (live ? g % 3 : 0);
    const double *R = rho + static_cast<std::size_t>(st) * 128;
    C2<double> A[8], V[8];
#pragma unroll
    for (int r = 0; r < 8; ++r)
    {
        const int sr = (r & ~mask) | (c & mask), sc = (c & ~mask) | (r & mask);
        A[r] = live ? C2<double>{R[2 * (sr * 8 + sc)], R[2 * (sr * 8 + sc) + 1]} : C2<double>{r == c ? 1.0 : 0.0, 0.0};
        V[r] = C2<double>{0.0, 0.0};
    }
    jacobi8<double, false>(A, V, c, gbase, gmask, 10);
    double t = fabs(pick(A, c).re);
#pragma unroll
    for (int off = 4; off > 0; off >>= 1) t += __shfl_xor_sync(gmask, t, off);
    if (live && c == 0)
    {
        double n = 0.5 * (t - 1.0);
        if (n < 0.0 && n > -1e-10) n = 0.0;
        neg[g] = n;
    }
}
} // namespace

extern "C" int mipt_gb300_cut_negativities(const double *rho, int count, double *negativity)
{
    if (!rho || !negativity || count <= 0) return api_fail(MIPT_GB300_E_INVALID, "bad negativity arguments");
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return api_fail(MIPT_GB300_E_NODEVICE, "no CUDA device");
    const std::size_t P = static_cast<std::size_t>(count);
    DevMem d_rho, d_neg;
    GMN_CUDA(d_rho.ensure(P * 128 * sizeof(double)));
    GMN_CUDA(d_neg.ensure(P * 3 * sizeof(double)));
    GMN_CUDA(cudaMemcpy(d_rho.p, rho, P * 128 * sizeof(double), cudaMemcpyHostToDevice));
    const std::size_t threads = P * 3 * kLanes;
    k_cut_negativity<<<static_cast<unsigned>((threads + kThreads - 1) / kThreads), kThreads>>>(
        count, static_cast<const double *>(d_rho.p), static_cast<double *>(d_neg.p));
    GMN_CUDA(cudaGetLastError());
    GMN_CUDA(cudaMemcpy(negativity, d_neg.p, P * 3 * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int mipt_gb300_gmn_solve_sigma(const mipt_gb300_gmn_config *cfg, const double *rho, int count,
                                          const double *sigma, const float *warm_start, double *gmn, double *gap,
                                          int *iterations, double *solution)
{
    if (!cfg || !rho || !sigma || count <= 0 || cfg->max_iter <= 0 || !(cfg->gap_tol > 0) || !(cfg->feas_tol > 0))
        return api_fail(MIPT_GB300_E_INVALID, "bad GMN arguments");
    for (int i = 0; i < count; ++i)
        if (!(sigma[i] > 0) || !std::isfinite(sigma[i]))
            return api_fail(MIPT_GB300_E_INVALID, "per-state ADMM penalties must be positive and finite");
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return api_fail(MIPT_GB300_E_NODEVICE, "no CUDA device");
    return cfg->fp64 ? gmn_solve<double>(*cfg, rho, count, warm_start, gmn, gap, iterations, solution, sigma)
                     : gmn_solve<float>(*cfg, rho, count, warm_start, gmn, gap, iterations, solution, sigma);
}

extern "C" int mipt_gb300_gmn_solve(const mipt_gb300_gmn_config *cfg, const double *rho, int count,
                                    const float *warm_start, double *gmn, double *gap, int *iterations,
                                    double *solution)
{
    if (!cfg || !rho || count <= 0 || cfg->max_iter <= 0 || !(cfg->gap_tol > 0) || !(cfg->feas_tol > 0))
        return api_fail(MIPT_GB300_E_INVALID, "bad GMN arguments");
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return api_fail(MIPT_GB300_E_NODEVICE, "no CUDA device");
    return cfg->fp64 ? gmn_solve<double>(*cfg, rho, count, warm_start, gmn, gap, iterations, solution)
                     : gmn_solve<float>(*cfg, rho, count, warm_start, gmn, gap, iterations, solution);
}
