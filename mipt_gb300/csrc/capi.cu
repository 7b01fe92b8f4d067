// C ABI of the GB300 trajectory path: reference-compatible observables,
// the single-state engine, and the batched trajectory runner.
#include "mipt_gb300.h"

#include "engine.cuh"
#include "observables.cuh"
#include "sampler.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <complex>
#include <thread>
#include <tuple>
#include <mutex>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

using namespace mg;

namespace
{
thread_local std::string g_error;
thread_local std::string g_measure_error;

int fail(int code, const std::string &what)
{
    g_error = what;
    return code == 0 ? MIPT_GB300_E_INTERNAL : code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    g_error = std::string(what) + ": " + cudaGetErrorString(e);
    return static_cast<int>(e);
}

#define MG_CUDA(expr)                                                                                            \
    do                                                                                                           \
    {                                                                                                            \
        cudaError_t e_ = (expr);                                                                                 \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);                                                      \
    } while (0)

// Growable device buffer.
struct DevBuf
{
    void *p = nullptr;
    std::size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
    cudaError_t ensure(std::size_t need)
    {
        if (need <= bytes && p) return cudaSuccess;
        if (p)
        {
            cudaFree(p);
            p = nullptr;
            bytes = 0;
        }
        cudaError_t e = cudaMalloc(&p, std::max<std::size_t>(need, 256));
        if (e == cudaSuccess) bytes = std::max<std::size_t>(need, 256);
        return e;
    }
    template <typename T> T *as() { return static_cast<T *>(p); }
};

struct PinnedBuf
{
    void *p = nullptr;
    std::size_t bytes = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf &) = delete;
    PinnedBuf &operator=(const PinnedBuf &) = delete;
    ~PinnedBuf()
    {
        if (p) cudaFreeHost(p);
    }
    cudaError_t ensure(std::size_t need)
    {
        if (need <= bytes && p) return cudaSuccess;
        if (p)
        {
            cudaFreeHost(p);
            p = nullptr;
            bytes = 0;
        }
        cudaError_t e = cudaMallocHost(&p, std::max<std::size_t>(need, 256));
        if (e == cudaSuccess) bytes = std::max<std::size_t>(need, 256);
        return e;
    }
    template <typename T> T *as() { return static_cast<T *>(p); }
};

// Pinned staging for the small host tables an execute uploads (Gram job
// records, output slots). Each upload takes the next chunk in call order; the
// chunks live until the owner is destroyed, so a captured CUDA graph can copy
// from them on every replay. A chunk is rewritten only when its content
// changes, after the device has finished any earlier copy out of it.
struct PinnedArena
{
    std::vector<std::pair<void *, std::size_t>> blocks;
    std::size_t block = 0, off = 0;
    PinnedArena() = default;
    PinnedArena(const PinnedArena &) = delete;
    PinnedArena &operator=(const PinnedArena &) = delete;
    ~PinnedArena()
    {
        for (auto &b : blocks) cudaFreeHost(b.first);
    }
    void rewind()
    {
        block = 0;
        off = 0;
    }
    cudaError_t stage(const void *src, std::size_t bytes, void **out)
    {
        const std::size_t need = (std::max<std::size_t>(bytes, 1) + 255) & ~std::size_t{255};
        while (block < blocks.size() && off + need > blocks[block].second)
        {
            ++block;
            off = 0;
        }
        if (block == blocks.size())
        {
            void *p = nullptr;
            const std::size_t sz = std::max<std::size_t>(need, std::size_t{1} << 20);
            cudaError_t e = cudaMallocHost(&p, sz);
            if (e != cudaSuccess) return e;
            std::memset(p, 0, sz);
            blocks.push_back({p, sz});
            off = 0;
        }
        unsigned char *h = static_cast<unsigned char *>(blocks[block].first) + off;
        off += need;
        if (std::memcmp(h, src, bytes) != 0)
        {
            // An earlier execute may still be copying out of this chunk.
            cudaError_t e = cudaDeviceSynchronize();
            if (e != cudaSuccess) return e;
            std::memcpy(h, src, bytes);
        }
        *out = h;
        return cudaSuccess;
    }
};

__global__ void k_fill_double(double *p, std::size_t n, double v)
{
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x)
        p[i] = v;
}

// The Jordan-Wigner closure string of the fermionic ring, on every state of a
// batch: amplitudes whose site n-1 is occupied and whose sites 1..n-2 hold an
// odd number of particles change sign (the reference brackets the closure bond
// with this diagonal, cpp/include/mipt/cusv/gates.hpp:243-271). One thread per
// amplitude with bit n-1 set.
template <typename Real>
__global__ void k_jw_closure(Cx<Real> *states, int n, int count)
{
    const std::uint64_t half = 1ull << (n - 1), mid = half - 2ull;
    const std::uint64_t total = half * static_cast<std::uint64_t>(count);
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<std::uint64_t>(gridDim.x) * blockDim.x)
    {
        const std::uint64_t traj = i >> (n - 1), x = (i & (half - 1)) | half;
        if (__popcll(x & mid) & 1)
        {
            Cx<Real> &a = states[(traj << n) | x];
            a.re = -a.re;
            a.im = -a.im;
        }
    }
}

// Collapse records with the outcome test of `col` and no renormalisation or
// parity condition: for states the collapse has already been applied to
// (expanded parity-sector states), so that the entropies can still leave
// the measured stored sites out of the Gram.
__global__ void k_mask_records(const Collapse *__restrict__ col, std::size_t col_stride, int count,
                               Collapse *__restrict__ out)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= count) return;
    const Collapse c = col[b * col_stride];
    out[b] = Collapse{c.mask, c.value, 1.0, 0};
}

// Parity-sector states: trajectory b keeps the 2^ne amplitudes of its stored
// qubits 0..ne-1 at cs[b * 2^ne ..]; qubit ne (the chain's top qubit) is
// sector[b] xor the parity of the stored bits. Expansion writes the full
// 2^(ne+1) state (at st[b * 2^(ne+1) ..]) with an optional pending collapse
// applied; compaction reads a full state that lies in the sector.
template <typename Real>
__global__ void k_expand(const Cx<Real> *__restrict__ cs, Cx<Real> *__restrict__ st, int ne, int count,
                         const signed char *__restrict__ sector, const Collapse *__restrict__ col,
                         std::size_t col_stride)
{
    const std::uint64_t edim = 1ull << ne, dim = edim << 1;
    const std::uint64_t total = dim * static_cast<std::uint64_t>(count);
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<std::uint64_t>(gridDim.x) * blockDim.x)
    {
        const std::uint64_t b = i / dim, x = i % dim, c = x & (edim - 1);
        const int top = static_cast<int>(x >> ne);
        Cx<Real> v{Real(0), Real(0)};
        if (top == ((sector[b] + __popcll(c)) & 1))
        {
            v = cs[b * edim + c];
            if (col)
            {
                const Collapse cl = col[b * col_stride];
                if (!collapse_keeps(c, cl))
                    v = Cx<Real>{Real(0), Real(0)};
                else
                {
                    const Real sc = static_cast<Real>(cl.scale);
                    v = Cx<Real>{v.re * sc, v.im * sc};
                }
            }
        }
        st[i] = v;
    }
}

template <typename Real>
__global__ void k_compact(const Cx<Real> *__restrict__ st, Cx<Real> *__restrict__ cs, int ne, int b,
                          const signed char *__restrict__ sector)
{
    const std::uint64_t edim = 1ull << ne;
    for (std::uint64_t c = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; c < edim;
         c += static_cast<std::uint64_t>(gridDim.x) * blockDim.x)
    {
        const std::uint64_t top = static_cast<std::uint64_t>((sector[b] + __popcll(c)) & 1);
        cs[static_cast<std::uint64_t>(b) * edim + c] = st[(static_cast<std::uint64_t>(b) * edim << 1) + c +
                                                          (top << ne)];
    }
}

__global__ void k_reset_layers(Collapse *col, LayerResult *res, std::size_t n)
{
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x)
    {
        col[i] = Collapse{0ull, 0ull, 1.0, 0ull};
        LayerResult r{};
        res[i] = r;
    }
}

// out[idx[i]] = f(in[i]); f = identity (mode 0) or S_2 from a purity (mode 1).
__global__ void k_scatter(const double *in, const int *idx, int n, double *out, int mode)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = in[i];
    out[idx[i]] = mode == 1 ? renyi2_from_purity(v) : v;
}

// S = -sum lambda log2 lambda over lambda > 1e-15 (fixed-order reduction).
// Block b: entropy (bits) of the spectrum w[b*d .. b*d + d) into out[b].
// ------------------------------------------------------------ entropies

struct EntReq
{
    int traj;
    int order; // 1 = von Neumann, 2 = Renyi-2
    int fermion;
    std::vector<int> kept;
    int out; // index into the output array
};

struct Workspace
{
    DevBuf jobs, rho, scratch, vals, idx, eig, err, eig_err, rows, dims;
    PinnedArena stage;
    // Host -> device copy of a small table through the pinned staging arena.
    cudaError_t upload(void *dst, const void *src, std::size_t bytes, cudaStream_t s)
    {
        void *h = nullptr;
        cudaError_t e = stage.stage(src, bytes, &h);
        if (e != cudaSuccess) return e;
        return cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, s);
    }
};

// Spectra up to this many rows go to the one-block Jacobi eigensolver, larger
// ones to Householder tridiagonalisation + QL (MIPT_GB300_JACOBI_MAX_D, at
// most 64; default 16: from 32 rows on the reduction needs far fewer FP64
// operations than Jacobi sweeps).
int jacobi_max_dim()
{
    static const int d = [] {
        const char *v = std::getenv("MIPT_GB300_JACOBI_MAX_D");
        const int x = v ? std::atoi(v) : 16;
        return std::max(1, std::min(64, x));
    }();
    return d;
}

constexpr std::size_t kMaxRhoBytes = std::size_t{1} << 31;
// Largest buffer of pre-split TF32 operand rows (16 bytes per amplitude).
constexpr std::size_t kMaxRowsBytes = std::size_t{16} << 30;

// Evaluates every request into d_out[req.out]; all requests share n.
template <typename Real>
int run_entropies(const Cx<Real> *states, int n, const std::vector<EntReq> &reqs, const Collapse *col,
                  std::size_t col_stride, Workspace &ws, cudaStream_t s, double *d_out, long long &launches)
{
    // Group by (k, needs_rho).
    std::map<std::pair<int, int>, std::vector<const EntReq *>> groups;
    for (const auto &r : reqs)
    {
        const int k = static_cast<int>(r.kept.size());
        if (k == 0)
        {
            groups[{0, 0}].push_back(&r);
            continue;
        }
        const bool purity_only = (r.order == 2);
        groups[{k, purity_only ? 0 : 1}].push_back(&r);
    }
    for (auto &kv : groups)
    {
        const int k = kv.first.first;
        const bool vn = kv.first.second == 1;
        auto &list = kv.second;
        if (k == 0)
        {
            // Empty subsystem: entropy 0.
            std::vector<double> zeros(list.size(), 0.0);
            std::vector<int> idx;
            for (auto *r : list) idx.push_back(r->out);
            MG_CUDA(ws.vals.ensure(sizeof(double) * zeros.size()));
            MG_CUDA(ws.idx.ensure(sizeof(int) * idx.size()));
            MG_CUDA(ws.upload(ws.vals.p, zeros.data(), sizeof(double) * zeros.size(), s));
            MG_CUDA(ws.upload(ws.idx.p, idx.data(), sizeof(int) * idx.size(), s));
            k_scatter<<<(static_cast<int>(idx.size()) + 255) / 256, 256, 0, s>>>(ws.vals.as<double>(), ws.idx.as<int>(),
                                                                              static_cast<int>(idx.size()), d_out, 0);
            ++launches;
            continue;
        }
        const int d = 1 << k;
        const std::size_t rho_bytes = sizeof(double) * 2 * static_cast<std::size_t>(d) * d;
        const int tiles = gram_tiles(k);
        if constexpr (sizeof(Real) == 4)
        {
            // Renyi-2 of FP32 states on the tensor cores (3xTF32 tcgen05 Gram).
            if (!vn && gram_tc_supported(n, k))
            {
                const int nb = static_cast<int>(list.size());
                std::vector<GramJob> jobs(nb);
                std::vector<int> idx(nb);
                // Operands by TMA when every job keeps modes 0..k-1 in order.
                bool low_cut = true;
                int traj_count = 0;
                for (int i = 0; i < nb; ++i)
                {
                    jobs[i] = make_gram_job(list[i]->traj, n, list[i]->kept.data(), k, list[i]->fermion != 0);
                    idx[i] = list[i]->out;
                    for (int b = 0; b < k; ++b) low_cut = low_cut && list[i]->kept[b] == b;
                    traj_count = std::max(traj_count, list[i]->traj + 1);
                }
                MG_CUDA(ws.jobs.ensure(sizeof(GramJob) * nb));
                MG_CUDA(ws.idx.ensure(sizeof(int) * nb));
                MG_CUDA(ws.vals.ensure(sizeof(double) * nb));
                MG_CUDA(ws.scratch.ensure(gram_tc_scratch_bytes(k, nb)));
                if (!ws.err.p)
                {
                    MG_CUDA(ws.err.ensure(sizeof(int)));
                    MG_CUDA(cudaMemsetAsync(ws.err.p, 0, sizeof(int), s));
                }
                MG_CUDA(ws.upload(ws.jobs.p, jobs.data(), sizeof(GramJob) * nb, s));
                MG_CUDA(ws.upload(ws.idx.p, idx.data(), sizeof(int) * nb, s));
                // Low cuts: TF32 operand rows split once per observation, in
                // job groups of at most kMaxRowsBytes.
                // Pre-split operand rows for any kept set (the row split
                // gathers, with fermionic signs); the state's own tensor map
                // only serves the gathered fallback of low cuts.
                bool presplit = k <= gram_tc_presplit_max_k() && gram_tc_presplit_enabled();
                if (presplit)
                {
                    const std::size_t per_job = gram_tc_rows_bytes_per_job(n);
                    presplit = per_job <= kMaxRowsBytes &&
                               ws.rows.ensure(std::min(kMaxRowsBytes / per_job, static_cast<std::size_t>(nb)) *
                                              per_job) == cudaSuccess;
                    if (!presplit) cudaGetLastError(); // no room: the Gram gathers its operands itself
                }
                MG_CUDA(gram_purity_tc(states, n, ws.jobs.as<GramJob>(), nb, k, col, col_stride, ws.vals.as<double>(),
                                       ws.scratch.p, ws.scratch.bytes, ws.err.as<int>(), s, low_cut ? traj_count : 0,
                                       presplit ? ws.rows.p : nullptr, presplit ? ws.rows.bytes : 0));
                // Pre-split: the job table, then rows + Gram per group of
                // jobs that fits the row buffer, then the partial sums.
                if (presplit)
                {
                    const std::size_t group = std::max<std::size_t>(
                        1, std::min<std::size_t>(nb, ws.rows.bytes / gram_tc_rows_bytes_per_job(n)));
                    launches += 2 + 2 * static_cast<long long>((nb + group - 1) / group);
                }
                else
                    launches += 2;
                k_scatter<<<(nb + 255) / 256, 256, 0, s>>>(ws.vals.as<double>(), ws.idx.as<int>(), nb, d_out, 1);
                ++launches;
                continue;
            }
        }
        // Purity straight from tiles when there are enough tiles to fill the GPU.
        const bool tile_purity = !vn && tiles * static_cast<long long>(list.size()) >= 2 * 152;
        std::size_t per_launch = list.size();
        if (!tile_purity) per_launch = std::max<std::size_t>(1, std::min(list.size(), kMaxRhoBytes / rho_bytes));
        for (std::size_t b0 = 0; b0 < list.size(); b0 += per_launch)
        {
            const std::size_t nb = std::min(per_launch, list.size() - b0);
            std::vector<GramJob> jobs(nb);
            std::vector<int> idx(nb);
            for (std::size_t i = 0; i < nb; ++i)
            {
                const EntReq *r = list[b0 + i];
                jobs[i] = make_gram_job(r->traj, n, r->kept.data(), k, r->fermion != 0);
                idx[i] = r->out;
            }
            MG_CUDA(ws.jobs.ensure(sizeof(GramJob) * nb));
            MG_CUDA(ws.idx.ensure(sizeof(int) * nb));
            MG_CUDA(ws.vals.ensure(sizeof(double) * nb));
            MG_CUDA(ws.upload(ws.jobs.p, jobs.data(), sizeof(GramJob) * nb, s));
            MG_CUDA(ws.upload(ws.idx.p, idx.data(), sizeof(int) * nb, s));
            const int nbi = static_cast<int>(nb);
            if (tile_purity)
            {
                MG_CUDA(ws.scratch.ensure(gram_scratch_bytes(n, k, nbi, false)));
                MG_CUDA(gram_purity<Real>(states, n, ws.jobs.as<GramJob>(), nbi, k, col, col_stride,
                                          ws.vals.as<double>(), ws.scratch.p, ws.scratch.bytes, s));
                launches += 2;
                k_scatter<<<(nbi + 255) / 256, 256, 0, s>>>(ws.vals.as<double>(), ws.idx.as<int>(), nbi, d_out, 1);
                ++launches;
                continue;
            }
            MG_CUDA(ws.rho.ensure(rho_bytes * nb));
            MG_CUDA(ws.scratch.ensure(gram_scratch_bytes(n, k, nbi, true)));
            // Rows of each rho that hold data once measured sites are left
            // out; the large-spectrum eigensolver runs on those only.
            const bool large = vn && d > jacobi_max_dim();
            if (large) MG_CUDA(ws.dims.ensure(sizeof(int) * nb));
            MG_CUDA(gram_rho<Real>(states, n, ws.jobs.as<GramJob>(), nbi, k, col, col_stride, ws.rho.as<double>(),
                                   ws.scratch.p, ws.scratch.bytes, s, large ? ws.dims.as<int>() : nullptr));
            launches += 2;
            if (!vn)
            {
                MG_CUDA(purity_of(ws.rho.as<double>(), d, nbi, ws.vals.as<double>(), s));
                ++launches;
                k_scatter<<<(nbi + 255) / 256, 256, 0, s>>>(ws.vals.as<double>(), ws.idx.as<int>(), nbi, d_out, 1);
                ++launches;
            }
            else if (d <= jacobi_max_dim())
            {
                MG_CUDA(jacobi_entropy(ws.rho.as<double>(), d, nbi, ws.vals.as<double>(), nullptr, s));
                ++launches;
                k_scatter<<<(nbi + 255) / 256, 256, 0, s>>>(ws.vals.as<double>(), ws.idx.as<int>(), nbi, d_out, 0);
                ++launches;
            }
            else
            {
                // Large spectra: FP64 Householder tridiagonalisation and
                // implicit QL of every matrix of the group (eigen.cu).
                MG_CUDA(ws.eig.ensure(sizeof(double) * hermitian_eig_scratch_doubles(d, nbi)));
                if (!ws.eig_err.p)
                {
                    MG_CUDA(ws.eig_err.ensure(sizeof(int)));
                    MG_CUDA(cudaMemsetAsync(ws.eig_err.p, 0, sizeof(int), s));
                }
                MG_CUDA(hermitian_eig_entropy(ws.rho.as<double>(), d, nbi, ws.vals.as<double>(), nullptr,
                                              ws.eig.as<double>(), ws.eig_err.as<int>(), s, ws.dims.as<int>()));
                launches += 2;
                k_scatter<<<(nbi + 255) / 256, 256, 0, s>>>(ws.vals.as<double>(), ws.idx.as<int>(), nbi, d_out, 0);
                ++launches;
            }
        }
    }
    return 0;
}

// ------------------------------------------------------ compat scratch
struct CompatCtx
{
    Workspace ws;
    DevBuf out, subs, rho3, scratch, sums;
};
thread_local std::unique_ptr<CompatCtx> g_compat;
CompatCtx &compat()
{
    if (!g_compat) g_compat.reset(new CompatCtx());
    return *g_compat;
}

template <typename Real>
int compat_entropy(const void *state, int n, const int *kept, int k, int fermion, int order, double *out)
{
    if (!state || !kept || !out || n < 1 || n > 32 || k < 0 || k > n || k > 16)
        return fail(MIPT_GB300_E_INVALID, "invalid subsystem request");
    auto &c = compat();
    EntReq r{0, order, fermion, std::vector<int>(kept, kept + k), 0};
    for (int i = 0; i < k; ++i)
        if (kept[i] < 0 || kept[i] >= n) return fail(MIPT_GB300_E_INVALID, "kept mode out of range");
    MG_CUDA(c.out.ensure(sizeof(double)));
    c.ws.stage.rewind();
    if (c.ws.err.p) MG_CUDA(cudaMemsetAsync(c.ws.err.p, 0, sizeof(int), 0));
    if (c.ws.eig_err.p) MG_CUDA(cudaMemsetAsync(c.ws.eig_err.p, 0, sizeof(int), 0));
    long long l = 0;
    try
    {
        const int rc = run_entropies<Real>(static_cast<const Cx<Real> *>(state), n, {r}, nullptr, 0, c.ws, 0,
                                           c.out.as<double>(), l);
        if (rc) return rc;
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
    MG_CUDA(cudaMemcpy(out, c.out.p, sizeof(double), cudaMemcpyDeviceToHost));
    if (c.ws.err.p)
    {
        int err = 0;
        MG_CUDA(cudaMemcpy(&err, c.ws.err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) return fail(MIPT_GB300_E_INTERNAL, "tensor-core Gram pipeline wait timed out");
    }
    if (c.ws.eig_err.p)
    {
        int err = 0;
        MG_CUDA(cudaMemcpy(&err, c.ws.eig_err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (err & 2) return fail(MIPT_GB300_E_INTERNAL, "eigensolver barrier wait timed out");
        if (err) return fail(MIPT_GB300_E_NUMERIC, "an eigenvalue iteration did not converge");
    }
    return 0;
}

template <typename Real>
int compat_rdm(const void *state, int n, const int *kept, int k, int fermion, double *host_rho)
{
    if (!state || !kept || !host_rho || n < 1 || n > 32 || k < 1 || k > n || k > 14)
        return fail(MIPT_GB300_E_INVALID, "invalid subsystem request");
    auto &c = compat();
    GramJob job;
    try
    {
        job = make_gram_job(0, n, kept, k, fermion != 0);
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
    const std::size_t d = std::size_t{1} << k;
    MG_CUDA(c.ws.jobs.ensure(sizeof(GramJob)));
    MG_CUDA(cudaMemcpy(c.ws.jobs.p, &job, sizeof(GramJob), cudaMemcpyHostToDevice));
    MG_CUDA(c.ws.rho.ensure(sizeof(double) * 2 * d * d));
    MG_CUDA(c.ws.scratch.ensure(gram_scratch_bytes(n, k, 1, true)));
    MG_CUDA(gram_rho<Real>(static_cast<const Cx<Real> *>(state), n, c.ws.jobs.as<GramJob>(), 1, k, nullptr, 0,
                           c.ws.rho.as<double>(), c.ws.scratch.p, c.ws.scratch.bytes, 0));
    MG_CUDA(cudaMemcpy(host_rho, c.ws.rho.p, sizeof(double) * 2 * d * d, cudaMemcpyDeviceToHost));
    return 0;
}

template <typename Real>
int compat_rho3(const void *state, int n, const int *subs, int count, int fermion, double *out)
{
    if (!state || !subs || !out || count <= 0 || n < 3 || n > 32)
        return fail(MIPT_GB300_E_INVALID, "invalid three-site request");
    for (int s = 0; s < count; ++s)
    {
        const int a = subs[3 * s], b = subs[3 * s + 1], c = subs[3 * s + 2];
        if (a < 0 || a >= n || b < 0 || b >= n || c < 0 || c >= n || a == b || a == c || b == c)
            return fail(MIPT_GB300_E_INVALID, "three-site subsystem out of range or repeated");
    }
    auto &c = compat();
    MG_CUDA(c.subs.ensure(sizeof(int) * 3 * count));
    MG_CUDA(cudaMemcpy(c.subs.p, subs, sizeof(int) * 3 * count, cudaMemcpyHostToDevice));
    MG_CUDA(c.rho3.ensure(sizeof(double) * 128 * count));
    MG_CUDA(c.scratch.ensure(rho3_scratch_bytes(n, 1, count)));
    MG_CUDA(rho3_sweep<Real>(static_cast<const Cx<Real> *>(state), n, 1, c.subs.as<int>(), count, fermion, nullptr, 0,
                             c.rho3.as<double>(), c.scratch.p, c.scratch.bytes, 0));
    MG_CUDA(cudaMemcpy(out, c.rho3.p, sizeof(double) * 128 * count, cudaMemcpyDeviceToHost));
    return 0;
}

// Host-resident state vectors: one reusable device copy per calling thread.
template <typename Real>
int host_rho3(const void *host_state, int n, const int *subs, int count, int fermion, double *out, double *fout)
{
    if (!host_state || n < 3 || n > 32) return fail(MIPT_GB300_E_INVALID, "invalid host state vector");
    static thread_local DevBuf dev;
    const std::size_t bytes = sizeof(Real) * 2 * (std::size_t{1} << n);
    MG_CUDA(dev.ensure(bytes));
    MG_CUDA(cudaMemcpy(dev.p, host_state, bytes, cudaMemcpyHostToDevice));
    if (fermion == 2)
    {
        const int rc = compat_rho3<Real>(dev.p, n, subs, count, 0, out);
        return rc ? rc : compat_rho3<Real>(dev.p, n, subs, count, 1, fout);
    }
    return compat_rho3<Real>(dev.p, n, subs, count, fermion, out);
}

// --------------------------------------------- single-site measurement
constexpr int kNormBlocks = 256;

template <typename Real>
__global__ void k_branch_norms(const Cx<Real> *psi, std::uint64_t dim, std::uint64_t mask, double *part)
{
    __shared__ double r0[256], r1[256];
    double tot = 0.0, one = 0.0;
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < dim;
         i += static_cast<std::uint64_t>(gridDim.x) * blockDim.x)
    {
        const double w = static_cast<double>(psi[i].re) * psi[i].re + static_cast<double>(psi[i].im) * psi[i].im;
        tot += w;
        if (i & mask) one += w;
    }
    r0[threadIdx.x] = tot;
    r1[threadIdx.x] = one;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k /= 2)
    {
        if (threadIdx.x < k)
        {
            r0[threadIdx.x] += r0[threadIdx.x + k];
            r1[threadIdx.x] += r1[threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        part[2 * blockIdx.x] = r0[0];
        part[2 * blockIdx.x + 1] = r1[0];
    }
}

template <typename Real>
__global__ void k_project(Cx<Real> *psi, std::uint64_t dim, std::uint64_t mask, std::uint64_t value, double scale)
{
    const Real s = static_cast<Real>(scale);
    for (std::uint64_t i = blockIdx.x * static_cast<std::uint64_t>(blockDim.x) + threadIdx.x; i < dim;
         i += static_cast<std::uint64_t>(gridDim.x) * blockDim.x)
    {
        if ((i & mask) != value)
            psi[i] = Cx<Real>{Real(0), Real(0)};
        else
        {
            psi[i].re *= s;
            psi[i].im *= s;
        }
    }
}

template <typename Real>
int measure_collapse(void *state, int n, int q, double u, int *outcome, double *prob)
{
    if (!state || n < 1 || n > 34 || q < 0 || q >= n || !(u >= 0.0 && u < 1.0) || !outcome || !prob)
    {
        g_measure_error = "Invalid sequential-measurement request.";
        return fail(MIPT_GB300_E_INVALID, g_measure_error);
    }
    auto &c = compat();
    const std::uint64_t dim = 1ull << n;
    cudaError_t e = c.sums.ensure(sizeof(double) * 2 * kNormBlocks);
    if (e != cudaSuccess) return cuda_fail(e, "measure scratch");
    Cx<Real> *psi = static_cast<Cx<Real> *>(state);
    k_branch_norms<Real><<<kNormBlocks, 256>>>(psi, dim, 1ull << q, c.sums.as<double>());
    std::vector<double> h(2 * kNormBlocks);
    e = cudaMemcpy(h.data(), c.sums.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
    {
        g_measure_error = cudaGetErrorString(e);
        return cuda_fail(e, "measure norms");
    }
    double tot = 0.0, one = 0.0;
    for (int i = 0; i < kNormBlocks; ++i)
    {
        tot += h[2 * i];
        one += h[2 * i + 1];
    }
    if (!(tot > 0.0) || !std::isfinite(tot) || !std::isfinite(one) || one < 0.0 || one > tot * (1.0 + 1e-10))
    {
        g_measure_error = "Sequential measurement received invalid branch norms.";
        return fail(MIPT_GB300_E_NUMERIC, g_measure_error);
    }
    const double p1 = std::clamp(one / tot, 0.0, 1.0);
    const int bit = u < p1 ? 1 : 0;
    const double cp = bit ? p1 : 1.0 - p1;
    const double branch = bit ? one : tot - one;
    if (!(cp > 0.0) || !(branch > 0.0))
    {
        g_measure_error = "Sampled an outcome with invalid conditional probability.";
        return fail(MIPT_GB300_E_NUMERIC, g_measure_error);
    }
    k_project<Real><<<1024, 256>>>(psi, dim, 1ull << q, bit ? (1ull << q) : 0ull, 1.0 / std::sqrt(branch));
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
    {
        g_measure_error = cudaGetErrorString(e);
        return cuda_fail(e, "measure collapse");
    }
    *outcome = bit;
    *prob = cp;
    g_measure_error.clear();
    return 0;
}

int default_tile_qubits(bool fp64) { return fp64 ? 13 : 14; }
constexpr int kCoalesceQubits = 4;

// Bond lists of every colour of a batch geometry (1-D brickwork: even and odd
// layers; lattice: four colours).
std::vector<std::vector<Bond>> geometry_bonds(int n, int closed, int lx, int ly)
{
    std::vector<std::vector<Bond>> out;
    if (ly > 1)
    {
        for (int colour = 0; colour < 4; ++colour)
        {
            out.emplace_back();
            for (const auto &pr : lattice_bonds(lx, ly, colour)) out.back().push_back(Bond{pr.first, pr.second});
        }
    }
    else
        for (int colour = 0; colour < 2; ++colour)
        {
            out.emplace_back();
            const int stop = (closed && colour == 1 && n > 2) ? n : n - 1;
            for (int i = colour; i < stop; i += 2) out.back().push_back(Bond{i, (i + 1) % n});
        }
    return out;
}

// Tile-shape autotuner: times one cycle of every layer colour (passes only)
// on `trajectories` scratch states for each candidate local-qubit count and
// returns the fastest. Candidates: the default and the two below it, where the
// tile still fits the geometry.
template <typename Real>
int autotune_tile_impl(int n, int closed, int lx, int ly, int trajectories, int *best, double *ms, int *cand,
                       int *ncand)
{
    const int def = default_tile_qubits(sizeof(Real) == 8);
    const auto bonds = geometry_bonds(n, closed, lx, ly);
    std::vector<int> ks;
    for (int k = def - 2; k <= def; ++k)
    {
        const int kk = std::min(k, n);
        if (n - kk + kCoalesceQubits > 20) continue;
        if (std::find(ks.begin(), ks.end(), kk) == ks.end()) ks.push_back(kk);
    }
    const std::size_t dim = std::size_t{1} << n;
    DevBuf states, gates, err;
    MG_CUDA(states.ensure(sizeof(Cx<Real>) * dim * static_cast<std::size_t>(trajectories)));
    MG_CUDA(err.ensure(sizeof(int)));
    MG_CUDA(cudaMemset(err.p, 0, sizeof(int)));
    // Every bond gets the same fixed unitary, H x H (timing does not depend on it).
    const int G = n;
    std::vector<Cx<Real>> h(static_cast<std::size_t>(G) * 16);
    for (int g = 0; g < G; ++g)
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c)
                h[g * 16 + r * 4 + c] = Cx<Real>{static_cast<Real>((__builtin_popcount(r & c) & 1) ? -0.5 : 0.5), Real(0)};
    MG_CUDA(gates.ensure(sizeof(Cx<Real>) * h.size()));
    MG_CUDA(cudaMemcpy(gates.p, h.data(), sizeof(Cx<Real>) * h.size(), cudaMemcpyHostToDevice));
    MG_CUDA(launch_init_zero<Real>(states.as<Cx<Real>>(), dim, trajectories, nullptr));
    cudaEvent_t a, b;
    MG_CUDA(cudaEventCreate(&a));
    MG_CUDA(cudaEventCreate(&b));
    double best_ms = -1.0;
    int count = 0;
    for (int k : ks)
    {
        std::vector<std::vector<PassPlan>> plans;
        try
        {
            for (const auto &bl : bonds) plans.push_back(plan_layer(n, bl, k, kCoalesceQubits, register_bits<Real>()));
        }
        catch (const std::exception &)
        {
            continue;
        }
        auto cycle = [&]() -> cudaError_t {
            for (const auto &pl : plans)
                for (const auto &pp : pl)
                {
                    cudaError_t e = launch_pass<Real>(states.as<Cx<Real>>(), trajectories, pp, gates.as<Cx<Real>>(), 0,
                                                      nullptr, 0, nullptr, 0, nullptr, 0, err.as<int>(), nullptr);
                    if (e != cudaSuccess) return e;
                }
            return cudaSuccess;
        };
        MG_CUDA(cycle());
        MG_CUDA(cudaEventRecord(a));
        for (int rep = 0; rep < 3; ++rep) MG_CUDA(cycle());
        MG_CUDA(cudaEventRecord(b));
        MG_CUDA(cudaEventSynchronize(b));
        float t = 0.f;
        MG_CUDA(cudaEventElapsedTime(&t, a, b));
        const double per = t / 3.0;
        if (ms) ms[count] = per;
        if (cand) cand[count] = k;
        ++count;
        if (best_ms < 0.0 || per < best_ms)
        {
            best_ms = per;
            *best = k;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    int e_flag = 0;
    MG_CUDA(cudaMemcpy(&e_flag, err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e_flag) return fail(MIPT_GB300_E_INTERNAL, "tile load wait timed out");
    if (ncand) *ncand = count;
    if (count == 0) *best = def;
    return 0;
}

// Tile choice of a batch created with tile_qubits = 0: the table below,
// measured on GB300 with mipt_gb300/tune_tiles.py (the fastest candidate per
// geometry; the default where the table has no entry), or, with
// MIPT_GB300_AUTOTUNE=1, a live autotune of this geometry (cached per
// process). The table keeps results reproducible run to run: the tile shape
// changes the order in which disjoint gates round.
struct TileChoice
{
    int n, fp64, lattice, tile;
};
constexpr TileChoice kTunedTiles[] = {
    // {n, fp64, lattice, tile}: FP32 keeps 14 everywhere (2-30 % ahead of 12
    // and 13 at batch-sized grids); FP64 is within 1-2 % across 11..13.
    {14, 0, 0, 14},
    {16, 0, 0, 14},
    {18, 0, 0, 14},
    {20, 0, 0, 14},
    {22, 0, 0, 14},
    {24, 0, 0, 14},
    {26, 0, 0, 14},
    {28, 0, 0, 14},
    {30, 0, 0, 14},
    {14, 1, 0, 11},
    {16, 1, 0, 12},
    {18, 1, 0, 12},
    {20, 1, 0, 12},
    {22, 1, 0, 13},
    {24, 1, 0, 12},
    {26, 1, 0, 12},
    {28, 1, 0, 12},
    {28, 0, 1, 14},
    {20, 0, 1, 14},
};

// MIPT_GB300_PARITY_ENCODED=0 runs the RPPU / qRPPU gate sets on full-size
// states (default: half-size parity-sector states where every trajectory has
// a definite parity).
bool use_parity_encoding()
{
    static const bool on = [] {
        const char *v = std::getenv("MIPT_GB300_PARITY_ENCODED");
        return !(v && v[0] == '0');
    }();
    return on;
}

// MIPT_GB300_SPARSE_PASS=0 makes the first pass after a measurement visit
// every tile (default: only the tiles that agree with the outcome).
bool use_sparse_pass()
{
    static const bool on = [] {
        const char *v = std::getenv("MIPT_GB300_SPARSE_PASS");
        return !(v && v[0] == '0');
    }();
    return on;
}

int chosen_tile(const mipt_gb300_batch_config &cfg, int capacity)
{
    const bool fp64 = cfg.fp64 != 0;
    const bool lattice = cfg.lattice_y > 1;
    const char *v = std::getenv("MIPT_GB300_AUTOTUNE");
    if (v && v[0] == '1')
    {
        static std::mutex m;
        static std::map<std::tuple<int, int, int, int, int>, int> cache;
        const auto key = std::make_tuple(cfg.n_qubits, cfg.fp64, cfg.closed, cfg.lattice_x, cfg.lattice_y);
        std::lock_guard<std::mutex> lock(m);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
        const std::size_t state = (std::size_t{1} << cfg.n_qubits) * (fp64 ? 16 : 8);
        const int traj = static_cast<int>(std::max<std::size_t>(
            1, std::min<std::size_t>(static_cast<std::size_t>(capacity), (std::size_t{4} << 30) / state)));
        int best = default_tile_qubits(fp64);
        const int rc = fp64 ? autotune_tile_impl<double>(cfg.n_qubits, cfg.closed, cfg.lattice_x, cfg.lattice_y, traj,
                                                         &best, nullptr, nullptr, nullptr)
                            : autotune_tile_impl<float>(cfg.n_qubits, cfg.closed, cfg.lattice_x, cfg.lattice_y, traj,
                                                        &best, nullptr, nullptr, nullptr);
        if (rc != 0) best = default_tile_qubits(fp64);
        cache[key] = best;
        return best;
    }
    for (const TileChoice &t : kTunedTiles)
        if (t.n == cfg.n_qubits && t.fp64 == (fp64 ? 1 : 0) && t.lattice == (lattice ? 1 : 0)) return t.tile;
    return default_tile_qubits(fp64);
}

} // namespace

namespace mg
{
int api_fail(int code, const std::string &what) { return fail(code, what); }
int api_cuda_fail(cudaError_t e, const char *what) { return cuda_fail(e, what); }
} // namespace mg

// ======================================================================= engine
struct mipt_gb300_engine
{
    bool fp64 = false;
    int n = 0;
    void *owned = nullptr;
    void *borrowed = nullptr;
    std::size_t owned_bytes = 0;
    DevBuf gates, meas, col, res, part, bins, err;
    ~mipt_gb300_engine()
    {
        if (owned) cudaFree(owned);
    }
    void *data() { return borrowed ? borrowed : owned; }
};

// ======================================================================= batch
struct mipt_gb300_batch
{
    mipt_gb300_batch_config cfg{};
    int capacity = 0;
    int count = 0;
    int T = 0, G = 0, kmax = 0, cmin = 0;
    std::uint64_t dim = 0;
    std::size_t elem = 0;
    std::vector<PassPlan> plan[4]; // per colour: 2 (1-D even/odd) or 4 (2-D)
    // Parity-sector (half-size) execution of the RPPU / qRPPU gate sets: the
    // plans over the n-1 stored qubits, whether the prepared trajectories
    // run that way (every one in a definite parity sector), the compact
    // states and the device copy of the sectors.
    std::vector<PassPlan> plan_enc[2];
    bool can_encode = false, enc = false;
    std::vector<int> enc_sector; // the sectors the gates were uploaded for
    DevBuf cstates, d_sector;
    DevBuf mask_col; // outcome-only collapse records of expanded states (count)
    int ncolour = 2;
    bool lattice = false;
    std::vector<int> region_slots; // request index of each added region
    int rho3_count = 0;            // three-site subsystems
    DevBuf rho3_pts;               // [points][count][rho3_count][128]
    DevBuf states, gates, meas, forced, col, res, part, bins, err, ent, subs, rho3, r3scratch;
    PinnedBuf h_gates, h_meas, h_forced, h_res;
    std::vector<std::uint64_t> measured;
    std::vector<char> any_meas, fusable;
    // [layer][chunk]: every trajectory's chunk lies outside the histogram tile
    // (one total per tile, streamed without shared-memory staging).
    std::vector<char> direct_hist;
    std::vector<int> max_chunks;
    bool has_forced = false;
    int points = 0;
    int reqs_per_point = 0;
    // Explicit observation schedule (mipt_gb300_batch_set_observation_steps):
    // obs_point[t] is the point index observed after t layers (t = 0: the
    // initial state), -1 where none; empty = the observe_every rule.
    std::vector<int> obs_point;
    // Trajectories whose initial state was uploaded for the next execute.
    std::vector<char> custom_init;
    // Global parity sector of each trajectory's initial state (-1: not a
    // parity eigenstate), and the sector the FermionRPPU closure gates were
    // folded for at upload (-1: not folded, the closure string runs as two
    // diagonal passes).
    std::vector<int> sector, folded;
    bool per_point() const { return !obs_point.empty() || cfg.observe_every > 0; }
    std::vector<EntReq> reqs; // for one point, trajectory index filled per launch
    int col_half_vn = -1, col_half_s2 = -1;
    std::vector<int> tmi_vn, tmi_s2; // 7 request slots (A,B,C,D,AB,AC,BC) per cyclic offset
    int tmi_cycles = 0;
    Workspace ws;
    long long launches = 0;
    bool executed = false;
    // Optional per-category kernel timing with CUDA events on the launch stream.
    bool profile = false;
    std::vector<cudaEvent_t> event_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    std::size_t next_event = 0;
    double kind_ms[5] = {0, 0, 0, 0, 0};
    long long kind_launches[5] = {0, 0, 0, 0, 0};
    // CUDA graph of one execute (mipt_gb300_batch_execute_graph) and the
    // host-side structure it was captured for.
    cudaGraphExec_t graph_exec = nullptr;
    cudaStream_t cap_stream = nullptr;
    std::vector<long long> graph_key;
    long long graph_launches = 0;
    ~mipt_gb300_batch()
    {
        for (auto e : event_pool) cudaEventDestroy(e);
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (cap_stream) cudaStreamDestroy(cap_stream);
    }
    cudaEvent_t take_event()
    {
        if (next_event == event_pool.size())
        {
            cudaEvent_t e;
            cudaEventCreate(&e);
            event_pool.push_back(e);
        }
        return event_pool[next_event++];
    }
};

namespace
{
// Brackets one launch (or a group) with events when profiling is on.
struct Mark
{
    mipt_gb300_batch *b;
    int kind;
    cudaStream_t s;
    cudaEvent_t start = nullptr;
    Mark(mipt_gb300_batch *b_, int kind_, cudaStream_t s_) : b(b_), kind(kind_), s(s_)
    {
        if (b->profile)
        {
            start = b->take_event();
            cudaEventRecord(start, s);
        }
    }
    ~Mark()
    {
        if (b->profile)
        {
            cudaEvent_t end = b->take_event();
            cudaEventRecord(end, s);
            b->marks.push_back({kind, {start, end}});
        }
    }
};
enum
{
    K_PASS = 0,
    K_HIST = 1,
    K_MEASURE = 2,
    K_OBS = 3,
    K_OTHER = 4
};
} // namespace

extern "C" {

const char *mipt_gb300_last_error(void) { return g_error.c_str(); }


int mipt_cuda_rho3_subsystems_complex_host_f64(const void *s, int n, const int *subs, int c, double *o)
{
    return host_rho3<double>(s, n, subs, c, 0, o, nullptr);
}
int mipt_cuda_rho3_subsystems_complex_host_f32(const void *s, int n, const int *subs, int c, double *o)
{
    return host_rho3<float>(s, n, subs, c, 0, o, nullptr);
}
int mipt_cuda_rho3_subsystems_complex_host_fermion_f64(const void *s, int n, const int *subs, int c, double *o)
{
    return host_rho3<double>(s, n, subs, c, 1, o, nullptr);
}
int mipt_cuda_rho3_subsystems_complex_host_fermion_f32(const void *s, int n, const int *subs, int c, double *o)
{
    return host_rho3<float>(s, n, subs, c, 1, o, nullptr);
}
int mipt_cuda_rho3_subsystems_complex_host_both_f64(const void *s, int n, const int *subs, int c, double *o,
                                                    double *fo)
{
    return host_rho3<double>(s, n, subs, c, 2, o, fo);
}
int mipt_cuda_rho3_subsystems_complex_host_both_f32(const void *s, int n, const int *subs, int c, double *o,
                                                    double *fo)
{
    return host_rho3<float>(s, n, subs, c, 2, o, fo);
}
const char *mipt_gb300_version(void) { return "mipt_gb300 0.1 (sm_103a)"; }
std::uint64_t mipt_gb300_splitmix64(std::uint64_t v) { return mg::splitmix64(v); }
std::uint64_t mipt_gb300_trajectory_seed(std::uint64_t m, std::uint64_t i) { return mg::trajectory_seed(m, i); }

namespace
{
int export_draw(const TrajectoryDraw &d, int *gates_per_layer, int *bond_q, double *bond_u, std::uint64_t *measured,
                double *uniforms, int *n_uniforms)
{
    for (int t = 0; t < d.layers; ++t)
    {
        if (gates_per_layer) gates_per_layer[t] = d.bond_count[t];
        if (measured) measured[t] = d.measured[t];
    }
    if (bond_q) std::copy(d.bond_q.begin(), d.bond_q.end(), bond_q);
    if (bond_u)
        for (std::size_t i = 0; i < d.bond_u.size(); ++i)
        {
            bond_u[2 * i] = d.bond_u[i].real();
            bond_u[2 * i + 1] = d.bond_u[i].imag();
        }
    if (uniforms) std::copy(d.uniforms.begin(), d.uniforms.end(), uniforms);
    if (n_uniforms) *n_uniforms = static_cast<int>(d.uniforms.size());
    return 0;
}
} // namespace

int mipt_gb300_draw_haar_workspace(std::uint32_t seed, int n, int layers, double p, int chunk_bits,
                                   int *gates_per_layer, int *bond_q, double *bond_u, std::uint64_t *measured,
                                   double *uniforms, int *n_uniforms)
{
    try
    {
        TrajectoryDraw d;
        draw_haar_trajectory_workspace(seed, n, layers, p, true, chunk_bits, d);
        return export_draw(d, gates_per_layer, bond_q, bond_u, measured, uniforms, n_uniforms);
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
}

int mipt_gb300_draw_rppu(std::uint64_t seed, int n, int periods, double p, int chunk_bits, int split_last,
                         int workspace, int *gates_per_layer, int *bond_q, double *bond_u, std::uint64_t *measured,
                         double *uniforms, int *n_uniforms)
{
    try
    {
        TrajectoryDraw d;
        if (workspace)
            draw_rppu_workspace(static_cast<std::uint32_t>(seed), n, 2 * periods, p, chunk_bits, split_last != 0,
                                2 * periods + 1, d);
        else
            draw_rppu_trajectory(seed, n, periods, p, chunk_bits, split_last != 0, 2 * periods + 1, d);
        return export_draw(d, gates_per_layer, bond_q, bond_u, measured, uniforms, n_uniforms);
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
}

int mipt_gb300_draw_haar(std::uint64_t seed, int n, int periods, double p, int closed, int chunk_bits,
                         int *gates_per_layer, int *bond_q, double *bond_u, std::uint64_t *measured, double *uniforms,
                         int *n_uniforms)
{
    try
    {
        TrajectoryDraw d;
        draw_haar_trajectory(seed, n, periods, p, closed != 0, chunk_bits, d);
        for (int t = 0; t < d.layers; ++t)
        {
            if (gates_per_layer) gates_per_layer[t] = d.bond_count[t];
            if (measured) measured[t] = d.measured[t];
        }
        if (bond_q) std::copy(d.bond_q.begin(), d.bond_q.end(), bond_q);
        if (bond_u)
            for (std::size_t i = 0; i < d.bond_u.size(); ++i)
            {
                bond_u[2 * i] = d.bond_u[i].real();
                bond_u[2 * i + 1] = d.bond_u[i].imag();
            }
        if (uniforms) std::copy(d.uniforms.begin(), d.uniforms.end(), uniforms);
        if (n_uniforms) *n_uniforms = static_cast<int>(d.uniforms.size());
        return 0;
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
}

// ---------------------------------------------------------- compat ABI
int mipt_cuda_rdm_subsystem_f64(const void *s, int n, const int *kept, int k, int f, double *rho)
{
    return compat_rdm<double>(s, n, kept, k, f, rho);
}
int mipt_cuda_rdm_subsystem_f32(const void *s, int n, const int *kept, int k, int f, double *rho)
{
    return compat_rdm<float>(s, n, kept, k, f, rho);
}
int mipt_cuda_entropy_svd_f64(const void *s, int n, const int *kept, int k, int f, double *out)
{
    return compat_entropy<double>(s, n, kept, k, f, 1, out);
}
int mipt_cuda_entropy_svd_f32(const void *s, int n, const int *kept, int k, int f, double *out)
{
    return compat_entropy<float>(s, n, kept, k, f, 1, out);
}
int mipt_cuda_renyi2_f64(const void *s, int n, const int *kept, int k, int f, double *out)
{
    return compat_entropy<double>(s, n, kept, k, f, 2, out);
}
int mipt_cuda_renyi2_f32(const void *s, int n, const int *kept, int k, int f, double *out)
{
    return compat_entropy<float>(s, n, kept, k, f, 2, out);
}
int mipt_cuda_rho3_subsystems_complex_f64(const void *s, int n, const int *subs, int c, double *o)
{
    return compat_rho3<double>(s, n, subs, c, 0, o);
}
int mipt_cuda_rho3_subsystems_complex_f32(const void *s, int n, const int *subs, int c, double *o)
{
    return compat_rho3<float>(s, n, subs, c, 0, o);
}
int mipt_cuda_rho3_subsystems_complex_fermion_f64(const void *s, int n, const int *subs, int c, double *o)
{
    return compat_rho3<double>(s, n, subs, c, 1, o);
}
int mipt_cuda_rho3_subsystems_complex_fermion_f32(const void *s, int n, const int *subs, int c, double *o)
{
    return compat_rho3<float>(s, n, subs, c, 1, o);
}
int mipt_cuda_rho3_subsystems_complex_both_f64(const void *s, int n, const int *subs, int c, double *o, double *fo)
{
    int rc = compat_rho3<double>(s, n, subs, c, 0, o);
    return rc ? rc : compat_rho3<double>(s, n, subs, c, 1, fo);
}
int mipt_cuda_rho3_subsystems_complex_both_f32(const void *s, int n, const int *subs, int c, double *o, double *fo)
{
    int rc = compat_rho3<float>(s, n, subs, c, 0, o);
    return rc ? rc : compat_rho3<float>(s, n, subs, c, 1, fo);
}
int mipt_cuda_measure_collapse_f32(void *s, int n, int q, double u, int *o, double *p)
{
    return measure_collapse<float>(s, n, q, u, o, p);
}
int mipt_cuda_measure_collapse_f64(void *s, int n, int q, double u, int *o, double *p)
{
    return measure_collapse<double>(s, n, q, u, o, p);
}
const char *mipt_cuda_measure_collapse_last_error(void) { return g_measure_error.c_str(); }

// ---------------------------------------------------------------- engine
int mipt_gb300_engine_create(int fp64, mipt_gb300_engine **out)
{
    if (!out) return fail(MIPT_GB300_E_INVALID, "null output pointer");
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return fail(MIPT_GB300_E_NODEVICE, "no CUDA device");
    auto *e = new mipt_gb300_engine();
    e->fp64 = fp64 != 0;
    *out = e;
    return 0;
}

void mipt_gb300_engine_destroy(mipt_gb300_engine *e) { delete e; }

int mipt_gb300_engine_reset(mipt_gb300_engine *e, int n)
{
    if (!e || n < 1 || n > 32) return fail(MIPT_GB300_E_INVALID, "engine supports 1..32 qubits");
    const std::size_t bytes = (std::size_t{1} << n) * (e->fp64 ? 16u : 8u);
    e->borrowed = nullptr;
    if (!e->owned || e->owned_bytes < bytes)
    {
        if (e->owned) cudaFree(e->owned);
        e->owned = nullptr;
        MG_CUDA(cudaMalloc(&e->owned, bytes));
        e->owned_bytes = bytes;
    }
    e->n = n;
    if (e->fp64)
        MG_CUDA(launch_init_zero<double>(static_cast<Cx<double> *>(e->owned), 1ull << n, 1, 0));
    else
        MG_CUDA(launch_init_zero<float>(static_cast<Cx<float> *>(e->owned), 1ull << n, 1, 0));
    MG_CUDA(cudaDeviceSynchronize());
    return 0;
}

int mipt_gb300_engine_adopt(mipt_gb300_engine *e, void *ptr, int n)
{
    if (!e || !ptr || n < 1 || n > 32) return fail(MIPT_GB300_E_INVALID, "engine adopt got an invalid buffer");
    e->borrowed = ptr;
    e->n = n;
    return 0;
}

void *mipt_gb300_engine_data(mipt_gb300_engine *e) { return e ? e->data() : nullptr; }

int mipt_gb300_engine_set_from_host(mipt_gb300_engine *e, const double *h, int n)
{
    if (!e || !h || n < 1 || n > 32) return fail(MIPT_GB300_E_INVALID, "invalid host state");
    if (!e->borrowed)
    {
        int rc = mipt_gb300_engine_reset(e, n);
        if (rc) return rc;
    }
    e->n = n;
    const std::size_t dim = std::size_t{1} << n;
    if (e->fp64)
    {
        MG_CUDA(cudaMemcpy(e->data(), h, dim * 16, cudaMemcpyHostToDevice));
    }
    else
    {
        std::vector<float> f(2 * dim);
        for (std::size_t i = 0; i < 2 * dim; ++i) f[i] = static_cast<float>(h[i]);
        MG_CUDA(cudaMemcpy(e->data(), f.data(), dim * 8, cudaMemcpyHostToDevice));
    }
    return 0;
}

int mipt_gb300_engine_to_host(mipt_gb300_engine *e, double *h)
{
    if (!e || !h || !e->data()) return fail(MIPT_GB300_E_INVALID, "engine has no state");
    const std::size_t dim = std::size_t{1} << e->n;
    if (e->fp64)
    {
        MG_CUDA(cudaMemcpy(h, e->data(), dim * 16, cudaMemcpyDeviceToHost));
    }
    else
    {
        std::vector<float> f(2 * dim);
        MG_CUDA(cudaMemcpy(f.data(), e->data(), dim * 8, cudaMemcpyDeviceToHost));
        for (std::size_t i = 0; i < 2 * dim; ++i) h[i] = f[i];
    }
    return 0;
}

int mipt_gb300_engine_apply_bonds(mipt_gb300_engine *e, const int *pairs, int nb, const double *m)
{
    if (!e || !e->data() || nb < 0 || (nb > 0 && (!pairs || !m))) return fail(MIPT_GB300_E_INVALID, "bad bonds");
    if (nb == 0) return 0;
    std::vector<Bond> bonds(nb);
    std::uint64_t seen = 0;
    for (int i = 0; i < nb; ++i)
    {
        const int a = pairs[2 * i], b = pairs[2 * i + 1];
        if (a < 0 || a >= e->n || b < 0 || b >= e->n || a == b || ((seen >> a) & 1ull) || ((seen >> b) & 1ull))
            return fail(MIPT_GB300_E_INVALID, "bonds must be pairwise disjoint and in range");
        seen |= (1ull << a) | (1ull << b);
        bonds[i] = Bond{a, b};
    }
    std::vector<PassPlan> plan;
    try
    {
        plan = plan_layer(e->n, bonds, default_tile_qubits(e->fp64), kCoalesceQubits,
                          e->fp64 ? register_bits<double>() : register_bits<float>());
    }
    catch (const std::exception &ex)
    {
        return fail(MIPT_GB300_E_INVALID, ex.what());
    }
    MG_CUDA(e->err.ensure(sizeof(int) + sizeof(std::uint64_t)));
    MG_CUDA(cudaMemset(e->err.p, 0, sizeof(int)));
    if (e->fp64)
    {
        MG_CUDA(e->gates.ensure(sizeof(double) * 32 * nb));
        MG_CUDA(cudaMemcpy(e->gates.p, m, sizeof(double) * 32 * nb, cudaMemcpyHostToDevice));
        for (const auto &p : plan)
            MG_CUDA(launch_pass<double>(static_cast<Cx<double> *>(e->data()), 1, p, e->gates.as<Cx<double>>(), 0,
                                        nullptr, 0, nullptr, 0, nullptr, 0, e->err.as<int>(), 0));
    }
    else
    {
        std::vector<float> f(32 * static_cast<std::size_t>(nb));
        for (std::size_t i = 0; i < f.size(); ++i) f[i] = static_cast<float>(m[i]);
        MG_CUDA(e->gates.ensure(sizeof(float) * f.size()));
        MG_CUDA(cudaMemcpy(e->gates.p, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
        for (const auto &p : plan)
            MG_CUDA(launch_pass<float>(static_cast<Cx<float> *>(e->data()), 1, p, e->gates.as<Cx<float>>(), 0, nullptr,
                                       0, nullptr, 0, nullptr, 0, e->err.as<int>(), 0));
    }
    MG_CUDA(cudaDeviceSynchronize());
    int err = 0;
    MG_CUDA(cudaMemcpy(&err, e->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return fail(MIPT_GB300_E_INTERNAL, "tile load wait timed out");
    return 0;
}

int mipt_gb300_engine_measure_layer(mipt_gb300_engine *e, const int *sites, int ns, int chunk_bits,
                                    const double *uniforms, const int *forced, int *outcomes, double *surprisal)
{
    if (!e || !e->data() || ns < 0 || chunk_bits < 1 || chunk_bits > 20)
        return fail(MIPT_GB300_E_INVALID, "bad measurement request");
    if (surprisal) *surprisal = 0.0;
    if (ns == 0) return 0;
    if (!sites || !uniforms) return fail(MIPT_GB300_E_INVALID, "null sites/uniforms");
    LayerMeas M{};
    std::uint64_t forced_mask = 0;
    for (int i = 0; i < ns; ++i)
    {
        if (sites[i] < 0 || sites[i] >= e->n || (i > 0 && sites[i] <= sites[i - 1]))
            return fail(MIPT_GB300_E_INVALID, "sites must be ascending and in range");
        if (forced) forced_mask |= static_cast<std::uint64_t>(forced[i] & 1) << sites[i];
    }
    const int nchunks = (ns + chunk_bits - 1) / chunk_bits;
    if (nchunks > kMaxChunks) return fail(MIPT_GB300_E_INVALID, "too many measurement chunks");
    if (e->n - std::min(default_tile_qubits(e->fp64), e->n) + kCoalesceQubits > 20)
        return fail(MIPT_GB300_E_INVALID, "state too large for the joint-measurement scratch");
    M.nchunks = nchunks;
    for (int c = 0; c < nchunks; ++c)
    {
        std::uint64_t m = 0;
        for (int i = c * chunk_bits; i < std::min(ns, (c + 1) * chunk_bits); ++i) m |= 1ull << sites[i];
        M.chunk[c] = m;
        M.uniform[c] = uniforms[c];
    }
    MG_CUDA(e->meas.ensure(sizeof(LayerMeas)));
    MG_CUDA(e->col.ensure(sizeof(Collapse)));
    MG_CUDA(e->res.ensure(sizeof(LayerResult)));
    MG_CUDA(e->part.ensure(sizeof(double) * kHistScratch));
    MG_CUDA(e->bins.ensure(sizeof(double) * kHistScratch));
    MG_CUDA(e->err.ensure(sizeof(int) + sizeof(std::uint64_t)));
    MG_CUDA(cudaMemcpy(e->meas.p, &M, sizeof(LayerMeas), cudaMemcpyHostToDevice));
    std::uint64_t *d_forced = nullptr;
    if (forced)
    {
        d_forced = reinterpret_cast<std::uint64_t *>(static_cast<char *>(e->err.p) + 8);
        MG_CUDA(cudaMemcpy(d_forced, &forced_mask, sizeof(std::uint64_t), cudaMemcpyHostToDevice));
    }
    k_reset_layers<<<1, 32>>>(e->col.as<Collapse>(), e->res.as<LayerResult>(), 1);
    MG_CUDA(cudaMemset(e->err.p, 0, sizeof(int)));
    const int kmax = default_tile_qubits(e->fp64);
    for (int c = 0; c < nchunks; ++c)
    {
        if (e->fp64)
            MG_CUDA(launch_hist<double>(static_cast<const Cx<double> *>(e->data()), 1, e->n, kmax, kCoalesceQubits, c,
                                        e->col.as<Collapse>(), 1, e->meas.as<LayerMeas>(), 1, e->part.as<double>(), false, 0));
        else
            MG_CUDA(launch_hist<float>(static_cast<const Cx<float> *>(e->data()), 1, e->n, kmax, kCoalesceQubits, c,
                                       e->col.as<Collapse>(), 1, e->meas.as<LayerMeas>(), 1, e->part.as<double>(), false, 0));
        MG_CUDA(launch_measure(1, e->n, nullptr, kmax, kCoalesceQubits, c, e->meas.as<LayerMeas>(), 1,
                               e->part.as<double>(), e->bins.as<double>(), kHistScratch, d_forced, 1,
                               e->col.as<Collapse>(), 1,
                               e->res.as<LayerResult>(), 1, e->err.as<int>(), 0));
    }
    if (e->fp64)
        MG_CUDA(launch_collapse<double>(static_cast<Cx<double> *>(e->data()), 1ull << e->n, 1, e->col.as<Collapse>(), 1, 0));
    else
        MG_CUDA(launch_collapse<float>(static_cast<Cx<float> *>(e->data()), 1ull << e->n, 1, e->col.as<Collapse>(), 1, 0));
    LayerResult r{};
    int err = 0;
    MG_CUDA(cudaMemcpy(&r, e->res.p, sizeof(LayerResult), cudaMemcpyDeviceToHost));
    MG_CUDA(cudaMemcpy(&err, e->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return fail(MIPT_GB300_E_NUMERIC, "measurement layer found a zero-norm state or no outcome with weight");
    if (outcomes)
        for (int i = 0; i < ns; ++i) outcomes[i] = static_cast<int>((r.outcome >> sites[i]) & 1ull);
    if (surprisal) *surprisal = r.surprisal;
    return 0;
}

// ----------------------------------------------------------------- batch
} // extern "C"

namespace
{
// Uploads the rho3 triples and sizes the rho3 outputs and scratch.
int set_rho3_subs(mipt_gb300_batch *b, const std::vector<int> &subs)
{
    const int n = b->cfg.n_qubits, S = static_cast<int>(subs.size() / 3);
    if (S <= 0) return fail(MIPT_GB300_E_INVALID, "no rho3 subsystems");
    for (int i = 0; i < S; ++i)
    {
        const int a = subs[3 * i], c = subs[3 * i + 1], d = subs[3 * i + 2];
        if (a < 0 || a >= n || c < 0 || c >= n || d < 0 || d >= n || a == c || a == d || c == d)
            return fail(MIPT_GB300_E_INVALID, "three-site subsystem out of range or repeated");
    }
    const std::size_t C = static_cast<std::size_t>(b->capacity);
    cudaError_t e;
    if ((e = b->subs.ensure(sizeof(int) * subs.size())) != cudaSuccess) return cuda_fail(e, "subs");
    if ((e = cudaMemcpy(b->subs.p, subs.data(), sizeof(int) * subs.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e, "subs upload");
    if ((e = b->rho3.ensure(C * S * 128 * sizeof(double))) != cudaSuccess) return cuda_fail(e, "rho3");
    if ((e = b->r3scratch.ensure(rho3_scratch_bytes(n, b->capacity, S))) != cudaSuccess)
        return cuda_fail(e, "rho3 scratch");
    if (b->per_point())
        if ((e = b->rho3_pts.ensure(static_cast<std::size_t>(b->points) * C * S * 128 * sizeof(double))) !=
            cudaSuccess)
            return cuda_fail(e, "rho3 per point");
    b->rho3_count = S;
    return 0;
}
} // namespace

extern "C" {
int mipt_gb300_batch_parity_encoded(const mipt_gb300_batch *b) { return (b && b->enc) ? 1 : 0; }

int mipt_gb300_test_withhold_tile_loads(int count)
{
    if (count < 0) return fail(MIPT_GB300_E_INVALID, "count must be >= 0");
    set_withheld_tile_loads(count);
    return 0;
}

int mipt_gb300_autotune_tile(int n_qubits, int fp64, int closed, int lattice_x, int lattice_y, int trajectories,
                             int *best_tile, int *candidates, double *ms_per_cycle, int *candidate_count)
{
    if (!best_tile || trajectories < 1 || n_qubits < 4 || n_qubits > 30 ||
        (lattice_y > 1 && lattice_x * lattice_y != n_qubits))
        return fail(MIPT_GB300_E_INVALID, "bad autotune arguments");
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return fail(MIPT_GB300_E_NODEVICE, "no CUDA device");
    return fp64 ? autotune_tile_impl<double>(n_qubits, closed, lattice_x, lattice_y, trajectories, best_tile,
                                             ms_per_cycle, candidates, candidate_count)
                : autotune_tile_impl<float>(n_qubits, closed, lattice_x, lattice_y, trajectories, best_tile,
                                            ms_per_cycle, candidates, candidate_count);
}

int mipt_gb300_batch_create(const mipt_gb300_batch_config *cfg, int capacity, mipt_gb300_batch **out)
{
    if (!cfg || !out || capacity <= 0) return fail(MIPT_GB300_E_INVALID, "null config or capacity <= 0");
    const int n = cfg->n_qubits;
    const bool lattice = cfg->lattice_y > 1;
    if (lattice)
    {
        if (cfg->lattice_x < 2 || cfg->lattice_x * cfg->lattice_y != n || n < 4 || n > 30)
            return fail(MIPT_GB300_E_INVALID, "lattice needs x >= 2, y >= 2 and x * y = n_qubits <= 30");
    }
    else if (n < 4 || n > 30 || (n % 2) != 0)
        return fail(MIPT_GB300_E_INVALID, "n_qubits must be even, 4..30");
    if (cfg->periods < 1) return fail(MIPT_GB300_E_INVALID, "periods must be >= 1");
    if (cfg->chunk_bits < 1 || cfg->chunk_bits > 20) return fail(MIPT_GB300_E_INVALID, "chunk_bits must be 1..20");
    if ((cfg->observables & (MIPT_GB300_OBS_TMI_VN | MIPT_GB300_OBS_TMI_S2)) && (n % 4) != 0)
        return fail(MIPT_GB300_E_INVALID, "TMI needs n divisible by 4");
    if (cfg->observe_every < 0) return fail(MIPT_GB300_E_INVALID, "observe_every must be >= 0");
    const bool rppu = cfg->circuit == 2 || cfg->circuit == 4;
    if (cfg->circuit != 0 && cfg->circuit != 1 && !rppu)
        return fail(MIPT_GB300_E_INVALID, "circuit must be 0/1 (Haar), 2 (FermionRPPU) or 4 (qRPPU)");
    if (rppu && (lattice || !cfg->closed))
        return fail(MIPT_GB300_E_INVALID, "RPPU circuits run on the closed 1-D ring");
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return fail(MIPT_GB300_E_NODEVICE, "no CUDA device");

    std::unique_ptr<mipt_gb300_batch> b(new mipt_gb300_batch());
    b->cfg = *cfg;
    b->capacity = capacity;
    b->T = 2 * cfg->periods + (rppu ? 1 : 0);
    b->G = n / 2;
    b->kmax = cfg->tile_qubits > 0 ? std::min(cfg->tile_qubits, kMaxLocal) : chosen_tile(*cfg, capacity);
    b->cmin = kCoalesceQubits;
    if (n - std::min(b->kmax, n) + b->cmin > 20) return fail(MIPT_GB300_E_INVALID, "tile too small for this n");
    b->dim = 1ull << n;
    b->elem = cfg->fp64 ? 16 : 8;
    b->lattice = lattice;
    b->ncolour = lattice ? 4 : 2;
    try
    {
        const auto bonds = geometry_bonds(n, cfg->closed, cfg->lattice_x, cfg->lattice_y);
        for (int colour = 0; colour < b->ncolour; ++colour)
            b->plan[colour] = plan_layer(n, bonds[colour], b->kmax, b->cmin,
                                         cfg->fp64 ? register_bits<double>() : register_bits<float>());
        if (rppu && n >= 8 && cfg->split_last && !cfg->full_state && use_parity_encoding())
        {
            // Half-size states: qubit n-1 is the parity of the others and of
            // the sector, so a bond on (q, n-1) is a parity-selected 2x2 gate
            // on q over n-1 stored qubits. Site n-1 must then be measured in
            // a chunk of its own (split_last), as the reference's encoded
            // engine does (cpp/include/mipt/cusv/engine.hpp:372-477).
            for (int colour = 0; colour < 2; ++colour)
            {
                std::vector<Bond> eb;
                for (const Bond &bd : bonds[colour])
                {
                    if (bd.q0 == n - 1)
                        eb.push_back(Bond{bd.q1, -1});
                    else if (bd.q1 == n - 1)
                        eb.push_back(Bond{bd.q0, -1});
                    else
                        eb.push_back(bd);
                }
                b->plan_enc[colour] = plan_layer(n - 1, eb, b->kmax, b->cmin,
                                                 cfg->fp64 ? register_bits<double>() : register_bits<float>());
            }
            b->can_encode = true;
        }
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
    // Observable requests of one evaluation point (trajectory 0; shifted per trajectory).
    auto range = [n](int a, int c) {
        std::vector<int> v;
        for (int i = 0; i < c; ++i) v.push_back((a + i) % n);
        return v;
    };
    auto cat = [](std::vector<int> x, const std::vector<int> &y) {
        x.insert(x.end(), y.begin(), y.end());
        return x;
    };
    const int ft = cfg->fermion_trace ? 1 : 0;
    if (cfg->observables & MIPT_GB300_OBS_SVN_HALF)
    {
        b->col_half_vn = static_cast<int>(b->reqs.size());
        b->reqs.push_back(EntReq{0, 1, ft, range(0, n / 2), 0});
    }
    if (cfg->observables & MIPT_GB300_OBS_S2_HALF)
    {
        b->col_half_s2 = static_cast<int>(b->reqs.size());
        b->reqs.push_back(EntReq{0, 2, ft, range(0, n / 2), 0});
    }
    if (cfg->observables & (MIPT_GB300_OBS_TMI_VN | MIPT_GB300_OBS_TMI_S2))
    {
        if (cfg->tmi_cycles < 0 || cfg->tmi_cycles > n / 4)
            return fail(MIPT_GB300_E_INVALID, "tmi_cycles must be 0..n/4");
        b->tmi_cycles = std::max(1, cfg->tmi_cycles);
    }
    for (int order = 1; order <= 2; ++order)
    {
        const int flag = order == 1 ? MIPT_GB300_OBS_TMI_VN : MIPT_GB300_OBS_TMI_S2;
        if (!(cfg->observables & flag)) continue;
        const int q = n / 4;
        auto &slots = order == 1 ? b->tmi_vn : b->tmi_s2;
        for (int c = 0; c < b->tmi_cycles; ++c)
        {
            const auto A = range(c, q), B = range(c + q, q), C = range(c + 2 * q, q), D = range(c + 3 * q, q);
            const std::vector<std::vector<int>> sets = {A, B, C, D, cat(A, B), cat(A, C), cat(B, C)};
            for (const auto &s : sets)
            {
                slots.push_back(static_cast<int>(b->reqs.size()));
                b->reqs.push_back(EntReq{0, order, ft, s, 0});
            }
        }
    }
    b->reqs_per_point = static_cast<int>(b->reqs.size());
    b->points = cfg->observe_every > 0 ? b->T / cfg->observe_every : 1;

    const std::size_t C = static_cast<std::size_t>(capacity), T = b->T;
    cudaError_t e;
    if ((e = b->states.ensure(C * b->dim * b->elem)) != cudaSuccess) return cuda_fail(e, "state allocation");
    if (b->can_encode)
    {
        if ((e = b->cstates.ensure(C * (b->dim / 2) * b->elem)) != cudaSuccess)
            return cuda_fail(e, "parity-sector state allocation");
        if ((e = b->d_sector.ensure(C)) != cudaSuccess) return cuda_fail(e, "sector allocation");
    }
    if ((e = b->gates.ensure(C * T * b->G * 16 * b->elem)) != cudaSuccess) return cuda_fail(e, "gate allocation");
    if ((e = b->meas.ensure(C * T * sizeof(LayerMeas))) != cudaSuccess) return cuda_fail(e, "meas allocation");
    if ((e = b->forced.ensure(C * T * sizeof(std::uint64_t))) != cudaSuccess) return cuda_fail(e, "forced allocation");
    if ((e = b->col.ensure(C * T * sizeof(Collapse))) != cudaSuccess) return cuda_fail(e, "collapse allocation");
    if ((e = b->res.ensure(C * T * sizeof(LayerResult))) != cudaSuccess) return cuda_fail(e, "result allocation");
    if ((e = b->part.ensure(C * kHistScratch * sizeof(double))) != cudaSuccess) return cuda_fail(e, "partials");
    if ((e = b->bins.ensure(C * (std::size_t{1} << cfg->chunk_bits) * sizeof(double))) != cudaSuccess)
        return cuda_fail(e, "bins");
    if ((e = b->err.ensure(sizeof(int))) != cudaSuccess) return cuda_fail(e, "error flag");
    if (b->reqs_per_point > 0)
        if ((e = b->ent.ensure(C * b->points * b->reqs_per_point * sizeof(double))) != cudaSuccess)
            return cuda_fail(e, "entropy outputs");
    if (cfg->rho3)
    {
        // Default triples: the ring {s, s+1, s+2} in 1-D; in 2-D the horizontal
        // then the vertical lattice triples (cpp/include/mipt/rdm.hpp:92-127).
        std::vector<int> subs;
        if (lattice)
        {
            const int X = cfg->lattice_x, Y = cfg->lattice_y;
            for (int r = 0; r < Y; ++r)
                for (int c = 0; c < X; ++c)
                    for (int k = 0; k < 3; ++k) subs.push_back(r * X + (c + k) % X);
            for (int c = 0; c < X; ++c)
                for (int r = 0; r < Y; ++r)
                    for (int k = 0; k < 3; ++k) subs.push_back(((r + k) % Y) * X + c);
        }
        else
        {
            for (int s = 0; s < n; ++s)
                for (int k = 0; k < 3; ++k) subs.push_back((s + k) % n);
        }
        const int rc = set_rho3_subs(b.get(), subs);
        if (rc) return rc;
    }
    if ((e = b->h_gates.ensure(C * T * b->G * 16 * b->elem)) != cudaSuccess) return cuda_fail(e, "pinned gates");
    if ((e = b->h_meas.ensure(C * T * sizeof(LayerMeas))) != cudaSuccess) return cuda_fail(e, "pinned meas");
    if ((e = b->h_forced.ensure(C * T * sizeof(std::uint64_t))) != cudaSuccess) return cuda_fail(e, "pinned forced");
    if ((e = b->h_res.ensure(C * T * sizeof(LayerResult))) != cudaSuccess) return cuda_fail(e, "pinned results");
    b->custom_init.assign(C, 0);
    b->sector.assign(C, 0);
    b->folded.assign(C, -1);
    *out = b.release();
    return 0;
}

void mipt_gb300_batch_destroy(mipt_gb300_batch *b) { delete b; }

} // extern "C"

namespace
{
// Packs drawn trajectories into the batch's pinned layer tables and uploads
// them (gates in the state's precision, measured-site chunks with their
// uniforms, optional forced outcomes).
int upload_draws(mipt_gb300_batch *b, const std::vector<TrajectoryDraw> &draws, const std::uint64_t *forced)
{
    const int count = static_cast<int>(draws.size());
    const int n = b->cfg.n_qubits, T = b->T, G = b->G, cb = b->cfg.chunk_bits;
    b->count = count;
    b->measured.assign(static_cast<std::size_t>(count) * T, 0);
    b->any_meas.assign(T, 0);
    b->fusable.assign(T, 1);
    b->direct_hist.assign(static_cast<std::size_t>(T) * kMaxChunks, 1);
    b->max_chunks.assign(T, 0);
    b->has_forced = forced != nullptr;
    // Parity-sector execution needs every trajectory in a definite sector.
    b->enc = b->can_encode;
    for (int i = 0; i < count && b->enc; ++i)
        if (b->sector[i] < 0) b->enc = false;
    const int ne = b->enc ? n - 1 : n;
    const auto *plans = b->enc ? b->plan_enc : b->plan;
    LayerMeas *hm = b->h_meas.as<LayerMeas>();
    std::uint64_t *hf = b->h_forced.as<std::uint64_t>();
    for (int i = 0; i < count; ++i)
    {
        const TrajectoryDraw &d = draws[i];
        // FermionRPPU: within a parity sector the closure's JW string is a
        // diagonal on the closure bond itself -- (-1)^(n_hi * (n_lo + n_hi)) in
        // the even sector, (-1)^(n_hi * n_lo) in the odd one -- so it folds into
        // the closure gate (cpp/include/mipt/cusv/parity.hpp:38-45 makes the
        // same reduction for the even sector).
        const int fold = b->cfg.circuit == 2 ? b->sector[i] : -1;
        b->folded[i] = fold;
        std::vector<std::complex<double>> folded_layer;
        for (int t = 0; t < T; ++t)
        {
            const std::size_t slot = static_cast<std::size_t>(i) * T + t;
            // Gates: the draw's bond list matches the planned brickwork order.
            const std::complex<double> *src = &d.bond_u[static_cast<std::size_t>(t) * G * 16];
            if (fold >= 0 && (t & 1))
            {
                // The closure bond is the layer's last, stored for (n-1, 0):
                // index j = n_{n-1} + 2 n_0.
                folded_layer.assign(src, src + static_cast<std::size_t>(G) * 16);
                const double dg[4] = {1.0, fold == 0 ? -1.0 : 1.0, 1.0, fold == 0 ? 1.0 : -1.0};
                std::complex<double> *u = folded_layer.data() + static_cast<std::size_t>(G - 1) * 16;
                for (int r = 0; r < 4; ++r)
                    for (int c = 0; c < 4; ++c) u[4 * r + c] *= dg[r] * dg[c];
                src = folded_layer.data();
            }
            std::vector<std::complex<double>> enc_layer;
            if (b->enc)
            {
                // The layer's last bond touches qubit n-1: (n-2, n-1) in even
                // layers (index bit0 = n-2), (n-1, 0) in odd ones (bit0 =
                // n-1). As a parity-selected 2x2 on the other qubit q it keeps
                // the pair (00, 11) when q's partner bit equals q (entries
                // 0..3) and the pair (01, 10) otherwise (entries 4..7); the
                // stored order puts the block for an even parity of the other
                // stored bits first, so sector 1 swaps the two.
                enc_layer.assign(src, src + static_cast<std::size_t>(G) * 16);
                std::complex<double> *u = enc_layer.data() + static_cast<std::size_t>(G - 1) * 16;
                const std::complex<double> g[16] = {u[0], u[1], u[2],  u[3],  u[4],  u[5],  u[6],  u[7],
                                                    u[8], u[9], u[10], u[11], u[12], u[13], u[14], u[15]};
                auto G4 = [&](int r, int c) { return g[4 * r + c]; };
                const std::complex<double> E[4] = {G4(0, 0), G4(0, 3), G4(3, 0), G4(3, 3)};
                std::complex<double> O[4];
                if ((t & 1) == 0)
                {
                    O[0] = G4(2, 2), O[1] = G4(2, 1), O[2] = G4(1, 2), O[3] = G4(1, 1);
                }
                else
                {
                    O[0] = G4(1, 1), O[1] = G4(1, 2), O[2] = G4(2, 1), O[3] = G4(2, 2);
                }
                const bool swap = b->sector[i] == 1;
                for (int e = 0; e < 4; ++e)
                {
                    u[e] = swap ? O[e] : E[e];
                    u[4 + e] = swap ? E[e] : O[e];
                    u[8 + e] = u[12 + e] = 0.0;
                }
                src = enc_layer.data();
            }
            if (b->cfg.fp64)
            {
                double *dst = b->h_gates.as<double>() + slot * G * 32;
                for (int e = 0; e < d.bond_count[t] * 16; ++e)
                {
                    dst[2 * e] = src[e].real();
                    dst[2 * e + 1] = src[e].imag();
                }
            }
            else
            {
                float *dst = b->h_gates.as<float>() + slot * G * 32;
                for (int e = 0; e < d.bond_count[t] * 16; ++e)
                {
                    dst[2 * e] = static_cast<float>(src[e].real());
                    dst[2 * e + 1] = static_cast<float>(src[e].imag());
                }
            }
            const std::uint64_t mask = d.measured[t];
            b->measured[slot] = mask;
            LayerMeas M{};
            // Sites in ascending chunks of cb; with split_last, site n-1 forms
            // a final chunk of its own.
            const std::uint64_t last = 1ull << (n - 1);
            const bool alone = d.split_last && (mask & last);
            const std::uint64_t plain = alone ? (mask & ~last) : mask;
            const int m = __builtin_popcountll(plain);
            M.nchunks = (m + cb - 1) / cb + (alone ? 1 : 0);
            if (M.nchunks > kMaxChunks) return fail(MIPT_GB300_E_INVALID, "too many measurement chunks per layer");
            int c = -1, in_chunk = cb;
            for (int q = 0; q < n; ++q)
            {
                if (!((plain >> q) & 1ull)) continue;
                if (in_chunk == cb)
                {
                    ++c;
                    in_chunk = 0;
                }
                M.chunk[c] |= 1ull << q;
                ++in_chunk;
            }
            if (alone) M.chunk[++c] = last;
            for (int cc = 0; cc < M.nchunks; ++cc)
            {
                M.uniform[cc] = d.uniforms[d.uniform_offset[t] + cc];
                if (M.chunk[cc] >> ne) continue; // the parity chunk of a half-size state
                PassGeom hg{};
                histogram_geometry(ne, b->kmax, b->cmin, M.chunk[cc], hg);
                for (int li = 0; li < hg.k; ++li)
                    if ((M.chunk[cc] >> hg.pos[li]) & 1ull) b->direct_hist[static_cast<std::size_t>(t) * kMaxChunks + cc] = 0;
            }
            hm[slot] = M;
            hf[slot] = forced ? forced[slot] : 0ull;
            if (M.nchunks > 0)
            {
                b->any_meas[t] = 1;
                b->max_chunks[t] = std::max(b->max_chunks[t], M.nchunks);
                const PassGeom &hg = fused_hist_geometry(plans[t % b->ncolour].back(), b->cfg.fp64 == 0);
                const int ml = local_measured_count(hg, M.chunk[0]);
                if ((std::size_t{1} << (hg.n_nl + ml)) > kHistScratch) b->fusable[t] = 0;
                if (M.chunk[0] >> ne) b->fusable[t] = 0;
            }
        }
    }
    const std::size_t C = static_cast<std::size_t>(count);
    if (b->enc)
    {
        b->enc_sector.assign(b->sector.begin(), b->sector.begin() + count);
        std::vector<signed char> sec(b->sector.begin(), b->sector.begin() + count);
        MG_CUDA(cudaMemcpy(b->d_sector.p, sec.data(), sec.size(), cudaMemcpyHostToDevice));
    }
    MG_CUDA(cudaMemcpy(b->gates.p, b->h_gates.p, C * T * G * 16 * b->elem, cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(b->meas.p, b->h_meas.p, C * T * sizeof(LayerMeas), cudaMemcpyHostToDevice));
    if (forced) MG_CUDA(cudaMemcpy(b->forced.p, b->h_forced.p, C * T * sizeof(std::uint64_t), cudaMemcpyHostToDevice));
    b->executed = false;
    return 0;
}
} // namespace

extern "C" {
int mipt_gb300_batch_prepare_haar(mipt_gb300_batch *b, const std::uint64_t *seeds, const double *p, int count,
                                  const std::uint64_t *forced)
{
    if (!b || !seeds || !p || count <= 0 || count > b->capacity)
        return fail(MIPT_GB300_E_INVALID, "bad batch prepare arguments");
    std::vector<TrajectoryDraw> draws;
    try
    {
        if (b->lattice)
            draw_haar_lattice_batch(seeds, p, count, b->cfg.lattice_x, b->cfg.lattice_y, b->T, b->cfg.chunk_bits,
                                    draws, b->cfg.host_threads);
        else if (b->cfg.circuit == 2 || b->cfg.circuit == 4)
            draw_rppu_batch(seeds, p, count, b->cfg.n_qubits, b->cfg.periods, b->cfg.chunk_bits,
                            b->cfg.split_last != 0, b->T, draws, b->cfg.host_threads);
        else
            draw_haar_batch(seeds, p, count, b->cfg.n_qubits, b->cfg.periods, b->cfg.closed != 0,
                            b->cfg.chunk_bits, draws, b->cfg.host_threads);
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
    return upload_draws(b, draws, forced);
}

int mipt_gb300_batch_prepare_haar_workspace(mipt_gb300_batch *b, const std::uint32_t *seeds, const double *p,
                                            int count)
{
    if (!b || !seeds || !p || count <= 0 || count > b->capacity)
        return fail(MIPT_GB300_E_INVALID, "bad batch prepare arguments");
    if (b->lattice) return fail(MIPT_GB300_E_INVALID, "the workspace draw is the 1-D brickwork");
    std::vector<TrajectoryDraw> draws;
    try
    {
        if (b->cfg.circuit == 2 || b->cfg.circuit == 4)
            draw_rppu_workspace_batch(seeds, p, count, b->cfg.n_qubits, 2 * b->cfg.periods, b->cfg.chunk_bits,
                                      b->cfg.split_last != 0, b->T, draws, b->cfg.host_threads);
        else
            draw_haar_workspace_batch(seeds, p, count, b->cfg.n_qubits, b->T, b->cfg.closed != 0,
                                      b->cfg.chunk_bits, draws, b->cfg.host_threads);
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
    return upload_draws(b, draws, nullptr);
}

int mipt_gb300_batch_set_observation_steps(mipt_gb300_batch *b, const int *steps, int count)
{
    if (!b || count < 0 || (count > 0 && !steps)) return fail(MIPT_GB300_E_INVALID, "bad observation schedule");
    std::vector<int> point;
    if (count > 0)
    {
        point.assign(static_cast<std::size_t>(b->T) + 1, -1);
        for (int i = 0; i < count; ++i)
        {
            if (steps[i] < 0 || steps[i] > b->T || (i > 0 && steps[i] <= steps[i - 1]))
                return fail(MIPT_GB300_E_INVALID, "observation steps must be increasing within 0..layers");
            point[static_cast<std::size_t>(steps[i])] = i;
        }
    }
    const int points = count > 0 ? count : (b->cfg.observe_every > 0 ? b->T / b->cfg.observe_every : 1);
    const std::size_t C = static_cast<std::size_t>(b->capacity);
    cudaError_t e;
    if (b->reqs_per_point > 0)
        if ((e = b->ent.ensure(C * points * b->reqs_per_point * sizeof(double))) != cudaSuccess)
            return cuda_fail(e, "entropy outputs");
    if (b->cfg.rho3 && (count > 0 || b->cfg.observe_every > 0))
        if ((e = b->rho3_pts.ensure(static_cast<std::size_t>(points) * C * b->rho3_count * 128 * sizeof(double))) !=
            cudaSuccess)
            return cuda_fail(e, "rho3 per point");
    b->obs_point = std::move(point);
    b->points = points;
    b->executed = false;
    return 0;
}

int mipt_gb300_batch_set_initial_state(mipt_gb300_batch *b, int index, const double *host_ri)
{
    if (!b || !host_ri || index < 0 || index >= b->capacity)
        return fail(MIPT_GB300_E_INVALID, "bad initial-state arguments");
    const std::size_t dim = b->dim;
    void *dst = static_cast<char *>(b->states.p) + static_cast<std::size_t>(index) * dim * b->elem;
    if (b->cfg.fp64)
        MG_CUDA(cudaMemcpy(dst, host_ri, dim * 16, cudaMemcpyHostToDevice));
    else
    {
        std::vector<float> f(2 * dim);
        for (std::size_t i = 0; i < 2 * dim; ++i) f[i] = static_cast<float>(host_ri[i]);
        MG_CUDA(cudaMemcpy(dst, f.data(), dim * 8, cudaMemcpyHostToDevice));
    }
    b->custom_init[static_cast<std::size_t>(index)] = 1;
    b->sector[static_cast<std::size_t>(index)] = -1;
    return 0;
}

int mipt_gb300_batch_set_initial_states(mipt_gb300_batch *b, const std::uint64_t *seeds, int kind, int fixed_parity,
                                        int count, int *parity_sectors)
{
    if (!b || !seeds || count <= 0 || count > b->capacity || (kind != 0 && kind != 1))
        return fail(MIPT_GB300_E_INVALID, "bad initial-state arguments");
    const int n = b->cfg.n_qubits;
    const std::size_t dim = b->dim, bytes = dim * b->elem;
    // Host threads draw into their own staging buffers, bounded to 8 GiB.
    int threads = b->cfg.host_threads > 0 ? b->cfg.host_threads
                                          : static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    threads = std::max(1, std::min<int>({threads, count, static_cast<int>(std::max<std::size_t>(1, (8ull << 30) / bytes))}));
    std::vector<std::vector<char>> stage(static_cast<std::size_t>(threads), std::vector<char>(bytes));
    std::vector<int> sector(static_cast<std::size_t>(count), -1);
    for (int first = 0; first < count; first += threads)
    {
        const int group = std::min(threads, count - first);
        std::vector<std::thread> pool;
        std::atomic<bool> failed{false};
        std::string what;
        std::mutex what_mu;
        for (int k = 0; k < group; ++k)
            pool.emplace_back([&, k]() {
                try
                {
                    const int i = first + k;
                    sector[i] = b->cfg.fp64
                                    ? draw_initial_state<double>(seeds[i], n, kind, fixed_parity != 0,
                                                                 reinterpret_cast<std::complex<double> *>(stage[k].data()))
                                    : draw_initial_state<float>(seeds[i], n, kind, fixed_parity != 0,
                                                                reinterpret_cast<std::complex<float> *>(stage[k].data()));
                }
                catch (const std::exception &e)
                {
                    std::lock_guard<std::mutex> lock(what_mu);
                    what = e.what();
                    failed = true;
                }
            });
        for (auto &th : pool) th.join();
        if (failed) return fail(MIPT_GB300_E_INVALID, what.c_str());
        for (int k = 0; k < group; ++k)
        {
            MG_CUDA(cudaMemcpy(static_cast<char *>(b->states.p) + static_cast<std::size_t>(first + k) * bytes,
                               stage[k].data(), bytes, cudaMemcpyHostToDevice));
            b->custom_init[static_cast<std::size_t>(first + k)] = 1;
            b->sector[static_cast<std::size_t>(first + k)] = sector[first + k];
        }
    }
    if (parity_sectors) std::copy(sector.begin(), sector.end(), parity_sectors);
    return 0;
}

int mipt_gb300_draw_initial_state(std::uint64_t seed, int n_qubits, int kind, int fixed_parity, int fp64,
                                  double *host_ri, int *parity_sector)
{
    if (!host_ri || n_qubits < 1 || n_qubits > 30 || (kind != 0 && kind != 1))
        return fail(MIPT_GB300_E_INVALID, "bad initial-state arguments");
    try
    {
        const std::size_t dim = std::size_t{1} << n_qubits;
        int sector;
        if (fp64)
            sector = draw_initial_state<double>(seed, n_qubits, kind, fixed_parity != 0,
                                                reinterpret_cast<std::complex<double> *>(host_ri));
        else
        {
            std::vector<std::complex<float>> f(dim);
            sector = draw_initial_state<float>(seed, n_qubits, kind, fixed_parity != 0, f.data());
            for (std::size_t i = 0; i < dim; ++i)
            {
                host_ri[2 * i] = f[i].real();
                host_ri[2 * i + 1] = f[i].imag();
            }
        }
        if (parity_sector) *parity_sector = sector;
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
    return 0;
}

} // extern "C"

namespace
{
template <typename Real>
int batch_execute(mipt_gb300_batch *b, cudaStream_t s)
{
    const int n = b->cfg.n_qubits, T = b->T, G = b->G, count = b->count;
    Cx<Real> *states = b->states.as<Cx<Real>>();
    // Parity-sector execution: the layers run on the compact states (ne
    // stored qubits); observables and the final state are expanded into
    // `states`.
    const bool enc = b->enc;
    const int ne = enc ? n - 1 : n;
    const std::uint64_t edim = 1ull << ne;
    Cx<Real> *xs = enc ? b->cstates.as<Cx<Real>>() : states;
    const signed char *sec = enc ? b->d_sector.as<signed char>() : nullptr;
    const auto *plans = enc ? b->plan_enc : b->plan;
    const int xgrid = static_cast<int>(std::min<std::uint64_t>(152ull * 16, (edim * 2 * count + 255) / 256));
    const Cx<Real> *gates = b->gates.as<Cx<Real>>();
    LayerMeas *meas = b->meas.as<LayerMeas>();
    Collapse *col = b->col.as<Collapse>();
    LayerResult *res = b->res.as<LayerResult>();
    const std::uint64_t *forced = b->has_forced ? b->forced.as<std::uint64_t>() : nullptr;
    long long L = 0;
    b->marks.clear();
    b->next_event = 0;
    b->ws.stage.rewind();
    {
        Mark m(b, K_OTHER, s);
        int custom = 0;
        for (int i = 0; i < count; ++i) custom += b->custom_init[i] ? 1 : 0;
        if (custom == 0)
        {
            MG_CUDA(launch_init_zero<Real>(xs, edim, count, s));
            ++L;
        }
        else
            for (int i = 0; i < count; ++i)
                if (!b->custom_init[i])
                {
                    MG_CUDA(launch_init_zero<Real>(xs + static_cast<std::size_t>(i) * edim, edim, 1, s));
                    ++L;
                }
                else if (enc)
                {
                    k_compact<Real><<<static_cast<int>(std::min<std::uint64_t>(4096, (edim + 255) / 256)), 256, 0,
                                      s>>>(states, xs, ne, i, sec);
                    MG_CUDA(cudaGetLastError());
                    ++L;
                }
        std::fill(b->custom_init.begin(), b->custom_init.end(), 0);
    }
    // FermionRPPU: closure strings not folded at upload run as diagonal passes
    // on those trajectories; a fold for another sector than the state's is an
    // ordering error of the caller.
    std::vector<int> unfolded;
    if (b->cfg.circuit == 2)
        for (int i = 0; i < count; ++i)
        {
            if (b->folded[i] < 0)
                unfolded.push_back(i);
            else if (b->folded[i] != b->sector[i])
                return fail(MIPT_GB300_E_INVALID,
                            "FermionRPPU: set the initial states before mipt_gb300_batch_prepare_haar*");
        }
    if (enc)
        for (int i = 0; i < count; ++i)
            if (b->sector[i] != b->enc_sector[i])
                return fail(MIPT_GB300_E_INVALID, "parity-sector batch: set the initial states before "
                                                  "mipt_gb300_batch_prepare_haar* (the gates are uploaded for "
                                                  "the initial states' sectors)");
    std::fill(b->sector.begin(), b->sector.end(), 0);
    const std::size_t slots = static_cast<std::size_t>(count) * T;
    k_reset_layers<<<std::min<std::size_t>((slots + 255) / 256, 1024), 256, 0, s>>>(col, res, slots);
    ++L;
    MG_CUDA(cudaMemsetAsync(b->err.p, 0, sizeof(int), s));
    // A timed-out Gram wait of an earlier execute is reported once.
    if (b->ws.err.p) MG_CUDA(cudaMemsetAsync(b->ws.err.p, 0, sizeof(int), s));
    if (b->ws.eig_err.p) MG_CUDA(cudaMemsetAsync(b->ws.eig_err.p, 0, sizeof(int), s));
    if (b->reqs_per_point > 0)
    {
        const std::size_t ne = static_cast<std::size_t>(count) * b->points * b->reqs_per_point;
        k_fill_double<<<std::min<std::size_t>((ne + 255) / 256, 1024), 256, 0, s>>>(b->ent.as<double>(), ne, NAN);
        ++L;
    }
    // Observations of point `point` on the current states (`pending`: the
    // collapse each trajectory still owes, or null).
    // Expanded parity-sector states carry their collapse already; their
    // entropies get outcome-only records (stride 1) instead.
    auto mask_records = [&](const Collapse *pending) -> const Collapse * {
        k_mask_records<<<(count + 127) / 128, 128, 0, s>>>(pending, T, count, b->mask_col.as<Collapse>());
        ++L;
        return b->mask_col.as<Collapse>();
    };
    if (enc) MG_CUDA(b->mask_col.ensure(sizeof(Collapse) * static_cast<std::size_t>(b->capacity)));
    auto observe = [&](int point, const Collapse *pending) -> int {
        std::size_t pstride = T;
        if (enc)
        {
            Mark m(b, K_OTHER, s);
            k_expand<Real><<<xgrid, 256, 0, s>>>(xs, states, ne, count, sec, pending, T);
            MG_CUDA(cudaGetLastError());
            ++L;
            if (pending != nullptr)
            {
                pending = mask_records(pending);
                MG_CUDA(cudaGetLastError());
                pstride = 1;
            }
        }
        if (b->reqs_per_point > 0)
        {
            std::vector<EntReq> reqs;
            for (int i = 0; i < count; ++i)
                for (int r = 0; r < b->reqs_per_point; ++r)
                {
                    EntReq q = b->reqs[r];
                    q.traj = i;
                    q.out = (i * b->points + point) * b->reqs_per_point + r;
                    reqs.push_back(q);
                }
            Mark m(b, K_OBS, s);
            const int rc = run_entropies<Real>(states, n, reqs, pending, pstride, b->ws, s, b->ent.as<double>(), L);
            if (rc) return rc;
        }
        if (b->cfg.rho3)
        {
            Mark m(b, K_OBS, s);
            MG_CUDA(rho3_sweep<Real>(states, n, count, b->subs.as<int>(), b->rho3_count,
                                     b->cfg.fermion_trace ? 1 : 0, pending, pstride,
                                     b->rho3_pts.as<double>() +
                                         static_cast<std::size_t>(point) * b->capacity * b->rho3_count * 128,
                                     b->r3scratch.p, b->r3scratch.bytes, s));
            L += 2;
        }
        return 0;
    };
    const bool sched = !b->obs_point.empty();
    if (sched && b->obs_point[0] >= 0)
    {
        const int rc = observe(b->obs_point[0], nullptr);
        if (rc) return rc;
    }
    const std::size_t gstride = static_cast<std::size_t>(T) * G * 16;
    for (int t = 0; t < T; ++t)
    {
        const auto &plan = plans[t % b->ncolour];
        const bool fuse = b->any_meas[t] && b->fusable[t];
        // Fermionic closure: the odd layer's gates run between two JW strings;
        // every other odd-layer bond lies inside the string and preserves its
        // parity, so the bracket covers the whole layer.
        const bool jw = !unfolded.empty() && (t & 1);
        auto jw_closure = [&]() {
            Mark m(b, K_OTHER, s);
            const int grid = static_cast<int>(std::min<std::uint64_t>(4 * 152, (b->dim / 2 + 255) / 256));
            for (int i : unfolded)
            {
                k_jw_closure<Real><<<std::max(1, grid), 256, 0, s>>>(states + static_cast<std::size_t>(i) * b->dim,
                                                                      n, 1);
                ++L;
            }
        };
        if (jw) jw_closure();
        // After a measurement the layer's first pass visits only the tiles
        // that agree with the outcome on its non-local measured bits (the
        // rest are zero); the second pass zeroes those bits' other values as
        // it loads.
        const bool sparse = t > 0 && plan.size() >= 2 && use_sparse_pass() &&
                            sparse_pass_supported(plan[0], sizeof(Real) == 4, count) &&
                            sparse_pass_supported(plan[1], sizeof(Real) == 4, count);
        for (std::size_t pi = 0; pi < plan.size(); ++pi)
        {
            const Collapse *cin = (pi == 0 && t > 0) ? col + (t - 1) : nullptr;
            std::uint64_t keep = ~0ull;
            int scaled = 1;
            if (sparse && pi == 1)
            {
                cin = col + (t - 1);
                keep = nonlocal_mask(plan[0].geom);
                scaled = 0;
            }
            const bool last = pi + 1 == plan.size();
            Mark m(b, K_PASS, s);
            MG_CUDA(launch_pass<Real>(xs, count, plan[pi], gates + static_cast<std::size_t>(t) * G * 16, gstride,
                                      cin, T, meas + t, T, b->part.as<double>(), last && fuse ? 1 : 0,
                                      b->err.as<int>(), s, keep, scaled, sparse && pi == 0 ? 1 : 0, enc ? 1 : 0));
            ++L;
        }
        if (jw) jw_closure();
        if (b->any_meas[t])
        {
            for (int ci = 0; ci < b->max_chunks[t]; ++ci)
            {
                const bool fused = ci == 0 && fuse;
                if (!fused)
                {
                    Mark m(b, K_HIST, s);
                    MG_CUDA(launch_hist<Real>(xs, count, ne, b->kmax, b->cmin, ci, col + t, T, meas + t, T,
                                              b->part.as<double>(),
                                              b->direct_hist[static_cast<std::size_t>(t) * kMaxChunks + ci] != 0, s,
                                              sec));
                    ++L;
                }
                Mark m(b, K_MEASURE, s);
                MG_CUDA(launch_measure(count, ne, fused ? &fused_hist_geometry(plan.back(), sizeof(Real) == 4) : nullptr,
                                       b->kmax, b->cmin, ci, meas + t, T,
                                       b->part.as<double>(), b->bins.as<double>(),
                                       std::size_t{1} << b->cfg.chunk_bits, forced ? forced + t : nullptr, T,
                                       col + t, T, res + t, T, b->err.as<int>(), s, sec));
                ++L;
            }
        }
        int point = -1;
        if (sched)
            point = b->obs_point[t + 1];
        else if (b->cfg.observe_every > 0 && (t + 1) % b->cfg.observe_every == 0)
            point = (t + 1) / b->cfg.observe_every - 1;
        if (point >= 0)
        {
            const int rc = observe(point, col + t);
            if (rc) return rc;
        }
    }
    // Final-state entropies. Full states are observed with the last layer's
    // collapse still pending (so the measured sites leave the Gram), parity-
    // sector states after their expansion.
    auto final_entropies = [&](const Collapse *fc, std::size_t fstride) -> int {
        std::vector<EntReq> reqs;
        for (int i = 0; i < count; ++i)
            for (int r = 0; r < b->reqs_per_point; ++r)
            {
                EntReq q = b->reqs[r];
                q.traj = i;
                q.out = i * b->reqs_per_point + r;
                reqs.push_back(q);
            }
        Mark m(b, K_OBS, s);
        return run_entropies<Real>(states, n, reqs, fc, fstride, b->ws, s, b->ent.as<double>(), L);
    };
    const bool final_obs = b->reqs_per_point > 0 && !b->per_point();
    if (final_obs && !enc)
    {
        const int rc = T > 0 ? final_entropies(col + (T - 1), T) : final_entropies(nullptr, 0);
        if (rc) return rc;
    }
    // Leave every trajectory in its collapsed, normalised final state.
    {
        Mark m(b, K_OTHER, s);
        if (enc)
        {
            k_expand<Real><<<xgrid, 256, 0, s>>>(xs, states, ne, count, sec, col + (T - 1), T);
            MG_CUDA(cudaGetLastError());
        }
        else
            MG_CUDA(launch_collapse<Real>(states, b->dim, count, col + (T - 1), T, s));
    }
    ++L;
    if (final_obs && enc)
    {
        const Collapse *mc = mask_records(col + (T - 1));
        MG_CUDA(cudaGetLastError());
        const int rc = final_entropies(mc, 1);
        if (rc) return rc;
    }
    if (b->cfg.rho3)
    {
        // The final-state blocks are written in every mode.
        Mark m(b, K_OBS, s);
        MG_CUDA(rho3_sweep<Real>(states, n, count, b->subs.as<int>(), b->rho3_count, b->cfg.fermion_trace ? 1 : 0,
                                 nullptr, 0, b->rho3.as<double>(), b->r3scratch.p, b->r3scratch.bytes, s));
        L += 2;
    }
    b->launches = L;
    b->executed = true;
    return 0;
}
} // namespace

namespace
{
int execute_any(mipt_gb300_batch *b, cudaStream_t s)
{
    try
    {
        return b->cfg.fp64 ? batch_execute<double>(b, s) : batch_execute<float>(b, s);
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INTERNAL, e.what());
    }
}

// Everything on the host that decides which kernels an execute enqueues and
// with which arguments (the device buffers themselves are fixed per batch).
std::vector<long long> structure_key(const mipt_gb300_batch *b)
{
    std::vector<long long> k{b->count, b->has_forced ? 1 : 0, b->points, b->reqs_per_point, b->rho3_count,
                             b->tmi_cycles, b->enc ? 1 : 0};
    for (char c : b->any_meas) k.push_back(c);
    for (char c : b->fusable) k.push_back(c);
    for (int c : b->max_chunks) k.push_back(c);
    for (char c : b->direct_hist) k.push_back(c);
    for (int c : b->obs_point) k.push_back(c);
    for (char c : b->custom_init) k.push_back(c);
    for (int i = 0; i < b->count && b->cfg.circuit == 2; ++i)
    {
        k.push_back(b->folded[i]);
        k.push_back(b->sector[i]);
    }
    for (const auto &r : b->reqs)
    {
        k.push_back(r.order * 4 + r.fermion);
        k.push_back(static_cast<long long>(r.kept.size()));
        for (int q : r.kept) k.push_back(q);
    }
    return k;
}

bool graph_ready(const mipt_gb300_batch *b)
{
    for (char c : b->custom_init)
        if (c) return false;
    return !b->profile;
}

// Captures one execute of each batch into a graph, batch i on streams[i]
// forked from and joined into `root`. The caller has run each batch once
// normally, so every buffer has its final size and no capture allocates.
int capture_graph(mipt_gb300_batch *const *bs, int nb, cudaStream_t root, cudaStream_t *streams,
                  cudaEvent_t *events, cudaGraphExec_t *exec)
{
    cudaError_t e = cudaStreamBeginCapture(root, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
    int rc = 0;
    if (nb == 1 && streams[0] == root)
        rc = execute_any(bs[0], root);
    else
    {
        e = cudaEventRecord(events[nb], root);
        for (int i = 0; i < nb && !rc && e == cudaSuccess; ++i)
        {
            e = cudaStreamWaitEvent(streams[i], events[nb], 0);
            if (e == cudaSuccess) rc = execute_any(bs[i], streams[i]);
            if (!rc && e == cudaSuccess) e = cudaEventRecord(events[i], streams[i]);
            if (!rc && e == cudaSuccess) e = cudaStreamWaitEvent(root, events[i], 0);
        }
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(root, &g);
    if (rc || e != cudaSuccess || ee != cudaSuccess)
    {
        if (g) cudaGraphDestroy(g);
        if (rc) return rc;
        return cuda_fail(e != cudaSuccess ? e : ee, "graph capture of a batch execute");
    }
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return 0;
}
} // namespace

extern "C" {

int mipt_gb300_batch_execute(mipt_gb300_batch *b, void *stream)
{
    if (!b || b->count <= 0) return fail(MIPT_GB300_E_INVALID, "batch has no prepared trajectories");
    return execute_any(b, static_cast<cudaStream_t>(stream));
}

int mipt_gb300_batch_execute_graph(mipt_gb300_batch *b, void *stream)
{
    if (!b || b->count <= 0) return fail(MIPT_GB300_E_INVALID, "batch has no prepared trajectories");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!graph_ready(b)) return execute_any(b, s);
    const std::vector<long long> key = structure_key(b);
    if (b->graph_exec && key == b->graph_key)
    {
        std::fill(b->sector.begin(), b->sector.end(), 0);
        MG_CUDA(cudaGraphLaunch(b->graph_exec, s));
        b->launches = b->graph_launches;
        b->executed = true;
        return 0;
    }
    // This call's results come from a normal execute, which also sizes every
    // buffer; the graph is captured from a second execute on a private stream.
    if (const int rc = execute_any(b, s)) return rc;
    MG_CUDA(cudaStreamSynchronize(s));
    if (b->graph_exec)
    {
        cudaGraphExecDestroy(b->graph_exec);
        b->graph_exec = nullptr;
    }
    if (!b->cap_stream) MG_CUDA(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
    mipt_gb300_batch *one[1] = {b};
    if (const int rc = capture_graph(one, 1, b->cap_stream, &b->cap_stream, nullptr, &b->graph_exec)) return rc;
    b->graph_key = key;
    b->graph_launches = b->launches;
    return 0;
}

} // extern "C"

struct mipt_gb300_batch_group
{
    std::vector<mipt_gb300_batch *> batches;
    std::vector<cudaStream_t> streams; // one per batch
    std::vector<cudaEvent_t> events;   // one per batch + the fork event
    cudaStream_t root = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<std::vector<long long>> keys;
    ~mipt_gb300_batch_group()
    {
        if (exec) cudaGraphExecDestroy(exec);
        for (auto st : streams) cudaStreamDestroy(st);
        for (auto ev : events) cudaEventDestroy(ev);
        if (root) cudaStreamDestroy(root);
    }
};

extern "C" {

int mipt_gb300_batch_group_create(mipt_gb300_batch *const *batches, int count, mipt_gb300_batch_group **out)
{
    if (!batches || count < 1 || !out) return fail(MIPT_GB300_E_INVALID, "a batch group needs at least one batch");
    std::unique_ptr<mipt_gb300_batch_group> g(new mipt_gb300_batch_group());
    for (int i = 0; i < count; ++i)
    {
        if (!batches[i]) return fail(MIPT_GB300_E_INVALID, "null batch in group");
        for (int j = 0; j < i; ++j)
            if (batches[j] == batches[i]) return fail(MIPT_GB300_E_INVALID, "a batch appears twice in the group");
        g->batches.push_back(batches[i]);
    }
    MG_CUDA(cudaStreamCreateWithFlags(&g->root, cudaStreamNonBlocking));
    for (int i = 0; i < count; ++i)
    {
        cudaStream_t st;
        MG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        g->streams.push_back(st);
    }
    for (int i = 0; i <= count; ++i)
    {
        cudaEvent_t ev;
        MG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        g->events.push_back(ev);
    }
    *out = g.release();
    return 0;
}

void mipt_gb300_batch_group_destroy(mipt_gb300_batch_group *g) { delete g; }

int mipt_gb300_batch_group_execute(mipt_gb300_batch_group *g, void *stream)
{
    if (!g) return fail(MIPT_GB300_E_INVALID, "null batch group");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nb = static_cast<int>(g->batches.size());
    for (auto *b : g->batches)
        if (b->count <= 0) return fail(MIPT_GB300_E_INVALID, "batch has no prepared trajectories");
    bool ready = true;
    for (auto *b : g->batches) ready = ready && graph_ready(b);
    if (!ready)
    {
        for (auto *b : g->batches)
            if (const int rc = execute_any(b, s)) return rc;
        return 0;
    }
    std::vector<std::vector<long long>> keys;
    for (auto *b : g->batches) keys.push_back(structure_key(b));
    if (g->exec && keys == g->keys)
    {
        for (auto *b : g->batches) std::fill(b->sector.begin(), b->sector.end(), 0);
        MG_CUDA(cudaGraphLaunch(g->exec, s));
        for (auto *b : g->batches)
        {
            b->launches = b->graph_launches;
            b->executed = true;
        }
        return 0;
    }
    // This call runs every batch normally (its results, and every buffer at
    // its final size); the graph is captured from a second execute.
    for (auto *b : g->batches)
        if (const int rc = execute_any(b, s)) return rc;
    MG_CUDA(cudaStreamSynchronize(s));
    if (g->exec)
    {
        cudaGraphExecDestroy(g->exec);
        g->exec = nullptr;
    }
    if (const int rc = capture_graph(g->batches.data(), nb, g->root, g->streams.data(), g->events.data(), &g->exec))
        return rc;
    for (auto *b : g->batches) b->graph_launches = b->launches;
    g->keys = keys;
    return 0;
}

int mipt_gb300_batch_fetch(mipt_gb300_batch *b, std::uint64_t *measured, std::uint64_t *outcomes, double *surprisal,
                           double *obs, double *rho3)
{
    if (!b || !b->executed) return fail(MIPT_GB300_E_INVALID, "batch not executed");
    MG_CUDA(cudaDeviceSynchronize());
    for (int k = 0; k < 5; ++k)
    {
        b->kind_ms[k] = 0.0;
        b->kind_launches[k] = 0;
    }
    for (const auto &m : b->marks)
    {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, m.second.first, m.second.second) == cudaSuccess) b->kind_ms[m.first] += ms;
        ++b->kind_launches[m.first];
    }
    b->marks.clear();
    int err = 0;
    MG_CUDA(cudaMemcpy(&err, b->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err & 8) return fail(MIPT_GB300_E_INTERNAL, "tile load wait timed out");
    if (err) return fail(MIPT_GB300_E_NUMERIC, "a measurement found a zero-norm state or no outcome with weight");
    if (b->ws.err.p)
    {
        MG_CUDA(cudaMemcpy(&err, b->ws.err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) return fail(MIPT_GB300_E_INTERNAL, "tensor-core Gram pipeline wait timed out");
    }
    if (b->ws.eig_err.p)
    {
        MG_CUDA(cudaMemcpy(&err, b->ws.eig_err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (err & 2) return fail(MIPT_GB300_E_INTERNAL, "eigensolver barrier wait timed out");
        if (err) return fail(MIPT_GB300_E_NUMERIC, "an eigenvalue iteration did not converge");
    }
    const int count = b->count, T = b->T;
    if (measured) std::copy(b->measured.begin(), b->measured.end(), measured);
    if (outcomes || surprisal)
    {
        LayerResult *hr = b->h_res.as<LayerResult>();
        MG_CUDA(cudaMemcpy(hr, b->res.p, sizeof(LayerResult) * count * T, cudaMemcpyDeviceToHost));
        for (std::size_t i = 0; i < static_cast<std::size_t>(count) * T; ++i)
        {
            if (outcomes) outcomes[i] = hr[i].outcome;
            if (surprisal) surprisal[i] = hr[i].surprisal;
        }
    }
    if (obs)
    {
        const std::size_t P = b->points, R = b->reqs_per_point;
        std::vector<double> ent(static_cast<std::size_t>(count) * P * R);
        if (R > 0) MG_CUDA(cudaMemcpy(ent.data(), b->ent.p, sizeof(double) * ent.size(), cudaMemcpyDeviceToHost));
        for (int i = 0; i < count; ++i)
            for (std::size_t pt = 0; pt < P; ++pt)
            {
                const double *e = ent.data() + (static_cast<std::size_t>(i) * P + pt) * R;
                double *o = obs + (static_cast<std::size_t>(i) * P + pt) * 4;
                o[0] = b->col_half_vn >= 0 ? e[b->col_half_vn] : NAN;
                o[1] = b->col_half_s2 >= 0 ? e[b->col_half_s2] : NAN;
                auto tmi = [&](const std::vector<int> &s) {
                    if (s.empty()) return static_cast<double>(NAN);
                    return e[s[0]] + e[s[1]] + e[s[2]] + e[s[3]] - e[s[4]] - e[s[5]] - e[s[6]];
                };
                o[2] = tmi(b->tmi_vn);
                o[3] = tmi(b->tmi_s2);
            }
    }
    if (rho3)
    {
        if (!b->cfg.rho3) return fail(MIPT_GB300_E_INVALID, "batch was created without rho3");
        MG_CUDA(cudaMemcpy(rho3, b->rho3.p, sizeof(double) * 128 * b->rho3_count * count, cudaMemcpyDeviceToHost));
    }
    return 0;
}

int mipt_gb300_batch_add_region(mipt_gb300_batch *b, const int *modes, int k, int order, int *region_id)
{
    if (!b || !modes || !region_id || k < 0 || k > 16 || (order != 1 && order != 2))
        return fail(MIPT_GB300_E_INVALID, "bad region (k <= 16, order 1 or 2)");
    const int n = b->cfg.n_qubits;
    std::uint64_t used = 0;
    for (int i = 0; i < k; ++i)
    {
        if (modes[i] < 0 || modes[i] >= n || ((used >> modes[i]) & 1ull))
            return fail(MIPT_GB300_E_INVALID, "region modes must be distinct and in range");
        used |= 1ull << modes[i];
    }
    b->region_slots.push_back(static_cast<int>(b->reqs.size()));
    b->reqs.push_back(EntReq{0, order, b->cfg.fermion_trace ? 1 : 0, std::vector<int>(modes, modes + k), 0});
    b->reqs_per_point = static_cast<int>(b->reqs.size());
    MG_CUDA(b->ent.ensure(static_cast<std::size_t>(b->capacity) * b->points * b->reqs_per_point * sizeof(double)));
    *region_id = static_cast<int>(b->region_slots.size()) - 1;
    b->executed = false;
    return 0;
}

int mipt_gb300_batch_fetch_regions(mipt_gb300_batch *b, double *out)
{
    if (!b || !b->executed || !out) return fail(MIPT_GB300_E_INVALID, "batch not executed or null output");
    if (b->region_slots.empty()) return fail(MIPT_GB300_E_INVALID, "batch has no regions");
    MG_CUDA(cudaDeviceSynchronize());
    const std::size_t P = b->points, R = b->reqs_per_point, G = b->region_slots.size();
    std::vector<double> ent(static_cast<std::size_t>(b->count) * P * R);
    MG_CUDA(cudaMemcpy(ent.data(), b->ent.p, sizeof(double) * ent.size(), cudaMemcpyDeviceToHost));
    for (int i = 0; i < b->count; ++i)
        for (std::size_t pt = 0; pt < P; ++pt)
            for (std::size_t g = 0; g < G; ++g)
                out[(static_cast<std::size_t>(i) * P + pt) * G + g] =
                    ent[(static_cast<std::size_t>(i) * P + pt) * R + b->region_slots[g]];
    return 0;
}

int mipt_gb300_batch_set_rho3_subsystems(mipt_gb300_batch *b, const int *triples, int count)
{
    if (!b || !triples || count <= 0) return fail(MIPT_GB300_E_INVALID, "bad rho3 subsystems");
    if (!b->cfg.rho3) return fail(MIPT_GB300_E_INVALID, "batch was created without rho3");
    b->executed = false;
    return set_rho3_subs(b, std::vector<int>(triples, triples + 3 * static_cast<std::size_t>(count)));
}

int mipt_gb300_batch_rho3_subsystem_count(mipt_gb300_batch *b) { return b ? b->rho3_count : -1; }

int mipt_gb300_batch_fetch_rho3_points(mipt_gb300_batch *b, double *out)
{
    if (!b || !b->executed || !out) return fail(MIPT_GB300_E_INVALID, "batch not executed or null output");
    if (!b->cfg.rho3 || !b->per_point())
        return fail(MIPT_GB300_E_INVALID, "rho3 per point needs rho3 and observe_every > 0 or an observation schedule");
    MG_CUDA(cudaDeviceSynchronize());
    const std::size_t P = b->points, S = b->rho3_count, C = b->capacity, per = S * 128;
    for (std::size_t pt = 0; pt < P; ++pt)
        for (int i = 0; i < b->count; ++i)
            MG_CUDA(cudaMemcpy(out + (static_cast<std::size_t>(i) * P + pt) * per,
                               b->rho3_pts.as<double>() + (pt * C + i) * per, sizeof(double) * per,
                               cudaMemcpyDeviceToHost));
    return 0;
}

int mipt_gb300_lattice_bonds(int x, int y, int colour, int *pairs, int *count)
{
    try
    {
        const auto bonds = lattice_bonds(x, y, colour);
        if (count) *count = static_cast<int>(bonds.size());
        if (pairs)
            for (std::size_t i = 0; i < bonds.size(); ++i)
            {
                pairs[2 * i] = bonds[i].first;
                pairs[2 * i + 1] = bonds[i].second;
            }
        return 0;
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
}

int mipt_gb300_draw_haar_lattice(std::uint64_t seed, int x, int y, int layers, double p, int chunk_bits,
                                 int *gates_per_layer, int *bond_q, double *bond_u, std::uint64_t *measured,
                                 double *uniforms, int *n_uniforms)
{
    try
    {
        TrajectoryDraw d;
        draw_haar_lattice_trajectory(seed, x, y, layers, p, chunk_bits, d);
        for (int t = 0; t < d.layers; ++t)
        {
            if (gates_per_layer) gates_per_layer[t] = d.bond_count[t];
            if (measured) measured[t] = d.measured[t];
        }
        if (bond_q) std::copy(d.bond_q.begin(), d.bond_q.end(), bond_q);
        if (bond_u)
            for (std::size_t i = 0; i < d.bond_u.size(); ++i)
            {
                bond_u[2 * i] = d.bond_u[i].real();
                bond_u[2 * i + 1] = d.bond_u[i].imag();
            }
        if (uniforms) std::copy(d.uniforms.begin(), d.uniforms.end(), uniforms);
        if (n_uniforms) *n_uniforms = static_cast<int>(d.uniforms.size());
        return 0;
    }
    catch (const std::exception &e)
    {
        return fail(MIPT_GB300_E_INVALID, e.what());
    }
}

int mipt_gb300_batch_fetch_tmi(mipt_gb300_batch *b, int order, double *tmi)
{
    if (!b || !b->executed || !tmi) return fail(MIPT_GB300_E_INVALID, "batch not executed or null output");
    if (order != 1 && order != 2) return fail(MIPT_GB300_E_INVALID, "order must be 1 or 2");
    const std::vector<int> &slots = order == 1 ? b->tmi_vn : b->tmi_s2;
    if (slots.empty()) return fail(MIPT_GB300_E_INVALID, "batch was created without this TMI order");
    MG_CUDA(cudaDeviceSynchronize());
    const std::size_t P = b->points, R = b->reqs_per_point, Cy = b->tmi_cycles;
    std::vector<double> ent(static_cast<std::size_t>(b->count) * P * R);
    MG_CUDA(cudaMemcpy(ent.data(), b->ent.p, sizeof(double) * ent.size(), cudaMemcpyDeviceToHost));
    for (int i = 0; i < b->count; ++i)
        for (std::size_t pt = 0; pt < P; ++pt)
        {
            const double *e = ent.data() + (static_cast<std::size_t>(i) * P + pt) * R;
            for (std::size_t c = 0; c < Cy; ++c)
            {
                const int *s = slots.data() + 7 * c;
                tmi[(static_cast<std::size_t>(i) * P + pt) * Cy + c] =
                    e[s[0]] + e[s[1]] + e[s[2]] + e[s[3]] - e[s[4]] - e[s[5]] - e[s[6]];
            }
        }
    return 0;
}

int mipt_gb300_batch_run_haar(mipt_gb300_batch *b, const std::uint64_t *seeds, const double *p, int count,
                              const std::uint64_t *forced, std::uint64_t *measured, std::uint64_t *outcomes,
                              double *surprisal, double *obs, double *rho3)
{
    int rc = mipt_gb300_batch_prepare_haar(b, seeds, p, count, forced);
    if (rc) return rc;
    rc = mipt_gb300_batch_execute(b, nullptr);
    if (rc) return rc;
    return mipt_gb300_batch_fetch(b, measured, outcomes, surprisal, obs, rho3);
}

void *mipt_gb300_batch_state(mipt_gb300_batch *b, int i)
{
    if (!b || i < 0 || i >= b->count) return nullptr;
    return static_cast<char *>(b->states.p) + static_cast<std::size_t>(i) * b->dim * b->elem;
}

long long mipt_gb300_batch_launches(mipt_gb300_batch *b) { return b ? b->launches : -1; }

int mipt_gb300_batch_set_profiling(mipt_gb300_batch *b, int enable)
{
    if (!b) return fail(MIPT_GB300_E_INVALID, "null batch");
    b->profile = enable != 0;
    return 0;
}

int mipt_gb300_batch_kernel_stats(mipt_gb300_batch *b, double *ms, long long *launches)
{
    if (!b) return fail(MIPT_GB300_E_INVALID, "null batch");
    for (int k = 0; k < 5; ++k)
    {
        if (ms) ms[k] = b->kind_ms[k];
        if (launches) launches[k] = b->kind_launches[k];
    }
    return 0;
}

} // extern "C"
