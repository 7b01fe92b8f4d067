// Allocation-free Renyi-2 entropy of an FP32 device state vector.
//
// A variant of the FP32 Renyi-2 entry point (mipt_cuda_renyi2_f32) for
// callers that cannot allocate device memory: the Gram purity kernel
// (k_gram with FP64 accumulation, run in purity mode, then a fixed-order
// row sum) takes its job record, per-tile partials and purity from one
// file-scope static __device__ array instead of cudaMalloc'd workspace.
//
// Limits and rules:
//   - kScratchBytes = 512 KiB per device; n_kept <= 14 (job record 336 B,
//     purity 8 B, tile partials 8 * 32,896 B at n_kept = 14; n_kept = 15
//     would need 1,050,624 B). Larger requests are rejected with
//     MIPT_GB300_E_INVALID before any device work.
//   - Set-up: every call, with the caller's device current, looks up the
//     array's device address (cudaGetSymbolAddress) and checks the return
//     code before any launch. The lookup is cheap next to the call's copies,
//     and it never hands out an address cached from an earlier context (a
//     device reset, or another context on the same ordinal, reloads the
//     module at a possibly different address).
//   - No call may be made while a stream capture is active on the device:
//     the job record and the purity travel by synchronous cudaMemcpy and the
//     purity slot is cleared on the legacy default stream, which the CUDA
//     runtime forbids during capture (it would invalidate the capture).
//   - Nothing in the array needs to start at zero: every word a kernel reads
//     is written earlier in the same call (job record by the host copy, tile
//     partials by the Gram kernel, purity by the row sum). The purity slot is
//     still cleared before the launch.
//   - One array per device is shared by every call on that device: calls that
//     overlap on the GPU (from several host threads, or on several streams)
//     race. Callers serialise them.
#include "mipt_gb300.h"

#include "observables.cuh"

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

namespace mg
{
int api_fail(int code, const std::string &what);
int api_cuda_fail(cudaError_t e, const char *what);
} // namespace mg

using namespace mg;

namespace
{
constexpr std::size_t kScratchBytes = std::size_t{512} << 10;
constexpr std::size_t kJobOffset = 0;
constexpr std::size_t kPurityOffset = 512;
constexpr std::size_t kTileOffset = 1024;
constexpr int kMaxKept = 14;

constexpr std::size_t tiles_of(int k)
{
    return k >= 6 ? ((std::size_t{1} << (k - 6)) * ((std::size_t{1} << (k - 6)) + 1)) / 2 : 1;
}
static_assert(sizeof(GramJob) <= kPurityOffset - kJobOffset, "job record overlaps the purity slot");
static_assert(kTileOffset + sizeof(double) * tiles_of(kMaxKept) <= kScratchBytes, "tile partials exceed scratch");
static_assert(kTileOffset + sizeof(double) * tiles_of(kMaxKept + 1) > kScratchBytes, "limit is not the largest fit");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the static scratch in the current context, looked up on
// every call.
int scratch_address(unsigned char **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return api_cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
    *out = static_cast<unsigned char *>(p);
    return 0;
}
} // namespace

extern "C" int mipt_gb300_renyi2_f32_noalloc(const void *device_state_vector, int n_qubits,
                                             const int *host_kept_modes, int n_kept, int fermion_trace,
                                             double *host_out)
{
    const int n = n_qubits, k = n_kept;
    if (!device_state_vector || !host_kept_modes || !host_out || n < 1 || n > 32 || k < 0 || k > n)
        return api_fail(MIPT_GB300_E_INVALID, "invalid subsystem request");
    if (k > kMaxKept)
        return api_fail(MIPT_GB300_E_INVALID, "n_kept = " + std::to_string(k) +
                                                  " exceeds the allocation-free limit of 14 kept modes "
                                                  "(512 KiB static device scratch); use mipt_cuda_renyi2_f32");
    for (int i = 0; i < k; ++i)
        if (host_kept_modes[i] < 0 || host_kept_modes[i] >= n)
            return api_fail(MIPT_GB300_E_INVALID, "kept mode out of range");
    if (k == 0)
    {
        *host_out = 0.0;
        return 0;
    }
    GramJob job;
    try
    {
        job = make_gram_job(0, n, host_kept_modes, k, fermion_trace != 0);
    }
    catch (const std::exception &e)
    {
        return api_fail(MIPT_GB300_E_INVALID, e.what());
    }
    unsigned char *base = nullptr;
    if (const int rc = scratch_address(&base)) return rc;
    GramJob *d_job = reinterpret_cast<GramJob *>(base + kJobOffset);
    double *d_purity = reinterpret_cast<double *>(base + kPurityOffset);
    cudaError_t e = cudaMemcpy(d_job, &job, sizeof(GramJob), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return api_cuda_fail(e, "copy of the job record");
    e = cudaMemsetAsync(d_purity, 0, sizeof(double), 0);
    if (e != cudaSuccess) return api_cuda_fail(e, "clear of the purity slot");
    e = gram_purity_f64acc(static_cast<const Cx<float> *>(device_state_vector), n, d_job, 1, k, d_purity,
                           base + kTileOffset, kScratchBytes - kTileOffset, 0);
    if (e != cudaSuccess) return api_cuda_fail(e, "Gram purity launch");
    double purity = 0.0;
    e = cudaMemcpy(&purity, d_purity, sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return api_cuda_fail(e, "copy of the purity");
    *host_out = renyi2_from_purity(purity);
    return 0;
}
