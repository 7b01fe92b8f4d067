// Small multilayer perceptron trained and run on the GPU with the project's
// own kernels: the learned warm start of the GMN solver (64 -> 256 -> 256 ->
// 448: rho3 features in, ADMM state W, Q_1..3, Z_1..3 out).
//
// Layers y = x W^T + b with ReLU between layers; weights are kept as FP32
// master copies for the optimiser and as BF16 copies that every product
// reads, with FP32 accumulation. Training minimises the mean squared error
// with Adam. One tiled SIMT GEMM kernel serves the forward pass (X W^T), the
// input gradient (dY W) and the weight gradient (dY^T X) through strides; the
// matrices are a few hundred wide, so these are latency- rather than
// throughput-bound and stay off the tensor cores.
#include "mipt_gb300.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
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
constexpr int kTile = 64, kK = 16, kGemmThreads = 256;

template <typename T> __device__ __forceinline__ float ld(const T *p, std::size_t i) { return static_cast<float>(p[i]); }
template <> __device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16 *p, std::size_t i)
{
    return __bfloat162float(p[i]);
}

// C[m][n] = alpha * sum_k A(m, k) B(k, n) (+ beta C) (+ bias[n]) (ReLU),
// A(m, k) = A[m * a_m + k * a_k], B(k, n) = B[k * b_k + n * b_n], C row-major.
template <typename TB>
__global__ void __launch_bounds__(kGemmThreads)
    k_gemm(int M, int N, int K, const float *__restrict__ A, std::size_t a_m, std::size_t a_k,
           const TB *__restrict__ B, std::size_t b_k, std::size_t b_n, float *__restrict__ C, float beta,
           const float *__restrict__ bias, int relu)
{
    __shared__ float As[kK][kTile + 1], Bs[kK][kTile + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += kK)
    {
        for (int i = threadIdx.x; i < kTile * kK; i += kGemmThreads)
        {
            const int kk = i % kK, mm = i / kK;
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < K) ? A[m * a_m + k * a_k] : 0.f;
            const int nn = i / kK, n = n0 + nn;
            Bs[kk][nn] = (n < N && k < K) ? ld(B, k * b_k + n * b_n) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kK; ++kk)
        {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
            {
                a[i] = As[kk][ty * 4 + i];
                b[i] = Bs[kk][tx * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
            if (m >= M || n >= N) continue;
            float v = acc[i][j];
            if (beta != 0.f) v += beta * C[static_cast<std::size_t>(m) * N + n];
            if (bias) v += bias[n];
            if (relu) v = fmaxf(v, 0.f);
            C[static_cast<std::size_t>(m) * N + n] = v;
        }
}

// dX *= (X > 0): back through the ReLU that produced X.
__global__ void k_relu_mask(float *__restrict__ d, const float *__restrict__ x, std::size_t n)
{
    const std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x;
    if (i < n && !(x[i] > 0.f)) d[i] = 0.f;
}

// dY = 2 (Y - T) / count and per-block partial sums of (Y - T)^2.
__global__ void k_mse(const float *__restrict__ y, const float *__restrict__ t, std::size_t n, float scale,
                      float *__restrict__ dy, float *__restrict__ part)
{
    __shared__ float red[256];
    float s = 0.f;
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x)
    {
        const float e = y[i] - t[i];
        dy[i] = 2.f * e * scale;
        s += e * e;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = 128; k > 0; k /= 2)
    {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// db[n] = sum_b dY[b][n].
__global__ void k_col_sum(const float *__restrict__ d, int rows, int cols, float *__restrict__ out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.f;
    for (int r = 0; r < rows; ++r) s += d[static_cast<std::size_t>(r) * cols + c];
    out[c] = s;
}

__global__ void k_adam(float *__restrict__ w, __nv_bfloat16 *__restrict__ wb, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, std::size_t n, float lr, float b1, float b2,
                       float c1, float c2, float eps)
{
    const std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    m[i] = b1 * m[i] + (1.f - b1) * gi;
    v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
    w[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
    if (wb) wb[i] = __float2bfloat16_rn(w[i]);
}

// dst[i] = src[idx[i]] for rows of `width` floats.
__global__ void k_gather_rows(const float *__restrict__ src, const int *__restrict__ idx, int rows, int width,
                              float *__restrict__ dst)
{
    const std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<std::size_t>(rows) * width) return;
    const std::size_t r = i / width, c = i % width;
    dst[i] = src[static_cast<std::size_t>(idx[r]) * width + c];
}

__global__ void k_to_bf16(const float *__restrict__ w, __nv_bfloat16 *__restrict__ wb, std::size_t n)
{
    const std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

struct Buf
{
    void *p = nullptr;
    std::size_t bytes = 0;
    ~Buf()
    {
        if (p) cudaFree(p);
    }
    cudaError_t ensure(std::size_t need)
    {
        if (need <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        const cudaError_t e = cudaMalloc(&p, need);
        if (e == cudaSuccess) bytes = need;
        return e;
    }
    template <typename T> T *as() const { return static_cast<T *>(p); }
};

int blocks_for(std::size_t n) { return static_cast<int>((n + 255) / 256); }
} // namespace

struct mipt_gb300_mlp
{
    std::vector<int> dims; // layer widths, dims[0] = inputs
    std::vector<std::size_t> woff, boff;
    std::size_t nparams = 0;
    Buf params, params_bf16, grads, adam_m, adam_v;
    Buf act;  // activations of every layer for the current batch
    Buf dact; // gradients of activations
    Buf x, y, part;
    long long step = 0;
    int layers() const { return static_cast<int>(dims.size()) - 1; }
};

namespace
{
#define MLP_CUDA(x)                                                                                              \
    do                                                                                                           \
    {                                                                                                            \
        cudaError_t e_ = (x);                                                                                    \
        if (e_ != cudaSuccess) return api_cuda_fail(e_, #x);                                                     \
    } while (0)

// Activation offsets for a batch of B rows: layer l output at act + B * aoff[l].
std::vector<std::size_t> act_offsets(const mipt_gb300_mlp &m)
{
    std::vector<std::size_t> o(m.dims.size(), 0);
    for (std::size_t l = 1; l < m.dims.size(); ++l) o[l] = o[l - 1] + m.dims[l - 1];
    return o;
}

template <typename TB>
void gemm(int M, int N, int K, const float *A, std::size_t a_m, std::size_t a_k, const TB *B, std::size_t b_k,
          std::size_t b_n, float *C, float beta, const float *bias, int relu)
{
    dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
    k_gemm<TB><<<grid, kGemmThreads>>>(M, N, K, A, a_m, a_k, B, b_k, b_n, C, beta, bias, relu);
}

// Forward pass of B rows whose inputs sit at act (layer 0 block).
void forward(mipt_gb300_mlp &m, int B)
{
    const auto ao = act_offsets(m);
    float *act = m.act.as<float>();
    const __nv_bfloat16 *wb = m.params_bf16.as<__nv_bfloat16>();
    const float *p = m.params.as<float>();
    for (int l = 0; l < m.layers(); ++l)
    {
        const int in = m.dims[l], out = m.dims[l + 1];
        // y[b][o] = sum_i x[b][i] W[o][i] + bias[o]: B(k = i, n = o) = W[o * in + i].
        gemm<__nv_bfloat16>(B, out, in, act + B * ao[l], in, 1, wb + m.woff[l], 1, in, act + B * ao[l + 1], 0.f,
                            p + m.boff[l], l + 1 < m.layers() ? 1 : 0);
    }
}

// Backward pass from dY (at dact's last block) to parameter gradients.
void backward(mipt_gb300_mlp &m, int B)
{
    const auto ao = act_offsets(m);
    float *act = m.act.as<float>(), *dact = m.dact.as<float>(), *g = m.grads.as<float>();
    const __nv_bfloat16 *wb = m.params_bf16.as<__nv_bfloat16>();
    for (int l = m.layers() - 1; l >= 0; --l)
    {
        const int in = m.dims[l], out = m.dims[l + 1];
        const float *dy = dact + B * ao[l + 1];
        const float *x = act + B * ao[l];
        // dW[o][i] = sum_b dy[b][o] x[b][i]: A(m = o, k = b) = dy[b * out + o], B(k = b, n = i) = x[b * in + i].
        gemm<float>(out, in, B, dy, 1, out, x, in, 1, g + m.woff[l], 0.f, nullptr, 0);
        k_col_sum<<<(out + 255) / 256, 256>>>(dy, B, out, g + m.boff[l]);
        if (l > 0)
        {
            // dx[b][i] = sum_o dy[b][o] W[o][i]: B(k = o, n = i) = W[o * in + i].
            float *dx = dact + B * ao[l];
            gemm<__nv_bfloat16>(B, in, out, dy, out, 1, wb + m.woff[l], in, 1, dx, 0.f, nullptr, 0);
            k_relu_mask<<<blocks_for(static_cast<std::size_t>(B) * in), 256>>>(dx, x, static_cast<std::size_t>(B) * in);
        }
    }
}

int ensure_batch(mipt_gb300_mlp &m, int B)
{
    std::size_t total = 0;
    for (int d : m.dims) total += d;
    MLP_CUDA(m.act.ensure(sizeof(float) * total * B));
    MLP_CUDA(m.dact.ensure(sizeof(float) * total * B));
    MLP_CUDA(m.y.ensure(sizeof(float) * m.dims.back() * B));
    MLP_CUDA(m.part.ensure(sizeof(float) * 1024));
    return 0;
}

// Loss (mean over rows and outputs) and gradients of B rows (x, t on device).
int loss_and_grad(mipt_gb300_mlp &m, const float *d_x, const float *d_t, int B, double *loss)
{
    if (const int rc = ensure_batch(m, B)) return rc;
    const auto ao = act_offsets(m);
    MLP_CUDA(cudaMemcpy(m.act.as<float>(), d_x, sizeof(float) * B * m.dims[0], cudaMemcpyDeviceToDevice));
    forward(m, B);
    const int out = m.dims.back();
    const std::size_t n = static_cast<std::size_t>(B) * out;
    const int blocks = std::min(1024, blocks_for(n));
    k_mse<<<blocks, 256>>>(m.act.as<float>() + B * ao.back(), d_t, n, 1.f / static_cast<float>(n),
                           m.dact.as<float>() + B * ao.back(), m.part.as<float>());
    backward(m, B);
    MLP_CUDA(cudaGetLastError());
    if (loss)
    {
        std::vector<float> part(blocks);
        MLP_CUDA(cudaMemcpy(part.data(), m.part.p, sizeof(float) * blocks, cudaMemcpyDeviceToHost));
        double s = 0;
        for (float v : part) s += v;
        *loss = s / static_cast<double>(n);
    }
    return 0;
}
} // namespace

extern "C" {

int mipt_gb300_mlp_create(const int *dims, int n_dims, uint64_t seed, mipt_gb300_mlp **out)
{
    if (!dims || n_dims < 2 || !out) return api_fail(MIPT_GB300_E_INVALID, "bad MLP shape");
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return api_fail(MIPT_GB300_E_NODEVICE, "no CUDA device");
    auto *m = new mipt_gb300_mlp();
    m->dims.assign(dims, dims + n_dims);
    std::size_t off = 0;
    for (int l = 0; l + 1 < n_dims; ++l)
    {
        m->woff.push_back(off);
        off += static_cast<std::size_t>(dims[l]) * dims[l + 1];
        m->boff.push_back(off);
        off += dims[l + 1];
    }
    m->nparams = off;
    // He-uniform initialisation, biases zero (host, seeded).
    std::vector<float> p(off, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l + 1 < n_dims; ++l)
    {
        const float lim = std::sqrt(6.f / static_cast<float>(dims[l]));
        std::uniform_real_distribution<float> u(-lim, lim);
        for (std::size_t i = 0; i < static_cast<std::size_t>(dims[l]) * dims[l + 1]; ++i) p[m->woff[l] + i] = u(rng);
    }
    cudaError_t e;
    if ((e = m->params.ensure(sizeof(float) * off)) != cudaSuccess ||
        (e = m->params_bf16.ensure(sizeof(__nv_bfloat16) * off)) != cudaSuccess ||
        (e = m->grads.ensure(sizeof(float) * off)) != cudaSuccess ||
        (e = m->adam_m.ensure(sizeof(float) * off)) != cudaSuccess ||
        (e = m->adam_v.ensure(sizeof(float) * off)) != cudaSuccess)
    {
        delete m;
        return api_cuda_fail(e, "MLP parameter allocation");
    }
    cudaMemcpy(m->params.p, p.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
    cudaMemset(m->adam_m.p, 0, sizeof(float) * off);
    cudaMemset(m->adam_v.p, 0, sizeof(float) * off);
    k_to_bf16<<<blocks_for(off), 256>>>(m->params.as<float>(), m->params_bf16.as<__nv_bfloat16>(), off);
    if ((e = cudaGetLastError()) != cudaSuccess)
    {
        delete m;
        return api_cuda_fail(e, "MLP init");
    }
    *out = m;
    return 0;
}

void mipt_gb300_mlp_destroy(mipt_gb300_mlp *m) { delete m; }

long long mipt_gb300_mlp_param_count(const mipt_gb300_mlp *m) { return m ? static_cast<long long>(m->nparams) : -1; }

int mipt_gb300_mlp_get_params(mipt_gb300_mlp *m, float *out)
{
    if (!m || !out) return api_fail(MIPT_GB300_E_INVALID, "null MLP or output");
    MLP_CUDA(cudaMemcpy(out, m->params.p, sizeof(float) * m->nparams, cudaMemcpyDeviceToHost));
    return 0;
}

int mipt_gb300_mlp_set_params(mipt_gb300_mlp *m, const float *in)
{
    if (!m || !in) return api_fail(MIPT_GB300_E_INVALID, "null MLP or input");
    MLP_CUDA(cudaMemcpy(m->params.p, in, sizeof(float) * m->nparams, cudaMemcpyHostToDevice));
    k_to_bf16<<<blocks_for(m->nparams), 256>>>(m->params.as<float>(), m->params_bf16.as<__nv_bfloat16>(),
                                               m->nparams);
    MLP_CUDA(cudaGetLastError());
    return 0;
}

int mipt_gb300_mlp_forward(mipt_gb300_mlp *m, const float *x, int n, float *y)
{
    if (!m || !x || !y || n <= 0) return api_fail(MIPT_GB300_E_INVALID, "bad MLP forward arguments");
    const int chunk = 8192, in = m->dims[0], out = m->dims.back();
    if (const int rc = ensure_batch(*m, std::min(n, chunk))) return rc;
    const auto ao = act_offsets(*m);
    for (int r0 = 0; r0 < n; r0 += chunk)
    {
        const int B = std::min(chunk, n - r0);
        MLP_CUDA(cudaMemcpy(m->act.as<float>(), x + static_cast<std::size_t>(r0) * in, sizeof(float) * B * in,
                            cudaMemcpyHostToDevice));
        forward(*m, B);
        MLP_CUDA(cudaGetLastError());
        MLP_CUDA(cudaMemcpy(y + static_cast<std::size_t>(r0) * out, m->act.as<float>() + B * ao.back(),
                            sizeof(float) * B * out, cudaMemcpyDeviceToHost));
    }
    return 0;
}

int mipt_gb300_mlp_loss_grad(mipt_gb300_mlp *m, const float *x, const float *t, int n, double *loss, float *grad)
{
    if (!m || !x || !t || n <= 0) return api_fail(MIPT_GB300_E_INVALID, "bad MLP gradient arguments");
    MLP_CUDA(m->x.ensure(sizeof(float) * n * m->dims[0]));
    MLP_CUDA(m->y.ensure(sizeof(float) * n * m->dims.back()));
    MLP_CUDA(cudaMemcpy(m->x.p, x, sizeof(float) * n * m->dims[0], cudaMemcpyHostToDevice));
    Buf tb;
    MLP_CUDA(tb.ensure(sizeof(float) * n * m->dims.back()));
    MLP_CUDA(cudaMemcpy(tb.p, t, sizeof(float) * n * m->dims.back(), cudaMemcpyHostToDevice));
    if (const int rc = loss_and_grad(*m, m->x.as<float>(), tb.as<float>(), n, loss)) return rc;
    if (grad) MLP_CUDA(cudaMemcpy(grad, m->grads.p, sizeof(float) * m->nparams, cudaMemcpyDeviceToHost));
    return 0;
}

int mipt_gb300_mlp_train(mipt_gb300_mlp *m, const float *x, const float *t, int n, int epochs, int batch, float lr,
                         uint64_t shuffle_seed, double *final_loss)
{
    if (!m || !x || !t || n <= 0 || epochs <= 0 || batch <= 0 || !(lr > 0))
        return api_fail(MIPT_GB300_E_INVALID, "bad MLP training arguments");
    const int in = m->dims[0], out = m->dims.back();
    Buf dx, dt, bx, bt, didx;
    MLP_CUDA(dx.ensure(sizeof(float) * static_cast<std::size_t>(n) * in));
    MLP_CUDA(dt.ensure(sizeof(float) * static_cast<std::size_t>(n) * out));
    MLP_CUDA(cudaMemcpy(dx.p, x, sizeof(float) * static_cast<std::size_t>(n) * in, cudaMemcpyHostToDevice));
    MLP_CUDA(cudaMemcpy(dt.p, t, sizeof(float) * static_cast<std::size_t>(n) * out, cudaMemcpyHostToDevice));
    MLP_CUDA(bx.ensure(sizeof(float) * batch * in));
    MLP_CUDA(bt.ensure(sizeof(float) * batch * out));
    MLP_CUDA(didx.ensure(sizeof(int) * n));
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::mt19937_64 rng(shuffle_seed);
    double loss_sum = 0;
    long long loss_n = 0;
    for (int ep = 0; ep < epochs; ++ep)
    {
        std::shuffle(order.begin(), order.end(), rng);
        MLP_CUDA(cudaMemcpy(didx.p, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
        loss_sum = 0;
        loss_n = 0;
        for (int b0 = 0; b0 + batch <= n; b0 += batch)
        {
            // Gather the batch rows on the device.
            const int *bi = didx.as<int>() + b0;
            k_gather_rows<<<blocks_for(static_cast<std::size_t>(batch) * in), 256>>>(dx.as<float>(), bi, batch, in,
                                                                                     bx.as<float>());
            k_gather_rows<<<blocks_for(static_cast<std::size_t>(batch) * out), 256>>>(dt.as<float>(), bi, batch, out,
                                                                                      bt.as<float>());
            double l = 0;
            const bool want = b0 + 2 * batch > n; // loss of the epoch's last batch
            if (const int rc = loss_and_grad(*m, bx.as<float>(), bt.as<float>(), batch, want ? &l : nullptr))
                return rc;
            ++m->step;
            const float b1 = 0.9f, b2 = 0.999f;
            const float c1 = 1.f - std::pow(b1, static_cast<float>(m->step));
            const float c2 = 1.f - std::pow(b2, static_cast<float>(m->step));
            k_adam<<<blocks_for(m->nparams), 256>>>(m->params.as<float>(), m->params_bf16.as<__nv_bfloat16>(),
                                                     m->grads.as<float>(), m->adam_m.as<float>(),
                                                     m->adam_v.as<float>(), m->nparams, lr, b1, b2, c1, c2, 1e-8f);
            MLP_CUDA(cudaGetLastError());
            if (want)
            {
                loss_sum += l;
                ++loss_n;
            }
        }
    }
    MLP_CUDA(cudaDeviceSynchronize());
    if (final_loss) *final_loss = loss_n ? loss_sum / loss_n : NAN;
    return 0;
}
}
