// Compile-only stand-in for the CUDA-Q header, used solely to build the
// reference's host-side samplers and matrix builders into the parity harness
// (oracle/_ref). Every quantum operation is a no-op: the harness never runs a
// CUDA-Q kernel, it only calls the reference's host functions (layer draws,
// fused bond matrices, measurement and entropy algebra).
#pragma once
#include <complex>
#include <cstddef>
#include <vector>

#define __qpu__

namespace cudaq
{
struct ctrl {};
struct adj {};
struct qubit {};

template <std::size_t Levels = 2>
struct qvector
{
    explicit qvector(std::size_t n = 0) : q(n) {}
    template <typename S> explicit qvector(const S &) {}
    qubit &operator[](std::size_t i) { return q[i]; }
    std::size_t size() const { return q.size(); }
    std::vector<qubit> q;
};
template <typename T> qvector(T) -> qvector<2>;

struct SimulationState
{
    enum class precision { fp32, fp64 };
};

struct tensor_view
{
    void *data = nullptr;
    std::size_t get_rank() const { return 0; }
    std::size_t get_num_elements() const { return 0; }
};

// Inert state: the harness passes host vectors to the reference's host
// functions directly and never reaches these members at run time.
struct state
{
    template <typename T> std::vector<T> amplitudes(const T &) const { return {}; }
    template <typename B> std::vector<std::complex<double>> amplitudes(const std::vector<B> &) const
    {
        return {};
    }
    SimulationState::precision get_precision() const { return SimulationState::precision::fp64; }
    tensor_view get_tensor() const { return {}; }
    std::size_t get_num_tensors() const { return 0; }
    bool is_on_gpu() const { return false; }
    template <typename T> void to_host(T *, std::size_t) const {}
    template <typename T> static state from_data(const T &) { return {}; }
};

template <typename... A> state get_state(A &&...) { return {}; }
} // namespace cudaq

// Gate entry points the reference kernels name; all are inert.
#define MIPT_STUB_GATE(name)                                                   \
    template <typename Mod = void, typename... A> inline void name(A &&...) {}
MIPT_STUB_GATE(x)
MIPT_STUB_GATE(y)
MIPT_STUB_GATE(z)
MIPT_STUB_GATE(h)
MIPT_STUB_GATE(s)
MIPT_STUB_GATE(t)
MIPT_STUB_GATE(rx)
MIPT_STUB_GATE(ry)
MIPT_STUB_GATE(rz)
MIPT_STUB_GATE(r1)
MIPT_STUB_GATE(u3)
MIPT_STUB_GATE(swap)
MIPT_STUB_GATE(cx)
MIPT_STUB_GATE(cz)
template <typename... A> inline bool mz(A &&...) { return false; }
#undef MIPT_STUB_GATE
