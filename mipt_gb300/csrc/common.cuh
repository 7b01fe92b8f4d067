// Shared device/host definitions for the GB300 trajectory engine.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

namespace mg
{

// Nanoseconds of the GPU's global timer: the clock the bounded device waits
// measure their limits against (mbarrier.try_wait suspends for a
// hardware-chosen time per poll, so a poll count alone is no time limit).
__device__ __forceinline__ std::uint64_t device_ns()
{
    std::uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Interleaved complex amplitude; float2 / double2 layout in HBM.
template <typename Real> struct Cx;
template <> struct __align__(8) Cx<float>
{
    float re, im;
};
template <> struct __align__(16) Cx<double>
{
    double re, im;
};

template <typename Real>
__host__ __device__ __forceinline__ Cx<Real> cmul(Cx<Real> a, Cx<Real> b)
{
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}

template <typename Real>
__host__ __device__ __forceinline__ Cx<Real> cfma(Cx<Real> a, Cx<Real> b, Cx<Real> c)
{
    // a*b + c
    c.re = fma(a.re, b.re, c.re);
    c.re = fma(-a.im, b.im, c.re);
    c.im = fma(a.re, b.im, c.im);
    c.im = fma(a.im, b.re, c.im);
    return c;
}

// Scatter the low bits of `v` into the bit positions listed in pos[0..count).
__host__ __device__ __forceinline__ std::uint64_t scatter_bits(std::uint64_t v, const std::int8_t *pos, int count)
{
    std::uint64_t out = 0;
    for (int i = 0; i < count; ++i) out |= ((v >> i) & 1ull) << pos[i];
    return out;
}

// Insert a zero bit at position p (bits at and above p move up one place).
__host__ __device__ __forceinline__ std::uint64_t insert_zero(std::uint64_t v, int p)
{
    const std::uint64_t low = v & ((1ull << p) - 1ull);
    return ((v >> p) << (p + 1)) | low;
}

// Maximum qubits handled by the engine (amplitude index fits 2^34 elements).
constexpr int kMaxQubits = 34;
// Maximum tile width (local qubits) of one pass.
constexpr int kMaxLocal = 15;
// Maximum bonds applied by one pass.
constexpr int kMaxPassGates = 16;

// Pending projective collapse of a trajectory: amplitudes whose bits on `mask`
// differ from `value` become zero, the rest are multiplied by `scale`. A
// nonzero `parity` (parity-sector states, whose top qubit is the parity of
// the others) also zeroes the amplitudes whose bits on parity & ~kParityBit
// have a parity other than the bit kParityBit of `parity`.
struct Collapse
{
    std::uint64_t mask;
    std::uint64_t value;
    double scale;
    std::uint64_t parity;
};
constexpr std::uint64_t kParityBit = 1ull << 63;

__host__ __device__ __forceinline__ bool collapse_keeps(std::uint64_t idx, const Collapse &cl)
{
    if ((idx & cl.mask) != cl.value) return false;
    if (cl.parity == 0) return true;
#ifdef __CUDA_ARCH__
    const int par = __popcll(idx & cl.parity & ~kParityBit) & 1;
#else
    const int par = __builtin_popcountll(idx & cl.parity & ~kParityBit) & 1;
#endif
    return par == static_cast<int>(cl.parity >> 63);
}

// Geometry of one tiled pass over a 2^n state. A tile holds 2^k amplitudes:
// local bit i <-> qubit pos[i]; the first `c` local bits are the contiguous
// low qubits 0..c-1. The tile index enumerates the remaining qubits nl[].
struct PassGeom
{
    int n;        // qubits
    int k;        // local qubits
    int c;        // contiguous low local qubits (pos[i] == i for i < c)
    int n_nl;     // non-local qubits = n - k
    std::int8_t pos[kMaxLocal + 1];
    std::int8_t nl[kMaxQubits];
};

// Gates of one pass: indices into the layer's gate list plus local bit
// positions of the gate's two qubits (a = matrix bit 0, b = matrix bit 1).
// kind 1: a parity-selected 2x2 gate on qubit a of a parity-sector state
// (gate entries 0..3 when the other qubits' parity is even, 4..7 when odd,
// both row-major); b is an untouched partner the register rounds pair it with.
struct PassGates
{
    int count;
    std::int16_t gate[kMaxPassGates];
    std::int8_t la[kMaxPassGates];
    std::int8_t lb[kMaxPassGates];
    std::int8_t kind[kMaxPassGates];
};

} // namespace mg
