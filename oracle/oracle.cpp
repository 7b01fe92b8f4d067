// CPU FP64 oracle for the monitored-circuit trajectory path.
//
// TEST INFRASTRUCTURE. Only the tests, __graft_entry__.smoke() and bench.py's
// CPU-baseline / reference arm load this library, and only as the checker or
// as the timed CPU baseline; the product never calls it.
//
// This is a restatement, written for this project, of the reference's
// algorithm (paths are inside the reference project):
//   * seeding: splitmix64 and trajectory_seed   cpp/include/mipt/types.hpp:262-273
//     two mt19937 streams per trajectory         cpp/include/mipt/circuit.hpp:129-140
//   * Haar brickwork layer draw                  cpp/include/mipt/circuits/haar.hpp:226-305
//     (gates of a layer first, then Bernoulli(p) measurement flags per site;
//     odd layers close the ring with bond (n-1, 0) when closed)
//   * Haar U(4): Gram-Schmidt of four complex   cpp/include/mipt/circuits/haar.hpp:39-85
//     Gaussian columns, row-major, bit 0 = q0. The reference then runs a
//     cosine-sine decomposition and rebuilds the 4x4 from it
//     (cpp/include/mipt/cusv/gates.hpp:139-173); the rebuilt matrix equals the
//     drawn unitary to ~1e-15, so the oracle applies the drawn unitary itself
//     and keeps only the decomposition's retry rule (haar.hpp:171-181,211-224).
//   * joint layer measurement: chunks of <=16 sites in ascending order, one
//     U(0,1) per chunk, histogram bin i has bit j = outcome of chunk site j,
//     linear CDF scan, starved-bin fallback, collapse scaled by
//     1/sqrt(branch weight)                      cpp/include/mipt/cusv/engine.hpp:293-368
//   * sequential single-site measurement         cpp/include/mipt/free_energy_measure.hpp:18-96
//   * reduced density matrix of any kept-mode list, qubit or fermionic trace
//                                                cpp/include/mipt/tmi/linalg.hpp:1098-1142,
//                                                cpp/include/mipt/cuda/schmidt_gram.cuh:196-249
//   * entropies in bits with the 1e-15 eigenvalue cut and 1e-12 zero snap
//                                                cpp/include/mipt/tmi/linalg.hpp:125-141,201-208
//   * TMI over four contiguous cyclic quarters   cpp/include/mipt/tmi/compute.hpp:186-227
//   * three-site RDMs on the periodic ring       cpp/include/mipt/rdm.hpp:92-106,149-305
//   * free-energy protocol                       cpp/apps/free_energy.cpp:454-533
//     per-trajectory streams: trajectory_seed = splitmix64(master ^ index);
//     workspace seed = low 32 bits of splitmix64(trajectory_seed ^ "CIRCUITU");
//     initial-state stream mt19937_64(splitmix64(trajectory_seed ^ "INITIALS"))
//     workspace layer/measurement streams       cpp/include/mipt/probed.hpp:103-108
//     random product / Haar initial states       cpp/include/mipt/free_energy.hpp:125-222
//     half-chain S1 schedule                     cpp/include/mipt/free_energy_resume.hpp:150-166
//   * RPPU / qRPPU brickwork                     cpp/include/mipt/circuits/rppu_layer.hpp:51-285
//     (haar_unitary_2 blocks, even block first; random extra even layer drawn
//     first; closure gate first in the odd layer: FSWAP chain, JW-string or
//     direct qubit form), ops as cpp/include/mipt/cusv/gates.hpp:229-281
//     builds them; encoded measurement (site n-1 as its own final chunk)
//                                                cpp/include/mipt/cusv/engine.hpp:364-458
#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <random>
#include <stdexcept>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using cd = std::complex<double>;

namespace
{
std::uint64_t mix64(std::uint64_t v)
{
    v += 0x9e3779b97f4a7c15ull;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ull;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebull;
    return v ^ (v >> 31);
}

void seed_pair(std::uint64_t s, std::mt19937 &gates, std::mt19937 &meas)
{
    std::seed_seq a{static_cast<std::uint32_t>(s), static_cast<std::uint32_t>(s >> 32)};
    gates.seed(a);
    const std::uint64_t m = mix64(s ^ 0xa0761d0dull);
    std::seed_seq b{static_cast<std::uint32_t>(m), static_cast<std::uint32_t>(m >> 32)};
    meas.seed(b);
}

// One Haar U(4) (row-major), redrawn while its cosine-sine split would be
// singular, exactly as often as the reference redraws.
std::array<cd, 16> draw_u4(std::mt19937 &rng)
{
    for (;;)
    {
        std::normal_distribution<double> gauss(0.0, 1.0);
        std::array<cd, 16> q{};
        for (int c = 0; c < 4; ++c)
        {
            cd v[4];
            for (int r = 0; r < 4; ++r)
            {
                // The reference writes cd(normal(rng), normal(rng)); the order
                // in which those two arguments are evaluated is unspecified in
                // C++, and the g++ build that serves as the parity record
                // evaluates the imaginary part first. Draw in that order
                // explicitly.
                const double im = gauss(rng);
                const double re = gauss(rng);
                v[r] = cd(re, im);
            }
            for (int k = 0; k < c; ++k)
            {
                cd dot = 0.0;
                for (int r = 0; r < 4; ++r) dot += std::conj(q[r * 4 + k]) * v[r];
                for (int r = 0; r < 4; ++r) v[r] -= q[r * 4 + k] * dot;
            }
            double nn = 0.0;
            for (int r = 0; r < 4; ++r) nn += std::norm(v[r]);
            const double len = std::sqrt(nn);
            if (len < 1e-14)
            {
                --c;
                continue;
            }
            for (int r = 0; r < 4; ++r) q[r * 4 + c] = v[r] / len;
        }
        // Singular-value check of the top-left 2x2 block X: eigenvalues of
        // X^H X are the squared cosines; a cosine or sine below 1e-12 makes
        // the reference discard the draw.
        const cd x00 = q[0], x01 = q[1], x10 = q[4], x11 = q[5];
        const double h00 = std::norm(x00) + std::norm(x10);
        const double h11 = std::norm(x01) + std::norm(x11);
        const cd h01 = std::conj(x00) * x01 + std::conj(x10) * x11;
        const double disc = std::sqrt(std::max(0.0, (h00 - h11) * (h00 - h11) + 4.0 * std::norm(h01)));
        const double l0 = std::clamp(0.5 * (h00 + h11 + disc), 0.0, 1.0);
        const double l1 = std::clamp(0.5 * (h00 + h11 - disc), 0.0, 1.0);
        const double eps = 1e-12;
        if (std::sqrt(l0) < eps || std::sqrt(l1) < eps || std::sqrt(std::max(0.0, 1.0 - l0)) < eps ||
            std::sqrt(std::max(0.0, 1.0 - l1)) < eps)
            continue;
        return q;
    }
}

struct Layer
{
    std::vector<int> q;          // 2 per gate
    std::vector<cd> m;           // 16 per gate
    std::vector<int> sites;      // measured sites, ascending
};

void draw_layer(Layer &L, int n, int start, double p, bool closed, std::mt19937 &rng)
{
    const int stop = (closed && start == 1 && n > 2) ? n : n - 1;
    L.q.clear();
    L.m.clear();
    L.sites.clear();
    for (int i = start; i < stop; i += 2)
    {
        const auto u = draw_u4(rng);
        L.q.push_back(i);
        L.q.push_back((i + 1) % n);
        L.m.insert(L.m.end(), u.begin(), u.end());
    }
    if (p >= 1.0)
    {
        for (int s = 0; s < n; ++s) L.sites.push_back(s);
    }
    else if (p > 0.0)
    {
        std::bernoulli_distribution flag(p);
        for (int s = 0; s < n; ++s)
            if (flag(rng)) L.sites.push_back(s);
    }
}

void draw_trajectory(std::vector<Layer> &layers, std::uint64_t seed, int n, int periods, double p,
                     bool closed, std::mt19937 &meas)
{
    if (n % 2 != 0) throw std::invalid_argument("Haar brickwork needs even n");
    std::mt19937 gates;
    seed_pair(seed, gates, meas);
    layers.resize(2 * periods);
    for (int t = 0; t < 2 * periods; ++t) draw_layer(layers[t], n, t & 1, p, closed, gates);
}

// Four-colour 2-D brickwork on an X x Y torus, qubit q = r * X + c: the loops
// of the reference's python/mipt.py:244-311 (colour 0/1 horizontal, 2/3
// vertical; lines of the colour's parity pair from site 0, the other lines
// take the wrap bond first and pair from site 1). Lines of odd length get no
// wrap bond (the reference's square-lattice indexing leaves them undefined).
std::vector<std::pair<int, int>> lattice_colour(int X, int Y, int colour)
{
    std::vector<std::pair<int, int>> b;
    const bool horizontal = colour < 2;
    const int lines = horizontal ? Y : X, len = horizontal ? X : Y;
    for (int i = 0; i < lines; ++i)
    {
        auto site = [&](int j) { return horizontal ? i * X + j : j * X + i; };
        if (i % 2 == colour % 2)
        {
            for (int j = 0; j + 1 < len; j += 2) b.emplace_back(site(j), site(j + 1));
        }
        else
        {
            if (len % 2 == 0) b.emplace_back(site(0), site(len - 1));
            for (int j = 1; j + 1 < len - (len % 2 == 0 ? 1 : 0); j += 2) b.emplace_back(site(j), site(j + 1));
        }
    }
    return b;
}

void draw_lattice_trajectory(std::vector<Layer> &layers, std::uint64_t seed, int X, int Y, int T, double p,
                             std::mt19937 &meas)
{
    std::mt19937 gates;
    seed_pair(seed, gates, meas);
    const int n = X * Y;
    layers.resize(T);
    for (int t = 0; t < T; ++t)
    {
        Layer &L = layers[t];
        L.q.clear();
        L.m.clear();
        L.sites.clear();
        for (const auto &pr : lattice_colour(X, Y, t % 4))
        {
            const auto u = draw_u4(gates);
            L.q.push_back(pr.first);
            L.q.push_back(pr.second);
            L.m.insert(L.m.end(), u.begin(), u.end());
        }
        if (p >= 1.0)
        {
            for (int s = 0; s < n; ++s) L.sites.push_back(s);
        }
        else if (p > 0.0)
        {
            std::bernoulli_distribution flag(p);
            for (int s = 0; s < n; ++s)
                if (flag(gates)) L.sites.push_back(s);
        }
    }
}

// psi <- U psi on (q0, q1); U row-major with index bit 0 = q0, bit 1 = q1.
void apply_bond(cd *psi, int n, int q0, int q1, const cd *U)
{
    const std::uint64_t a = 1ull << q0, b = 1ull << q1;
    const std::uint64_t lo = std::min(a, b), hi = std::max(a, b);
    const std::uint64_t groups = 1ull << (n - 2);
    for (std::uint64_t g = 0; g < groups; ++g)
    {
        std::uint64_t base = g;
        base = ((base & ~(lo - 1)) << 1) | (base & (lo - 1));
        base = ((base & ~(hi - 1)) << 1) | (base & (hi - 1));
        const std::uint64_t idx[4] = {base, base | a, base | b, base | a | b};
        cd in[4];
        for (int c = 0; c < 4; ++c) in[c] = psi[idx[c]];
        for (int r = 0; r < 4; ++r)
        {
            cd acc = 0.0;
            for (int c = 0; c < 4; ++c) acc += U[r * 4 + c] * in[c];
            psi[idx[r]] = acc;
        }
    }
}

// Joint measurement of `sites` (ascending) in chunks; returns the layer's
// surprisal -log P. `forced` (optional) replays recorded outcomes instead of
// sampling; `probs` (optional) receives each chunk's branch/total.
double measure_layer(cd *psi, int n, const std::vector<int> &sites, int chunk_bits,
                     const double *uniforms, int &u_used, const int *forced, int *outcomes)
{
    double surprisal = 0.0;
    const std::uint64_t dim = 1ull << n;
    std::vector<double> bins;
    for (std::size_t begin = 0; begin < sites.size(); begin += chunk_bits)
    {
        const std::size_t end = std::min(sites.size(), begin + static_cast<std::size_t>(chunk_bits));
        const int m = static_cast<int>(end - begin);
        bins.assign(1ull << m, 0.0);
        for (std::uint64_t x = 0; x < dim; ++x)
        {
            std::uint64_t bin = 0;
            for (int j = 0; j < m; ++j) bin |= ((x >> sites[begin + j]) & 1ull) << j;
            bins[bin] += std::norm(psi[x]);
        }
        double total = 0.0;
        for (double v : bins) total += v;
        if (!(total > 0.0) || !std::isfinite(total)) throw std::runtime_error("zero-norm state");
        const double u = uniforms[u_used++];
        std::uint64_t chosen = bins.size() - 1;
        if (forced)
        {
            chosen = 0;
            for (int j = 0; j < m; ++j) chosen |= static_cast<std::uint64_t>(forced[begin + j] & 1) << j;
        }
        else
        {
            const double draw = u * total;
            double run = 0.0;
            for (std::uint64_t i = 0; i < bins.size(); ++i)
            {
                run += bins[i];
                if (draw < run)
                {
                    chosen = i;
                    break;
                }
            }
        }
        double branch = bins[chosen];
        if (!(branch > 0.0))
        {
            if (forced) throw std::runtime_error("forced outcome has zero weight");
            chosen = static_cast<std::uint64_t>(std::max_element(bins.begin(), bins.end()) - bins.begin());
            branch = bins[chosen];
            if (!(branch > 0.0)) throw std::runtime_error("no outcome with positive weight");
        }
        for (int j = 0; j < m; ++j) outcomes[begin + j] = static_cast<int>((chosen >> j) & 1ull);
        surprisal += -std::log(branch / total);
        const double scale = 1.0 / std::sqrt(branch);
        for (std::uint64_t x = 0; x < dim; ++x)
        {
            std::uint64_t bin = 0;
            for (int j = 0; j < m; ++j) bin |= ((x >> sites[begin + j]) & 1ull) << j;
            psi[x] = (bin == chosen) ? psi[x] * scale : cd(0.0, 0.0);
        }
    }
    return surprisal;
}

// rho[row*D + col] = sum_env M[row, env] conj(M[col, env]); row bit k <-> kept[k],
// env index over the complement in ascending mode order; fermionic trace flips
// the sign of M[row, env] once per occupied environment mode below each
// occupied kept mode.
void rdm(const cd *psi, int n, const int *kept, int k, bool fermion, cd *rho)
{
    std::vector<int> env;
    std::vector<char> is_kept(n, 0);
    for (int i = 0; i < k; ++i)
    {
        if (kept[i] < 0 || kept[i] >= n || is_kept[kept[i]]) throw std::invalid_argument("bad kept modes");
        is_kept[kept[i]] = 1;
    }
    for (int q = 0; q < n; ++q)
        if (!is_kept[q]) env.push_back(q);
    const std::uint64_t D = 1ull << k, E = 1ull << env.size();
    std::vector<std::uint64_t> roff(D), cross(D, 0);
    std::vector<std::uint64_t> below(k, 0);
    for (int i = 0; i < k; ++i)
        for (std::size_t e = 0; e < env.size(); ++e)
            if (env[e] < kept[i]) below[i] |= 1ull << e;
    for (std::uint64_t r = 0; r < D; ++r)
    {
        std::uint64_t o = 0, c = 0;
        for (int i = 0; i < k; ++i)
            if ((r >> i) & 1ull)
            {
                o |= 1ull << kept[i];
                c ^= below[i];
            }
        roff[r] = o;
        cross[r] = c;
    }
    std::fill(rho, rho + D * D, cd(0.0, 0.0));
    std::vector<cd> col(D);
    for (std::uint64_t e = 0; e < E; ++e)
    {
        std::uint64_t eo = 0;
        for (std::size_t j = 0; j < env.size(); ++j)
            if ((e >> j) & 1ull) eo |= 1ull << env[j];
        for (std::uint64_t r = 0; r < D; ++r)
        {
            cd v = psi[eo | roff[r]];
            if (fermion && (__builtin_popcountll(e & cross[r]) & 1)) v = -v;
            col[r] = v;
        }
        for (std::uint64_t r = 0; r < D; ++r)
            for (std::uint64_t c = 0; c < D; ++c) rho[r * D + c] += col[r] * std::conj(col[c]);
    }
}

// Eigenvalues of a Hermitian matrix (row-major, destroyed) by cyclic complex
// Jacobi rotations, to full double accuracy.
void eig_hermitian(std::vector<cd> &a, int n, std::vector<double> &w)
{
    for (int i = 0; i < n; ++i)
    {
        a[i * n + i] = cd(a[i * n + i].real(), 0.0);
        for (int j = i + 1; j < n; ++j)
        {
            const cd h = 0.5 * (a[i * n + j] + std::conj(a[j * n + i]));
            a[i * n + j] = h;
            a[j * n + i] = std::conj(h);
        }
    }
    for (int sweep = 0; sweep < 100; ++sweep)
    {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; ++i)
        {
            diag += a[i * n + i].real() * a[i * n + i].real();
            for (int j = i + 1; j < n; ++j) off += std::norm(a[i * n + j]);
        }
        if (off <= 1e-32 * std::max(diag, 1e-300)) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q)
            {
                const cd apq = a[p * n + q];
                const double mag = std::abs(apq);
                if (mag < 1e-300) continue;
                const double app = a[p * n + p].real(), aqq = a[q * n + q].real();
                const double theta = (aqq - app) / (2.0 * mag);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::abs(theta) + std::sqrt(1.0 + theta * theta));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
                const cd ph = apq / mag; // e^{i phi}
                // Rotation acting on columns p, q:  [c, s*ph; -s*conj(ph), c]
                for (int k = 0; k < n; ++k)
                {
                    const cd akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * std::conj(ph) * akq;
                    a[k * n + q] = s * ph * akp + c * akq;
                }
                for (int k = 0; k < n; ++k)
                {
                    const cd apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * ph * aqk;
                    a[q * n + k] = s * std::conj(ph) * apk + c * aqk;
                }
                a[p * n + q] = 0.0;
                a[q * n + p] = 0.0;
            }
    }
    w.resize(n);
    for (int i = 0; i < n; ++i) w[i] = a[i * n + i].real();
}

double snap(double s) { return std::abs(s) < 1e-12 ? 0.0 : s; }

double entropy_from_rdm(const cd *rho, int d, int order)
{
    if (d == 1) return 0.0;
    if (order == 2)
    {
        double pur = 0.0;
        for (int i = 0; i < d; ++i)
        {
            pur += rho[i * d + i].real() * rho[i * d + i].real();
            for (int j = i + 1; j < d; ++j)
            {
                const cd h = 0.5 * (rho[i * d + j] + std::conj(rho[j * d + i]));
                pur += 2.0 * std::norm(h);
            }
        }
        if (!(pur > 0.0) || pur >= 1.0) return 0.0;
        return snap(-std::log2(pur));
    }
    std::vector<cd> a(rho, rho + static_cast<std::size_t>(d) * d);
    std::vector<double> w;
    eig_hermitian(a, d, w);
    double s = 0.0;
    for (double l : w)
        if (l > 1e-15) s -= l * std::log2(l);
    return snap(s);
}

double subsystem_entropy(const cd *psi, int n, const std::vector<int> &kept, int order, bool fermion = false)
{
    const int d = 1 << kept.size();
    std::vector<cd> rho(static_cast<std::size_t>(d) * d);
    rdm(psi, n, kept.data(), static_cast<int>(kept.size()), fermion, rho.data());
    return entropy_from_rdm(rho.data(), d, order);
}

std::vector<int> cyc(int begin, int count, int n)
{
    std::vector<int> v;
    for (int i = 0; i < count; ++i) v.push_back(((begin + i) % n + n) % n);
    return v;
}

double tmi(const cd *psi, int n, int offset, int order)
{
    const int b = n / 4;
    const auto A = cyc(offset, b, n), B = cyc(offset + b, b, n), C = cyc(offset + 2 * b, b, n),
               D = cyc(offset + 3 * b, b, n);
    auto cat = [](std::vector<int> x, const std::vector<int> &y) {
        x.insert(x.end(), y.begin(), y.end());
        return x;
    };
    return subsystem_entropy(psi, n, A, order) + subsystem_entropy(psi, n, B, order) +
           subsystem_entropy(psi, n, C, order) + subsystem_entropy(psi, n, D, order) -
           subsystem_entropy(psi, n, cat(A, B), order) - subsystem_entropy(psi, n, cat(A, C), order) -
           subsystem_entropy(psi, n, cat(B, C), order);
}

std::vector<int> half_chain(int n)
{
    std::vector<int> v;
    for (int i = 0; i < n / 2; ++i) v.push_back(i);
    return v;
}
} // namespace


// ---------------------------------------------------------------------------
// Free-fermion (Gaussian) monitored circuit on the Majorana covariance
// matrix. The reference has no code for this path (it simulates fermionic
// circuits only as Jordan-Wigner state vectors); this is a restatement from
// the mathematics, cross-checked in the tests against the state-vector
// restatement above with the fermionic trace.
//
//   Gamma_ab = (i/2) <[g_a, g_b]>, real antisymmetric, Gamma^2 = -1 (pure)
//   product state: Gamma_{2j,2j+1} = 1 (i g_{2j} g_{2j+1} = +1 on every mode)
//   gate on modes (k, k+1 mod N): Haar SO(4) rotation O on Majoranas
//     (2k, 2k+1, 2k', 2k'+1), Gamma <- O Gamma O^T
//   measurement of P_j = i g_{2j} g_{2j+1}: outcome s = +1 with probability
//     (1 + Gamma_ab)/2 (a = 2j, b = 2j+1); then for k, l outside {a, b}
//     Gamma_kl += (Gamma_kb Gamma_la - Gamma_ka Gamma_lb) / (Gamma_ab + s),
//     rows/columns a, b are cleared and Gamma_ab = s.
//   re-purification: Gamma <- Gamma (3 + Gamma^2) / 2 (Newton-Schulz step of
//     the matrix sign of i Gamma).
//   entropy of a mode set M (bits): eigenvalues +-nu of i Gamma_M,
//     S = sum_{pairs} H2((1 + nu)/2).
namespace ff
{
using Mat = std::vector<double>;

void so4_haar(std::mt19937 &rng, double *O)
{
    std::normal_distribution<double> gauss(0.0, 1.0);
    double q[16];
    for (int c = 0; c < 4; ++c)
    {
        double v[4];
        for (int r = 0; r < 4; ++r) v[r] = gauss(rng);
        for (int k = 0; k < c; ++k)
        {
            double dot = 0.0;
            for (int r = 0; r < 4; ++r) dot += q[r * 4 + k] * v[r];
            for (int r = 0; r < 4; ++r) v[r] -= q[r * 4 + k] * dot;
        }
        double nn = 0.0;
        for (int r = 0; r < 4; ++r) nn += v[r] * v[r];
        const double len = std::sqrt(nn);
        for (int r = 0; r < 4; ++r) q[r * 4 + c] = v[r] / len;
    }
    // determinant sign by cofactor expansion
    auto det3 = [&](int r0, int r1, int r2, int c0, int c1, int c2) {
        return q[r0 * 4 + c0] * (q[r1 * 4 + c1] * q[r2 * 4 + c2] - q[r1 * 4 + c2] * q[r2 * 4 + c1]) -
               q[r0 * 4 + c1] * (q[r1 * 4 + c0] * q[r2 * 4 + c2] - q[r1 * 4 + c2] * q[r2 * 4 + c0]) +
               q[r0 * 4 + c2] * (q[r1 * 4 + c0] * q[r2 * 4 + c1] - q[r1 * 4 + c1] * q[r2 * 4 + c0]);
    };
    const double det = q[0] * det3(1, 2, 3, 1, 2, 3) - q[1] * det3(1, 2, 3, 0, 2, 3) + q[2] * det3(1, 2, 3, 0, 1, 3) -
                       q[3] * det3(1, 2, 3, 0, 1, 2);
    if (det < 0)
        for (int r = 0; r < 4; ++r) q[r * 4] = -q[r * 4];
    std::copy(q, q + 16, O);
}

struct Layer
{
    std::vector<int> modes;   // first mode of each gate (gate on (m, m+1 mod N))
    std::vector<double> rot;  // 16 per gate, row-major
    std::vector<int> sites;   // measured modes, ascending
};

void draw(std::vector<Layer> &layers, std::uint64_t seed, int N, int depth, double p, bool closed,
          std::mt19937 &meas)
{
    std::mt19937 g;
    seed_pair(seed, g, meas);
    layers.resize(depth);
    for (int t = 0; t < depth; ++t)
    {
        Layer &L = layers[t];
        L.modes.clear();
        L.rot.clear();
        L.sites.clear();
        const int start = t & 1;
        const int stop = (closed && start == 1 && N > 2) ? N : N - 1;
        for (int m = start; m < stop; m += 2)
        {
            double O[16];
            so4_haar(g, O);
            L.modes.push_back(m);
            L.rot.insert(L.rot.end(), O, O + 16);
        }
        if (p >= 1.0)
            for (int j = 0; j < N; ++j) L.sites.push_back(j);
        else if (p > 0.0)
        {
            std::bernoulli_distribution flag(p);
            for (int j = 0; j < N; ++j)
                if (flag(g)) L.sites.push_back(j);
        }
    }
}

void rotate(Mat &G, int N, int m, const double *O)
{
    const int M = 2 * N;
    const int m2 = (m + 1) % N;
    const int idx[4] = {2 * m, 2 * m + 1, 2 * m2, 2 * m2 + 1};
    // rows: G[idx, :] = O G[idx, :]
    std::vector<double> tmp(4 * M);
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < M; ++c)
        {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += O[r * 4 + k] * G[idx[k] * M + c];
            tmp[r * M + c] = s;
        }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < M; ++c) G[idx[r] * M + c] = tmp[r * M + c];
    // columns: G[:, idx] = G[:, idx] O^T
    for (int r = 0; r < M; ++r)
    {
        double row[4];
        for (int k = 0; k < 4; ++k) row[k] = G[r * M + idx[k]];
        for (int c = 0; c < 4; ++c)
        {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += row[k] * O[c * 4 + k];
            G[r * M + idx[c]] = s;
        }
    }
}

// Returns the outcome s and the probability of it.
int measure(Mat &G, int N, int j, double u, const int *forced, double &prob)
{
    const int M = 2 * N, a = 2 * j, b = 2 * j + 1;
    const double g = G[a * M + b];
    const double p_plus = std::clamp((1.0 + g) / 2.0, 0.0, 1.0);
    int s = forced ? (*forced > 0 ? 1 : -1) : (u < p_plus ? 1 : -1);
    prob = s > 0 ? p_plus : 1.0 - p_plus;
    const double denom = g + s;
    std::vector<double> ua(M), vb(M);
    for (int k = 0; k < M; ++k)
    {
        ua[k] = G[k * M + a];
        vb[k] = G[k * M + b];
    }
    for (int k = 0; k < M; ++k)
    {
        if (k == a || k == b) continue;
        for (int l = 0; l < M; ++l)
        {
            if (l == a || l == b) continue;
            G[k * M + l] += (vb[k] * ua[l] - ua[k] * vb[l]) / denom;
        }
    }
    for (int k = 0; k < M; ++k)
    {
        G[k * M + a] = G[a * M + k] = 0.0;
        G[k * M + b] = G[b * M + k] = 0.0;
    }
    G[a * M + b] = s;
    G[b * M + a] = -s;
    return s;
}

void repurify(Mat &G, int N)
{
    const int M = 2 * N;
    Mat G2(M * M, 0.0), out(M * M, 0.0);
    for (int i = 0; i < M; ++i)
        for (int k = 0; k < M; ++k)
        {
            const double gik = G[i * M + k];
            if (gik == 0.0) continue;
            for (int j = 0; j < M; ++j) G2[i * M + j] += gik * G[k * M + j];
        }
    for (int i = 0; i < M; ++i) G2[i * M + i] += 3.0;
    for (int i = 0; i < M; ++i)
        for (int k = 0; k < M; ++k)
        {
            const double gik = G[i * M + k];
            if (gik == 0.0) continue;
            for (int j = 0; j < M; ++j) out[i * M + j] += 0.5 * gik * G2[k * M + j];
        }
    G.swap(out);
}

double h2(double x)
{
    double s = 0.0;
    if (x > 1e-15) s -= x * std::log2(x);
    if (1.0 - x > 1e-15) s -= (1.0 - x) * std::log2(1.0 - x);
    return s;
}

double block_entropy(const Mat &G, int N, const std::vector<int> &modes)
{
    const int m = static_cast<int>(modes.size());
    if (m == 0) return 0.0;
    const int M = 2 * N, d = 2 * m;
    std::vector<int> maj;
    for (int q : modes)
    {
        maj.push_back(2 * q);
        maj.push_back(2 * q + 1);
    }
    // i * Gamma_M is Hermitian; its eigenvalues come in +-nu pairs.
    std::vector<cd> H(d * d);
    for (int r = 0; r < d; ++r)
        for (int c = 0; c < d; ++c) H[r * d + c] = cd(0.0, G[maj[r] * M + maj[c]]);
    std::vector<double> w;
    eig_hermitian(H, d, w);
    double s = 0.0;
    for (double l : w) s += 0.5 * h2(std::clamp((1.0 + l) / 2.0, 0.0, 1.0));
    return std::abs(s) < 1e-12 ? 0.0 : s;
}
} // namespace ff

extern "C" {

std::uint64_t orc_splitmix64(std::uint64_t v) { return mix64(v); }
std::uint64_t orc_trajectory_seed(std::uint64_t master, std::uint64_t index)
{
    return mix64(master + 0x2545f4914f6cdd1dull * (index + 1ull));
}

// Same output layout as the reference harness's ref_haar_draw.
int orc_haar_draw(std::uint64_t seed, int n, int periods, double p, int closed, int chunk_bits,
                  int *gates_per_layer, int *gate_q, double *gate_m, int *sites_per_layer, int *sites,
                  double *uniforms, int *n_uniforms)
{
    try
    {
        std::mt19937 meas;
        std::vector<Layer> layers;
        draw_trajectory(layers, seed, n, periods, p, closed != 0, meas);
        const int mg = n / 2;
        int u = 0;
        std::uniform_real_distribution<double> unif(0.0, 1.0);
        for (std::size_t t = 0; t < layers.size(); ++t)
        {
            const int g = static_cast<int>(layers[t].q.size() / 2);
            gates_per_layer[t] = g;
            for (int i = 0; i < g; ++i)
            {
                gate_q[(t * mg + i) * 2] = layers[t].q[2 * i];
                gate_q[(t * mg + i) * 2 + 1] = layers[t].q[2 * i + 1];
                for (int e = 0; e < 16; ++e)
                {
                    gate_m[(t * mg + i) * 32 + 2 * e] = layers[t].m[16 * i + e].real();
                    gate_m[(t * mg + i) * 32 + 2 * e + 1] = layers[t].m[16 * i + e].imag();
                }
            }
            sites_per_layer[t] = static_cast<int>(layers[t].sites.size());
            for (std::size_t s = 0; s < layers[t].sites.size(); ++s) sites[t * n + s] = layers[t].sites[s];
            for (std::size_t s = 0; s < layers[t].sites.size(); s += chunk_bits) uniforms[u++] = unif(meas);
        }
        *n_uniforms = u;
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

int orc_lattice_bonds(int X, int Y, int colour, int *pairs)
{
    const auto b = lattice_colour(X, Y, colour);
    for (std::size_t i = 0; i < b.size(); ++i)
    {
        pairs[2 * i] = b[i].first;
        pairs[2 * i + 1] = b[i].second;
    }
    return static_cast<int>(b.size());
}

// The 2-D draw in orc_haar_draw's output layout (layers = T).
int orc_haar_lattice_draw(std::uint64_t seed, int X, int Y, int T, double p, int chunk_bits, int *gates_per_layer,
                          int *gate_q, double *gate_m, int *sites_per_layer, int *sites, double *uniforms,
                          int *n_uniforms)
{
    try
    {
        std::mt19937 meas;
        std::vector<Layer> layers;
        draw_lattice_trajectory(layers, seed, X, Y, T, p, meas);
        const int n = X * Y, mg = n / 2;
        int u = 0;
        std::uniform_real_distribution<double> unif(0.0, 1.0);
        for (std::size_t t = 0; t < layers.size(); ++t)
        {
            const int g = static_cast<int>(layers[t].q.size() / 2);
            gates_per_layer[t] = g;
            for (int i = 0; i < g; ++i)
            {
                gate_q[(t * mg + i) * 2] = layers[t].q[2 * i];
                gate_q[(t * mg + i) * 2 + 1] = layers[t].q[2 * i + 1];
                for (int e = 0; e < 16; ++e)
                {
                    gate_m[(t * mg + i) * 32 + 2 * e] = layers[t].m[16 * i + e].real();
                    gate_m[(t * mg + i) * 32 + 2 * e + 1] = layers[t].m[16 * i + e].imag();
                }
            }
            sites_per_layer[t] = static_cast<int>(layers[t].sites.size());
            for (std::size_t s = 0; s < layers[t].sites.size(); ++s) sites[t * n + s] = layers[t].sites[s];
            for (std::size_t s = 0; s < layers[t].sites.size(); s += chunk_bits) uniforms[u++] = unif(meas);
        }
        *n_uniforms = u;
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// A 2-D trajectory in FP64: outcomes[layer][n] (ascending measured sites, -1
// padding), surprisal[layer], the state after every layer whose index+1 is a
// multiple of observe_every into states_ri[point] (nullable), final state.
int orc_run_lattice_trajectory(std::uint64_t seed, int X, int Y, int T, double p, int chunk_bits,
                               const int *forced, int *outcomes, double *surprisal, int observe_every,
                               double *states_ri, double *final_psi_ri)
{
    try
    {
        std::mt19937 meas;
        std::vector<Layer> layers;
        draw_lattice_trajectory(layers, seed, X, Y, T, p, meas);
        const int n = X * Y;
        const std::uint64_t dim = 1ull << n;
        std::vector<cd> psi(dim, cd(0.0, 0.0));
        psi[0] = 1.0;
        std::uniform_real_distribution<double> unif(0.0, 1.0);
        for (int t = 0; t < T; ++t)
        {
            const Layer &L = layers[t];
            for (std::size_t g = 0; g < L.q.size() / 2; ++g)
                apply_bond(psi.data(), n, L.q[2 * g], L.q[2 * g + 1], &L.m[16 * g]);
            std::vector<double> us;
            for (std::size_t s = 0; s < L.sites.size(); s += chunk_bits) us.push_back(unif(meas));
            std::vector<int> oc(L.sites.size(), 0);
            int used = 0;
            const double sp = measure_layer(psi.data(), n, L.sites, chunk_bits, us.data(), used,
                                            forced ? forced + static_cast<std::size_t>(t) * n : nullptr, oc.data());
            if (surprisal) surprisal[t] = sp;
            if (outcomes)
            {
                for (int s = 0; s < n; ++s) outcomes[static_cast<std::size_t>(t) * n + s] = -1;
                for (std::size_t s = 0; s < oc.size(); ++s) outcomes[static_cast<std::size_t>(t) * n + s] = oc[s];
            }
            if (states_ri && observe_every > 0 && (t + 1) % observe_every == 0)
                std::memcpy(states_ri + static_cast<std::size_t>((t + 1) / observe_every - 1) * 2 * dim, psi.data(),
                            dim * sizeof(cd));
        }
        if (final_psi_ri) std::memcpy(final_psi_ri, psi.data(), dim * sizeof(cd));
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

void orc_apply_bond(double *psi_ri, int n, int q0, int q1, const double *m_ri)
{
    apply_bond(reinterpret_cast<cd *>(psi_ri), n, q0, q1, reinterpret_cast<const cd *>(m_ri));
}

int orc_measure_layer(double *psi_ri, int n, const int *sites, int m, int chunk_bits, const double *uniforms,
                      const int *forced, int *outcomes, double *surprisal)
{
    try
    {
        std::vector<int> s(sites, sites + m);
        int used = 0;
        *surprisal = measure_layer(reinterpret_cast<cd *>(psi_ri), n, s, chunk_bits, uniforms, used, forced, outcomes);
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

int orc_measure_collapse(double *psi_ri, int n, int q, double u, int *outcome, double *cond_p)
{
    cd *psi = reinterpret_cast<cd *>(psi_ri);
    const std::uint64_t dim = 1ull << n, mask = 1ull << q;
    long double tot = 0.0L, one = 0.0L;
    for (std::uint64_t x = 0; x < dim; ++x)
    {
        const long double w = std::norm(psi[x]);
        tot += w;
        if (x & mask) one += w;
    }
    const double t = static_cast<double>(tot), o = static_cast<double>(one);
    if (!(t > 0.0) || !std::isfinite(t) || !(u >= 0.0 && u < 1.0)) return 1;
    const double p1 = std::clamp(o / t, 0.0, 1.0);
    const int bit = u < p1 ? 1 : 0;
    const double branch = bit ? o : t - o;
    if (!(branch > 0.0)) return 1;
    const double scale = 1.0 / std::sqrt(branch);
    for (std::uint64_t x = 0; x < dim; ++x)
        psi[x] = (((x & mask) != 0) == (bit == 1)) ? psi[x] * scale : cd(0.0, 0.0);
    *outcome = bit;
    *cond_p = bit ? p1 : 1.0 - p1;
    return 0;
}

int orc_rdm(const double *psi_ri, int n, const int *kept, int k, int fermion, double *rho_ri)
{
    try
    {
        rdm(reinterpret_cast<const cd *>(psi_ri), n, kept, k, fermion != 0, reinterpret_cast<cd *>(rho_ri));
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

double orc_entropy_hermitian(const double *rho_ri, int d, int order)
{
    return entropy_from_rdm(reinterpret_cast<const cd *>(rho_ri), d, order);
}

int orc_eigvalsh(const double *rho_ri, int d, double *w_out)
{
    std::vector<cd> a(reinterpret_cast<const cd *>(rho_ri), reinterpret_cast<const cd *>(rho_ri) + d * d);
    std::vector<double> w;
    eig_hermitian(a, d, w);
    std::sort(w.begin(), w.end());
    std::copy(w.begin(), w.end(), w_out);
    return 0;
}

double orc_tmi(const double *psi_ri, int n, int offset, int order)
{
    return tmi(reinterpret_cast<const cd *>(psi_ri), n, offset, order);
}

int orc_rho3(const double *psi_ri, int n, const int *subs, int count, int fermion, double *out)
{
    try
    {
        for (int s = 0; s < count; ++s)
        {
            const int *q = subs + 3 * s;
            cd *rho = reinterpret_cast<cd *>(out + 128 * s);
            rdm(reinterpret_cast<const cd *>(psi_ri), n, q, 3, fermion != 0, rho);
            if (!fermion) continue;
            // The three-site trace orders modes as (q0, q1, q2, environment
            // ascending), so besides the kept/environment crossings it also
            // carries the sign of sorting the occupied kept modes among
            // themselves (cpp/src/cuda/rho_reduce.cu:49-68, rdm.hpp:41-75).
            int sgn[8];
            for (int r = 0; r < 8; ++r)
            {
                int par = 0;
                for (int i = 0; i < 3; ++i)
                    for (int j = i + 1; j < 3; ++j)
                        if (((r >> i) & 1) && ((r >> j) & 1) && q[i] > q[j]) par ^= 1;
                sgn[r] = par ? -1 : 1;
            }
            for (int r = 0; r < 8; ++r)
                for (int c = 0; c < 8; ++c) rho[r * 8 + c] *= static_cast<double>(sgn[r] * sgn[c]);
        }
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// One whole Haar trajectory in FP64.
//   obs_flags bit 0: half-chain S_vN, bit 1: half-chain S_2,
//             bit 2: TMI (von Neumann, offset 0), bit 3: TMI (Renyi-2, offset 0)
//   layer_obs[layer][4] gets those values (NaN where not requested) after
//   every layer whose index+1 is a multiple of observe_every (0 = last only).
//   outcomes[layer][n]: outcome of each measured site (in ascending-site
//   order), -1 padding; forced (same layout, optional) replays outcomes.
//   surprisal[layer]: -log P of the layer's joint outcome.
int orc_run_haar_trajectory(std::uint64_t seed, int n, int periods, double p, int closed, int chunk_bits,
                            int obs_flags, int observe_every, const int *forced, int *outcomes,
                            double *surprisal, double *layer_obs, double *final_psi_ri)
{
    try
    {
        std::mt19937 meas;
        std::vector<Layer> layers;
        draw_trajectory(layers, seed, n, periods, p, closed != 0, meas);
        const std::uint64_t dim = 1ull << n;
        std::vector<cd> psi(dim, cd(0.0, 0.0));
        psi[0] = 1.0;
        std::uniform_real_distribution<double> unif(0.0, 1.0);
        const int T = static_cast<int>(layers.size());
        for (int t = 0; t < T; ++t)
        {
            const Layer &L = layers[t];
            for (std::size_t g = 0; g < L.q.size() / 2; ++g)
                apply_bond(psi.data(), n, L.q[2 * g], L.q[2 * g + 1], &L.m[16 * g]);
            std::vector<double> us;
            for (std::size_t s = 0; s < L.sites.size(); s += chunk_bits) us.push_back(unif(meas));
            std::vector<int> oc(L.sites.size(), 0);
            int used = 0;
            const double sp = measure_layer(psi.data(), n, L.sites, chunk_bits, us.data(), used,
                                            forced ? forced + static_cast<std::size_t>(t) * n : nullptr, oc.data());
            if (surprisal) surprisal[t] = sp;
            if (outcomes)
            {
                for (int s = 0; s < n; ++s) outcomes[static_cast<std::size_t>(t) * n + s] = -1;
                for (std::size_t s = 0; s < oc.size(); ++s) outcomes[static_cast<std::size_t>(t) * n + s] = oc[s];
            }
            if (layer_obs)
            {
                double *o = layer_obs + 4 * static_cast<std::size_t>(t);
                for (int j = 0; j < 4; ++j) o[j] = std::nan("");
                const bool due = observe_every > 0 ? ((t + 1) % observe_every == 0) : (t == T - 1);
                if (due)
                {
                    if (obs_flags & 1) o[0] = subsystem_entropy(psi.data(), n, half_chain(n), 1);
                    if (obs_flags & 2) o[1] = subsystem_entropy(psi.data(), n, half_chain(n), 2);
                    if ((obs_flags & 4) && n % 4 == 0) o[2] = tmi(psi.data(), n, 0, 1);
                    if ((obs_flags & 8) && n % 4 == 0) o[3] = tmi(psi.data(), n, 0, 2);
                }
            }
        }
        if (final_psi_ri) std::memcpy(final_psi_ri, psi.data(), dim * sizeof(cd));
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// Many trajectories (trajectory_seed(master, first + i)), spread over host
// threads; returns the per-trajectory final half-chain S_2 in s2_out and
// the per-layer surprisal sum in surprisal_out. Used as the timed CPU
// baseline.
int orc_run_batch(std::uint64_t master, int first, int count, int n, int periods, double p, int closed,
                  int chunk_bits, int obs_flags, double *s2_out, double *surprisal_out, int threads)
{
    int failed = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : failed)
#endif
    for (int i = 0; i < count; ++i)
    {
        const std::uint64_t seed = orc_trajectory_seed(master, static_cast<std::uint64_t>(first + i));
        std::vector<double> sp(2 * periods), obs(4 * 2 * periods);
        const int rc = orc_run_haar_trajectory(seed, n, periods, p, closed, chunk_bits, obs_flags, 0, nullptr,
                                               nullptr, sp.data(), obs.data(), nullptr);
        if (rc) failed |= 1;
        double tot = 0.0;
        for (double v : sp) tot += v;
        if (surprisal_out) surprisal_out[i] = tot;
        if (s2_out) s2_out[i] = obs[4 * (2 * periods - 1) + 1];
    }
    return failed;
}


// Free-fermion trajectory: N modes, `depth` layers, measurement rate p.
//   forced[depth][N] (optional, +-1 per measured mode in ascending order)
//   outcomes[depth][N] receives +-1 (0 padding); probs likewise
//   gamma_out[2N x 2N] final covariance (optional)
//   block_len[nb] -> S of modes [0, len) in s_blocks[nb]; tmi_out: TMI of
//   contiguous quarters (N % 4 == 0), both in bits, final state.
int orc_ff_trajectory(std::uint64_t seed, int N, int depth, double p, int closed, int repurify_every,
                      const int *forced, int *outcomes, double *probs, double *gamma_out, const int *block_len,
                      int nb, double *s_blocks, double *tmi_out)
{
    try
    {
        std::mt19937 meas;
        std::vector<ff::Layer> layers;
        ff::draw(layers, seed, N, depth, p, closed != 0, meas);
        const int M = 2 * N;
        ff::Mat G(M * M, 0.0);
        for (int j = 0; j < N; ++j)
        {
            G[(2 * j) * M + 2 * j + 1] = 1.0;
            G[(2 * j + 1) * M + 2 * j] = -1.0;
        }
        std::uniform_real_distribution<double> unif(0.0, 1.0);
        for (int t = 0; t < depth; ++t)
        {
            const ff::Layer &L = layers[t];
            for (std::size_t g = 0; g < L.modes.size(); ++g) ff::rotate(G, N, L.modes[g], &L.rot[16 * g]);
            if (outcomes)
                for (int j = 0; j < N; ++j) outcomes[t * N + j] = 0;
            for (std::size_t i = 0; i < L.sites.size(); ++i)
            {
                const double u = unif(meas);
                double pr = 0.0;
                const int *f = forced ? &forced[t * N + i] : nullptr;
                const int s = ff::measure(G, N, L.sites[i], u, f, pr);
                if (outcomes) outcomes[t * N + i] = s;
                if (probs) probs[t * N + i] = pr;
            }
            if (repurify_every > 0 && (t + 1) % repurify_every == 0) ff::repurify(G, N);
        }
        if (gamma_out) std::copy(G.begin(), G.end(), gamma_out);
        for (int i = 0; i < nb; ++i)
        {
            std::vector<int> modes;
            for (int q = 0; q < block_len[i]; ++q) modes.push_back(q);
            s_blocks[i] = ff::block_entropy(G, N, modes);
        }
        if (tmi_out && N % 4 == 0)
        {
            const int b = N / 4;
            auto rng_ = [&](int a, int c) {
                std::vector<int> v;
                for (int i = 0; i < c; ++i) v.push_back(a + i);
                return v;
            };
            auto cat = [](std::vector<int> x, const std::vector<int> &y) {
                x.insert(x.end(), y.begin(), y.end());
                return x;
            };
            const auto A = rng_(0, b), B = rng_(b, b), C = rng_(2 * b, b), D = rng_(3 * b, b);
            *tmi_out = ff::block_entropy(G, N, A) + ff::block_entropy(G, N, B) + ff::block_entropy(G, N, C) +
                       ff::block_entropy(G, N, D) - ff::block_entropy(G, N, cat(A, B)) -
                       ff::block_entropy(G, N, cat(A, C)) - ff::block_entropy(G, N, cat(B, C));
        }
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// Layer draw of a free-fermion trajectory: gate first modes, rotations
// (16 per gate, row-major), measured-mode lists and measurement uniforms.
int orc_ff_draw(std::uint64_t seed, int N, int depth, double p, int closed, int *gates_per_layer, int *gate_mode,
                double *rot, int *sites_per_layer, int *sites, double *uniforms)
{
    try
    {
        std::mt19937 meas;
        std::vector<ff::Layer> layers;
        ff::draw(layers, seed, N, depth, p, closed != 0, meas);
        std::uniform_real_distribution<double> unif(0.0, 1.0);
        const int mg = N / 2 + 1;
        int u = 0;
        for (int t = 0; t < depth; ++t)
        {
            gates_per_layer[t] = static_cast<int>(layers[t].modes.size());
            for (std::size_t g = 0; g < layers[t].modes.size(); ++g)
            {
                gate_mode[t * mg + g] = layers[t].modes[g];
                std::copy(&layers[t].rot[16 * g], &layers[t].rot[16 * g] + 16, &rot[(t * mg + g) * 16]);
            }
            sites_per_layer[t] = static_cast<int>(layers[t].sites.size());
            for (std::size_t i = 0; i < layers[t].sites.size(); ++i)
            {
                sites[t * N + i] = layers[t].sites[i];
                uniforms[u++] = unif(meas);
            }
        }
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

double orc_ff_block_entropy(const double *gamma, int N, const int *modes, int m)
{
    ff::Mat G(gamma, gamma + 4 * N * N);
    return ff::block_entropy(G, N, std::vector<int>(modes, modes + m));
}

// Free-energy initial state: kind 0 random product, 1 random Haar; with
// fixed_parity a random global-parity sector. fp32 rounds every stored
// amplitude to float exactly where an FP32 state stores it. Returns 0; the
// sector (or -1) in *parity.
int orc_fe_initial_state(std::uint64_t seed, int n, int kind, int fixed_parity, int fp32, double *out_ri,
                         int *parity)
{
    try
    {
        const std::uint64_t dim = 1ull << n;
        std::mt19937_64 rng(seed);
        auto store = [fp32](cd v) { return fp32 ? cd(static_cast<float>(v.real()), static_cast<float>(v.imag())) : v; };
        std::vector<cd> a(dim, cd(0.0, 0.0));
        int sector = -1;
        if (kind == 0 && fixed_parity)
        {
            std::bernoulli_distribution coin(0.5);
            sector = coin(rng) ? 1 : 0;
            std::uint64_t x = 0;
            int par = 0;
            for (int q = 0; q < n - 1; ++q)
                if (coin(rng))
                {
                    x |= 1ull << q;
                    par ^= 1;
                }
            if (par != sector) x |= 1ull << (n - 1);
            a[x] = 1.0;
        }
        else if (kind == 0)
        {
            std::uniform_real_distribution<double> u01(0.0, 1.0);
            a[0] = 1.0;
            for (int q = 0; q < n; ++q)
            {
                const double cos_theta = std::clamp(1.0 - 2.0 * u01(rng), -1.0, 1.0);
                const double half = 0.5 * std::acos(cos_theta);
                const double phi = 2.0 * 3.14159265358979323846 * u01(rng);
                const cd c0(std::cos(half), 0.0);
                const cd c1 = std::polar(std::sin(half), phi);
                const std::uint64_t m = 1ull << q;
                for (std::uint64_t x = 0; x < m; ++x)
                {
                    const cd v = a[x];
                    a[x] = store(v * c0);
                    a[x + m] = store(v * c1);
                }
            }
        }
        else
        {
            std::normal_distribution<double> gauss(0.0, 1.0);
            if (fixed_parity)
            {
                std::bernoulli_distribution coin(0.5);
                sector = coin(rng) ? 1 : 0;
            }
            long double nn = 0.0L;
            for (std::uint64_t x = 0; x < dim; ++x)
            {
                if (fixed_parity && (__builtin_popcountll(x) & 1) != sector) continue;
                // cd(normal, normal) in the reference: imaginary argument drawn first.
                const double im = gauss(rng);
                const double re = gauss(rng);
                a[x] = store(cd(re, im));
                nn += static_cast<long double>(re * re + im * im);
            }
            const double inv = 1.0 / std::sqrt(static_cast<double>(nn));
            const double scale = fp32 ? static_cast<double>(static_cast<float>(inv)) : inv;
            for (auto &v : a) v = store(v * scale);
        }
        for (std::uint64_t x = 0; x < dim; ++x)
        {
            out_ri[2 * x] = a[x].real();
            out_ri[2 * x + 1] = a[x].imag();
        }
        if (parity) *parity = sector;
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// Workspace-seeded Haar draw (32-bit seed): gates and measured sites of
// `layers` layers, plus the measurement uniforms (one per chunk). Layout as
// orc_haar_draw.
int orc_fe_draw(std::uint32_t seed, int n, int layers, double p, int chunk_bits, int *gates_per_layer, int *gate_q,
                double *gate_m, int *sites_per_layer, int *sites, double *uniforms, int *n_uniforms)
{
    try
    {
        std::mt19937 gates(seed), meas(seed ^ 0x9e3779b9u);
        std::uniform_real_distribution<double> unif(0.0, 1.0);
        const int mg = n / 2;
        int u = 0;
        for (int t = 0; t < layers; ++t)
        {
            Layer L;
            draw_layer(L, n, t & 1, p, true, gates);
            gates_per_layer[t] = static_cast<int>(L.q.size() / 2);
            for (std::size_t g = 0; g < L.q.size() / 2; ++g)
            {
                gate_q[(static_cast<std::size_t>(t) * mg + g) * 2] = L.q[2 * g];
                gate_q[(static_cast<std::size_t>(t) * mg + g) * 2 + 1] = L.q[2 * g + 1];
                for (int e = 0; e < 16; ++e)
                {
                    gate_m[(static_cast<std::size_t>(t) * mg + g) * 32 + 2 * e] = L.m[16 * g + e].real();
                    gate_m[(static_cast<std::size_t>(t) * mg + g) * 32 + 2 * e + 1] = L.m[16 * g + e].imag();
                }
            }
            sites_per_layer[t] = static_cast<int>(L.sites.size());
            for (std::size_t k = 0; k < L.sites.size(); ++k) sites[static_cast<std::size_t>(t) * n + k] = L.sites[k];
            for (std::size_t k = 0; k < L.sites.size(); k += chunk_bits) uniforms[u++] = unif(meas);
        }
        *n_uniforms = u;
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// One free-energy trajectory of the Haar brickwork on the closed ring:
// 28n timesteps (4n equilibration + 24n production), each one layer and its
// joint measurement. surprisal[T], measured[T] (site counts), s_half[T+1]
// (half-chain S1 in bits on the sampled timesteps, NaN elsewhere).
int orc_fe_trajectory_circuit(std::uint64_t trajectory_seed, int n, double p, int circuit, int init_kind,
                              int fp32_init, int chunk_bits, int entropy_max_t, int entropy_stride, double *surprisal,
                              int *measured, double *s_half, int *parity);

int orc_fe_trajectory(std::uint64_t trajectory_seed, int n, double p, int init_kind, int fp32_init,
                      int chunk_bits, int entropy_max_t, int entropy_stride, double *surprisal, int *measured,
                      double *s_half, int *parity)
{
    return orc_fe_trajectory_circuit(trajectory_seed, n, p, 1, init_kind, fp32_init, chunk_bits, entropy_max_t,
                                     entropy_stride, surprisal, measured, s_half, parity);
}

int orc_fe_haar_trajectory(std::uint64_t trajectory_seed, int n, double p, int init_kind, int fp32_init,
                           int chunk_bits, int entropy_max_t, int entropy_stride, double *surprisal, int *measured,
                           double *s_half, int *parity)
{
    try
    {
        const int T = 28 * n;
        const std::uint32_t ws = static_cast<std::uint32_t>(mix64(trajectory_seed ^ 0x4349524355495455ull));
        const std::uint64_t init_seed = mix64(trajectory_seed ^ 0x494e495449414c53ull);
        const std::uint64_t dim = 1ull << n;
        std::vector<double> ri(2 * dim);
        if (orc_fe_initial_state(init_seed, n, init_kind, 0, fp32_init, ri.data(), parity)) return 1;
        std::vector<cd> psi(dim);
        for (std::uint64_t x = 0; x < dim; ++x) psi[x] = cd(ri[2 * x], ri[2 * x + 1]);
        std::mt19937 gates(ws), meas(ws ^ 0x9e3779b9u);
        std::uniform_real_distribution<double> unif(0.0, 1.0);
        auto sampled = [&](int t) {
            if (entropy_max_t < 0) return false;
            if (t == 0) return true;
            if (t > entropy_max_t) return false;
            return t % entropy_stride == 0 || t == entropy_max_t;
        };
        // The workspace draws every layer before the first one runs; the
        // layer stream is separate from the measurement stream, so drawing
        // layer by layer consumes both in the same order.
        std::vector<Layer> layers(T);
        for (int t = 0; t < T; ++t) draw_layer(layers[t], n, t & 1, p, true, gates);
        for (int t = 0; t <= T; ++t) s_half[t] = std::nan("");
        if (sampled(0)) s_half[0] = subsystem_entropy(psi.data(), n, half_chain(n), 1);
        for (int t = 0; t < T; ++t)
        {
            const Layer &L = layers[t];
            for (std::size_t g = 0; g < L.q.size() / 2; ++g)
                apply_bond(psi.data(), n, L.q[2 * g], L.q[2 * g + 1], &L.m[16 * g]);
            std::vector<double> us;
            for (std::size_t k = 0; k < L.sites.size(); k += chunk_bits) us.push_back(unif(meas));
            std::vector<int> oc(L.sites.size(), 0);
            int used = 0;
            surprisal[t] = measure_layer(psi.data(), n, L.sites, chunk_bits, us.data(), used, nullptr, oc.data());
            measured[t] = static_cast<int>(L.sites.size());
            if (sampled(t + 1)) s_half[t + 1] = subsystem_entropy(psi.data(), n, half_chain(n), 1);
        }
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// Free-energy trajectories master/first..first+count-1 on host threads:
// F_total (sum of all layer surprisals) per trajectory, no entropies. The
// timed CPU baseline of the free-energy workload.
int orc_fe_batch(std::uint64_t master, int first, int count, int n, double p, int init_kind, int chunk_bits,
                 double *f_total, int threads)
{
    int failed = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : failed)
#endif
    for (int i = 0; i < count; ++i)
    {
        const std::uint64_t ts = mix64(master ^ static_cast<std::uint64_t>(first + i));
        const int T = 28 * n;
        std::vector<double> sp(T), sh(T + 1);
        std::vector<int> mc(T);
        int parity = -1;
        if (orc_fe_trajectory(ts, n, p, init_kind, 0, chunk_bits, -1, 1, sp.data(), mc.data(), sh.data(), &parity))
            failed |= 1;
        double tot = 0.0;
        for (double v : sp) tot += v;
        f_total[i] = tot;
    }
    return failed;
}

namespace rp
{
// One op of an RPPU layer in application order: kind 0 matrix on (q0, q1)
// (bit 0 = q0), 1 FSWAP, 2 JW string (sign where bit q1 is set and the
// sites strictly between q0 and q1 hold odd parity).
struct Op
{
    int kind, q0, q1;
    std::array<cd, 16> m;
};

void u2(std::mt19937 &rng, cd *q)
{
    std::normal_distribution<double> normal(0.0, 1.0);
    cd z[4];
    for (int i = 0; i < 4; ++i)
    {
        // cd(normal(rng), normal(rng)) in the reference: imaginary draw first.
        const double im = normal(rng);
        const double re = normal(rng);
        z[i] = cd(re, im);
    }
    cd a = z[0], c = z[2];
    double na = std::sqrt(std::norm(a) + std::norm(c));
    if (na == 0.0)
    {
        a = 1.0;
        c = 0.0;
        na = 1.0;
    }
    const cd q00 = a / na, q10 = c / na;
    const cd r = std::conj(q00) * z[1] + std::conj(q10) * z[3];
    cd b0 = z[1] - q00 * r, b1 = z[3] - q10 * r;
    double nb = std::sqrt(std::norm(b0) + std::norm(b1));
    if (nb < 1e-15)
    {
        b0 = -std::conj(q10);
        b1 = std::conj(q00);
        nb = std::sqrt(std::norm(b0) + std::norm(b1));
    }
    q[0] = q00;
    q[1] = b0 / nb;
    q[2] = q10;
    q[3] = b1 / nb;
}

Op gate(std::mt19937 &rng, int q0, int q1)
{
    cd e[4], o[4];
    u2(rng, e);
    u2(rng, o);
    Op g{0, q0, q1, {}};
    // Even block on basis (0, 3), odd block on basis (2, 1).
    g.m[0] = e[0];
    g.m[3] = e[1];
    g.m[12] = e[2];
    g.m[15] = e[3];
    g.m[10] = o[0];
    g.m[9] = o[1];
    g.m[6] = o[2];
    g.m[5] = o[3];
    return g;
}

Op fswap(int q0, int q1)
{
    Op g{1, q0, q1, {}};
    g.m[0] = 1.0;
    g.m[6] = 1.0;
    g.m[9] = 1.0;
    g.m[15] = -1.0;
    return g;
}

struct Layer
{
    std::vector<Op> ops;
    std::vector<int> sites;
};

// boundary: 0 FSWAP chain, 1 JW string, 2 direct qubit gate.
void draw_layer(Layer &L, int n, bool odd, double p, int boundary, std::mt19937 &rng)
{
    std::bernoulli_distribution flag(p);
    L.ops.clear();
    L.sites.clear();
    if (!odd)
        for (int q = 0; q < n; q += 2) L.ops.push_back(gate(rng, q, q + 1));
    else
    {
        if (boundary == 1)
        {
            Op s{2, 0, n - 1, {}};
            L.ops.push_back(s);
            L.ops.push_back(gate(rng, 0, n - 1));
            L.ops.push_back(s);
        }
        else if (boundary == 2)
            L.ops.push_back(gate(rng, 0, n - 1));
        else
        {
            for (int k = n - 2; k > 0; --k) L.ops.push_back(fswap(k, k + 1));
            L.ops.push_back(gate(rng, 0, 1));
            for (int k = 1; k < n - 1; ++k) L.ops.push_back(fswap(k, k + 1));
        }
        for (int q = 1; q < n - 1; q += 2) L.ops.push_back(gate(rng, q, q + 1));
    }
    if (p >= 1.0)
        for (int s = 0; s < n; ++s) L.sites.push_back(s);
    else if (p > 0.0)
        for (int s = 0; s < n; ++s)
            if (flag(rng)) L.sites.push_back(s);
}

void apply(cd *psi, int n, const Op &op)
{
    if (op.kind == 2)
    {
        std::uint64_t mid = 0;
        for (int k = std::min(op.q0, op.q1) + 1; k < std::max(op.q0, op.q1); ++k) mid |= 1ull << k;
        const std::uint64_t ctl = 1ull << std::max(op.q0, op.q1);
        for (std::uint64_t x = 0; x < (1ull << n); ++x)
            if ((x & ctl) && (__builtin_popcountll(x & mid) & 1)) psi[x] = -psi[x];
        return;
    }
    apply_bond(psi, n, op.q0, op.q1, op.m.data());
}
} // namespace rp

// RPPU draw in the reference's op order: for each layer, ops[] (kind, q0,
// q1, 4x4 re/im) and measured sites. Circuit1D streams (workspace = 0: the
// random extra even layer drawn first) or the probed workspace's (workspace
// = 1, seed's low 32 bits, `periods` meaning the layer count). Returns the
// layer count; op_count[layer], ops flattened as [kind, q0, q1] in op_meta
// and 32 doubles each in op_m; sites_per_layer/sites as orc_haar_draw.
int orc_rppu_draw(std::uint64_t seed, int n, int periods, double p, int boundary, int workspace, int *op_count,
                  int *op_meta, double *op_m, int *sites_per_layer, int *sites)
{
    try
    {
        std::mt19937 gates, meas;
        int T;
        bool extra = false;
        if (workspace)
        {
            gates.seed(static_cast<std::uint32_t>(seed));
            T = periods;
        }
        else
        {
            seed_pair(seed, gates, meas);
            std::bernoulli_distribution coin(0.5);
            extra = coin(gates);
            T = 2 * periods + (extra ? 1 : 0);
        }
        int k = 0;
        for (int t = 0; t < T; ++t)
        {
            rp::Layer L;
            const bool odd = workspace ? (t % 2) != 0 : (t < 2 * periods && (t & 1));
            rp::draw_layer(L, n, odd, p, boundary, gates);
            op_count[t] = static_cast<int>(L.ops.size());
            for (const auto &op : L.ops)
            {
                op_meta[3 * k] = op.kind;
                op_meta[3 * k + 1] = op.q0;
                op_meta[3 * k + 2] = op.q1;
                for (int e = 0; e < 16; ++e)
                {
                    op_m[32 * k + 2 * e] = op.m[e].real();
                    op_m[32 * k + 2 * e + 1] = op.m[e].imag();
                }
                ++k;
            }
            sites_per_layer[t] = static_cast<int>(L.sites.size());
            for (std::size_t j = 0; j < L.sites.size(); ++j) sites[static_cast<std::size_t>(t) * n + j] = L.sites[j];
        }
        return T;
    }
    catch (...)
    {
        return -1;
    }
}

// One RPPU / qRPPU trajectory on the Circuit1D streams from |0...0>:
// surprisal[layer] (-ln P), outcomes as orc_run_haar_trajectory's (in the
// order measured: with `encoded`, site n-1 last), the final state, and the
// layer count (2*periods or 2*periods + 1) returned.
int orc_run_rppu_trajectory(std::uint64_t seed, int n, int periods, double p, int boundary, int encoded,
                            int chunk_bits, double *surprisal, int *outcomes, double *final_psi_ri)
{
    try
    {
        std::mt19937 gates, meas;
        seed_pair(seed, gates, meas);
        std::bernoulli_distribution coin(0.5);
        const bool extra = coin(gates);
        const int T = 2 * periods + (extra ? 1 : 0);
        const std::uint64_t dim = 1ull << n;
        std::vector<cd> psi(dim, cd(0.0, 0.0));
        psi[0] = 1.0;
        std::uniform_real_distribution<double> unif(0.0, 1.0);
        for (int t = 0; t < T; ++t)
        {
            rp::Layer L;
            rp::draw_layer(L, n, t < 2 * periods && (t & 1), p, boundary, gates);
            for (const auto &op : L.ops) rp::apply(psi.data(), n, op);
            // Encoded measurement: sites below n-1 in chunks, then n-1 alone.
            std::vector<int> plain, last;
            for (int s : L.sites) (encoded && s == n - 1 ? last : plain).push_back(s);
            std::vector<double> us;
            for (std::size_t j = 0; j < plain.size(); j += chunk_bits) us.push_back(unif(meas));
            if (!last.empty()) us.push_back(unif(meas));
            std::vector<int> oc(L.sites.size(), 0);
            int used = 0;
            double sp = measure_layer(psi.data(), n, plain, chunk_bits, us.data(), used, nullptr, oc.data());
            if (!last.empty()) sp += measure_layer(psi.data(), n, last, 1, us.data(), used, nullptr, oc.data() + plain.size());
            surprisal[t] = sp;
            if (outcomes)
            {
                for (int s = 0; s < n; ++s) outcomes[static_cast<std::size_t>(t) * n + s] = -1;
                for (std::size_t s = 0; s < oc.size(); ++s) outcomes[static_cast<std::size_t>(t) * n + s] = oc[s];
            }
        }
        if (final_psi_ri) std::memcpy(final_psi_ri, psi.data(), dim * sizeof(cd));
        return T;
    }
    catch (...)
    {
        return -1;
    }
}

// The free-energy trajectory for any gate set on this path: circuit 1 Haar
// (orc_fe_haar_trajectory), 2 FermionRPPU (JW closure, fermionic S1), 4
// qRPPU; the parity-preserving sets start from a fixed-parity initial state
// (cpp/include/mipt/free_energy.hpp:224-248) and draw their layers with
// fill_rppu_layer on the workspace stream (cpp/include/mipt/probed.hpp:208-224).
int orc_fe_trajectory_circuit(std::uint64_t trajectory_seed, int n, double p, int circuit, int init_kind,
                              int fp32_init, int chunk_bits, int entropy_max_t, int entropy_stride, double *surprisal,
                              int *measured, double *s_half, int *parity)
{
    if (circuit == 1 || circuit == 0)
        return orc_fe_haar_trajectory(trajectory_seed, n, p, init_kind, fp32_init, chunk_bits, entropy_max_t,
                                      entropy_stride, surprisal, measured, s_half, parity);
    try
    {
        const int T = 28 * n;
        const bool fermion = circuit == 2;
        const std::uint32_t ws = static_cast<std::uint32_t>(mix64(trajectory_seed ^ 0x4349524355495455ull));
        const std::uint64_t init_seed = mix64(trajectory_seed ^ 0x494e495449414c53ull);
        const std::uint64_t dim = 1ull << n;
        std::vector<double> ri(2 * dim);
        if (orc_fe_initial_state(init_seed, n, init_kind, 1, fp32_init, ri.data(), parity)) return 1;
        std::vector<cd> psi(dim);
        for (std::uint64_t x = 0; x < dim; ++x) psi[x] = cd(ri[2 * x], ri[2 * x + 1]);
        std::mt19937 gates(ws), meas(ws ^ 0x9e3779b9u);
        std::uniform_real_distribution<double> unif(0.0, 1.0);
        auto sampled = [&](int t) {
            if (entropy_max_t < 0) return false;
            if (t == 0) return true;
            if (t > entropy_max_t) return false;
            return t % entropy_stride == 0 || t == entropy_max_t;
        };
        std::vector<rp::Layer> layers(T);
        for (int t = 0; t < T; ++t) rp::draw_layer(layers[t], n, (t % 2) != 0, p, fermion ? 1 : 2, gates);
        for (int t = 0; t <= T; ++t) s_half[t] = std::nan("");
        if (sampled(0)) s_half[0] = subsystem_entropy(psi.data(), n, half_chain(n), 1, fermion);
        for (int t = 0; t < T; ++t)
        {
            const rp::Layer &L = layers[t];
            for (const auto &op : L.ops) rp::apply(psi.data(), n, op);
            std::vector<double> us;
            for (std::size_t k = 0; k < L.sites.size(); k += chunk_bits) us.push_back(unif(meas));
            std::vector<int> oc(L.sites.size(), 0);
            int used = 0;
            surprisal[t] = measure_layer(psi.data(), n, L.sites, chunk_bits, us.data(), used, nullptr, oc.data());
            measured[t] = static_cast<int>(L.sites.size());
            if (sampled(t + 1)) s_half[t + 1] = subsystem_entropy(psi.data(), n, half_chain(n), 1, fermion);
        }
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

int orc_max_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

} // extern "C"
