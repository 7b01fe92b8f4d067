#include "sampler.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <random>
#include <stdexcept>
#include <thread>

namespace mg
{

std::uint64_t splitmix64(std::uint64_t v)
{
    v += 0x9e3779b97f4a7c15ull;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ull;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebull;
    return v ^ (v >> 31);
}

std::uint64_t trajectory_seed(std::uint64_t master, std::uint64_t index)
{
    return splitmix64(master + 0x2545f4914f6cdd1dull * (index + 1ull));
}

namespace
{
using C = std::complex<double>;

void seed_mt(std::mt19937 &rng, std::uint64_t v)
{
    std::seed_seq seq{static_cast<std::uint32_t>(v & 0xffffffffu), static_cast<std::uint32_t>(v >> 32)};
    rng.seed(seq);
}

// Gram-Schmidt of four complex Gaussian columns into a Haar unitary,
// row-major; writes into u[16]. Each column entry takes two normal draws,
// imaginary part first (the order the g++-built reference evaluates
// ComplexD(normal(rng), normal(rng)) in).
void gram_schmidt_u4(std::mt19937 &rng, std::normal_distribution<double> &gauss, C *u)
{
    int col = 0;
    while (col < 4)
    {
        C v[4];
        for (auto &x : v)
        {
            const double im = gauss(rng);
            const double re = gauss(rng);
            x = C(re, im);
        }
        for (int k = 0; k < col; ++k)
        {
            C proj(0.0, 0.0);
            for (int r = 0; r < 4; ++r) proj += std::conj(u[4 * r + k]) * v[r];
            for (int r = 0; r < 4; ++r) v[r] -= u[4 * r + k] * proj;
        }
        double norm2 = 0.0;
        for (const auto &x : v) norm2 += std::norm(x);
        const double len = std::sqrt(norm2);
        if (len < 1e-14) continue; // redraw this column
        for (int r = 0; r < 4; ++r) u[4 * r + col] = v[r] / len;
        ++col;
    }
}

// The reference splits each drawn unitary with a cosine-sine decomposition
// and redraws when a cosine or sine of the split falls below 1e-12. The
// cosines squared are the eigenvalues of X^H X for the top-left block X.
bool csd_is_singular(const C *u)
{
    const double a = std::norm(u[0]) + std::norm(u[4]);
    const double d = std::norm(u[1]) + std::norm(u[5]);
    const C b = std::conj(u[0]) * u[1] + std::conj(u[4]) * u[5];
    const double root = std::sqrt(std::max(0.0, (a - d) * (a - d) + 4.0 * std::norm(b)));
    const double hi = std::clamp(0.5 * (a + d + root), 0.0, 1.0);
    const double lo = std::clamp(0.5 * (a + d - root), 0.0, 1.0);
    const double tiny = 1e-12;
    return std::sqrt(hi) < tiny || std::sqrt(lo) < tiny || std::sqrt(std::max(0.0, 1.0 - hi)) < tiny ||
           std::sqrt(std::max(0.0, 1.0 - lo)) < tiny;
}

// Run `fn(i)` for i in [0, count) on up to `threads` host threads.
template <typename Fn> void parallel_for(int count, int threads, Fn fn, const char *what)
{
    if (threads <= 0) threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    threads = std::min(threads, std::max(1, count));
    std::atomic<int> next{0};
    std::atomic<bool> failed{false};
    auto work = [&]() {
        for (;;)
        {
            const int i = next.fetch_add(1);
            if (i >= count) return;
            try
            {
                fn(i);
            }
            catch (...)
            {
                failed = true;
            }
        }
    };
    if (threads == 1)
        work();
    else
    {
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; ++t) pool.emplace_back(work);
        for (auto &th : pool) th.join();
    }
    if (failed) throw std::runtime_error(what);
}

// The 1-D brickwork layer loop shared by both seedings: layer t's unitaries
// (bonds from t % 2), its Bernoulli(p) flags from the layer stream, then one
// measurement uniform per chunk from the measurement stream.
void draw_haar_layers(std::mt19937 &gates_rng, std::mt19937 &meas_rng, int n, int T, double p, bool closed,
                      int chunk_bits, TrajectoryDraw &out)
{
    if (n < 2 || n % 2 != 0 || n > 62) throw std::invalid_argument("Haar brickwork needs even 2 <= n <= 62");
    if (chunk_bits < 1) throw std::invalid_argument("chunk_bits must be positive");
    const int mb = n / 2;
    out.n = n;
    out.layers = T;
    out.max_bonds = mb;
    out.bond_count.assign(T, 0);
    out.bond_q.assign(static_cast<std::size_t>(T) * mb * 2, 0);
    out.bond_u.assign(static_cast<std::size_t>(T) * mb * 16, C(0.0, 0.0));
    out.measured.assign(T, 0);
    out.uniforms.clear();
    out.uniform_offset.assign(T + 1, 0);

    std::uniform_real_distribution<double> unif(0.0, 1.0);
    for (int t = 0; t < T; ++t)
    {
        const int start = t & 1;
        const int stop = (closed && start == 1 && n > 2) ? n : n - 1;
        int j = 0;
        for (int i = start; i < stop; i += 2, ++j)
        {
            C *u = &out.bond_u[(static_cast<std::size_t>(t) * mb + j) * 16];
            do
            {
                // A fresh distribution per draw, as the reference constructs one
                // inside haar_unitary_4 (its cached second normal is dropped).
                std::normal_distribution<double> gauss(0.0, 1.0);
                gram_schmidt_u4(gates_rng, gauss, u);
            } while (csd_is_singular(u));
            out.bond_q[(static_cast<std::size_t>(t) * mb + j) * 2] = i;
            out.bond_q[(static_cast<std::size_t>(t) * mb + j) * 2 + 1] = (i + 1) % n;
        }
        out.bond_count[t] = j;
        std::uint64_t mask = 0;
        if (p >= 1.0)
        {
            mask = (n == 64) ? ~0ull : ((1ull << n) - 1ull);
        }
        else if (p > 0.0)
        {
            std::bernoulli_distribution flag(p);
            for (int s = 0; s < n; ++s)
                if (flag(gates_rng)) mask |= 1ull << s;
        }
        out.measured[t] = mask;
        out.uniform_offset[t] = static_cast<int>(out.uniforms.size());
        const int m = __builtin_popcountll(mask);
        for (int c = 0; c < m; c += chunk_bits) out.uniforms.push_back(unif(meas_rng));
    }
    out.uniform_offset[T] = static_cast<int>(out.uniforms.size());
}
} // namespace

void draw_haar_trajectory(std::uint64_t seed, int n, int periods, double p, bool closed, int chunk_bits,
                          TrajectoryDraw &out)
{
    std::mt19937 gates_rng, meas_rng;
    seed_mt(gates_rng, seed);
    seed_mt(meas_rng, splitmix64(seed ^ 0xa0761d0dull));
    draw_haar_layers(gates_rng, meas_rng, n, 2 * periods, p, closed, chunk_bits, out);
}

void draw_haar_trajectory_workspace(std::uint32_t seed, int n, int layers, double p, bool closed, int chunk_bits,
                                    TrajectoryDraw &out)
{
    std::mt19937 gates_rng(seed), meas_rng(seed ^ 0x9e3779b9u);
    draw_haar_layers(gates_rng, meas_rng, n, layers, p, closed, chunk_bits, out);
}

void draw_haar_workspace_batch(const std::uint32_t *seeds, const double *p, int count, int n, int layers,
                               bool closed, int chunk_bits, std::vector<TrajectoryDraw> &out, int threads)
{
    out.resize(count);
    parallel_for(
        count, threads,
        [&](int i) { draw_haar_trajectory_workspace(seeds[i], n, layers, p[i], closed, chunk_bits, out[i]); },
        "workspace trajectory draw failed");
}

template <typename Real>
int draw_initial_state(std::uint64_t seed, int n, int kind, bool fixed_parity, std::complex<Real> *out)
{
    if (n < 1 || n > 40) throw std::invalid_argument("initial state needs 1 <= n <= 40");
    if (kind != 0 && kind != 1) throw std::invalid_argument("initial state kind must be 0 or 1");
    const std::size_t dim = std::size_t{1} << n;
    std::fill(out, out + dim, std::complex<Real>(0, 0));
    std::mt19937_64 rng(seed);
    if (kind == 0 && fixed_parity)
    {
        // A basis product state: n-1 fair bits, the last one fixing the parity.
        std::bernoulli_distribution bit(0.5);
        const int sector = bit(rng) ? 1 : 0;
        std::uint64_t basis = 0;
        int parity = 0;
        for (int q = 0; q + 1 < n; ++q)
        {
            const int v = bit(rng) ? 1 : 0;
            parity ^= v;
            basis |= static_cast<std::uint64_t>(v) << q;
        }
        basis |= static_cast<std::uint64_t>(parity ^ sector) << (n - 1);
        out[basis] = std::complex<Real>(1, 0);
        return sector;
    }
    if (kind == 0)
    {
        // Site q's Bloch vector uniform on the sphere (z = cos theta uniform,
        // phi uniform); the amplitude table doubles per site, each product
        // rounded to Real as it is stored.
        std::uniform_real_distribution<double> unit(0.0, 1.0);
        constexpr double two_pi = 6.283185307179586476925286766559;
        out[0] = std::complex<Real>(1, 0);
        std::size_t active = 1;
        for (int q = 0; q < n; ++q)
        {
            const double z = 1.0 - 2.0 * unit(rng);
            const double theta = std::acos(std::clamp(z, -1.0, 1.0));
            const double phi = two_pi * unit(rng);
            const std::complex<double> up(std::cos(0.5 * theta), 0.0);
            const std::complex<double> down = std::polar(std::sin(0.5 * theta), phi);
            for (std::size_t i = 0; i < active; ++i)
            {
                const std::complex<double> prior(out[i]);
                out[i] = static_cast<std::complex<Real>>(prior * up);
                out[i | active] = static_cast<std::complex<Real>>(prior * down);
            }
            active <<= 1;
        }
        return -1;
    }
    // Gaussian amplitudes: two normal draws per kept index (real part first,
    // as the reference's g++ build evaluates its constructor arguments
    // right to left -- the imaginary draw is taken first), norm accumulated in
    // long double, one rounded scale applied in Real.
    std::normal_distribution<double> normal(0.0, 1.0);
    std::bernoulli_distribution coin(0.5);
    const int sector = fixed_parity ? (coin(rng) ? 1 : 0) : -1;
    long double norm2 = 0.0L;
    for (std::size_t i = 0; i < dim; ++i)
    {
        if (fixed_parity && (__builtin_popcountll(static_cast<unsigned long long>(i)) & 1) != sector) continue;
        const double im = normal(rng);
        const double re = normal(rng);
        const std::complex<double> v(re, im);
        out[i] = static_cast<std::complex<Real>>(v);
        norm2 += static_cast<long double>(std::norm(v));
    }
    if (!(norm2 > 0.0L)) throw std::runtime_error("random Haar state normalisation vanished");
    const Real scale = static_cast<Real>(1.0 / std::sqrt(static_cast<double>(norm2)));
    for (std::size_t i = 0; i < dim; ++i) out[i] *= scale;
    return sector;
}
template int draw_initial_state<float>(std::uint64_t, int, int, bool, std::complex<float> *);
template int draw_initial_state<double>(std::uint64_t, int, int, bool, std::complex<double> *);

namespace
{
// haar_unitary_2: Gram-Schmidt of a complex Gaussian 2x2 (row-major), each
// entry's imaginary draw first as the g++-built reference evaluates
// std::complex<double>(normal(rng), normal(rng)).
void haar_u2(std::mt19937 &rng, C *q)
{
    std::normal_distribution<double> normal(0.0, 1.0);
    C z[4];
    for (auto &v : z)
    {
        const double im = normal(rng);
        const double re = normal(rng);
        v = C(re, im);
    }
    C z00 = z[0], z10 = z[2];
    const C z01 = z[1], z11 = z[3];
    double n0 = std::sqrt(std::norm(z00) + std::norm(z10));
    if (n0 == 0.0)
    {
        z00 = 1.0;
        z10 = 0.0;
        n0 = 1.0;
    }
    const C q00 = z00 / n0, q10 = z10 / n0;
    const C r01 = std::conj(q00) * z01 + std::conj(q10) * z11;
    C u01 = z01 - q00 * r01, u11 = z11 - q10 * r01;
    double n1 = std::sqrt(std::norm(u01) + std::norm(u11));
    if (n1 < 1e-15)
    {
        u01 = -std::conj(q10);
        u11 = std::conj(q00);
        n1 = std::sqrt(std::norm(u01) + std::norm(u11));
    }
    q[0] = q00;
    q[1] = u01 / n1;
    q[2] = q10;
    q[3] = u11 / n1;
}

// One parity-preserving bond (even block drawn first), as a row-major 4x4
// with bit 0 = the gate's first qubit; `swapped` stores it for the reversed
// qubit order.
void parity_gate(std::mt19937 &rng, C *m, bool swapped)
{
    C e[4], o[4], g[16] = {};
    haar_u2(rng, e);
    haar_u2(rng, o);
    g[0] = e[0];
    g[3] = e[1];
    g[12] = e[2];
    g[15] = e[3];
    g[10] = o[0];
    g[9] = o[1];
    g[6] = o[2];
    g[5] = o[3];
    auto sw = [swapped](int i) { return swapped ? ((i & 1) << 1) | ((i >> 1) & 1) : i; };
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) m[4 * sw(r) + sw(c)] = g[4 * r + c];
}

// Layer t of `out` (odd or even) from the layer stream, then its flags and
// measurement uniforms.
void rppu_layer(std::mt19937 &gates_rng, std::mt19937 &meas_rng, int n, bool odd, double p, int chunk_bits,
                bool split_last, int t, TrajectoryDraw &out)
{
    const int mb = n / 2;
    C *u = &out.bond_u[static_cast<std::size_t>(t) * mb * 16];
    int *q = &out.bond_q[static_cast<std::size_t>(t) * mb * 2];
    std::bernoulli_distribution flag(p);
    if (!odd)
    {
        for (int j = 0; j < mb; ++j)
        {
            parity_gate(gates_rng, u + 16 * j, false);
            q[2 * j] = 2 * j;
            q[2 * j + 1] = 2 * j + 1;
        }
    }
    else
    {
        // Closure first in the draw, last in the plan's bond order.
        parity_gate(gates_rng, u + 16 * (mb - 1), true);
        q[2 * (mb - 1)] = n - 1;
        q[2 * (mb - 1) + 1] = 0;
        for (int j = 0; j + 1 < mb; ++j)
        {
            parity_gate(gates_rng, u + 16 * j, false);
            q[2 * j] = 2 * j + 1;
            q[2 * j + 1] = 2 * j + 2;
        }
    }
    out.bond_count[t] = mb;
    std::uint64_t mask = 0;
    if (p >= 1.0)
        mask = (1ull << n) - 1ull;
    else if (p > 0.0)
        for (int s = 0; s < n; ++s)
            if (flag(gates_rng)) mask |= 1ull << s;
    out.measured[t] = mask;
    out.uniform_offset[t] = static_cast<int>(out.uniforms.size());
    std::uniform_real_distribution<double> unif(0.0, 1.0);
    const bool last_alone = split_last && ((mask >> (n - 1)) & 1ull);
    const int plain = __builtin_popcountll(mask) - (last_alone ? 1 : 0);
    for (int c = 0; c < plain; c += chunk_bits) out.uniforms.push_back(unif(meas_rng));
    if (last_alone) out.uniforms.push_back(unif(meas_rng));
}

void rppu_init(TrajectoryDraw &out, int n, int layers_out, bool split_last)
{
    if (n < 4 || n % 2 != 0 || n > 62) throw std::invalid_argument("RPPU brickwork needs even 4 <= n <= 62");
    const int mb = n / 2;
    out.n = n;
    out.layers = layers_out;
    out.max_bonds = mb;
    out.split_last = split_last;
    out.bond_count.assign(layers_out, 0);
    out.bond_q.assign(static_cast<std::size_t>(layers_out) * mb * 2, 0);
    out.bond_u.assign(static_cast<std::size_t>(layers_out) * mb * 16, C(0.0, 0.0));
    out.measured.assign(layers_out, 0);
    out.uniforms.clear();
    out.uniform_offset.assign(layers_out + 1, 0);
}

// Identity even layer (no gates drawn, nothing measured) in slot t.
void identity_layer(TrajectoryDraw &out, int t)
{
    const int mb = out.max_bonds;
    for (int j = 0; j < mb; ++j)
    {
        C *u = &out.bond_u[(static_cast<std::size_t>(t) * mb + j) * 16];
        for (int e = 0; e < 16; ++e) u[e] = (e % 5 == 0) ? C(1.0, 0.0) : C(0.0, 0.0);
        out.bond_q[(static_cast<std::size_t>(t) * mb + j) * 2] = 2 * j;
        out.bond_q[(static_cast<std::size_t>(t) * mb + j) * 2 + 1] = 2 * j + 1;
    }
    out.bond_count[t] = mb;
    out.measured[t] = 0;
    out.uniform_offset[t] = static_cast<int>(out.uniforms.size());
}
} // namespace

void draw_rppu_trajectory(std::uint64_t seed, int n, int periods, double p, int chunk_bits, bool split_last,
                          int layers_out, TrajectoryDraw &out)
{
    if (layers_out < 2 * periods + 1) throw std::invalid_argument("RPPU draw needs 2*periods + 1 layer slots");
    if (chunk_bits < 1) throw std::invalid_argument("chunk_bits must be positive");
    std::mt19937 gates_rng, meas_rng;
    seed_mt(gates_rng, seed);
    seed_mt(meas_rng, splitmix64(seed ^ 0xa0761d0dull));
    rppu_init(out, n, layers_out, split_last);
    std::bernoulli_distribution extra_even(0.5);
    const bool extra = extra_even(gates_rng);
    int t = 0;
    for (; t < 2 * periods; ++t) rppu_layer(gates_rng, meas_rng, n, (t & 1) != 0, p, chunk_bits, split_last, t, out);
    if (extra) rppu_layer(gates_rng, meas_rng, n, false, p, chunk_bits, split_last, t++, out);
    for (; t < layers_out; ++t) identity_layer(out, t);
    out.uniform_offset[layers_out] = static_cast<int>(out.uniforms.size());
}

void draw_rppu_workspace(std::uint32_t seed, int n, int layers, double p, int chunk_bits, bool split_last,
                         int layers_out, TrajectoryDraw &out)
{
    if (layers_out < layers) throw std::invalid_argument("too few layer slots");
    if (chunk_bits < 1) throw std::invalid_argument("chunk_bits must be positive");
    std::mt19937 gates_rng(seed), meas_rng(seed ^ 0x9e3779b9u);
    rppu_init(out, n, layers_out, split_last);
    int t = 0;
    for (; t < layers; ++t) rppu_layer(gates_rng, meas_rng, n, (t & 1) != 0, p, chunk_bits, split_last, t, out);
    for (; t < layers_out; ++t) identity_layer(out, t);
    out.uniform_offset[layers_out] = static_cast<int>(out.uniforms.size());
}

void draw_rppu_batch(const std::uint64_t *seeds, const double *p, int count, int n, int periods, int chunk_bits,
                     bool split_last, int layers_out, std::vector<TrajectoryDraw> &out, int threads)
{
    out.resize(count);
    parallel_for(
        count, threads,
        [&](int i) { draw_rppu_trajectory(seeds[i], n, periods, p[i], chunk_bits, split_last, layers_out, out[i]); },
        "RPPU trajectory draw failed");
}

void draw_rppu_workspace_batch(const std::uint32_t *seeds, const double *p, int count, int n, int layers,
                               int chunk_bits, bool split_last, int layers_out, std::vector<TrajectoryDraw> &out,
                               int threads)
{
    out.resize(count);
    parallel_for(
        count, threads,
        [&](int i) { draw_rppu_workspace(seeds[i], n, layers, p[i], chunk_bits, split_last, layers_out, out[i]); },
        "RPPU workspace draw failed");
}

std::vector<std::pair<int, int>> lattice_bonds(int X, int Y, int colour)
{
    if (X < 2 || Y < 1 || colour < 0 || colour > 3) throw std::invalid_argument("bad lattice or colour");
    std::vector<std::pair<int, int>> out;
    // One line of `len` sites (site i at base + i*step): pairs from 0 when the
    // line's parity matches the colour, else the wrap bond (even lengths) and
    // pairs from 1.
    auto line = [&](int base, int step, int len, bool from_zero) {
        if (len < 2) return;
        if (from_zero)
        {
            for (int i = 0; i + 1 < len; i += 2) out.emplace_back(base + i * step, base + (i + 1) * step);
            return;
        }
        if (len % 2 == 0) out.emplace_back(base, base + (len - 1) * step);
        for (int i = 1; i + 1 < len; i += 2) out.emplace_back(base + i * step, base + (i + 1) * step);
    };
    if (colour < 2)
        for (int r = 0; r < Y; ++r) line(r * X, 1, X, (r % 2) == colour);
    else
        for (int c = 0; c < X; ++c) line(c, X, Y, (c % 2) == colour - 2);
    return out;
}

void draw_haar_lattice_trajectory(std::uint64_t seed, int X, int Y, int layers, double p, int chunk_bits,
                                  TrajectoryDraw &out)
{
    const int n = X * Y;
    if (X < 2 || Y < 2 || n > 62) throw std::invalid_argument("lattice needs X, Y >= 2 and X*Y <= 62");
    if (chunk_bits < 1) throw std::invalid_argument("chunk_bits must be positive");
    std::mt19937 gates_rng, meas_rng;
    seed_mt(gates_rng, seed);
    seed_mt(meas_rng, splitmix64(seed ^ 0xa0761d0dull));
    std::vector<std::pair<int, int>> colours[4];
    for (int c = 0; c < 4; ++c) colours[c] = lattice_bonds(X, Y, c);
    const int mb = n / 2;
    out.n = n;
    out.layers = layers;
    out.max_bonds = mb;
    out.bond_count.assign(layers, 0);
    out.bond_q.assign(static_cast<std::size_t>(layers) * mb * 2, 0);
    out.bond_u.assign(static_cast<std::size_t>(layers) * mb * 16, C(0.0, 0.0));
    out.measured.assign(layers, 0);
    out.uniforms.clear();
    out.uniform_offset.assign(layers + 1, 0);
    std::uniform_real_distribution<double> unif(0.0, 1.0);
    for (int t = 0; t < layers; ++t)
    {
        const auto &bonds = colours[t % 4];
        for (std::size_t j = 0; j < bonds.size(); ++j)
        {
            C *u = &out.bond_u[(static_cast<std::size_t>(t) * mb + j) * 16];
            do
            {
                std::normal_distribution<double> gauss(0.0, 1.0);
                gram_schmidt_u4(gates_rng, gauss, u);
            } while (csd_is_singular(u));
            out.bond_q[(static_cast<std::size_t>(t) * mb + j) * 2] = bonds[j].first;
            out.bond_q[(static_cast<std::size_t>(t) * mb + j) * 2 + 1] = bonds[j].second;
        }
        out.bond_count[t] = static_cast<int>(bonds.size());
        std::uint64_t mask = 0;
        if (p >= 1.0)
        {
            mask = (1ull << n) - 1ull;
        }
        else if (p > 0.0)
        {
            std::bernoulli_distribution flag(p);
            for (int s = 0; s < n; ++s)
                if (flag(gates_rng)) mask |= 1ull << s;
        }
        out.measured[t] = mask;
        out.uniform_offset[t] = static_cast<int>(out.uniforms.size());
        const int m = __builtin_popcountll(mask);
        for (int c = 0; c < m; c += chunk_bits) out.uniforms.push_back(unif(meas_rng));
    }
    out.uniform_offset[layers] = static_cast<int>(out.uniforms.size());
}

void draw_haar_lattice_batch(const std::uint64_t *seeds, const double *p, int count, int X, int Y, int layers,
                             int chunk_bits, std::vector<TrajectoryDraw> &out, int threads)
{
    out.resize(count);
    if (threads <= 0) threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    threads = std::min(threads, std::max(1, count));
    std::atomic<int> next{0};
    std::atomic<bool> failed{false};
    auto work = [&]() {
        for (;;)
        {
            const int i = next.fetch_add(1);
            if (i >= count) return;
            try
            {
                draw_haar_lattice_trajectory(seeds[i], X, Y, layers, p[i], chunk_bits, out[i]);
            }
            catch (...)
            {
                failed = true;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(work);
    for (auto &th : pool) th.join();
    if (failed) throw std::runtime_error("lattice trajectory draw failed");
}

void draw_haar_batch(const std::uint64_t *seeds, const double *p, int count, int n, int periods, bool closed,
                     int chunk_bits, std::vector<TrajectoryDraw> &out, int threads)
{
    out.resize(count);
    if (threads <= 0) threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    threads = std::min(threads, std::max(1, count));
    std::atomic<int> next{0};
    std::atomic<bool> failed{false};
    auto work = [&]() {
        for (;;)
        {
            const int i = next.fetch_add(1);
            if (i >= count) return;
            try
            {
                draw_haar_trajectory(seeds[i], n, periods, p[i], closed, chunk_bits, out[i]);
            }
            catch (...)
            {
                failed = true;
            }
        }
    };
    if (threads == 1)
    {
        work();
    }
    else
    {
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; ++t) pool.emplace_back(work);
        for (auto &th : pool) th.join();
    }
    if (failed) throw std::runtime_error("trajectory draw failed");
}

} // namespace mg

namespace mg
{
namespace
{
// Haar SO(4): Gram-Schmidt of a real Gaussian 4x4 (columns), then the first
// column negated when the determinant is negative.
void so4_draw(std::mt19937 &rng, double *O)
{
    std::normal_distribution<double> gauss(0.0, 1.0);
    double q[16];
    for (int c = 0; c < 4; ++c)
    {
        double v[4];
        for (double &x : v) x = gauss(rng);
        for (int k = 0; k < c; ++k)
        {
            double proj = 0.0;
            for (int r = 0; r < 4; ++r) proj += q[4 * r + k] * v[r];
            for (int r = 0; r < 4; ++r) v[r] -= q[4 * r + k] * proj;
        }
        double nn = 0.0;
        for (double x : v) nn += x * x;
        const double len = std::sqrt(nn);
        for (int r = 0; r < 4; ++r) q[4 * r + c] = v[r] / len;
    }
    auto m3 = [&](int c0, int c1, int c2) {
        // minor of rows 1..3 and columns c0, c1, c2
        return q[4 + c0] * (q[8 + c1] * q[12 + c2] - q[8 + c2] * q[12 + c1]) -
               q[4 + c1] * (q[8 + c0] * q[12 + c2] - q[8 + c2] * q[12 + c0]) +
               q[4 + c2] * (q[8 + c0] * q[12 + c1] - q[8 + c1] * q[12 + c0]);
    };
    const double det = q[0] * m3(1, 2, 3) - q[1] * m3(0, 2, 3) + q[2] * m3(0, 1, 3) - q[3] * m3(0, 1, 2);
    if (det < 0)
        for (int r = 0; r < 4; ++r) q[4 * r] = -q[4 * r];
    for (int i = 0; i < 16; ++i) O[i] = q[i];
}
} // namespace

void draw_fermion_trajectory(std::uint64_t seed, int n, int depth, double p, bool closed, FermionDraw &out)
{
    if (n < 2 || n > 128) throw std::invalid_argument("free-fermion chains need 2 <= N <= 128 modes");
    std::mt19937 g, meas;
    seed_mt(g, seed);
    seed_mt(meas, splitmix64(seed ^ 0xa0761d0dull));
    const int mg_ = n / 2 + 1;
    out.n = n;
    out.depth = depth;
    out.max_gates = mg_;
    out.gate_count.assign(depth, 0);
    out.gate_mode.assign(static_cast<std::size_t>(depth) * mg_, 0);
    out.rot.assign(static_cast<std::size_t>(depth) * mg_ * 16, 0.0);
    out.meas_count.assign(depth, 0);
    out.meas_mode.assign(static_cast<std::size_t>(depth) * n, 0);
    out.uniform.assign(static_cast<std::size_t>(depth) * n, 0.0);
    std::uniform_real_distribution<double> unif(0.0, 1.0);
    for (int t = 0; t < depth; ++t)
    {
        const int start = t & 1;
        const int stop = (closed && start == 1 && n > 2) ? n : n - 1;
        int gi = 0;
        for (int m = start; m < stop; m += 2, ++gi)
        {
            out.gate_mode[static_cast<std::size_t>(t) * mg_ + gi] = m;
            so4_draw(g, &out.rot[(static_cast<std::size_t>(t) * mg_ + gi) * 16]);
        }
        out.gate_count[t] = gi;
        int mc = 0;
        if (p >= 1.0)
        {
            for (int j = 0; j < n; ++j) out.meas_mode[static_cast<std::size_t>(t) * n + mc++] = j;
        }
        else if (p > 0.0)
        {
            std::bernoulli_distribution flag(p);
            for (int j = 0; j < n; ++j)
                if (flag(g)) out.meas_mode[static_cast<std::size_t>(t) * n + mc++] = j;
        }
        out.meas_count[t] = mc;
        for (int i = 0; i < mc; ++i) out.uniform[static_cast<std::size_t>(t) * n + i] = unif(meas);
    }
}

void draw_fermion_batch(const std::uint64_t *seeds, const double *p, int count, int n, int depth, bool closed,
                        std::vector<FermionDraw> &out, int threads)
{
    out.resize(count);
    if (threads <= 0) threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    threads = std::min(threads, std::max(1, count));
    std::atomic<int> next{0};
    std::atomic<bool> failed{false};
    auto work = [&]() {
        for (;;)
        {
            const int i = next.fetch_add(1);
            if (i >= count) return;
            try
            {
                draw_fermion_trajectory(seeds[i], n, depth, p[i], closed, out[i]);
            }
            catch (...)
            {
                failed = true;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(work);
    for (auto &th : pool) th.join();
    if (failed) throw std::runtime_error("free-fermion trajectory draw failed");
}
} // namespace mg
