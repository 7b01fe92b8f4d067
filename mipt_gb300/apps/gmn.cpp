// gmn.exe: drop-in for the reference's rho3.bin -> "p,gmn,bipneg" consumer
// (cpp/apps/gmn.cpp:330-516 over cpp/include/mipt/analysis/rdm_batch_cli.hpp),
// on the GPU through the C ABI: the bipartite-negativity prefilter is
// mipt_gb300_cut_negativities and the GMN SDP, which the reference hands to
// MOSEK, is the batched ADMM of mipt_gb300_gmn_solve.
//
//   gmn.exe [0|1] [input_file] [output_csv] [limit_per_p]
//
// Same arguments, defaults (mode 0, rho3.bin, data.csv), environment
// (GMN_LIMIT_PER_P, GMN_BATCH_RECORDS), output rows (p, gmn, bipneg with 17
// significant digits), "<output>_meta.csv" sidecar, per-p record limit and
// exit codes (0, 1 on an error) as the reference. Per matrix, as
// cpp/apps/gmn.cpp:237-328,406-440 does:
//   - non-finite entries are replaced and the matrix made Hermitian
//     (average of rho[r][c] and conj(rho[c][r]); real diagonal);
//   - mode 0 evaluates Re(rho), mode 1 the complex matrix;
//   - min over the three single-qubit cuts of the negativity <= 1e-10
//     certifies GMN = 0 without a solve;
//   - GMN values in (-1e-10, 0) and non-finite ones are written as 0.
// GPU solver settings: MIPT_GB300_GMN_GAP (certified duality gap, default
// 1e-7), MIPT_GB300_GMN_MAX_ITER (default 20000), MIPT_GB300_FP64=1 (FP64
// iterations). A state that reaches the iteration limit uncertified is
// written with the midpoint of its certified bracket and counted on stderr.
#include "cli_common.hpp"

#include <algorithm>
#include <array>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <limits>

namespace
{
using namespace mgcli;

constexpr double kPrefilterTol = 1.0e-10;

void usage(const char *prog)
{
    std::cout << "Usage: " << prog << " [0|1] [input_file] [output_csv] [limit_per_p]\n\n"
              << "Modes:\n"
              << "  0    Real-only GMN SDP on Re(rho).\n"
              << "  1    Complex Hermitian GMN SDP on the full rho.\n\n"
              << "Defaults: " << prog << " 0 rho3.bin data.csv (no per-p limit)\n\n"
              << "limit_per_p: largest number of records evaluated per p value; 0 or omitted = no limit.\n\n"
              << "Environment variables:\n"
              << "  GMN_BATCH_RECORDS=N        records per GPU batch (default 256)\n"
              << "  GMN_LIMIT_PER_P=N          per-p record limit when the argument is omitted\n"
              << "  MIPT_GB300_GMN_GAP=x       certified duality gap of the GPU solver (default 1e-7)\n"
              << "  MIPT_GB300_GMN_MAX_ITER=N  ADMM iterations per state at most (default 20000)\n"
              << "  MIPT_GB300_FP64=1          FP64 ADMM iterations (certificates are FP64 either way)\n\n"
              << "Input must contain three-qubit 8x8 reduced density matrices.\n";
}

std::uint64_t parse_u64(const char *v, const char *name)
{
    if (!v || !*v || v[0] == '-') throw std::invalid_argument(std::string(name) + " must be a non-negative integer.");
    char *end = nullptr;
    errno = 0;
    const unsigned long long x = std::strtoull(v, &end, 10);
    if (errno != 0 || end == v || *end != '\0')
        throw std::invalid_argument(std::string(name) + " must be a non-negative integer.");
    return x;
}

int parse_mode(const std::string &v)
{
    if (v == "0") return 0;
    if (v == "1") return 1;
    if (v == "3")
        throw std::invalid_argument("The former leading argument '3' has been removed. Use '0' for real-only GMN or "
                                    "'1' for complex GMN.");
    if (v == "6") throw std::invalid_argument("Six-qubit retained-subsystem analysis has been removed; use rho3 data only.");
    throw std::invalid_argument("First argument must be evaluation mode 0 or 1.");
}

// Replaces non-finite entries and makes the 8x8 (re, im) matrix Hermitian;
// returns the number of non-finite values seen and whether anything changed.
std::pair<std::uint64_t, bool> sanitize(double *m)
{
    std::uint64_t bad = 0;
    bool changed = false;
    for (int r = 0; r < 8; ++r)
    {
        double *d = m + 2 * (r * 8 + r);
        if (!std::isfinite(d[0]))
        {
            d[0] = 0.0;
            ++bad;
            changed = true;
        }
        if (!std::isfinite(d[1])) ++bad;
        if (d[1] != 0.0)
        {
            d[1] = 0.0;
            changed = true;
        }
    }
    for (int r = 0; r < 8; ++r)
        for (int c = r + 1; c < 8; ++c)
        {
            double *a = m + 2 * (r * 8 + c), *b = m + 2 * (c * 8 + r);
            for (double v : {a[0], a[1], b[0], b[1]}) bad += std::isfinite(v) ? 0u : 1u;
            const bool fa = std::isfinite(a[0]) && std::isfinite(a[1]);
            const bool fb = std::isfinite(b[0]) && std::isfinite(b[1]);
            double re = 0.0, im = 0.0;
            if (fa && fb)
            {
                re = 0.5 * (a[0] + b[0]);
                im = 0.5 * (a[1] - b[1]);
            }
            else if (fa)
            {
                re = a[0];
                im = a[1];
            }
            else if (fb)
            {
                re = b[0];
                im = -b[1];
            }
            if (a[0] != re || a[1] != im || b[0] != re || b[1] != -im) changed = true;
            a[0] = re;
            a[1] = im;
            b[0] = re;
            b[1] = -im;
        }
    return {bad, changed};
}

std::string csv_quote(const std::string &v)
{
    std::string q("\"");
    for (char ch : v) q += ch == '"' ? std::string("\"\"") : std::string(1, ch);
    return q + "\"";
}

std::string sidecar_path(const std::string &out)
{
    const auto dot = out.find_last_of('.');
    const auto slash = out.find_last_of("/\\");
    const bool ext = dot != std::string::npos && (slash == std::string::npos || dot > slash);
    return ext ? out.substr(0, dot) + "_meta.csv" : out + "_meta.csv";
}

void write_sidecar(const std::string &out, const Rho3Metadata &m, std::uint32_t subsystems, const std::string &input,
                   const std::string &solver)
{
    const std::string path = sidecar_path(out);
    std::ofstream f(path, std::ios::out | std::ios::trunc);
    if (!f)
    {
        std::cerr << "Warning: could not write the metadata sidecar " << path << ".\n";
        return;
    }
    std::string line = "N,spatial_dimension,grid_x,grid_y,periods,realizations,resolution,p_min,p_max,kept_qubits,"
                       "subsystem_count,record_count,solver,source\n";
    line += std::to_string(m.total_qubits) + ',' + std::to_string(m.spatial_dimension) + ',' + std::to_string(m.grid_x) +
            ',' + std::to_string(m.grid_y) + ',' + std::to_string(m.periods) + ',' + std::to_string(m.realizations) +
            ',' + std::to_string(m.resolution) + ',';
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.17g,%.17g,", m.p_min, m.p_max);
    line += buf;
    line += std::to_string(m.kept_qubits) + ',' + std::to_string(subsystems) + ',' + std::to_string(m.record_count) +
            ',' + csv_quote(solver) + ',' + csv_quote(input) + '\n';
    f << line;
    if (!f) std::cerr << "Warning: failed while writing the metadata sidecar " << path << ".\n";
}

struct Job
{
    double p = 0.0;
    std::array<double, 128> rho{};
};
} // namespace

int main(int argc, char **argv)
{
    try
    {
        if (argc > 1 && (std::string(argv[1]) == "--help" || std::string(argv[1]) == "-h"))
        {
            usage(argv[0]);
            return 0;
        }
        int mode = 0, next = 1;
        if (argc > 1)
        {
            mode = parse_mode(argv[1]);
            next = 2;
        }
        const std::string input = argc > next ? argv[next] : "rho3.bin";
        const std::string output = argc > next + 1 ? argv[next + 1] : "data.csv";
        std::uint64_t limit_per_p = 0;
        if (argc > next + 2)
            limit_per_p = parse_u64(argv[next + 2], "limit_per_p");
        else if (const char *v = std::getenv("GMN_LIMIT_PER_P"); v && *v)
            limit_per_p = parse_u64(v, "GMN_LIMIT_PER_P");
        if (argc > next + 3) throw std::invalid_argument("Too many command-line arguments.");

        Rho3Reader reader(input);
        const Rho3Metadata &meta = reader.metadata();
        if (meta.kept_qubits != 3 || meta.matrix_dimension != 8)
            throw std::runtime_error("Input file must contain three-qubit 8x8 reduced density matrices.");
        const std::uint32_t S = reader.subsystem_count();
        const long batch_records = std::max(1L, env_long("GMN_BATCH_RECORDS", 256));
        mipt_gb300_gmn_config cfg{};
        cfg.max_iter = static_cast<int>(std::max(1L, env_long("MIPT_GB300_GMN_MAX_ITER", 20000)));
        cfg.check_every = 10;
        const char *gv = std::getenv("MIPT_GB300_GMN_GAP");
        cfg.gap_tol = (gv && *gv) ? std::stod(gv) : 1e-7;
        cfg.feas_tol = cfg.gap_tol;
        cfg.sigma = 0.0; // the library's default penalty
        cfg.fp64 = use_fp64() ? 1 : 0;

        std::ofstream out(output);
        if (!out) throw std::runtime_error("Could not create output CSV: " + output);
        out << "p,gmn,bipneg\n";
        const char *mname = mode == 1 ? "complex" : "real-only";
        write_sidecar(output, meta, S, input, std::string("gmn.exe ") + mname);

        std::uint64_t max_records = meta.record_count;
        if (limit_per_p != 0 && meta.resolution != 0)
            max_records = std::min<std::uint64_t>(max_records, limit_per_p * meta.resolution);
        const std::uint64_t total = max_records * S;
        std::cout << "Calculating three-qubit " << mname << " GMN values from " << input << " (" << meta.record_count
                  << " input records, " << S << " retained subsystems each, up to " << total << " total solves";
        if (limit_per_p != 0) std::cout << "; limit_per_p=" << limit_per_p << " records/p-value";
        std::cout << ").\nGMN on the GPU: batched ADMM, certified duality gap " << cfg.gap_tol << ", "
                  << "batches of " << batch_records << " records.\n";

        std::vector<std::uint64_t> accepted(meta.resolution, 0);
        std::uint64_t scanned = 0, evaluated = 0, skipped = 0, processed = 0, prefiltered = 0, nonfinite_in = 0,
                      sanitized = 0, nonfinite_out = 0, clipped = 0, uncertified = 0;
        double max_imag = 0.0;
        PauseSentinel pause;
        Rho3Record rec;
        bool exhausted = false;
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<Job> jobs;
        while (processed < total && !exhausted)
        {
            pause.wait([&] { out.flush(); });
            jobs.clear();
            for (long got = 0; got < batch_records;)
            {
                if (!reader.read_record(rec))
                {
                    exhausted = true;
                    break;
                }
                ++scanned;
                ++got;
                if (rec.p_index >= accepted.size())
                    throw std::runtime_error("Input record has p_index outside metadata.resolution.");
                if (limit_per_p != 0 && accepted[rec.p_index] >= limit_per_p)
                {
                    ++skipped;
                    continue;
                }
                ++accepted[rec.p_index];
                ++evaluated;
                for (std::uint32_t s = 0; s < S; ++s)
                {
                    Job j;
                    j.p = rec.p;
                    std::copy(rec.rho_ri.begin() + s * 128, rec.rho_ri.begin() + (s + 1) * 128, j.rho.begin());
                    const auto r = sanitize(j.rho.data());
                    nonfinite_in += r.first;
                    if (r.second) ++sanitized;
                    double im2 = 0.0;
                    for (int i = 1; i < 128; i += 2) im2 += j.rho[i] * j.rho[i];
                    max_imag = std::max(max_imag, std::sqrt(im2));
                    if (mode == 0)
                        for (int i = 1; i < 128; i += 2) j.rho[i] = 0.0;
                    jobs.push_back(j);
                }
            }
            if (jobs.empty()) continue;
            const int n = static_cast<int>(jobs.size());
            std::vector<double> rho(static_cast<std::size_t>(n) * 128), neg(static_cast<std::size_t>(n) * 3);
            for (int i = 0; i < n; ++i) std::copy(jobs[i].rho.begin(), jobs[i].rho.end(), rho.begin() + i * 128);
            check(mipt_gb300_cut_negativities(rho.data(), n, neg.data()), "mipt_gb300_cut_negativities");
            std::vector<double> bip(n), value(n, 0.0);
            std::vector<int> solve;
            for (int i = 0; i < n; ++i)
            {
                double b = std::numeric_limits<double>::infinity();
                for (int m = 0; m < 3; ++m)
                    b = std::isfinite(neg[3 * i + m]) ? std::min(b, neg[3 * i + m])
                                                      : std::numeric_limits<double>::quiet_NaN();
                bip[i] = b;
                if (std::isfinite(b) && b <= kPrefilterTol)
                    ++prefiltered; // a separable cut certifies GMN = 0
                else
                    solve.push_back(i);
            }
            if (!solve.empty())
            {
                const int ns = static_cast<int>(solve.size());
                std::vector<double> sr(static_cast<std::size_t>(ns) * 128), g(ns), gap(ns);
                std::vector<int> it(ns);
                for (int k = 0; k < ns; ++k) std::copy(rho.begin() + solve[k] * 128, rho.begin() + (solve[k] + 1) * 128,
                                                       sr.begin() + k * 128);
                check(mipt_gb300_gmn_solve(&cfg, sr.data(), ns, nullptr, g.data(), gap.data(), it.data(), nullptr),
                      "mipt_gb300_gmn_solve");
                for (int k = 0; k < ns; ++k)
                {
                    value[solve[k]] = g[k];
                    if (it[k] < 0) ++uncertified;
                }
            }
            std::string rows;
            char buf[96];
            for (int i = 0; i < n; ++i)
            {
                double v = value[i];
                if (!std::isfinite(v)) ++nonfinite_out;
                double safe = std::isfinite(v) ? ((v < 0.0 && v > -1.0e-10) ? 0.0 : v) : 0.0;
                if (std::isfinite(v) && safe != v) ++clipped;
                std::snprintf(buf, sizeof(buf), "%.17g,%.17g,%.17g\n", jobs[i].p, safe, bip[i]);
                rows += buf;
            }
            out << rows;
            out.flush();
            processed += n;
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            std::cout << "\rProcessed " << processed << "/" << total << " matrices from " << evaluated << " records";
            if (skipped) std::cout << " (skipped " << skipped << " by limit)";
            std::cout << "; avg " << (el > 0 ? processed / el : 0.0) << "/s        " << std::flush;
        }
        std::cout << "\nWrote " << output << ".\nRecords scanned: " << scanned << "; evaluated: " << evaluated
                  << "; records skipped by limit_per_p: " << skipped
                  << "\nMatrices skipped by bipartite-negativity zero prefilter: " << prefiltered
                  << "\nMaximum imaginary Frobenius norm in input records: " << max_imag << "\n";
        if (nonfinite_in > 0)
            std::cerr << "Warning: replaced " << nonfinite_in << " non-finite density-matrix value(s) with 0 before "
                      << "solving; " << sanitized << " matrix/matrices were sanitized.\n";
        if (nonfinite_out > 0)
            std::cerr << "Warning: solver returned " << nonfinite_out
                      << " non-finite GMN value(s); those CSV entries were written as 0.\n";
        if (clipped > 0) std::cerr << "Warning: clipped " << clipped << " tiny negative GMN value(s) to 0.\n";
        if (uncertified > 0)
            std::cerr << "Warning: " << uncertified << " state(s) reached " << cfg.max_iter
                      << " ADMM iterations without a certified gap of " << cfg.gap_tol
                      << "; their rows hold the midpoint of the certified bracket.\n";
        if (mode == 0 && max_imag > 1.0e-10)
            std::cerr << "Warning: real-only mode evaluates Re(rho). For full complex Hermitian GMN evaluation, "
                      << "rerun as: " << argv[0] << " 1 " << input << ' ' << output << "\n";
        return 0;
    }
    catch (const std::exception &e)
    {
        std::cerr << "gmn.exe error: " << e.what() << "\n";
        return 1;
    }
}
