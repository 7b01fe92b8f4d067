// entropy.exe: drop-in for the reference's translation-averaged entropy
// scan (cpp/apps/entropy.cpp, writer and usage in
// cpp/include/mipt/entropy.hpp:403-420,580-676, checkpoint contract in
// cpp/include/mipt/entropy_resume.hpp:44-246) on the GB300 batched runner.
//
//   entropy.exe [N] [periods] [p] [realizations] [circ_type] [output_csv]
//
// Per trajectory of the periodic Haar brickwork, S2 = -ln Tr(rho_A^2) for
// every contiguous cyclic block of L_A = 2..N/2 sites and, up to
// MIPT_ENTROPY_S1_MAX_LA (0 = no cap; MIPT_ENTROPY_S1=0 turns it off),
// S1 = -Tr(rho_A ln rho_A), each averaged over the N translations; the
// per-L_A means are accumulated over trajectories (mean, sample stddev,
// stderr) and the CSV is rewritten after every batch of trajectories, so it
// is the checkpoint a re-issued command resumes from (MIPT_ENTROPY_RESUME=0
// starts over). Entropies come from the batch's region observables (GPU RDM
// Grams, bits) times ln 2. Trajectory seeds: mipt_gb300_trajectory_seed
// (MIPT_GB300_SEED or a random master, trajectory index); MIPT_GB300_FP64=1
// selects FP64 states, MIPT_GB300_BATCH the trajectories per launch.
#include "cli_common.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <limits>
#include <sstream>

namespace
{
using namespace mgcli;

constexpr const char *kHeader =
    "N,periods,p,requested_realizations,completed_realizations,circ_type,circuit_name,fermionic_trace,L_A,x,ln_x,"
    "S1_mean,S1_stddev,S1_stderr,S2_mean,S2_stddev,S2_stderr,subsystems_per_realization,total_subsystems";
constexpr const char *kLegacyHeader =
    "N,periods,p,requested_realizations,completed_realizations,circ_type,circuit_name,fermionic_trace,L_A,x,ln_x,"
    "S2_mean,S2_stddev,S2_stderr,subsystems_per_realization,total_subsystems";
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kLn2 = 0.693147180559945309417232121458176568;

// Welford accumulator (the reference's util::RunningStats semantics).
struct Stats
{
    std::uint64_t count = 0;
    double mean = 0.0, m2 = 0.0;
    void add(double v)
    {
        ++count;
        const double d = v - mean;
        mean += d / static_cast<double>(count);
        m2 += d * (v - mean);
    }
    double stddev() const { return count > 1 ? std::sqrt(std::max(0.0, m2 / static_cast<double>(count - 1))) : 0.0; }
    double stderr_() const { return count > 1 ? stddev() / std::sqrt(static_cast<double>(count)) : 0.0; }
};

bool env_bool(const char *name, bool fallback)
{
    const char *v = std::getenv(name);
    if (!v || !*v) return fallback;
    std::string t(v);
    for (auto &c : t) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    if (t == "1" || t == "true" || t == "on" || t == "yes") return true;
    if (t == "0" || t == "false" || t == "off" || t == "no") return false;
    throw std::invalid_argument(std::string(name) + " must be a boolean (0/1).");
}

void usage(const char *prog)
{
    std::cout << "Usage: " << prog << " [N] [periods] [p] [realizations] [circ_type] [output_csv]\n\n"
              << "  N            fixed number of sites/qubits in the periodic 1D ring\n"
              << "  periods      number of brickwork periods (even layer + odd layer)\n"
              << "  p            measurement rate in [0,1]\n"
              << "  realizations number of independent quantum trajectories\n"
              << "  circ_type    same convention as mipt.exe:\n";
    print_circuit_type_help(std::cout, "                 ");
    std::cout << "  output_csv   one row per L_A=2,...,floor(N/2)\n\n"
              << "The CSV provides ln_x together with S1_mean and S2_mean (natural logarithms):\n"
              << "  S1 = -Tr(rho_A ln rho_A), S2 = -ln Tr(rho_A^2), each averaged over the N\n"
              << "  contiguous cyclic translations of the block, then over trajectories.\n"
              << "  MIPT_ENTROPY_S1=0            report S2 only\n"
              << "  MIPT_ENTROPY_S1_MAX_LA=k     compute S1 only for L_A<=k (0 = no cap); others report NaN\n"
              << "  MIPT_ENTROPY_RESUME=0        discard an existing output_csv and start over\n"
              << "  MIPT_GB300_SEED, MIPT_GB300_FP64, MIPT_GB300_BATCH as for mipt.exe\n";
}

std::string fmt(double v)
{
    char b[64];
    std::snprintf(b, sizeof(b), "%.17g", v);
    return b;
}

std::string quote(const std::string &v)
{
    std::string q("\"");
    for (char ch : v) q += ch == '"' ? std::string("\"\"") : std::string(1, ch);
    return q + "\"";
}

void write_results(const std::string &path, int n, int periods, double p, int requested, int circ_type,
                   const std::vector<Stats> &s1, const std::vector<Stats> &s2)
{
    std::ofstream csv(path, std::ios::out | std::ios::trunc);
    if (!csv) throw std::runtime_error("Could not open output CSV: " + path);
    std::string out = std::string(kHeader) + "\n";
    const double nan = std::numeric_limits<double>::quiet_NaN();
    for (int kept = 2; kept <= n / 2; ++kept)
    {
        const double x = (static_cast<double>(n) / kPi) * std::sin(kPi * kept / static_cast<double>(n));
        const Stats &a = s1[kept], &b = s2[kept];
        const bool has1 = a.count > 0;
        out += std::to_string(n) + ',' + std::to_string(periods) + ',' + fmt(p) + ',' + std::to_string(requested) +
               ',' + std::to_string(b.count) + ',' + std::to_string(circ_type) + ',' +
               quote(circuit_info(circ_type).name) + ',' + (circuit_info(circ_type).fermionic_trace ? "1" : "0") +
               ',' + std::to_string(kept) + ',' + fmt(x) + ',' +
               fmt(std::log(x)) + ',' + fmt(has1 ? a.mean : nan) + ',' + fmt(has1 ? a.stddev() : nan) + ',' +
               fmt(has1 ? a.stderr_() : nan) + ',' + fmt(b.mean) + ',' + fmt(b.stddev()) + ',' + fmt(b.stderr_()) +
               ',' + std::to_string(n) + ',' + std::to_string(static_cast<std::uint64_t>(n) * b.count) + '\n';
    }
    csv << out;
    csv.flush();
    if (!csv) throw std::runtime_error("Failed while writing output CSV: " + path);
}

std::vector<std::string> split_csv(const std::string &row)
{
    std::vector<std::string> f;
    std::string cur;
    bool quoted = false;
    for (std::size_t i = 0; i < row.size(); ++i)
    {
        const char c = row[i];
        if (quoted)
        {
            if (c != '"')
                cur += c;
            else if (i + 1 < row.size() && row[i + 1] == '"')
            {
                cur += '"';
                ++i;
            }
            else
                quoted = false;
        }
        else if (c == '"')
            quoted = true;
        else if (c == ',')
        {
            f.push_back(cur);
            cur.clear();
        }
        else
            cur += c;
    }
    f.push_back(cur);
    return f;
}

[[noreturn]] void refuse(const std::string &why)
{
    throw std::runtime_error("Resume refused: " + why);
}

double real_field(const std::string &s, const std::string &path)
{
    if (s == "nan" || s == "-nan") return std::numeric_limits<double>::quiet_NaN();
    std::size_t used = 0;
    double v = 0.0;
    try
    {
        v = std::stod(s, &used);
    }
    catch (...)
    {
        refuse(path + " holds a non-numeric field '" + s + "'.");
    }
    if (used != s.size()) refuse(path + " holds a non-numeric field '" + s + "'.");
    return v;
}

long int_field(const std::string &s, const std::string &path)
{
    std::size_t used = 0;
    long v = 0;
    try
    {
        v = std::stol(s, &used);
    }
    catch (...)
    {
        refuse(path + " holds a non-integer field '" + s + "'.");
    }
    if (used != s.size()) refuse(path + " holds a non-integer field '" + s + "'.");
    return v;
}

// stderr = stddev / sqrt(count): a cross-check of the recorded count.
bool spread_matches(double sd, double se, std::uint64_t count)
{
    if (!(sd > 0.0) || !(se > 0.0) || count < 2) return true;
    const double implied = (sd / se) * (sd / se);
    return std::abs(implied - static_cast<double>(count)) <= 1.0e-6 * static_cast<double>(count);
}

Stats from_spread(double mean, double sd, std::uint64_t count)
{
    Stats s;
    s.count = count;
    s.mean = count > 0 ? mean : 0.0;
    s.m2 = count > 1 ? sd * sd * static_cast<double>(count - 1) : 0.0;
    return s;
}

// Reads the checkpoint CSV (the reference's resume::load contract).
long load_checkpoint(const std::string &path, int n, int periods, double p, int requested, int circ_type,
                     int max_s1, std::vector<Stats> &s1, std::vector<Stats> &s2)
{
    std::ifstream in(path);
    if (!in) refuse("could not read " + path + ".");
    std::string header;
    if (!std::getline(in, header)) return 0; // nothing was ever written
    if (!header.empty() && header.back() == '\r') header.pop_back();
    const bool legacy = header == kLegacyHeader;
    if (!legacy && header != kHeader)
        refuse(path + " has a different column layout than this binary writes. Finish it with that binary, move it "
                      "aside, or set MIPT_ENTROPY_RESUME=0 to overwrite it.");
    if (legacy && max_s1 >= 2)
        refuse(path + " has no S1 columns, but this run computes the von Neumann entropy. Re-run with "
                      "MIPT_ENTROPY_S1=0 to continue it as an S2-only scan, or move it aside.");
    const std::vector<std::string> cols = split_csv(header);
    auto col = [&](const char *name) {
        const auto it = std::find(cols.begin(), cols.end(), name);
        return static_cast<std::size_t>(it - cols.begin());
    };
    std::vector<std::vector<std::string>> rows;
    for (std::string line; std::getline(in, line);)
    {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.empty()) continue;
        rows.push_back(split_csv(line));
        if (rows.back().size() != cols.size()) refuse(path + " has a row with " + std::to_string(rows.back().size()) +
                                                      " fields where the header has " + std::to_string(cols.size()) + ".");
    }
    const std::size_t expected_rows = static_cast<std::size_t>(n / 2 - 1);
    if (rows.size() != expected_rows)
        refuse(path + " holds " + std::to_string(rows.size()) + " block rows, but N=" + std::to_string(n) + " has " +
               std::to_string(expected_rows) + " (L_A = 2..N/2). The checkpoint belongs to a different N.");
    long completed = -1;
    for (std::size_t r = 0; r < rows.size(); ++r)
    {
        const auto &f = rows[r];
        auto same = [&](const char *what, bool ok) {
            if (!ok) refuse(path + " was written for a different " + what + "; this run would mix two experiments.");
        };
        same("N", int_field(f[col("N")], path) == n);
        same("periods", int_field(f[col("periods")], path) == periods);
        same("p", real_field(f[col("p")], path) == p);
        same("circ_type", int_field(f[col("circ_type")], path) == circ_type);
        same("realizations", int_field(f[col("requested_realizations")], path) == requested);
        const long kept = int_field(f[col("L_A")], path);
        if (kept != static_cast<long>(r) + 2)
            refuse(path + " line " + std::to_string(r + 2) + " has L_A=" + std::to_string(kept) + " where " +
                   std::to_string(r + 2) + " was expected; the rows must run L_A = 2..N/2 in order.");
        const long done = int_field(f[col("completed_realizations")], path);
        if (done < 0) refuse(path + " reports a negative completed_realizations.");
        if (completed < 0)
            completed = done;
        else if (done != completed)
            refuse(path + " line " + std::to_string(r + 2) + " reports completed_realizations=" + std::to_string(done) +
                   " but earlier rows report " + std::to_string(completed) + ".");
        const auto count = static_cast<std::uint64_t>(done);
        const double m2 = real_field(f[col("S2_mean")], path), d2 = real_field(f[col("S2_stddev")], path);
        if (count > 0 && !std::isfinite(m2))
            refuse(path + " line " + std::to_string(r + 2) + " has a non-finite S2_mean.");
        if (!spread_matches(d2, real_field(f[col("S2_stderr")], path), count))
            refuse(path + " line " + std::to_string(r + 2) +
                   " has S2_stddev and S2_stderr that do not agree with completed_realizations=" +
                   std::to_string(count) + ". The file has been edited or two runs were concatenated.");
        s2[kept] = from_spread(m2, d2, count);
        if (legacy) continue;
        const double m1 = real_field(f[col("S1_mean")], path), d1 = real_field(f[col("S1_stddev")], path);
        const bool file_s1 = std::isfinite(m1), run_s1 = kept <= max_s1;
        if (count > 0 && file_s1 != run_s1)
            refuse(path + " records S1 for L_A up to " + std::to_string(file_s1 ? kept : kept - 1) +
                   " but this run is configured for L_A up to " + std::to_string(max_s1) +
                   ". Re-run with the MIPT_ENTROPY_S1 / MIPT_ENTROPY_S1_MAX_LA values the original run used.");
        if (file_s1 && !spread_matches(d1, real_field(f[col("S1_stderr")], path), count))
            refuse(path + " line " + std::to_string(r + 2) +
                   " has S1_stddev and S1_stderr that do not agree with completed_realizations=" +
                   std::to_string(count) + '.');
        s1[kept] = from_spread(m1, d1, file_s1 ? count : 0);
    }
    return completed < 0 ? 0 : completed;
}
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
        if (argc != 7)
        {
            usage(argv[0]);
            return 2;
        }
        const int n = std::stoi(argv[1]);
        const int periods = std::stoi(argv[2]);
        const double p = std::stod(argv[3]);
        const int realizations = std::stoi(argv[4]);
        const int circ_type = std::stoi(argv[5]);
        const std::string output = argv[6];
        circuit_info(circ_type);
        if (n < 4) throw std::invalid_argument("N must be at least 4 for the requested cyclic entropy scan.");
        if (n >= 63) throw std::invalid_argument("N must be less than 63 for exact basis indexing.");
        if (periods < 0) throw std::invalid_argument("periods must be non-negative.");
        if (p < 0.0 || p > 1.0) throw std::invalid_argument("p must be in [0,1].");
        if (realizations <= 0) throw std::invalid_argument("realizations must be positive.");
        validate_circuit_site_count(circ_type, n, "N");
        require_gb300_circuit(circ_type);
        if (n > 30) throw std::invalid_argument("N must be at most 30 for the GB300 state-vector path.");

        const int max_block = n / 2, min_kept = 2;
        int max_s1 = 0;
        if (env_bool("MIPT_ENTROPY_S1", true))
        {
            const long cap = env_long("MIPT_ENTROPY_S1_MAX_LA", 0);
            if (cap < 0 || cap > 62) throw std::invalid_argument("MIPT_ENTROPY_S1_MAX_LA must lie in [0, 62].");
            max_s1 = cap == 0 ? max_block : std::min(max_block, static_cast<int>(cap));
        }
        std::vector<Stats> s1(static_cast<std::size_t>(n + 1)), s2(static_cast<std::size_t>(n + 1));
        long start = 0;
        if (env_bool("MIPT_ENTROPY_RESUME", true) && std::filesystem::exists(output))
            start = load_checkpoint(output, n, periods, p, realizations, circ_type, max_s1, s1, s2);
        if (start > 0)
        {
            std::cout << "Resuming from " << output << ": " << start << '/' << realizations
                      << " trajectories already averaged in.\n";
            if (start >= realizations)
            {
                std::cout << output << " is already complete. Nothing to do.\n";
                return 0;
            }
        }
        const bool fp64 = use_fp64();
        const std::uint64_t seed = master_seed();
        std::cout << "Running entanglement-entropy chord-length scan: N=" << n << ", periods=" << periods
                  << ", p=" << p << ", realizations=" << realizations << ", circ_type=" << circ_type << " ("
                  << circuit_info(circ_type).name << "), fermionic_trace="
                  << (circuit_info(circ_type).fermionic_trace ? 1 : 0) << "\n"
                  << "Averaging each L_A over " << n << " contiguous cyclic translations per traj.\n"
                  << "Entropies: S2 for L_A=" << min_kept << ".." << max_block << "; S1 ";
        if (max_s1 < min_kept)
            std::cout << "disabled (MIPT_ENTROPY_S1=0 or MIPT_ENTROPY_S1_MAX_LA below " << min_kept << ")\n";
        else
            std::cout << "for L_A=" << min_kept << ".." << max_s1
                      << (max_s1 < max_block ? " (larger blocks report NaN)\n" : "\n");

        const int remaining = realizations - static_cast<int>(start);
        const int capacity = batch_capacity(n, fp64, remaining);
        mipt_gb300_batch_config cfg{};
        cfg.n_qubits = n;
        cfg.periods = periods;
        cfg.closed = 1;
        cfg.fp64 = fp64 ? 1 : 0;
        cfg.chunk_bits = 16;
        configure_circuit(cfg, circ_type);
        Batch batch(cfg, capacity);
        // Regions: (L_A, translation) -> S2 column and, when computed, S1 column.
        std::vector<int> col2(static_cast<std::size_t>((max_block + 1) * n), -1), col1(col2.size(), -1);
        int regions = 0;
        for (int kept = min_kept; kept <= max_block; ++kept)
            for (int c = 0; c < n; ++c)
            {
                std::vector<int> modes(static_cast<std::size_t>(kept));
                for (int j = 0; j < kept; ++j) modes[j] = (c + j) % n;
                int id = 0;
                check(mipt_gb300_batch_add_region(batch.get(), modes.data(), kept, 2, &id), "mipt_gb300_batch_add_region");
                col2[kept * n + c] = id;
                if (kept <= max_s1)
                {
                    check(mipt_gb300_batch_add_region(batch.get(), modes.data(), kept, 1, &id),
                          "mipt_gb300_batch_add_region");
                    col1[kept * n + c] = id;
                }
                regions = id + 1;
            }
        std::cout << "GB300 path: " << mipt_gb300_version() << ", " << (fp64 ? "FP64" : "FP32") << " state vectors, "
                  << capacity << " trajectories per launch, MIPT_GB300_SEED=" << seed << "\n";

        std::vector<std::uint64_t> seeds(static_cast<std::size_t>(capacity));
        std::vector<double> pv(static_cast<std::size_t>(capacity), p);
        std::vector<double> ent(static_cast<std::size_t>(capacity) * regions);
        PauseSentinel pause;
        const auto t_start = std::chrono::steady_clock::now();
        for (long r0 = start; r0 < realizations; r0 += capacity)
        {
            pause.wait([] {});
            const int count = static_cast<int>(std::min<long>(capacity, realizations - r0));
            for (int i = 0; i < count; ++i) seeds[i] = mipt_gb300_trajectory_seed(seed, static_cast<std::uint64_t>(r0 + i));
            check(mipt_gb300_batch_prepare_haar(batch.get(), seeds.data(), pv.data(), count, nullptr),
                  "mipt_gb300_batch_prepare_haar");
            check(mipt_gb300_batch_execute(batch.get(), nullptr), "mipt_gb300_batch_execute");
            check(mipt_gb300_batch_fetch(batch.get(), nullptr, nullptr, nullptr, nullptr, nullptr), "mipt_gb300_batch_fetch");
            check(mipt_gb300_batch_fetch_regions(batch.get(), ent.data()), "mipt_gb300_batch_fetch_regions");
            for (int i = 0; i < count; ++i)
            {
                const double *e = ent.data() + static_cast<std::size_t>(i) * regions;
                for (int kept = min_kept; kept <= max_block; ++kept)
                {
                    double a2 = 0.0, a1 = 0.0;
                    for (int c = 0; c < n; ++c)
                    {
                        a2 += e[col2[kept * n + c]] * kLn2;
                        if (kept <= max_s1) a1 += e[col1[kept * n + c]] * kLn2;
                    }
                    s2[kept].add(a2 / n);
                    if (kept <= max_s1) s1[kept].add(a1 / n);
                }
            }
            write_results(output, n, periods, p, realizations, circ_type, s1, s2);
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
            const long done = r0 + count;
            const double rate = el > 0.0 ? static_cast<double>(done - start) / el : 0.0;
            std::cout << "\r" << done << '/' << realizations << " traj. | avg. " << std::round(rate * 100.0) / 100.0
                      << " traj/s | ETA " << static_cast<int>(rate > 0.0 ? (realizations - done) / rate : 0.0)
                      << "s          " << std::flush;
        }
        const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        std::cout << "\nSaved entropy scaling data to " << output << ". Elapsed: " << total << "s\n";
        return 0;
    }
    catch (const std::exception &e)
    {
        std::cerr << "entropy.exe error: " << e.what() << '\n';
        return 1;
    }
}
