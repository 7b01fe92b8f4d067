// free_energy.exe: drop-in for the reference's measurement-record free energy
// (cpp/apps/free_energy.cpp) on the GB300 batched runner.
//
//   free_energy.exe [N] [p] [realizations] [circ_type] [init_state]
//
// Each trajectory of the periodic Haar brickwork starts from a random product
// (init_state 0) or random Haar (1) state and runs 4N equilibration plus 24N
// production timesteps, one brickwork layer and its measurement layer each.
// The layer surprisal -ln P(joint outcome) accumulates into F; the production
// part is fitted by least squares against the production timestep, and the
// half-chain S1 (bits) is sampled on the reference's schedule. Output, file
// names, environment controls and the resume contract follow the reference
// (paths inside the reference project):
//   usage, loop, samples and time-series rows     cpp/apps/free_energy.cpp:96-629
//   stream derivation per trajectory              cpp/apps/free_energy.cpp:454-466
//   CSV headers, seed recovery, entropy schedule,
//   checkpoint readers                            cpp/include/mipt/free_energy_resume.hpp:70-534
//   Welford accumulators and their reconstruction cpp/include/mipt/util/stats.hpp:19-48,
//                                                 cpp/include/mipt/util/resume_csv.hpp:129-207
//   file-name spelling                            cpp/include/mipt/util/text.hpp:80-133
//
// The GB300 path: trajectories run in batches on the device (initial states
// drawn on host threads and uploaded, every layer and joint measurement in
// the batched pass kernels, S1 from the batch's observation schedule); the
// host keeps the per-timestep accumulators in trajectory order, appends one
// samples row per trajectory and rewrites the time series after each batch.
// MIPT_GB300_FP64=1 selects FP64 states, MIPT_GB300_BATCH the trajectories per
// launch. MIPT_FREE_ENERGY_CUDA_ENTROPY(_MIN_KEPT) are accepted and have no
// effect: every entropy is computed on the device.
#include "cli_common.hpp"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <iomanip>
#include <limits>
#include <sstream>

namespace
{
using namespace mgcli;

constexpr const char *kSamplesHeader =
    "N,p,circ_type,circuit_name,init_state,trajectory,parity_sector,"
    "trajectory_seed,equil_timesteps,production_timesteps,total_timesteps,"
    "measurements_total,measurements_production,F_total,F_production,"
    "production_rate_endpoint,production_slope,free_energy_density_tilde";
constexpr const char *kTimeseriesHeader =
    "N,p,circ_type,circuit_name,init_state,requested_realizations,"
    "completed_realizations,t,t_over_L,phase,F_mean,F_stddev,F_stderr,"
    "F_over_tL_mean,F_over_tL_stddev,F_over_tL_stderr,S_half_mean,"
    "S_half_stddev,S_half_stderr,S_half_count";
constexpr std::uint64_t kCircuitSalt = 0x4349524355495455ull; // "CIRCUITU"
constexpr std::uint64_t kInitialSalt = 0x494e495449414c53ull; // "INITIALS"

// ------------------------------------------------------------ statistics
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
    // Welford state back from a written (mean, sample stddev, count); nan or
    // count 0 mean "no samples".
    static Stats from_stddev(double mean, double sd, std::uint64_t count)
    {
        Stats s;
        if (count == 0 || std::isnan(mean)) return s;
        s.count = count;
        s.mean = mean;
        s.m2 = count > 1 ? sd * sd * static_cast<double>(count - 1) : 0.0;
        return s;
    }
};

struct TimeStats
{
    Stats cumulative_f, f_over_tl, half_entropy;
};

// Least-squares slope of F_production against the production timestep.
struct LineFit
{
    std::uint64_t count = 0;
    double sx = 0, sy = 0, sxx = 0, sxy = 0;
    void add(double x, double y)
    {
        ++count;
        sx += x;
        sy += y;
        sxx += x * x;
        sxy += x * y;
    }
    double slope() const
    {
        const double den = static_cast<double>(count) * sxx - sx * sx;
        if (count < 2 || !(den > 0.0)) throw std::runtime_error("Not enough production points for a free-energy slope.");
        return (static_cast<double>(count) * sxy - sx * sy) / den;
    }
};

// ------------------------------------------------------------ seeds
std::uint64_t splitmix(std::uint64_t v) { return mipt_gb300_splitmix64(v); }

std::uint64_t odd_inverse(std::uint64_t odd)
{
    std::uint64_t x = 1;
    for (int i = 0; i < 6; ++i) x *= 2ull - odd * x; // Newton: doubles the correct low bits
    return x;
}

std::uint64_t unxorshift(std::uint64_t v, int shift)
{
    std::uint64_t r = v;
    for (int done = shift; done < 64; done += shift) r = v ^ (r >> shift);
    return r;
}

// splitmix64 is a bijection: undo its three mixing steps and the increment.
std::uint64_t splitmix_inverse(std::uint64_t v)
{
    v = unxorshift(v, 31);
    v *= odd_inverse(0x94d049bb133111ebull);
    v = unxorshift(v, 27);
    v *= odd_inverse(0xbf58476d1ce4e5b9ull);
    v = unxorshift(v, 30);
    return v - 0x9e3779b97f4a7c15ull;
}

// ------------------------------------------------------------ text
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

std::string compact_decimal(double v)
{
    std::ostringstream o;
    o << std::fixed << std::setprecision(12) << v;
    std::string t = o.str();
    while (!t.empty() && t.back() == '0') t.pop_back();
    if (!t.empty() && t.back() == '.') t.pop_back();
    return t == "-0" ? "0" : t;
}

std::string compact_count(std::uint64_t c)
{
    if (c >= 1000000 && c % 1000000 == 0) return std::to_string(c / 1000000) + "m";
    if (c >= 1000 && c % 1000 == 0) return std::to_string(c / 1000) + "k";
    return std::to_string(c);
}

std::string duration(double seconds)
{
    if (!std::isfinite(seconds) || seconds < 0.0) return "--h --m --s";
    const auto total = static_cast<std::uint64_t>(std::llround(seconds));
    char b[64];
    std::snprintf(b, sizeof(b), "%02lluh %02llum %02llus", static_cast<unsigned long long>(total / 3600),
                  static_cast<unsigned long long>((total % 3600) / 60), static_cast<unsigned long long>(total % 60));
    return b;
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

[[noreturn]] void refuse(const std::string &why) { throw std::runtime_error("Resume refused: " + why); }

double parse_double(const std::string &t, const std::string &where)
{
    try
    {
        std::size_t used = 0;
        const double v = std::stod(t, &used);
        if (used == t.size()) return v;
    }
    catch (const std::exception &)
    {
    }
    refuse("could not parse '" + t + "' as a number in " + where);
}

long parse_long(const std::string &t, const std::string &where)
{
    try
    {
        std::size_t used = 0;
        const long v = std::stol(t, &used);
        if (used == t.size()) return v;
    }
    catch (const std::exception &)
    {
    }
    refuse("could not parse '" + t + "' as an integer in " + where);
}

std::uint64_t parse_u64(const std::string &t, const std::string &where)
{
    try
    {
        std::size_t used = 0;
        const unsigned long long v = std::stoull(t, &used);
        if (used == t.size()) return v;
    }
    catch (const std::exception &)
    {
    }
    refuse("could not parse '" + t + "' as an unsigned integer in " + where);
}

std::string read_file(const std::string &path)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("Could not read " + path);
    std::ostringstream s;
    s << in.rdbuf();
    return s.str();
}

// ------------------------------------------------------------ environment
bool env_flag(const char *name, bool fallback)
{
    const char *v = std::getenv(name);
    if (!v) return fallback;
    std::string t(v);
    for (auto &c : t) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    if (t == "1" || t == "true" || t == "yes" || t == "on") return true;
    if (t == "0" || t == "false" || t == "no" || t == "off") return false;
    return fallback;
}

// An integer setting; unset, unparsable or out-of-range values take the default.
long env_int(const char *name, long fallback, long lo, long hi)
{
    const char *v = std::getenv(name);
    if (!v || !*v) return fallback;
    char *end = nullptr;
    errno = 0;
    const long x = std::strtol(v, &end, 10);
    if (errno != 0 || end == v || *end != '\0' || x < lo || x > hi) return fallback;
    return x;
}

// ------------------------------------------------------------ run identity
struct Identity
{
    int n = 0;
    double p = 0.0;
    int circ_type = 0, init_state = 0;
    long requested = 0; // 0: not recorded (samples rows)
};

void require_match(const Identity &want, const Identity &got, const std::string &where)
{
    auto mismatch = [&](const char *what, const std::string &was, const std::string &now) {
        refuse(where + " was produced with " + what + '=' + was + ", but this run uses " + now +
               ". Move the existing files aside, or set MIPT_FREE_ENERGY_RESUME=0 to overwrite them.");
    };
    if (got.n != want.n) mismatch("N", std::to_string(got.n), std::to_string(want.n));
    if (std::abs(got.p - want.p) > 1.0e-12 * std::max(1.0, std::abs(want.p)))
        mismatch("p", std::to_string(got.p), std::to_string(want.p));
    if (got.circ_type != want.circ_type)
        mismatch("circ_type", std::to_string(got.circ_type), std::to_string(want.circ_type));
    if (got.init_state != want.init_state)
        mismatch("init_state", std::to_string(got.init_state), std::to_string(want.init_state));
    if (want.requested > 0 && got.requested > 0 && got.requested != want.requested)
        mismatch("realizations", std::to_string(got.requested), std::to_string(want.requested));
}

bool samples_entropy_at(int t, bool enabled, int max_t, int stride)
{
    if (!enabled || max_t < 0) return false;
    if (t == 0) return true;
    if (t > max_t) return false;
    return t % stride == 0 || t == max_t;
}

// ------------------------------------------------------------ checkpoint readers
struct SamplesScan
{
    long completed = 0;
    std::uint64_t master = 0;
    bool has_master = false;
    std::uintmax_t valid_bytes = 0, file_bytes = 0;
};

SamplesScan scan_samples(const std::string &path, const Identity &want)
{
    const std::string text = read_file(path);
    SamplesScan scan;
    scan.file_bytes = text.size();
    std::size_t cur = 0;
    auto next_line = [&](std::string &line) {
        if (cur >= text.size()) return false;
        const std::size_t nl = text.find('\n', cur);
        if (nl == std::string::npos) return false; // unterminated: killed mid-flush
        line = text.substr(cur, nl - cur);
        cur = nl + 1;
        return true;
    };
    std::string line;
    if (!next_line(line)) return scan;
    if (line != kSamplesHeader)
        refuse(path + " has a different column layout than this binary writes. It was made by another version of "
                      "free_energy.exe; finish it with that binary, move it aside, or set MIPT_FREE_ENERGY_RESUME=0.");
    scan.valid_bytes = cur;
    long line_no = 1;
    while (next_line(line))
    {
        ++line_no;
        const auto f = split_csv(line);
        const std::string where = path + " line " + std::to_string(line_no);
        if (f.size() != 18)
            refuse(where + " has " + std::to_string(f.size()) +
                   " fields, expected 18. The file is corrupt beyond a simple truncation.");
        Identity got;
        got.n = static_cast<int>(parse_long(f[0], where));
        got.p = parse_double(f[1], where);
        got.circ_type = static_cast<int>(parse_long(f[2], where));
        got.init_state = static_cast<int>(parse_long(f[4], where));
        require_match(want, got, path);
        const long trajectory = parse_long(f[5], where);
        if (trajectory != scan.completed)
            refuse(where + " has trajectory=" + std::to_string(trajectory) + " where " +
                   std::to_string(scan.completed) +
                   " was expected. Trajectory indices must run 0,1,2,... with no gaps; this file looks like two runs "
                   "concatenated.");
        scan.master = splitmix_inverse(parse_u64(f[7], where)) ^ static_cast<std::uint64_t>(trajectory);
        scan.has_master = true;
        ++scan.completed;
        scan.valid_bytes = cur;
    }
    return scan;
}

struct SeriesScan
{
    long completed = 0;
    std::vector<TimeStats> stats;
};

SeriesScan load_series(const std::string &path, const Identity &want, int total, bool record, int max_t, int stride)
{
    const std::string text = read_file(path);
    std::vector<std::string> lines;
    for (std::size_t cur = 0; cur < text.size();)
    {
        const std::size_t nl = text.find('\n', cur);
        if (nl == std::string::npos) break;
        lines.push_back(text.substr(cur, nl - cur));
        cur = nl + 1;
    }
    if (lines.empty() || lines.front() != kTimeseriesHeader)
        refuse(path + " has a different column layout than this binary writes. It was made by another version of "
                      "free_energy.exe; finish it with that binary, move it aside, or set MIPT_FREE_ENERGY_RESUME=0.");
    const std::size_t rows = static_cast<std::size_t>(total) + 1;
    if (lines.size() != rows + 1)
        refuse(path + " holds " + std::to_string(lines.size() - 1) + " timestep rows, but this run has " +
               std::to_string(rows) + ". The time-series checkpoint belongs to a different N.");
    SeriesScan scan;
    scan.stats.resize(rows);
    long completed = -1;
    for (std::size_t r = 0; r < rows; ++r)
    {
        const auto f = split_csv(lines[r + 1]);
        const std::string where = path + " line " + std::to_string(r + 2);
        if (f.size() != 20)
            refuse(where + " has " + std::to_string(f.size()) + " fields, expected 20.");
        Identity got;
        got.n = static_cast<int>(parse_long(f[0], where));
        got.p = parse_double(f[1], where);
        got.circ_type = static_cast<int>(parse_long(f[2], where));
        got.init_state = static_cast<int>(parse_long(f[4], where));
        got.requested = parse_long(f[5], where);
        require_match(want, got, path);
        const long t = parse_long(f[7], where);
        if (t != static_cast<long>(r))
            refuse(where + " has t=" + std::to_string(t) + " on the row for t=" + std::to_string(r) + '.');
        const long row_completed = parse_long(f[6], where);
        if (completed < 0)
            completed = row_completed;
        else if (row_completed != completed)
            refuse(where + " reports completed_realizations=" + std::to_string(row_completed) +
                   " but earlier rows report " + std::to_string(completed) + '.');
        if (row_completed < 0) refuse(where + " reports a negative completed_realizations.");
        const auto count = static_cast<std::uint64_t>(row_completed);
        TimeStats &s = scan.stats[r];
        s.cumulative_f = Stats::from_stddev(parse_double(f[10], where), parse_double(f[11], where), count);
        s.f_over_tl = Stats::from_stddev(parse_double(f[13], where), parse_double(f[14], where), count);
        const auto ecount = static_cast<std::uint64_t>(parse_long(f[19], where));
        s.half_entropy = Stats::from_stddev(parse_double(f[16], where), parse_double(f[17], where), ecount);
        const std::uint64_t wanted = samples_entropy_at(static_cast<int>(r), record, max_t, stride) ? count : 0;
        if (ecount != wanted)
            refuse(where + " has S_half_count=" + std::to_string(ecount) + " at t=" + std::to_string(r) +
                   ", but the current half-chain entropy settings imply " + std::to_string(wanted) +
                   ". Re-run with the MIPT_FREE_ENERGY_HALF_ENTROPY / _ENTROPY_MAX_T / _ENTROPY_STRIDE values the "
                   "original run used.");
    }
    scan.completed = completed < 0 ? 0 : completed;
    return scan;
}

// ------------------------------------------------------------ writers
void write_stat(std::string &o, const Stats &s)
{
    if (s.count == 0)
        o += "nan,nan,nan";
    else
        o += fmt(s.mean) + ',' + fmt(s.stddev()) + ',' + fmt(s.stderr_());
}

void write_series(const std::string &path, int n, double p, int circ_type, int init_state, int requested, int eq,
                  const std::vector<TimeStats> &stats)
{
    const std::uint64_t completed = stats.empty() ? 0 : stats.front().cumulative_f.count;
    const std::string tmp = path + ".tmp";
    std::string o = std::string(kTimeseriesHeader) + "\n";
    const std::string lead = std::to_string(n) + ',' + fmt(p) + ',' + std::to_string(circ_type) + ',' +
                             quote(circuit_info(circ_type).name) + ',' + std::to_string(init_state) + ',' +
                             std::to_string(requested) + ',' + std::to_string(completed) + ',';
    for (std::size_t i = 0; i < stats.size(); ++i)
    {
        const int t = static_cast<int>(i);
        const char *phase = t == 0 ? "initial" : (t <= eq ? "equilibration" : "production");
        o += lead + std::to_string(t) + ',' + fmt(static_cast<double>(t) / static_cast<double>(n)) + ',' + phase + ',';
        write_stat(o, stats[i].cumulative_f);
        o += ',';
        write_stat(o, stats[i].f_over_tl);
        o += ',';
        write_stat(o, stats[i].half_entropy);
        o += ',' + std::to_string(stats[i].half_entropy.count) + '\n';
    }
    {
        std::ofstream csv(tmp, std::ios::out | std::ios::trunc);
        if (!csv) throw std::runtime_error("Could not open time-series CSV: " + tmp);
        csv << o;
        csv.flush();
        if (!csv) throw std::runtime_error("Failed while writing time-series CSV: " + path);
    }
    if (std::rename(tmp.c_str(), path.c_str()) != 0)
        throw std::runtime_error("Could not replace time-series CSV: " + path);
}

void usage(const char *prog)
{
    std::cout << "Usage: " << prog << " [N] [p] [realizations] [circ_type] [init_state]\n\n"
              << "  N          number of sites in the periodic 1D ring\n"
              << "  p          measurement rate in [0,1]\n"
              << "  realizations number of Monte Carlo trajectories\n"
              << "  circ_type  same convention as the other MIPT simulators:\n";
    print_circuit_type_help(std::cout, "               ");
    std::cout << "  init_state 0 = random product state, 1 = random Haar state\n\n"
              << "The first 4L timesteps equilibrate the trajectory; the following 24L\n"
              << "timesteps determine the free-energy density. One timestep is one even\n"
              << "or odd unitary brickwork layer followed by its measurement layer.\n"
              << "For circ_type 2, 3, or 4, every initial state has a definite randomly\n"
              << "selected global parity.\n\n"
              << "An interrupted run is resumed by re-issuing the identical command: the\n"
              << "two CSVs it already wrote are the checkpoint, so trajectories, the\n"
              << "per-timestep aggregates and the seed stream all continue where they\n"
              << "stopped. MIPT_FREE_ENERGY_RESUME=0 discards them and starts over.\n\n"
              << "Environment controls:\n"
              << "  MIPT_FREE_ENERGY_RESUME=1\n"
              << "  MIPT_FREE_ENERGY_SEED=<integer>\n"
              << "  MIPT_FREE_ENERGY_PROGRESS_MS=1000\n"
              << "  MIPT_FREE_ENERGY_HALF_ENTROPY=1\n"
              << "  MIPT_FREE_ENERGY_ENTROPY_MAX_T=<absolute timestep> (default 2L)\n"
              << "  MIPT_FREE_ENERGY_ENTROPY_STRIDE=1\n"
              << "  MIPT_GB300_FP64=1 (FP64 states), MIPT_GB300_BATCH=<trajectories per launch>\n";
}

int run(int argc, char **argv)
{
    if (argc > 1 && (std::strcmp(argv[1], "--help") == 0 || std::strcmp(argv[1], "-h") == 0))
    {
        usage(argv[0]);
        return 0;
    }
    if (argc != 6)
    {
        usage(argv[0]);
        return 2;
    }
    const int n = std::stoi(argv[1]);
    const double p = std::stod(argv[2]);
    const long parsed_reals = std::stol(argv[3]);
    if (parsed_reals < 1 || parsed_reals > 1000000000L)
        throw std::invalid_argument("realizations must lie in [1,1000000000].");
    const int realizations = static_cast<int>(parsed_reals);
    const int circ_type = std::stoi(argv[4]);
    circuit_info(circ_type);
    const int init_state = std::stoi(argv[5]);
    if (n < 2 || n >= 31) throw std::invalid_argument("N must lie in [2,30] for the dense exact-state protocol.");
    validate_circuit_site_count(circ_type, n, "N");
    if (!(p >= 0.0 && p <= 1.0)) throw std::invalid_argument("p must lie in [0,1].");
    if (init_state != 0 && init_state != 1) throw std::invalid_argument("init_state must be 0 or 1.");
    require_gb300_circuit(circ_type);
    if (n < 4) throw std::invalid_argument("the GB300 batched runner needs N >= 4.");

    const int eq = 4 * n, production = 24 * n, total = eq + production;
    const int progress_ms = static_cast<int>(env_int("MIPT_FREE_ENERGY_PROGRESS_MS", 1000, 50, 600000L));
    const bool record = env_flag("MIPT_FREE_ENERGY_HALF_ENTROPY", true);
    const int max_t = record ? static_cast<int>(env_int("MIPT_FREE_ENERGY_ENTROPY_MAX_T", 2 * n, 0, total)) : -1;
    const int stride = static_cast<int>(env_int("MIPT_FREE_ENERGY_ENTROPY_STRIDE", 1, 1, total));
    const long configured_seed =
        env_int("MIPT_FREE_ENERGY_SEED", -1, -1, std::numeric_limits<long>::max());
    const bool resume_enabled = env_flag("MIPT_FREE_ENERGY_RESUME", true);
    const bool fp64 = use_fp64();

    const std::string prefix = "free_energy_" + std::string(circuit_info(circ_type).tag) + "_n_" +
                               std::to_string(n) + "_p_" + compact_decimal(p) + "_init_" +
                               std::to_string(init_state) + "_reals_" +
                               compact_count(static_cast<std::uint64_t>(realizations));
    const std::string samples_path = prefix + "_samples.csv";
    const std::string series_path = prefix + "_timeseries.csv";

    // --- resume: the two CSVs are the checkpoint; read before writing anything.
    Identity id;
    id.n = n;
    id.p = p;
    id.circ_type = circ_type;
    id.init_state = init_state;
    id.requested = realizations;
    const bool samples_exist = std::filesystem::exists(samples_path);
    const bool series_exist = std::filesystem::exists(series_path);
    SamplesScan sscan;
    SeriesScan tscan;
    bool resuming = false;
    if (resume_enabled && (samples_exist || series_exist))
    {
        if (samples_exist) sscan = scan_samples(samples_path, id);
        if (!series_exist && sscan.completed == 0)
        {
            // Killed inside the first batch: nothing completed, start over.
        }
        else if (!samples_exist || !series_exist)
            throw std::runtime_error(std::string("Resume refused: only ") +
                                     (samples_exist ? samples_path : series_path) +
                                     " is present. Both CSVs are needed to continue a run -- the samples file carries "
                                     "the trajectories and the seed stream, the time series carries the per-timestep "
                                     "aggregates, and neither can be rebuilt from the other. Move it aside, or set "
                                     "MIPT_FREE_ENERGY_RESUME=0 to start over.");
        else
        {
            tscan = load_series(series_path, id, total, record, max_t, stride);
            if (tscan.completed > sscan.completed)
                throw std::runtime_error("Resume refused: " + series_path + " aggregates " +
                                         std::to_string(tscan.completed) + " trajectories but " + samples_path +
                                         " holds only " + std::to_string(sscan.completed) +
                                         " rows. The samples file has been truncated or edited; resuming would "
                                         "count those trajectories twice.");
            resuming = sscan.completed > 0 || tscan.completed > 0;
        }
    }
    std::uint64_t master;
    if (resuming && sscan.has_master)
        master = sscan.master;
    else if (configured_seed >= 0)
        master = static_cast<std::uint64_t>(configured_seed);
    else
    {
        std::random_device rd;
        master = (static_cast<std::uint64_t>(rd()) << 32) ^ static_cast<std::uint64_t>(rd());
    }
    const int start = resuming ? static_cast<int>(sscan.completed) : 0;
    if (resuming)
    {
        std::cout << "Resuming from " << samples_path << ": " << sscan.completed << '/' << realizations
                  << " trajectories already recorded";
        if (sscan.has_master) std::cout << ", seed stream recovered";
        std::cout << ".\n";
        if (sscan.file_bytes > sscan.valid_bytes)
            std::cout << "  Dropping " << (sscan.file_bytes - sscan.valid_bytes)
                      << " bytes of an unterminated trailing row (killed mid-flush); every complete row is kept.\n";
        if (tscan.completed != sscan.completed)
            std::cout << "  The time-series aggregate holds " << tscan.completed
                      << " trajectories against the samples file's " << sscan.completed
                      << "; the run stopped between the two writes. Every sample row is kept and "
                         "completed_realizations reports the aggregate's own count.\n";
        if (configured_seed >= 0 && sscan.has_master && static_cast<std::uint64_t>(configured_seed) != sscan.master)
            std::cout << "  Ignoring MIPT_FREE_ENERGY_SEED=" << configured_seed << "; continuing the recovered stream "
                      << master << " so no trajectory is simulated twice.\n";
        if (start >= realizations)
        {
            std::cout << samples_path << " is already complete (" << sscan.completed << '/' << realizations
                      << " trajectories). Nothing to do.\n";
            return 0;
        }
        if (sscan.file_bytes > sscan.valid_bytes) std::filesystem::resize_file(samples_path, sscan.valid_bytes);
    }
    std::ofstream samples(samples_path, resuming ? (std::ios::out | std::ios::app) : (std::ios::out | std::ios::trunc));
    if (!samples) throw std::runtime_error("Could not open sample CSV: " + samples_path);
    if (!resuming) samples << kSamplesHeader << '\n';

    std::cout << "Measurement-record free energy: N=" << n << ", p=" << fmt(p) << ", circ_type=" << circ_type << " ("
              << circuit_info(circ_type).name << ")" << ", init_state=" << init_state
              << (init_state == 0 ? " (product)" : " (Haar)") << ", realizations=" << realizations
              << ", seed=" << master << '\n'
              << (resuming ? "trajectories " + std::to_string(start) + ".." + std::to_string(realizations - 1) +
                                 " remaining\n"
                           : std::string())
              << "t_eq=" << eq << ", t_production=" << production << ", t_total=" << total << '\n';
    if (record) std::cout << "Half-chain S1 recorded through t=" << max_t << " with stride=" << stride << ".\n";
    std::cout << "GB300 batched runner: " << (fp64 ? "FP64" : "FP32") << " states\n";

    std::vector<TimeStats> stats = resuming ? std::move(tscan.stats) : std::vector<TimeStats>(total + 1);

    // --- device batch: the whole 28N-step trajectory per execute.
    std::vector<int> steps;
    for (int t = 0; t <= total; ++t)
        if (samples_entropy_at(t, record, max_t, stride)) steps.push_back(t);
    const int capacity = batch_capacity(n, fp64, realizations - start);
    mipt_gb300_batch_config cfg{};
    cfg.n_qubits = n;
    cfg.periods = total / 2;
    cfg.closed = 1;
    cfg.fp64 = fp64 ? 1 : 0;
    cfg.chunk_bits = 16;
    cfg.observables = steps.empty() ? 0 : MIPT_GB300_OBS_SVN_HALF;
    configure_circuit(cfg, circ_type);
    cfg.split_last = 0; // the free-energy loop measures the full state (cpp/include/mipt/probed.hpp:589-598)
    Batch batch(cfg, capacity);
    // RPPU batches carry one more (identity) layer slot after the 28N timesteps.
    const int slots = total + (cfg.circuit == 2 || cfg.circuit == 4 ? 1 : 0);
    const bool fixed_parity = circ_type == 2 || circ_type == 3 || circ_type == 4;
    if (!steps.empty())
        check(mipt_gb300_batch_set_observation_steps(batch.get(), steps.data(), static_cast<int>(steps.size())),
              "mipt_gb300_batch_set_observation_steps");
    const int points = steps.empty() ? 1 : static_cast<int>(steps.size());

    std::vector<std::uint64_t> tseed(capacity), init_seed(capacity), measured(static_cast<std::size_t>(capacity) * slots);
    std::vector<std::uint32_t> wseed(capacity);
    std::vector<double> prob(capacity, p), surprisal(static_cast<std::size_t>(capacity) * slots),
        obs(static_cast<std::size_t>(capacity) * points * 4);
    std::vector<int> sector(capacity);

    PauseSentinel pause;
    const auto t0 = std::chrono::steady_clock::now();
    auto last_report = t0;
    for (int first = start; first < realizations; first += capacity)
    {
        pause.wait([&]() { samples.flush(); });
        const auto batch_t0 = std::chrono::steady_clock::now();
        const int count = std::min(capacity, realizations - first);
        for (int i = 0; i < count; ++i)
        {
            tseed[i] = splitmix(master ^ static_cast<std::uint64_t>(first + i));
            wseed[i] = static_cast<std::uint32_t>(splitmix(tseed[i] ^ kCircuitSalt));
            init_seed[i] = splitmix(tseed[i] ^ kInitialSalt);
        }
        check(mipt_gb300_batch_set_initial_states(batch.get(), init_seed.data(), init_state, fixed_parity ? 1 : 0,
                                                  count, sector.data()),
              "mipt_gb300_batch_set_initial_states");
        check(mipt_gb300_batch_prepare_haar_workspace(batch.get(), wseed.data(), prob.data(), count),
              "mipt_gb300_batch_prepare_haar_workspace");
        check(mipt_gb300_batch_execute(batch.get(), nullptr), "mipt_gb300_batch_execute");
        check(mipt_gb300_batch_fetch(batch.get(), measured.data(), nullptr, surprisal.data(),
                                     steps.empty() ? nullptr : obs.data(), nullptr),
              "mipt_gb300_batch_fetch");
        std::string rows;
        for (int i = 0; i < count; ++i)
        {
            const double *sp = surprisal.data() + static_cast<std::size_t>(i) * slots;
            const std::uint64_t *mm = measured.data() + static_cast<std::size_t>(i) * slots;
            double cumulative = 0.0, prod_f = 0.0;
            std::uint64_t meas_total = 0, meas_prod = 0;
            LineFit fit;
            stats[0].cumulative_f.add(0.0);
            int point = 0;
            if (!steps.empty() && steps[0] == 0)
                stats[0].half_entropy.add(obs[(static_cast<std::size_t>(i) * points + point++) * 4]);
            for (int s = 0; s < total; ++s)
            {
                const int t = s + 1;
                const int m = __builtin_popcountll(mm[s]);
                cumulative += sp[s];
                meas_total += static_cast<std::uint64_t>(m);
                stats[t].cumulative_f.add(cumulative);
                stats[t].f_over_tl.add(cumulative / (static_cast<double>(t) * static_cast<double>(n)));
                if (point < points && !steps.empty() && steps[point] == t)
                    stats[t].half_entropy.add(obs[(static_cast<std::size_t>(i) * points + point++) * 4]);
                if (t > eq)
                {
                    prod_f += sp[s];
                    meas_prod += static_cast<std::uint64_t>(m);
                    fit.add(static_cast<double>(t - eq), prod_f);
                }
            }
            const double slope = fit.slope();
            rows += std::to_string(n) + ',' + fmt(p) + ',' + std::to_string(circ_type) + ',' +
                    quote(circuit_info(circ_type).name) + ',' + std::to_string(init_state) + ',' +
                    std::to_string(first + i) + ',' + std::to_string(sector[i]) + ',' + std::to_string(tseed[i]) +
                    ',' + std::to_string(eq) + ',' + std::to_string(production) + ',' + std::to_string(total) + ',' +
                    std::to_string(meas_total) + ',' + std::to_string(meas_prod) + ',' + fmt(cumulative) + ',' +
                    fmt(prod_f) + ',' + fmt(prod_f / static_cast<double>(production)) + ',' + fmt(slope) + ',' +
                    fmt(slope / static_cast<double>(n)) + '\n';
        }
        samples << rows;
        samples.flush();
        if (!samples) throw std::runtime_error("Failed while writing sample CSV: " + samples_path);
        write_series(series_path, n, p, circ_type, init_state, realizations, eq, stats);

        const auto now = std::chrono::steady_clock::now();
        const double batch_s = std::chrono::duration<double>(now - batch_t0).count();
        const int done = first + count;
        if (done == realizations ||
            std::chrono::duration_cast<std::chrono::milliseconds>(now - last_report).count() >= progress_ms)
        {
            const double elapsed = std::chrono::duration<double>(now - t0).count();
            const double rate = elapsed > 0.0 ? static_cast<double>(done - start) / elapsed : 0.0;
            const double eta = rate > 0.0 ? static_cast<double>(realizations - done) / rate
                                          : std::numeric_limits<double>::infinity();
            std::cout << '\r' << "realizations: " << done << '/' << realizations << " | avg=" << std::fixed
                      << std::setprecision(3) << rate << " traj/s"
                      << " | current=" << (batch_s > 0.0 ? count / batch_s : 0.0) << " traj/s"
                      << " | ETA=" << duration(eta) << std::flush;
            std::cout.unsetf(std::ios::fixed);
            last_report = now;
        }
    }
    std::cout << "\nSaved " << samples_path << " and " << series_path << ".\n";
    return 0;
}
} // namespace

int main(int argc, char **argv)
{
    try
    {
        return run(argc, argv);
    }
    catch (const std::exception &e)
    {
        std::cerr << "free_energy.exe: " << e.what() << '\n';
        return 1;
    }
}
