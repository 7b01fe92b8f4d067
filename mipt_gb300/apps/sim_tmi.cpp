// sim_tmi.exe -- drop-in for the reference's online TMI simulator on the
// GB300 path.
//
//   sim_tmi.exe [n = 10] [periods = 10] [realizations = 10] [resolution = 5]
//               [p_min = 0.0] [p_max = 1.0] [circ_type = 0]
//               [all_cycles = 0] [output.csv = auto]   (either order)
//
// Same arguments, defaults, exit codes, CSV schema (p,tmi; 17 significant
// digits), default output path, entropy-order switch (SIM_TMI_ENTROPY_ORDER)
// and resume contract (SIM_TMI_RESUME; the CSV is the checkpoint, only whole
// circuits are kept) as cpp/apps/sim_tmi.cpp and
// cpp/include/mipt/tmi/{runner,resume}.hpp of the reference. One row per
// (trajectory, cyclic offset): I_3 = S_A + S_B + S_C + S_D - S_AB - S_AC - S_BC
// of the final state over quarters starting at the offset
// (cpp/include/mipt/tmi/compute.hpp:89-113), evaluated on the device for a
// whole batch of trajectories at once.
//
// Environment as for mipt.exe (MIPT_GB300_SEED, MIPT_GB300_FP64,
// MIPT_GB300_BATCH), plus SIM_TMI_PAUSE_FILE / MIPT_PAUSE_FILE.
#include "cli_common.hpp"

#include <algorithm>
#include <cerrno>
#include <iomanip>
#include <sstream>
#include <sys/stat.h>

namespace
{
using namespace mgcli;

int entropy_order()
{
    const char *raw = std::getenv("SIM_TMI_ENTROPY_ORDER");
    if (raw == nullptr || *raw == '\0') return 1;
    const std::string_view t(raw);
    if (t == "1") return 1;
    if (t == "2") return 2;
    throw std::invalid_argument("SIM_TMI_ENTROPY_ORDER must be 1 (von Neumann) or 2 (Renyi-2), got \"" +
                                std::string(t) + "\".");
}

bool resume_enabled()
{
    const char *v = std::getenv("SIM_TMI_RESUME");
    return !env_falsey_path(v);
}

std::string number_for_filename(double v)
{
    if (std::abs(v) < 1.0e-15) v = 0.0;
    std::ostringstream o;
    o << std::fixed << std::setprecision(12) << v;
    std::string t = o.str();
    if (t.find('.') != std::string::npos)
    {
        while (!t.empty() && t.back() == '0') t.pop_back();
        if (!t.empty() && t.back() == '.') t.pop_back();
    }
    if (t == "-0") t = "0";
    return t;
}

std::string output_tag(int circ_type, bool all_cycles, int order)
{
    std::string tag = circuit_info(circ_type).tag;
    if (all_cycles) tag += 'c';
    if (order == 2) tag += "_s2";
    return tag;
}

std::string default_output_path(int n, int realizations, int res, double p_min, double p_max, int circ_type,
                                bool all_cycles, int order)
{
    const std::string tag = output_tag(circ_type, all_cycles, order);
    std::ostringstream f;
    f << "tmi_" << tag << "_n_" << n << "_real_" << realizations << '_' << number_for_filename(p_min) << '_'
      << number_for_filename(p_max) << "_res_" << res << ".csv";
    return "csv/tmi/" + tag + "/" + f.str();
}

void ensure_parent_directory(const std::string &path)
{
    const std::size_t slash = path.find_last_of("/\\");
    if (slash == std::string::npos || slash == 0) return;
    std::string parent = path.substr(0, slash), cur;
    std::size_t pos = 0;
    if (parent[0] == '/')
    {
        cur = "/";
        pos = 1;
    }
    while (pos < parent.size())
    {
        const std::size_t next = parent.find_first_of("/\\", pos);
        const std::string part = parent.substr(pos, next == std::string::npos ? std::string::npos : next - pos);
        if (!part.empty())
        {
            if (!cur.empty() && cur.back() != '/') cur += '/';
            cur += part;
            if (::mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST)
                throw std::runtime_error("Could not create output directory: " + cur + " (" + std::strerror(errno) +
                                         ")");
        }
        if (next == std::string::npos) break;
        pos = next + 1;
    }
}

// ------------------------------------------------------------- checkpoint
struct Identity
{
    std::string tag, pmin, pmax;
    long n = 0, realizations = 0, res = 0;
};

bool parse_name(std::string_view base, Identity &id)
{
    const std::string_view pre = "tmi_", suf = ".csv";
    if (base.size() <= pre.size() + suf.size() || base.substr(0, pre.size()) != pre ||
        base.substr(base.size() - suf.size()) != suf)
        return false;
    std::string_view stem = base.substr(pre.size(), base.size() - pre.size() - suf.size());
    auto split_last = [](std::string_view t, std::string_view tok, std::string_view &h, std::string_view &tl) {
        const std::size_t at = t.rfind(tok);
        if (at == std::string_view::npos) return false;
        h = t.substr(0, at);
        tl = t.substr(at + tok.size());
        return true;
    };
    auto parse_long = [](std::string_view t, long &v) {
        if (t.empty()) return false;
        v = 0;
        for (char c : t)
        {
            if (c < '0' || c > '9') return false;
            v = v * 10 + (c - '0');
        }
        return true;
    };
    std::string_view h, tl;
    if (!split_last(stem, "_res_", h, tl) || !parse_long(tl, id.res)) return false;
    stem = h;
    if (!split_last(stem, "_real_", h, tl)) return false;
    const std::size_t a = tl.find('_');
    if (a == std::string_view::npos) return false;
    const std::size_t b = tl.find('_', a + 1);
    if (b == std::string_view::npos || tl.find('_', b + 1) != std::string_view::npos) return false;
    if (!parse_long(tl.substr(0, a), id.realizations)) return false;
    id.pmin = std::string(tl.substr(a + 1, b - a - 1));
    id.pmax = std::string(tl.substr(b + 1));
    stem = h;
    if (!split_last(stem, "_n_", h, tl) || !parse_long(tl, id.n)) return false;
    id.tag = std::string(h);
    return !id.tag.empty();
}

std::string_view basename_of(std::string_view p)
{
    const std::size_t s = p.find_last_of("/\\");
    return s == std::string_view::npos ? p : p.substr(s + 1);
}

struct Checkpoint
{
    bool name_verified = false;
    std::uint64_t rows = 0, dropped_rows = 0;
    std::uintmax_t kept_bytes = 0;
    std::size_t start_p_index = 0;
    int start_realization = 0;
};

[[noreturn]] void refuse(const std::string &why) { throw std::runtime_error("Resume refused: " + why); }

Checkpoint load_checkpoint(const std::string &path, const std::string &expected_name, int realizations, int cycles,
                           const std::vector<std::string> &p_texts)
{
    Checkpoint ck;
    Identity want, got;
    if (parse_name(basename_of(expected_name), want) && parse_name(basename_of(path), got))
    {
        std::string mismatch;
        auto tf = [&](const char *f, const std::string &w, const std::string &g) {
            if (mismatch.empty() && w != g) mismatch = std::string(f) + "=" + g + " (this run uses " + w + ")";
        };
        auto lf = [&](const char *f, long w, long g) {
            if (mismatch.empty() && w != g)
                mismatch = std::string(f) + "=" + std::to_string(g) + " (this run uses " + std::to_string(w) + ")";
        };
        tf("circuit tag", want.tag, got.tag);
        lf("n", want.n, got.n);
        lf("realizations", want.realizations, got.realizations);
        tf("p_min", want.pmin, got.pmin);
        tf("p_max", want.pmax, got.pmax);
        lf("resolution", want.res, got.res);
        if (!mismatch.empty())
            refuse(path + " was produced with " + mismatch +
                   ". Move the existing file aside, or set SIM_TMI_RESUME=0 to overwrite it.");
        ck.name_verified = true;
    }
    std::ifstream in(path, std::ios::binary);
    const std::string content((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    std::vector<std::string_view> lines;
    std::size_t pos = 0;
    while (true)
    {
        const std::size_t nl = content.find('\n', pos);
        if (nl == std::string::npos) break; // an unterminated last line is not a row
        lines.emplace_back(content.data() + pos, nl - pos);
        pos = nl + 1;
    }
    if (lines.empty()) return ck;
    if (lines.front() != "p,tmi")
        refuse(path + " does not start with the expected header \"p,tmi\"; found \"" + std::string(lines.front()) + "\".");
    const std::uint64_t per_p = static_cast<std::uint64_t>(realizations) * cycles;
    std::size_t group = 0;
    std::uint64_t in_group = 0, total = 0;
    std::uintmax_t offset = lines.front().size() + 1, boundary = offset;
    for (std::size_t i = 1; i < lines.size(); ++i)
    {
        const std::string_view row = lines[i];
        const std::size_t comma = row.find(',');
        if (comma == std::string_view::npos)
            refuse(path + " has a malformed row at line " + std::to_string(i + 1) + ": \"" + std::string(row) + "\".");
        const std::string_view pt = row.substr(0, comma);
        if (pt != p_texts[group])
        {
            if (in_group != per_p)
                refuse(path + " switches away from p=" + p_texts[group] + " after " + std::to_string(in_group) +
                       " rows, but a complete p group holds realizations*cycles = " + std::to_string(per_p) +
                       ". The file does not match this run's arguments.");
            ++group;
            if (group >= p_texts.size() || pt != p_texts[group])
                refuse(path + " carries p=" + std::string(pt) + " where this run's grid expects " +
                       (group < p_texts.size() ? p_texts[group] : std::string("no further values")) +
                       ". The file was produced with different p arguments.");
            in_group = 0;
        }
        ++in_group;
        ++total;
        offset += row.size() + 1;
        if (in_group % static_cast<std::uint64_t>(cycles) == 0) boundary = offset;
    }
    if (in_group > per_p)
        refuse(path + " holds " + std::to_string(in_group) + " rows for p=" + p_texts[group] + ", more than the " +
               std::to_string(per_p) + " a complete group can hold.");
    const std::uint64_t complete = in_group / static_cast<std::uint64_t>(cycles);
    ck.dropped_rows = in_group - complete * static_cast<std::uint64_t>(cycles);
    ck.rows = total - ck.dropped_rows;
    ck.kept_bytes = boundary;
    if (complete >= static_cast<std::uint64_t>(realizations))
    {
        ck.start_p_index = group + 1;
        ck.start_realization = 0;
    }
    else
    {
        ck.start_p_index = group;
        ck.start_realization = static_cast<int>(complete);
    }
    return ck;
}

// ------------------------------------------------------------------- run
void run(int n, int periods, int realizations, int res, double p_min, double p_max, int circ_type, bool all_cycles,
         const std::string &out_path, int order)
{
    if (n < 4 || (n % 4) != 0) throw std::invalid_argument("Online TMI requires n >= 4 and n divisible by 4.");
    if (periods <= 0) throw std::invalid_argument("periods must be positive.");
    if (realizations <= 0) throw std::invalid_argument("realizations must be positive.");
    if (res <= 0) throw std::invalid_argument("resolution must be positive.");
    if (!(0.0 <= p_min && p_min <= 1.0 && 0.0 <= p_max && p_max <= 1.0))
        throw std::invalid_argument("p_min and p_max must lie in [0, 1].");
    validate_circuit_site_count(circ_type, n);
    require_gb300_circuit(circ_type);

    const int cycles = all_cycles ? n / 4 : 1;
    const std::vector<double> ps = linspace(p_min, p_max, res);
    const std::uint64_t total = static_cast<std::uint64_t>(res) * realizations * cycles;
    std::vector<std::string> p_texts;
    for (double p : ps)
    {
        std::string t;
        append_double(t, p);
        p_texts.push_back(t);
    }
    ensure_parent_directory(out_path);

    Checkpoint ck;
    const bool resume = resume_enabled();
    if (resume && std::filesystem::exists(out_path))
        ck = load_checkpoint(out_path,
                             default_output_path(n, realizations, res, p_min, p_max, circ_type, all_cycles, order),
                             realizations, cycles, p_texts);
    if (ck.rows >= total)
    {
        std::cerr << out_path << " already holds all " << total << " TMI row(s) for this scan; nothing to do.\n"
                  << "Set SIM_TMI_RESUME=0 to overwrite it instead.\n";
        return;
    }
    const bool resuming = ck.rows > 0;
    if (resuming && ck.kept_bytes < std::filesystem::file_size(out_path))
        std::filesystem::resize_file(out_path, ck.kept_bytes);
    std::ofstream csv(out_path, resuming ? (std::ios::binary | std::ios::app) : (std::ios::binary | std::ios::trunc));
    if (!csv) throw std::runtime_error("Could not create output CSV: " + out_path);
    if (!resuming)
    {
        csv << "p,tmi\n";
        csv.flush();
    }

    const bool fp64 = use_fp64();
    PauseSentinel pause("SIM_TMI_PAUSE_FILE");
    std::cerr << "Online TMI simulation (GB300 path, " << mipt_gb300_version() << ")\n"
              << "n=" << n << ", periods=" << periods << ", realizations=" << realizations << ", resolution=" << res
              << ", p_min=" << p_min << ", p_max=" << p_max << ", block_qubits=" << n / 4
              << ", all_cycles=" << (all_cycles ? 1 : 0) << ", tmi_cycles_per_circuit=" << cycles
              << ", mode=" << circuit_info(circ_type).name << ", entropy_order=" << (order == 2 ? "renyi2" : "von_neumann")
              << ", precision=" << (fp64 ? "fp64" : "fp32") << ", output=" << out_path << '\n'
              << pause.describe() << '\n';
    if (resuming)
    {
        std::cerr << "RESUMED from " << out_path << ": " << ck.rows << " TMI row(s) already recorded";
        if (ck.dropped_rows > 0) std::cerr << "; dropped " << ck.dropped_rows << " row(s) of a partially written circuit";
        std::cerr << ".\nContinuing at p[" << ck.start_p_index << "]=" << ps[ck.start_p_index] << ", realization "
                  << ck.start_realization << '/' << realizations << ".\n";
        if (!ck.name_verified)
            std::cerr << "Warning: this output path does not follow the generated naming convention, so n, "
                         "realizations, the p range, the resolution and the circuit tag could not be checked against "
                         "it. Only the p grid and the per-p row counts inside the CSV were verified.\n";
        std::cerr << "Note: periods is recorded neither in the file nor in its name, so it is not validated on "
                     "resume.\n";
    }
    else if (!resume)
    {
        std::cerr << "Resume disabled by SIM_TMI_RESUME=0; any existing output was overwritten.\n";
    }

    const int capacity = batch_capacity(n, fp64, realizations);
    mipt_gb300_batch_config cfg{};
    cfg.n_qubits = n;
    cfg.periods = periods;
    cfg.closed = 1;
    cfg.fp64 = fp64 ? 1 : 0;
    cfg.chunk_bits = 16;
    cfg.observables = order == 2 ? MIPT_GB300_OBS_TMI_S2 : MIPT_GB300_OBS_TMI_VN;
    configure_circuit(cfg, circ_type);
    cfg.tmi_cycles = cycles;
    Batch batch(cfg, capacity);
    const std::uint64_t seed = master_seed();
    std::cerr << "trajectories per launch=" << capacity << ", MIPT_GB300_SEED=" << seed << '\n';

    std::vector<std::uint64_t> seeds(static_cast<std::size_t>(capacity));
    std::vector<double> pv(static_cast<std::size_t>(capacity));
    std::vector<double> tmi(static_cast<std::size_t>(capacity) * cycles);
    std::string buf;
    const auto start = std::chrono::steady_clock::now();
    std::uint64_t processed = ck.rows;
    const std::uint64_t resumed = ck.rows;
    for (std::size_t pi = ck.start_p_index; pi < ps.size(); ++pi)
    {
        const int first = (pi == ck.start_p_index) ? ck.start_realization : 0;
        for (int r0 = first; r0 < realizations; r0 += capacity)
        {
            pause.wait([&] { csv.flush(); });
            const int count = std::min(capacity, realizations - r0);
            for (int i = 0; i < count; ++i)
            {
                seeds[i] = mipt_gb300_trajectory_seed(seed, pi * static_cast<std::uint64_t>(realizations) + r0 + i);
                pv[i] = ps[pi];
            }
            check(mipt_gb300_batch_prepare_haar(batch.get(), seeds.data(), pv.data(), count, nullptr),
                  "mipt_gb300_batch_prepare_haar");
            check(mipt_gb300_batch_execute(batch.get(), nullptr), "mipt_gb300_batch_execute");
            check(mipt_gb300_batch_fetch(batch.get(), nullptr, nullptr, nullptr, nullptr, nullptr),
                  "mipt_gb300_batch_fetch");
            check(mipt_gb300_batch_fetch_tmi(batch.get(), order, tmi.data()), "mipt_gb300_batch_fetch_tmi");
            buf.clear();
            for (int i = 0; i < count; ++i)
                for (int c = 0; c < cycles; ++c)
                {
                    buf += p_texts[pi];
                    buf.push_back(',');
                    append_double(buf, tmi[static_cast<std::size_t>(i) * cycles + c]);
                    buf.push_back('\n');
                }
            csv.write(buf.data(), static_cast<std::streamsize>(buf.size()));
            csv.flush();
            if (!csv) throw std::runtime_error("Failed while writing output CSV.");
            processed += static_cast<std::uint64_t>(count) * cycles;
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count() -
                              pause.paused_seconds();
            const double avg = (processed - resumed) / std::max(1e-12, el);
            std::cerr << "\rprocessed TMI " << processed << '/' << total << " | avg " << std::fixed
                      << std::setprecision(2) << avg << "/s | ETA " << (avg > 0 ? (total - processed) / avg : 0.0)
                      << "s          " << std::defaultfloat << std::flush;
        }
    }
    csv.close();
    const double active = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count() -
                          pause.paused_seconds();
    std::cerr << "\nCompleted " << (processed - resumed) << " TMI row(s) in " << active << "s active time";
    if (resumed > 0) std::cerr << " (" << processed << " total in " << out_path << ")";
    std::cerr << ". Overall active throughput " << std::fixed << std::setprecision(2)
              << (processed - resumed) / std::max(1e-12, active) << "/s.\n";
}

void print_usage(const char *argv0)
{
    std::cerr << "Usage:\n  " << argv0
              << " [n = 10] [periods = 10] [realizations = 10] [resolution = 5] [p_min = 0.0] [p_max = 1.0]"
                 " [circ_type = 0] [all_cycles = 0] [output.csv = auto]\n\nArguments:\n  circ_type:\n";
    print_circuit_type_help(std::cerr, "    ");
    std::cerr << "  On the GB300 path circ_type=1 (Haar brickwork), 2 (FermionRPPU) and 4 (qRPPU) run.\n"
              << "  all_cycles = 0 computes the original offset only.\n"
              << "  all_cycles = 1 computes N/4 cyclic offsets; e.g. N=8 gives [0,1]|[2,3]|[4,5]|[6,7] and "
                 "[1,2]|[3,4]|[5,6]|[7,0].\n"
              << "  For backward compatibility, output.csv may also be supplied before all_cycles.\n"
              << "  If output.csv is omitted, the default path is:\n"
              << "    csv/tmi/<tag>/tmi_<tag>_n_<n>_real_<realizations>_<p_min>_<p_max>_res_<resolution>.csv\n"
              << "  all_cycles=1 appends c to the tag, SIM_TMI_ENTROPY_ORDER=2 appends _s2.\n\n"
              << "Output CSV columns:\n  p,tmi\n\n"
              << "Entropy order: SIM_TMI_ENTROPY_ORDER=1 (default, von Neumann) or 2 (Renyi-2).\n"
              << "Resume: re-issue the identical command (and MIPT_GB300_SEED) to continue an interrupted run;\n"
              << "SIM_TMI_RESUME=0 overwrites instead.\n"
              << "Host pause: create PAUSE_MIPT (or SIM_TMI_PAUSE_FILE / MIPT_PAUSE_FILE) to pause.\n";
}

bool is_bool01(std::string_view v) { return v == "0" || v == "1"; }
bool parse_bool01(std::string_view v, const char *name)
{
    if (v == "0") return false;
    if (v == "1") return true;
    throw std::invalid_argument(std::string(name) + " must be 0 or 1.");
}
} // namespace

int main(int argc, char **argv)
{
    try
    {
        if (argc > 1 && (std::strcmp(argv[1], "--help") == 0 || std::strcmp(argv[1], "-h") == 0))
        {
            print_usage(argv[0]);
            return 0;
        }
        if (argc > 10)
        {
            std::cerr << "Too many arguments. Use --help for usage.\n";
            return 2;
        }
        const int n = (argc > 1) ? std::stoi(argv[1]) : 10;
        const int periods = (argc > 2) ? std::stoi(argv[2]) : 10;
        const int realizations = (argc > 3) ? std::stoi(argv[3]) : 10;
        const int res = (argc > 4) ? std::stoi(argv[4]) : 5;
        const double p_min = (argc > 5) ? std::stod(argv[5]) : 0.0;
        const double p_max = (argc > 6) ? std::stod(argv[6]) : 1.0;
        const int circ_type = (argc > 7) ? std::stoi(argv[7]) : 0;
        bool all_cycles = false;
        std::string out;
        bool explicit_out = false;
        if (argc > 8)
        {
            const std::string_view a8(argv[8]);
            if (is_bool01(a8))
            {
                all_cycles = parse_bool01(a8, "all_cycles");
                if (argc > 9)
                {
                    out = argv[9];
                    explicit_out = true;
                }
            }
            else
            {
                out = argv[8];
                explicit_out = true;
                if (argc > 9) all_cycles = parse_bool01(argv[9], "all_cycles");
            }
        }
        circuit_info(circ_type);
        const int order = entropy_order();
        if (!explicit_out) out = default_output_path(n, realizations, res, p_min, p_max, circ_type, all_cycles, order);
        run(n, periods, realizations, res, p_min, p_max, circ_type, all_cycles, out, order);
        return 0;
    }
    catch (const std::exception &e)
    {
        std::cerr << "\nerror: " << e.what() << '\n';
        return 1;
    }
}
