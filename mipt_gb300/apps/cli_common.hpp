// Shared host code of the drop-in executables (mipt.exe, sim_tmi.exe): the
// reference's run-parameter conventions, output formats and host controls,
// driving the GB300 path through the C ABI of libmipt_gb300.so only.
//
// Reference behaviour kept (paths inside the reference project):
//   linspace grid (last point pinned to p_max)     cpp/include/mipt/types.hpp:24-38
//   circuit-type table (names, tags, help, parity) cpp/include/mipt/types.hpp:155-243
//   even-site check for brickwork circuits         cpp/include/mipt/types.hpp:417-431
//   17-significant-digit CSV numbers               cpp/include/mipt/tmi/linalg.hpp:223-234
//   host pause sentinel (PAUSE_MIPT)               cpp/include/mipt/util/pause.hpp
//   rho3.bin version-2 writer and reader           cpp/include/mipt/density.hpp:12-345
#pragma once

#include "mipt_gb300.h"

#include <charconv>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <random>
#include <stdexcept>
#include <string>
#include <string_view>
#include <thread>
#include <vector>

namespace mgcli
{

// ------------------------------------------------------------ circuits
struct CircuitInfo
{
    const char *name;
    const char *tag;
    const char *help;
    bool fermionic_trace;
    bool requires_even_sites;
};

inline constexpr CircuitInfo kCircuits[5] = {
    {"MMS", "mms", "MMS gate set", false, false},
    {"Random Haar Unitary", "haar", "random Haar U(4) brickwork circuit", false, true},
    {"Fermionic Random Parity Preserving Unitary", "rppu", "fermionic RPPU with fermionic partial tracing", true,
     true},
    {"RFGS", "rfgs", "fermionic reduced gate set with fermionic partial tracing", true, true},
    {"qRPPU (qubit parity-preserving unitary)", "qrppu", "qRPPU without JW/CZ chains, using qubit partial tracing",
     false, true},
};
constexpr int kHaar = 1;

inline const CircuitInfo &circuit_info(int type)
{
    if (type < 0 || type >= 5) throw std::invalid_argument("circ_type must be one of 0, 1, 2, 3, 4.");
    return kCircuits[type];
}

inline void print_circuit_type_help(std::ostream &out, const char *indent)
{
    for (int i = 0; i < 5; ++i) out << indent << i << " = " << kCircuits[i].help << '\n';
}

// The GB300 path runs the Haar brickwork and the parity-preserving RPPU /
// qRPPU gate sets; MMS and RFGS stay with the reference.
inline bool on_gb300_path(int type) { return type == kHaar || type == 2 || type == 4; }

inline void require_gb300_circuit(int type)
{
    const CircuitInfo &c = circuit_info(type);
    if (!on_gb300_path(type))
        throw std::invalid_argument(std::string("circ_type ") + std::to_string(type) + " (" + c.name +
                                    ") is not on the GB300 trajectory path; use circ_type=1 (" +
                                    kCircuits[kHaar].name + "), 2 (" + kCircuits[2].name + ") or 4 (" +
                                    kCircuits[4].name + ").");
}

inline bool env_bool_flag(const char *name, bool fallback);

// Gate set, partial-trace convention and, for the RPPU sets, the measurement
// chunking of the reference's parity-sector engine (site n-1 on its own;
// MIPT_CUSV_PARITY=0 selects the plain chunking, as in the reference).
inline void configure_circuit(mipt_gb300_batch_config &cfg, int type)
{
    cfg.circuit = type == kHaar ? 0 : type;
    cfg.fermion_trace = circuit_info(type).fermionic_trace ? 1 : 0;
    cfg.split_last = (type == 2 || type == 4) && env_bool_flag("MIPT_CUSV_PARITY", true) ? 1 : 0;
}

inline void validate_circuit_site_count(int type, int sites, const char *site_name = "n")
{
    const CircuitInfo &c = circuit_info(type);
    if (c.requires_even_sites && sites % 2 != 0)
        throw std::invalid_argument(std::string(c.name) + " requires an even " + site_name +
                                    " for periodic brickwork geometry.");
}

// --------------------------------------------------------------- numbers
inline std::vector<double> linspace(double first, double last, int count)
{
    if (count <= 0) return {};
    if (count == 1) return {first};
    std::vector<double> v(static_cast<std::size_t>(count));
    const double step = (last - first) / static_cast<double>(count - 1);
    for (int i = 0; i < count; ++i) v[static_cast<std::size_t>(i)] = first + step * static_cast<double>(i);
    v.back() = last;
    return v;
}

inline void append_double(std::string &s, double value)
{
    char buf[64];
    const auto r = std::to_chars(buf, buf + sizeof(buf), value, std::chars_format::general, 17);
    if (r.ec == std::errc{})
        s.append(buf, r.ptr);
    else
        s += std::to_string(value);
}

// ------------------------------------------------------------ environment
inline bool env_falsey_path(const char *v)
{
    if (!v) return false;
    std::string t(v);
    for (auto &c : t) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return t == "0" || t == "false" || t == "off" || t == "no" || t == "none" || t == "disabled";
}

inline bool env_bool_flag(const char *name, bool fallback)
{
    const char *v = std::getenv(name);
    if (!v) return fallback;
    std::string t(v);
    for (auto &c : t) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    if (t == "1" || t == "true" || t == "yes" || t == "on") return true;
    if (t == "0" || t == "false" || t == "no" || t == "off") return false;
    return fallback;
}

inline long env_long(const char *name, long fallback)
{
    const char *v = std::getenv(name);
    if (!v || !*v) return fallback;
    return std::stol(v);
}

// Trajectory seeds: splitmix64-derived per (p index, realization) from one
// master seed, MIPT_GB300_SEED when set, otherwise drawn from the OS.
inline std::uint64_t master_seed()
{
    const char *v = std::getenv("MIPT_GB300_SEED");
    if (v && *v) return std::stoull(v, nullptr, 0);
    std::random_device rd;
    return (static_cast<std::uint64_t>(rd()) << 32) ^ rd();
}

inline bool use_fp64() { return env_long("MIPT_GB300_FP64", 0) != 0; }

// Trajectories per device launch: MIPT_GB300_BATCH, else as many FP32/FP64
// states as fit in 32 GiB (at most 1024, at most what the run needs).
inline int batch_capacity(int n, bool fp64, int needed)
{
    long cap = env_long("MIPT_GB300_BATCH", 0);
    if (cap <= 0)
    {
        const double state = static_cast<double>(1ull << n) * (fp64 ? 16.0 : 8.0);
        cap = static_cast<long>(std::max(1.0, std::min(1024.0, 34359738368.0 / state)));
    }
    return static_cast<int>(std::max(1L, std::min<long>(cap, needed)));
}

// ---------------------------------------------------------------- pause
class PauseSentinel
{
  public:
    explicit PauseSentinel(const char *legacy_env = nullptr)
    {
        for (const char *name : {legacy_env, "MIPT_PAUSE_FILE"})
        {
            if (!name) continue;
            const char *v = std::getenv(name);
            if (env_falsey_path(v))
            {
                path_.clear();
                return;
            }
            if (v && *v)
            {
                path_ = v;
                return;
            }
        }
        path_ = "PAUSE_MIPT";
    }
    std::string describe() const
    {
        return path_.empty() ? std::string("host_pause_control=disabled")
                             : "host_pause_file=" + path_ + " (create it to pause, remove it to resume)";
    }
    double paused_seconds() const { return paused_; }
    template <typename Flush> double wait(Flush flush)
    {
        std::error_code ec;
        if (path_.empty() || !std::filesystem::exists(path_, ec)) return 0.0;
        flush();
        const auto t0 = std::chrono::steady_clock::now();
        std::cerr << "\nPAUSED by host sentinel " << path_ << "; remove it to resume.\n";
        while (std::filesystem::exists(path_, ec)) std::this_thread::sleep_for(std::chrono::seconds(1));
        const double d = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        paused_ += d;
        std::cerr << "RESUMED after " << d << "s.\n";
        return d;
    }

  private:
    std::string path_;
    double paused_ = 0.0;
};

// ------------------------------------------------------------ C ABI glue
inline void check(int rc, const char *what)
{
    if (rc != 0)
        throw std::runtime_error(std::string(what) + " failed (status " + std::to_string(rc) +
                                 "): " + mipt_gb300_last_error());
}

class Batch
{
  public:
    Batch(const mipt_gb300_batch_config &cfg, int capacity)
    {
        check(mipt_gb300_batch_create(&cfg, capacity, &b_), "mipt_gb300_batch_create");
    }
    ~Batch()
    {
        if (b_) mipt_gb300_batch_destroy(b_);
    }
    Batch(const Batch &) = delete;
    Batch &operator=(const Batch &) = delete;
    mipt_gb300_batch *get() const { return b_; }

  private:
    mipt_gb300_batch *b_ = nullptr;
};

// --------------------------------------------------------------- rho3.bin
// Version-2 density-matrix file: magic "MIPTRHO2", u32 0x01020304, u32 2,
// u32 x 10 header, u64 record count, f64 p_min, f64 p_max, u32 subsystem
// qubits; then per record u32 p_index, u32 realization, f64 p and the
// payload (subsystem-major, row-major re/im of each D x D matrix).
struct Rho3Metadata
{
    std::uint32_t spatial_dimension = 1, total_qubits = 0, kept_qubits = 3, matrix_dimension = 8;
    std::uint32_t periods = 0, realizations = 0, resolution = 0, grid_x = 0, grid_y = 1;
    std::uint64_t record_count = 0;
    double p_min = 0.0, p_max = 0.0;
    std::vector<std::uint32_t> subsystem_qubits; // [subsystem][kept]
};

class Rho3Writer
{
  public:
    Rho3Writer(const std::string &path, const Rho3Metadata &m) : m_(m), out_(path, std::ios::binary | std::ios::trunc)
    {
        if (!out_) throw std::runtime_error("Could not create density-matrix file: " + path);
        if (m.kept_qubits == 0 || m.kept_qubits >= 31 || m.matrix_dimension != (1u << m.kept_qubits) ||
            m.subsystem_qubits.empty() || m.subsystem_qubits.size() % m.kept_qubits != 0)
            throw std::invalid_argument("Inconsistent density-matrix metadata.");
        subsystems_ = static_cast<std::uint32_t>(m.subsystem_qubits.size() / m.kept_qubits);
        values_ = static_cast<std::size_t>(subsystems_) * 2u * m.matrix_dimension * m.matrix_dimension;
        out_.write("MIPTRHO2", 8);
        put(std::uint32_t{0x01020304u});
        put(std::uint32_t{2u});
        for (std::uint32_t v : {m.spatial_dimension, m.total_qubits, m.kept_qubits, m.matrix_dimension, m.periods,
                                m.realizations, m.resolution, m.grid_x, m.grid_y, subsystems_})
            put(v);
        put(m.record_count);
        put(m.p_min);
        put(m.p_max);
        out_.write(reinterpret_cast<const char *>(m.subsystem_qubits.data()),
                   static_cast<std::streamsize>(m.subsystem_qubits.size() * sizeof(std::uint32_t)));
        if (!out_) throw std::runtime_error("Failed while writing subsystem-qubit metadata.");
    }
    std::size_t values_per_record() const { return values_; }
    void write_record(std::uint32_t p_index, std::uint32_t realization, double p, const double *payload)
    {
        if (written_ >= m_.record_count) throw std::runtime_error("Attempted to write too many density-matrix records.");
        put(p_index);
        put(realization);
        put(p);
        out_.write(reinterpret_cast<const char *>(payload), static_cast<std::streamsize>(values_ * sizeof(double)));
        if (!out_) throw std::runtime_error("Failed while writing density-matrix payload.");
        ++written_;
    }
    void flush() { out_.flush(); }
    void close()
    {
        if (written_ != m_.record_count)
            throw std::runtime_error("Density-matrix file closed before all records were written.");
        out_.flush();
        out_.close();
    }

  private:
    template <typename T> void put(const T &v) { out_.write(reinterpret_cast<const char *>(&v), sizeof(T)); }
    Rho3Metadata m_;
    std::ofstream out_;
    std::uint32_t subsystems_ = 0;
    std::size_t values_ = 0;
    std::uint64_t written_ = 0;
};

// rho3.bin version-2 reader (the layout Rho3Writer writes; the reference's
// DensityMatrixReader, cpp/include/mipt/density.hpp:253-345, with its checks).
struct Rho3Record
{
    std::uint32_t p_index = 0, realization = 0;
    double p = 0.0;
    std::vector<double> rho_ri; // [subsystem][D][D][re, im]
};

class Rho3Reader
{
  public:
    explicit Rho3Reader(const std::string &path) : in_(path, std::ios::binary)
    {
        if (!in_) throw std::runtime_error("Could not open density-matrix file: " + path);
        char magic[8]{};
        in_.read(magic, 8);
        if (!in_) throw std::runtime_error("Could not read density-matrix file header.");
        if (std::memcmp(magic, "MIPTRHO2", 8) != 0) throw std::runtime_error("Not a version-2 MIPT density-matrix file.");
        std::uint32_t endian = 0, version = 0, subsystems = 0;
        get(endian);
        get(version);
        if (endian != 0x01020304u) throw std::runtime_error("Density-matrix file endianness is not supported on this host.");
        if (version != 2u) throw std::runtime_error("Unsupported density-matrix file version.");
        for (std::uint32_t *v : {&m_.spatial_dimension, &m_.total_qubits, &m_.kept_qubits, &m_.matrix_dimension,
                                 &m_.periods, &m_.realizations, &m_.resolution, &m_.grid_x, &m_.grid_y, &subsystems})
            get(*v);
        get(m_.record_count);
        get(m_.p_min);
        get(m_.p_max);
        if (m_.kept_qubits == 0 || m_.kept_qubits >= 31 || m_.matrix_dimension != (1u << m_.kept_qubits) ||
            subsystems == 0)
            throw std::runtime_error("Inconsistent density-matrix metadata.");
        m_.subsystem_qubits.resize(static_cast<std::size_t>(subsystems) * m_.kept_qubits);
        in_.read(reinterpret_cast<char *>(m_.subsystem_qubits.data()),
                 static_cast<std::streamsize>(m_.subsystem_qubits.size() * sizeof(std::uint32_t)));
        if (!in_) throw std::runtime_error("Density-matrix subsystem metadata is incomplete.");
        values_ = static_cast<std::size_t>(subsystems) * 2u * m_.matrix_dimension * m_.matrix_dimension;
    }
    const Rho3Metadata &metadata() const { return m_; }
    std::uint32_t subsystem_count() const
    {
        return static_cast<std::uint32_t>(m_.subsystem_qubits.size() / m_.kept_qubits);
    }
    bool read_record(Rho3Record &r)
    {
        if (read_ >= m_.record_count) return false;
        get(r.p_index);
        get(r.realization);
        get(r.p);
        r.rho_ri.resize(values_);
        in_.read(reinterpret_cast<char *>(r.rho_ri.data()), static_cast<std::streamsize>(values_ * sizeof(double)));
        if (!in_) throw std::runtime_error("Density-matrix record payload is incomplete.");
        ++read_;
        return true;
    }

  private:
    template <typename T> void get(T &v)
    {
        in_.read(reinterpret_cast<char *>(&v), sizeof(T));
        if (!in_) throw std::runtime_error("Density-matrix file is truncated.");
    }
    std::ifstream in_;
    Rho3Metadata m_;
    std::size_t values_ = 0;
    std::uint64_t read_ = 0;
};

} // namespace mgcli
