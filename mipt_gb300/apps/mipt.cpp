// mipt.exe -- drop-in for the reference's rho3 producer on the GB300 path.
//
//   mipt.exe [d = 1] [n = 10] [periods = 10] [realizations = 10] [resolution = 5]
//            [p_min = 0.0] [p_max = 1.0] [circ_type = 0]
//
// Same run parameters, defaults, validation messages, exit codes and output
// files as cpp/apps/mipt.cpp:312-414 of the reference: info.csv
// (cpp/apps/mipt.cpp:91-97) and rho3.bin (version-2 density-matrix file,
// cpp/include/mipt/density.hpp), one record per trajectory holding the n
// cyclic three-site RDMs {s, s+1, s+2} (cpp/include/mipt/rdm.hpp:92-106).
// Trajectories run in device batches through mipt_gb300_batch_*; circ_type 1
// (Haar brickwork, periodic) is the gate set on this path.
//
// Environment: MIPT_GB300_SEED (master seed; trajectory (p_index, r) uses
// mipt_gb300_trajectory_seed(seed, p_index * realizations + r)),
// MIPT_GB300_FP64=1 (FP64 state vectors; default FP32), MIPT_GB300_BATCH
// (trajectories per launch), MIPT_PAUSE_FILE (host pause sentinel).
#include "cli_common.hpp"

#include <algorithm>
#include <cmath>
#include <iomanip>

namespace
{
using namespace mgcli;

class RateTracker
{
  public:
    void observe(int done, double seconds_per_circuit)
    {
        if (samples_ == 0 || done == 0)
            spc_ = seconds_per_circuit;
        else
            spc_ = (spc_ * samples_ + seconds_per_circuit) / (samples_ + 1);
        ++samples_;
    }
    double rate() const { return spc_ > 0.0 ? 1.0 / spc_ : 0.0; }
    double eta(int completed, int total) const { return std::max(0, total - completed) * spc_; }

  private:
    double spc_ = 0.0;
    int samples_ = 0;
};

void run_1d(int n, int periods, int realizations, int res, double p_min, double p_max, int circ_type)
{
    if (n < 3) throw std::invalid_argument("Saving three-qubit reduced density matrices requires n >= 3.");
    validate_circuit_site_count(circ_type, n);
    require_gb300_circuit(circ_type);
    const bool fermion_trace = circuit_info(circ_type).fermionic_trace;
    const bool fp64 = use_fp64();
    const std::vector<double> ps = linspace(p_min, p_max, res);

    std::ofstream info("info.csv");
    info << "n,periods,realizations,resolution,p_min,p_max,circ_type,circuit_name,fermion_trace,cudaq_backend\n";
    info << n << "," << periods << "," << realizations << "," << res << "," << p_min << "," << p_max << ","
         << circ_type << "," << circuit_info(circ_type).name << "," << (fermion_trace ? 1 : 0) << ","
         << (fp64 ? "gb300-fp64" : "gb300-fp32") << "\n";
    info.close();

    Rho3Metadata meta;
    meta.spatial_dimension = 1;
    meta.total_qubits = static_cast<std::uint32_t>(n);
    meta.periods = static_cast<std::uint32_t>(periods);
    meta.realizations = static_cast<std::uint32_t>(realizations);
    meta.resolution = static_cast<std::uint32_t>(res);
    meta.grid_x = static_cast<std::uint32_t>(n);
    meta.grid_y = 1;
    meta.record_count = static_cast<std::uint64_t>(realizations) * static_cast<std::uint64_t>(res);
    meta.p_min = p_min;
    meta.p_max = p_max;
    for (int s = 0; s < n; ++s)
        for (int k = 0; k < 3; ++k) meta.subsystem_qubits.push_back(static_cast<std::uint32_t>((s + k) % n));
    Rho3Writer rho3_file("rho3.bin", meta);

    if (periods == 0)
    {
        // No layers: every trajectory stays |0...0>, whose three-site blocks
        // are |000><000|.
        std::vector<double> payload(rho3_file.values_per_record(), 0.0);
        for (int s = 0; s < n; ++s) payload[static_cast<std::size_t>(s) * 128] = 1.0;
        for (std::size_t pi = 0; pi < ps.size(); ++pi)
            for (int r = 0; r < realizations; ++r)
                rho3_file.write_record(static_cast<std::uint32_t>(pi), static_cast<std::uint32_t>(r), ps[pi],
                                       payload.data());
        rho3_file.close();
        std::cout << "Saved " << n << " cyclic three-qubit reduced density matrices per trajectory to rho3.bin.\n";
        return;
    }
    const int capacity = batch_capacity(n, fp64, realizations);
    mipt_gb300_batch_config cfg{};
    cfg.n_qubits = n;
    cfg.periods = periods;
    cfg.closed = 1;
    cfg.fp64 = fp64 ? 1 : 0;
    cfg.chunk_bits = 16;
    cfg.rho3 = 1;
    cfg.fermion_trace = fermion_trace ? 1 : 0;
    configure_circuit(cfg, circ_type);
    Batch batch(cfg, capacity);
    const std::uint64_t seed = master_seed();
    std::cout << "GB300 path: " << mipt_gb300_version() << ", " << (fp64 ? "FP64" : "FP32")
              << " state vectors, " << capacity << " trajectories per launch, MIPT_GB300_SEED=" << seed << "\n";

    std::vector<std::uint64_t> seeds(static_cast<std::size_t>(capacity));
    std::vector<double> pv(static_cast<std::size_t>(capacity));
    std::vector<double> rho3(static_cast<std::size_t>(capacity) * n * 128);
    PauseSentinel pause;
    for (std::size_t pi = 0; pi < ps.size(); ++pi)
    {
        const double p = ps[pi];
        std::cout << "Simulating p = " << p << "...\n " << std::flush;
        RateTracker rate;
        for (int r0 = 0; r0 < realizations; r0 += capacity)
        {
            pause.wait([&] { rho3_file.flush(); });
            const int count = std::min(capacity, realizations - r0);
            const auto t0 = std::chrono::steady_clock::now();
            for (int i = 0; i < count; ++i)
            {
                seeds[i] = mipt_gb300_trajectory_seed(seed, pi * static_cast<std::uint64_t>(realizations) + r0 + i);
                pv[i] = p;
            }
            check(mipt_gb300_batch_run_haar(batch.get(), seeds.data(), pv.data(), count, nullptr, nullptr, nullptr,
                                            nullptr, nullptr, rho3.data()),
                  "mipt_gb300_batch_run_haar");
            for (int i = 0; i < count; ++i)
                rho3_file.write_record(static_cast<std::uint32_t>(pi), static_cast<std::uint32_t>(r0 + i), p,
                                       rho3.data() + static_cast<std::size_t>(i) * n * 128);
            const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            rate.observe(r0, secs / count);
            std::cout << "\rAverage circuits/second: " << std::round(rate.rate() * 100.0) / 100.0
                      << ", Realisations ETA: " << static_cast<int>(rate.eta(r0 + count, realizations))
                      << "s               " << std::flush;
        }
        std::cout << "\n";
    }
    rho3_file.close();
    std::cout << "Saved " << n << " cyclic three-qubit reduced density matrices per trajectory to rho3.bin for circ_type "
              << circ_type << " (" << circuit_info(circ_type).name << ")"
              << (fermion_trace ? " using fermionic partial traces.\n" : ".\n");
}

void print_usage(const char *argv0)
{
    std::cout << "Usage: " << argv0
              << " [d = 1] [n = 10] [periods = 10] [realizations = 10] [resolution = 5] [p_min = 0.0] [p_max = 1.0] "
                 "[circ_type = 0]\n";
    std::cout << "Description:\n";
    std::cout << "  d = dimensionality (1 or 2)\n";
    std::cout << "  n = number of qubits per dimension; for d=2 this means an n x n lattice\n";
    std::cout << "  periods = number of brickwork periods (1D period = even layer + odd layer)\n";
    std::cout << "  realizations = number of realizations per p value\n";
    std::cout << "  resolution = number of p grid points\n";
    std::cout << "  p_min = minimum measurement rate\n";
    std::cout << "  p_max = maximum measurement rate\n";
    std::cout << "  circ_type:\n";
    print_circuit_type_help(std::cout, "    ");
    std::cout << "  On the GB300 path circ_type=1 (Haar brickwork), 2 (FermionRPPU) and 4 (qRPPU) run; d=2 is not on\n"
                 "  this path.\n";
}

int run_cli(int argc, char *argv[])
{
    if (argc > 1 && (std::strcmp(argv[1], "--help") == 0 || std::strcmp(argv[1], "-h") == 0))
    {
        print_usage(argv[0]);
        return 0;
    }
    if (argc > 9)
    {
        std::cerr << "Too many arguments. Use --help for usage.\n";
        return 2;
    }
    const int d = (argc > 1) ? std::stoi(argv[1]) : 1;
    const int n = (argc > 2) ? std::stoi(argv[2]) : ((d == 1) ? 10 : 4);
    const int periods = (argc > 3) ? std::stoi(argv[3]) : ((d == 1) ? 10 : 32);
    const int realizations = (argc > 4) ? std::stoi(argv[4]) : 10;
    const int res = (argc > 5) ? std::stoi(argv[5]) : 5;
    const double p_min = (argc > 6) ? std::stod(argv[6]) : 0.0;
    const double p_max = (argc > 7) ? std::stod(argv[7]) : 1.0;
    const int circ_type = (argc > 8) ? std::stoi(argv[8]) : 0;
    circuit_info(circ_type);

    if (n <= 0) throw std::invalid_argument("n must be positive.");
    if (d != 1 && d != 2) throw std::invalid_argument("d must be 1 or 2.");
    if (res <= 0) throw std::invalid_argument("resolution must be positive.");
    if (realizations <= 0) throw std::invalid_argument("realizations must be positive.");
    if (periods < 0) throw std::invalid_argument("periods must be non-negative.");
    if (p_min < 0.0 || p_max > 1.0 || p_min > p_max) throw std::invalid_argument("Require 0 <= p_min <= p_max <= 1.");

    const auto start = std::chrono::steady_clock::now();
    if (d == 1)
    {
        std::cout << "Running 1D " << n << "-qubit circ_type " << circ_type << " (" << circuit_info(circ_type).name
                  << ") simulation of " << realizations * res << " circuits.\n";
        run_1d(n, periods, realizations, res, p_min, p_max, circ_type);
    }
    else
    {
        throw std::invalid_argument("d=2 runs the reference's MMS gate set, which is not on the GB300 path.");
    }
    const std::chrono::duration<double> elapsed = std::chrono::steady_clock::now() - start;
    std::cout << "Elapsed time: " << elapsed.count() << "s\n";
    return 0;
}
} // namespace

int main(int argc, char *argv[])
{
    try
    {
        return run_cli(argc, argv);
    }
    catch (const std::exception &error)
    {
        std::cerr << "mipt.exe error: " << error.what() << '\n';
        return 1;
    }
}
