// Test driver for the drop-in executables' rho3.bin writer and reader
// (mipt_gb300/apps/cli_common.hpp: Rho3Writer, Rho3Reader). Built and run by
// tests/test_cli_cpu.py against files the reference's DensityMatrixWriter
// wrote (tests/golden/ref_fixtures.npz).
//
//   rho3_io write <out.bin> <spec.txt>   write the file a spec describes
//   rho3_io read  <in.bin>               print metadata and records as a spec
//
// spec: spatial total kept periods realizations resolution grid_x grid_y
//       subsystems records p_min p_max, the subsystem qubits, then per record
//       p_index realization p and the payload values; doubles in hex-float.
#include "cli_common.hpp"

#include <cstdio>
#include <cstdlib>

namespace
{
double hexd(std::FILE *f)
{
    char buf[64];
    if (std::fscanf(f, "%63s", buf) != 1) throw std::runtime_error("spec ended early");
    return std::strtod(buf, nullptr);
}

unsigned long long u(std::FILE *f)
{
    unsigned long long v = 0;
    if (std::fscanf(f, "%llu", &v) != 1) throw std::runtime_error("spec ended early");
    return v;
}
} // namespace

int main(int argc, char **argv)
{
    try
    {
        if (argc == 4 && std::string(argv[1]) == "write")
        {
            std::FILE *f = std::fopen(argv[3], "r");
            if (!f) throw std::runtime_error("cannot open spec");
            mgcli::Rho3Metadata m;
            m.spatial_dimension = static_cast<std::uint32_t>(u(f));
            m.total_qubits = static_cast<std::uint32_t>(u(f));
            m.kept_qubits = static_cast<std::uint32_t>(u(f));
            m.matrix_dimension = 1u << m.kept_qubits;
            m.periods = static_cast<std::uint32_t>(u(f));
            m.realizations = static_cast<std::uint32_t>(u(f));
            m.resolution = static_cast<std::uint32_t>(u(f));
            m.grid_x = static_cast<std::uint32_t>(u(f));
            m.grid_y = static_cast<std::uint32_t>(u(f));
            const unsigned long long subsystems = u(f);
            m.record_count = u(f);
            m.p_min = hexd(f);
            m.p_max = hexd(f);
            for (unsigned long long i = 0; i < subsystems * m.kept_qubits; ++i)
                m.subsystem_qubits.push_back(static_cast<std::uint32_t>(u(f)));
            mgcli::Rho3Writer w(argv[2], m);
            std::vector<double> payload(w.values_per_record());
            for (std::uint64_t r = 0; r < m.record_count; ++r)
            {
                const auto pi = static_cast<std::uint32_t>(u(f));
                const auto re = static_cast<std::uint32_t>(u(f));
                const double p = hexd(f);
                for (auto &v : payload) v = hexd(f);
                w.write_record(pi, re, p, payload.data());
            }
            w.close();
            std::fclose(f);
            return 0;
        }
        if (argc == 3 && std::string(argv[1]) == "read")
        {
            mgcli::Rho3Reader rd(argv[2]);
            const auto &m = rd.metadata();
            std::printf("%u %u %u %u %u %u %u %u %u %llu %a %a\n", m.spatial_dimension, m.total_qubits, m.kept_qubits,
                        m.periods, m.realizations, m.resolution, m.grid_x, m.grid_y, rd.subsystem_count(),
                        static_cast<unsigned long long>(m.record_count), m.p_min, m.p_max);
            for (std::uint32_t q : m.subsystem_qubits) std::printf("%u ", q);
            std::printf("\n");
            mgcli::Rho3Record rec;
            while (rd.read_record(rec))
            {
                std::printf("%u %u %a", rec.p_index, rec.realization, rec.p);
                for (double v : rec.rho_ri) std::printf(" %a", v);
                std::printf("\n");
            }
            return 0;
        }
        std::fprintf(stderr, "usage: rho3_io write <out.bin> <spec.txt> | read <in.bin>\n");
        return 2;
    }
    catch (const std::exception &e)
    {
        std::fprintf(stderr, "rho3_io: %s\n", e.what());
        return 1;
    }
}
