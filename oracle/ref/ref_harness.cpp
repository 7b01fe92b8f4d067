// Parity harness: the reference's own host code, compiled from its headers in
// place (see oracle/ref/build_ref.sh), behind a small C ABI that the fixture
// generator (tests/golden/make_golden.py) calls through ctypes.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product links or loads this; it
// exists to pin the CPU oracle (oracle/oracle.cpp) and the product's host
// sampler to the reference's actual outputs.
//
// Reference functions exercised here (paths inside the reference project):
//   seeding::splitmix64 / trajectory_seed      cpp/include/mipt/types.hpp:262-273
//   Circuit1D::seed (seed_seq of the two halves, measurement stream from
//   splitmix64(seed ^ 0xa0761d0d))              cpp/include/mipt/circuit.hpp:129-140
//   build_haar_layers / fill_haar_layer         cpp/include/mipt/circuits/haar.hpp:226-305
//   haar_unitary_4                              cpp/include/mipt/circuits/haar.hpp:39-85
//   build_haar_layer_ops / haar_bond_matrix     cpp/include/mipt/cusv/gates.hpp:139-193
//   Engine::measure_layer's uniform draws       cpp/include/mipt/cusv/engine.hpp:300-327
//   measure_collapse_host                       cpp/include/mipt/free_energy_measure.hpp:18-96
//   reduced_density_manual_from_state           cpp/include/mipt/tmi/linalg.hpp:1098-1142
//   entropy_hermitian_inplace (Jacobi path)     cpp/include/mipt/tmi/linalg.hpp:524-583
//   reduced_density_complex_from_host_statevector cpp/include/mipt/rdm.hpp:149-305
//   random_product_amplitudes / random_haar_amplitudes
//                                               cpp/include/mipt/free_energy.hpp:125-222
//   CircuitWorkspace1D::seed (restated below: the class itself needs a live
//   CUDA-Q runtime)                             cpp/include/mipt/probed.hpp:103-108
//   DensityMatrixWriter (rho3.bin version 2)   cpp/include/mipt/density.hpp:134-251
//   entropy.exe's checkpoint reader            cpp/include/mipt/entropy_resume.hpp:102-246
//   sim_tmi.exe's checkpoint reader            cpp/include/mipt/tmi/resume.hpp:188-330
//   free_energy.exe's checkpoint readers (scan_samples, load_timeseries)
//                                               cpp/include/mipt/free_energy_resume.hpp:246-534
//   build_rppu_layers_with_boundary / fill_rppu_layer, build_rppu_layer_ops
//                                               cpp/include/mipt/circuits/rppu_layer.hpp:167-285,
//                                               cpp/include/mipt/cusv/gates.hpp:219-281
#include "mipt/circuits/haar.hpp"
#include "mipt/circuits/rppu_layer.hpp"
#include "mipt/density.hpp"
#include "mipt/entropy_resume.hpp"
#include "mipt/tmi/resume.hpp"
#include "mipt/free_energy.hpp"
#include "mipt/free_energy_resume.hpp"
#include "mipt/cusv/gates.hpp"
#include "mipt/free_energy_measure.hpp"
#include "mipt/rdm.hpp"
#include "mipt/tmi/linalg.hpp"
#include "mipt/types.hpp"

#include <complex>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

using C64 = std::complex<double>;

namespace
{
// Same construction as Circuit1D::seed: the layer stream is seeded with the
// 32-bit halves of the trajectory seed, the measurement stream with the halves
// of splitmix64(seed ^ 0xa0761d0d).
void seed_streams(std::uint64_t value, std::mt19937 &layer_rng, std::mt19937 &measure_rng)
{
    std::seed_seq sequence{static_cast<std::uint32_t>(value & 0xffffffffu),
                           static_cast<std::uint32_t>(value >> 32)};
    layer_rng.seed(sequence);
    const std::uint64_t m = mipt::seeding::splitmix64(value ^ 0xa0761d0dull);
    std::seed_seq measure_sequence{static_cast<std::uint32_t>(m & 0xffffffffu),
                                   static_cast<std::uint32_t>(m >> 32)};
    measure_rng.seed(measure_sequence);
}

std::vector<C64> unpack(const double *ri, std::size_t count)
{
    std::vector<C64> out(count);
    for (std::size_t i = 0; i < count; ++i) out[i] = C64(ri[2 * i], ri[2 * i + 1]);
    return out;
}
} // namespace

extern "C" {

std::uint64_t ref_splitmix64(std::uint64_t v) { return mipt::seeding::splitmix64(v); }

std::uint64_t ref_trajectory_seed(std::uint64_t master, std::uint64_t index)
{
    return mipt::seeding::trajectory_seed(master, index);
}

// One Haar trajectory drawn exactly as HaarCircuit1D::simulate draws it, with
// the measurement uniforms the cuStateVec engine would consume.
//   gates_per_layer[2*periods]
//   gate_q[layer][max_gates][2]          (q0, q1)
//   gate_m[layer][max_gates][32]         row-major 4x4 complex (re, im)
//   sites_per_layer[2*periods], sites[layer][n]
//   uniforms[...] one per measured chunk of <= chunk_bits sites, in order
int ref_haar_draw(std::uint64_t seed, int n, int periods, double p, int closed, int chunk_bits,
                  int *gates_per_layer, int *gate_q, double *gate_m, int *sites_per_layer,
                  int *sites, double *uniforms, int *n_uniforms)
{
    try
    {
        std::mt19937 layer_rng, measure_rng;
        seed_streams(seed, layer_rng, measure_rng);
        std::vector<mipt::HaarLayer> layers;
        mipt::build_haar_layers(layers, n, periods, p, layer_rng, closed != 0);
        const int max_gates = n / 2;
        int u = 0;
        for (std::size_t l = 0; l < layers.size(); ++l)
        {
            const auto ops = mipt::cusv::build_haar_layer_ops(layers[l], n);
            gates_per_layer[l] = static_cast<int>(ops.ops.size());
            for (std::size_t g = 0; g < ops.ops.size(); ++g)
            {
                const auto &op = ops.ops[g];
                gate_q[(l * max_gates + g) * 2 + 0] = op.targets[0];
                gate_q[(l * max_gates + g) * 2 + 1] = op.targets[1];
                for (int e = 0; e < 16; ++e)
                {
                    gate_m[(l * max_gates + g) * 32 + 2 * e + 0] = op.matrix.values[e].real();
                    gate_m[(l * max_gates + g) * 32 + 2 * e + 1] = op.matrix.values[e].imag();
                }
            }
            sites_per_layer[l] = static_cast<int>(ops.measure_sites.size());
            for (std::size_t s = 0; s < ops.measure_sites.size(); ++s)
                sites[l * n + s] = ops.measure_sites[s];
            // Engine::measure_layer: one U(0,1) per chunk, none for an empty layer.
            std::uniform_real_distribution<double> uniform(0.0, 1.0);
            for (std::size_t b = 0; b < ops.measure_sites.size(); b += static_cast<std::size_t>(chunk_bits))
                uniforms[u++] = uniform(measure_rng);
        }
        *n_uniforms = u;
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// Raw haar_unitary_4 draws from an mt19937 seeded with seed_seq{lo, hi}.
int ref_haar_unitary(std::uint64_t seed, int count, double *out)
{
    std::mt19937 rng, unused;
    seed_streams(seed, rng, unused);
    for (int i = 0; i < count; ++i)
    {
        const auto u = mipt::haar_unitary_4(rng);
        for (int e = 0; e < 16; ++e)
        {
            out[i * 32 + 2 * e] = u[e].real();
            out[i * 32 + 2 * e + 1] = u[e].imag();
        }
    }
    return 0;
}

int ref_measure_collapse(double *psi_ri, int n, int q, double u, int *outcome, double *cond_p,
                         double *surprisal)
{
    try
    {
        auto psi = unpack(psi_ri, std::size_t{1} << n);
        const auto r = mipt::free_energy::measure_collapse_host(psi.data(), n, q, u);
        for (std::size_t i = 0; i < psi.size(); ++i)
        {
            psi_ri[2 * i] = psi[i].real();
            psi_ri[2 * i + 1] = psi[i].imag();
        }
        *outcome = r.outcome;
        *cond_p = r.conditional_probability;
        *surprisal = r.surprisal;
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

int ref_rdm_from_state(const double *psi_ri, int n, const int *kept, int k, int fermion,
                       double *rho_ri)
{
    try
    {
        const auto psi = unpack(psi_ri, std::size_t{1} << n);
        mipt::tmi::StateEntropyWorkspace ws;
        std::vector<C64> out;
        const std::vector<int> modes(kept, kept + k);
        mipt::tmi::reduced_density_manual_from_state(psi.data(), n, modes, fermion != 0, ws, out);
        for (std::size_t i = 0; i < out.size(); ++i)
        {
            rho_ri[2 * i] = out[i].real();
            rho_ri[2 * i + 1] = out[i].imag();
        }
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// Entropy in bits of a row-major (re, im) density matrix; order 1 = von
// Neumann (Jacobi path: no LAPACK is loadable here), order 2 = Renyi-2.
double ref_entropy_hermitian(const double *rho_ri, int dim, int order)
{
    std::vector<C64> a = unpack(rho_ri, static_cast<std::size_t>(dim) * dim);
    mipt::tmi::EntropyWorkspace ws;
    return mipt::tmi::entropy_hermitian_inplace(
        a, static_cast<std::size_t>(dim), ws,
        order == 2 ? mipt::tmi::EntropyOrder::Renyi2 : mipt::tmi::EntropyOrder::VonNeumann);
}

double ref_renyi2_from_purity(double purity) { return mipt::tmi::renyi2_from_purity(purity); }

int ref_rho3_from_state(const double *psi_ri, int n, const int *subs, int count, int fermion,
                        double *out)
{
    try
    {
        const auto psi = unpack(psi_ri, std::size_t{1} << n);
        std::vector<mipt::Subsystem> s(static_cast<std::size_t>(count));
        for (int i = 0; i < count; ++i) s[i] = {subs[3 * i], subs[3 * i + 1], subs[3 * i + 2]};
        mipt::reduced_density_complex_from_host_statevector(psi.data(), n, s, out, fermion != 0);
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// The free-energy protocol's initial state, from the reference's own
// functions (FP64 amplitudes; this build has no MIPT_CUDAQ_PRECISION=32).
int ref_fe_initial_state(std::uint64_t seed, int n, int kind, int fixed_parity, double *out_ri, int *parity)
{
    try
    {
        std::mt19937_64 rng(seed);
        int sector = -1;
        const auto amps = kind == 0
                              ? mipt::free_energy::random_product_amplitudes(n, fixed_parity != 0, sector, rng)
                              : mipt::free_energy::random_haar_amplitudes(n, fixed_parity != 0, sector, rng);
        for (std::size_t i = 0; i < amps.size(); ++i)
        {
            out_ri[2 * i] = amps[i].real();
            out_ri[2 * i + 1] = amps[i].imag();
        }
        *parity = sector;
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// The probed workspace's Haar layers for a 32-bit seed: fill_haar_layer per
// timestep on the layer stream, uniforms from the measurement stream. Layout
// as ref_haar_draw.
int ref_fe_draw(std::uint32_t seed, int n, int layers, double p, int chunk_bits, int *gates_per_layer, int *gate_q,
                double *gate_m, int *sites_per_layer, int *sites, double *uniforms, int *n_uniforms)
{
    try
    {
        std::mt19937 layer_rng, measure_rng;
        layer_rng.seed(seed);
        measure_rng.seed(seed ^ 0x9e3779b9u);
        const int max_gates = n / 2;
        int u = 0;
        for (int l = 0; l < layers; ++l)
        {
            mipt::HaarLayer layer;
            mipt::fill_haar_layer(layer, n, l % 2, p, true, layer_rng);
            const auto ops = mipt::cusv::build_haar_layer_ops(layer, n);
            gates_per_layer[l] = static_cast<int>(ops.ops.size());
            for (std::size_t g = 0; g < ops.ops.size(); ++g)
            {
                const auto &op = ops.ops[g];
                gate_q[(l * max_gates + g) * 2 + 0] = op.targets[0];
                gate_q[(l * max_gates + g) * 2 + 1] = op.targets[1];
                for (int e = 0; e < 16; ++e)
                {
                    gate_m[(l * max_gates + g) * 32 + 2 * e + 0] = op.matrix.values[e].real();
                    gate_m[(l * max_gates + g) * 32 + 2 * e + 1] = op.matrix.values[e].imag();
                }
            }
            sites_per_layer[l] = static_cast<int>(ops.measure_sites.size());
            for (std::size_t s = 0; s < ops.measure_sites.size(); ++s) sites[l * n + s] = ops.measure_sites[s];
            std::uniform_real_distribution<double> uniform(0.0, 1.0);
            for (std::size_t b = 0; b < ops.measure_sites.size(); b += static_cast<std::size_t>(chunk_bits))
                uniforms[u++] = uniform(measure_rng);
        }
        *n_uniforms = u;
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// A rho3.bin written by the reference's DensityMatrixWriter: dims = spatial
// dimension, total qubits, kept qubits, periods, realizations, resolution,
// grid_x, grid_y, subsystem count; records[i] = (p_index, realization) with
// probability ps[i] and payload[i * values ...].
int ref_rho3_write(const char *path, const std::uint32_t *dims, std::uint64_t record_count, double p_min,
                   double p_max, const std::uint32_t *subsystem_qubits, const std::uint32_t *p_index,
                   const std::uint32_t *realization, const double *ps, const double *payload)
{
    try
    {
        mipt::io::DensityFileMetadata m;
        m.spatial_dimension = dims[0];
        m.total_qubits = dims[1];
        m.kept_qubits = dims[2];
        m.matrix_dimension = 1u << dims[2];
        m.periods = dims[3];
        m.realizations = dims[4];
        m.resolution = dims[5];
        m.grid_x = dims[6];
        m.grid_y = dims[7];
        m.subsystem_count = dims[8];
        m.record_count = record_count;
        m.p_min = p_min;
        m.p_max = p_max;
        m.subsystem_qubits.assign(subsystem_qubits, subsystem_qubits + dims[8] * dims[2]);
        mipt::io::DensityMatrixWriter w(path, m);
        const std::size_t values = mipt::io::payload_value_count(m);
        for (std::uint64_t i = 0; i < record_count; ++i)
            w.write_record(p_index[i], realization[i], ps[i], payload + i * values, values);
        w.close();
        return 0;
    }
    catch (...)
    {
        return 1;
    }
}

// sim_tmi.exe's resume decision: out = loaded, name_verified, rows,
// dropped_rows, kept_bytes, start_p_index, start_realization; or 1 with the
// refusal text.
int ref_tmi_resume(const char *output_path, const char *expected_name, int realizations, int cycles,
                   const char *const *p_texts, int p_count, long *out, char *message, int message_len)
{
    try
    {
        std::vector<std::string> texts(p_texts, p_texts + p_count);
        const auto ck = mipt::tmi::resume::load(output_path, expected_name, realizations, cycles, texts);
        out[0] = ck.loaded ? 1 : 0;
        out[1] = ck.name_verified ? 1 : 0;
        out[2] = static_cast<long>(ck.rows);
        out[3] = static_cast<long>(ck.dropped_rows);
        out[4] = static_cast<long>(ck.kept_bytes);
        out[5] = static_cast<long>(ck.start_p_index);
        out[6] = ck.start_realization;
        return 0;
    }
    catch (const std::exception &e)
    {
        std::snprintf(message, static_cast<std::size_t>(message_len), "%s", e.what());
        return 1;
    }
}

// entropy.exe's resume decision for the CSV at `path`: *completed, or 1 with
// the refusal text when the reference refuses it.
int ref_entropy_resume(const char *path, int n, int periods, double p, long requested, int circ_type,
                       int max_s1_block, long *completed, char *message, int message_len)
{
    namespace r = mipt::entropy::resume;
    try
    {
        r::RunIdentity id;
        id.n = n;
        id.periods = periods;
        id.p = p;
        id.requested_realizations = requested;
        id.circ_type = circ_type;
        *completed = r::load(path, id, max_s1_block).completed;
        return 0;
    }
    catch (const std::exception &e)
    {
        std::snprintf(message, static_cast<std::size_t>(message_len), "%s", e.what());
        return 1;
    }
}

// free_energy.exe's resume decision for the two CSVs at `samples_path` /
// `series_path`: out[0] completed samples rows, out[1] time-series aggregate
// count, out[2] valid bytes of the samples file; *master the recovered master
// seed (has_master in out[3]). Returns 0, or 1 when the reference refuses the
// checkpoint (its message in `message`, up to `message_len` bytes).
int ref_fe_resume(const char *samples_path, const char *series_path, int n, double p, int circ_type, int init_state,
                  long requested, int record, int max_t, int stride, long *out, std::uint64_t *master, char *message,
                  int message_len)
{
    namespace r = mipt::free_energy::resume;
    try
    {
        r::RunIdentity id;
        id.n = n;
        id.p = p;
        id.circ_type = circ_type;
        id.init_state = init_state;
        id.requested_realizations = requested;
        const auto samples = r::scan_samples(samples_path, r::kSamplesHeader, id);
        const auto series = r::load_timeseries(series_path, r::kTimeseriesHeader, id, 28 * n, record != 0, max_t,
                                               stride);
        out[0] = samples.completed;
        out[1] = series.completed;
        out[2] = static_cast<long>(samples.valid_bytes);
        out[3] = samples.has_master_seed ? 1 : 0;
        *master = samples.master_seed;
        return 0;
    }
    catch (const std::exception &e)
    {
        std::snprintf(message, static_cast<std::size_t>(message_len), "%s", e.what());
        return 1;
    }
}

// RPPU layers as the reference's engine receives them: per layer the ops of
// build_rppu_layer_ops in order -- op_meta [kind, q0, q1] with kind 0 a 4x4
// matrix on (q0, q1) (bit 0 = q0) and kind 2 a JW string (q0 = the site below
// the string, q1 = its control) -- and the measured sites. boundary: 0 FSWAP
// chain, 1 JW string, 2 direct qubit gate (qRPPU). workspace = 0: Circuit1D
// streams and build_rppu_layers_with_boundary (periods, random extra layer);
// workspace = 1: fill_rppu_layer per timestep on mt19937(seed), `periods`
// meaning the layer count. Returns the layer count.
int ref_rppu_draw(std::uint64_t seed, int n, int periods, double p, int boundary, int workspace, int *op_count,
                  int *op_meta, double *op_m, int *sites_per_layer, int *sites)
{
    try
    {
        const auto mode = static_cast<mipt::RppuBoundaryMode>(boundary);
        std::vector<mipt::RppuLayer> layers;
        if (workspace)
        {
            std::mt19937 rng;
            rng.seed(static_cast<std::uint32_t>(seed));
            layers.resize(static_cast<std::size_t>(periods));
            for (int t = 0; t < periods; ++t) mipt::fill_rppu_layer(layers[t], n, (t % 2) != 0, p, true, rng, mode);
        }
        else
        {
            std::mt19937 layer_rng, measure_rng;
            seed_streams(seed, layer_rng, measure_rng);
            mipt::build_rppu_layers_with_boundary(layers, n, periods, p, true, layer_rng, mode);
        }
        int k = 0;
        for (std::size_t l = 0; l < layers.size(); ++l)
        {
            const auto ops = mipt::cusv::build_rppu_layer_ops(layers[l], n);
            op_count[l] = static_cast<int>(ops.ops.size());
            for (const auto &op : ops.ops)
            {
                if (op.kind == mipt::cusv::OpKind::JwString)
                {
                    int lo = 0;
                    while (!((op.string_mask >> (lo + 1)) & 1ull)) ++lo;
                    op_meta[3 * k] = 2;
                    op_meta[3 * k + 1] = lo;
                    op_meta[3 * k + 2] = op.string_control;
                }
                else
                {
                    op_meta[3 * k] = 0;
                    op_meta[3 * k + 1] = op.targets[0];
                    op_meta[3 * k + 2] = op.targets[1];
                    for (int e = 0; e < 16; ++e)
                    {
                        op_m[32 * k + 2 * e] = op.matrix.values[e].real();
                        op_m[32 * k + 2 * e + 1] = op.matrix.values[e].imag();
                    }
                }
                ++k;
            }
            sites_per_layer[l] = static_cast<int>(ops.measure_sites.size());
            for (std::size_t j = 0; j < ops.measure_sites.size(); ++j) sites[l * n + j] = ops.measure_sites[j];
        }
        return static_cast<int>(layers.size());
    }
    catch (...)
    {
        return -1;
    }
}

} // extern "C"
