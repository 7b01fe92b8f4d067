// Host-side trajectory sampler: seeded Haar brickwork layer draws and the
// measurement uniforms, reproducing the reference's random streams.
//
// Reference behaviour this follows (paths inside the reference project):
//   seeding::splitmix64, trajectory_seed          cpp/include/mipt/types.hpp:262-273
//   Circuit1D::seed (layer and measurement mt19937 streams)
//                                                 cpp/include/mipt/circuit.hpp:129-140
//   fill_haar_layer / build_haar_layers            cpp/include/mipt/circuits/haar.hpp:226-305
//   haar_unitary_4                                 cpp/include/mipt/circuits/haar.hpp:39-85
//   random_haar_bond_gate retry rule               cpp/include/mipt/circuits/haar.hpp:171-181,211-224
//   Engine::measure_layer uniform draws            cpp/include/mipt/cusv/engine.hpp:300-327
#pragma once

#include <complex>
#include <cstdint>
#include <vector>

namespace mg
{

std::uint64_t splitmix64(std::uint64_t v);
std::uint64_t trajectory_seed(std::uint64_t master, std::uint64_t index);

// One trajectory's complete random record. Layer t has gate_count(t) bonds;
// bond j of layer t occupies qubits bond_q[2*(t*max_bonds+j) + {0,1}] and its
// row-major 4x4 unitary (index bit 0 = first qubit) starts at
// bond_u[16*(t*max_bonds+j)]. Measured sites of layer t are the set bits of
// measured[t]; uniforms are consumed one per chunk of `chunk_bits` measured
// sites, layer by layer, in order.
struct TrajectoryDraw
{
    int n = 0;
    int layers = 0;
    int max_bonds = 0;
    std::vector<int> bond_count;
    std::vector<int> bond_q;
    std::vector<std::complex<double>> bond_u;
    std::vector<std::uint64_t> measured;
    std::vector<double> uniforms;
    std::vector<int> uniform_offset; // first uniform of layer t
    // Site n-1 is measured as its own chunk, after the others (the reference's
    // parity-sector engine measures it as the parity of the encoded index).
    bool split_last = false;
};

// Random parity-preserving (RPPU / qRPPU) brickwork, 1-D closed ring
// (cpp/include/mipt/circuits/rppu_layer.hpp:51-285). Each bond is
// U_even (+) U_odd, two haar_unitary_2 draws (even block on |00>,|11>, odd
// block on |10>,|01>). The odd layer's closure gate is drawn first; it acts on
// (0, n-1) and is stored in the plan's orientation (n-1, 0) as the last bond.
// For the fermionic gate set the closure carries the Jordan-Wigner string on
// sites 1..n-2 (the batch brackets odd layers with that diagonal; the
// reference's FSWAP-chain form of the closure is the same operator).
//   draw_rppu_trajectory: Circuit1D streams, 2*periods layers plus, with
//   probability 1/2 (drawn first), one extra even layer; `layers_out` layers
//   are written (>= 2*periods + 1), a missing extra layer as identity gates
//   and no measurements. split_last: the encoded-measurement chunking.
//   draw_rppu_workspace: the probed workspace's streams, `layers` layers.
void draw_rppu_trajectory(std::uint64_t seed, int n, int periods, double p, int chunk_bits, bool split_last,
                          int layers_out, TrajectoryDraw &out);
void draw_rppu_workspace(std::uint32_t seed, int n, int layers, double p, int chunk_bits, bool split_last,
                         int layers_out, TrajectoryDraw &out);
void draw_rppu_batch(const std::uint64_t *seeds, const double *p, int count, int n, int periods, int chunk_bits,
                     bool split_last, int layers_out, std::vector<TrajectoryDraw> &out, int threads);
void draw_rppu_workspace_batch(const std::uint32_t *seeds, const double *p, int count, int n, int layers,
                               int chunk_bits, bool split_last, int layers_out, std::vector<TrajectoryDraw> &out,
                               int threads);

// Draws a 1-D Haar brickwork trajectory (2*periods layers; odd layers close
// the ring with bond (n-1, 0) when `closed`).
void draw_haar_trajectory(std::uint64_t seed, int n, int periods, double p, bool closed, int chunk_bits,
                          TrajectoryDraw &out);

// Draws many trajectories on `threads` host threads (0 = hardware count).
void draw_haar_batch(const std::uint64_t *seeds, const double *p, int count, int n, int periods, bool closed,
                     int chunk_bits, std::vector<TrajectoryDraw> &out, int threads);

// The same brickwork draw (`layers` layers, layer t starting at bond t % 2)
// from the streams of the probed circuit workspace that free_energy.exe uses:
// the layer stream is an mt19937 seeded with the 32-bit `seed` itself, the
// measurement stream one seeded with seed ^ 0x9e3779b9
// (cpp/include/mipt/probed.hpp:103-108,196-206).
void draw_haar_trajectory_workspace(std::uint32_t seed, int n, int layers, double p, bool closed, int chunk_bits,
                                    TrajectoryDraw &out);
void draw_haar_workspace_batch(const std::uint32_t *seeds, const double *p, int count, int n, int layers,
                               bool closed, int chunk_bits, std::vector<TrajectoryDraw> &out, int threads);

// Random initial states of the free-energy protocol
// (cpp/include/mipt/free_energy.hpp:125-222), drawn from an mt19937_64 seeded
// with `seed`, amplitudes rounded to Real exactly where the reference stores
// them. kind 0: product of Haar-random single-site states (with
// `fixed_parity`: a uniformly random basis state of a random global parity);
// kind 1: normalised complex Gaussian amplitudes (with `fixed_parity`: only
// those of a random parity sector). Writes 2^n amplitudes; returns the parity
// sector (0/1) or -1.
template <typename Real>
int draw_initial_state(std::uint64_t seed, int n, int kind, bool fixed_parity, std::complex<Real> *out);

} // namespace mg

namespace mg
{
// One free-fermion (Majorana covariance) trajectory: N modes, `depth`
// layers. Layer t applies a Haar SO(4) rotation to the Majoranas of modes
// (m, m+1 mod N) for each gate start m in gate_mode[t] (rot[16*g], row-major),
// then measures the parity of every mode in measured[t] (ascending, one
// uniform each, from the measurement stream). Same streams as the Haar path.
struct FermionDraw
{
    int n = 0, depth = 0, max_gates = 0;
    std::vector<int> gate_count;
    std::vector<int> gate_mode;  // [depth][max_gates]
    std::vector<double> rot;     // [depth][max_gates][16]
    std::vector<int> meas_count;
    std::vector<int> meas_mode;  // [depth][n]
    std::vector<double> uniform; // [depth][n]
};

void draw_fermion_trajectory(std::uint64_t seed, int n, int depth, double p, bool closed, FermionDraw &out);
void draw_fermion_batch(const std::uint64_t *seeds, const double *p, int count, int n, int depth, bool closed,
                        std::vector<FermionDraw> &out, int threads);
} // namespace mg

namespace mg
{
// Four-colour brickwork on an X x Y torus, qubit q = r * X + c. Colour 0/1:
// horizontal bonds, rows of parity 0/1 pair (c, c+1) from c = 0, the other
// rows take the wrap bond (0, X-1) first and pair from c = 1; colour 2/3: the
// same for columns and vertical bonds. Bond order and first qubits follow the
// reference's 2-D loops (python/mipt.py:244-311); a direction of odd length has
// no wrap bond (one idle site per line), which the reference's square-lattice
// indexing does not define.
std::vector<std::pair<int, int>> lattice_bonds(int X, int Y, int colour);

// A 2-D Haar trajectory of `layers` layers (colour t % 4 at layer t), drawn
// with the streams and per-layer order of the 1-D path: the layer's unitaries,
// then Bernoulli(p) flags site by site, then one measurement uniform per chunk.
void draw_haar_lattice_trajectory(std::uint64_t seed, int X, int Y, int layers, double p, int chunk_bits,
                                  TrajectoryDraw &out);
void draw_haar_lattice_batch(const std::uint64_t *seeds, const double *p, int count, int X, int Y, int layers,
                             int chunk_bits, std::vector<TrajectoryDraw> &out, int threads);
} // namespace mg
