"""The drop-in executables (mipt.exe, sim_tmi.exe, gmn.exe) on the host:
argument handling, exit codes and messages of the reference apps
(cpp/apps/mipt.cpp:312-414, cpp/apps/sim_tmi.cpp, cpp/apps/gmn.cpp:330-516), the rho3.bin / info.csv
formats (cpp/include/mipt/density.hpp, cpp/apps/mipt.cpp:91-97) and the
sim_tmi resume contract (cpp/include/mipt/tmi/resume.hpp). Nothing here
needs a GPU: every case ends before device work (or runs none)."""
import os
import subprocess

import numpy as np
import pytest

from mipt_gb300 import build, rho3file

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def exes():
    build.build()
    out = os.path.join(ROOT, "mipt_gb300", "_build")
    return os.path.join(out, "mipt.exe"), os.path.join(out, "sim_tmi.exe")


def run(args, cwd, env=None):
    e = dict(os.environ)
    e.pop("CUDA_VISIBLE_DEVICES", None)
    e.update(env or {})
    return subprocess.run(args, cwd=cwd, capture_output=True, text=True, env=e, timeout=120)


def test_mipt_usage_and_argument_errors(exes, tmp_path):
    mipt, _ = exes
    r = run([mipt, "--help"], tmp_path)
    assert r.returncode == 0 and "Usage:" in r.stdout and "circ_type" in r.stdout
    r = run([mipt] + ["1"] * 9, tmp_path)
    assert r.returncode == 2 and "Too many arguments" in r.stderr
    r = run([mipt, "3"], tmp_path)
    assert r.returncode == 1 and "mipt.exe error: d must be 1 or 2." in r.stderr
    r = run([mipt, "1", "10", "2", "1", "1", "0.5", "0.2", "1"], tmp_path)
    assert r.returncode == 1 and "Require 0 <= p_min <= p_max <= 1." in r.stderr
    r = run([mipt, "1", "9", "2", "1", "1", "0.1", "0.2", "1"], tmp_path)
    assert r.returncode == 1 and "Random Haar Unitary requires an even n" in r.stderr
    r = run([mipt, "1", "10", "2", "1", "1", "0.1", "0.2", "7"], tmp_path)
    assert r.returncode == 1 and "circ_type must be one of" in r.stderr
    r = run([mipt, "1", "10", "2", "1", "1", "0.1", "0.2", "0"], tmp_path)
    assert r.returncode == 1 and "not on the GB300 trajectory path" in r.stderr


def test_rho3_bin_and_info_csv_round_trip(exes, tmp_path):
    """periods = 0 needs no device: every record is |000><000| per triple."""
    mipt, _ = exes
    n, R, res = 6, 3, 2
    r = run([mipt, "1", str(n), "0", str(R), str(res), "0.1", "0.3", "1"], tmp_path)
    assert r.returncode == 0, r.stderr
    info = (tmp_path / "info.csv").read_text().splitlines()
    assert info[0] == "n,periods,realizations,resolution,p_min,p_max,circ_type,circuit_name,fermion_trace,cudaq_backend"
    assert info[1].startswith("6,0,3,2,0.1,0.3,1,Random Haar Unitary,0,gb300-")
    meta, rec = rho3file.read(tmp_path / "rho3.bin")
    assert (meta["spatial_dimension"], meta["total_qubits"], meta["kept_qubits"], meta["matrix_dimension"]) == (1, 6, 3, 8)
    assert (meta["periods"], meta["realizations"], meta["resolution"], meta["grid_x"], meta["grid_y"]) == (0, 3, 2, 6, 1)
    assert meta["subsystem_count"] == n and meta["record_count"] == R * res
    assert (meta["p_min"], meta["p_max"]) == (0.1, 0.3)
    np.testing.assert_array_equal(meta["subsystem_qubits"], [[s, (s + 1) % n, (s + 2) % n] for s in range(n)])
    np.testing.assert_array_equal(rec["p_index"], np.repeat(np.arange(res), R))
    np.testing.assert_array_equal(rec["realization"], np.tile(np.arange(R), res))
    np.testing.assert_array_equal(rec["p"], np.repeat([0.1, 0.3], R))
    want = np.zeros((8, 8), complex)
    want[0, 0] = 1
    assert np.all(rec["rho"] == want)


def test_sim_tmi_usage_and_argument_errors(exes, tmp_path):
    _, tmi = exes
    r = run([tmi, "--help"], tmp_path)
    assert r.returncode == 0 and "p,tmi" in r.stderr
    r = run([tmi] + ["1"] * 10, tmp_path)
    assert r.returncode == 2
    r = run([tmi, "10", "2", "2", "2", "0.1", "0.3", "1"], tmp_path)
    assert r.returncode == 1 and "n >= 4 and n divisible by 4" in r.stderr
    r = run([tmi, "12", "2", "2", "2", "0.1", "0.3", "1", "out.csv", "2"], tmp_path)
    assert r.returncode == 1 and "all_cycles must be 0 or 1" in r.stderr
    r = run([tmi, "12", "2", "2", "2", "0.1", "0.3", "1"], tmp_path, {"SIM_TMI_ENTROPY_ORDER": "3"})
    assert r.returncode == 1 and "SIM_TMI_ENTROPY_ORDER must be 1" in r.stderr


def default_path(tmp_path, tag, n, R, pmin, pmax, res):
    return tmp_path / "csv" / "tmi" / tag / f"tmi_{tag}_n_{n}_real_{R}_{pmin}_{pmax}_res_{res}.csv"


def test_sim_tmi_complete_file_is_left_alone(exes, tmp_path):
    _, tmi = exes
    path = default_path(tmp_path, "haarc", 8, 2, "0.1", "0.3", 2)
    path.parent.mkdir(parents=True)
    rows = ["p,tmi"] + [f"{p},-0.5" for p in ("0.10000000000000001", "0.29999999999999999") for _ in range(2 * 2)]
    path.write_text("\n".join(rows) + "\n")
    r = run([tmi, "8", "2", "2", "2", "0.1", "0.3", "1", "1"], tmp_path)
    assert r.returncode == 0, r.stderr
    assert "already holds all 8 TMI row(s)" in r.stderr


def test_sim_tmi_resume_trims_partial_circuit(exes, tmp_path):
    """A partially written circuit (1 of 2 cycle rows) is cut off before the
    run continues (without a GPU the run then stops at device creation; with
    one it appends the remaining circuits after the kept rows)."""
    _, tmi = exes
    path = default_path(tmp_path, "haarc", 8, 2, "0.1", "0.3", 2)
    path.parent.mkdir(parents=True)
    keep = "p,tmi\n" + "0.10000000000000001,-0.25\n" * 2
    path.write_text(keep + "0.10000000000000001,-0.125\n0.1000")
    r = run([tmi, "8", "2", "2", "2", "0.1", "0.3", "1", "1"], tmp_path)
    assert "RESUMED from" in r.stderr and "dropped 1 row(s)" in r.stderr, r.stderr
    text = path.read_text()
    assert text.startswith(keep) and "-0.125" not in text


def test_sim_tmi_refuses_foreign_checkpoint(exes, tmp_path):
    _, tmi = exes
    path = default_path(tmp_path, "haar", 8, 2, "0.1", "0.3", 2)
    path.parent.mkdir(parents=True)
    path.write_text("p,tmi\n0.2,-1\n")
    r = run([tmi, "8", "2", "2", "2", "0.1", "0.3", "1", "0"], tmp_path)
    assert r.returncode == 1 and "switches away from p=0.10000000000000001 after 0 rows" in r.stderr
    other = tmp_path / "csv" / "tmi" / "haar" / "tmi_haar_n_12_real_2_0.1_0.3_res_2.csv"
    other.write_text("p,tmi\n")
    r = run([tmi, "8", "2", "2", "2", "0.1", "0.3", "1", "0", str(other)], tmp_path)
    assert r.returncode == 1 and "n=12 (this run uses 8)" in r.stderr


def test_gmn_usage_and_argument_errors(exes, tmp_path):
    """gmn.exe's argument contract (cpp/apps/gmn.cpp:253-280,330-370); every
    case ends before device work."""
    gmn = os.path.join(os.path.dirname(exes[0]), "gmn.exe")
    r = run([gmn, "--help"], tmp_path)
    assert r.returncode == 0 and "Usage:" in r.stdout and "limit_per_p" in r.stdout
    r = run([gmn, "3"], tmp_path)
    assert r.returncode == 1 and "gmn.exe error: The former leading argument '3' has been removed." in r.stderr
    r = run([gmn, "6"], tmp_path)
    assert r.returncode == 1 and "Six-qubit retained-subsystem analysis has been removed" in r.stderr
    r = run([gmn, "2"], tmp_path)
    assert r.returncode == 1 and "First argument must be evaluation mode 0 or 1." in r.stderr
    r = run([gmn, "1", "a.bin", "b.csv", "0", "extra"], tmp_path)
    assert r.returncode == 1 and "Too many command-line arguments." in r.stderr
    r = run([gmn, "1", "a.bin", "b.csv", "-1"], tmp_path)
    assert r.returncode == 1 and "limit_per_p must be a non-negative integer." in r.stderr
    r = run([gmn, "1", "missing.bin", "b.csv"], tmp_path)
    assert r.returncode == 1 and "Could not open density-matrix file: missing.bin" in r.stderr
    (tmp_path / "bad.bin").write_bytes(b"NOTARHO2" + bytes(64))
    r = run([gmn, "1", "bad.bin", "b.csv"], tmp_path)
    assert r.returncode == 1 and "Not a version-2 MIPT density-matrix file." in r.stderr
    two = np.zeros((2, 1, 4, 4), complex)
    two[:, 0, 0, 0] = 1
    rho3file.write(tmp_path / "two.bin", two, p=[0.1, 0.2], p_index=[0, 1], total_qubits=4)
    r = run([gmn, "1", "two.bin", "b.csv"], tmp_path)
    assert r.returncode == 1 and "three-qubit 8x8 reduced density matrices" in r.stderr
    r = run([gmn, "1", "two.bin", "b.csv"], tmp_path, {"GMN_LIMIT_PER_P": "x"})
    assert r.returncode == 1 and "GMN_LIMIT_PER_P must be a non-negative integer." in r.stderr


ENTROPY_HEADER = ("N,periods,p,requested_realizations,completed_realizations,circ_type,circuit_name,fermionic_trace,"
                  "L_A,x,ln_x,S1_mean,S1_stddev,S1_stderr,S2_mean,S2_stddev,S2_stderr,subsystems_per_realization,"
                  "total_subsystems")


def entropy_rows(n, periods, p, requested, done, circ=1):
    """A well-formed entropy.exe checkpoint (cpp/include/mipt/entropy.hpp:580-636)."""
    rows = [ENTROPY_HEADER]
    for kept in range(2, n // 2 + 1):
        x = float((n / np.pi) * np.sin(np.pi * kept / n))
        sd = 0.25
        se = float(sd / np.sqrt(done)) if done > 1 else 0.0
        rows.append(f'{n},{periods},{p!r},{requested},{done},{circ},"Random Haar Unitary",0,{kept},{x!r},'
                    f'{float(np.log(x))!r},{0.5 * kept!r},{sd!r},{se!r},{0.4 * kept!r},{sd!r},{se!r},{n},{n * done}')
    return "\n".join(rows) + "\n"


def test_entropy_usage_argument_errors_and_checkpoints(exes, tmp_path):
    """entropy.exe's argument contract (cpp/apps/entropy.cpp:16-60) and the
    checkpoint refusals of cpp/include/mipt/entropy_resume.hpp:96-244; every
    case ends before device work."""
    ent = os.path.join(os.path.dirname(exes[0]), "entropy.exe")
    r = run([ent, "--help"], tmp_path)
    assert r.returncode == 0 and "Usage:" in r.stdout and "MIPT_ENTROPY_S1_MAX_LA" in r.stdout
    r = run([ent, "8", "2"], tmp_path)
    assert r.returncode == 2 and "Usage:" in r.stdout
    for args, msg in [(["3", "2", "0.1", "2", "1"], "N must be at least 4"),
                      (["8", "-1", "0.1", "2", "1"], "periods must be non-negative."),
                      (["8", "2", "1.5", "2", "1"], "p must be in [0,1]."),
                      (["8", "2", "0.1", "0", "1"], "realizations must be positive."),
                      (["9", "2", "0.1", "2", "1"], "requires an even N"),
                      (["8", "2", "0.1", "2", "0"], "not on the GB300 trajectory path"),
                      (["8", "2", "0.1", "2", "7"], "circ_type must be one of")]:
        r = run([ent] + args + ["out.csv"], tmp_path)
        assert r.returncode == 1 and "entropy.exe error: " in r.stderr and msg in r.stderr, (args, r.stderr)
    (tmp_path / "done.csv").write_text(entropy_rows(8, 2, 0.1, 2, 2))
    r = run([ent, "8", "2", "0.1", "2", "1", "done.csv"], tmp_path)
    assert r.returncode == 0 and "already complete. Nothing to do." in r.stdout, r.stdout + r.stderr
    r = run([ent, "10", "2", "0.1", "2", "1", "done.csv"], tmp_path)
    assert r.returncode == 1 and "The checkpoint belongs to a different N." in r.stderr
    r = run([ent, "8", "2", "0.2", "2", "1", "done.csv"], tmp_path)
    assert r.returncode == 1 and "different p" in r.stderr
    r = run([ent, "8", "2", "0.1", "2", "1", "done.csv"], tmp_path, {"MIPT_ENTROPY_S1_MAX_LA": "3"})
    assert r.returncode == 1 and "records S1 for L_A up to 4 but this run is configured for L_A up to 3" in r.stderr
    lines = entropy_rows(8, 2, 0.1, 4, 3).splitlines()
    cells = lines[1].split(",")
    cells[16] = "0.2"  # S2_stderr no longer stddev / sqrt(3)
    lines[1] = ",".join(cells)
    (tmp_path / "edited.csv").write_text("\n".join(lines) + "\n")
    r = run([ent, "8", "2", "0.1", "4", "1", "edited.csv"], tmp_path)
    assert r.returncode == 1 and "two runs were concatenated" in r.stderr, r.stderr
    (tmp_path / "other.csv").write_text("a,b\n1,2\n")
    r = run([ent, "8", "2", "0.1", "2", "1", "other.csv"], tmp_path)
    assert r.returncode == 1 and "different column layout" in r.stderr


FE_SAMPLES_HEADER = ("N,p,circ_type,circuit_name,init_state,trajectory,parity_sector,trajectory_seed,"
                     "equil_timesteps,production_timesteps,total_timesteps,measurements_total,"
                     "measurements_production,F_total,F_production,production_rate_endpoint,production_slope,"
                     "free_energy_density_tilde")
FE_SERIES_HEADER = ("N,p,circ_type,circuit_name,init_state,requested_realizations,completed_realizations,t,"
                    "t_over_L,phase,F_mean,F_stddev,F_stderr,F_over_tL_mean,F_over_tL_stddev,F_over_tL_stderr,"
                    "S_half_mean,S_half_stddev,S_half_stderr,S_half_count")


def fe_files(n, p, init, requested, completed, master, entropy_max_t=None):
    """A free-energy checkpoint of `completed` trajectories in the reference's
    layout (cpp/include/mipt/free_energy_resume.hpp:79-88); values are
    placeholders, seeds follow splitmix64(master ^ trajectory)."""
    from oracle import pyoracle as orc
    T, eq = 28 * n, 4 * n
    mt = 2 * n if entropy_max_t is None else entropy_max_t
    name = '"Random Haar Unitary"'
    rows = [FE_SAMPLES_HEADER]
    for t in range(completed):
        ts = orc.fe_trajectory_seed(master, t)
        rows.append(f"{n},{float(p)!r},1,{name},{init},{t},-1,{ts},{eq},{24 * n},{T},10,8,1.5,1.25,0.1,0.1,0.0125")
    series = [FE_SERIES_HEADER]
    for t in range(T + 1):
        phase = "initial" if t == 0 else ("equilibration" if t <= eq else "production")
        s_count = completed if (t == 0 or (t <= mt)) else 0
        s_stat = "0.5,0.1,0.05" if s_count else "nan,nan,nan"
        f = "0,0,0" if t == 0 else "0.25,0.01,0.005"
        ftl = "nan,nan,nan" if t == 0 else "0.01,0.001,0.0005"
        series.append(f"{n},{float(p)!r},1,{name},{init},{requested},{completed},{t},{t / n!r},{phase},"
                      f"{f},{ftl},{s_stat},{s_count}")
    return "\n".join(rows) + "\n", "\n".join(series) + "\n"


def test_free_energy_usage_argument_errors_and_checkpoints(exes, tmp_path):
    """free_energy.exe's argument contract (cpp/apps/free_energy.cpp:164-240)
    and its checkpoint refusals (cpp/apps/free_energy.cpp:254-358,
    cpp/include/mipt/free_energy_resume.hpp:246-534); every case ends
    before device work."""
    fe = os.path.join(os.path.dirname(exes[0]), "free_energy.exe")
    r = run([fe, "--help"], tmp_path)
    assert r.returncode == 0 and "Usage:" in r.stdout and "MIPT_FREE_ENERGY_ENTROPY_STRIDE" in r.stdout
    r = run([fe, "8", "0.1"], tmp_path)
    assert r.returncode == 2 and "Usage:" in r.stdout
    for args, msg in [(["8", "0.1", "0", "1", "0"], "realizations must lie in [1,1000000000]."),
                      (["31", "0.1", "2", "1", "0"], "N must lie in [2,30]"),
                      (["9", "0.1", "2", "1", "0"], "requires an even N"),
                      (["8", "1.5", "2", "1", "0"], "p must lie in [0,1]."),
                      (["8", "0.1", "2", "1", "2"], "init_state must be 0 or 1."),
                      (["8", "0.1", "2", "3", "0"], "not on the GB300 trajectory path"),
                      (["8", "0.1", "2", "9", "0"], "circ_type must be one of")]:
        r = run([fe] + args, tmp_path)
        assert r.returncode == 1 and "free_energy.exe: " in r.stderr and msg in r.stderr, (args, r.stderr)
    stem = "free_energy_haar_n_8_p_0.1_init_0_reals_3"
    samples, series = fe_files(8, 0.1, 0, 3, 3, master=77)
    (tmp_path / f"{stem}_samples.csv").write_text(samples)
    (tmp_path / f"{stem}_timeseries.csv").write_text(series)
    r = run([fe, "8", "0.1", "3", "1", "0"], tmp_path)
    assert r.returncode == 0 and "is already complete (3/3 trajectories). Nothing to do." in r.stdout, r.stderr
    assert "seed stream recovered" in r.stdout
    # Only one of the two files: refused.
    (tmp_path / f"{stem}_timeseries.csv").unlink()
    r = run([fe, "8", "0.1", "3", "1", "0"], tmp_path)
    assert r.returncode == 1 and "Both CSVs are needed to continue a run" in r.stderr
    # A different entropy schedule than the checkpoint's.
    (tmp_path / f"{stem}_timeseries.csv").write_text(series)
    r = run([fe, "8", "0.1", "3", "1", "0"], tmp_path, {"MIPT_FREE_ENERGY_ENTROPY_MAX_T": "5"})
    assert r.returncode == 1 and "S_half_count=3 at t=6" in r.stderr, r.stderr
    # An aggregate ahead of the samples file.
    samples2, _ = fe_files(8, 0.1, 0, 3, 2, master=77)
    (tmp_path / f"{stem}_samples.csv").write_text(samples2)
    r = run([fe, "8", "0.1", "3", "1", "0"], tmp_path)
    assert r.returncode == 1 and "aggregates 3 trajectories but" in r.stderr
    # Trajectory indices with a gap.
    lines = samples.splitlines()
    del lines[2]
    (tmp_path / f"{stem}_samples.csv").write_text("\n".join(lines) + "\n")
    r = run([fe, "8", "0.1", "3", "1", "0"], tmp_path)
    assert r.returncode == 1 and "has trajectory=2 where 1 was expected" in r.stderr
    # Another run's identity and another layout.
    (tmp_path / f"{stem}_samples.csv").write_text(samples.replace(",0,0,-1,", ",1,0,-1,", 1))
    r = run([fe, "8", "0.1", "3", "1", "0"], tmp_path)
    assert r.returncode == 1 and "was produced with init_state=1" in r.stderr, r.stderr
    (tmp_path / f"{stem}_samples.csv").write_text("a,b\n1,2\n")
    r = run([fe, "8", "0.1", "3", "1", "0"], tmp_path)
    assert r.returncode == 1 and "different column layout" in r.stderr
    # The recovered master seed wins over MIPT_FREE_ENERGY_SEED.
    (tmp_path / f"{stem}_samples.csv").write_text(samples)
    r = run([fe, "8", "0.1", "3", "1", "0"], tmp_path, {"MIPT_FREE_ENERGY_SEED": "5"})
    assert r.returncode == 0 and "Nothing to do." in r.stdout


def test_rppu_circuit_types_pass_argument_checks(exes, tmp_path):
    """circ_type 2 (FermionRPPU) and 4 (qRPPU) are on the GB300 path: the
    executables accept them up to device work (here: no device) and keep the
    reference's even-N rule for them (cpp/include/mipt/types.hpp:174-185)."""
    mipt, tmi = exes
    fe = os.path.join(os.path.dirname(mipt), "free_energy.exe")
    for ct in ("2", "4"):
        r = run([mipt, "1", "9", "2", "1", "1", "0.1", "0.2", ct], tmp_path)
        assert r.returncode == 1 and "requires an even n" in r.stderr, r.stderr
        r = run([fe, "9", "0.1", "2", ct, "0"], tmp_path)
        assert r.returncode == 1 and "requires an even N" in r.stderr, r.stderr
        r = run([mipt, "1", "8", "2", "1", "1", "0.1", "0.2", ct], tmp_path)
        assert "not on the GB300 trajectory path" not in r.stderr


GOLD = np.load(os.path.join(ROOT, "tests", "golden", "ref_fixtures.npz"))


@pytest.mark.parametrize("k", range(len(GOLD["feck_params"])))
def test_free_energy_resume_matches_reference_reader(exes, tmp_path, k):
    """free_energy.exe reads six checkpoints exactly as the reference's own
    readers (scan_samples / load_timeseries, recorded in the fixtures) do:
    completed rows, aggregate lag, trimmed tail and recovered master seed, or
    the same refusal text. With no device visible the accepted runs stop at
    batch creation, after the resume report."""
    n, p, init, R, max_t, stride, rc, completed, agg, valid, has_master, _ = GOLD["feck_params"][k]
    n, init, R, completed, agg, valid = int(n), int(init), int(R), int(completed), int(agg), int(valid)
    master = int(GOLD[f"feck{k}_master"][0])
    samples, series = str(GOLD[f"feck{k}_samples"]), str(GOLD[f"feck{k}_series"])
    stem = f"free_energy_haar_n_{n}_p_{p:g}_init_{init}_reals_{R}"
    sp, tp = tmp_path / f"{stem}_samples.csv", tmp_path / f"{stem}_timeseries.csv"
    sp.write_text(samples)
    tp.write_text(series)
    fe = os.path.join(os.path.dirname(exes[0]), "free_energy.exe")
    env = {"CUDA_VISIBLE_DEVICES": "", "MIPT_FREE_ENERGY_ENTROPY_MAX_T": str(int(max_t)),
           "MIPT_FREE_ENERGY_ENTROPY_STRIDE": str(int(stride))}
    r = run([fe, str(n), str(p), str(R), "1", str(init)], tmp_path, env)
    if int(rc) != 0:
        msg = str(GOLD[f"feck{k}_message"]).replace(f"s{k}.csv", sp.name).replace(f"t{k}.csv", tp.name)
        assert r.returncode == 1 and msg in r.stderr, (msg, r.stderr)
        return
    assert f"Resuming from {sp.name}: {completed}/{R} trajectories already recorded, seed stream recovered." \
        in r.stdout, r.stdout + r.stderr
    assert f"seed={master}\n" in r.stdout
    if agg != completed:
        assert f"The time-series aggregate holds {agg} trajectories against the samples file's {completed}" in r.stdout
    if valid < len(samples.encode()):
        assert f"Dropping {len(samples.encode()) - valid} bytes of an unterminated trailing row" in r.stdout
        assert len(sp.read_bytes()) == valid
    assert r.returncode == 1 and "free_energy.exe: " in r.stderr and "Resume refused" not in r.stderr


@pytest.fixture(scope="module")
def rho3_io(tmp_path_factory):
    exe = tmp_path_factory.mktemp("rho3io") / "rho3_io"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "mipt_gb300", "apps"), os.path.join(ROOT, "tests", "golden", "rho3_io.cpp"),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


@pytest.mark.parametrize("k", range(3))
def test_rho3_bin_matches_reference_writer(rho3_io, tmp_path, k):
    """rho3.bin files the reference's DensityMatrixWriter wrote
    (cpp/include/mipt/density.hpp:134-251): the executables' C++ writer
    reproduces them byte for byte from the same content, their C++ reader and
    mipt_gb300.rho3file read back exactly that content."""
    want = GOLD[f"rho3file{k}_bytes"].tobytes()
    dims = [int(x) for x in GOLD[f"rho3file{k}_dims"]]
    subs, pidx, real = GOLD[f"rho3file{k}_subs"], GOLD[f"rho3file{k}_pidx"], GOLD[f"rho3file{k}_real"]
    ps, payload = GOLD[f"rho3file{k}_p"], GOLD[f"rho3file{k}_payload"]
    nrec = len(ps)
    per = payload.size // nrec
    spec = [" ".join(str(x) for x in dims + [nrec]), (0.125).hex(), (0.875).hex(), " ".join(str(int(q)) for q in subs)]
    for r in range(nrec):
        spec.append(f"{int(pidx[r])} {int(real[r])} {float(ps[r]).hex()} " +
                    " ".join(float(v).hex() for v in payload[r * per:(r + 1) * per]))
    (tmp_path / "spec.txt").write_text("\n".join(spec) + "\n")
    r = subprocess.run([rho3_io, "write", str(tmp_path / "ours.bin"), str(tmp_path / "spec.txt")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "ours.bin").read_bytes() == want
    (tmp_path / "ref.bin").write_bytes(want)
    r = subprocess.run([rho3_io, "read", str(tmp_path / "ref.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    head = lines[0].split()
    assert [int(x) for x in head[:10]] == dims[:9] + [nrec]
    assert float.fromhex(head[10]) == 0.125 and float.fromhex(head[11]) == 0.875
    assert [int(x) for x in lines[1].split()] == [int(q) for q in subs]
    for r_, line in enumerate(lines[2:]):
        cells = line.split()
        assert int(cells[0]) == pidx[r_] and int(cells[1]) == real[r_] and float.fromhex(cells[2]) == ps[r_]
        assert np.array_equal(np.array([float.fromhex(c) for c in cells[3:]]), payload[r_ * per:(r_ + 1) * per])
    meta, rec = rho3file.read(tmp_path / "ref.bin")
    assert meta["spatial_dimension"] == dims[0] and meta["grid_y"] == dims[7] and meta["record_count"] == nrec
    assert np.array_equal(meta["subsystem_qubits"].ravel(), subs)
    D = 1 << dims[2]
    np.testing.assert_array_equal(rec["rho"].reshape(nrec, -1),
                                  payload.reshape(nrec, -1, 2)[..., 0] + 1j * payload.reshape(nrec, -1, 2)[..., 1])
    assert rec["rho"].shape == (nrec, dims[8], D, D)
    rho = payload.reshape(nrec, dims[8], D, D, 2)
    rho3file.write(tmp_path / "py.bin", rho[..., 0] + 1j * rho[..., 1], ps, pidx, real, total_qubits=dims[1],
                   periods=dims[3], realizations=dims[4], resolution=dims[5], p_min=0.125, p_max=0.875,
                   subsystem_qubits=subs, spatial_dimension=dims[0], grid_x=dims[6], grid_y=dims[7])
    assert (tmp_path / "py.bin").read_bytes() == want


@pytest.mark.parametrize("k", range(len(GOLD["entck_params"])))
def test_entropy_resume_matches_reference_reader(exes, tmp_path, k):
    """entropy.exe decides on eight checkpoints as the reference's own reader
    (cpp/include/mipt/entropy_resume.hpp:102-246, recorded in the fixtures)
    does: resume from the same completed count, finish, or refuse."""
    n, periods, p, requested, circ, s1max, rc, done = GOLD["entck_params"][k]
    n, periods, requested, circ, s1max, done = int(n), int(periods), int(requested), int(circ), int(s1max), int(done)
    (tmp_path / "e.csv").write_text(str(GOLD[f"entck{k}_text"]))
    ent = os.path.join(os.path.dirname(exes[0]), "entropy.exe")
    env = {"CUDA_VISIBLE_DEVICES": "", "MIPT_ENTROPY_S1_MAX_LA": "0" if s1max >= n // 2 else str(s1max)}
    r = run([ent, str(n), str(periods), repr(float(p)), str(requested), str(circ), "e.csv"], tmp_path, env)
    if int(rc) != 0:
        assert r.returncode == 1 and "Resume refused: e.csv" in r.stderr, (str(GOLD[f"entck{k}_message"]), r.stderr)
    elif done == requested:
        assert r.returncode == 0 and "e.csv is already complete. Nothing to do." in r.stdout, r.stdout + r.stderr
    else:
        assert f"Resuming from e.csv: {done}/{requested}" in r.stdout, r.stdout + r.stderr
        assert "Resume refused" not in r.stderr


@pytest.mark.parametrize("k", range(len(GOLD["tmick_params"])))
def test_sim_tmi_resume_matches_reference_reader(exes, tmp_path, k):
    """sim_tmi.exe reads seven `p,tmi` checkpoints as the reference's own
    reader (cpp/include/mipt/tmi/resume.hpp:188-330, recorded in the
    fixtures) does: rows kept, partial circuit dropped, file truncated to the
    same byte, the same restart point and name check, or the same refusal."""
    n, R, res, pmin, pmax, allc, rc, loaded, verified, rows, dropped, kept, sp_, sr = GOLD["tmick_params"][k]
    n, R, res, allc = int(n), int(R), int(res), int(allc)
    name = str(GOLD[f"tmick{k}_name"])
    text = str(GOLD[f"tmick{k}_text"])
    path = tmp_path / name
    path.write_text(text)
    _, tmi = exes
    r = run([tmi, str(n), "2", str(R), str(res), repr(float(pmin)), repr(float(pmax)), "1", str(allc), str(path)],
            tmp_path, {"CUDA_VISIBLE_DEVICES": ""})
    if int(rc) != 0:
        msg = str(GOLD[f"tmick{k}_message"]).replace(name, str(path), 1)
        assert r.returncode == 1 and msg in r.stderr, (msg, r.stderr)
        return
    total = res * R * (n // 4 if allc else 1)
    if int(rows) >= total:
        assert r.returncode == 0 and f"already holds all {total} TMI row(s)" in r.stderr, r.stderr
        assert path.read_text() == text
        return
    line = f"RESUMED from {path}: {int(rows)} TMI row(s) already recorded"
    if int(dropped) > 0:
        line += f"; dropped {int(dropped)} row(s) of a partially written circuit"
    assert line + "." in r.stderr, r.stderr
    assert f"realization {int(sr)}/{R}." in r.stderr and f"Continuing at p[{int(sp_)}]=" in r.stderr
    assert ("does not follow the generated naming convention" in r.stderr) == (not int(verified))
    assert len(path.read_bytes()) == int(kept)
