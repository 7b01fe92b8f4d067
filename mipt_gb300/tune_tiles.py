"""Measures the pass-tile table a batch uses when created with tile_qubits = 0:
for every geometry below, mipt_gb300_autotune_tile times one cycle of all
layer colours for each candidate local-qubit count, and the fastest is
printed as a C++ table entry {n, fp64, lattice, tile} for capi.cu's
kTunedTiles, followed by the timings.

    python -m mipt_gb300.tune_tiles
"""
import json
import sys


def geometries():
    for fp64 in (False, True):
        for n in range(14, 31, 2):
            if fp64 and n > 28:
                continue
            yield dict(n=n, fp64=fp64, lattice=None)
    yield dict(n=28, fp64=False, lattice=(4, 7))
    yield dict(n=20, fp64=False, lattice=(4, 5))


def main():
    import mipt_gb300 as mg
    rows, log = [], []
    for g in geometries():
        n, fp64 = g["n"], g["fp64"]
        state = (1 << n) * (16 if fp64 else 8)
        traj = max(1, min(1024, (4 << 30) // state))  # batch-sized grids: up to 4 GiB of states
        best, ms = mg.autotune_tile(n, fp64=fp64, closed=True, lattice=g["lattice"], trajectories=traj)
        rows.append(f"    {{{n}, {int(fp64)}, {int(g['lattice'] is not None)}, {best}}},")
        log.append(dict(n=n, fp64=fp64, lattice=g["lattice"], trajectories=traj, best=best, ms_per_cycle=ms))
    print("\n".join(rows))
    for entry in log:
        print(json.dumps(entry), file=sys.stderr)


if __name__ == "__main__":
    main()
