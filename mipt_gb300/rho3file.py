"""Reader for version-2 MIPT density-matrix files (rho3.bin, rho3_2d.bin).

Layout (the reference's cpp/include/mipt/density.hpp:12-14,148-199):
magic "MIPTRHO2", u32 0x01020304, u32 version 2; u32 spatial_dimension,
total_qubits, kept_qubits, matrix_dimension, periods, realizations,
resolution, grid_x, grid_y, subsystem_count; u64 record_count; f64 p_min,
p_max; u32 subsystem_qubits[subsystem_count * kept_qubits]; then per record
u32 p_index, u32 realization, f64 p and subsystem_count * 2 * D^2 doubles
(subsystem-major, row-major (re, im) of each D x D matrix).
"""
import struct

import numpy as np

MAGIC = b"MIPTRHO2"
_HEADER_FIELDS = ("spatial_dimension", "total_qubits", "kept_qubits", "matrix_dimension", "periods",
                  "realizations", "resolution", "grid_x", "grid_y", "subsystem_count")


def read(path):
    """Returns (metadata dict, records) with records a structured array of
    p_index, realization, p and rho[subsystem][D][D] (complex128)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != MAGIC:
        raise ValueError("Not a version-2 MIPT density-matrix file.")
    endian, version = struct.unpack_from("<II", data, 8)
    if endian != 0x01020304:
        raise ValueError("Density-matrix file endianness is not supported on this host.")
    if version != 2:
        raise ValueError("Unsupported density-matrix file version.")
    off = 16
    vals = struct.unpack_from("<10I", data, off)
    off += 40
    meta = dict(zip(_HEADER_FIELDS, vals))
    meta["record_count"], = struct.unpack_from("<Q", data, off)
    off += 8
    meta["p_min"], meta["p_max"] = struct.unpack_from("<dd", data, off)
    off += 16
    S, K, D = meta["subsystem_count"], meta["kept_qubits"], meta["matrix_dimension"]
    if D != 1 << K:
        raise ValueError("Density-matrix dimension does not match kept-qubit count.")
    meta["subsystem_qubits"] = np.frombuffer(data, np.uint32, S * K, off).reshape(S, K).copy()
    off += 4 * S * K
    rec = np.dtype([("p_index", "<u4"), ("realization", "<u4"), ("p", "<f8"), ("rho", "<f8", (S * 2 * D * D,))])
    n = meta["record_count"]
    if len(data) - off != n * rec.itemsize:
        raise ValueError(f"file holds {(len(data) - off) / rec.itemsize} records, header says {n}")
    raw = np.frombuffer(data, rec, n, off)
    rho = raw["rho"].reshape(n, S, D, D, 2)
    records = dict(p_index=raw["p_index"].copy(), realization=raw["realization"].copy(), p=raw["p"].copy(),
                   rho=rho[..., 0] + 1j * rho[..., 1])
    return meta, records
