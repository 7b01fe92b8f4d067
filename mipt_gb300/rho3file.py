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


def write(path, rho, p, p_index, realization=None, *, total_qubits=0, periods=0, realizations=0, resolution=None,
          p_min=None, p_max=None, subsystem_qubits=None, spatial_dimension=1, grid_x=None, grid_y=1):
    """Writes records rho[n][S][D][D] (complex) with per-record p and p_index
    in the same version-2 layout (the inverse of read)."""
    rho = np.asarray(rho, np.complex128)
    n, S, D = rho.shape[0], rho.shape[1], rho.shape[2]
    K = D.bit_length() - 1
    if D != 1 << K or rho.shape[3] != D:
        raise ValueError("rho must be [n][S][D][D] with D a power of two")
    p = np.asarray(p, np.float64).reshape(n)
    p_index = np.asarray(p_index, np.uint32).reshape(n)
    realization = np.zeros(n, np.uint32) if realization is None else np.asarray(realization, np.uint32).reshape(n)
    if subsystem_qubits is None:
        subsystem_qubits = np.arange(S * K, dtype=np.uint32).reshape(S, K)
    subsystem_qubits = np.asarray(subsystem_qubits, np.uint32).reshape(S, K)
    resolution = int(p_index.max()) + 1 if resolution is None else resolution
    p_min = float(p.min()) if p_min is None else p_min
    p_max = float(p.max()) if p_max is None else p_max
    grid_x = total_qubits if grid_x is None else grid_x
    head = MAGIC + struct.pack("<II", 0x01020304, 2)
    head += struct.pack("<10I", spatial_dimension, total_qubits, K, D, periods, realizations, resolution, grid_x,
                        grid_y, S)
    head += struct.pack("<Q", n) + struct.pack("<dd", p_min, p_max) + subsystem_qubits.tobytes()
    rec = np.dtype([("p_index", "<u4"), ("realization", "<u4"), ("p", "<f8"), ("rho", "<f8", (S * 2 * D * D,))])
    out = np.zeros(n, rec)
    out["p_index"], out["realization"], out["p"] = p_index, realization, p
    out["rho"] = np.stack([rho.real, rho.imag], -1).reshape(n, -1)
    with open(path, "wb") as f:
        f.write(head)
        f.write(out.tobytes())
