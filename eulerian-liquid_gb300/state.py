"""State files of el_state_save / el_state_load, read and written on the host with numpy.

Layout (little-endian): a 64-byte header -- magic "ELGBSTAT", uint32 version 1, uint32 dtype
(0 = FP32, 1 = FP64), int32 ni, nj, nk, uint32 field count, float64 dx, float64 time, 16 zero
bytes -- then per field: uint32 field id, uint32 element bytes, uint64 byte count and the
field's bytes (i-fastest, the layout of el_upload).  Used to restart a run exactly, to hand a
GPU state to the CPU oracle, and to keep recorded scenes."""

import struct

import numpy as np

MAGIC = b"ELGBSTAT"
HEADER = struct.Struct("<8sIIiiiIdd16s")
RECORD = struct.Struct("<IIQ")
FIELD_NAMES = ["phi", "u", "v", "w", "solid_nodal", "weight_u", "weight_v", "weight_w", "pressure",
               "solid_cell", "valid_u", "valid_v", "valid_w", "valid_phi", "indices"]


def field_shape(name, ni, nj, nk):
    if name in ("u", "weight_u", "valid_u"):
        return (nk, nj, ni + 1)
    if name in ("v", "weight_v", "valid_v"):
        return (nk, nj + 1, ni)
    if name in ("w", "weight_w", "valid_w"):
        return (nk + 1, nj, ni)
    if name == "solid_nodal":
        return (nk + 1, nj + 1, ni + 1)
    return (nk, nj, ni)


def field_dtype(name, dtype):
    if name.startswith("valid"):
        return np.dtype(np.uint8)
    if name == "indices":
        return np.dtype(np.int32)
    return np.dtype(np.float64 if dtype == 1 else np.float32)


def read_state(path):
    """Returns {"ni", "nj", "nk", "dx", "time", "dtype", "fields": {name: array}}."""
    with open(path, "rb") as f:
        raw = f.read()
    if len(raw) < HEADER.size:
        raise ValueError("truncated state file")
    magic, version, dtype, ni, nj, nk, nfields, dx, time, _ = HEADER.unpack_from(raw, 0)
    if magic != MAGIC or version != 1:
        raise ValueError("not a state file (magic or version)")
    off = HEADER.size
    fields = {}
    for _ in range(nfields):
        if off + RECORD.size > len(raw):
            raise ValueError("truncated state file")
        fid, elem, nbytes = RECORD.unpack_from(raw, off)
        off += RECORD.size
        if fid >= len(FIELD_NAMES) or off + nbytes > len(raw):
            raise ValueError("bad field record")
        name = FIELD_NAMES[fid]
        dt = field_dtype(name, dtype)
        shape = field_shape(name, ni, nj, nk)
        if dt.itemsize != elem or int(np.prod(shape)) * elem != nbytes:
            raise ValueError(f"bad field record {name}")
        fields[name] = np.frombuffer(raw, dtype=dt, count=int(np.prod(shape)), offset=off).reshape(shape).copy()
        off += nbytes
    return {"ni": ni, "nj": nj, "nk": nk, "dx": dx, "time": time, "dtype": dtype, "fields": fields}


def write_state(path, ni, nj, nk, dx, dtype, fields, time=0.0):
    """Writes the given fields ({name: array}) in the state format (any subset; el_state_load
    leaves the others as they are)."""
    recs = []
    for name, a in fields.items():
        fid = FIELD_NAMES.index(name)
        dt = field_dtype(name, dtype)
        a = np.ascontiguousarray(a, dtype=dt)
        if a.shape != field_shape(name, ni, nj, nk):
            raise ValueError(f"{name}: shape {a.shape}")
        recs.append(RECORD.pack(fid, dt.itemsize, a.nbytes) + a.tobytes())
    with open(path, "wb") as f:
        f.write(HEADER.pack(MAGIC, 1, dtype, ni, nj, nk, len(recs), float(dx), float(time), bytes(16)))
        for r in recs:
            f.write(r)
