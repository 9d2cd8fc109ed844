"""Gadget-1 glass / snapshot files and the potential dumps of the 2LPT code.

Formats follow the reference:
  - io_header_1, 256 bytes (Aarambam/LPT/Basis/allvars.h:27-49), written
    between 4-byte Fortran record markers;
  - glass files: header record then a positions record of float32 triplets,
    optionally split over <name>.0, <name>.1, ... (read_glass.c:10-84,
    find_files read_glass.c:226-260);
  - snapshots: header, Pos float32[3n], Vel float32[3n], ID int32[n]
    (NO64BITID build, save.c:162-520);
  - potential dumps: int total_size, int Nmesh, double Box, then N^3 records
    (int coord, double value) with coord = (i*N + j)*2*(N/2+1) + k
    (write_phi, save.c:14-105).
"""
from __future__ import annotations

import os
import struct

import numpy as np

HEADER_DTYPE = np.dtype([
    ("npart", "<u4", 6), ("mass", "<f8", 6), ("time", "<f8"), ("redshift", "<f8"),
    ("flag_sfr", "<i4"), ("flag_feedback", "<i4"), ("npartTotal", "<u4", 6), ("flag_cooling", "<i4"),
    ("num_files", "<i4"), ("BoxSize", "<f8"), ("Omega0", "<f8"), ("OmegaLambda", "<f8"),
    ("HubbleParam", "<f8"), ("flag_stellarage", "<i4"), ("flag_metals", "<i4"), ("hashtabsize", "<i4"),
    ("fill", "u1", 84),
])
assert HEADER_DTYPE.itemsize == 256


class GadgetError(Exception):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def _read_record(f, what: str) -> bytes:
    raw = f.read(4)
    if len(raw) != 4:
        raise GadgetError(778, f"I/O error (fread) reading {what}")
    (n,) = struct.unpack("<I", raw)
    data = f.read(n)
    tail = f.read(4)
    if len(data) != n or len(tail) != 4:
        raise GadgetError(778, f"I/O error (fread) reading {what}")
    (n2,) = struct.unpack("<I", tail)
    if n2 != n:
        raise GadgetError(3, f"record markers disagree in {what}")
    return data


def _write_record(f, payload: bytes) -> None:
    f.write(struct.pack("<I", len(payload)))
    f.write(payload)
    f.write(struct.pack("<I", len(payload)))


def make_header(**kw) -> np.ndarray:
    h = np.zeros((), dtype=HEADER_DTYPE)
    for k, v in kw.items():
        h[k] = v
    return h


def glass_files(fname: str) -> list:
    """The file list find_files (read_glass.c:226-260) would use."""
    first = f"{fname}.0"
    if os.path.exists(first):
        with open(first, "rb") as f:
            h = np.frombuffer(_read_record(f, "glass header"), dtype=HEADER_DTYPE)[0]
        n = int(h["num_files"])
        return [f"{fname}.{i}" for i in range(n)] if n > 1 else [fname]
    if os.path.exists(fname):
        return [fname]
    raise GadgetError(121, f"can't find glass file '{fname}'")


def read_glass(fname: str):
    """Return (positions float32 [n,3], header of the first file)."""
    files = glass_files(fname)
    chunks = []
    header0 = None
    for path in files:
        try:
            f = open(path, "rb")
        except OSError:
            raise GadgetError(1, f"can't open file `{path}' for reading glass file.") from None
        with f:
            raw = _read_record(f, "glass header")
            if len(raw) != 256:
                raise GadgetError(2, "incorrect header size!")
            h = np.frombuffer(raw, dtype=HEADER_DTYPE)[0]
            nlocal = int(np.sum(h["npart"].astype(np.int64)))
            pos = _read_record(f, "glass positions")
            if len(pos) != 12 * nlocal:
                raise GadgetError(3, "incorrect block structure in positions block!")
            chunks.append(np.frombuffer(pos, dtype="<f4").reshape(-1, 3))
            if header0 is None:
                header0 = h
    ntot = int(np.sum(header0["npartTotal"].astype(np.int64)))
    pos = np.concatenate(chunks, axis=0)
    if pos.shape[0] != ntot:
        raise GadgetError(3, "glass particle count does not match npartTotal")
    return np.ascontiguousarray(pos), header0


def write_glass(fname: str, pos: np.ndarray, box: float) -> None:
    pos = np.ascontiguousarray(pos, dtype="<f4").reshape(-1, 3)
    n = pos.shape[0]
    h = make_header(npart=[0, n, 0, 0, 0, 0], npartTotal=[0, n, 0, 0, 0, 0], num_files=1, BoxSize=box)
    with open(fname, "wb") as f:
        _write_record(f, h.tobytes())
        _write_record(f, pos.tobytes())


def lattice_glass(n: int, box: float) -> np.ndarray:
    """A regular n^3 lattice (the layout of the reference's default glass)."""
    g = (np.arange(n, dtype=np.float64) * (box / n)).astype(np.float32)
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)


def write_snapshot(fname: str, header: np.ndarray, pos: np.ndarray, vel: np.ndarray, ids: np.ndarray) -> None:
    """Gadget-1 snapshot with 32-bit IDs (save.c:162-520, NO64BITID)."""
    with open(fname, "wb") as f:
        _write_record(f, header.tobytes())
        _write_record(f, np.ascontiguousarray(pos, dtype="<f4").tobytes())
        _write_record(f, np.ascontiguousarray(vel, dtype="<f4").tobytes())
        _write_record(f, np.ascontiguousarray(ids, dtype="<i4").tobytes())


def read_snapshot(fname: str):
    with open(fname, "rb") as f:
        h = np.frombuffer(_read_record(f, "header"), dtype=HEADER_DTYPE)[0]
        pos = np.frombuffer(_read_record(f, "positions"), dtype="<f4").reshape(-1, 3)
        vel = np.frombuffer(_read_record(f, "velocities"), dtype="<f4").reshape(-1, 3)
        ids = np.frombuffer(_read_record(f, "ids"), dtype="<i4")
    return h, pos, vel, ids


POT_DTYPE = np.dtype([("coord", "<i4"), ("val", "<f8")])


def write_potential(fname: str, field: np.ndarray, box: float) -> None:
    """Potential dump in write_phi's record layout (save.c:64-98)."""
    n = field.shape[0]
    total = n * n * 2 * (n // 2 + 1) + n * 2 * (n // 2 + 1)  # TotalSizePlusAdditional
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    rec = np.empty(n**3, dtype=POT_DTYPE)
    rec["coord"] = ((i * n + j) * (2 * (n // 2 + 1)) + k).ravel()
    rec["val"] = np.asarray(field, dtype=np.float64).ravel()
    with open(fname, "wb") as f:
        f.write(struct.pack("<iid", np.int32(total).item() if total < 2**31 else total - 2**32, n, box))
        f.write(rec.tobytes())


def read_potential(fname: str):
    with open(fname, "rb") as f:
        total, n, box = struct.unpack("<iid", f.read(16))
        rec = np.frombuffer(f.read(), dtype=POT_DTYPE)
    return rec["val"].reshape(n, n, n), n, box
