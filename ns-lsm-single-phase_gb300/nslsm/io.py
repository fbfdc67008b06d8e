"""The reference's on-disk formats that feed and checkpoint the level-set path.

All three are Fortran unformatted sequential files (gfortran's layout: each
record is framed by its byte length as a 4-byte little-endian integer before
and after the data; a record longer than 2**31 - 1 bytes is written as
subrecords whose leading marker is negative for every subrecord but the
last) holding REAL(8) arrays in Fortran order (i fastest):

  grid      per zone: x, y, z records (img x jmg x kmg each), and a wall
            distance record when the turbulence model is on
            (src/init.F90:1863-1876)
  phi_ini   per zone: phi, then phi_n (src/init_LSM.F90:373-385)
  phi.NNN   restart of rank NNN (zero-padded to three digits) under
            `<dirOUT>solufiles/`: phi, then phi_n, ghost planes stripped
            (output_restart_lsm, src/main.F90:404-455)

The ind3dmg_LSM.dat deck is read by nslsm.params.read_ind3dmg_lsm.
"""
from __future__ import annotations

import os
import struct
from typing import List, Sequence, Tuple

import numpy as np

_MAX = 2 ** 31 - 1


def read_records(path: str) -> List[bytes]:
    """Every record of a Fortran unformatted sequential file (subrecords joined)."""
    out = []
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        chunks = []
        while True:
            if pos + 4 > len(data):
                raise ValueError(f"{path}: truncated record marker at byte {pos}")
            (head,) = struct.unpack_from("<i", data, pos)
            n = abs(head)
            body = data[pos + 4: pos + 4 + n]
            if len(body) != n:
                raise ValueError(f"{path}: truncated record at byte {pos}")
            (tail,) = struct.unpack_from("<i", data, pos + 4 + n)
            if abs(tail) != n:
                raise ValueError(f"{path}: record markers {head} / {tail} disagree at byte {pos}")
            chunks.append(body)
            pos += 8 + n
            if head >= 0:          # the last (or only) subrecord
                break
        out.append(b"".join(chunks))
    return out


def write_records(path: str, records: Sequence[bytes], max_subrecord: int = _MAX) -> None:
    """Write records with gfortran's framing (long ones split in subrecords)."""
    with open(path, "wb") as f:
        for rec in records:
            rec = bytes(rec)
            parts = [rec[i:i + max_subrecord] for i in range(0, len(rec), max_subrecord)] or [b""]
            for q, part in enumerate(parts):
                last = q == len(parts) - 1
                # gfortran: the leading marker of a continued record is negative,
                # the trailing marker of a subrecord other than the first too
                head = len(part) if last else -len(part)
                tail = len(part) if q == 0 else -len(part)
                f.write(struct.pack("<i", head))
                f.write(part)
                f.write(struct.pack("<i", tail))


def _real8(rec: bytes, shape: Tuple[int, int, int], what: str) -> np.ndarray:
    n = int(np.prod(shape))
    if len(rec) != 8 * n:
        raise ValueError(f"{what}: record holds {len(rec) // 8} values, expected {n} for {shape}")
    return np.frombuffer(rec, dtype="<f8").reshape(shape, order="F").astype(np.float64).copy(order="F")


def _rec(a: np.ndarray) -> bytes:
    return np.asfortranarray(a, dtype="<f8").tobytes(order="F")


def read_grid(path: str, zones: Sequence[Tuple[int, int, int]], turbulence: bool = False):
    """-> list per zone of (x, y, z) (plus the wall distance when `turbulence`)."""
    recs = read_records(path)
    per = 4 if turbulence else 3
    if len(recs) < per * len(zones):
        raise ValueError(f"{path}: {len(recs)} records for {len(zones)} zones")
    out = []
    for z, shp in enumerate(zones):
        out.append(tuple(_real8(recs[per * z + c], shp, f"{path} zone {z + 1}") for c in range(per)))
    return out


def write_grid(path: str, zones: Sequence[Sequence[np.ndarray]]) -> None:
    write_records(path, [_rec(a) for zone in zones for a in zone])


def read_phi_ini(path: str, zones: Sequence[Tuple[int, int, int]]):
    """-> list per zone of (phi, phi_n)."""
    recs = read_records(path)
    if len(recs) < 2 * len(zones):
        raise ValueError(f"{path}: {len(recs)} records for {len(zones)} zones")
    return [(_real8(recs[2 * z], shp, f"{path} phi zone {z + 1}"),
             _real8(recs[2 * z + 1], shp, f"{path} phi_n zone {z + 1}")) for z, shp in enumerate(zones)]


def write_phi_ini(path: str, zones: Sequence[Tuple[np.ndarray, np.ndarray]]) -> None:
    write_records(path, [_rec(a) for pz in zones for a in pz])


def restart_path(dir_out: str, rank: int) -> str:
    """`<dirOUT>solufiles/phi.NNN` as output_restart_lsm builds it (i3.3)."""
    return os.path.join(dir_out, "solufiles", "phi.%03d" % rank)


def _strip(a: np.ndarray, gp: Tuple[int, int, int]) -> np.ndarray:
    gi, gj, gk = gp
    ni, nj, nk = a.shape
    return a[gi:ni - gi, gj:nj - gj, gk:nk - gk]


def write_phi_restart(dir_out: str, rank: int, phi: np.ndarray, phi_n: np.ndarray,
                      ghost: Tuple[int, int, int] = (0, 0, 0)) -> str:
    """Write phi and phi_n of one rank with `ghost` planes stripped per side."""
    path = restart_path(dir_out, rank)
    os.makedirs(os.path.dirname(path), exist_ok=True)
    write_records(path, [_rec(_strip(phi, ghost)), _rec(_strip(phi_n, ghost))])
    return path


def read_phi_restart(path: str, shape: Tuple[int, int, int]):
    """-> (phi, phi_n) of one rank's restart file (ghost-free shape)."""
    recs = read_records(path)
    if len(recs) != 2:
        raise ValueError(f"{path}: {len(recs)} records, expected 2")
    return _real8(recs[0], shape, path), _real8(recs[1], shape, path)
