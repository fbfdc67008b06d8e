"""The reference's on-disk formats (nslsm.io): Fortran unformatted sequential
framing (gfortran), the `grid` and `phi_ini` decks and the `phi.NNN`
restart files.  CPU only."""
import os
import struct

import numpy as np
import pytest

from nslsm import io


def test_record_framing_bytes(tmp_path):
    p = str(tmp_path / "f")
    a = np.array([1.5, -2.0])
    io.write_records(p, [a.astype("<f8").tobytes(), b""])
    raw = open(p, "rb").read()
    assert raw[:4] == struct.pack("<i", 16) and raw[20:24] == struct.pack("<i", 16)
    assert np.frombuffer(raw[4:20], "<f8").tolist() == [1.5, -2.0]
    assert raw[24:] == struct.pack("<i", 0) * 2
    assert io.read_records(p) == [a.astype("<f8").tobytes(), b""]


def test_subrecords_round_trip(tmp_path):
    p = str(tmp_path / "f")
    rec = bytes(range(100))
    io.write_records(p, [rec, b"xy"], max_subrecord=24)
    raw = open(p, "rb").read()
    # five subrecords (24, 24, 24, 24, 4): leading markers negative but the last,
    # trailing markers negative but the first
    heads = []
    pos = 0
    for _ in range(5):
        (h,) = struct.unpack_from("<i", raw, pos)
        (t,) = struct.unpack_from("<i", raw, pos + 4 + abs(h))
        heads.append((h, t))
        pos += 8 + abs(h)
    assert heads == [(-24, 24), (-24, -24), (-24, -24), (-24, -24), (4, -4)]
    assert io.read_records(p) == [rec, b"xy"]


def test_bad_markers_are_reported(tmp_path):
    p = str(tmp_path / "f")
    with open(p, "wb") as f:
        f.write(struct.pack("<i", 8) + b"\0" * 8 + struct.pack("<i", 7))
    with pytest.raises(ValueError):
        io.read_records(p)


def test_grid_and_phi_ini_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    zones = [(5, 4, 3), (3, 6, 2)]
    grid = [tuple(np.asfortranarray(rng.standard_normal(s)) for _ in range(4)) for s in zones]
    io.write_grid(str(tmp_path / "grid"), [g[:3] for g in grid])
    back = io.read_grid(str(tmp_path / "grid"), zones)
    for g, b in zip(grid, back):
        assert all(np.array_equal(u, v) for u, v in zip(g[:3], b)) and b[0].flags.f_contiguous
    io.write_grid(str(tmp_path / "grid_t"), grid)
    back = io.read_grid(str(tmp_path / "grid_t"), zones, turbulence=True)
    assert all(np.array_equal(u, v) for g, b in zip(grid, back) for u, v in zip(g, b))
    phis = [(np.asfortranarray(rng.standard_normal(s)), np.asfortranarray(rng.standard_normal(s))) for s in zones]
    io.write_phi_ini(str(tmp_path / "phi_ini"), phis)
    back = io.read_phi_ini(str(tmp_path / "phi_ini"), zones)
    assert all(np.array_equal(u, v) for p, b in zip(phis, back) for u, v in zip(p, b))
    with pytest.raises(ValueError):
        io.read_phi_ini(str(tmp_path / "phi_ini"), [(5, 4, 4)])


def test_restart_strips_ghosts_and_names_the_rank(tmp_path):
    rng = np.random.default_rng(1)
    phi = np.asfortranarray(rng.standard_normal((10, 9, 6)))
    phin = np.asfortranarray(rng.standard_normal((10, 9, 6)))
    path = io.write_phi_restart(str(tmp_path) + os.sep, 7, phi, phin, ghost=(2, 2, 0))
    assert path.endswith(os.path.join("solufiles", "phi.007"))
    a, b = io.read_phi_restart(path, (6, 5, 6))
    assert np.array_equal(a, phi[2:8, 2:7, :]) and np.array_equal(b, phin[2:8, 2:7, :])
