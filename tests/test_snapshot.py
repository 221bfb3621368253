"""Snapshot file format (nb_snapshot_write / nb_snapshot_read): host code,
no GPU.  Round trip, the byte layout of the header and the float payload
(little-endian), and the refusals."""
import struct

import numpy as np
import pytest


def test_round_trip_and_layout(nbgb_lib, tmp_path):
    nb = nbgb_lib
    rng = np.random.default_rng(5)
    n = 1000
    pos = rng.normal(size=(n, 3)).astype(np.float32)
    vel = rng.normal(size=(n, 3)).astype(np.float32)
    mass = rng.random(n).astype(np.float32)
    path = tmp_path / "s.nbsnap"
    nb.write_snapshot(path, pos, mass, vel, step=1234567890123, time=0.125)
    raw = path.read_bytes()
    assert len(raw) == 32 + 28 * n
    magic, ver, count, step, t = struct.unpack("<8sIIqd", raw[:32])
    assert (magic, ver, count, step, t) == (b"NBSNAP01", 1, n, 1234567890123, 0.125)
    np.testing.assert_array_equal(np.frombuffer(raw[32:32 + 12 * n], "<f4").reshape(n, 3), pos)
    np.testing.assert_array_equal(np.frombuffer(raw[32 + 24 * n:], "<f4"), mass)
    s, tt, p2, v2, m2 = nb.read_snapshot(path)
    assert s == 1234567890123 and tt == 0.125
    np.testing.assert_array_equal(p2, pos)
    np.testing.assert_array_equal(v2, vel)
    np.testing.assert_array_equal(m2, mass)


def test_zero_velocities_and_refusals(nbgb_lib, tmp_path):
    nb = nbgb_lib
    import ctypes
    pos = np.ones((3, 3), np.float32)
    mass = np.ones(3, np.float32)
    path = tmp_path / "z.nbsnap"
    nb.write_snapshot(path, pos, mass)
    _, _, _, v, _ = nb.read_snapshot(path)
    assert not v.any()
    bad = tmp_path / "bad.nbsnap"
    bad.write_bytes(b"NOTASNAP" + bytes(24))
    with pytest.raises(nb.NbError):
        nb.read_snapshot(bad)
    # a buffer smaller than N is refused
    L = nb.load()
    n = ctypes.c_int32(0)
    small = np.zeros(3, np.float32)
    st = L.nb_snapshot_read(str(path).encode(), None, None, small.ctypes.data, None, None, 1, ctypes.byref(n))
    assert st == 1 and n.value == 3
    with pytest.raises(nb.NbError):
        nb.read_snapshot(tmp_path / "missing.nbsnap")
