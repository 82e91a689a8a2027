"""Mesh files (gm_mesh_store, host only): OFF in the reference's text form,
PN (float32 position + normal) and binary PLY, with and without dropping
unused vertices."""
import struct

import numpy as np

from broxy_gb300 import api


def _mesh():
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [5, 5, 5]], np.float32) * 0.25
    N = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0]], np.float32)
    T = np.array([[0, 1, 2], [0, 2, 3], [1, 3, 2]], np.uint32)
    return V, N, T


def _read_off(path):
    tok = open(path).read().split()
    assert tok[0] == "OFF"
    nv, nf = int(tok[1]), int(tok[2])
    vals = tok[4:]
    V = np.array(vals[:3 * nv], np.float32).reshape(nv, 3)
    F = np.array(vals[3 * nv:3 * nv + 4 * nf], np.int64).reshape(nf, 4)
    assert (F[:, 0] == 3).all()
    return V, F[:, 1:]


def test_off_roundtrip(tmp_path):
    V, N, T = _mesh()
    p = tmp_path / "m.off"
    api.store_mesh(p, V, None, T)
    V2, T2 = _read_off(p)
    assert np.array_equal(V2, V) and np.array_equal(T2, T)


def test_off_drop_unused(tmp_path):
    V, N, T = _mesh()
    p = tmp_path / "m.off"
    api.store_mesh(p, V, N, T, drop_unused=True)
    V2, T2 = _read_off(p)
    assert V2.shape == (4, 3) and np.array_equal(V2, V[:4]) and np.array_equal(T2, T)


def test_pn(tmp_path):
    V, N, T = _mesh()
    p = tmp_path / "m.pn"
    api.store_mesh(p, V, N, T)
    a = np.fromfile(p, np.float32).reshape(-1, 6)
    assert np.array_equal(a[:, :3], V) and np.array_equal(a[:, 3:], N)


def test_ply_binary(tmp_path):
    V, N, T = _mesh()
    p = tmp_path / "m.ply"
    api.store_mesh(p, V, N, T, drop_unused=True)
    raw = open(p, "rb").read()
    end = raw.index(b"end_header\n") + len(b"end_header\n")
    head = raw[:end].decode()
    assert "format binary_little_endian 1.0" in head and "element vertex 4" in head and "element face 3" in head
    body = raw[end:]
    verts = np.frombuffer(body[:4 * 24], "<f4").reshape(4, 6)
    assert np.array_equal(verts[:, :3], V[:4]) and np.array_equal(verts[:, 3:], N[:4])
    faces = body[4 * 24:]
    assert len(faces) == 3 * 13
    for i in range(3):
        n, a, b, c = struct.unpack("<BIII", faces[13 * i:13 * i + 13])
        assert n == 3 and (a, b, c) == tuple(T[i])


def test_bad_arguments(tmp_path):
    import pytest
    V, N, T = _mesh()
    with pytest.raises(Exception):
        api.store_mesh(tmp_path / "m.xyz", V, N, T)
    with pytest.raises(Exception):
        api.store_mesh(tmp_path / "m.off", V, N, np.array([[0, 1, 9]], np.uint32))
