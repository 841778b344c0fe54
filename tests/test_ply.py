"""CPU tests of scene ingestion: lrx_ply_load (ascii and both binary byte
orders; triangles kept, quads split (0,1,2)+(0,2,3), other polygons dropped,
other properties and elements skipped -- the geometry semantics of the
reference's ExtTriangleMesh::LoadPly, exttrianglemeshfile.cpp:207-290) and
lrx_scene_key (equal inputs, equal keys)."""
import struct

import numpy as np
import pytest

from luxcore_gb300 import build, lrx
from luxcore_gb300 import workloads as W


@pytest.fixture(scope="module", autouse=True)
def lib():
    build.build()
    return lrx.load()


VERTS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0.5, 0.5, 1], [2, 2, 2]], np.float64)
FACES = [[0, 1, 2], [0, 2, 3, 4], [0, 1, 2, 3, 5], [3, 4, 5]]   # tri, quad, pentagon (dropped), tri
EXPECT = np.array([[0, 1, 2], [0, 2, 3], [0, 3, 4], [3, 4, 5]], np.uint32)


def write_ply(path, fmt, vtype="float", itype="int", ctype="uchar", extras=True):
    codes = {"float": "f", "double": "d", "int": "i", "uint": "I", "uchar": "B", "ushort": "H", "short": "h"}
    head = ["ply", f"format {fmt} 1.0", "comment made by the tests"]
    head += [f"element vertex {len(VERTS)}", f"property {vtype} x", f"property {vtype} y", f"property {vtype} z"]
    if extras:
        head += ["property float nx", "property uchar red"]
    head += [f"element face {len(FACES)}", f"property list {ctype} {itype} vertex_indices"]
    if extras:
        head += ["property float area", "element edge 2", "property int vertex1", "property int vertex2"]
    head += ["end_header"]
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        if fmt == "ascii":
            for v in VERTS:
                f.write((" ".join(repr(float(x)) for x in v) + (" 0.5 7" if extras else "") + "\n").encode())
            for fc in FACES:
                f.write((f"{len(fc)} " + " ".join(map(str, fc)) + (" 1.25" if extras else "") + "\n").encode())
            if extras:
                f.write(b"0 1\n1 2\n")
            return
        e = "<" if fmt == "binary_little_endian" else ">"
        for v in VERTS:
            f.write(struct.pack(e + codes[vtype] * 3, *v))
            if extras:
                f.write(struct.pack(e + "fB", 0.5, 7))
        for fc in FACES:
            f.write(struct.pack(e + codes[ctype], len(fc)))
            f.write(struct.pack(e + codes[itype] * len(fc), *fc))
            if extras:
                f.write(struct.pack(e + "f", 1.25))
        if extras:
            f.write(struct.pack(e + "iiii", 0, 1, 1, 2))


@pytest.mark.parametrize("fmt", ["ascii", "binary_little_endian", "binary_big_endian"])
@pytest.mark.parametrize("vtype,itype,ctype", [("float", "int", "uchar"), ("double", "uint", "ushort"),
                                               ("float", "ushort", "uchar")])
def test_ply_formats_and_types(tmp_path, fmt, vtype, itype, ctype):
    p = tmp_path / "m.ply"
    write_ply(str(p), fmt, vtype, itype, ctype)
    m = lrx.ply_load(str(p))
    assert m.vertices.dtype == np.float32 and m.vertices.shape == VERTS.shape
    assert np.array_equal(m.vertices, VERTS.astype(np.float32))
    assert np.array_equal(m.triangles, EXPECT)


def test_ply_without_extra_properties(tmp_path):
    p = tmp_path / "plain.ply"
    write_ply(str(p), "binary_little_endian", extras=False)
    m = lrx.ply_load(str(p))
    assert np.array_equal(m.triangles, EXPECT)


def test_ply_errors(tmp_path):
    with pytest.raises(lrx.LrxError):
        lrx.ply_load(str(tmp_path / "missing.ply"))
    bad = tmp_path / "bad.ply"
    bad.write_bytes(b"not a ply\n")
    with pytest.raises(lrx.LrxError):
        lrx.ply_load(str(bad))
    full = tmp_path / "full.ply"
    write_ply(str(full), "binary_little_endian")
    trunc = tmp_path / "trunc.ply"
    trunc.write_bytes(full.read_bytes()[:-20])
    with pytest.raises(lrx.LrxError, match="parse"):
        lrx.ply_load(str(trunc))
    nofaces = tmp_path / "nofaces.ply"
    nofaces.write_bytes(b"ply\nformat ascii 1.0\nelement vertex 1\nproperty float x\nproperty float y\n"
                        b"property float z\nend_header\n0 0 0\n")
    with pytest.raises(lrx.LrxError, match="no faces"):
        lrx.ply_load(str(nofaces))


def test_scene_key_tracks_inputs():
    a = W.SceneDesc([W.random_triangles(1000, 1), W.random_triangles(500, 2)])
    b = W.SceneDesc([W.random_triangles(1000, 1), W.random_triangles(500, 2)])
    assert lrx.scene_key(a) == lrx.scene_key(b)
    c = W.SceneDesc([W.random_triangles(1000, 1), W.random_triangles(500, 2)])
    c.meshes[1].vertices[7, 2] += 1e-3
    assert lrx.scene_key(c) != lrx.scene_key(a)
    assert lrx.scene_key(a, treelet_passes=0) != lrx.scene_key(a)
    m = np.eye(4, dtype=np.float32)
    i1 = W.SceneDesc(a.meshes, [(0, None), (1, m)])
    m2 = m.copy()
    m2[0, 3] = 0.5
    i2 = W.SceneDesc(a.meshes, [(0, None), (1, m2)])
    assert lrx.scene_key(i1) != lrx.scene_key(i2)
