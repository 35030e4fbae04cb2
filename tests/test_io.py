"""Scene and film I/O without a GPU: the library's OBJ reader against the Python restatement of
OBJ::read (src/io/obj.rs:16-123), its error cases, and the EXR writer / reader round trip."""
import struct
from pathlib import Path

import numpy as np
import pytest

from bonsai_gb300 import io as bio
from oracle import obj as OO

OBJ_TEXT = """# comment line
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0.5 0.25 0.75 0.5
vt 0 0
vt 1 0
vt 1 1
vn 0 0 1
vn 0 0 -1
  v   2.5e-1 -3 1e2
f 1 2 3
f 1/1 2/2 4/3
f 3//1 4//2 5//1
f 1/1/1 3/3/2 5/2/1
o ignored object name
g group
s off
f 2 3 4 5
f 1 2
"""


def _write(tmp_path, text, name="m.obj"):
    p = tmp_path / name
    p.write_text(text)
    return p


@pytest.mark.parametrize("xf", [None, np.array([[0.5, 0, 0, 1], [0, 2, 0, -1], [0.25, 0, 1, 3]], np.float32),
                                np.array([[0, -1, 0, 0.3], [1, 0, 0, 0.1], [0, 0, 1, -0.7]], np.float32)])
def test_obj_matches_reference_rules(tmp_path, xf):
    p = _write(tmp_path, OBJ_TEXT)
    got = bio.read_obj(p, xf)
    want = OO.read_obj(p, xf)
    # 18 face indices -> 6 triangles (the quad and the 2-index face shift the triples, as in the reference)
    assert got.shape == want.shape == (6, 9)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("text", [
    "v 0 0 0\nf 1 2 3\n",            # index past the end
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n",  # index 0
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 -3\n",  # negative index
    "v 0 0\n",                         # too few values
    "v 0 0 x\n",                       # bad number
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1/ 2 3\n",  # empty texture index
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1//4 2 3\n",  # normal index past the end
])
def test_obj_errors(tmp_path, text):
    p = _write(tmp_path, text)
    with pytest.raises(ValueError):
        OO.read_obj(p)
    with pytest.raises(ValueError):
        bio.read_obj(p)


MESH_TEXT = """v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 1
vn 0.1 0 0.9
vn 0 0.2 0.8
f 1/1/1 2/2/2 3/3/3
f 1/1/1 3/3/3 4/4/2
"""


@pytest.mark.parametrize("xf", [None, np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32),
                                np.array([[0.5, 0.1, 0, 1], [0, 2, 0.3, -1], [0.25, 0, 1, 3]], np.float32),
                                np.array([[-1, 0, 0, 0.3], [0, 1, 0, 0.1], [0, 0, 1, -0.7]], np.float32)])
def test_obj_mesh_attributes_match_reference_rules(tmp_path, xf):
    p = _write(tmp_path, MESH_TEXT)
    tri, nrm, uv, flags = bio.read_obj_mesh(p, xf)
    wt, wn, wuv, wswap = OO.read_obj_mesh(p, xf)
    np.testing.assert_array_equal(tri, wt)
    np.testing.assert_array_equal(nrm, wn)
    np.testing.assert_array_equal(uv, wuv)
    assert uv[1].tolist() == [0, 0, 1, 1, 0, 1]
    assert bool(flags & 2) == wswap == (xf is not None and np.linalg.det(xf[:, :3]) < 0)


def test_obj_mesh_positions_only(tmp_path):
    p = _write(tmp_path, "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    tri, nrm, uv, flags = bio.read_obj_mesh(p)
    assert tri.shape == (1, 9) and nrm is None and uv is None and flags == 0


def test_obj_mesh_rejects_partial_normals(tmp_path):
    # the second face has no normals: the reference would index past its normal list
    p = _write(tmp_path, "v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\nf 1 2 3\n")
    with pytest.raises(ValueError):
        OO.read_obj_mesh(p)
    with pytest.raises(ValueError, match="normal indices"):
        bio.read_obj_mesh(p)


def test_obj_missing_file(tmp_path):
    with pytest.raises(ValueError, match="cannot open"):
        bio.read_obj(tmp_path / "nope.obj")


def test_obj_empty(tmp_path):
    p = _write(tmp_path, "# nothing\n")
    assert bio.read_obj(p).shape == (0, 9)


def test_exr_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.normal(0, 10, (37, 53, 3)).astype(np.float32)
    img[0, 0] = [np.inf, 0.0, -0.0]
    p = tmp_path / "a.exr"
    bio.write_exr(p, img)
    data = p.read_bytes()
    assert struct.unpack_from("<II", data, 0) == (20000630, 2)
    for key in (b"channels\0chlist\0", b"compression\0compression\0", b"dataWindow\0box2i\0", b"lineOrder\0lineOrder\0"):
        assert key in data
    back = bio.read_exr(p)
    assert back.shape == img.shape
    np.testing.assert_array_equal(back, img)


def test_exr_matches_the_spec_fixture(tmp_path):
    """The writer's bytes for a 2 x 2 image equal tests/golden/exr_2x2.bin, which
    tests/golden/make_exr_fixture.py spells out field by field from the OpenEXR file layout
    (independent of this package's reader and of the library's writer)."""
    img = np.zeros((2, 2, 3), np.float32)
    for y in range(2):
        for x in range(2):
            r = 1.0 + x + 2 * y
            img[y, x] = (r, 10 * r, 100 * r)
    p = tmp_path / "fixture.exr"
    bio.write_exr(p, img)
    want = (Path(__file__).resolve().parent / "golden" / "exr_2x2.bin").read_bytes()
    assert p.read_bytes() == want


def test_exr_rejects_bad_arguments(tmp_path):
    with pytest.raises(OSError):
        bio.write_exr(tmp_path / "missing_dir" / "x.exr", np.zeros((2, 2, 3), np.float32))
