"""Scene and film I/O through the library: OBJ meshes in (bg_obj_read, the reference's OBJ::read
rules), OpenEXR images out (bg_write_exr / bg_film_write_exr), and a reader for the EXR files the
library writes (uncompressed scanline, float channels)."""
from __future__ import annotations

import ctypes as C
import os
import struct

import numpy as np

from . import _abi as A


def read_obj(path: str | os.PathLike, object_to_world: np.ndarray | None = None) -> np.ndarray:
    """World-space triangles (n, 9) of an OBJ file; raises ValueError with the library's message."""
    lib = A.load()
    xf = None if object_to_world is None else np.ascontiguousarray(object_to_world, np.float32).reshape(12)
    n = C.c_size_t()
    err = C.create_string_buffer(512)
    p = os.fsencode(str(path))
    st = lib.bg_obj_read(p, None if xf is None else xf.ctypes.data, None, 0, C.byref(n), err, len(err))
    if st != A.BG_OK:
        raise ValueError(err.value.decode(errors="replace"))
    tri = np.zeros((n.value, 9), np.float32)
    st = lib.bg_obj_read(p, None if xf is None else xf.ctypes.data, tri.ctypes.data if n.value else None, n.value,
                         C.byref(n), err, len(err))
    if st != A.BG_OK:
        raise ValueError(err.value.decode(errors="replace"))
    return tri


def read_obj_mesh(path: str | os.PathLike, object_to_world: np.ndarray | None = None):
    """(triangles (n, 9), vertex normals (n, 9) or None, uvs (n, 6) or None, BG_TRI_* flags) of an OBJ
    file, as bg_scene_add_obj adds it; raises ValueError with the library's message."""
    lib = A.load()
    xf = None if object_to_world is None else np.ascontiguousarray(object_to_world, np.float32).reshape(12)
    info = A.bg_obj_info()
    err = C.create_string_buffer(512)
    p = os.fsencode(str(path))
    xp = None if xf is None else xf.ctypes.data
    if lib.bg_obj_read_mesh(p, xp, None, None, None, 0, C.byref(info), err, len(err)) != A.BG_OK:
        raise ValueError(err.value.decode(errors="replace"))
    n = info.ntri
    tri = np.zeros((n, 9), np.float32)
    nrm = np.zeros((n, 9), np.float32) if info.has_normals else None
    uv = np.zeros((n, 6), np.float32) if info.has_uvs else None
    ptr = lambda a: None if a is None or not n else a.ctypes.data  # noqa: E731
    if lib.bg_obj_read_mesh(p, xp, ptr(tri), ptr(nrm), ptr(uv), n, C.byref(info), err, len(err)) != A.BG_OK:
        raise ValueError(err.value.decode(errors="replace"))
    return tri, nrm, uv, int(info.flags)


def write_exr(path: str | os.PathLike, rgb: np.ndarray) -> None:
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w, c = rgb.shape
    assert c == 3
    if A.load().bg_write_exr(os.fsencode(str(path)), rgb.ctypes.data, w, h) != A.BG_OK:
        raise OSError(f"cannot write {path}")


def read_exr(path: str | os.PathLike) -> np.ndarray:
    """Reads an uncompressed single-part scanline EXR with 32-bit float channels (as written above)
    into (h, w, channels) in alphabetical channel order reversed to R, G, B when those are present."""
    data = open(path, "rb").read()
    if struct.unpack_from("<I", data, 0)[0] != 20000630:
        raise ValueError("not an OpenEXR file")
    pos = 8
    attrs = {}
    while data[pos] != 0:
        end = data.index(b"\0", pos)
        name = data[pos:end].decode()
        pos = end + 1
        end = data.index(b"\0", pos)
        typ = data[pos:end].decode()
        pos = end + 1
        size = struct.unpack_from("<I", data, pos)[0]
        pos += 4
        attrs[name] = (typ, data[pos:pos + size])
        pos += size
    pos += 1
    chans = []
    raw = attrs["channels"][1]
    q = 0
    while raw[q] != 0:
        end = raw.index(b"\0", q)
        name = raw[q:end].decode()
        ptype = struct.unpack_from("<I", raw, end + 1)[0]
        chans.append((name, ptype))
        q = end + 1 + 16
    if attrs["compression"][1][0] != 0 or any(t != 2 for _, t in chans):
        raise ValueError("only uncompressed float channels are supported")
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    offsets = struct.unpack_from(f"<{h}Q", data, pos)
    img = np.zeros((h, w, len(chans)), np.float32)
    for off in offsets:
        y, nbytes = struct.unpack_from("<iI", data, off)
        line = np.frombuffer(data, np.float32, w * len(chans), off + 8).reshape(len(chans), w)
        img[y - y0] = line.T
    names = [n for n, _ in chans]
    if {"R", "G", "B"} <= set(names):
        img = img[:, :, [names.index("R"), names.index("G"), names.index("B")]]
    return img
