"""OBJ::read (src/io/obj.rs:16-123) restated in Python - TEST INFRASTRUCTURE ONLY.

Line rules: after trim, a line starting with 'f' appends one 1-based vertex index per token
("v", "v/vt", "v/vt/vn", "v//vn"); a line starting with 'v' is "vt" (2 values), "vn" (3) or a
position (first 3 values).  Triangles are consecutive triples of all face indices, positions
through object_to_world (Transform::transform_point, affine).  Raises ValueError where the
reference panics.
"""
from __future__ import annotations

import numpy as np


def read_obj(path, object_to_world=None) -> np.ndarray:
    pos, vi = [], []
    nn = nt = 0
    ni, ti = [], []
    for raw in open(path, "r", encoding="utf-8", errors="strict"):
        line = raw.strip()
        if line.startswith("f"):
            for v in line.split()[1:]:
                if "//" in v:
                    a, b = v.split("//")
                    vi.append(_idx(a))
                    ni.append(_idx(b))
                elif "/" in v:
                    p = v.split("/")
                    if len(p) not in (2, 3):
                        raise ValueError(v)
                    vi.append(_idx(p[0]))
                    ti.append(_idx(p[1]))
                    if len(p) == 3:
                        ni.append(_idx(p[2]))
                else:
                    vi.append(_idx(v))
        if line.startswith("v"):
            p = [np.float32(float(x)) for x in line.split()[1:]]
            if line.startswith("vt"):
                if len(p) < 2:
                    raise ValueError(line)
                nt += 1
            elif line.startswith("vn"):
                if len(p) < 3:
                    raise ValueError(line)
                nn += 1
            else:
                if len(p) < 3:
                    raise ValueError(line)
                pos.append(p[:3])
    if any(i < 1 or i > len(pos) for i in vi) or any(i < 1 or i > nn for i in ni) or any(i < 1 or i > nt for i in ti):
        raise ValueError("index out of range")
    P = np.array(pos, np.float32).reshape(-1, 3)
    k = len(vi) // 3 * 3
    corners = P[np.array(vi[:k], np.int64) - 1] if k else np.zeros((0, 3), np.float32)
    if object_to_world is not None:
        m = np.asarray(object_to_world, np.float32).reshape(3, 4)
        x, y, z = corners[:, 0], corners[:, 1], corners[:, 2]
        corners = np.stack([m[r, 0] * x + m[r, 1] * y + m[r, 2] * z + m[r, 3] for r in range(3)], 1).astype(np.float32)
    return corners.reshape(-1, 9)


def _idx(tok: str) -> int:
    t = tok[1:] if tok.startswith("+") else tok
    if not t.isdigit():
        raise ValueError(tok)
    return int(t)
