"""OBJ::read (src/io/obj.rs:16-123) restated in Python - TEST INFRASTRUCTURE ONLY.

Line rules: after trim, a line starting with 'f' appends one 1-based vertex index per token
("v", "v/vt", "v/vt/vn", "v//vn"); a line starting with 'v' is "vt" (2 values), "vn" (3) or a
position (first 3 values).  Triangles are consecutive triples of all face indices, positions
through object_to_world (Transform::transform_point, affine), vertex normals through its
inverse transpose (TriangleMesh::new, src/shapes/triangle.rs:48-90), both skipped for the
identity; the i-th face vertex takes the i-th normal / texture index.  Raises ValueError where the
reference panics.
"""
from __future__ import annotations

import numpy as np


def read_obj(path, object_to_world=None) -> np.ndarray:
    return read_obj_mesh(path, object_to_world, attrs=False)[0]


def mat4_inverse_f32(m) -> np.ndarray:
    """Mat4::inverse (src/geometries/mat4.rs:72-140): Gauss-Jordan with full pivoting in f32."""
    a = [[np.float32(m[i][j]) for j in range(4)] for i in range(4)]
    indxc, indxr, ipiv = [0] * 4, [0] * 4, [0] * 4
    for i in range(4):
        irow = icol = 0
        big = np.float32(0)
        for j in range(4):
            if ipiv[j] != 1:
                for k in range(4):
                    if ipiv[k] == 0 and abs(a[j][k]) >= big:
                        big = np.float32(abs(a[j][k]))
                        irow, icol = j, k
        ipiv[icol] += 1
        if irow != icol:
            a[irow], a[icol] = a[icol], a[irow]
        indxr[i], indxc[i] = irow, icol
        pivinv = np.float32(1) / a[icol][icol]
        a[icol][icol] = np.float32(1)
        a[icol] = [x * pivinv for x in a[icol]]
        for j in range(4):
            if j != icol:
                save = a[j][icol]
                a[j][icol] = np.float32(0)
                a[j] = [a[j][k] - a[icol][k] * save for k in range(4)]
    for j in range(3, -1, -1):
        if indxr[j] != indxc[j]:
            for k in range(4):
                a[k][indxr[j]], a[k][indxc[j]] = a[k][indxc[j]], a[k][indxr[j]]
    return np.array(a, np.float32)


def read_obj_mesh(path, object_to_world=None, attrs=True):
    """(triangles (n, 9), normals (n, 9) or None, uvs (n, 6) or None, swaps_handedness); without
    `attrs` only the positions are assembled (normal and texture indices are still range-checked)."""
    pos, vi = [], []
    nrm, uvs = [], []
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
                uvs.append(p[:2])
            elif line.startswith("vn"):
                if len(p) < 3:
                    raise ValueError(line)
                nrm.append(p[:3])
            else:
                if len(p) < 3:
                    raise ValueError(line)
                pos.append(p[:3])
    if (any(i < 1 or i > len(pos) for i in vi) or any(i < 1 or i > len(nrm) for i in ni)
            or any(i < 1 or i > len(uvs) for i in ti)):
        raise ValueError("index out of range")
    k = len(vi) // 3 * 3
    if not attrs:
        ni, ti = [], []
    if (ni and len(ni) < k) or (ti and len(ti) < k):
        raise ValueError("fewer normal / texture indices than triangle vertices")
    P = np.array(pos, np.float32).reshape(-1, 3)
    corners = P[np.array(vi[:k], np.int64) - 1] if k else np.zeros((0, 3), np.float32)
    N = np.array(nrm, np.float32).reshape(-1, 3)[np.array(ni[:k], np.int64) - 1] if ni else None
    UV = np.array(uvs, np.float32).reshape(-1, 2)[np.array(ti[:k], np.int64) - 1] if ti else None
    swaps = False
    m = None if object_to_world is None else np.asarray(object_to_world, np.float32).reshape(3, 4)
    if m is not None and not np.array_equal(m, np.eye(3, 4, dtype=np.float32)):
        x, y, z = corners[:, 0], corners[:, 1], corners[:, 2]
        corners = np.stack([m[r, 0] * x + m[r, 1] * y + m[r, 2] * z + m[r, 3] for r in range(3)], 1).astype(np.float32)
        inv = mat4_inverse_f32(np.vstack([m, [0, 0, 0, 1]]))
        if N is not None:  # Normal::transform: m_inverse transposed (normal.rs:21-30)
            x, y, z = N[:, 0], N[:, 1], N[:, 2]
            N = np.stack([inv[0, c] * x + inv[1, c] * y + inv[2, c] * z for c in range(3)], 1).astype(np.float32)
        d = inv  # Transform::swaps_handedness of world_to_object (transform.rs:218-224)
        det = (d[0, 0] * (d[1, 1] * d[2, 2] - d[1, 2] * d[2, 1]) - d[0, 1] * (d[1, 0] * d[2, 2] - d[1, 2] * d[2, 0])
               + d[0, 2] * (d[1, 0] * d[2, 1] - d[1, 1] * d[2, 0]))
        swaps = bool(det < 0)
    return (corners.reshape(-1, 9), None if N is None else N.reshape(-1, 9),
            None if UV is None else UV.reshape(-1, 6), swaps)


def _idx(tok: str) -> int:
    t = tok[1:] if tok.startswith("+") else tok
    if not t.isdigit():
        raise ValueError(tok)
    return int(t)
