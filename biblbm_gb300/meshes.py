"""Triangulated membrane meshes used by the benchmark configurations.

The reference ships only gmsh spheres/ellipsoids (``progs/*/*.msh``, read by
``read_gmsh_mesh`` in ``src/fsi/ParticleShapeFactory.hh:32-83``).  The
configurations of this project need subdivided icospheres (162 / 642 / 2562
vertices) and the Evans-Fung biconcave red-cell shape, so they are generated
here.  Triangles are wound counter-clockwise seen from outside, so the signed
volume ``sum v0.(v1 x v2)/6`` (``src/fsi/TriangleUtils.h:104-109``) is positive.
"""
from __future__ import annotations

import numpy as np

__all__ = ["icosphere", "evans_fung", "rotation_matrix", "random_rotation", "place"]


def _icosahedron():
    p = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array(
        [
            [-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0],
            [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
            [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1],
        ],
        dtype=np.float64,
    )
    f = np.array(
        [
            [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
            [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
            [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
            [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1],
        ],
        dtype=np.int64,
    )
    return v / np.linalg.norm(v, axis=1, keepdims=True), f


def icosphere(level: int, radius: float = 1.0):
    """Unit icosahedron subdivided ``level`` times (10*4**level + 2 vertices), scaled to ``radius``.

    Returns ``(xyz float64 [nv,3], tri int64 [nt,3])``.
    """
    v, f = _icosahedron()
    verts = [tuple(x) for x in v]
    for _ in range(level):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            idx = cache.get(key)
            if idx is None:
                m = (np.asarray(verts[a]) + np.asarray(verts[b])) * 0.5
                m = m / np.linalg.norm(m)
                verts.append(tuple(m))
                idx = len(verts) - 1
                cache[key] = idx
            return idx

        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        f = np.asarray(nf, dtype=np.int64)
    xyz = np.asarray(verts, dtype=np.float64) * float(radius)
    return xyz, f


def evans_fung(level: int, radius: float):
    """Biconcave red-cell surface of Evans & Fung (1972) from an icosphere.

    A unit-sphere point (x, y, z) maps to ``(R x, R y, sign(z) R/2 sqrt(1-r^2) (c0 + c1 r^2 + c2 r^4))``
    with ``r^2 = x^2 + y^2``, c0 = 0.2072, c1 = 2.0026, c2 = -1.1228 and ``R`` the
    major radius; the symmetry axis is z.
    """
    xyz, tri = icosphere(level, 1.0)
    c0, c1, c2 = 0.2072, 2.0026, -1.1228
    r2 = np.clip(xyz[:, 0] ** 2 + xyz[:, 1] ** 2, 0.0, 1.0)
    h = 0.5 * np.sqrt(1.0 - r2) * (c0 + c1 * r2 + c2 * r2 * r2)
    out = np.empty_like(xyz)
    out[:, 0] = radius * xyz[:, 0]
    out[:, 1] = radius * xyz[:, 1]
    out[:, 2] = radius * np.sign(xyz[:, 2]) * h
    return out, tri


def rotation_matrix(axis, angle: float) -> np.ndarray:
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    x, y, z = a
    c, s = np.cos(angle), np.sin(angle)
    C = 1.0 - c
    return np.array(
        [
            [c + x * x * C, x * y * C - z * s, x * z * C + y * s],
            [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
            [z * x * C - y * s, z * y * C + x * s, c + z * z * C],
        ]
    )


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform rotation on SO(3) from a unit quaternion (Shoemake's method)."""
    u1, u2, u3 = rng.random(3)
    q = np.array(
        [
            np.sqrt(1 - u1) * np.sin(2 * np.pi * u2),
            np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
            np.sqrt(u1) * np.sin(2 * np.pi * u3),
            np.sqrt(u1) * np.cos(2 * np.pi * u3),
        ]
    )
    x, y, z, w = q
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
            [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
            [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
        ]
    )


def place(xyz: np.ndarray, rot: np.ndarray | None = None, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Rotate a mesh about its vertex centroid and move the centroid to ``center``."""
    c = xyz.mean(axis=0)
    p = xyz - c
    if rot is not None:
        p = p @ np.asarray(rot).T
    return p + np.asarray(center, dtype=np.float64)
