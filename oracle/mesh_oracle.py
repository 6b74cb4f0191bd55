"""ORACLE — test infrastructure only.  CPU restatement (numpy, FP64) of the
signed distance field of a closed triangle mesh that eb_sdf_from_mesh computes
on the device, plus a reader/writer pair for the legacy-VTK triangle meshes the
reference reads (read_vtk_triangle_mesh, src/IO/read_input_files.jl:81-152).

The reference has no mesh-to-SDF step (its SDFs come from files); the two
published methods restated here are the closest-point region tests of
Ericson, "Real-Time Collision Detection" (2005) §5.1.5, and the triangle
solid angle of Van Oosterom & Strackee (1983), summed into the generalized
winding number.  Values: distance, positive inside the mesh, negative outside.
"""
from __future__ import annotations

import numpy as np


def grid_points(origin, spacing, dims) -> np.ndarray:
    """Grid points (nx*ny*nz, 3), x fastest."""
    nx, ny, nz = (int(d) for d in dims)
    o = np.asarray(origin, float)
    h = np.broadcast_to(np.asarray(spacing, float), (3,))
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return np.stack([o[0] + i.ravel() * h[0], o[1] + j.ravel() * h[1], o[2] + k.ravel() * h[2]], axis=1)


def dist2_point_triangle(P: np.ndarray, a, b, c) -> np.ndarray:
    """Squared distance of each point of P (n, 3) to triangle abc (region tests in order)."""
    a, b, c = (np.asarray(x, float) for x in (a, b, c))
    ab, ac = b - a, c - a
    ap = P - a
    d1, d2 = ap @ ab, ap @ ac
    bp = P - b
    d3, d4 = bp @ ab, bp @ ac
    cp = P - c
    d5, d6 = cp @ ab, cp @ ac
    vc = d1 * d4 - d3 * d2
    vb = d5 * d2 - d1 * d6
    va = d3 * d6 - d5 * d4
    Q = np.empty_like(P)
    todo = np.ones(len(P), bool)

    def take(mask, q):
        m = todo & mask
        Q[m] = q[m] if q.ndim == 2 else q
        todo[m] = False

    with np.errstate(divide="ignore", invalid="ignore"):
        take((d1 <= 0) & (d2 <= 0), a)
        take((d3 >= 0) & (d4 <= d3), b)
        take((vc <= 0) & (d1 >= 0) & (d3 <= 0), a + (d1 / (d1 - d3))[:, None] * ab)
        take((d6 >= 0) & (d5 <= d6), c)
        take((vb <= 0) & (d2 >= 0) & (d6 <= 0), a + (d2 / (d2 - d6))[:, None] * ac)
        take((va <= 0) & ((d4 - d3) >= 0) & ((d5 - d6) >= 0),
             b + ((d4 - d3) / ((d4 - d3) + (d5 - d6)))[:, None] * (c - b))
        den = 1.0 / (va + vb + vc)
        take(np.ones(len(P), bool), a + (vb * den)[:, None] * ab + (vc * den)[:, None] * ac)
    D = P - Q
    return np.einsum("ij,ij->i", D, D)


def solid_angle(P: np.ndarray, A, B, C) -> np.ndarray:
    """Signed solid angle of triangle ABC seen from each point of P."""
    a, b, c = np.asarray(A, float) - P, np.asarray(B, float) - P, np.asarray(C, float) - P
    la, lb, lc = (np.sqrt(np.einsum("ij,ij->i", x, x)) for x in (a, b, c))
    num = np.einsum("ij,ij->i", a, np.cross(b, c))
    den = la * lb * lc + np.einsum("ij,ij->i", a, b) * lc + np.einsum("ij,ij->i", a, c) * lb + \
        np.einsum("ij,ij->i", b, c) * la
    return 2.0 * np.arctan2(num, den)


def sdf_from_mesh(verts, tris, origin, spacing, dims) -> np.ndarray:
    """Signed distance at the grid points (x fastest); tris 0-based."""
    V = np.asarray(verts, float).reshape(-1, 3)
    T = np.asarray(tris, np.int64).reshape(-1, 3)
    P = grid_points(origin, spacing, dims)
    d2 = np.full(len(P), np.inf)
    om = np.zeros(len(P))
    for t in T:
        a, b, c = V[t[0]], V[t[1]], V[t[2]]
        d2 = np.minimum(d2, dist2_point_triangle(P, a, b, c))
        om += solid_angle(P, a, b, c)
    d = np.sqrt(d2)
    return np.where(np.abs(om) > 2 * np.pi, d, -d)


def cube_mesh(lo=0.0, hi=1.0):
    """Axis-aligned cube [lo, hi]^3 as 12 outward-oriented triangles."""
    v = np.array([[x, y, z] for z in (lo, hi) for y in (lo, hi) for x in (lo, hi)], float)
    # vertex id = x + 2 y + 4 z
    quads = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    tris = []
    for q in quads:
        tris += [(q[0], q[1], q[2]), (q[0], q[2], q[3])]
    return v, np.array(tris, np.int64)


def icosphere(level: int = 1, radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """Subdivided icosahedron on a sphere (20 * 4^level triangles)."""
    t = (1 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    V = [np.array(p, float) / np.linalg.norm(p) for p in v]
    for _ in range(level):
        mid = {}
        nf = []

        def m(i, j):
            key = (min(i, j), max(i, j))
            if key not in mid:
                p = V[i] + V[j]
                V.append(p / np.linalg.norm(p))
                mid[key] = len(V) - 1
            return mid[key]
        for a, b, c in f:
            ab, bc, ca = m(a, b), m(b, c), m(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return np.asarray(center, float) + radius * np.array(V), np.array(f, np.int64)


def write_vtk_triangle_mesh(path, verts, tris):
    """Legacy-VTK ASCII unstructured grid of triangles (one point per line, "3 i j k" cells)."""
    V = np.asarray(verts, float)
    T = np.asarray(tris, np.int64)
    with open(path, "w") as fh:
        fh.write("# vtk DataFile Version 3.0\ntriangle mesh\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        fh.write(f"POINTS {len(V)} double\n")
        for p in V:
            fh.write(f"{float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n")
        fh.write(f"CELLS {len(T)} {4 * len(T)}\n")
        for t in T:
            fh.write(f"3 {t[0]} {t[1]} {t[2]}\n")
        fh.write(f"CELL_TYPES {len(T)}\n")
        for _ in T:
            fh.write("5\n")
