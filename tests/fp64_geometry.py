"""FP64 point-to-primitive distances for the parity tests (test infrastructure): the distance
from a query to a given segment or triangle of a mesh, computed in double precision from the
FP32 inputs, to show that two primitives are tied for the closest one."""
import numpy as np


def _segment_dist(x, a, b):
    u = b - a
    t = np.clip(np.einsum("ij,ij->i", x - a, u) / np.maximum(np.einsum("ij,ij->i", u, u), 1e-300), 0.0, 1.0)
    return np.linalg.norm(x - (a + t[:, None] * u), axis=1)


def _triangle_dist(p, a, b, c):
    """Distance from points to triangles in FP64 (closest point by Voronoi regions)."""
    ab, ac, ap = b - a, c - a, p - a
    dot = lambda u, v: np.einsum("ij,ij->i", u, v)
    d1, d2 = dot(ab, ap), dot(ac, ap)
    bp = p - b
    d3, d4 = dot(ab, bp), dot(ac, bp)
    cp = p - c
    d5, d6 = dot(ab, cp), dot(ac, cp)
    vc = d1 * d4 - d3 * d2
    vb = d5 * d2 - d1 * d6
    va = d3 * d6 - d5 * d4
    denom = np.where(va + vb + vc == 0, 1.0, va + vb + vc)
    q = a + (vb / denom)[:, None] * ab + (vc / denom)[:, None] * ac          # interior
    with np.errstate(divide="ignore", invalid="ignore"):
        e_bc = b + np.nan_to_num(((d4 - d3) / ((d4 - d3) + (d5 - d6))))[:, None] * (c - b)
        e_ac = a + np.nan_to_num((d2 / (d2 - d6)))[:, None] * ac
        e_ab = a + np.nan_to_num((d1 / (d1 - d3)))[:, None] * ab
    m = lambda cond: cond[:, None]
    q = np.where(m((va <= 0) & (d4 - d3 >= 0) & (d5 - d6 >= 0)), e_bc, q)
    # regions in reverse order of precedence (vertex a first, then b, edge ab, c, edge ac, edge bc)
    q = np.where(m((vb <= 0) & (d2 >= 0) & (d6 <= 0)), e_ac, q)
    q = np.where(m((d6 >= 0) & (d5 <= d6)), c, q)
    q = np.where(m((vc <= 0) & (d1 >= 0) & (d3 <= 0)), e_ab, q)
    q = np.where(m((d3 >= 0) & (d4 <= d3)), b, q)
    q = np.where(m((d1 <= 0) & (d2 <= 0)), a, q)
    return np.linalg.norm(p - q, axis=1)


def prim_dist64(pos, idx, prim, x):
    """FP64 distance from x[i] to primitive prim[i] of the mesh (pos, idx)."""
    pos = pos.astype(np.float64)
    x = x.astype(np.float64)
    v = idx[prim]
    if idx.shape[1] == 2:
        return _segment_dist(x, pos[v[:, 0]], pos[v[:, 1]])
    return _triangle_dist(x, pos[v[:, 0]], pos[v[:, 1]], pos[v[:, 2]])
