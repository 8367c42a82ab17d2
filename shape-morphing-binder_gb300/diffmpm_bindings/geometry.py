"""Mesh -> particle lattice sampling (setup time).

Restates GeometryLoading::LoadMPMPointCloudFromObj (GeometryLoading.cpp:85-143):
a lattice of spacing ``point_dx`` over the mesh's bounding box
(dims = ceil((max - min) / dx) + 1, k fastest), keeping the lattice points
inside the mesh.  The reference classifies points with libigl's signed
distance under the winding-number sign (GeometryLoading.cpp:57-77); here the
inside test is the generalized winding number computed on the GPU
(``mpm_winding_numbers``: |w| >= 1/2 inside, points on the surface kept).
OBJ parsing and the lattice are host work.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def read_obj(path: str):
    """Vertices (V,3) float32 and triangles (F,3) int from a Wavefront OBJ."""
    verts, faces = [], []
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        for line in f:
            if line.startswith("v "):
                verts.append([float(t) for t in line.split()[1:4]])
            elif line.startswith("f "):
                idx = [int(t.split("/")[0]) for t in line.split()[1:]]
                idx = [i - 1 if i > 0 else len(verts) + i for i in idx]
                for k in range(1, len(idx) - 1):  # fan-triangulate polygons
                    faces.append([idx[0], idx[k], idx[k + 1]])
    if not verts or not faces:
        raise ValueError(f"no triangles in {path}")
    return np.asarray(verts, np.float32), np.asarray(faces, np.int64)


def winding_numbers(points: np.ndarray, V: np.ndarray, F: np.ndarray) -> np.ndarray:
    """Generalized winding number of each point w.r.t. the triangle mesh (V, F),
    computed on the GPU (points on the surface: exactly 0.5)."""
    P = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    T = np.ascontiguousarray(np.asarray(V, np.float32)[np.asarray(F, np.int64)]).reshape(-1, 9)
    out = np.zeros(len(P))
    _lib.check(_lib.lib.mpm_winding_numbers(len(P), P.ctypes.data_as(C.c_void_p), len(T),
                                            T.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p), 0, None),
               "winding_numbers")
    return out


def lattice(V: np.ndarray, point_dx: float) -> np.ndarray:
    """Lattice points over the bounding box (GeometryLoading.cpp:19-35), k fastest."""
    V = np.asarray(V, np.float32)
    mn, mx = V.min(0), V.max(0)
    dx = np.float32(point_dx)
    dims = [int(np.ceil((mx[i] - mn[i]) / dx)) + 1 for i in range(3)]
    i, j, k = np.meshgrid(*(np.arange(d, dtype=np.float32) for d in dims), indexing="ij")
    ijk = np.stack([i, j, k], -1).reshape(-1, 3)
    return (mn + dx * ijk).astype(np.float32)


def lattice_inside_mesh(V: np.ndarray, F: np.ndarray, point_dx: float) -> np.ndarray:
    pts = lattice(V, point_dx)
    w = winding_numbers(pts, V, F)
    return pts[np.abs(w) >= 0.5]
