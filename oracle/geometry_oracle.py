"""Generalized winding numbers on the CPU (TEST INFRASTRUCTURE ONLY).

The checker for the GPU inside test of mesh sampling (the reference's
GeometryLoading.cpp:57-77 classifies lattice points with libigl's signed
distance under the winding-number sign): the sum over triangles of the signed
solid angle from the Van Oosterom-Strackee formula
tan(Omega/2) = a.(b x c) / (|a||b||c| + (a.b)|c| + (a.c)|b| + (b.c)|a|),
over 4 pi, in float64.  Points on the surface (on a vertex, or in a
triangle's plane inside it) get exactly 0.5, the convention of the GPU path.
"""
from __future__ import annotations

import numpy as np


def winding_numbers(points, V, F, chunk: int = 1 << 22) -> np.ndarray:
    P = np.asarray(points, np.float64).reshape(-1, 3)
    T = np.asarray(V, np.float64)[np.asarray(F, np.int64)]  # (t,3,3)
    out = np.zeros(len(P))
    step = max(1, chunk // max(1, len(T)))
    for s in range(0, len(P), step):
        p = P[s:s + step, None, None, :]
        a, b, c = T[None, :, 0] - p[:, :, 0], T[None, :, 1] - p[:, :, 0], T[None, :, 2] - p[:, :, 0]
        la, lb, lc = (np.linalg.norm(u, axis=-1) for u in (a, b, c))
        num = np.einsum("ptk,ptk->pt", a, np.cross(b, c))
        den = la * lb * lc + np.einsum("ptk,ptk->pt", a, b) * lc + np.einsum("ptk,ptk->pt", a, c) * lb + \
            np.einsum("ptk,ptk->pt", b, c) * la
        on = ((la == 0) | (lb == 0) | (lc == 0) | ((num == 0) & (den <= 0))).any(axis=1)
        w = (2.0 * np.arctan2(num, den)).sum(axis=1) / (4.0 * np.pi)
        out[s:s + step] = np.where(on, 0.5, w)
    return out
