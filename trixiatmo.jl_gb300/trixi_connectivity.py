"""Trixi's P4estMesh interface description -> the connectivity arrays of the C ABI.

Trixi keeps, for every interface, the two neighbour elements
(`cache.interfaces.neighbor_ids[side, interface]`, 1-based, side 1 = primary)
and, per side, a tuple of index symbols (`cache.interfaces.node_indices[side,
interface]`) saying where the face's nodes sit in that element: per element axis
either "begin" / "end" (the face lies at that end of the axis) or "i_forward",
"i_backward", "j_forward", "j_backward" (the axis runs along the first (i) or
second (j) surface index, forward or backward).  Boundaries carry the same
tuples (`cache.boundaries.node_indices[b]`).  TrixiAtmo's own interface loop
reads them this way: `indices2direction` for the face, `index_to_start_step_2d`
for start and step, and the secondary side running backward when
`:i_backward in secondary_indices`
(src/solvers/dgsem_p4est/dg_2d_manifold_in_3d_covariant.jl:239-278).

The C ABI (include/trixiatmo_gpu.h) wants 0-based elements and faces
(0 = xi-, 1 = xi+, 2 = eta-, 3 = eta+, 4 = zeta-, 5 = zeta+), face-local node
indices (l1, l2) along the face's two other axes in ascending order, and per
interface the secondary's node order relative to the primary's: in 2D a flip
flag, in 3D an orientation code o in 0..7 (swap when o & 1, then reverse s1
when o & 2 and s2 when o & 4).  This module converts the first into the
second; the Julia shim in INTEGRATION.md applies the same rule.
"""
from __future__ import annotations

import numpy as np

_ENDS = ("begin", "end")
_DIRS = ("i_forward", "i_backward", "j_forward", "j_backward")


def face_of(indices) -> int:
    """0-based face of an index tuple: 2 a (+1 for "end") for the axis a that
    holds "begin" or "end" (Trixi's `indices2direction` minus one)."""
    axes = [a for a, s in enumerate(indices) if s in _ENDS]
    if len(axes) != 1:
        raise ValueError(f"index tuple {indices!r} names no single face")
    a = axes[0]
    return 2 * a + (1 if indices[a] == "end" else 0)


def face_local(indices, i_s: int, j_s: int, n: int):
    """Face-local indices (l1, l2, ... one per non-normal axis, ascending) of
    the surface node (i_s, j_s) on the side described by `indices`."""
    out = []
    for s in indices:
        if s in _ENDS:
            continue
        if s not in _DIRS:
            raise ValueError(f"unknown index symbol {s!r}")
        v = i_s if s[0] == "i" else j_s
        out.append(n - 1 - v if s.endswith("backward") else v)
    return tuple(out)


def _surface_nodes(ndims: int, n: int):
    return [(i, 0) for i in range(n)] if ndims == 2 else \
        [(i, j) for j in range(n) for i in range(n)]


def orientation(primary, secondary) -> int:
    """The ABI's relative order of the secondary face: 2D flip flag (0 or 1),
    3D orientation code (0..7).  Derived from where each surface node sits on
    both sides, so it holds whichever way the primary's own indices run."""
    ndims = len(primary)
    n = 3  # three nodes per direction determine the map
    pairs = [(face_local(primary, i, j, n), face_local(secondary, i, j, n))
             for i, j in _surface_nodes(ndims, n)]
    if ndims == 2:
        if all(s[0] == p[0] for p, s in pairs):
            return 0
        if all(s[0] == n - 1 - p[0] for p, s in pairs):
            return 1
        raise ValueError(f"sides {primary!r} / {secondary!r} do not match node by node")
    for o in range(8):
        ok = True
        for (l1, l2), s in pairs:
            a, b = (l2, l1) if o & 1 else (l1, l2)
            if o & 2:
                a = n - 1 - a
            if o & 4:
                b = n - 1 - b
            if (a, b) != s:
                ok = False
                break
        if ok:
            return o
    raise ValueError(f"sides {primary!r} / {secondary!r} do not match node by node")


def interface_arrays(neighbor_ids, node_indices):
    """(interface_elements [I, 2], interface_faces [I, 2], interface_flip [I])
    of the ABI from Trixi's `neighbor_ids` [2, I] (1-based) and `node_indices`
    [2][I] (tuples of the symbols above, as strings)."""
    neighbor_ids = np.asarray(neighbor_ids)
    nif = neighbor_ids.shape[1]
    el = np.empty((nif, 2), dtype=np.int32)
    fa = np.empty((nif, 2), dtype=np.int32)
    fl = np.empty(nif, dtype=np.int32)
    for k in range(nif):
        for side in range(2):
            el[k, side] = int(neighbor_ids[side, k]) - 1
            fa[k, side] = face_of(node_indices[side][k])
        fl[k] = orientation(node_indices[0][k], node_indices[1][k])
    return el, fa, fl


def boundary_arrays(neighbor_ids, node_indices):
    """(boundary_elements [B], boundary_faces [B]) of the ABI from Trixi's
    `cache.boundaries.neighbor_ids` [B] (1-based) and `node_indices` [B]."""
    el = np.asarray(neighbor_ids, dtype=np.int32) - 1
    fa = np.asarray([face_of(t) for t in node_indices], dtype=np.int32)
    return el, fa
