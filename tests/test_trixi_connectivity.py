"""The rule that turns Trixi's P4estMesh interface description (neighbor_ids
and the index-symbol tuples of cache.interfaces.node_indices) into the C ABI's
connectivity arrays (trixiatmo.jl_gb300/trixi_connectivity.py; the Julia shim
in INTEGRATION.md applies the same rule).  CPU only.

Trixi-style tuples are built here from node coordinates alone: the primary side
gets the forward tuple of its face, the secondary side whichever tuple makes
every surface node land on the same physical point.  The rule must then give
back the host mirror's own connectivity (found by its independent face
matching), and, for primaries whose indices run backward or sides swapped, arrays
that still match node by node."""
import itertools

import numpy as np
import pytest

ENDS = ("begin", "end")


def forward_tuple(face, ndims):
    axis, end = divmod(face, 2)
    syms = iter(("i_forward", "j_forward"))
    return tuple(ENDS[end] if a == axis else next(syms) for a in range(ndims))


def candidate_tuples(face, ndims):
    axis, end = divmod(face, 2)
    others = [a for a in range(ndims) if a != axis]
    if ndims == 2:
        choices = [("i_forward",), ("i_backward",)]
    else:
        choices = []
        for first in ("i", "j"):
            second = "j" if first == "i" else "i"
            for d1, d2 in itertools.product(("forward", "backward"), repeat=2):
                choices.append((f"{first}_{d1}", f"{second}_{d2}"))
    out = []
    for ch in choices:
        t = [None] * ndims
        t[axis] = ENDS[end]
        for a, s in zip(others, ch):
            t[a] = s
        out.append(tuple(t))
    return out


def element_node(indices, i_s, j_s, n):
    idx = []
    for s in indices:
        if s in ENDS:
            idx.append(0 if s == "begin" else n - 1)
        else:
            v = i_s if s[0] == "i" else j_s
            idx.append(n - 1 - v if s.endswith("backward") else v)
    return tuple(idx)


def point(xyz, e, idx):
    # node coordinates are stored [e, (k,) j, i, c]: reverse the axis order
    return xyz[(e,) + tuple(reversed(idx))]


def surface_nodes(ndims, n):
    return [(i, 0) for i in range(n)] if ndims == 2 else \
        [(i, j) for j in range(n) for i in range(n)]


def matching_tuple(xyz, n, ndims, e0, t0, e1, f1, tol):
    for cand in candidate_tuples(f1, ndims):
        if all(np.abs(point(xyz, e0, element_node(t0, i, j, n)) -
                      point(xyz, e1, element_node(cand, i, j, n))).max() <= tol
               for i, j in surface_nodes(ndims, n)):
            return cand
    raise AssertionError("no tuple matches")


def face_point(xyz, e, f, l1, l2, n, ndims):
    """Physical point of the ABI's face-local node (l1, l2) of face f."""
    axis, end = divmod(f, 2)
    idx, ls = [], iter((l1, l2))
    for a in range(ndims):
        idx.append((n - 1) * end if a == axis else next(ls))
    return point(xyz, e, tuple(idx))


def abi_matches(xyz, n, ndims, el, fa, fl, tol):
    for k in range(len(fl)):
        for i, j in surface_nodes(ndims, n):
            if ndims == 2:
                s1, s2 = (n - 1 - i if fl[k] else i), 0
            else:
                a, b = (j, i) if fl[k] & 1 else (i, j)
                s1 = n - 1 - a if fl[k] & 2 else a
                s2 = n - 1 - b if fl[k] & 4 else b
            p = face_point(xyz, el[k, 0], fa[k, 0], i, j, n, ndims)
            q = face_point(xyz, el[k, 1], fa[k, 1], s1, s2, n, ndims)
            if np.abs(p - q).max() > tol:
                return False
    return True


def meshes(tg):
    from trixiatmo_gb300.initial_conditions import EARTH_RADIUS
    cv = tg.covariant
    basis2 = tg.LobattoLegendreBasis(3)
    sphere = cv.P4estMeshCubedSphere2D(3, EARTH_RADIUS, polydeg=3)
    eq = cv.CovariantShallowWaterEquations2D(9.80616, 7.292e-5)
    _, xyz2 = cv.compute_aux_vars(sphere, basis2, eq, None, None)
    ie, ifc, fl, be, bf = sphere.connectivity(basis2).arrays()
    yield "cubed sphere 2D", 2, basis2.n, np.asarray(xyz2), (ie, ifc, fl)
    shell = tg.P4estMeshCubedSphereTopography(2, 2, 6.371e6, 30000.0, polydeg=2)
    basis3 = tg.LobattoLegendreBasis(2)
    xyz3 = shell.geometry(basis3)[0]
    ie, ifc, fo, be, bf = shell.connectivity(basis3).arrays()
    yield "cubed-sphere shell 3D", 3, basis3.n, xyz3, (ie, ifc, fo)


def test_trixi_tuples_give_the_mirror_connectivity(tg):
    tc = tg.trixi_connectivity
    for name, ndims, n, xyz, (ie, ifc, fl) in meshes(tg):
        tol = 1e-9 * np.abs(xyz).max()
        nids = np.asarray(ie).T + 1                      # Trixi: [2, I], 1-based
        tuples = [[], []]
        for k in range(len(fl)):
            t0 = forward_tuple(int(ifc[k, 0]), ndims)
            tuples[0].append(t0)
            tuples[1].append(matching_tuple(xyz, n, ndims, int(ie[k, 0]), t0, int(ie[k, 1]),
                                            int(ifc[k, 1]), tol))
        el, fa, fo = tc.interface_arrays(nids, tuples)
        assert np.array_equal(el, ie) and np.array_equal(fa, ifc), name
        assert np.array_equal(fo, fl), name
        if ndims == 3:
            assert len(set(fo.tolist())) > 1  # panel edges of the shell exercise non-trivial codes
        else:
            assert fo.any()


def test_rule_holds_for_swapped_sides_and_backward_primaries(tg):
    """p4est may make either neighbour the primary, and the rule must not rely
    on the primary's indices running forward."""
    tc = tg.trixi_connectivity
    rng = np.random.default_rng(11)
    for name, ndims, n, xyz, (ie, ifc, fl) in meshes(tg):
        tol = 1e-9 * np.abs(xyz).max()
        nids, tuples = [[], []], [[], []]
        for k in range(len(fl)):
            a, b = (0, 1) if rng.random() < 0.5 else (1, 0)
            t0 = candidate_tuples(int(ifc[k, a]), ndims)[rng.integers(2 if ndims == 2 else 8)]
            t1 = matching_tuple(xyz, n, ndims, int(ie[k, a]), t0, int(ie[k, b]), int(ifc[k, b]),
                                tol)
            nids[0].append(int(ie[k, a]) + 1)
            nids[1].append(int(ie[k, b]) + 1)
            tuples[0].append(t0)
            tuples[1].append(t1)
        el, fa, fo = tc.interface_arrays(np.asarray(nids), tuples)
        assert abi_matches(xyz, n, ndims, el, fa, fo, tol), name


def test_boundary_faces_and_bad_tuples(tg):
    tc = tg.trixi_connectivity
    el, fa = tc.boundary_arrays([3, 7], [("i_forward", "j_forward", "begin"),
                                         ("end", "i_backward")])
    assert el.tolist() == [2, 6] and fa.tolist() == [4, 1]
    with pytest.raises(ValueError):
        tc.face_of(("i_forward", "j_forward"))
    with pytest.raises(ValueError):
        tc.orientation(("end", "i_forward"), ("begin", "j_sideways"))
