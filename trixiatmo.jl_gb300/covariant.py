"""Covariant shallow-water equations on the cubed sphere: the host mirror of
the reference's covariant API for the `rhs!` path.

Reference: src/equations/covariant_shallow_water.jl, covariant_shallow_water_split.jl,
equations.jl (auxiliary-variable layout, :139-215), src/meshes/p4est_cubed_sphere.jl
(P4estMeshCubedSphere2D with the element-local mapping of Guba et al. 2014),
src/solvers/dgsem_p4est/containers_2d_manifold_in_3d_covariant.jl (metric terms),
src/semidiscretization/metric_terms.jl, src/equations/reference_data.jl (test cases),
src/callbacks_step/analysis_covariant.jl (error norms).

The solution u[e, j, i, :] = (h, h v^1, h v^2) holds the contravariant momentum;
the 26 auxiliary variables per node (aux[e, j, i, :], the reference's
aux_node_vars[:, i, j, e]) are, in order: the covariant basis A (3x2,
column-major), the contravariant basis (2x3, column-major), the area element J,
G_11, G_12, G_22, G^11, G^12, G^22, the bottom topography h_s and the
Christoffel symbols Gamma^1_11, Gamma^1_12, Gamma^1_22, Gamma^2_11, Gamma^2_12,
Gamma^2_22.  They are computed once on the host (like the reference's cache)
and uploaded by tag_create.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from .basis import LobattoLegendreBasis
from .initial_conditions import (EARTH_GRAVITATIONAL_ACCELERATION, EARTH_ROTATION_RATE)
from .meshes import Connectivity

SECONDS_PER_DAY = 8.64e4
N_AUX = 26


# ---- global coordinate systems, metric-term options -------------------------
class GlobalCartesianCoordinates:
    pass


class GlobalSphericalCoordinates:
    pass


class ChristoffelSymbolsAutodiff:
    """Christoffel symbols from exact derivatives of the analytic metric
    (the reference differentiates it with ForwardDiff; here forward-mode dual
    numbers do the same)."""


class ChristoffelSymbolsCollocationDerivative:
    """Christoffel symbols from the collocation derivative of the metric."""


class MetricTermsCovariantSphere:
    def __init__(self, christoffel_symbols=None):
        self.christoffel_symbols = christoffel_symbols or ChristoffelSymbolsAutodiff()


# ---- equations ------------------------------------------------------------------
class CovariantShallowWaterEquations2D:
    """Shallow water in covariant form with the geometric and Coriolis sources
    (src/equations/covariant_shallow_water.jl:66-77)."""

    nvariables = 3
    ndims = 2
    split = False
    eq_id = _lib.TAG_EQ_COVARIANT_SWE

    def __init__(self, gravity, rotation_rate, global_coordinate_system=None):
        self.gravity = float(gravity)
        self.rotation_rate = float(rotation_rate)
        self.global_coordinate_system = global_coordinate_system or GlobalCartesianCoordinates()


class SplitCovariantShallowWaterEquations2D(CovariantShallowWaterEquations2D):
    """Split (entropy-conservative) form with nonconservative pressure,
    topography and curvature terms (src/equations/covariant_shallow_water_split.jl:46-57)."""

    split = True


class _NamedFlux:
    def __init__(self, name):
        self.name = name

    def __repr__(self):
        return self.name


flux_central = _NamedFlux("flux_central")
from .equations import flux_ec  # noqa: E402  (one name for both equation families)
flux_nonconservative_ec = _NamedFlux("flux_nonconservative_ec")
flux_nonconservative_surface_simplified = _NamedFlux("flux_nonconservative_surface_simplified")


class DissipationLocalLaxFriedrichs:
    pass


class FluxPlusDissipation:
    def __init__(self, numerical_flux, dissipation):
        self.numerical_flux = numerical_flux
        self.dissipation = dissipation


class _SourceTerms:
    def __init__(self, name):
        self.name = name

    def __repr__(self):
        return self.name


source_terms_geometric_coriolis = _SourceTerms("source_terms_geometric_coriolis")


# ---- cubed-sphere mesh ------------------------------------------------------------
def cubed_sphere_face_point(xi, eta, radius, direction):
    """Equiangular gnomonic projection (Ronchi et al. 1996) of the reference
    point (xi, eta) of cube face `direction` (1: -x, 2: +x, 3: -y, 4: +y,
    5: -z, 6: +z; each face parametrised right-handed with the outward normal)
    onto the sphere of the given radius."""
    x = np.tan(xi * np.pi / 4)
    y = np.tan(eta * np.pi / 4)
    one = np.ones_like(x)
    c = {1: (-one, -x, y), 2: (one, x, y), 3: (x, -one, y), 4: (-x, one, y),
         5: (-x, y, -one), 6: (x, y, one)}[direction]
    s = radius / np.sqrt(1 + x * x + y * y)
    return np.stack([s * c[0], s * c[1], s * c[2]], axis=-1)


def local_mapping(xi1, xi2, v1, v2, v3, v4, radius):
    """Element-local map of Guba et al. (2014), appendix A: bilinear in the four
    corner vertices, then projected radially onto the sphere."""
    xb = 0.25 * ((1 - xi1) * (1 - xi2) * v1 + (1 + xi1) * (1 - xi2) * v2 +
                 (1 + xi1) * (1 + xi2) * v3 + (1 - xi1) * (1 + xi2) * v4)
    return radius * xb / np.sqrt((xb ** 2).sum(-1, keepdims=True))


class P4estMeshCubedSphere2D:
    """`P4estMeshCubedSphere2D(trees_per_face_dimension, radius; polydeg,
    element_local_mapping = true)` (src/meshes/p4est_cubed_sphere.jl): 6 k^2
    elements (one per tree, refinement level 0), element e = cx + k (cy + k d)
    for cell (cx, cy) of face d (0-based).  Only the element-local mapping is
    provided: the reference's covariant metric terms require it."""

    ndims = 2
    manifold = True

    def __init__(self, trees_per_face_dimension, radius, *, polydeg,
                 element_local_mapping=True, initial_refinement_level=0):
        if not element_local_mapping:
            raise ValueError("the covariant metric terms need element_local_mapping = true")
        if initial_refinement_level != 0:
            raise ValueError("the covariant solver needs initial_refinement_level = 0")
        self.k = int(trees_per_face_dimension)
        self.radius = float(radius)
        self.polydeg = int(polydeg)
        k = self.k
        d = 2.0 / k
        verts = np.empty((6, k, k, 4, 3))          # [face, cy, cx, corner, xyz]
        c = np.arange(k, dtype=np.float64)
        xo = (-1 + c * d + d / 2)[None, :]           # [1, cx]
        yo = (-1 + c * d + d / 2)[:, None]           # [cy, 1]
        for direction in range(1, 7):
            for corner, (sx, sy) in enumerate(((-1, -1), (1, -1), (1, 1), (-1, 1))):
                xi = np.broadcast_to(xo + sx * d / 2, (k, k))
                eta = np.broadcast_to(yo + sy * d / 2, (k, k))
                verts[direction - 1, :, :, corner] = cubed_sphere_face_point(xi, eta, self.radius,
                                                                             direction)
        self.vertices = verts.reshape(6 * k * k, 4, 3)

    @property
    def nelements(self):
        return 6 * self.k * self.k

    def node_coordinates(self, basis):
        x = basis.nodes
        X1, X2 = np.meshgrid(x, x, indexing="xy")  # [j, i]
        v = self.vertices[:, None, None, :, :]
        return local_mapping(X1[None, :, :, None], X2[None, :, :, None], v[..., 0, :],
                             v[..., 1, :], v[..., 2, :], v[..., 3, :], self.radius)

    def connectivity(self, basis):
        """Interfaces by geometric matching of element edges (every edge is an
        interface: the sphere has no boundary); flip = 1 when the secondary
        edge runs backward."""
        xyz = self.node_coordinates(basis)
        n = basis.n
        edges = [xyz[:, :, 0], xyz[:, :, n - 1], xyz[:, 0, :], xyz[:, n - 1, :]]  # [E, l, 3]
        E = xyz.shape[0]
        scale = self.radius
        allf = np.stack(edges, axis=1)  # [E, 4, n, 3]
        mids = allf.mean(axis=2)
        q = np.round(mids / (scale * 1e-9)).astype(np.int64).reshape(-1, 3)
        order = np.lexsort((q[:, 2], q[:, 1], q[:, 0]))
        flat = q[order]
        same = np.all(flat[1:] == flat[:-1], axis=1)
        t = np.nonzero(same)[0]
        a, b = order[t], order[t + 1]
        # every edge is shared by exactly two elements
        if len(t) * 2 != E * 4 or np.unique(np.concatenate([a, b])).size != E * 4:
            raise RuntimeError("unmatched element edge on the cubed sphere")
        e0, f0 = np.divmod(a, 4)
        e1, f1 = np.divmod(b, 4)
        P, S = allf[e0, f0], allf[e1, f1]              # [I, n, 3]
        fwd = np.abs(S - P).max(axis=(1, 2))
        bwd = np.abs(S[:, ::-1] - P).max(axis=(1, 2))
        if (np.minimum(fwd, bwd) > 1e-6 * scale).any():
            raise RuntimeError("edges with equal midpoints do not match node by node")
        c = Connectivity()
        c.if_elements = np.stack([e0, e1], axis=1)
        c.if_faces = np.stack([f0, f1], axis=1)
        c.if_flip = (bwd < fwd).astype(np.int32)
        return c


# ---- metric terms (auxiliary variables) ---------------------------------------------
class _Dual:
    """Forward-mode dual number over numpy arrays (value, derivative)."""

    __slots__ = ("v", "d")
    __array_ufunc__ = None  # numpy arrays defer to the dual's reflected operators

    def __init__(self, v, d=0.0):
        self.v = np.asarray(v, dtype=np.float64)
        self.d = np.broadcast_to(np.asarray(d, dtype=np.float64), self.v.shape).copy()

    @staticmethod
    def lift(x):
        return x if isinstance(x, _Dual) else _Dual(x, 0.0)

    def __add__(self, o):
        o = _Dual.lift(o)
        return _Dual(self.v + o.v, self.d + o.d)

    __radd__ = __add__

    def __sub__(self, o):
        o = _Dual.lift(o)
        return _Dual(self.v - o.v, self.d - o.d)

    def __rsub__(self, o):
        return _Dual.lift(o) - self

    def __mul__(self, o):
        o = _Dual.lift(o)
        return _Dual(self.v * o.v, self.d * o.v + self.v * o.d)

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = _Dual.lift(o)
        return _Dual(self.v / o.v, (self.d * o.v - self.v * o.d) / (o.v * o.v))

    def __rtruediv__(self, o):
        return _Dual.lift(o) / self

    def __neg__(self):
        return _Dual(-self.v, -self.d)


def _sqrt(x):
    if isinstance(x, _Dual):
        s = np.sqrt(x.v)
        return _Dual(s, x.d / (2 * s))
    return np.sqrt(x)


def _sin(x):
    if isinstance(x, _Dual):
        return _Dual(np.sin(x.v), np.cos(x.v) * x.d)
    return np.sin(x)


def _cos(x):
    if isinstance(x, _Dual):
        return _Dual(np.cos(x.v), -np.sin(x.v) * x.d)
    return np.cos(x)


def _asin(x):
    if isinstance(x, _Dual):
        return _Dual(np.arcsin(x.v), x.d / np.sqrt(1 - x.v * x.v))
    return np.arcsin(x)


def _atan2(y, x):
    if isinstance(y, _Dual) or isinstance(x, _Dual):
        y, x = _Dual.lift(y), _Dual.lift(x)
        r2 = x.v * x.v + y.v * y.v
        return _Dual(np.arctan2(y.v, x.v), (x.v * y.d - y.v * x.d) / r2)
    return np.arctan2(y, x)


def _basis_covariant(v, xi1, xi2, radius, spherical):
    """Covariant basis A (rows: 3 global components, columns: a_1, a_2) of the
    element-local map at (xi1, xi2); v: vertices [.., 4, 3] (plain arrays);
    xi1/xi2 may be dual numbers.  Cartesian components: product and quotient
    rule on the radial projection of the bilinear map
    (containers_2d_manifold_in_3d_covariant.jl:306-327); spherical components:
    Guba et al. (2014), appendix A (:334-375)."""
    v1, v2, v3, v4 = (v[..., c, :] for c in range(4))
    comp = lambda a, k: a[..., k]  # noqa: E731
    if not spherical:
        xe = [0.25 * ((1 - xi1) * (1 - xi2) * comp(v1, k) + (1 + xi1) * (1 - xi2) * comp(v2, k) +
                      (1 + xi1) * (1 + xi2) * comp(v3, k) + (1 - xi1) * (1 + xi2) * comp(v4, k))
              for k in range(3)]
        d1 = [0.25 * (-(1 - xi2) * comp(v1, k) + (1 - xi2) * comp(v2, k) +
                      (1 + xi2) * comp(v3, k) - (1 + xi2) * comp(v4, k)) for k in range(3)]
        d2 = [0.25 * (-(1 - xi1) * comp(v1, k) - (1 + xi1) * comp(v2, k) +
                      (1 + xi1) * comp(v3, k) + (1 - xi1) * comp(v4, k)) for k in range(3)]
        nrm = _sqrt(xe[0] * xe[0] + xe[1] * xe[1] + xe[2] * xe[2])
        dot1 = xe[0] * d1[0] + xe[1] * d1[1] + xe[2] * d1[2]
        dot2 = xe[0] * d2[0] + xe[1] * d2[1] + xe[2] * d2[2]
        n2 = nrm * nrm
        a1 = [radius / nrm * (d1[k] - dot1 / n2 * xe[k]) for k in range(3)]
        a2 = [radius / nrm * (d2[k] - dot2 / n2 * xe[k]) for k in range(3)]
        return [[a1[0], a2[0]], [a1[1], a2[1]], [a1[2], a2[2]]]
    xe = [0.25 * ((1 - xi1) * (1 - xi2) * comp(v1, k) + (1 + xi1) * (1 - xi2) * comp(v2, k) +
                  (1 + xi1) * (1 + xi2) * comp(v3, k) + (1 - xi1) * (1 + xi2) * comp(v4, k))
          for k in range(3)]
    sf = radius / _sqrt(xe[0] * xe[0] + xe[1] * xe[1] + xe[2] * xe[2])
    x = [sf * xe[k] for k in range(3)]
    lon, lat = _atan2(x[1], x[0]), _asin(x[2] / radius)
    sl, cl = _sin(lon), _cos(lon)
    st, ct = _sin(lat), _cos(lat)
    # 3x3 projection matrix P (row-major) and the 2x3 spherical unit vectors
    P = [[sl * sl * ct * ct + st * st, -sl * cl * ct * ct, -cl * st * ct],
         [-sl * cl * ct * ct, cl * cl * ct * ct + st * st, -sl * st * ct],
         [-cl * st, -sl * st, ct]]
    S = [[-sl, cl, 0.0], [0.0, 0.0, 1.0]]
    # bilinear derivative weights of the vertices (4x2), times 0.25 * sf
    W = [[-1 + xi2, -1 + xi1], [1 - xi2, -1 - xi1], [1 + xi2, 1 + xi1], [-1 - xi2, 1 - xi1]]
    V = [v1, v2, v3, v4]
    # M = V W (3x2): M[k][c] = sum_q V[q][k] W[q][c]
    M = [[sum(comp(V[q], k) * W[q][c] for q in range(4)) for c in range(2)] for k in range(3)]
    PM = [[sum(P[r][k] * M[k][c] for k in range(3)) for c in range(2)] for r in range(3)]
    A = [[0.25 * sf * sum(S[r][k] * PM[k][c] for k in range(3)) for c in range(2)]
         for r in range(2)]
    zero = 0.0 * A[0][0]
    return [[A[0][0], A[0][1]], [A[1][0], A[1][1]], [zero, zero]]


def _metric_covariant(A):
    g11 = A[0][0] * A[0][0] + A[1][0] * A[1][0] + A[2][0] * A[2][0]
    g12 = A[0][0] * A[0][1] + A[1][0] * A[1][1] + A[2][0] * A[2][1]
    g22 = A[0][1] * A[0][1] + A[1][1] * A[1][1] + A[2][1] * A[2][1]
    return g11, g12, g22


def compute_aux_vars(mesh, basis, equations, metric_terms=None, bottom_topography=None,
                     device=False):
    """aux[e, j, i, 26] and node coordinates xyz[e, j, i, 3] of the reference's
    covariant cache (containers_2d_manifold_in_3d_covariant.jl:247-295,
    379-441, 455-490).  device=True computes them with tag_cov_metric_terms
    on the GPU (what the semidiscretizations use); otherwise in NumPy on the
    host."""
    metric_terms = metric_terms or MetricTermsCovariantSphere()
    spherical = isinstance(equations.global_coordinate_system, GlobalSphericalCoordinates)
    key = (basis.n, spherical, type(metric_terms.christoffel_symbols).__name__,
           id(bottom_topography), bool(device))
    cache = mesh.__dict__.setdefault("_aux_cache", {})
    if key in cache:
        return cache[key]
    f = _compute_aux_vars_device if device else _compute_aux_vars
    cache[key] = f(mesh, basis, metric_terms, spherical, bottom_topography)
    return cache[key]


def _compute_aux_vars_device(mesh, basis, metric_terms, spherical, bottom_topography):
    n, E = basis.n, mesh.nelements
    collocation = isinstance(metric_terms.christoffel_symbols,
                             ChristoffelSymbolsCollocationDerivative)
    v = np.ascontiguousarray(mesh.vertices, dtype=np.float64)
    x = np.ascontiguousarray(basis.nodes, dtype=np.float64)
    D = np.asfortranarray(basis.derivative_matrix, dtype=np.float64)
    aux = np.zeros((E, n, n, N_AUX))
    xyz = np.zeros((E, n, n, 3))
    dp = ctypes.POINTER(ctypes.c_double)
    _lib.check(_lib.load().tag_cov_metric_terms(
        v.ctypes.data_as(dp), E, n - 1, mesh.radius, int(spherical), int(collocation),
        x.ctypes.data_as(dp), D.ctypes.data_as(dp), aux.ctypes.data_as(dp),
        xyz.ctypes.data_as(dp)))
    if bottom_topography is not None:
        aux[..., 19] = bottom_topography(xyz)
        if not np.isfinite(aux[..., 19]).all():
            raise ValueError("the bottom topography is not finite at a node")
    return aux, xyz


def _compute_aux_vars(mesh, basis, metric_terms, spherical, bottom_topography):
    n = basis.n
    E = mesh.nelements
    X1, X2 = np.meshgrid(basis.nodes, basis.nodes, indexing="xy")  # [j, i]
    v = mesh.vertices[:, None, None, :, :]
    xi1 = np.broadcast_to(X1[None], (E, n, n))
    xi2 = np.broadcast_to(X2[None], (E, n, n))
    A = _basis_covariant(v, xi1, xi2, mesh.radius, spherical)
    A = np.stack([np.stack([np.broadcast_to(A[r][c], (E, n, n)) for c in range(2)], -1)
                  for r in range(3)], -2)  # [E, n, n, 3, 2]
    G = np.einsum("...ki,...kj->...ij", A, A)
    det = G[..., 0, 0] * G[..., 1, 1] - G[..., 0, 1] * G[..., 1, 0]
    Gi = np.empty_like(G)
    Gi[..., 0, 0] = G[..., 1, 1] / det
    Gi[..., 1, 1] = G[..., 0, 0] / det
    Gi[..., 0, 1] = -G[..., 0, 1] / det
    Gi[..., 1, 0] = -G[..., 1, 0] / det
    Acon = np.einsum("...ij,...kj->...ik", Gi, A)  # [E, n, n, 2, 3]
    aux = np.zeros((E, n, n, N_AUX))
    aux[..., 0:6] = A.transpose(0, 1, 2, 4, 3).reshape(E, n, n, 6)      # column-major 3x2
    aux[..., 6:12] = Acon.transpose(0, 1, 2, 4, 3).reshape(E, n, n, 6)  # column-major 2x3
    aux[..., 12] = np.sqrt(det)
    aux[..., 13], aux[..., 14], aux[..., 15] = G[..., 0, 0], G[..., 0, 1], G[..., 1, 1]
    aux[..., 16], aux[..., 17], aux[..., 18] = Gi[..., 0, 0], Gi[..., 0, 1], Gi[..., 1, 1]
    xyz = mesh.node_coordinates(basis)
    if bottom_topography is not None:
        aux[..., 19] = bottom_topography(xyz)
    # metric derivatives dG/dxi1, dG/dxi2
    if isinstance(metric_terms.christoffel_symbols, ChristoffelSymbolsCollocationDerivative):
        D = basis.derivative_matrix
        Gc = np.stack([aux[..., 13], aux[..., 14], aux[..., 15]], -1)  # [E, j, i, 3]
        d1 = np.einsum("ik,ejkc->ejic", D, Gc)
        d2 = np.einsum("jk,ekic->ejic", D, Gc)
    else:
        d = []
        with np.errstate(invalid="ignore", divide="ignore"):
            for wrt in (0, 1):
                a = _Dual(xi1, 1.0 if wrt == 0 else 0.0)
                b = _Dual(xi2, 1.0 if wrt == 1 else 0.0)
                Ad = _basis_covariant(v, a, b, mesh.radius, spherical)
                Ad = [[_Dual.lift(Ad[r][c]) for c in range(2)] for r in range(3)]
                g = _metric_covariant(Ad)
                d.append(np.stack([np.broadcast_to(gg.d, (E, n, n)) for gg in g], -1))
        d1, d2 = d
    # Christoffel symbols of the first kind, then raised with G^-1
    # (containers_2d_manifold_in_3d_covariant.jl:417-441)
    G11_1, G12_1, G22_1 = d1[..., 0], d1[..., 1], d1[..., 2]
    G11_2, G12_2, G22_2 = d2[..., 0], d2[..., 1], d2[..., 2]
    g1 = [[0.5 * G11_1, 0.5 * G11_2], [0.5 * G11_2, G12_2 - 0.5 * G22_1]]
    g2 = [[G12_1 - 0.5 * G11_2, 0.5 * G22_1], [0.5 * G22_1, 0.5 * G22_2]]
    c11, c12, c22 = aux[..., 16], aux[..., 17], aux[..., 18]
    aux[..., 20] = c11 * g1[0][0] + c12 * g2[0][0]
    aux[..., 21] = c11 * g1[0][1] + c12 * g2[0][1]
    aux[..., 22] = c11 * g1[1][1] + c12 * g2[1][1]
    aux[..., 23] = c12 * g1[0][0] + c22 * g2[0][0]
    aux[..., 24] = c12 * g1[0][1] + c22 * g2[0][1]
    aux[..., 25] = c12 * g1[1][1] + c22 * g2[1][1]
    if not np.isfinite(aux).all():
        raise ValueError("the metric terms are singular at a node (spherical global coordinates "
                         "are singular at the poles; use GlobalCartesianCoordinates)")
    return np.ascontiguousarray(aux), np.ascontiguousarray(xyz)


# ---- test cases (src/equations/reference_data.jl) --------------------------------------
def _lonlat(x):
    a = np.sqrt((x ** 2).sum(-1))
    return np.arctan2(x[..., 1], x[..., 0]), np.arcsin(x[..., 2] / a), a


def spherical2cartesian(vlon, vlat, vrad, x):
    lon, lat, _ = _lonlat(x)
    sl, cl, st, ct = np.sin(lon), np.cos(lon), np.sin(lat), np.cos(lat)
    return (-sl * vlon - st * cl * vlat + ct * cl * vrad,
            cl * vlon - st * sl * vlat + ct * sl * vrad,
            ct * vlat + st * vrad)


def cartesian2spherical(vx, vy, vz, x):
    lon, lat, _ = _lonlat(x)
    sl, cl, st, ct = np.sin(lon), np.cos(lon), np.sin(lat), np.cos(lat)
    return (-sl * vx + cl * vy,
            -st * cl * vx - st * sl * vy + ct * vz,
            ct * cl * vx + ct * sl * vy + st * vz)


def initial_condition_geostrophic_balance(x, t, equations):
    """Williamson et al. (1992) case 2 (reference_data.jl:145-164); returns
    (h, v components in the global system, b) with the velocity in spherical
    components (converted to the equations' global system)."""
    lon, lat, a = _lonlat(x)
    v0 = 2 * np.pi * a / (12 * SECONDS_PER_DAY)
    vlon = v0 * np.cos(lat)
    h = 1 / EARTH_GRAVITATIONAL_ACCELERATION * (
        2.94e4 - (a * EARTH_ROTATION_RATE * v0 + 0.5 * v0 ** 2) * np.sin(lat) ** 2)
    return _spherical_out(h, vlon, np.zeros_like(h), np.zeros_like(h), x, equations)


def initial_condition_rossby_haurwitz(x, t, equations):
    """Williamson et al. (1992) case 6 (reference_data.jl:202-227).  The
    reference writes h_0, omega, K and R as single-precision literals, so
    products of those alone are rounded to single precision before they meet
    double-precision values; the same promotion is kept here."""
    lon, lat, a = _lonlat(x)
    f32, f64 = np.float32, np.float64
    h0, omega, K, R = f32(8.0e3), f32(7.848e-6), f32(7.848e-6), f32(4.0)
    cl = np.cos(lat)
    # EARTH_ROTATION_RATE is a double, so every sum with it is a double; NumPy
    # would round a Python float plus a float32 scalar to float32.
    Om = f64(EARTH_ROTATION_RATE)
    A = (f32(0.5) * omega * (2 * Om + f64(omega)) * cl ** 2 +
         f32(0.25) * K ** 2 * cl ** (2 * R) * ((R + 1) * cl ** 2 + (2 * R ** 2 - R - 2) -
                                               2 * R ** 2 / cl ** 2))
    B = (2 * (Om + f64(omega)) * f64(K) / ((R + 1) * (R + 2)) * cl ** R *
         ((R ** 2 + 2 * R + 2) - (R + 1) ** 2 * cl ** 2))
    C = f32(0.25) * K ** 2 * cl ** (2 * R) * ((R + 1) * cl ** 2 - (R + 2))
    h = h0 + (1 / EARTH_GRAVITATIONAL_ACCELERATION) * (
        a ** 2 * A + a ** 2 * B * np.cos(R * lon) + a ** 2 * C * np.cos(2 * R * lon))
    vlon = (a * omega * cl + a * K * cl ** (R - 1) * (R * np.sin(lat) ** 2 - cl ** 2) *
            np.cos(R * lon))
    vlat = -a * K * R * cl ** (R - 1) * np.sin(lat) * np.sin(R * lon)
    return _spherical_out(np.asarray(h, dtype=np.float64), vlon, vlat, np.zeros_like(h), x,
                          equations)


def bottom_topography_isolated_mountain(x):
    """reference_data.jl:286-297."""
    lon, lat, a = _lonlat(x)
    lon0, lat0, b0, R = -np.pi / 2, np.pi / 6, 2000.0, np.pi / 9
    return b0 * (1.0 - np.sqrt(np.minimum(R ** 2, (lon - lon0) ** 2 + (lat - lat0) ** 2)) / R)


def initial_condition_isolated_mountain(x, t, equations):
    """Williamson et al. (1992) case 5 (reference_data.jl:262-284): total
    height H; h = H - h_s."""
    lon, lat, a = _lonlat(x)
    h0, v0 = 5960.0, 20.0
    vlon = v0 * np.cos(lat)
    H = h0 - 1 / EARTH_GRAVITATIONAL_ACCELERATION * (
        a * EARTH_ROTATION_RATE * v0 + 0.5 * v0 ** 2) * np.sin(lat) ** 2
    return _spherical_out(H, vlon, np.zeros_like(H), bottom_topography_isolated_mountain(x), x,
                          equations)


def bottom_topography_unsteady_solid_body_rotation(x):
    """reference_data.jl:386-388."""
    return 0.5 * (EARTH_ROTATION_RATE * x[..., 2]) ** 2 / EARTH_GRAVITATIONAL_ACCELERATION


def initial_condition_unsteady_solid_body_rotation(x, t, equations):
    """Läuter et al. (2005) (reference_data.jl:348-383); velocity given in
    Cartesian components."""
    a = np.sqrt((x ** 2).sum(-1))
    v0 = 2 * np.pi * a / (12 * SECONDS_PER_DAY)
    k1 = 133681.0
    alpha = np.pi / 4
    Om = EARTH_ROTATION_RATE
    b1 = np.array([math.cos(Om * t), math.sin(Om * t), 0.0])
    b2 = np.array([-math.sin(Om * t), math.cos(Om * t), 0.0])
    b3 = np.array([0.0, 0.0, 1.0])
    c = np.array([-math.sin(alpha), 0.0, math.cos(alpha)])
    nvec = x / a[..., None]
    Omx = Om * x[..., 2]
    phi = np.array([c @ b1, c @ b2, c @ b3])
    v = v0[..., None] * np.cross(phi, nvec)
    H = (-0.5 * (v0 * (nvec @ phi) + Omx) ** 2 + 0.5 * Omx ** 2 + k1) / EARTH_GRAVITATIONAL_ACCELERATION
    b = bottom_topography_unsteady_solid_body_rotation(x)
    if isinstance(equations.global_coordinate_system, GlobalSphericalCoordinates):
        vlon, vlat, vrad = cartesian2spherical(v[..., 0], v[..., 1], v[..., 2], x)
        return np.stack([H, vlon, vlat, vrad, b], -1)
    return np.stack([H, v[..., 0], v[..., 1], v[..., 2], b], -1)


def galewsky_velocity(lat, u0=80.0, lat0=np.pi / 7, lat1=np.pi / 2 - np.pi / 7):
    """Zonal jet of Galewsky et al. (2004) (reference_data.jl:461-469): a
    C-infinity bump supported on (lat0, lat1)."""
    lat = np.asarray(lat, dtype=np.float64)
    inside = (lat0 < lat) & (lat < lat1)
    lc = np.where(inside, lat, 0.5 * (lat0 + lat1))
    u = u0 / math.exp(-4.0 / (lat1 - lat0) ** 2) * np.exp(1.0 / (lc - lat0) * 1.0 / (lc - lat1))
    return np.where(inside, u, 0.0)


def _galewsky_height_integrals(lat, panels=64, order=16):
    """(I1, I2) with the integral of galewsky_integrand (reference_data.jl:471-474)
    from pi/2 to lat equal to I1 + I2 / a:
    I1 = int u 2 Omega sin, I2 = int u^2 tan.  The reference integrates
    adaptively (QuadGK); here a composite Gauss-Legendre rule (`panels` panels
    of `order` points) over [max(lat, lat0), lat1], the jet's support, which
    is exact to rounding for this smooth integrand (doubling the panels moves
    the result by < 1e-15 relative)."""
    lat0, lat1 = np.pi / 7, np.pi / 2 - np.pi / 7
    xg, wg = np.polynomial.legendre.leggauss(order)
    s = ((np.arange(panels)[:, None] + 0.5 * (xg[None, :] + 1.0)) / panels).ravel()
    ws = (np.broadcast_to(wg, (panels, order)) / (2.0 * panels)).ravel()
    flat = np.asarray(lat, dtype=np.float64).ravel()
    I1 = np.zeros_like(flat)
    I2 = np.zeros_like(flat)
    for c0 in range(0, flat.size, 4096):
        lo = np.clip(flat[c0:c0 + 4096], lat0, lat1)
        length = lat1 - lo
        q = lo[:, None] + length[:, None] * s[None, :]
        u = galewsky_velocity(q)
        I1[c0:c0 + 4096] = -(u * 2 * EARTH_ROTATION_RATE * np.sin(q)) @ ws * length
        I2[c0:c0 + 4096] = -(u * u * np.tan(q)) @ ws * length
    shape = np.shape(lat)
    return I1.reshape(shape), I2.reshape(shape)


def initial_condition_barotropic_instability(x, t, equations):
    """Galewsky et al. (2004) barotropic instability (reference_data.jl:427-459):
    the balanced zonal jet with the height
    h_0 = 10158 - a/g int_{pi/2}^{lat} u (2 Omega sin + u tan / a), a the
    node's radius, plus the 120 m perturbation at lat_2 = pi/4 for
    -pi < lon < pi."""
    lon, lat, a = _lonlat(x)
    vlon = galewsky_velocity(lat)
    I1, I2 = _galewsky_height_integrals(lat)
    h = 10158.0 - a / EARTH_GRAVITATIONAL_ACCELERATION * (I1 + I2 / a)
    alpha, beta, lat2 = 1.0 / 3.0, 1.0 / 15.0, np.pi / 4
    pert = 120.0 * np.cos(lat) * np.exp(-((lon / alpha) ** 2)) * np.exp(-((lat2 - lat) / beta) ** 2)
    h = np.where((-np.pi < lon) & (lon < np.pi), h + pert, h)
    return _spherical_out(h, vlon, np.zeros_like(h), np.zeros_like(h), x, equations)


def initial_condition_well_balanced(H=5960.0):
    """The constant total height at rest of examples/shallow_water/covariant/elixir_well_balanced.jl."""
    def ic(x, t, equations):
        z = np.zeros(x.shape[:-1])
        return np.stack([H + z, z, z, z], -1)
    return ic


def _spherical_out(h, vlon, vlat, b, x, equations):
    if isinstance(equations.global_coordinate_system, GlobalSphericalCoordinates):
        return np.stack([h, vlon, vlat, np.zeros_like(h), b], -1)
    vx, vy, vz = spherical2cartesian(vlon, vlat, np.zeros_like(h), x)
    return np.stack([h, vx, vy, vz, b], -1)


def transform_initial_condition(initial_condition, equations):
    """(x, t, aux) -> conservative covariant state (equations.jl:89-99): the
    global velocity is projected with the contravariant basis, then
    h = H - h_s and h v^i."""
    def ic(x, t, aux, eq=equations):
        p = initial_condition(x, t, eq)
        Acon = aux[..., 6:12].reshape(aux.shape[:-1] + (3, 2)).swapaxes(-1, -2)  # [.., 2, 3]
        vg = p[..., 1:4]
        vcon = np.einsum("...ij,...j->...i", Acon, vg)
        h = p[..., 0] - aux[..., 19]
        return np.stack([h, h * vcon[..., 0], h * vcon[..., 1]], -1)
    return ic


def error_norms(u, u_exact, aux, basis):
    """l2 (weighted by the area element) and linf errors at the solution nodes
    (src/callbacks_step/analysis_covariant.jl:144-189)."""
    w = basis.weights
    wJ = w[None, :, None] * w[None, None, :] * aux[..., 12]
    d = u_exact - u
    l2 = np.sqrt((d ** 2 * wJ[..., None]).sum(axis=(0, 1, 2)) / wJ.sum())
    linf = np.abs(d).max(axis=(0, 1, 2))
    return l2, linf
