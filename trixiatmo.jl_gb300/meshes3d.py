"""Host-side 3D hexahedral meshes: the cubed-sphere shell.

`P4estMeshCubedSphereTopography` mirrors TrixiAtmo's constructor of the same
name (src/meshes/p4est_cubed_sphere_topography.jl:114-167), by default for a
perfect sphere, optionally with an initial topography spread over the column
by GalChen or Sleve vertical coordinates: 6 faces x trees_per_face^2 x layers
hexahedra, the
equiangular cubed-sphere map of :596-620, boundaries `inside` (zeta-) and
`outside` (zeta+).  Elements are numbered column first (layer fastest), then
cell x, cell y, cube face; the reference orders the cells of a face along a
Gilbert curve, which changes only the numbering.

Geometry follows the collocation form Trixi uses for curved P4estMesh{3}
meshes: the Jacobian matrix by the LGL derivative matrix applied to the node
coordinates, J = det, and the contravariant vectors in the invariant curl
form of D. A. Kopriva, J. Sci. Comput. 26 (2006) 301-327:
    (Ja^i)_n = -1/2 e_i . curl_xi I^N( X_l grad_xi X_m - X_m grad_xi X_l ),
(n, m, l) cyclic, which satisfies the discrete metric identities.

Connectivity is derived geometrically: two element faces are an interface when
their node sets coincide; the orientation code o (see include/trixiatmo_gpu.h)
maps the primary's face-local indices (l1, l2) to the secondary's.

Array layouts (C order == Trixi's column-major):
  node_coordinates[e, k, j, i, c], contravariant_vectors[e, k, j, i, d, c],
  inverse_jacobian[e, k, j, i].
"""
from __future__ import annotations

import numpy as np

from .basis import LobattoLegendreBasis


class GalChen:
    """Gal-Chen & Somerville's terrain-following coordinate
    (src/meshes/p4est_cubed_sphere_topography.jl:54-79): the topography's
    influence decays linearly from the ground to the top H,
    z = z_ref + (H - z_ref) z_s / H."""

    def __call__(self, z_reference, z_topography, H):
        return z_reference + (H - z_reference) * z_topography / H


class Sleve:
    """SLEVE coordinate of Schaer et al. (2002) (p4est_cubed_sphere_topography.jl:7-52):
    with eta = z_ref / H, z = eta H + z_s sinh((eta_H - eta) / s / eta_H) / sinh(1 / s)
    for eta <= eta_H and z = eta H above."""

    def __init__(self, eta_H, s):
        self.eta_H, self.s = float(eta_H), float(s)

    def __call__(self, z_reference, z_topography, H):
        eta = z_reference / H
        low = eta <= self.eta_H
        decay = np.sinh((self.eta_H - eta) / self.s / self.eta_H) / np.sinh(1.0 / self.s)
        return np.where(low, eta * H + z_topography * decay, eta * H)


def cubed_sphere_mapping(xi, eta, zeta, inner_radius, thickness, direction, topography=None,
                         adapt_vertical_grid=None):
    """Equiangular cubed-sphere shell map of one cube face (1-based direction
    1..6 as in the reference: -z, +x, +y, -x, -y, +z).  With a topography
    (a function of latitude and longitude, p4est_cubed_sphere_topography.jl:596-620)
    the reference height z_ref = thickness (zeta + 1) / 2 is moved by
    adapt_vertical_grid (GalChen or Sleve); the latitude is taken as the
    reference takes it, asin of the unit vector's z component divided once
    more by r."""
    alpha = xi * np.pi / 4
    beta = eta * np.pi / 4
    x = np.tan(alpha)
    y = np.tan(beta)
    one = np.ones_like(x)
    cube = {
        1: (-y, -x, -one),
        2: (one, x, y),
        3: (-x, one, y),
        4: (-one, -x, y),
        5: (x, -one, y),
        6: (x, y, one),
    }[direction]
    r = np.sqrt(1 + x * x + y * y)
    z = thickness * 0.5 * (zeta + 1)
    if topography is not None:
        ux, uy, uz = cube[0] / r, cube[1] / r, cube[2] / r
        lat = np.arcsin(uz / r)
        lon = np.arctan2(uy, ux)
        z = (adapt_vertical_grid or GalChen())(z, topography(lat, lon), thickness)
    s = (inner_radius + z) / r
    return s * cube[0], s * cube[1], s * cube[2]


def _face_nodes(arr, f, n):
    """View of the face-f nodes of arr[e, k, j, i, ...] as [e, l2, l1, ...]."""
    end = n - 1 if f & 1 else 0
    d = f >> 1
    if d == 0:    # xi face: (l1, l2) = (j, k)
        return arr[:, :, :, end]
    if d == 1:    # eta face: (l1, l2) = (i, k)
        return arr[:, :, end, :]
    return arr[:, end, :, :]  # zeta face: (l1, l2) = (i, j)


def _orient(a, o, n):
    """Secondary-face view of primary-ordered data: out[l2, l1] = a[s2, s1]."""
    l1, l2 = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    s1, s2 = l1.copy(), l2.copy()
    if o & 1:
        s1, s2 = s2, s1
    if o & 2:
        s1 = n - 1 - s1
    if o & 4:
        s2 = n - 1 - s2
    return s1, s2


def metric_terms_3d(xyz, D):
    """Jacobian determinant and invariant-curl contravariant vectors of node
    coordinates xyz[e, k, j, i, 3] on LGL nodes with derivative matrix D."""
    def dxi(f):   # derivative along i (last spatial axis)
        return np.einsum("ia,ekja...->ekji...", D, f)

    def deta(f):
        return np.einsum("ja,ekai...->ekji...", D, f)

    def dzeta(f):
        return np.einsum("ka,eaji...->ekji...", D, f)

    X = [xyz[..., c] for c in range(3)]
    grads = [(dxi(x), deta(x), dzeta(x)) for x in X]
    # Jacobian matrix J[c][d] = dX_c / dxi_d
    Jm = np.empty(xyz.shape[:-1] + (3, 3))
    for c in range(3):
        for d in range(3):
            Jm[..., c, d] = grads[c][d]
    det = np.linalg.det(Jm)
    Ja = np.empty(xyz.shape[:-1] + (3, 3))  # [..., d, c] = (Ja^d)_c
    for nc in range(3):
        m, l = (nc + 1) % 3, (nc + 2) % 3
        # W = X_l grad X_m - X_m grad X_l  (three components along xi, eta, zeta)
        W = [X[l] * grads[m][d] - X[m] * grads[l][d] for d in range(3)]
        curl = (deta(W[2]) - dzeta(W[1]), dzeta(W[0]) - dxi(W[2]), dxi(W[1]) - deta(W[0]))
        for d in range(3):
            Ja[..., d, nc] = -0.5 * curl[d]
    return det, Ja


class Connectivity3D:
    def __init__(self, if_elements, if_faces, if_orient, bd_elements, bd_faces, bd_names):
        self.if_elements = if_elements
        self.if_faces = if_faces
        self.if_orient = if_orient
        self.bd_elements = bd_elements
        self.bd_faces = bd_faces
        self.bd_names = bd_names

    def arrays(self):
        return (self.if_elements, self.if_faces, self.if_orient, self.bd_elements,
                self.bd_faces)


def match_faces(xyz, n, boundary_face_names):
    """Interfaces and boundary faces of a conforming hexahedral mesh from its
    node coordinates.  boundary_face_names: {face index: name} for faces that
    are unmatched."""
    E = xyz.shape[0]
    scale = np.abs(xyz).max()
    keys = {}
    faces_xyz = [_face_nodes(xyz, f, n) for f in range(6)]  # [e, l2, l1, 3]
    cents = np.stack([fx.mean(axis=(1, 2)) for fx in faces_xyz], axis=1)  # [E, 6, 3]
    q = np.round(cents / (scale * 1e-9)).astype(np.int64)
    order = np.lexsort((q[..., 2].ravel(), q[..., 1].ravel(), q[..., 0].ravel()))
    flat = q.reshape(-1, 3)[order]
    same = np.all(flat[1:] == flat[:-1], axis=1)
    paired = np.zeros(E * 6, dtype=bool)
    pairs = []
    for t in np.nonzero(same)[0]:
        a, b = order[t], order[t + 1]
        if paired[a] or paired[b]:
            continue
        paired[a] = paired[b] = True
        pairs.append((int(a), int(b)))
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    e0, f0 = np.divmod(pairs[:, 0], 6)
    e1, f1 = np.divmod(pairs[:, 1], 6)
    allf = np.stack(faces_xyz, axis=1)  # [E, 6, l2, l1, 3]
    P = allf[e0, f0]
    Sf = allf[e1, f1]
    dists = np.empty((8, len(pairs)))
    for o in range(8):
        s1, s2 = _orient(None, o, n)
        dists[o] = np.abs(Sf[:, s2, s1] - P).max(axis=(1, 2, 3))
    bo = np.argmin(dists, axis=0)
    if len(pairs) and dists[bo, np.arange(len(pairs))].max() > 1e-6 * scale:
        raise RuntimeError("faces with equal centroids do not match node by node")
    if_e = np.stack([e0, e1], axis=1)
    if_f = np.stack([f0, f1], axis=1)
    if_o = bo
    bd_e, bd_f, bd_n = [], [], []
    for a in np.nonzero(~paired)[0]:
        e, f = divmod(int(a), 6)
        if f not in boundary_face_names:
            raise RuntimeError(f"unmatched face {f} of element {e}")
        bd_e.append(e); bd_f.append(f); bd_n.append(boundary_face_names[f])
    return Connectivity3D(np.asarray(if_e, dtype=np.int32).reshape(-1, 2),
                          np.asarray(if_f, dtype=np.int32).reshape(-1, 2),
                          np.asarray(if_o, dtype=np.int32),
                          np.asarray(bd_e, dtype=np.int32), np.asarray(bd_f, dtype=np.int32),
                          bd_n)


class P4estMeshCubedSphereTopography:
    """Cubed-sphere shell of 6 * trees_per_face_dimension^2 * layers hexahedra;
    initial_topography(lat, lon) (default: none, a perfect sphere) raises the
    ground, adapt_vertical_grid (GalChen() by default, or Sleve(eta_H, s))
    spreads it over the column."""

    ndims = 3

    def __init__(self, trees_per_face_dimension, layers, inner_radius, thickness, *, polydeg,
                 initial_topography=None, adapt_vertical_grid=None, geometry_on_device=False):
        """geometry_on_device: build node coordinates and metric terms with
        the library's kernel (tag_shell_geometry) instead of NumPy; the two
        agree to rounding (1e-15 relative)."""
        self.geometry_on_device = bool(geometry_on_device)
        self.initial_topography = initial_topography
        self.adapt_vertical_grid = adapt_vertical_grid or GalChen()
        self.nc = int(trees_per_face_dimension)
        self.nz = int(layers)
        self.inner_radius = float(inner_radius)
        self.thickness = float(thickness)
        self.polydeg = int(polydeg)
        self._geom = {}
        self._conn = None

    @property
    def nelements(self):
        return 6 * self.nc * self.nc * self.nz

    def node_coordinates(self, basis: LobattoLegendreBasis):
        nc, nz, n = self.nc, self.nz, basis.n
        nodes = basis.nodes
        dx = 2.0 / nc
        dz = 2.0 / nz
        out = np.empty((6, nc, nc, nz, n, n, n, 3))  # [dir, cy, cx, cz, k, j, i, c]
        cx = np.arange(nc)
        cz = np.arange(nz)
        XI = (-1 + cx * dx + dx / 2)[None, :, None, None, None, None] + \
            (dx / 2 * nodes)[None, None, None, None, None, :]
        ETA = (-1 + cx * dx + dx / 2)[:, None, None, None, None, None] + \
            (dx / 2 * nodes)[None, None, None, None, :, None]
        ZETA = (-1 + cz * dz + dz / 2)[None, None, :, None, None, None] + \
            (dz / 2 * nodes)[None, None, None, :, None, None]
        XI, ETA, ZETA = np.broadcast_arrays(XI, ETA, ZETA)  # [cy, cx, cz, k, j, i]
        for d in range(6):
            X, Y, Z = cubed_sphere_mapping(XI, ETA, ZETA, self.inner_radius, self.thickness, d + 1,
                                           self.initial_topography, self.adapt_vertical_grid)
            out[d, ..., 0], out[d, ..., 1], out[d, ..., 2] = X, Y, Z
        # element e = cz + nz * (cx + nc * (cy + nc * dir))
        out = out.transpose(0, 1, 2, 3, 4, 5, 6, 7).reshape(6, nc, nc, nz, n, n, n, 3)
        return np.ascontiguousarray(out.reshape(-1, n, n, n, 3))

    def ground_heights(self, basis: LobattoLegendreBasis):
        """Ground height of every column node [E, n(j), n(i)] (zero without a
        topography): the topography function at the latitude and longitude the
        reference takes for the node's column (cubed_sphere_mapping)."""
        nc, nz, n = self.nc, self.nz, basis.n
        E = self.nelements
        if self.initial_topography is None:
            return np.zeros((E, n, n))
        nodes = basis.nodes
        dx = 2.0 / nc
        c = -1 + np.arange(nc) * dx + dx / 2
        XI = c[None, :, None, None] + (dx / 2 * nodes)[None, None, None, :]   # [cy, cx, j, i]
        ETA = c[:, None, None, None] + (dx / 2 * nodes)[None, None, :, None]
        XI, ETA = np.broadcast_arrays(XI, ETA)
        out = np.empty((6, nc, nc, nz, n, n))
        for d in range(6):
            x, y = np.tan(XI * np.pi / 4), np.tan(ETA * np.pi / 4)
            one = np.ones_like(x)
            cube = {1: (-y, -x, -one), 2: (one, x, y), 3: (-x, one, y), 4: (-one, -x, y),
                    5: (x, -one, y), 6: (x, y, one)}[d + 1]
            r = np.sqrt(1 + x * x + y * y)
            ux, uy, uz = cube[0] / r, cube[1] / r, cube[2] / r
            zs = self.initial_topography(np.arcsin(uz / r), np.arctan2(uy, ux))
            out[d] = np.broadcast_to(zs[:, :, None], (nc, nc, nz, n, n))
        return np.ascontiguousarray(out.reshape(E, n, n))

    def geometry_device(self, basis: LobattoLegendreBasis):
        """(node coordinates, contravariant vectors, inverse Jacobian) built by
        the library's kernel, in the layouts of geometry()."""
        import ctypes
        from . import _lib
        L = _lib.load()
        n, E = basis.n, self.nelements
        xyz = np.empty((E, n, n, n, 3))
        Ja = np.empty((E, n, n, n, 3, 3))
        invJ = np.empty((E, n, n, n))
        dp = lambda a: a.ctypes.data_as(_lib._dp)  # noqa: E731
        nodes = np.ascontiguousarray(basis.nodes, dtype=np.float64)
        D = np.ascontiguousarray(basis.derivative_matrix, dtype=np.float64)
        zs = None if self.initial_topography is None else self.ground_heights(basis)
        vg = self.adapt_vertical_grid
        sleve = isinstance(vg, Sleve)
        _lib.check(L.tag_shell_geometry(
            self.nc, self.nz, self.inner_radius, self.thickness, basis.polydeg, dp(nodes), dp(D),
            dp(zs) if zs is not None else None, 1 if sleve else 0,
            vg.eta_H if sleve else 0.0, vg.s if sleve else 0.0, dp(xyz), dp(Ja), dp(invJ)))
        return xyz, Ja, invJ

    def geometry(self, basis: LobattoLegendreBasis):
        key = basis.polydeg
        if key not in self._geom and self.geometry_on_device:
            self._geom[key] = self.geometry_device(basis)
        if key not in self._geom:
            xyz = self.node_coordinates(basis)
            det, Ja = metric_terms_3d(xyz, basis.derivative_matrix)
            self._geom[key] = (xyz, np.ascontiguousarray(Ja), np.ascontiguousarray(1.0 / det))
        return self._geom[key]

    def connectivity(self, basis: LobattoLegendreBasis = None):
        if self._conn is None:
            basis = basis or LobattoLegendreBasis(self.polydeg)
            xyz = self.geometry(basis)[0]
            self._conn = match_faces(xyz, basis.n, {4: "inside", 5: "outside"})
        return self._conn
