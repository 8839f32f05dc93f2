"""Host-side mesh geometry and connectivity (the arrays Trixi's cache holds).

`StructuredMesh` mirrors `Trixi.StructuredMesh(cells_per_dimension,
coordinates_min, coordinates_max; periodicity)` as used by the reference's
elixirs (e.g. examples/euler/dry_air/buoyancy/elixir_energy_inertia_gravity_waves.jl:46-50).
Geometry is built once on the host, like Trixi's `create_cache`, and uploaded
by `tag_create`.  Arrays are stored so that their C-order memory equals
Trixi's column-major layout:
  node_coordinates[e, j, i, c]          == node_coordinates[c, i, j, e]
  contravariant_vectors[e, j, i, d, c]  == contravariant_vectors[c, d, i, j, e]
  inverse_jacobian[e, j, i]             == inverse_jacobian[i, j, e]
Element e of an nx x ny mesh is cell (cx, cy) with e = cx + nx * cy.
Faces: 0 = xi-, 1 = xi+, 2 = eta-, 3 = eta+.
"""
from __future__ import annotations

import numpy as np

from .basis import LobattoLegendreBasis


class Connectivity:
    """Interface and boundary-face lists in the C ABI's form."""

    def __init__(self):
        self.if_elements = []  # (primary, secondary)
        self.if_faces = []
        self.if_flip = []
        self.bd_elements = []
        self.bd_faces = []
        self.bd_names = []  # boundary name per face ("x_neg", ...)

    def arrays(self):
        ie = np.asarray(self.if_elements, dtype=np.int32).reshape(-1, 2)
        ifc = np.asarray(self.if_faces, dtype=np.int32).reshape(-1, 2)
        fl = np.asarray(self.if_flip, dtype=np.int32)
        be = np.asarray(self.bd_elements, dtype=np.int32)
        bf = np.asarray(self.bd_faces, dtype=np.int32)
        return ie, ifc, fl, be, bf


def transfinite_mapping(faces):
    """The Coons patch (transfinite interpolation) of four boundary curves, as
    `Trixi.StructuredMesh(cells_per_dimension, faces)` builds its mapping:
    faces = (xi = -1, xi = +1, eta = -1, eta = +1) curves, each s -> (x, y)
    for s in [-1, 1], meeting at the corners.  The mapping is the sum of the
    linear blends between opposite faces minus the bilinear blend of the four
    corners, so that it reproduces every face exactly."""
    f1, f2, f3, f4 = faces

    def pt(f, s):
        x, y = f(s)
        return np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)

    c00, c10 = pt(f1, -1.0), pt(f2, -1.0)  # bottom left / right
    c01, c11 = pt(f1, 1.0), pt(f2, 1.0)    # top left / right

    def mapping(xi, eta):
        out = []
        a1, a2, b3, b4 = pt(f1, eta), pt(f2, eta), pt(f3, xi), pt(f4, xi)
        for d in range(2):
            lin_xi = 0.5 * ((1.0 - xi) * a1[d] + (1.0 + xi) * a2[d])
            lin_eta = 0.5 * ((1.0 - eta) * b3[d] + (1.0 + eta) * b4[d])
            bil = 0.25 * (c00[d] * (1.0 - xi) * (1.0 - eta) + c10[d] * (1.0 + xi) * (1.0 - eta) +
                          c01[d] * (1.0 - xi) * (1.0 + eta) + c11[d] * (1.0 + xi) * (1.0 + eta))
            out.append(lin_xi + lin_eta - bil)
        return tuple(out)

    return mapping


class WitchOfAgnesi:
    """Bell-shaped ridge h(x) = height / (1 + (x / half_width)^2)
    (src/equations/initial_condition_compressible_euler_2d.jl:229-258)."""

    def __init__(self, *, height, half_width):
        self.height, self.half_width = float(height), float(half_width)

    def __call__(self, x):
        return self.height / (1.0 + (x / self.half_width) ** 2)


class SchaerMountain:
    """Schaer et al.'s ridges h(x) = height exp(-(x / half_width)^2)
    cos^2(pi x / wavelength) (initial_condition_compressible_euler_2d.jl:202-227)."""

    def __init__(self, *, height, half_width, wavelength):
        self.height, self.half_width = float(height), float(half_width)
        self.wavelength = float(wavelength)

    def __call__(self, x):
        return (self.height * np.exp(-(x / self.half_width) ** 2) *
                np.cos(np.pi * (x / self.wavelength)) ** 2)


SchärMountain = SchaerMountain


def terrain_following_faces(topography, x_min, x_max, z_top):
    """(left, right, bottom, top) boundary curves of a terrain-following
    domain [x_min, x_max] x [topography(x), z_top]
    (initial_condition_compressible_euler_2d.jl:260-285); each s in [-1, 1] ->
    (x, z)."""
    x_min, x_max, z_top = float(x_min), float(x_max), float(z_top)
    x_mid = 0.5 * (x_min + x_max)
    x_half = 0.5 * (x_max - x_min)
    z_left, z_right = float(topography(x_min)), float(topography(x_max))

    def x_of(s):
        return x_mid + x_half * s

    def f_left(s):
        return x_min + 0.0 * s, z_left + (z_top - z_left) * 0.5 * (s + 1)

    def f_right(s):
        return x_max + 0.0 * s, z_right + (z_top - z_right) * 0.5 * (s + 1)

    def f_bottom(s):
        return x_of(s), topography(x_of(s))

    def f_top(s):
        return x_of(s), z_top + 0.0 * s

    return f_left, f_right, f_bottom, f_top


class StructuredMesh:
    """2D StructuredMesh on [xmin, xmax] x [ymin, ymax], or of a mapping
    (xi, eta) in [-1, 1]^2 -> (x, y), or of four boundary curves `faces`
    (transfinite_mapping)."""

    ndims = 2

    def __init__(self, cells_per_dimension, coordinates_min=None, coordinates_max=None,
                 periodicity=(True, True), mapping=None, faces=None):
        self.nx, self.ny = map(int, cells_per_dimension)
        self.periodicity = tuple(bool(p) for p in periodicity)
        if faces is not None:
            mapping = transfinite_mapping(faces)
        if mapping is None:
            x0, y0 = map(float, coordinates_min)
            x1, y1 = map(float, coordinates_max)

            def mapping(xi, eta):
                return (x0 + 0.5 * (xi + 1.0) * (x1 - x0), y0 + 0.5 * (eta + 1.0) * (y1 - y0))
        self.mapping = mapping

    @property
    def nelements(self):
        return self.nx * self.ny

    def geometry(self, basis: LobattoLegendreBasis):
        """node_coordinates, contravariant_vectors, inverse_jacobian."""
        nx, ny, n = self.nx, self.ny, basis.n
        E = nx * ny
        xr = basis.nodes
        dxr, dyr = 2.0 / nx, 2.0 / ny
        cx = np.arange(nx)
        cy = np.arange(ny)
        ox = -1.0 + cx * dxr + 0.5 * dxr
        oy = -1.0 + cy * dyr + 0.5 * dyr
        # xi[cy, cx, j, i], eta[...]
        XI = ox[None, :, None, None] + 0.5 * dxr * xr[None, None, None, :]
        ETA = oy[:, None, None, None] + 0.5 * dyr * xr[None, None, :, None]
        XI, ETA = np.broadcast_arrays(XI, ETA)
        X, Y = self.mapping(XI, ETA)
        X = np.broadcast_to(X, XI.shape).reshape(E, n, n)
        Y = np.broadcast_to(Y, XI.shape).reshape(E, n, n)
        D = basis.derivative_matrix
        # derivatives: xi along i (last axis), eta along j
        x_xi = np.einsum("ik,ejk->eji", D, X)
        y_xi = np.einsum("ik,ejk->eji", D, Y)
        x_eta = np.einsum("jk,eki->eji", D, X)
        y_eta = np.einsum("jk,eki->eji", D, Y)
        coords = np.stack([X, Y], axis=-1)
        Ja = np.zeros((E, n, n, 2, 2))
        Ja[..., 0, 0] = y_eta
        Ja[..., 0, 1] = -x_eta
        Ja[..., 1, 0] = -y_xi
        Ja[..., 1, 1] = x_xi
        invJ = 1.0 / (x_xi * y_eta - x_eta * y_xi)
        return (np.ascontiguousarray(coords), np.ascontiguousarray(Ja),
                np.ascontiguousarray(invJ))

    def connectivity(self):
        c = Connectivity()
        nx, ny = self.nx, self.ny
        px, py = self.periodicity
        for cyi in range(ny):
            for cxi in range(nx):
                e = cxi + nx * cyi
                if cxi < nx - 1 or px:
                    c.if_elements.append((e, (cxi + 1) % nx + nx * cyi))
                    c.if_faces.append((1, 0))
                    c.if_flip.append(0)
                if cyi < ny - 1 or py:
                    c.if_elements.append((e, cxi + nx * ((cyi + 1) % ny)))
                    c.if_faces.append((3, 2))
                    c.if_flip.append(0)
                if not px and cxi == 0:
                    c.bd_elements.append(e); c.bd_faces.append(0); c.bd_names.append("x_neg")
                if not px and cxi == nx - 1:
                    c.bd_elements.append(e); c.bd_faces.append(1); c.bd_names.append("x_pos")
                if not py and cyi == 0:
                    c.bd_elements.append(e); c.bd_faces.append(2); c.bd_names.append("y_neg")
                if not py and cyi == ny - 1:
                    c.bd_elements.append(e); c.bd_faces.append(3); c.bd_names.append("y_pos")
        return c


def _morton(qx, qy, level):
    """p4est's Morton index of quadrant (qx, qy) at a uniform level (x is the
    low bit of each pair)."""
    m = 0
    for b in range(level):
        m |= ((qx >> b) & 1) << (2 * b)
        m |= ((qy >> b) & 1) << (2 * b + 1)
    return m


class P4estMesh:
    """2D `P4estMesh(trees_per_dimension; polydeg, coordinates_min,
    coordinates_max, initial_refinement_level, periodicity)` of a rectangle
    (the form the reference's elixirs use, e.g.
    examples/euler/dry_air/buoyancy/elixir_gemein_bubble.jl:72-77): a brick of
    trees, each refined uniformly, with an affine mapping.  Elements follow
    p4est's order (trees with x fastest, the quadrants of a tree in Morton
    order); slip walls take the outward-normal (P4estMesh) method."""

    ndims = 2
    normal_walls = True

    def __init__(self, trees_per_dimension, *, polydeg=1, coordinates_min=None,
                 coordinates_max=None, mapping=None, faces=None, initial_refinement_level=0,
                 periodicity=True):
        """mapping(xi, eta) -> (x, y) of the global reference square [-1, 1]^2
        (the `mapping` keyword of the reference's P4estMesh, e.g.
        examples/euler/dry_air/tests/elixir_potential_temperature_well_balanced_curvilinear.jl),
        or the transfinite mapping of four boundary curves `faces` (e.g.
        terrain_following_faces, examples/euler/dry_air/mountain_flow/*.jl);
        otherwise the affine map of coordinates_min / coordinates_max.  Trees
        are not refined when a mapping is given."""
        if faces is not None:
            mapping = transfinite_mapping(faces)
        tx, ty = map(int, trees_per_dimension)
        if isinstance(periodicity, bool):
            periodicity = (periodicity, periodicity)
        L = int(initial_refinement_level)
        if mapping is not None and L != 0:
            raise ValueError("a mapped P4estMesh is supported at initial_refinement_level = 0")
        k = 1 << L
        self.trees_per_dimension = (tx, ty)
        self.level = L
        self.polydeg = int(polydeg)
        self._grid = StructuredMesh((tx * k, ty * k), coordinates_min, coordinates_max,
                                    periodicity, mapping=mapping)
        nx = tx * k
        perm = np.empty(tx * ty * k * k, dtype=np.int64)
        for tyi in range(ty):
            for txi in range(tx):
                tree = txi + tx * tyi
                for qy in range(k):
                    for qx in range(k):
                        e = tree * k * k + _morton(qx, qy, L)
                        perm[e] = (txi * k + qx) + nx * (tyi * k + qy)
        self.perm = perm                 # p4est element -> row-major cell
        self.inv = np.argsort(perm)      # row-major cell -> p4est element

    @property
    def nelements(self):
        return self._grid.nelements

    def geometry(self, basis: LobattoLegendreBasis):
        xy, ja, ij = self._grid.geometry(basis)
        return (np.ascontiguousarray(xy[self.perm]), np.ascontiguousarray(ja[self.perm]),
                np.ascontiguousarray(ij[self.perm]))

    def connectivity(self):
        g = self._grid.connectivity()
        c = Connectivity()
        c.if_elements = [(int(self.inv[a]), int(self.inv[b])) for a, b in g.if_elements]
        c.if_faces = list(g.if_faces)
        c.if_flip = list(g.if_flip)
        c.bd_elements = [int(self.inv[e]) for e in g.bd_elements]
        c.bd_faces = list(g.bd_faces)
        c.bd_names = list(g.bd_names)
        return c
