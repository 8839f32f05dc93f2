"""Covariant metric terms computed on the device (tag_cov_metric_terms)
against the host NumPy construction of the same 26 auxiliary variables and
node coordinates: Cartesian and spherical global components, exact (dual
number) and collocation Christoffel symbols, degrees 1-7.  Tolerance: every
slot within 1e-12 of its largest magnitude over the mesh (the Christoffel
symbols, derivatives of the metric, within 1e-10 of the largest of them).  A pole node in spherical
components is reported as an error, as on the host."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(tg, k, N, spherical, collocation, topo=None):
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import EARTH_RADIUS
    coords = cv.GlobalSphericalCoordinates() if spherical else cv.GlobalCartesianCoordinates()
    eq = cv.CovariantShallowWaterEquations2D(9.80616, 7.292e-5, coords)
    mesh = cv.P4estMeshCubedSphere2D(k, EARTH_RADIUS, polydeg=N)
    basis = tg.LobattoLegendreBasis(N)
    metric = cv.MetricTermsCovariantSphere(cv.ChristoffelSymbolsCollocationDerivative()
                                           if collocation else cv.ChristoffelSymbolsAutodiff())
    return cv, mesh, basis, eq, metric


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 7])
@pytest.mark.parametrize("spherical,collocation", [(False, False), (False, True), (True, False)])
def test_device_metric_terms_match_host(tg, gpu_lib, N, spherical, collocation):
    if spherical and N % 2 == 0:
        # an even degree puts a node on a pole (the centre node of the middle
        # element for odd k, element corners for even k)
        pytest.skip("pole node in spherical components")
    cv, mesh, basis, eq, metric = _setup(tg, 3, N, spherical, collocation)
    topo = cv.bottom_topography_isolated_mountain
    aux_h, xyz_h = cv.compute_aux_vars(mesh, basis, eq, metric, topo)
    aux_d, xyz_d = cv.compute_aux_vars(mesh, basis, eq, metric, topo, device=True)
    assert np.abs(xyz_d - xyz_h).max() <= 1e-12 * np.abs(xyz_h).max()
    chris = np.abs(aux_h[..., 20:26]).max()
    for s in range(26):
        # the Christoffel symbols against the largest of them: some vanish
        # analytically and are rounding noise of either construction
        scale = chris if s >= 20 else max(np.abs(aux_h[..., s]).max(), 1e-300)
        tol = 1e-10 if s >= 20 else 1e-12
        err = np.abs(aux_d[..., s] - aux_h[..., s]).max()
        assert err <= tol * scale, (s, err / scale)


def test_device_metric_terms_report_pole_singularity(tg, gpu_lib):
    cv, mesh, basis, eq, metric = _setup(tg, 3, 2, True, False)
    with pytest.raises(Exception):
        cv.compute_aux_vars(mesh, basis, eq, metric, None, device=True)


@pytest.mark.parametrize("topo", [None, "galchen", "sleve"])
def test_shell_geometry_on_device_matches_host(tg, gpu_lib, topo):
    """tag_shell_geometry (node coordinates, curl-form contravariant vectors,
    inverse Jacobian of the cubed-sphere shell) against the host mirror's NumPy
    construction, on a perfect sphere and over a mountain spread by Gal-Chen
    or Sleve vertical coordinates.  Coordinates agree to 1e-13 of their
    size.  The contravariant vectors and the inverse Jacobian agree to 1e-11:
    the curl form differences products X_l grad X_m of size R^2 ~ 4e13 m^2
    down to entries of size R times an element's width, and the device's fma
    sums round differently from NumPy's matrix products, so the cancellation
    amplifies the rounding by about R over the element's thickness (~1e3)."""
    def mountain(lat, lon):
        return 2000.0 * np.exp(-((lat - 0.5) ** 2 + (lon - 1.0) ** 2) / 0.05)
    kw = {}
    if topo:
        kw = dict(initial_topography=mountain,
                  adapt_vertical_grid=tg.GalChen() if topo == "galchen" else tg.Sleve(0.7, 0.8))
    for N in (2, 5):
        basis = tg.LobattoLegendreBasis(N)
        host = tg.P4estMeshCubedSphereTopography(3, 2, 6.371e6, 30000.0, polydeg=N, **kw)
        dev = tg.P4estMeshCubedSphereTopography(3, 2, 6.371e6, 30000.0, polydeg=N,
                                                geometry_on_device=True, **kw)
        for a, b, tol in zip(host.geometry(basis), dev.geometry(basis), (1e-13, 1e-11, 1e-11)):
            assert a.shape == b.shape
            assert np.abs(a - b).max() <= tol * np.abs(a).max(), np.abs(a - b).max()
