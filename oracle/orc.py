"""ORACLE — test infrastructure only.

ctypes wrapper around ``oracle/_build/liboracle.so``, the C++ CPU restatement
of the reference's `rhs!` used as the checker for the CUDA path (and as the
timed CPU baseline).  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU legs may import this module; the product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_FLOPS_PATH = os.path.join(_HERE, "_build", "liborcflops.so")
_lib = None
_flops = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip_t = ctypes.POINTER(ctypes.c_int32)


def _ip(a):
    return a.ctypes.data_as(_ip_t)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ + OpenMP)."""
    cmd = ["make", "-C", _HERE]
    if force:
        cmd.insert(1, "-B")
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_euler2d_create.restype = ctypes.c_void_p
        L.orc_euler2d_create.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 4 + [
            ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 4
        L.orc_euler2d_destroy.argtypes = [ctypes.c_void_p]
        L.orc_euler2d_ndofs.restype = ctypes.c_int64
        L.orc_euler2d_ndofs.argtypes = [ctypes.c_void_p]
        L.orc_euler2d_basis.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp]
        L.orc_euler2d_geometry.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_euler2d_initial_condition.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
        L.orc_euler2d_rhs.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double]
        L.orc_euler2d_max_dt.restype = ctypes.c_double
        L.orc_euler2d_max_dt.argtypes = [ctypes.c_void_p, _dp]
        L.orc_euler2d_ck_steps.restype = ctypes.c_double
        L.orc_euler2d_ck_steps.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int, ctypes.c_double]
        L.orc_euler2d_ssprk43_run.restype = ctypes.c_int
        L.orc_euler2d_ssprk43_run.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_double]
        L.orc_euler2d_errors_gravity_waves.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        _ip = _ip_t
        L.orc_euler3d_create.restype = ctypes.c_void_p
        L.orc_euler3d_create.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int,
                                         _ip, _ip, _ip, ctypes.c_int, _ip, _ip] + \
            [ctypes.c_double] * 5
        L.orc_euler3d_destroy.argtypes = [ctypes.c_void_p]
        L.orc_euler3d_rhs.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double]
        L.orc_euler3d_max_dt.restype = ctypes.c_double
        L.orc_euler3d_max_dt.argtypes = [ctypes.c_void_p, _dp]
        L.orc_euler3d_ck_steps.restype = ctypes.c_double
        L.orc_euler3d_ck_steps.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int, ctypes.c_double]
        L.orc_cov_create.restype = ctypes.c_void_p
        L.orc_cov_create.argtypes = ([ctypes.c_int] * 2 + [_dp, _dp, ctypes.c_int, _ip, _ip, _ip] +
                                     [ctypes.c_double] * 2 + [ctypes.c_int] * 7)
        L.orc_cov_destroy.argtypes = [ctypes.c_void_p]
        L.orc_cov_rhs.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_cov_max_dt.restype = ctypes.c_double
        L.orc_cov_max_dt.argtypes = [ctypes.c_void_p, _dp]
        L.orc_cov_ck_steps.restype = ctypes.c_double
        L.orc_cov_ck_steps.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double]
        L.orc_pt_create.restype = ctypes.c_void_p
        L.orc_pt_create.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_double] * 4 + [ctypes.c_int] * 5 +
                                    [ctypes.c_double] * 4 + [ctypes.c_int] * 2)
        L.orc_pt_set_mountain.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_pt_create_mesh.restype = ctypes.c_void_p
        L.orc_pt_create_mesh.argtypes = ([ctypes.c_int] * 2 + [_dp] * 3 + [ctypes.c_int] +
                                         [_ip] * 3 + [ctypes.c_int] + [_ip] * 3 +
                                         [ctypes.c_int] * 4 + [ctypes.c_double] * 4)
        L.orc_pt_destroy.argtypes = [ctypes.c_void_p]
        L.orc_pt_initial_condition_gravity_waves.argtypes = [ctypes.c_void_p, _dp]
        L.orc_pt_errors_gravity_waves.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_pt_rhs.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double]
        L.orc_pt_max_dt.restype = ctypes.c_double
        L.orc_pt_max_dt.argtypes = [ctypes.c_void_p, _dp]
        L.orc_pt_ssprk43_run.restype = ctypes.c_int
        L.orc_pt_ssprk43_run.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double]
        for name in ("orc_euler2d_ssp_steps", "orc_moist_ssp_steps", "orc_pt_ssp_steps",
                     "orc_cov_ssp_steps", "orc_euler3d_ssp_steps"):
            f = getattr(L, name)
            f.restype = ctypes.c_double
            f.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                          ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_pt_ssprk43_adaptive.restype = ctypes.c_double
        L.orc_pt_ssprk43_adaptive.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double,
                                              ctypes.c_double, _dp, ctypes.c_int, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_int, _dp]
        L.orc_pt3d_ssprk43_adaptive.restype = ctypes.c_double
        L.orc_pt3d_ssprk43_adaptive.argtypes = L.orc_pt_ssprk43_adaptive.argtypes
        L.orc_rainy_ssprk43_adaptive.restype = ctypes.c_double
        L.orc_rainy_ssprk43_adaptive.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double,
                                                 ctypes.c_double, _dp, ctypes.c_int,
                                                 ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp]
        L.orc_pt_ck_steps.restype = ctypes.c_double
        L.orc_pt_ck_steps.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int]
        L.orc_pt_stolarsky.restype = ctypes.c_double
        L.orc_pt_stolarsky.argtypes = [ctypes.c_double] * 3
        for name in ("orc_ln_mean", "orc_inv_ln_mean"):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [ctypes.c_double] * 2
        L.orc_moist_create_mesh.restype = ctypes.c_void_p
        L.orc_moist_create_mesh.argtypes = ([ctypes.c_int] * 2 + [_dp] * 3 + [ctypes.c_int] +
                                            [_ip] * 3 + [ctypes.c_int] + [_ip] * 3 +
                                            [ctypes.c_int] * 3 + [ctypes.c_double] * 2 +
                                            [ctypes.c_int])
        L.orc_moist_create.restype = ctypes.c_void_p
        L.orc_moist_create.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_double] * 4 +
                                       [ctypes.c_int] * 6 + [ctypes.c_double] * 2 + [ctypes.c_int])
        L.orc_moist_destroy.argtypes = [ctypes.c_void_p]
        L.orc_moist_initial_condition.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp]
        L.orc_moist_errors.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, _dp, _dp]
        L.orc_moist_rhs.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double]
        L.orc_moist_max_dt.restype = ctypes.c_double
        L.orc_moist_max_dt.argtypes = [ctypes.c_void_p, _dp]
        L.orc_moist_ck_steps.restype = ctypes.c_double
        L.orc_moist_ck_steps.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double]
        L.orc_moist_flux_chandrashekar.argtypes = [_dp, _dp, _dp, _dp]
        L.orc_moist_flux.argtypes = [_dp, _dp, _dp]
        L.orc_rainy_flux_lmars.argtypes = [_dp, _dp, _dp, _dp]
        L.orc_rainy_slip_wall.argtypes = [_dp, _dp, _dp]
        L.orc_rainy_create_mesh.restype = ctypes.c_void_p
        L.orc_rainy_create_mesh.argtypes = ([ctypes.c_int] * 2 + [_dp] * 3 + [ctypes.c_int] +
                                            [_ip] * 3 + [ctypes.c_int] + [_ip] * 3 +
                                            [ctypes.c_int] * 4)
        L.orc_rainy_create.restype = ctypes.c_void_p
        L.orc_rainy_create.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 4 + [ctypes.c_int] * 4
        L.orc_rainy_geometry.argtypes = [ctypes.c_void_p, _dp]
        L.orc_rainy_initial_condition_convergence.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp]
        L.orc_rainy_errors_convergence.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, _dp, _dp]
        L.orc_rainy_destroy.argtypes = [ctypes.c_void_p]
        L.orc_rainy_rhs.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double]
        L.orc_rainy_max_dt.restype = ctypes.c_double
        L.orc_rainy_max_dt.argtypes = [ctypes.c_void_p, _dp]
        L.orc_rainy_newton.restype = ctypes.c_long
        L.orc_rainy_newton.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, _dp, _ip,
                                       ctypes.POINTER(ctypes.c_long)]
        L.orc_rainy_newton_states.restype = ctypes.c_long
        L.orc_rainy_newton_states.argtypes = [_dp, ctypes.c_long, ctypes.c_int, ctypes.c_double,
                                              ctypes.c_int, ctypes.c_int, _dp, _ip,
                                              ctypes.POINTER(ctypes.c_long)]
        L.orc_pt3d_create.restype = ctypes.c_void_p
        L.orc_pt3d_create.argtypes = ([ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int,
                                       _ip, _ip, _ip, ctypes.c_int, _ip, _ip] +
                                      [ctypes.c_double] * 5 + [ctypes.c_int] * 2)
        L.orc_pt3d_destroy.argtypes = [ctypes.c_void_p]
        L.orc_pt3d_rhs.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double]
        L.orc_pt3d_max_dt.restype = ctypes.c_double
        L.orc_pt3d_max_dt.argtypes = [ctypes.c_void_p, _dp]
        L.orc_pt3d_ck_steps.restype = ctypes.c_double
        L.orc_pt3d_ck_steps.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int, ctypes.c_double]
        L.orc_pt3d_ssp_steps.restype = ctypes.c_double
        L.orc_pt3d_ssp_steps.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double]
        for name in ("orc_pt3d_pointwise", "orc_pt2d_pointwise"):
            getattr(L, name).argtypes = [ctypes.c_int] * 3 + [ctypes.c_double, _dp, _dp, _dp, _dp]
        L.orc_ie_create.restype = ctypes.c_void_p
        L.orc_ie_create.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_double] * 4 +
                                    [ctypes.c_int] * 2 + [ctypes.c_double] * 3 + [ctypes.c_int])
        L.orc_ie_destroy.argtypes = [ctypes.c_void_p]
        L.orc_ie_rhs.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double]
        L.orc_ie_max_dt.restype = ctypes.c_double
        L.orc_ie_max_dt.argtypes = [ctypes.c_void_p, _dp]
        L.orc_ie_ssp_steps.restype = ctypes.c_double
        L.orc_ie_ssp_steps.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double]
        L.orc_ie_pointwise.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp]
        L.orc_rainy_ssp_steps.restype = ctypes.c_double
        L.orc_rainy_ssp_steps.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_int]
        L.orc_rainy_ck_steps.restype = ctypes.c_double
        L.orc_rainy_ck_steps.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_double]
        L.orc_rainy_flux_ec.argtypes = [_dp, _dp, _dp, _dp]
        L.orc_rainy_flux.argtypes = [_dp, _dp, _dp]
        L.orc_rainy_saturation_vapour_pressure.restype = ctypes.c_double
        L.orc_rainy_saturation_vapour_pressure.argtypes = [ctypes.c_double]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


class Euler2D:
    """Dry Euler (energy + gravity) on a StructuredMesh rectangle, CPU oracle."""

    nv = 5

    def __init__(self, polydeg, nx, ny, x0, x1, y0, y1, periodic_x=True, periodic_y=False,
                 c_p=1004.0, c_v=717.0, g=9.81, c_lmars=340.0):
        self.n = polydeg + 1
        self.nelem = nx * ny
        self.h = lib().orc_euler2d_create(polydeg, nx, ny, x0, x1, y0, y1, int(periodic_x),
                                          int(periodic_y), c_p, c_v, g, c_lmars)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_euler2d_destroy(self.h)
            self.h = None

    @property
    def ndofs(self):
        return self.nelem * self.n * self.n

    def shape(self):
        return (self.nelem, self.n, self.n, self.nv)

    def basis(self):
        n = self.n
        x, w = np.zeros(n), np.zeros(n)
        D, Ds = np.zeros((n, n)), np.zeros((n, n))
        lib().orc_euler2d_basis(self.h, _p(x), _p(w), _p(D), _p(Ds))
        return x, w, D, Ds

    def geometry(self):
        n, E = self.n, self.nelem
        Ja = np.zeros((E, n, n, 2, 2))
        invJ = np.zeros((E, n, n))
        xy = np.zeros((E, n, n, 2))
        lib().orc_euler2d_geometry(self.h, _p(Ja), _p(invJ), _p(xy))
        return Ja, invJ, xy

    def initial_condition(self, which=0, params=(10000.0, 2000.0, 2000.0, 2.0, 0.0)):
        u = np.zeros(self.shape())
        prm = np.asarray(params, dtype=np.float64)
        lib().orc_euler2d_initial_condition(self.h, which, _p(prm), _p(u))
        return u

    def rhs(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.zeros_like(u)
        lib().orc_euler2d_rhs(self.h, _p(u), _p(du), t)
        return du

    def max_dt(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        return lib().orc_euler2d_max_dt(self.h, _p(u))

    def ck_steps(self, u, k, t, cfl, nsteps, fixed_dt=0.0):
        return lib().orc_euler2d_ck_steps(self.h, _p(u), _p(k), t, cfl, nsteps, fixed_dt)

    def ssp_steps(self, u, t, cfl, nsteps, scheme, fixed_dt=0.0, t_end=0.0):
        """SSPRK43 (scheme 1) or SSPRK33 (scheme 2) steps; returns the new time."""
        return lib().orc_euler2d_ssp_steps(self.h, _p(u), t, cfl, nsteps, scheme, fixed_dt, t_end)

    def ssprk43_run(self, u, t0, t_end, cfl):
        return lib().orc_euler2d_ssprk43_run(self.h, _p(u), t0, t_end, cfl)

    def errors_gravity_waves(self, u):
        l2, linf = np.zeros(5), np.zeros(5)
        lib().orc_euler2d_errors_gravity_waves(self.h, _p(u), _p(l2), _p(linf))
        return l2, linf


class Euler3D:
    """Dry Euler (energy + gravity) 3D on a hexahedral mesh; geometry and
    connectivity are the host mirror's arrays (the same ones the C ABI takes)."""

    nv = 6

    def __init__(self, polydeg, Ja, invJ, xyz, if_elements, if_faces, if_orient, bd_elements,
                 bd_faces, c_p=1004.0, c_v=717.0, g=9.81, c_lmars=340.0, omega=0.0):
        self.n = polydeg + 1
        self.nelem = invJ.shape[0]
        self._keep = [np.ascontiguousarray(a) for a in (Ja, invJ, xyz)]
        ints = [np.ascontiguousarray(a, dtype=np.int32) for a in
                (if_elements, if_faces, if_orient, bd_elements, bd_faces)]
        self._keep += ints
        self.h = lib().orc_euler3d_create(polydeg, self.nelem, _p(self._keep[0]),
                                          _p(self._keep[1]), _p(self._keep[2]),
                                          len(ints[2]), _ip(ints[0]), _ip(ints[1]),
                                          _ip(ints[2]), len(ints[3]), _ip(ints[3]),
                                          _ip(ints[4]), c_p, c_v, g, c_lmars, omega)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_euler3d_destroy(self.h)
            self.h = None

    def rhs(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.zeros_like(u)
        lib().orc_euler3d_rhs(self.h, _p(u), _p(du), t)
        return du

    def max_dt(self, u):
        return lib().orc_euler3d_max_dt(self.h, _p(np.ascontiguousarray(u)))

    def ck_steps(self, u, k, t, cfl, nsteps, fixed_dt=0.0):
        return lib().orc_euler3d_ck_steps(self.h, _p(u), _p(k), t, cfl, nsteps, fixed_dt)

    def ssp_steps(self, u, t, cfl, nsteps, scheme, fixed_dt=0.0, t_end=0.0):
        """SSPRK43 (scheme 1) or SSPRK33 (scheme 2) steps; returns the new time."""
        return lib().orc_euler3d_ssp_steps(self.h, _p(u), t, cfl, nsteps, scheme, fixed_dt, t_end)


class PotTemp3D:
    """Potential-temperature Euler with gravity in 3D (shell geometry and
    connectivity are the host mirror's arrays).  volume 0 flux_tec, 1 flux_ec,
    2 flux_etec, 3 flux_kennedy_gruber; nc 0 waruszewski, 1 artiano, 2 souza."""

    nv = 6

    def __init__(self, polydeg, Ja, invJ, xyz, if_elements, if_faces, if_orient, bd_elements,
                 bd_faces, c_p=1004.0, c_v=717.0, g=9.80616, c_lmars=340.0, omega=0.0,
                 volume=0, nc=0):
        self.n = polydeg + 1
        self.nelem = invJ.shape[0]
        self._keep = [np.ascontiguousarray(a) for a in (Ja, invJ, xyz)]
        ints = [np.ascontiguousarray(a, dtype=np.int32) for a in
                (if_elements, if_faces, if_orient, bd_elements, bd_faces)]
        self._keep += ints
        self.h = lib().orc_pt3d_create(polydeg, self.nelem, _p(self._keep[0]), _p(self._keep[1]),
                                       _p(self._keep[2]), len(ints[2]), _ip(ints[0]),
                                       _ip(ints[1]), _ip(ints[2]), len(ints[3]), _ip(ints[3]),
                                       _ip(ints[4]), c_p, c_v, g, c_lmars, omega, volume, nc)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_pt3d_destroy(self.h)
            self.h = None

    def rhs(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.zeros_like(u)
        lib().orc_pt3d_rhs(self.h, _p(u), _p(du), t)
        return du

    def max_dt(self, u):
        return lib().orc_pt3d_max_dt(self.h, _p(np.ascontiguousarray(u)))

    def ck_steps(self, u, k, t, cfl, nsteps, fixed_dt=0.0):
        return lib().orc_pt3d_ck_steps(self.h, _p(u), _p(k), t, cfl, nsteps, fixed_dt)

    def ssp_steps(self, u, t, cfl, nsteps, scheme, fixed_dt=0.0, t_end=0.0):
        return lib().orc_pt3d_ssp_steps(self.h, _p(u), t, cfl, nsteps, scheme, fixed_dt, t_end)

    def ssprk43_adaptive(self, u, t, t_end, abstol=1e-6, reltol=1e-3, stops=(), variant=0):
        """Adaptive SSPRK43 (see PotTemp2D.ssprk43_adaptive)."""
        st = np.zeros(5)
        sp = np.ascontiguousarray(stops, dtype=np.float64)
        tf = lib().orc_pt3d_ssprk43_adaptive(self.h, _p(u), t, t_end, _p(sp) if sp.size else None,
                                             int(sp.size), abstol, reltol, variant, _p(st))
        return tf, dict(zip(("accepted", "rejected", "rhs_calls", "dt_first", "dt_last"), st))


def pt_pointwise(ndims, kind, ul, ur, n, volume=0, nc=0, c=340.0):
    """Pointwise potential-temperature fluxes (kind 0 flux, 1 volume flux,
    2 nonconservative gravity term, 3 LMARS) of the 2D or 3D equations."""
    nv = ndims + 3
    f = np.zeros(nv)
    fn = lib().orc_pt3d_pointwise if ndims == 3 else lib().orc_pt2d_pointwise
    fn(kind, volume, nc, c, _p(np.ascontiguousarray(ul, dtype=np.float64)),
       _p(np.ascontiguousarray(ur, dtype=np.float64)),
       _p(np.ascontiguousarray(n, dtype=np.float64)), _p(f))
    return f


class InternalEnergy2D:
    """Internal-energy Euler with gravity on a rectangle with outward-normal
    slip walls: (flux_conservative_etec, flux_nonconservative_etec) volume,
    (flux_conservative_es, flux_nonconservative_es) surface flux."""

    nv = 5

    def __init__(self, polydeg, nx, ny, x0, x1, y0, y1, periodic_x=True, periodic_y=False,
                 c_p=1004.0, c_v=717.0, g=9.81, surface_etec=False):
        self.n = polydeg + 1
        self.nelem = nx * ny
        self.h = lib().orc_ie_create(polydeg, nx, ny, x0, x1, y0, y1, int(periodic_x),
                                     int(periodic_y), c_p, c_v, g, int(surface_etec))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_ie_destroy(self.h)
            self.h = None

    def rhs(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.zeros_like(u)
        lib().orc_ie_rhs(self.h, _p(u), _p(du), t)
        return du

    def max_dt(self, u):
        return lib().orc_ie_max_dt(self.h, _p(np.ascontiguousarray(u)))

    def ssp_steps(self, u, t, cfl, nsteps, scheme, fixed_dt=0.0, t_end=0.0):
        return lib().orc_ie_ssp_steps(self.h, _p(u), t, cfl, nsteps, scheme, fixed_dt, t_end)


def ie_pointwise(kind, ul, ur, n):
    """kind 0 flux, 1 flux_conservative_etec, 2 flux_nonconservative_etec,
    3 flux_conservative_es, 4 flux_nonconservative_es."""
    f = np.zeros(5)
    lib().orc_ie_pointwise(kind, _p(np.ascontiguousarray(ul, dtype=np.float64)),
                           _p(np.ascontiguousarray(ur, dtype=np.float64)),
                           _p(np.ascontiguousarray(n, dtype=np.float64)), _p(f))
    return f


class CovSWE:
    """Covariant shallow water on the cubed sphere; geometry (aux, xyz) and
    connectivity are the arrays passed to the C ABI.  fluxes: dict with keys
    volume (0 weak, 1 flux differencing), vol_sym (0 central, 1 ec), vol_nc
    (0/1 noncons ec), surf_sym, surf_diss (LLF), surf_nc (0, 1 ec,
    2 surface_simplified)."""

    def __init__(self, polydeg, aux, xyz, if_e, if_f, if_flip, g, omega, split, fluxes):
        self.n = polydeg + 1
        self.aux = np.ascontiguousarray(aux, dtype=np.float64)
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.nelem = self.aux.shape[0]
        ie = np.ascontiguousarray(if_e, dtype=np.int32)
        ifc = np.ascontiguousarray(if_f, dtype=np.int32)
        fl = np.ascontiguousarray(if_flip, dtype=np.int32)
        f = dict(volume=0, vol_sym=0, vol_nc=0, surf_sym=0, surf_diss=1, surf_nc=0)
        f.update(fluxes)
        self.h = lib().orc_cov_create(polydeg, self.nelem, _p(self.aux), _p(self.xyz),
                                      len(fl), _ip(ie), _ip(ifc), _ip(fl), g, omega, int(split),
                                      f["volume"], f["vol_sym"], f["vol_nc"], f["surf_sym"],
                                      f["surf_diss"], f["surf_nc"])

    def rhs(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.zeros_like(u)
        lib().orc_cov_rhs(self.h, _p(u), _p(du))
        return du

    def max_dt(self, u):
        return lib().orc_cov_max_dt(self.h, _p(np.ascontiguousarray(u)))

    def ck_steps(self, u, k, t, cfl, nsteps, fixed_dt=0.0, t_end=0.0):
        return lib().orc_cov_ck_steps(self.h, _p(u), _p(k), t, cfl, nsteps, fixed_dt, t_end)

    def ssp_steps(self, u, t, cfl, nsteps, scheme, fixed_dt=0.0, t_end=0.0):
        """SSPRK43 (scheme 1) or SSPRK33 (scheme 2) steps; returns the new time."""
        return lib().orc_cov_ssp_steps(self.h, _p(u), t, cfl, nsteps, scheme, fixed_dt, t_end)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_cov_destroy(self.h)
            self.h = None


class PotTemp2D:
    """Potential-temperature Euler with gravity on a StructuredMesh rectangle.
    volume 0 flux_tec, 1 flux_ec, 2 flux_etec; nc 0 waruszewski, 1 artiano,
    2 souza; wall_kind 1 StructuredMesh slip wall, 2 outward normal."""

    nv = 5

    def __init__(self, polydeg, nx, ny, x0, x1, y0, y1, periodic_x=True, periodic_y=False,
                 volume=0, nc=0, wall_kind=1, c_p=1004.0, c_v=717.0, g=9.80616, c_lmars=340.0,
                 surface=0, snc=-1, mesh=None):
        """surface 0 (FluxLMARS(c), surface term snc) or 1 (flux_ec, surface term
        snc); snc -1 flux_zero, else a gravity-term kind as nc.  mesh: (xy, Ja,
        invJ, if_e, if_f, if_flip, bd_e, bd_f, bd_kind) arrays of the host
        mirror instead of the rectangle."""
        self.n = polydeg + 1
        if mesh is not None:
            self._keep = [np.ascontiguousarray(a, dtype=np.float64) for a in mesh[:3]]
            self._keep += [np.ascontiguousarray(a, dtype=np.int32) for a in mesh[3:]]
            xy, Ja, invJ, ie, ifc, fl, be, bf, bk = self._keep
            self.nelem = invJ.shape[0]
            self.h = lib().orc_pt_create_mesh(polydeg, self.nelem, _p(xy), _p(Ja), _p(invJ),
                                              len(fl), _ip(ie), _ip(ifc), _ip(fl), len(be),
                                              _ip(be), _ip(bf), _ip(bk), volume, nc, surface,
                                              snc, c_p, c_v, g, c_lmars)
            return
        self.nelem = nx * ny
        self.h = lib().orc_pt_create(polydeg, nx, ny, x0, x1, y0, y1, int(periodic_x),
                                     int(periodic_y), volume, nc, wall_kind, c_p, c_v, g, c_lmars,
                                     surface, snc)

    def set_mountain(self, mw=None, bd_values=None):
        """MountainWaveSetup's damping source, mw = (theta_0, u0, N, z_damping_start,
        z_damping_end, x_damping_start, x_damping_end, damping_rate), and the
        states [B, n, 5] of the Dirichlet boundary faces (kind 4)."""
        self._mw = None if mw is None else np.ascontiguousarray(mw, dtype=np.float64)
        self._bv = None if bd_values is None else np.ascontiguousarray(bd_values, dtype=np.float64)
        lib().orc_pt_set_mountain(self.h, None if self._mw is None else _p(self._mw),
                                  None if self._bv is None else _p(self._bv))

    def initial_condition_gravity_waves(self):
        u = np.zeros((self.nelem, self.n, self.n, 5))
        lib().orc_pt_initial_condition_gravity_waves(self.h, _p(u))
        return u

    def errors_gravity_waves(self, u):
        l2, linf = np.zeros(5), np.zeros(5)
        lib().orc_pt_errors_gravity_waves(self.h, _p(np.ascontiguousarray(u)), _p(l2), _p(linf))
        return l2, linf

    def rhs(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.zeros_like(u)
        lib().orc_pt_rhs(self.h, _p(u), _p(du), t)
        return du

    def max_dt(self, u):
        return lib().orc_pt_max_dt(self.h, _p(np.ascontiguousarray(u)))

    def ssprk43_run(self, u, t0, t_end, cfl):
        return lib().orc_pt_ssprk43_run(self.h, _p(u), t0, t_end, cfl)

    def ck_steps(self, u, k, t, cfl, nsteps):
        return lib().orc_pt_ck_steps(self.h, _p(u), _p(k), t, cfl, nsteps)

    def ssp_steps(self, u, t, cfl, nsteps, scheme, fixed_dt=0.0, t_end=0.0):
        """SSPRK43 (scheme 1) or SSPRK33 (scheme 2) steps; returns the new time."""
        return lib().orc_pt_ssp_steps(self.h, _p(u), t, cfl, nsteps, scheme, fixed_dt, t_end)

    def ssprk43_adaptive(self, u, t, t_end, abstol=1e-6, reltol=1e-3, stops=(), variant=0):
        """Adaptive SSPRK43 with OrdinaryDiffEq's default error control
        (orc_time.hpp) from t to t_end, never stepping past a stop; returns
        (final time, dict of accepted / rejected steps, rhs calls, first and
        last dt)."""
        st = np.zeros(5)
        sp = np.ascontiguousarray(stops, dtype=np.float64)
        tf = lib().orc_pt_ssprk43_adaptive(self.h, _p(u), t, t_end, _p(sp) if sp.size else None,
                                           int(sp.size), abstol, reltol, variant, _p(st))
        return tf, dict(zip(("accepted", "rejected", "rhs_calls", "dt_first", "dt_last"), st))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_pt_destroy(self.h)
            self.h = None


def stolarsky(x, y, gamma):
    return lib().orc_pt_stolarsky(x, y, gamma)


def ln_mean(x, y):
    return lib().orc_ln_mean(x, y)


def inv_ln_mean(x, y):
    return lib().orc_inv_ln_mean(x, y)


class Moist2D:
    """Moist Euler on a StructuredMesh rectangle.  surface_kind 0: FluxLMARS(c),
    1: flux_lax_friedrichs, 2: flux_chandrashekar; source_kind 0: none,
    1: geopotential, 2: moist bubble (geopotential + phase change), 3 / 4: the
    dry / moist convergence tests, 5: moist bubble + Rayleigh sponge;
    wall_kind 1: StructuredMesh slip wall, 2: outward normal (P4estMesh);
    ic_kind 0: gemein bubble (dry, v1 = 20), 1 / 2: dry / moist convergence
    test, 3: nonhydrostatic gravity wave.  mesh: (xy, Ja, invJ, if_e, if_f,
    if_flip, bd_e, bd_f, bd_kind) arrays of the host mirror instead of the
    rectangle."""

    nv = 6

    def __init__(self, polydeg, nx, ny, x0, x1, y0, y1, periodic_x=True, periodic_y=False,
                 weak_form=False, surface_kind=0, source_kind=1, wall_kind=1, c_lmars=360.0,
                 gravity=9.80616, ic_kind=0, mesh=None):
        self.n = polydeg + 1
        if mesh is not None:
            self._keep = [np.ascontiguousarray(a, dtype=np.float64) for a in mesh[:3]]
            self._keep += [np.ascontiguousarray(a, dtype=np.int32) for a in mesh[3:]]
            xy, Ja, invJ, ie, ifc, fl, be, bf, bk = self._keep
            self.nelem = invJ.shape[0]
            self.h = lib().orc_moist_create_mesh(polydeg, self.nelem, _p(xy), _p(Ja), _p(invJ),
                                                 len(fl), _ip(ie), _ip(ifc), _ip(fl), len(be),
                                                 _ip(be), _ip(bf), _ip(bk), int(weak_form),
                                                 int(surface_kind), int(source_kind), c_lmars,
                                                 gravity, int(ic_kind))
            return
        self.nelem = nx * ny
        self.h = lib().orc_moist_create(polydeg, nx, ny, x0, x1, y0, y1, int(periodic_x),
                                        int(periodic_y), int(weak_form), int(surface_kind),
                                        int(source_kind), int(wall_kind), c_lmars, gravity,
                                        int(ic_kind))

    def initial_condition(self, t=0.0):
        u = np.zeros((self.nelem, self.n, self.n, 6))
        lib().orc_moist_initial_condition(self.h, t, _p(u))
        return u

    def errors(self, u, t):
        l2, linf = np.zeros(6), np.zeros(6)
        lib().orc_moist_errors(self.h, _p(np.ascontiguousarray(u)), t, _p(l2), _p(linf))
        return l2, linf

    def rhs(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.zeros_like(u)
        lib().orc_moist_rhs(self.h, _p(u), _p(du), t)
        return du

    def max_dt(self, u):
        return lib().orc_moist_max_dt(self.h, _p(np.ascontiguousarray(u)))

    def ck_steps(self, u, k, t, cfl, nsteps, fixed_dt=0.0, t_end=0.0):
        return lib().orc_moist_ck_steps(self.h, _p(u), _p(k), t, cfl, nsteps, fixed_dt, t_end)

    def ssp_steps(self, u, t, cfl, nsteps, scheme, fixed_dt=0.0, t_end=0.0):
        """SSPRK43 (scheme 1) or SSPRK33 (scheme 2) steps; returns the new time."""
        return lib().orc_moist_ssp_steps(self.h, _p(u), t, cfl, nsteps, scheme, fixed_dt, t_end)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_moist_destroy(self.h)
            self.h = None


def rainy_flux_lmars(ul, ur, n):
    f = np.zeros(9)
    lib().orc_rainy_flux_lmars(_p(np.ascontiguousarray(ul, dtype=np.float64)),
                               _p(np.ascontiguousarray(ur, dtype=np.float64)),
                               _p(np.ascontiguousarray(n, dtype=np.float64)), _p(f))
    return f


def rainy_slip_wall(u, n):
    f = np.zeros(9)
    lib().orc_rainy_slip_wall(_p(np.ascontiguousarray(u, dtype=np.float64)),
                              _p(np.ascontiguousarray(n, dtype=np.float64)), _p(f))
    return f


def moist_flux_chandrashekar(ul, ur, n):
    f = np.zeros(6)
    lib().orc_moist_flux_chandrashekar(_p(np.ascontiguousarray(ul, dtype=np.float64)),
                                       _p(np.ascontiguousarray(ur, dtype=np.float64)),
                                       _p(np.ascontiguousarray(n, dtype=np.float64)), _p(f))
    return f


def moist_flux(u, n):
    f = np.zeros(6)
    lib().orc_moist_flux(_p(np.ascontiguousarray(u, dtype=np.float64)),
                         _p(np.ascontiguousarray(n, dtype=np.float64)), _p(f))
    return f


class Rainy2D:
    """Rainy Euler (flux_ec_rain / flux_lax_friedrichs, source_terms_rainy,
    simple slip walls) on a StructuredMesh rectangle, with the Newton stage
    limiter.  source_kind 0 source_terms_rainy, 1 convergence test, 2 none,
    3 source_terms_no_phase_change.  mesh: (xy, Ja, invJ, if_e, if_f, if_flip,
    bd_e, bd_f, bd_kind) arrays of the host mirror instead of the rectangle,
    with surface 0 flux_lax_friedrichs / 1 flux_LMARS and wall 0 simple /
    1 pressure-Riemann slip walls."""

    nv = 9

    def __init__(self, polydeg, nx, ny, x0, x1, y0, y1, periodic_x=True, periodic_y=False,
                 weak_form=False, source_kind=0, mesh=None, surface=0, wall=0):
        self.n = polydeg + 1
        if mesh is not None:
            self._keep = [np.ascontiguousarray(a, dtype=np.float64) for a in mesh[:3]]
            self._keep += [np.ascontiguousarray(a, dtype=np.int32) for a in mesh[3:]]
            xy, Ja, invJ, ie, ifc, fl, be, bf, bk = self._keep
            self.nelem = invJ.shape[0]
            self.h = lib().orc_rainy_create_mesh(polydeg, self.nelem, _p(xy), _p(Ja), _p(invJ),
                                                 len(fl), _ip(ie), _ip(ifc), _ip(fl), len(be),
                                                 _ip(be), _ip(bf), _ip(bk), int(weak_form),
                                                 int(source_kind), int(surface), int(wall))
            return
        self.nelem = nx * ny
        self.h = lib().orc_rainy_create(polydeg, nx, ny, x0, x1, y0, y1, int(periodic_x),
                                        int(periodic_y), int(weak_form), int(source_kind))

    def geometry(self):
        xy = np.zeros((self.nelem, self.n, self.n, 2))
        lib().orc_rainy_geometry(self.h, _p(xy))
        return xy

    def initial_condition_convergence(self, t=0.0):
        u = np.zeros((self.nelem, self.n, self.n, 9))
        lib().orc_rainy_initial_condition_convergence(self.h, t, _p(u))
        return u

    def errors_convergence(self, u, t):
        l2, linf = np.zeros(9), np.zeros(9)
        lib().orc_rainy_errors_convergence(self.h, _p(np.ascontiguousarray(u)), t, _p(l2), _p(linf))
        return l2, linf

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_rainy_destroy(self.h)
            self.h = None

    def rhs(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.zeros_like(u)
        lib().orc_rainy_rhs(self.h, _p(u), _p(du), t)
        return du

    def max_dt(self, u):
        return lib().orc_rainy_max_dt(self.h, _p(np.ascontiguousarray(u)))

    def newton(self, u, mode=1, tol=1e-12, maxit=20, polish=0, guesses=None):
        """In-place Newton limiter; returns (total updates, per-node updates, nfail)."""
        iters = np.zeros(u.size // 9, dtype=np.int32)
        nf = ctypes.c_long()
        g = None if guesses is None else _p(np.ascontiguousarray(guesses, dtype=np.float64))
        tot = lib().orc_rainy_newton(self.h, _p(u), mode, tol, maxit, polish, g, _ip(iters),
                                     ctypes.byref(nf))
        return tot, iters, nf.value

    def ssprk43_adaptive(self, u, t, t_end, abstol=1e-6, reltol=1e-3, stops=(), variant=0,
                         mode=0, tol=1e-9, maxit=20):
        """Adaptive SSPRK43 with the Newton stage limiter after every stage
        (see PotTemp2D.ssprk43_adaptive)."""
        st = np.zeros(5)
        sp = np.ascontiguousarray(stops, dtype=np.float64)
        tf = lib().orc_rainy_ssprk43_adaptive(self.h, _p(u), t, t_end,
                                              _p(sp) if sp.size else None, int(sp.size), abstol,
                                              reltol, variant, mode, tol, maxit, _p(st))
        return tf, dict(zip(("accepted", "rejected", "rhs_calls", "dt_first", "dt_last"), st))

    def ck_steps(self, u, k, t, cfl, nsteps, fixed_dt=0.0, mode=0, tol=1e-9, maxit=20,
                 t_end=0.0):
        return lib().orc_rainy_ck_steps(self.h, _p(u), _p(k), t, cfl, nsteps, fixed_dt, mode, tol,
                                        maxit, t_end)

    def ssp_steps(self, u, t, cfl, nsteps, scheme, fixed_dt=0.0, mode=0, tol=1e-9, maxit=20,
                  t_end=0.0):
        """SSPRK43 (scheme 1) or SSPRK33 (scheme 2) steps with the Newton stage
        limiter after every stage; returns the new time."""
        return lib().orc_rainy_ssp_steps(self.h, _p(u), t, cfl, nsteps, scheme, fixed_dt, t_end,
                                         mode, tol, maxit)


def rainy_newton_states(u, mode=1, tol=1e-12, maxit=20, polish=0, guesses=None):
    """In-place Newton solve of node states u[..., 9]; returns (total updates,
    per-node updates, nfail)."""
    assert u.flags.c_contiguous and u.dtype == np.float64
    n = u.size // 9
    iters = np.zeros(n, dtype=np.int32)
    nf = ctypes.c_long()
    g = None if guesses is None else _p(np.ascontiguousarray(guesses, dtype=np.float64))
    tot = lib().orc_rainy_newton_states(_p(u), n, mode, tol, maxit, polish, g, _ip(iters),
                                        ctypes.byref(nf))
    return tot, iters, nf.value


def rainy_flux_ec(ul, ur, n):
    f = np.zeros(9)
    lib().orc_rainy_flux_ec(_p(np.ascontiguousarray(ul, dtype=np.float64)),
                            _p(np.ascontiguousarray(ur, dtype=np.float64)),
                            _p(np.ascontiguousarray(n, dtype=np.float64)), _p(f))
    return f


def rainy_flux(u, n):
    f = np.zeros(9)
    lib().orc_rainy_flux(_p(np.ascontiguousarray(u, dtype=np.float64)),
                         _p(np.ascontiguousarray(n, dtype=np.float64)), _p(f))
    return f


# ---- operation counts of the oracle's formulas (orc_flopcount.cpp) ----------
COUNT_NAMES = ("add", "mul", "div", "sqrt", "log", "exp", "pow")


def _flops_lib():
    global _flops
    if _flops is None:
        if not os.path.exists(_FLOPS_PATH):
            build()
        L = ctypes.CDLL(_FLOPS_PATH)
        _ll = ctypes.POINTER(ctypes.c_longlong)
        L.orc_count_euler3d_step.argtypes = (
            [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _ip_t, _ip_t, _ip_t,
             ctypes.c_int, _ip_t, _ip_t] + [ctypes.c_double] * 6 + [_dp, _ll])
        L.orc_count_euler2d_step.argtypes = (
            [ctypes.c_int] * 3 + [ctypes.c_double] * 9 + [_dp, _ll])
        L.orc_count_cov_step.argtypes = (
            [ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int, _ip_t, _ip_t, _ip_t,
             ctypes.c_double, ctypes.c_double] + [ctypes.c_int] * 7 + [ctypes.c_double, _dp, _ll])
        _flops = L
    return _flops


PHASES = ("volume", "interface", "boundary", "surface_jacobian_sources", "stage_update",
          "max_dt")


def _counts(call):
    """{phase: {operation: count}} over one CK2N54 step (max_dt: once)."""
    out = np.zeros((len(PHASES), 7), dtype=np.int64)
    call(out.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
    return {ph: dict(zip(COUNT_NAMES, (int(v) for v in out[i]))) for i, ph in enumerate(PHASES)}


def count_euler3d_step(polydeg, Ja, invJ, xyz, if_e, if_f, if_o, bd_e, bd_f, u0, c_p=1004.0,
                       c_v=717.0, g=9.80616, c_lmars=340.0, omega=7.292e-5, cfl=1.0):
    """Operation counts of one CK2N54 step of the 3D dry-Euler oracle on u0."""
    c = np.ascontiguousarray
    ie, ifc, io = (c(a, dtype=np.int32) for a in (if_e, if_f, if_o))
    be, bf = c(bd_e, dtype=np.int32), c(bd_f, dtype=np.int32)
    Ja, invJ, xyz, u0 = (c(a, dtype=np.float64) for a in (Ja, invJ, xyz, u0))
    return _counts(lambda o: _flops_lib().orc_count_euler3d_step(
        polydeg, invJ.size // (polydeg + 1) ** 3, _p(Ja), _p(invJ), _p(xyz), io.size, _ip(ie),
        _ip(ifc), _ip(io), be.size, _ip(be), _ip(bf), c_p, c_v, g, c_lmars, omega, cfl, _p(u0), o))


def count_euler2d_step(polydeg, nx, ny, x0, x1, y0, y1, u0, c_p=1004.0, c_v=717.0, g=9.81,
                       c_lmars=340.0, cfl=1.0):
    """Operation counts of one CK2N54 step of one 2D dry-Euler member."""
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    return _counts(lambda o: _flops_lib().orc_count_euler2d_step(
        polydeg, nx, ny, x0, x1, y0, y1, c_p, c_v, g, c_lmars, cfl, _p(u0), o))


def count_cov_step(polydeg, aux, xyz, if_e, if_f, if_flip, g, omega, split, fluxes, u0, cfl=0.4):
    """Operation counts of one CK2N54 step of one covariant shallow-water mesh."""
    c = np.ascontiguousarray
    ie, ifc, fl = (c(a, dtype=np.int32) for a in (if_e, if_f, if_flip))
    aux, xyz, u0 = (c(a, dtype=np.float64) for a in (aux, xyz, u0))
    f = _cov_flux_ids(fluxes)
    return _counts(lambda o: _flops_lib().orc_count_cov_step(
        polydeg, aux.size // (26 * (polydeg + 1) ** 2), _p(aux), _p(xyz), fl.size, _ip(ie),
        _ip(ifc), _ip(fl), g, omega, int(split), f["volume"], f["vol_sym"], f["vol_nc"],
        f["surf_sym"], f["surf_diss"], f["surf_nc"], cfl, _p(u0), o))


def _cov_flux_ids(fluxes):
    f = dict(volume=0, vol_sym=0, vol_nc=0, surf_sym=0, surf_diss=1, surf_nc=0)
    f.update(fluxes)
    return f
