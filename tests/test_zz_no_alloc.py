"""tag_rhs_noalloc: the right-hand side for callers that cannot allocate GPU memory.

Some programs own all of their device memory through an arena or pool (or a
Julia GPU allocator) and cannot let a library call cudaMalloc.  For them the
library offers tag_rhs_noalloc: the caller hands in device buffers for the
state, the tendency, the geometry and the connectivity, and the only scratch
the kernels need (the surface fluxes between the interface and element
kernels) comes from a fixed-size device array inside the library.

This test allocates the caller's buffers with torch (standing in for such a
caller), calls the entry point through the C ABI twice in a row on two
different states, and checks each result against the regular entry point
tag_rhs within the parity tolerance used by the other GPU tests.  It lives in
its own file, named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # same whole-vector max-norm tolerance as tests/test_gpu_euler2d.py


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


@pytest.mark.parametrize("polydeg,cells", [(3, (16, 8)), (5, (6, 4))])
def test_rhs_noalloc_matches_tag_rhs_on_two_calls(tg, gpu_lib, polydeg, cells):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = gpu_lib
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    solver = tg.DGSEM(polydeg, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    mesh = tg.StructuredMesh(cells, (0.0, 0.0), (20000.0, 10000.0), periodicity=(True, False))
    bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall}
    semi = tg.SemidiscretizationHyperbolic(mesh, eq, tg.WarmBubble(), solver,
                                           boundary_conditions=bcs)
    u_a = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=501)
    u_b = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=502, amplitude=3e-2)
    ref_a, ref_b = semi.rhs(u_a), semi.rhs(u_b)

    # the caller's own device buffers
    conn = mesh.connectivity()
    ie, ifc, fl, be, bf = conn.arrays()
    bk = np.full(be.shape, tg._lib.TAG_BC_SLIP_WALL_STRUCTURED, dtype=np.int32)
    d = {
        "Ja": _dev(torch, semi.contravariant_vectors, np.float64),
        "invJ": _dev(torch, semi.inverse_jacobian, np.float64),
        "ie": _dev(torch, ie, np.int32), "ifc": _dev(torch, ifc, np.int32),
        "fl": _dev(torch, fl, np.int32), "be": _dev(torch, be, np.int32),
        "bf": _dev(torch, bf, np.int32), "bk": _dev(torch, bk, np.int32),
    }
    Ds = np.asfortranarray(solver.basis.derivative_split)
    w = np.ascontiguousarray(solver.basis.weights)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int32)
    cfg = tg._lib.TagConfig()
    cfg.equations = tg._lib.TAG_EQ_EULER_ENERGY_2D
    cfg.volume_flux = tg._lib.TAG_VF_RANOCHA_WARUSZEWSKI
    cfg.surface_flux = tg._lib.TAG_SF_LMARS
    cfg.polydeg = polydeg
    cfg.nelements = mesh.nelements
    cfg.ninterfaces = ie.shape[0]
    cfg.nboundaries = be.shape[0]
    cfg.nmembers = 1
    cfg.derivative_split = Ds.ctypes.data_as(dp)
    cfg.weights = w.ctypes.data_as(dp)
    cfg.contravariant_vectors = ctypes.cast(d["Ja"].data_ptr(), dp)
    cfg.inverse_jacobian = ctypes.cast(d["invJ"].data_ptr(), dp)
    cfg.interface_elements = ctypes.cast(d["ie"].data_ptr(), ip)
    cfg.interface_faces = ctypes.cast(d["ifc"].data_ptr(), ip)
    cfg.interface_flip = ctypes.cast(d["fl"].data_ptr(), ip)
    cfg.boundary_elements = ctypes.cast(d["be"].data_ptr(), ip)
    cfg.boundary_faces = ctypes.cast(d["bf"].data_ptr(), ip)
    cfg.boundary_kinds = ctypes.cast(d["bk"].data_ptr(), ip)
    for k, p in enumerate([eq.c_p, eq.c_v, eq.g, 340.0]):
        cfg.params[k] = p

    stream = torch.cuda.current_stream().cuda_stream
    for u, ref in ((u_a, ref_a), (u_b, ref_b)):
        du_dev = torch.full(u.shape, float("nan"), dtype=torch.float64, device="cuda")
        u_dev = _dev(torch, u, np.float64)
        status = ctypes.c_uint32(0xFFFF)
        rc = L.tag_rhs_noalloc(ctypes.byref(cfg), ctypes.cast(u_dev.data_ptr(), dp),
                               ctypes.cast(du_dev.data_ptr(), dp), ctypes.c_void_p(stream),
                               ctypes.byref(status))
        assert rc == tg._lib.TAG_OK, L.tag_last_error()
        assert status.value == 0
        du = du_dev.cpu().numpy()
        err = np.abs(du - ref).max() / np.abs(ref).max()
        assert err <= RTOL, err
    semi.close()


def test_rhs_noalloc_rejects_meshes_beyond_the_scratch_limit(tg, gpu_lib):
    L = gpu_lib
    cfg = tg._lib.TagConfig()
    cfg.equations = tg._lib.TAG_EQ_EULER_ENERGY_2D
    cfg.volume_flux = tg._lib.TAG_VF_RANOCHA_WARUSZEWSKI
    cfg.surface_flux = tg._lib.TAG_SF_LMARS
    cfg.polydeg = 3
    cfg.nelements = 70000  # 70000 * 4 * 4 * 4 doubles > the 1 Mi-double scratch
    dummy = np.zeros(16)
    dp = ctypes.POINTER(ctypes.c_double)
    cfg.derivative_split = dummy.ctypes.data_as(dp)
    cfg.weights = dummy.ctypes.data_as(dp)
    cfg.contravariant_vectors = dummy.ctypes.data_as(dp)
    cfg.inverse_jacobian = dummy.ctypes.data_as(dp)
    rc = L.tag_rhs_noalloc(ctypes.byref(cfg), dummy.ctypes.data_as(dp), dummy.ctypes.data_as(dp),
                           None, None)
    assert rc == tg._lib.TAG_E_INVALID
    assert b"too large" in L.tag_last_error()
