"""tag_rhs_noalloc: the right-hand side for callers that cannot allocate GPU memory.

Some programs own all of their device memory through an arena or pool (or a
Julia GPU allocator) and cannot let a library call cudaMalloc.  For them the
library offers tag_rhs_noalloc: the caller hands in device buffers for the
state, the tendency, the geometry and the connectivity, and the only scratch
the kernels need (the surface fluxes between the interface and element
kernels) comes from a fixed-size device array inside the library.

This test allocates the caller's buffers with torch (standing in for such a
caller), calls the entry point through the C ABI twice in a row on two
different states, and checks each result against the CPU oracle and against
the regular entry point tag_rhs within the parity tolerance used by the other
GPU tests; the device's free memory must not change across the second call.
It also checks the host-side rejections (meshes beyond the scratch limit,
boundary kinds that need data only a handle owns), which return before any
kernel runs.  It lives in its own file, named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # same whole-vector max-norm tolerance as tests/test_gpu_euler2d.py
DP = ctypes.POINTER(ctypes.c_double)
IP = ctypes.POINTER(ctypes.c_int32)


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


def _caller_buffers(tg, torch, polydeg, cells, kind=None):
    """The semidiscretization (for tag_rhs), the oracle case, the config of the
    caller's own device buffers, and those buffers (kept alive by the caller)."""
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    solver = tg.DGSEM(polydeg, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    mesh = tg.StructuredMesh(cells, (0.0, 0.0), (20000.0, 10000.0), periodicity=(True, False))
    bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall}
    semi = tg.SemidiscretizationHyperbolic(mesh, eq, tg.WarmBubble(), solver,
                                           boundary_conditions=bcs)
    conn = mesh.connectivity()
    ie, ifc, fl, be, bf = conn.arrays()
    bk = np.full(be.shape, tg._lib.TAG_BC_SLIP_WALL_STRUCTURED if kind is None else kind,
                 dtype=np.int32)
    d = {
        "Ja": _dev(torch, semi.contravariant_vectors, np.float64),
        "invJ": _dev(torch, semi.inverse_jacobian, np.float64),
        "ie": _dev(torch, ie, np.int32), "ifc": _dev(torch, ifc, np.int32),
        "fl": _dev(torch, fl, np.int32), "be": _dev(torch, be, np.int32),
        "bf": _dev(torch, bf, np.int32), "bk": _dev(torch, bk, np.int32),
        "Ds": np.asfortranarray(solver.basis.derivative_split),
        "w": np.ascontiguousarray(solver.basis.weights),
    }
    cfg = tg._lib.TagConfig()
    cfg.equations = tg._lib.TAG_EQ_EULER_ENERGY_2D
    cfg.volume_flux = tg._lib.TAG_VF_RANOCHA_WARUSZEWSKI
    cfg.surface_flux = tg._lib.TAG_SF_LMARS
    cfg.polydeg = polydeg
    cfg.nelements = mesh.nelements
    cfg.ninterfaces = ie.shape[0]
    cfg.nboundaries = be.shape[0]
    cfg.nmembers = 1
    cfg.derivative_split = d["Ds"].ctypes.data_as(DP)
    cfg.weights = d["w"].ctypes.data_as(DP)
    cfg.contravariant_vectors = ctypes.cast(d["Ja"].data_ptr(), DP)
    cfg.inverse_jacobian = ctypes.cast(d["invJ"].data_ptr(), DP)
    cfg.interface_elements = ctypes.cast(d["ie"].data_ptr(), IP)
    cfg.interface_faces = ctypes.cast(d["ifc"].data_ptr(), IP)
    cfg.interface_flip = ctypes.cast(d["fl"].data_ptr(), IP)
    cfg.boundary_elements = ctypes.cast(d["be"].data_ptr(), IP)
    cfg.boundary_faces = ctypes.cast(d["bf"].data_ptr(), IP)
    cfg.boundary_kinds = ctypes.cast(d["bk"].data_ptr(), IP)
    for k, p in enumerate([eq.c_p, eq.c_v, eq.g, 340.0]):
        cfg.params[k] = p
    return eq, semi, cfg, d


@pytest.mark.parametrize("polydeg,cells", [(3, (16, 8)), (5, (6, 4)), (7, (6, 4))])
def test_rhs_noalloc_matches_oracle_and_tag_rhs_on_two_calls(tg, orc, gpu_lib, polydeg, cells):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = gpu_lib
    eq, semi, cfg, keep = _caller_buffers(tg, torch, polydeg, cells)
    oracle = orc.Euler2D(polydeg, cells[0], cells[1], 0.0, 20000.0, 0.0, 10000.0, True, False,
                         1004.0, 717.0, 9.81, 340.0)
    u_a = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=501)
    u_b = tg.seeded_perturbation(semi.compute_coefficients(), eq, seed=502, amplitude=3e-2)
    calls = []
    for u in (u_a, u_b):
        calls.append((u, oracle.rhs(u), semi.rhs(u), _dev(torch, u, np.float64),
                      torch.full(u.shape, float("nan"), dtype=torch.float64, device="cuda")))
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    for k, (u, ref, ref_lib, u_dev, du_dev) in enumerate(calls):
        status = ctypes.c_uint32(0xFFFF)
        free_before = torch.cuda.mem_get_info()[0]
        rc = L.tag_rhs_noalloc(ctypes.byref(cfg), ctypes.cast(u_dev.data_ptr(), DP),
                               ctypes.cast(du_dev.data_ptr(), DP), ctypes.c_void_p(stream),
                               ctypes.byref(status))
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == tg._lib.TAG_OK, L.tag_last_error()
        assert status.value == 0
        if k == 1:  # the first call may load the library's module; the second allocates nothing
            assert free_after == free_before, (free_before, free_after)
        du = du_dev.cpu().numpy()
        err = np.abs(du - ref).max() / np.abs(ref).max()
        assert err <= RTOL, ("oracle", err)
        err_lib = np.abs(du - ref_lib).max() / np.abs(ref_lib).max()
        assert err_lib <= RTOL, ("tag_rhs", err_lib)
    semi.close()


def test_rhs_noalloc_rejects_dirichlet_faces(tg, gpu_lib):
    """A Dirichlet face needs boundary states that only a tag_create handle
    owns: the call reads the kinds on the host and returns TAG_E_INVALID before
    any kernel runs."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = gpu_lib
    eq, semi, cfg, keep = _caller_buffers(tg, torch, 3, (8, 4), kind=tg._lib.TAG_BC_DIRICHLET)
    u = semi.compute_coefficients()
    u_dev = _dev(torch, u, np.float64)
    du_dev = torch.zeros(u.shape, dtype=torch.float64, device="cuda")
    rc = L.tag_rhs_noalloc(ctypes.byref(cfg), ctypes.cast(u_dev.data_ptr(), DP),
                           ctypes.cast(du_dev.data_ptr(), DP), None, None)
    assert rc == tg._lib.TAG_E_INVALID
    assert b"slip walls only" in L.tag_last_error()
    assert float(du_dev.abs().max()) == 0.0  # nothing ran
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
    cfg.derivative_split = dummy.ctypes.data_as(DP)
    cfg.weights = dummy.ctypes.data_as(DP)
    cfg.contravariant_vectors = dummy.ctypes.data_as(DP)
    cfg.inverse_jacobian = dummy.ctypes.data_as(DP)
    rc = L.tag_rhs_noalloc(ctypes.byref(cfg), dummy.ctypes.data_as(DP), dummy.ctypes.data_as(DP),
                           None, None)
    assert rc == tg._lib.TAG_E_INVALID
    assert b"too large" in L.tag_last_error()
