"""Solution output on the GPU: the device conversions of tag_solution_variables
against the oracle's restatement (oracle/solution_variables.py), ensemble
members, cons2cons of a Cartesian system, and save_solution_file written by
the library's HDF5 encoder and read back by the strict checker
(tests/h5_reader.py) — the file of the reference's SaveSolutionCallback
(src/callbacks_step/save_solution_2d_manifold_in_3d_cartesian.jl:44-118,
src/callbacks_step/save_solution_covariant.jl:5-125)."""
import numpy as np
import pytest

from h5_reader import H5File
from test_gpu_cov_swe import G_, OM_, make_semi, perturbed

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def out(tg):
    import importlib
    return importlib.import_module("trixiatmo_gb300.output")


@pytest.fixture(scope="module")
def sv(orc):
    import solution_variables
    return solution_variables


def rel(a, b, scale=None):
    return np.abs(a - b).max() / max(np.abs(b).max() if scale is None else scale, 1e-300)


def check_rows(rows, ref, kind):
    """Rounding-level agreement.  Components of a vector (the global
    velocity or momentum, sums a_c m1 + a_(3+c) m2 that cancel in a small
    component) are scaled by the vector's largest component; the vorticity
    differentiates along grid lines (sums of n terms) and gets 1e-12."""
    vec = {2: range(1, 4), 3: range(1, 4)}.get(kind, ())
    vscale = np.abs(ref[list(vec)]).max() if vec else None
    for v in range(ref.shape[0]):
        tol = 1e-12 if (kind, v) == (3, 5) else 1e-14
        assert rel(rows[v], ref[v], vscale if v in vec else None) <= tol, (kind, v)


@pytest.mark.parametrize("polydeg", [3, 4, 7])
@pytest.mark.parametrize("name", ["isolated_mountain", "unsteady_solid_body_rotation"])
def test_covariant_solution_variables_match_oracle(tg, gpu_lib, out, sv, name, polydeg):
    eq, mesh, semi, _, _ = make_semi(tg, name, k=3, polydeg=polydeg)
    u = perturbed(semi.compute_coefficients(), seed=polydeg)
    semi.set_state(u)
    for fn, kind, nv in ((out.cons2cons, 0, 3), (out.cons2prim, 1, 3),
                         (out.contravariant2global, 2, 4), (out.cons2prim_and_vorticity, 3, 6)):
        rows = out.convert_variables(semi, fn)
        ref = sv.covariant_rows(u, semi.aux_node_vars, semi.solver.basis.nodes, kind)
        assert rows.shape == ref.shape == (nv, semi.ndofs)
        if kind == 0:
            assert np.array_equal(rows, ref)
        check_rows(rows, ref, kind)
        assert len(out.varnames(fn, eq)) == nv
    semi.close()


def test_covariant_ensemble_members(tg, gpu_lib, out, sv):
    """Members of different degrees: each member's rows are its slice of the
    whole handle's rows and match the oracle on that member's arrays."""
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import EARTH_RADIUS
    eq = cv.SplitCovariantShallowWaterEquations2D(G_, OM_)
    specs = [(3, 3), (2, 5), (3, 4)]
    meshes = [cv.P4estMeshCubedSphere2D(k, EARTH_RADIUS, polydeg=N) for k, N in specs]
    solvers = [tg.DGSEM(N, cv.flux_ec, tg.VolumeIntegralFluxDifferencing(cv.flux_ec))
               for _, N in specs]
    ics = [cv.transform_initial_condition(cv.initial_condition_geostrophic_balance, eq)] * 3
    ens = tg.SemidiscretizationCovariantEnsemble(meshes, eq, ics, solvers,
                                                 source_terms=cv.source_terms_geometric_coriolis)
    u = ens.compute_coefficients()
    u = u * (1 + 1e-3 * np.random.default_rng(1).standard_normal(u.shape))
    ens.set_state(u)
    whole = out.convert_variables(ens, out.cons2prim_and_vorticity)
    off = ens.member_node_offsets
    for m, (_, N) in enumerate(specs):
        rows = out.convert_variables(ens, out.cons2prim_and_vorticity, member=m)
        assert np.array_equal(rows, whole[:, off[m]:off[m + 1]])
        ref = sv.covariant_rows(ens.member_state(u, m), ens._H.aux[m],
                                tg.LobattoLegendreBasis(N).nodes, 3)
        check_rows(rows, ref, 3)
    with pytest.raises(tg._lib.TagError):
        out.convert_variables(ens, out.cons2cons, member=3)
    ens.close()


def test_cartesian_cons2cons(tg, gpu_lib, out):
    from test_gpu_euler2d import make_semi as make_euler
    eq, semi = make_euler(tg, 6, 4)
    u = semi.compute_coefficients()
    semi.set_state(u)
    rows = out.convert_variables(semi, out.cons2cons)
    assert np.array_equal(rows, u.reshape(-1, 5).T)
    assert out.varnames(out.cons2cons, eq) == ("rho", "rho_v1", "rho_v2", "rho_e", "phi")
    with pytest.raises(tg._lib.TagError, match="cons2cons only"):
        out.convert_variables(semi, out.cons2prim_and_vorticity)
    semi.close()


def test_save_solution_file_round_trip(tg, gpu_lib, out, tmp_path):
    eq, mesh, semi, _, cfl = make_semi(tg, "isolated_mountain", k=3, polydeg=4)
    semi.set_state(semi.compute_coefficients())
    t = semi.rk_steps(3, cfl=cfl, t=0.0)
    dt = semi.max_dt() * cfl
    fname = out.save_solution_file(semi, t, dt, 3, str(tmp_path), out.cons2prim_and_vorticity,
                                   mesh_file="mesh.h5")
    assert fname == str(tmp_path / "solution_000000003.h5")
    f = H5File(fname)
    assert f.attrs == {"ndims": 2, "equations": type(eq).__name__, "polydeg": 4, "n_vars": 6,
                       "n_elements": mesh.nelements, "mesh_type": "P4estMesh",
                       "mesh_file": "mesh.h5", "time": t, "dt": dt, "timestep": 3}
    rows = out.convert_variables(semi, out.cons2prim_and_vorticity)
    for v, name in enumerate(("H", "v1", "v2", "v3", "b", "vorticity")):
        d = f.datasets[f"variables_{v + 1}"]
        assert d.attrs == {"name": name}
        assert d.data.tobytes() == rows[v].tobytes()
    # the state is untouched by the output
    u1 = semi.get_state()
    out.save_solution_file(semi, t, dt, 3, str(tmp_path), system="fluid")
    assert np.array_equal(semi.get_state(), u1)
    g = H5File(tmp_path / "solution_fluid_000000003.h5")
    assert [g.datasets[f"variables_{v + 1}"].attrs["name"] for v in range(3)] == [
        "h", "h_vcon1", "h_vcon2"]
    assert g.datasets["variables_1"].data.tobytes() == u1.reshape(-1, 3)[:, 0].copy().tobytes()
    semi.close()


def test_ensemble_files_one_per_member(tg, gpu_lib, out, tmp_path):
    """A Cartesian ensemble written whole: one file per member (its own
    system), each with the member's element count and its slice of the state."""
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    solver = tg.DGSEM(3, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    meshes = [tg.StructuredMesh((nx, 2), (0.0, 0.0), (20000.0, 10000.0), periodicity=(True, False))
              for nx in (4, 6)]
    bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall}
    ens = tg.SemidiscretizationEnsemble(meshes, eq, [tg.WarmBubble()] * 2, solver,
                                        boundary_conditions=bcs)
    u = ens.compute_coefficients()
    ens.set_state(u)
    names = out.save_solution_file(ens, 0.0, 0.0, 0, str(tmp_path), system="bubble")
    assert names == [str(tmp_path / f"solution_bubble_member{m}_000000000.h5") for m in range(2)]
    for m, name in enumerate(names):
        f = H5File(name)
        assert f.attrs["n_elements"] == (8, 12)[m] and f.attrs["polydeg"] == 3
        assert f.attrs["mesh_type"] == "StructuredMesh" and f.attrs["n_vars"] == 5
        um = u.reshape(-1, 5)[ens.member_slice(m).start * 16:ens.member_slice(m).stop * 16]
        for v in range(5):
            assert np.array_equal(f.datasets[f"variables_{v + 1}"].data, um[:, v])
    ens.close()


def test_save_solution_file_3d_shell(tg, gpu_lib, out, tmp_path):
    """The 3D shell (a P4estMesh{3} in the reference): ndims 3, the
    conservative variables with their names, bit for bit the state."""
    from test_gpu_euler3d import make_semi as make_shell
    eq, mesh, semi = make_shell(tg, 2, 2, 4)
    u = semi.compute_coefficients()
    semi.set_state(u)
    fname = out.save_solution_file(semi, 0.5, 0.25, 7, str(tmp_path))
    f = H5File(fname)
    assert f.attrs["ndims"] == 3 and f.attrs["mesh_type"] == "P4estMesh"
    assert f.attrs["polydeg"] == 4 and f.attrs["n_elements"] == semi.nelements
    assert f.attrs["n_vars"] == 6 and f.attrs["timestep"] == 7 and f.attrs["time"] == 0.5
    names = ("rho", "rho_v1", "rho_v2", "rho_v3", "rho_e", "phi")
    for v, name in enumerate(names):
        d = f.datasets[f"variables_{v + 1}"]
        assert d.attrs == {"name": name}
        assert d.data.tobytes() == np.ascontiguousarray(u.reshape(-1, 6)[:, v]).tobytes()
    semi.close()
