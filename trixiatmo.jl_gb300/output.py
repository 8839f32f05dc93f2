"""Solution files as the reference's SaveSolutionCallback writes them.

`save_solution_file(semi, time, dt, timestep, output_directory, ...)` mirrors
Trixi.save_solution_file as TrixiAtmo.jl extends it
(src/callbacks_step/save_solution_2d_manifold_in_3d_cartesian.jl:44-118): the
solution variables are computed on the device (`tag_solution_variables`,
replacing convert_variables of src/callbacks_step/save_solution_covariant.jl:5-33),
copied to the host once, and written by the library's own HDF5 encoder
(`tag_h5_write`) as `solution_%09d.h5` with the root attributes ndims,
equations, polydeg, n_vars, n_elements, mesh_type, mesh_file, time, dt,
timestep and one dataset `variables_v` per variable carrying its name: the
file Trixi2Vtk reads.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib


class _SolutionVariables:
    """One of Trixi's `solution_variables` functions, by name."""

    def __init__(self, name, code):
        self.__name__ = name
        self.code = code

    def __repr__(self):
        return self.__name__


cons2cons = _SolutionVariables("cons2cons", _lib.TAG_SOLVAR_CONS2CONS)
cons2prim = _SolutionVariables("cons2prim", _lib.TAG_SOLVAR_CONS2PRIM)
contravariant2global = _SolutionVariables("contravariant2global",
                                          _lib.TAG_SOLVAR_CONTRAVARIANT2GLOBAL)
cons2prim_and_vorticity = _SolutionVariables("cons2prim_and_vorticity",
                                             _lib.TAG_SOLVAR_CONS2PRIM_AND_VORTICITY)

# conservative variable names of each equation system (the reference's
# varnames(::typeof(cons2cons), equations))
_CONS2CONS = {
    # src/equations/compressible_euler_energy_with_gravity_2d.jl:62-65
    "CompressibleEulerEnergyEquationsWithGravity2D": ("rho", "rho_v1", "rho_v2", "rho_e", "phi"),
    # src/equations/compressible_euler_energy_with_gravity_3d.jl:67-69
    "CompressibleEulerEnergyEquationsWithGravity3D": ("rho", "rho_v1", "rho_v2", "rho_v3",
                                                      "rho_e", "phi"),
    # src/equations/compressible_euler_internal_energy_with_gravity_2d.jl:64-67
    "CompressibleEulerInternalEnergyEquationsWithGravity2D": ("rho", "rho_v1", "rho_v2",
                                                              "rho_e_internal", "phi"),
    # src/equations/compressible_euler_potential_temperature_gravity_2d.jl:30-33
    "CompressibleEulerPotentialTemperatureEquationsWithGravity2D": ("rho", "rho_v1", "rho_v2",
                                                                    "rho_theta", "phi"),
    # src/equations/compressible_euler_potential_temperature_gravity_3d.jl:69-72
    "CompressibleEulerPotentialTemperatureEquationsWithGravity3D": ("rho", "rho_v1", "rho_v2",
                                                                    "rho_v3", "rho_theta", "phi"),
    # src/equations/compressible_moist_euler_2d.jl:1208-1211
    "CompressibleMoistEulerEquations2D": ("rho", "rho_v1", "rho_v2", "rho_E", "rho_qv",
                                          "rho_ql"),
    # src/equations/compressible_rainy_euler_2d.jl:281-289
    "CompressibleRainyEulerEquations2D": ("rho_dry", "rho_moist", "rho_rain", "rho_v1", "rho_v2",
                                          "energy_density", "rho_vapour", "rho_cloud",
                                          "temperature"),
}

# covariant shallow water: src/equations/covariant_shallow_water.jl:83-100 and
# src/callbacks_step/save_solution_covariant.jl:122-125
_COVARIANT = {
    "cons2cons": ("h", "h_vcon1", "h_vcon2"),
    "cons2prim": ("H", "vcon1", "vcon2"),
    "contravariant2global": ("h", "h_v1", "h_v2", "h_v3"),
    "cons2prim_and_vorticity": ("H", "v1", "v2", "v3", "b", "vorticity"),
}


def _is_covariant(equations):
    from .covariant import CovariantShallowWaterEquations2D
    return isinstance(equations, CovariantShallowWaterEquations2D)


def get_name(obj):
    """Trixi.get_name: the type's name without parameters (the equations'
    class; P4estMesh for the cubed-sphere meshes, which are P4estMesh values
    in the reference)."""
    name = type(obj).__name__
    return "P4estMesh" if name.startswith("P4estMesh") else name


def varnames(solution_variables, equations):
    """Trixi.varnames(solution_variables, equations)."""
    name = solution_variables.__name__
    if _is_covariant(equations):
        if name not in _COVARIANT:
            raise ValueError(f"no {name} for covariant equations")
        return _COVARIANT[name]
    if name != "cons2cons":
        raise ValueError(f"{get_name(equations)} writes cons2cons only")
    return _CONS2CONS[get_name(equations)]


def convert_variables(semi, solution_variables=cons2cons, member=None):
    """The solution variables of the handle's current state, computed on the
    device (convert_variables, src/callbacks_step/save_solution_covariant.jl:5-33):
    an array [n_vars, n_nodes] whose row v is Trixi's `vec(data[v, .., :])`
    (nodes in Julia order i, j, (k,) element); member selects one member of an
    ensemble."""
    L = _lib.load()
    m = -1 if member is None else int(member)
    nv, nq = ctypes.c_int32(), ctypes.c_int64()
    code = solution_variables.code
    _lib.check(L.tag_solution_variables(semi.handle, code, m, ctypes.byref(nv), ctypes.byref(nq),
                                        None))
    out = np.empty((nv.value, nq.value), dtype=np.float64)
    _lib.check(L.tag_solution_variables(semi.handle, code, m, ctypes.byref(nv), ctypes.byref(nq),
                                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return out


def _set_attribute(a, name, value, keep):
    """Fills a tag_h5_attribute in place; `keep` holds the encoded strings for
    the duration of the call."""
    keep.append(name.encode())
    a.name = keep[-1]
    if isinstance(value, (bool, np.bool_)):
        raise TypeError(f"attribute {name}: booleans are not written")
    if isinstance(value, (int, np.integer)):
        a.type, a.i = _lib.TAG_H5_INT64, int(value)
    elif isinstance(value, (float, np.floating)):
        a.type, a.d = _lib.TAG_H5_FLOAT64, float(value)
    elif isinstance(value, str):
        keep.append(value.encode("utf-8"))
        a.type, a.s = _lib.TAG_H5_STRING, keep[-1]
    else:
        raise TypeError(f"attribute {name}: int, float or str expected, got {type(value)}")


def write_h5(filename, attributes, datasets):
    """Writes an HDF5 file with scalar root attributes (name -> int, float or
    str) and one-dimensional float64 datasets ((name, array, var_name or None)
    triples) through the library's encoder."""
    keep = []
    attrs = list(attributes.items())
    A = (_lib.H5Attribute * max(1, len(attrs)))()
    for k, (name, value) in enumerate(attrs):
        _set_attribute(A[k], name, value, keep)
    D = (_lib.H5Dataset * max(1, len(datasets)))()
    for k, (name, arr, var_name) in enumerate(datasets):
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).ravel())
        keep += [a, name.encode()]
        D[k].name = keep[-1]
        D[k].data = a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        D[k].count = a.size
        if var_name is not None:
            keep.append(var_name.encode("utf-8"))
            D[k].var_name = keep[-1]
    _lib.check(_lib.load().tag_h5_write(os.fsencode(filename), A, len(attrs), D, len(datasets)))
    return filename


def write_solution_file(filename, data, names, *, ndims, equations, polydeg, n_elements,
                        mesh_type, mesh_file="", time=0.0, dt=0.0, timestep=0,
                        element_variables=None, node_variables=None):
    """Trixi's solution-file layout from rows data[v] and their names:
    save_solution_2d_manifold_in_3d_cartesian.jl:72-115.  element_variables /
    node_variables: dicts name -> array, written as element_variables_k /
    node_variables_k with their names."""
    data = np.asarray(data, dtype=np.float64)
    if data.ndim != 2 or data.shape[0] != len(names):
        raise ValueError("data must be [n_vars, n_nodes] with one name per row")
    attributes = {
        "ndims": int(ndims), "equations": str(equations), "polydeg": int(polydeg),
        "n_vars": int(data.shape[0]), "n_elements": int(n_elements),
        "mesh_type": str(mesh_type), "mesh_file": str(mesh_file),
        "time": float(time), "dt": float(dt), "timestep": int(timestep),
    }
    sets = [(f"variables_{v + 1}", data[v], names[v]) for v in range(data.shape[0])]
    for prefix, extra in (("element_variables", element_variables),
                          ("node_variables", node_variables)):
        for k, (key, arr) in enumerate((extra or {}).items()):
            sets.append((f"{prefix}_{k + 1}", arr, str(key)))
    return write_h5(filename, attributes, sets)


def _member_meta(semi, m):
    """(ndims, polydeg, n_elements, mesh) of member m (None: the whole semi)."""
    if hasattr(semi, "solvers"):          # covariant ensemble
        k = 0 if m is None else m
        return 2, semi.solvers[k].polydeg, semi.meshes[k].nelements, semi.meshes[k]
    if hasattr(semi, "meshes"):           # Cartesian ensemble
        k = 0 if m is None else m
        return semi.ndims, semi.solver.polydeg, int(semi.member_nelements[k]), semi.meshes[k]
    return semi.ndims, semi.solver.polydeg, semi.nelements, semi.mesh


def save_solution_file(semi, time, dt, timestep, output_directory,
                       solution_variables=cons2cons, system="", member=None, mesh_file="",
                       element_variables=None, node_variables=None):
    """Trixi.save_solution_file for the handle's current state; returns the
    file name (a list of names, one per member, for an ensemble written
    whole: each member is its own system, `member<m>` or `<system>_member<m>`)."""
    nm = getattr(semi, "nmembers", 1)
    if nm > 1 and member is None:
        return [save_solution_file(semi, time, dt, timestep, output_directory,
                                   solution_variables,
                                   f"{system}_member{m}" if system else f"member{m}", m, mesh_file)
                for m in range(nm)]
    names = varnames(solution_variables, semi.equations)
    data = convert_variables(semi, solution_variables, member)
    ndims, polydeg, n_elements, mesh = _member_meta(semi, member)
    if system:
        fname = os.path.join(output_directory, f"solution_{system}_{int(timestep):09d}.h5")
    else:
        fname = os.path.join(output_directory, f"solution_{int(timestep):09d}.h5")
    os.makedirs(output_directory, exist_ok=True)
    return write_solution_file(fname, data, names, ndims=ndims, equations=get_name(semi.equations),
                               polydeg=polydeg, n_elements=n_elements, mesh_type=get_name(mesh),
                               mesh_file=mesh_file, time=time, dt=dt, timestep=timestep,
                               element_variables=element_variables,
                               node_variables=node_variables)
