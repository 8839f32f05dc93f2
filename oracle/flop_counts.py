"""ORACLE — test infrastructure only: the algorithmic work of the bench workloads.

Runs one CarpenterKennedy2N54 step of the oracle compiled with a counting
scalar (orc_flopcount.cpp) on each workload's synthetic state and prints the
operation counts per DOF·stage, per phase of the right-hand side:

    python oracle/flop_counts.py

bench.py keeps the printed table (ALGORITHMIC_OPS) and divides the element
kernel's share of it by the kernel's time for the roofline; its CPU test
(tests/test_flop_counts.py) recomputes the cheap rows.  Weights: add, sub, mul,
div and sqrt count one; log, exp and pow count one operation each as well and
are also listed apart.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

import orc  # noqa: E402

ELEMENT_PHASES = ("volume", "surface_jacobian_sources", "stage_update")


def per_dof_stage(counts, dofs):
    """{phase: {op: count per DOF·stage}}; max_dt runs once per five stages."""
    return {ph: {op: v / (5.0 * dofs) for op, v in c.items()} for ph, c in counts.items()}


def summary(pds):
    """Totals per DOF·stage: all operations, the element kernel's share
    (volume, surface + Jacobian + sources, stage update, and the CFL reduction
    it does on the last stage), and the transcendental count alone."""
    tot = lambda c: sum(c.values())  # noqa: E731
    element = sum(tot(pds[ph]) for ph in ELEMENT_PHASES) + tot(pds["max_dt"])
    return {"total": sum(tot(c) for c in pds.values()), "element": element,
            "transcendental": sum(c["log"] + c["exp"] + c["pow"] for c in pds.values()),
            "div": sum(c["div"] for c in pds.values())}


def shell(tg, trees=16, layers=8):
    eq = tg.CompressibleEulerEnergyEquationsWithGravity3D(
        c_p=1004, c_v=717, gravity=tg.EARTH_GRAVITATIONAL_ACCELERATION)
    mesh = tg.P4estMeshCubedSphereTopography(trees, layers, 6.371e6, 30000.0, polydeg=5)
    basis = tg.LobattoLegendreBasis(5)
    xyz, Ja, invJ = mesh.geometry(basis)
    ie, ifc, fo, be, bf = mesh.connectivity(basis).arrays()
    ic = tg.IsothermalShell(T=250.0, amplitude=1e-3, width=500e3, ncenters=16, seed=1,
                            radius=6.371e6)
    u = np.ascontiguousarray(ic(xyz, 0.0, eq))
    c = orc.count_euler3d_step(5, Ja, invJ, xyz, ie, ifc, fo, be, bf, u,
                               g=tg.EARTH_GRAVITATIONAL_ACCELERATION, omega=tg.EARTH_ROTATION_RATE)
    return per_dof_stage(c, invJ.size)


def bubble_members(tg, members=(0, 1, 2, 3)):
    """Mean over a few members of the 64 x 32, polydeg 3 warm-bubble ensemble."""
    import bench
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    mesh = tg.StructuredMesh((64, 32), (0.0, 0.0), (20000.0, 10000.0), periodicity=(True, False))
    basis = tg.LobattoLegendreBasis(3)
    xy = mesh.geometry(basis)[0]
    params = bench.member_bubbles(max(members) + 1)
    acc = None
    for m in members:
        xc, zc, a = params[m]
        u = np.ascontiguousarray(tg.WarmBubble(xc=xc, zc=zc, dtheta=a)(xy, 0.0, eq))
        c = per_dof_stage(orc.count_euler2d_step(3, 64, 32, 0.0, 20000.0, 0.0, 10000.0, u),
                          64 * 32 * 16)
        if acc is None:
            acc = {ph: dict(v) for ph, v in c.items()}
        else:
            for ph in acc:
                for op in acc[ph]:
                    acc[ph][op] += c[ph][op]
    return {ph: {op: v / len(members) for op, v in d.items()} for ph, d in acc.items()}


def swe(tg, variant, polydeg, trees=4):
    """One covariant shallow-water member of the benchmark ensemble's kind
    (geostrophic balance with a height bump; weak form + LLF or the split
    entropy-conservative form); the counts per DOF depend on the degree only."""
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import (EARTH_GRAVITATIONAL_ACCELERATION as G,
                                                    EARTH_RADIUS, EARTH_ROTATION_RATE as OM)
    eq = (cv.SplitCovariantShallowWaterEquations2D(G, OM) if variant == "ec" else
          cv.CovariantShallowWaterEquations2D(G, OM))
    mesh = cv.P4estMeshCubedSphere2D(trees, EARTH_RADIUS, polydeg=polydeg)
    basis = tg.LobattoLegendreBasis(polydeg)
    aux, xyz = cv.compute_aux_vars(mesh, basis, eq, None, None)
    ie, ifc, fl, _, _ = mesh.connectivity(basis).arrays()

    def ic(x, t, e):
        p = cv.initial_condition_geostrophic_balance(x, t, e)
        r = x / np.sqrt((x ** 2).sum(-1, keepdims=True))
        p[..., 0] *= 1 + 0.03 * np.exp(-((r - np.array([1.0, 0, 0])) ** 2).sum(-1) / 0.05)
        return p
    u = np.ascontiguousarray(cv.transform_initial_condition(ic, eq)(xyz, 0.0, aux))
    fluxes = (dict(volume=0, surf_sym=0, surf_diss=1) if variant == "weak" else
              dict(volume=1, vol_sym=1, vol_nc=1, surf_sym=1, surf_diss=1, surf_nc=2))
    c = orc.count_cov_step(polydeg, aux, xyz, ie, ifc, fl, G, OM, eq.split, fluxes, u)
    return per_dof_stage(c, u.size // 3)


def table(tg, with_shell=True):
    rows = {}
    if with_shell:
        rows["shell"] = summary(shell(tg))
    rows["bubble"] = summary(bubble_members(tg))
    for variant in ("weak", "ec"):
        for N in (3, 5, 7):
            rows[f"swe_{variant}_{N}"] = summary(swe(tg, variant, N))
    return rows


def main():
    import __graft_entry__ as entry
    tg = entry.load_package()
    orc.build()
    rows = table(tg)
    print("ALGORITHMIC_OPS = {")
    for k, v in rows.items():
        print(f'    "{k}": {{' + ", ".join(f'"{a}": {b:.3f}' for a, b in v.items()) + "},")
    print("}")


if __name__ == "__main__":
    main()
