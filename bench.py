"""Benchmark: DOF·stage updates/s of the GB300 DGSEM path (FP64).

Workloads (--workload):
  shell (default) — 3D dry Euler on a cubed-sphere shell: radius 6.371e6 m,
      top at 30 km, 6 panels x 16x16 elements x 8 radial layers (12,288
      elements), polydeg 5 (2,654,208 DOF); isothermal 250 K hydrostatic
      atmosphere at rest with 16 seeded Gaussian density bumps (relative
      amplitude 1e-3, width 500 km); gravity (well-balanced nonconservative
      term) and Coriolis (Omega = 7.292e-5); (flux_ranocha,
      flux_nonconservative_waruszewski_etal) / (FluxLMARS(340), flux_zero);
      slip walls inside/outside; CarpenterKennedy2N54 at CFL 1.  The default
      20 steps are the 100 RK stages of the benchmark configuration.
  ensemble — 256 dry warm-bubble members, each a 64x32-element StructuredMesh
      of 20 km x 10 km at polydeg 3 (8,388,608 DOF), seeded bubble amplitude
      U[1, 3] K and centre jitter +-1 km, per-member dt.
One bench "step" is one RK step (5 stages) of the whole workload;
DOF·stage/s = DOF x 5 x steps / time.  Inputs are larger than L2 (shell: u
127 MB + Ja 191 MB + k 106 MB; ensemble: u 336 MB), so no flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload W]

Multi-GPU: replicas only (every rank runs its own ensemble; no collective on
the data path); value = all ranks' DOF·stages / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402

METRIC = "DOF·stage/s on 1 GB300 (FP64) vs CPU; rainy Newton iters/node learned vs plain"
UNIT = "DOF·stage/s"
LX, LZ = 20000.0, 10000.0
NX, NZ, POLYDEG = 64, 32, 3
C_LMARS = 340.0


def member_bubbles(nmembers, seed0=0):
    """Seeded per-member bubble parameters (Philox, one stream per member)."""
    out = []
    for m in range(nmembers):
        rng = np.random.Generator(np.random.Philox(seed0 + m))
        amp = rng.uniform(1.0, 3.0)
        dx, dz = rng.uniform(-1000.0, 1000.0, size=2)
        out.append((10000.0 + dx, 2000.0 + dz, amp))
    return out


def make_ensemble(tg, nmembers):
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    solver = tg.DGSEM(POLYDEG, (tg.FluxLMARS(C_LMARS), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    mesh = tg.StructuredMesh((NX, NZ), (0.0, 0.0), (LX, LZ), periodicity=(True, False))
    ics = [tg.WarmBubble(xc=xc, zc=zc, dtheta=a) for xc, zc, a in member_bubbles(nmembers)]
    bcs = {"y_neg": tg.boundary_condition_slip_wall, "y_pos": tg.boundary_condition_slip_wall}
    if nmembers == 1:
        semi = tg.SemidiscretizationHyperbolic(mesh, eq, ics[0], solver, boundary_conditions=bcs)
    else:
        semi = tg.SemidiscretizationEnsemble([mesh] * nmembers, eq, ics, solver,
                                             boundary_conditions=bcs)
    return eq, semi


def make_shell(tg, trees=16, layers=8, polydeg=5):
    eq = tg.CompressibleEulerEnergyEquationsWithGravity3D(
        c_p=1004, c_v=717, gravity=tg.EARTH_GRAVITATIONAL_ACCELERATION)
    mesh = tg.P4estMeshCubedSphereTopography(trees, layers, 6.371e6, 30000.0, polydeg=polydeg)
    solver = tg.DGSEM(polydeg, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing(
                          (tg.flux_ranocha, tg.flux_nonconservative_waruszewski_etal)))
    ic = tg.IsothermalShell(T=250.0, amplitude=1e-3, width=500e3, ncenters=16, seed=1,
                            radius=6.371e6)
    semi = tg.SemidiscretizationHyperbolic(
        mesh, eq, ic, solver, source_terms=tg.source_terms_coriolis,
        boundary_conditions={"inside": tg.boundary_condition_slip_wall,
                             "outside": tg.boundary_condition_slip_wall})
    return eq, semi


def make_rainy(tg, nx=128, ny=64, polydeg=3):
    """Moist bubble of the learned-guess benchmark: 128x64 elements over
    20 km x 10 km, polydeg 3 (131,072 nodes), flux_ec_rain / flux_lax_friedrichs,
    rain microphysics, simple slip walls in z."""
    eq = tg.CompressibleRainyEulerEquations2D()
    solver = tg.DGSEM(polydeg, tg.flux_lax_friedrichs,
                      tg.VolumeIntegralFluxDifferencing(tg.flux_ec_rain))
    mesh = tg.StructuredMesh((nx, ny), (0.0, 0.0), (LX, LZ), periodicity=(True, False))
    bcs = {"y_neg": tg.boundary_condition_simple_slip_wall,
           "y_pos": tg.boundary_condition_simple_slip_wall}
    semi = tg.SemidiscretizationHyperbolic(mesh, eq, tg.MoistBubbleRainy(), solver,
                                           source_terms=tg.source_terms_rainy,
                                           boundary_conditions=bcs)
    return eq, semi


def rainy_newton_section(tg, train_states=1_000_000, epochs=40):
    """Saturation Newton solve of the moist-bubble state at tolerance 1e-12
    (relative), once from the plain warm start and once from the learned
    guess; the network is trained first on GPU-generated pairs from a
    different seed (held-out states)."""
    import torch
    lg = tg.learned_guess
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    params, gen, losses = lg.train_guess(n=train_states, epochs=epochs, seed=11, batch=2048)
    t_train = time.perf_counter() - t0
    in_run = rainy_stage_section(tg, params)
    eq, semi = make_rainy(tg)
    u0 = semi.compute_coefficients()
    semi.set_mlp(params)
    semi.set_newton(mode=1, tol=1e-12, max_iterations=30, polish=1)
    res = {}
    for name, learned in (("plain", 0), ("closed_form", 2), ("learned", 1), ("selected", 3)):
        best = 1e30
        for _ in range(3):
            semi.set_state(u0)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            st, it = semi.newton_solve(learned=learned)
            best = min(best, time.perf_counter() - t1)
        res[name] = (st, it, semi.get_state(), best)
    same = np.all(res["plain"][2].reshape(-1, 9) == res["learned"][2].reshape(-1, 9), axis=1)
    ip, il = res["plain"][1].mean(), res["learned"][1].mean()
    sat = lg.saturated(u0.reshape(-1, 9))
    out = {
        "workload": "rainy moist bubble 128x64 elements, polydeg 3, 131072 nodes; "
                    "tolerance 1e-12 relative; canonical finish (snap + 1 update) on both",
        "iters_per_node_plain": ip, "iters_per_node_learned": il, "reduction": ip / il,
        "iters_per_node_closed_form": float(res["closed_form"][1].mean()),
        "iters_per_node_selected": float(res["selected"][1].mean()),
        "iters_saturated_nodes": {"plain": float(res["plain"][1][sat].mean()),
                                  "closed_form": float(res["closed_form"][1][sat].mean()),
                                  "learned": float(res["learned"][1][sat].mean()),
                                  "selected": float(res["selected"][1][sat].mean()),
                                  "fraction": float(sat.mean())},
        "bitwise_equal_fraction": float(same.mean()),
        "fallbacks": int(res["learned"][0]["fallbacks"]),
        "not_converged": int(res["plain"][0]["not_converged"] + res["learned"][0]["not_converged"]),
        "solve_ms_plain": res["plain"][3] * 1e3, "solve_ms_learned": res["learned"][3] * 1e3,
        "training": {"states": train_states, "epochs": epochs,
                     "seconds_incl_generation": t_train, "loss_first": float(losses[0]),
                     "loss_last": float(losses[-1])},
        "in_run": in_run,
    }
    semi.close()
    return out


def rainy_stage_section(tg, params, steps=20):
    """The learned guess where the reference uses the solve: config 2 (the
    128 x 64, polydeg 3 moist bubble) run for `steps` CK2N54 steps at CFL 1
    with the Newton stage limiter after every stage
    (src/callbacks_stage/nonlinear_solve_dg2d.jl:6-44, as
    examples/euler/moist_air/buoyancy/elixir_hoeck_bubble.jl:87-94 passes it),
    at tolerance 1e-12 relative with the canonical finish, from four starts:
    the warm start of the reference (slots 7-9 of the previous stage), the
    closed-form unsaturated branch alone (warm start on saturated nodes),
    closed form + MLP, and closed form + the smaller-residual one of MLP and
    warm start ("selected").  Newton updates per node solve over the run, the
    run's DOF·stage/s (CUDA events on the library's stream), and whether the
    runs end in the same bits."""
    import torch
    lg = tg.learned_guess
    out, finals = {}, {}
    for name, start in (("warm", 0), ("closed_form", 2), ("learned", 1), ("selected", 3)):
        eq, semi = make_rainy(tg)
        semi.set_mlp(params)
        semi.set_newton(mode=1, tol=1e-12, max_iterations=30, polish=1)
        semi.set_newton_start(start)
        semi.set_state(semi.compute_coefficients())
        t = semi.rk_steps(1, cfl=1.0, t=0.0)  # warm-up: graph capture
        semi.newton_counters(reset=True)
        stream = torch.cuda.ExternalStream(semi.stream())
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        t = semi.rk_steps(steps, cfl=1.0, t=t)
        ev1.record(stream)
        torch.cuda.synchronize()
        sec = ev0.elapsed_time(ev1) * 1e-3
        c = semi.newton_counters(reset=True)
        finals[name] = semi.get_state()
        sat = lg.saturated(finals[name].reshape(-1, 9))
        out[name] = {"updates_per_node_solve": c["updates"] / c["node_solves"],
                     "fallbacks": c["fallbacks"], "not_converged": c["not_converged"],
                     "node_solves": c["node_solves"],
                     "dof_stage_per_s": semi.ndofs * 5 * steps / sec,
                     "saturated_fraction_final": float(sat.mean())}
        semi.close()
    w = out["warm"]["updates_per_node_solve"]
    out["reduction_vs_warm"] = {k: w / out[k]["updates_per_node_solve"]
                                for k in ("closed_form", "learned", "selected")}
    out["bitwise_equal_final_fraction"] = {
        k: float(np.all(finals["warm"].reshape(-1, 9) == finals[k].reshape(-1, 9), axis=1).mean())
        for k in ("closed_form", "learned", "selected")}
    out["workload"] = (f"rainy moist bubble 128x64, polydeg 3, {steps} CK2N54 steps at CFL 1, "
                       "Newton limiter after every stage, tolerance 1e-12 relative, canonical "
                       "finish")
    return out


def sequential_member_rate(tg, steps):
    """DOF·stage/s of one ensemble member run alone (the rate of running the
    members one by one on the same GPU)."""
    import torch
    eq, semi = make_ensemble(tg, 1)
    semi.set_state(semi.compute_coefficients())
    t = semi.rk_steps(3, cfl=1.0, t=0.0)
    stream = torch.cuda.ExternalStream(semi.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    t = semi.rk_steps(steps, cfl=1.0, t=t)
    e1.record(stream)
    torch.cuda.synchronize()
    rate = semi.ndofs * 5 * steps / (e0.elapsed_time(e1) * 1e-3)
    semi.close()
    return rate


def swe_member_specs(nmembers, seed=5):
    """Seeded uneven members: trees per face edge U{8..32}, polydeg from
    {3, 5, 7}, Gaussian height bumps of 1-5 % on the geostrophic balance."""
    rng = np.random.Generator(np.random.Philox(seed))
    specs = []
    for m in range(nmembers):
        k = int(rng.integers(8, 33))
        N = int(rng.choice([3, 5, 7]))
        amp = float(rng.uniform(0.01, 0.05))
        z = rng.uniform(-1, 1)
        lon = rng.uniform(-np.pi, np.pi)
        c = np.array([np.sqrt(1 - z * z) * np.cos(lon), np.sqrt(1 - z * z) * np.sin(lon), z])
        specs.append((k, N, amp, c))
    return specs


def swe_equations(tg, variant):
    from trixiatmo_gb300.initial_conditions import (EARTH_GRAVITATIONAL_ACCELERATION as G,
                                                    EARTH_ROTATION_RATE as OM)
    cv = tg.covariant
    if variant == "ec":
        return cv.SplitCovariantShallowWaterEquations2D(G, OM)
    return cv.CovariantShallowWaterEquations2D(G, OM)


def make_swe_ensemble(tg, nmembers=64, variant="weak", seed=5, members=None):
    """64 covariant shallow-water members of uneven size and degree on the
    cubed sphere: weak form + flux_lax_friedrichs (elixir_geostrophic_balance)
    or the split entropy-conservative form; Cartesian global coordinates."""
    cv = tg.covariant
    from trixiatmo_gb300.initial_conditions import EARTH_RADIUS
    eq = swe_equations(tg, variant)
    specs = swe_member_specs(nmembers, seed)
    if members is not None:
        specs = [specs[m] for m in members]
    meshes, solvers, ics = [], [], []
    for k, N, amp, c in specs:
        meshes.append(cv.P4estMeshCubedSphere2D(k, EARTH_RADIUS, polydeg=N))
        if variant == "ec":
            solvers.append(tg.DGSEM(N, (cv.FluxPlusDissipation(cv.flux_ec,
                                                               cv.DissipationLocalLaxFriedrichs()),
                                        cv.flux_nonconservative_surface_simplified),
                                    tg.VolumeIntegralFluxDifferencing(
                                        (cv.flux_ec, cv.flux_nonconservative_ec))))
        else:
            solvers.append(tg.DGSEM(N, tg.flux_lax_friedrichs, tg.VolumeIntegralWeakForm()))

        def ic(x, t, e, amp=amp, c=c):
            p = cv.initial_condition_geostrophic_balance(x, t, e)
            r = x / np.sqrt((x ** 2).sum(-1, keepdims=True))
            d2 = ((r - c) ** 2).sum(-1)
            p[..., 0] *= 1 + amp * np.exp(-d2 / 0.05)
            return p
        ics.append(cv.transform_initial_condition(ic, eq))
    ens = tg.SemidiscretizationCovariantEnsemble(meshes, eq, ics, solvers,
                                                 source_terms=cv.source_terms_geometric_coriolis)
    return eq, ens, specs, (meshes, solvers, ics)


def cpu_oracle_rate_swe(tg, args, eq):
    """The oracle's covariant shallow-water steps on the host cores, on a
    bounded sample of the uneven ensemble (its first four members): the same
    members, states and step control as the GPU run.  The members' meshes and
    metric terms come from the package's mesh construction; only the oracle's
    CK2N54 steps are timed."""
    orc = entry.load_oracle()
    orc.build()
    M = args.swe_members
    sample = list(range(min(4, M)))
    _, ens_s, specs_s, _ = make_swe_ensemble(tg, M, args.swe_variant, members=sample)
    cov_ids = dict(volume=0, surf_sym=0, surf_diss=1) if args.swe_variant == "weak" else \
        dict(volume=1, vol_sym=1, vol_nc=1, surf_sym=1, surf_diss=1, surf_nc=2)
    a = time.perf_counter()
    cdofs = 0
    for i, m in enumerate(sample):
        mesh = ens_s.meshes[i]
        basis = ens_s.solvers[i].basis
        conn = mesh.connectivity(basis)
        ie, ifc, flip, _, _ = conn.arrays()
        c = orc.CovSWE(basis.n - 1, ens_s._H.aux[i], ens_s._H.xyz[i], ie, ifc, flip,
                       eq.gravity, eq.rotation_rate, eq.split, cov_ids)
        um = np.ascontiguousarray(ens_s.member_state(ens_s.compute_coefficients(), i))
        c.ck_steps(um, np.zeros_like(um), 0.0, 0.4, args.cpu_steps)
        cdofs += um.size // 3
    cel = time.perf_counter() - a
    ens_s.close()
    return {"value": cdofs * 5 * args.cpu_steps / cel, "unit": UNIT,
            "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
            "kind": "port",
            "sample": f"{len(sample)} of the members x {args.cpu_steps} CK2N54 steps, oracle/ "
                      f"C++ OpenMP ({cel:.1f} s)"}, cel


def run_swe(args):
    """Uneven covariant shallow-water ensemble: whole-ensemble DOF·stage/s,
    the same members run one by one, p50/p99 step latency."""
    import torch
    tg = entry.load_package()
    torch.cuda.set_device(0)
    t_build = time.perf_counter()
    eq, ens, specs, parts = make_swe_ensemble(tg, args.swe_members, args.swe_variant)
    t_build = time.perf_counter() - t_build
    u0 = ens.compute_coefficients()
    ens.set_state(u0)
    M = ens.nmembers
    dofs = ens.ndofs
    stream = torch.cuda.ExternalStream(ens.stream())
    t = ens.rk_steps(max(args.warmup, 1), cfl=0.4, t=np.zeros(M))
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    t = ens.rk_steps(args.steps, cfl=0.4, t=t)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clock_info = clocks.stop()
    value = dofs * 5 * args.steps / (ms * 1e-3)
    # per-step latency through the API (host-observed, one step per call)
    lat = []
    for _ in range(max(args.steps, 20)):
        a = time.perf_counter()
        t = ens.rk_steps(1, cfl=0.4, t=t)
        lat.append((time.perf_counter() - a) * 1e3)
    ms_if, ms_el = ens.time_kernels(reps=10)
    # the same members one by one, each in its own handle
    meshes, solvers, ics = parts
    seq_time = 0.0
    for m in range(M):
        alone = tg.SemidiscretizationHyperbolic(meshes[m], eq, ics[m], solvers[m],
                                                source_terms=tg.covariant.source_terms_geometric_coriolis)
        alone.set_state(np.ascontiguousarray(ens.member_state(u0, m)))
        tm = alone.rk_steps(max(args.warmup, 1), cfl=0.4, t=0.0)
        s = torch.cuda.ExternalStream(alone.stream())
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a0.record(s)
        alone.rk_steps(args.steps, cfl=0.4, t=tm)
        a1.record(s)
        torch.cuda.synchronize()
        seq_time += a0.elapsed_time(a1)
        alone.close()
    seq_value = dofs * 5 * args.steps / (seq_time * 1e-3)
    # end to end through the C ABI: H2D of the state, one step, D2H (stored
    # into the pinned buffer by the last stage's kernel, tag_set_state_sink)
    u_pin = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True).numpy()
    u_pin[...] = u0
    ens.set_state_sink(u_pin)
    t_e = np.zeros(M)
    a = time.perf_counter()
    for _ in range(args.steps):
        ens.set_state(u_pin)
        t_e = ens.rk_steps(1, cfl=0.4, t=t_e)
    e2e = dofs * 5 * args.steps / (time.perf_counter() - a)
    ens.set_state_sink(None)
    # bytes per element launch (stage mode): u, k read + written, packed
    # metric data (16 doubles) read per node, outward surface fluxes read
    nodes = dofs
    face_doubles = sum(6 * k * k * 4 * (N + 1) * 3 for k, N, _, _ in specs)
    by = 8 * (nodes * (3 + 3 + 16 + 3 + 3) + face_doubles)
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        hbm_peak, hbm_src = float(peaks["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        hbm_peak, hbm_src = 6800.0, "fallback"
    gbs = by / (ms_el * 1e-3) / 1e9
    fl = sum(6 * k * k * (N + 1) ** 2 * ALGORITHMIC_OPS[f"swe_{args.swe_variant}_{N}"]["element"]
             for k, N, _, _ in specs)
    peak_fp64, peak_src, probe_fp64 = fp64_roofline_peak(tg, clock_info)
    achieved_tf = fl / (ms_el * 1e-3) / 1e12
    traffic = TRAFFIC_PER_DOF.get("swe" if args.swe_variant == "weak" else "swe_ec")
    cpu = None if args.no_cpu else cpu_oracle_rate_swe(tg, args, eq)[0]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"{M} covariant shallow-water members on the cubed sphere, trees "
                               f"per face edge U{{8..32}}, polydeg in {{3, 5, 7}}, geostrophic "
                               f"balance + 1-5 % height bumps, "
                               f"{'weak form + LLF' if args.swe_variant == 'weak' else 'split EC'}"
                               f", CK2N54 CFL 0.4, per-member dt",
                   "dofs": dofs, "elements": ens.nelements, "members": M,
                   "degree_runs": int(ens._H.nmembers), "build_seconds": t_build,
                   "l2": "inputs larger than L2 (u + k + packed metric data)"},
        "roofline": {"bound": "fp64", "achieved": achieved_tf, "peak": peak_fp64 / 1e12,
                     "unit": "TFLOP/s", "frac": achieved_tf / (peak_fp64 / 1e12),
                     "traffic": (traffic * dofs) if traffic else None,
                     "traffic_source": "ncu dram__bytes_read+write per DOF of a capture, "
                                       "scaled by DOF" if traffic else None,
                     "kernel": "k_cov_element (volume + surface + Jacobian + sources + RK stage)",
                     "peak_source": peak_src, "fma_stream_tflops": probe_fp64 / 1e12,
                     "frac_of_fma_stream": achieved_tf / (probe_fp64 / 1e12),
                     "hbm_achieved_gbs": gbs, "hbm_peak_gbs": hbm_peak,
                     "hbm_frac": gbs / hbm_peak, "hbm_peak_source": hbm_src,
                     "ms_element": ms_el, "ms_interface": ms_if,
                     "flops_per_launch": fl, "flops_source": FLOPS_SOURCE,
                     "bytes_per_launch": by},
        "ensemble_vs_sequential": {"sequential_rate": seq_value, "speedup": value / seq_value},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "steps": len(lat)},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(u0.nbytes),
                "d2h_bytes_per_step": int(u0.nbytes)},
        "gpu_launches": args.steps * 11,
        "clocks": clock_info,
        "status": ens.status(),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))
    ens.close()


# ---- algorithmic work per DOF·stage ------------------------------------------
# Operation counts of the oracle's formulas (a restatement of the reference's
# flux_ranocha, flux_nonconservative_waruszewski_etal, FluxLMARS, covariant
# fluxes and sources, CK2N54 stage update and max_dt), obtained by running one
# CK2N54 step of the oracle compiled with a counting scalar on each workload's
# synthetic state (`python oracle/flop_counts.py`, which prints this table;
# tests/test_flop_counts.py recomputes the cheap rows).  add, sub, mul, div,
# sqrt, log, exp and pow count one operation each; "element" is the element
# kernel's share (volume integral, surface integral, apply_jacobian, sources,
# stage update, and the CFL reduction of the last stage spread over the five
# stages), "total" adds the interface and boundary fluxes; "transcendental"
# (log, exp, pow) and "div" are contained in the totals.  These count the
# reference's formulas as written, which recompute primitive variables in
# every two-point flux and evaluate the nonconservative term against every
# node of a line; the kernels compute per-node quantities once, so the
# algorithmic rate can exceed what the FP64 pipe executes.
FLOPS_SOURCE = ("operation count of the oracle's formulas per DOF·stage (counting scalar, "
                "oracle/flop_counts.py), element-kernel share, x DOF")
ALGORITHMIC_OPS = {
    "shell": {"total": 2381.223, "element": 2329.702, "transcendental": 7.500, "div": 232.592},
    "bubble": {"total": 874.958, "element": 835.060, "transcendental": 1.871, "div": 78.517},
    "swe_weak_3": {"total": 247.013, "element": 171.013, "transcendental": 0.000, "div": 11.400},
    "swe_weak_5": {"total": 243.339, "element": 192.672, "transcendental": 0.000, "div": 9.733},
    "swe_weak_7": {"total": 253.503, "element": 215.503, "transcendental": 0.000, "div": 8.900},
    "swe_ec_3": {"total": 578.013, "element": 506.013, "transcendental": 0.000, "div": 39.400},
    "swe_ec_5": {"total": 759.672, "element": 711.672, "transcendental": 0.000, "div": 53.067},
    "swe_ec_7": {"total": 954.503, "element": 918.503, "transcendental": 0.000, "div": 67.900},
}


def bytes_per_element_launch_3d(n, nelem):
    """Compulsory DRAM bytes of one 3D element-kernel (stage mode) launch: read
    u (6), Ja (9), invJ (1), k (5), sfv (6 faces x n^2 x 5 per element); write u
    (5 active) and k (5)."""
    nodes = n ** 3 * nelem
    return 8 * (nodes * (6 + 9 + 1 + 5 + 5 + 5) + nelem * 6 * n * n * 5)


def bytes_per_element_launch(n, nelem):
    """Compulsory DRAM bytes of one element-kernel (stage mode) launch: read u
    (5 vars), Ja (4), invJ (1), sfv (4 faces x n x 4 vars per element), k (4);
    write u (4 active vars) and k (4)."""
    nodes = n * n * nelem
    return 8 * (nodes * (5 + 4 + 1 + 4 + 4 + 4) + nelem * 4 * n * 4)


# ---- FP64 roofline denominator ---------------------------------------------
# GB300's FP64 pipe executes at most 2 DFMA (4 flops) per clock per SM: ncu on
# the FMA probe of tag_fp64_peak (profiles/fp64_pipe_gb300.md) counts 3.36
# flops per clock per SM at 84.2 % sm__pipe_fp64_cycles_active, i.e. a pipe
# peak of 4.0.  The denominator is that peak at the SM clock sampled during
# the timed region (1.259 TFLOP/s at 2070 MHz); the probe's own rate, the
# best a stream of independent FMAs reaches, is reported beside it.
FP64_FLOPS_PER_CLK_SM = 4.0


def fp64_roofline_peak(tg, clock_info):
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = clock_info.get("sm_mhz") or clock_info.get("sm_max_mhz") or 2070.0
    peak = FP64_FLOPS_PER_CLK_SM * sms * mhz * 1e6
    src = (f"FP64 pipe peak 4 flop/clk/SM (ncu, profiles/fp64_pipe_gb300.md) x {sms} SMs x "
           f"{mhz:.0f} MHz sampled in the timed region, of measured")
    return peak, src, tg.fp64_peak()


# ---- clocks during the timed region ----------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.lines = []
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---- CPU legs (the oracle, test infrastructure) -----------------------------
def cpu_oracle_rate(nmembers_sample, steps, warmup=0):
    """Times the C++ OpenMP oracle (restatement of the reference's rhs! + CK2N54
    stage) on `nmembers_sample` members for `steps` RK steps each; returns
    DOF·stage/s and the thread count."""
    orc = entry.load_oracle()
    orc.build()
    cases = []
    for xc, zc, amp in member_bubbles(nmembers_sample):
        c = orc.Euler2D(POLYDEG, NX, NZ, 0.0, LX, 0.0, LZ, True, False, 1004.0, 717.0, 9.81,
                        C_LMARS)
        u = c.initial_condition(1, (xc, zc, 2000.0, amp, 0.0))
        cases.append((c, u, np.zeros_like(u)))
    for c, u, k in cases[:1]:
        for _ in range(warmup):
            c.ck_steps(u, k, 0.0, 1.0, 1)
    t0 = time.perf_counter()
    for c, u, k in cases:
        c.ck_steps(u, k, 0.0, 1.0, steps)
    el = time.perf_counter() - t0
    dofs = nmembers_sample * NX * NZ * (POLYDEG + 1) ** 2
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return dofs * 5 * steps / el, threads, el


def cpu_oracle_rate_shell(steps):
    """Times the oracle on the full shell workload for `steps` RK steps (the
    host mirror builds the same geometry arrays the GPU path receives; no GPU
    code runs)."""
    orc = entry.load_oracle()
    orc.build()
    tg = entry.load_package()
    eq = tg.CompressibleEulerEnergyEquationsWithGravity3D(
        c_p=1004, c_v=717, gravity=tg.EARTH_GRAVITATIONAL_ACCELERATION)
    mesh = tg.P4estMeshCubedSphereTopography(16, 8, 6.371e6, 30000.0, polydeg=5)
    basis = tg.LobattoLegendreBasis(5)
    xyz, Ja, invJ = mesh.geometry(basis)
    conn = mesh.connectivity(basis)
    o = orc.Euler3D(5, Ja, invJ, xyz, *conn.arrays(), c_p=1004.0, c_v=717.0,
                    g=tg.EARTH_GRAVITATIONAL_ACCELERATION, c_lmars=340.0,
                    omega=tg.EARTH_ROTATION_RATE)
    ic = tg.IsothermalShell(T=250.0, amplitude=1e-3, width=500e3, ncenters=16, seed=1,
                            radius=6.371e6)
    u = np.ascontiguousarray(ic(xyz, 0.0, eq))
    k = np.zeros_like(u)
    t0 = time.perf_counter()
    o.ck_steps(u, k, 0.0, 1.0, steps)
    el = time.perf_counter() - t0
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return invJ.size * 5 * steps / el, threads, el


def max_over_ranks(x, world, device="cuda"):
    """Largest value of x over all ranks (x itself on one rank): the timing
    rule of the replicas-only multi-GPU run."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world, dofs, stages, seconds):
    """Whole-job DOF·stage/s of `world` replicas that each advanced `dofs`
    by `stages` stages, timed by the slowest rank."""
    return world * dofs * stages / seconds


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


L2_BYTES = 129e6  # GB300 L2


def l2_note_of(parts):
    """Whether the arrays one element launch streams (bytes by name) exceed
    the L2; the timing rule asks for inputs larger than L2 or a flush."""
    desc = ", ".join(f"{k} {v / 1e6:.0f} MB" for k, v in parts.items())
    if sum(parts.values()) > L2_BYTES:
        return f"inputs larger than L2 ({desc})"
    return f"inputs fit in L2 ({desc}); L2-resident timing, not a headline number"


def julia_probe():
    """Looks for a Julia installation with Trixi and TrixiAtmo on this machine
    (the reference's own CPU rhs! would be timed there); returns a one-line
    finding."""
    import shutil
    exe = shutil.which("julia")
    if exe is None:
        return "julia: not found on PATH"
    try:
        r = subprocess.run([exe, "--startup-file=no", "-e", "using Trixi, TrixiAtmo; print(1)"],
                           capture_output=True, text=True, timeout=300)
    except (OSError, subprocess.TimeoutExpired) as e:
        return f"julia at {exe}: probe failed ({e})"
    if r.returncode != 0:
        return f"julia at {exe}: `using Trixi, TrixiAtmo` failed"
    return f"julia at {exe} with Trixi and TrixiAtmo"


def _note():
    probe = julia_probe()
    state = "not timed by this bench" if "with Trixi" in probe else "unavailable on this box"
    return (f"reference Julia rhs! baseline: {state} ({probe}); the reference CPU rhs! is the "
            "C++ OpenMP restatement in oracle/ (pinned to the reference's golden l2/linf)")


def run_reference(args):
    world, rank, _ = dist_init()
    if rank != 0:
        return
    steps = max(args.steps, 1)
    if args.workload == "shell":
        rate, threads, el = cpu_oracle_rate_shell(steps)
        config = {"workload": "3D cubed-sphere shell 6x16x16x8, polydeg 5, isothermal + Coriolis, "
                              "CK2N54 CFL 1", "dofs": 2654208}
        sample = f"the full shell workload, {steps} CK2N54 steps"
    elif args.workload == "swe":
        # the sampled members' meshes and metric terms are built by the package
        tg = entry.load_package()
        args.cpu_steps = steps
        c, el = cpu_oracle_rate_swe(tg, args, swe_equations(tg, args.swe_variant))
        rate, threads = c["value"], c["cores"]
        config = {"workload": f"{args.swe_members} covariant shallow-water members on the cubed "
                              f"sphere, {args.swe_variant} form", "members": args.swe_members}
        sample = c["sample"]
    else:
        sample_m = args.ref_members
        rate, threads, el = cpu_oracle_rate(sample_m, steps, warmup=args.warmup > 0)
        config = {"workload": f"ensemble of {args.members} dry warm-bubble members (64x32, "
                              f"polydeg 3)", "members": args.members,
                  "dofs": args.members * NX * NZ * 16}
        sample = f"{sample_m} members x {steps} CK2N54 steps"
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config,
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": _note(),
    }
    print(json.dumps(line))


def run_ours(args):
    import torch
    world, rank, local = dist_init()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    tg = entry.load_package()
    if args.workload == "shell":
        eq, semi = make_shell(tg, args.trees, args.layers)
        n = semi.n
        fl = ALGORITHMIC_OPS["shell"]["element"] * semi.ndofs
        by = bytes_per_element_launch_3d(n, semi.nelements)
        workload = (f"3D dry Euler on a cubed-sphere shell, 6 panels x {args.trees}x{args.trees} "
                    f"elements x {args.layers} layers, polydeg 5, isothermal 250 K + seeded "
                    "density bumps, gravity + Coriolis, CK2N54 CFL 1")
        l2_note = l2_note_of({"u": semi.ndofs * 6 * 8, "Ja": semi.ndofs * 9 * 8,
                              "k": semi.ndofs * 5 * 8})
    else:
        eq, semi = make_ensemble(tg, args.members)
        n = semi.n
        fl = ALGORITHMIC_OPS["bubble"]["element"] * semi.ndofs
        by = bytes_per_element_launch(n, semi.nelements)
        workload = (f"ensemble of {args.members} dry warm-bubble members, 64x32 StructuredMesh, "
                    "polydeg 3, CK2N54 CFL 1, per-member dt")
        l2_note = l2_note_of({"u": semi.ndofs * 5 * 8, "k": semi.ndofs * 4 * 8})
    u0 = semi.compute_coefficients()
    semi.set_state(u0)
    nmem = semi.nmembers
    stream = torch.cuda.ExternalStream(semi.stream())
    dofs = semi.ndofs
    t_m = np.zeros(nmem)
    # warm-up (also runs the elements-per-CTA autotuner and the graph capture)
    t_m = semi.rk_steps(max(args.warmup, 1), cfl=1.0, t=t_m)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    t_m = semi.rk_steps(args.steps, cfl=1.0, t=t_m)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clock_info = clocks.stop()
    ms = max_over_ranks(ms, world)
    if world > 1:
        torch.distributed.barrier()
    value = replica_rate(world, dofs, 5 * args.steps, ms * 1e-3)
    status = semi.status()

    # kernel timing for the roofline (same stream, CUDA events, stage mode)
    ms_if, ms_el = semi.time_kernels(reps=10)
    peak_fp64, peak_src, probe_fp64 = fp64_roofline_peak(tg, clock_info)
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        hbm_peak, hbm_src = float(peaks["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        hbm_peak, hbm_src = 6800.0, "fallback"
    achieved_tf = fl / (ms_el * 1e-3) / 1e12
    achieved_gbs = by / (ms_el * 1e-3) / 1e9
    traffic = TRAFFIC_PER_DOF.get(args.workload)

    # end to end through the C ABI with pinned host buffers: per step, H2D of
    # the state, one RK step (5 stages), D2H of the state.  The last stage's
    # kernel stores the new state into the pinned buffer (tag_set_state_sink);
    # 3D: the state is also read from it by one kernel (tag_set_state)
    u_pin = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True).numpy()
    u_pin[...] = u0
    semi.set_state_sink(u_pin)

    def e2e_step(t_e):
        semi.set_state(u_pin)
        return semi.rk_steps(1, cfl=1.0, t=t_e)  # the result lands in u_pin

    t_e = np.zeros(nmem)
    for _ in range(2):
        t_e = e2e_step(t_e)
    e2e_steps = max(3, args.steps // 2)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        t_e = e2e_step(t_e)
    el = max_over_ranks(time.perf_counter() - t0, world)
    e2e = replica_rate(world, dofs, 5 * e2e_steps, el)
    semi.set_state_sink(None)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        if args.workload == "shell":
            rate, threads, cel = cpu_oracle_rate_shell(args.cpu_steps_shell)
            smp = (f"the full shell, {args.cpu_steps_shell} CK2N54 steps (5 stages each), "
                   f"oracle/ C++ OpenMP ({cel:.1f} s)")
        else:
            rate, threads, cel = cpu_oracle_rate(args.cpu_members, args.cpu_steps)
            smp = (f"{args.cpu_members} members x {args.cpu_steps} CK2N54 steps (5 stages each) "
                   f"of the same ensemble, oracle/ C++ OpenMP ({cel:.1f} s)")
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": smp}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": workload, "dofs": dofs, "elements": semi.nelements,
                       "polydeg": n - 1, "members": nmem,
                       "elements_per_cta": semi.elements_per_block(),
                       "threads_per_cta": semi.cta_threads(), "l2": l2_note,
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "fp64", "achieved": achieved_tf, "peak": peak_fp64 / 1e12,
                         "unit": "TFLOP/s", "frac": achieved_tf / (peak_fp64 / 1e12),
                         "traffic": (traffic * dofs) if traffic else None,
                         "traffic_source": "ncu dram__bytes_read+write per DOF of a capture, "
                                           "scaled by DOF" if traffic else None,
                         "kernel": "element kernel (volume + surface + Jacobian + sources + "
                                   "RK stage)",
                         "peak_source": peak_src, "fma_stream_tflops": probe_fp64 / 1e12,
                         "frac_of_fma_stream": achieved_tf / (probe_fp64 / 1e12),
                         "hbm_achieved_gbs": achieved_gbs, "hbm_peak_gbs": hbm_peak,
                         "hbm_frac": achieved_gbs / hbm_peak, "hbm_peak_source": hbm_src,
                         "ms_element": ms_el, "ms_interface": ms_if,
                         "flops_per_launch": fl, "flops_source": FLOPS_SOURCE,
                         "bytes_per_launch": by,
                         "executed": executed_roofline(args.workload, dofs, ms_el, peak_fp64)},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(u0.nbytes),
                    "d2h_bytes_per_step": int(u0.nbytes),
                    "d2h": "stored into the pinned buffer by the last stage's element kernel"},
            "gpu_launches": args.steps * 11,
            "clocks": clock_info,
            "status": status,
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
        if args.workload == "ensemble":
            seq = sequential_member_rate(tg, args.steps)
            line["ensemble_vs_sequential"] = {"sequential_member_rate": seq,
                                              "speedup": value / world / seq}
        if world == 1 and not args.no_rainy:
            line["rainy_newton"] = rainy_newton_section(tg)
        print(json.dumps(line))
    semi.close()
    if world > 1:
        torch.distributed.destroy_process_group()


# DRAM bytes per DOF of the element kernel from ncu captures (read + write),
# used to report `traffic` for the full-size launch.
TRAFFIC_PER_DOF = {"shell": 281.26,      # k_element3d, stage mode, full shell
                   "ensemble": 205.42,    # k_element 2D, stage mode, 128-member ensemble
                   "swe": 214.71,         # k_cov_element weak form, 8 of the SWE members
                   "swe_ec": 215.20}      # k_cov_element split EC form, the same 8 members
# FP64 operations the element kernel executes per DOF (DFMA counted as 2), from
# the same ncu captures (smsp__sass_thread_inst_executed_op_{dfma,dadd,dmul}),
# beside the algorithmic count: the kernel computes per-node quantities once
# where the reference's formulas recompute them per pair
EXECUTED_FLOPS_PER_DOF = {"shell": 950.7, "ensemble": 368.7}


def executed_roofline(workload, dofs, ms_el, peak_fp64):
    f = EXECUTED_FLOPS_PER_DOF.get(workload)
    if not f:
        return None
    tf = f * dofs / (ms_el * 1e-3) / 1e12
    return {"flops_per_dof": f, "achieved": tf, "frac": tf / (peak_fp64 / 1e12),
            "source": "ncu FP64 thread instructions of the element kernel (profiles/)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="shell", choices=["shell", "ensemble", "swe"])
    ap.add_argument("--swe-members", type=int, default=64)
    ap.add_argument("--swe-variant", default="weak", choices=["weak", "ec"])
    ap.add_argument("--cpu-steps-shell", type=int, default=2)
    ap.add_argument("--members", type=int, default=256)
    ap.add_argument("--cpu-members", type=int, default=64)
    ap.add_argument("--cpu-steps", type=int, default=8)
    ap.add_argument("--ref-members", type=int, default=16)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-rainy", action="store_true")
    ap.add_argument("--trees", type=int, default=16,
                    help="shell: trees per cube-face edge (16 = the benchmark configuration)")
    ap.add_argument("--layers", type=int, default=8,
                    help="shell: radial layers (8 = the benchmark configuration)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "swe":
        run_swe(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
