"""CPU-only checks of the host side: the C-ABI library loads and exports every
symbol include/*.h declares, argument validation fails cleanly without a GPU,
and the host mirror's geometry / initial states equal the oracle's."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(tag_\w+)\s*\(", src, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ["tag_create", "tag_destroy", "tag_rhs", "tag_rk_steps", "tag_max_dt",
                     "tag_status", "tag_set_state", "tag_get_state"]:
        assert required in names


def test_library_exports_every_declared_symbol(tg):
    import importlib
    importlib.import_module("trixiatmo_gb300.build").build()
    L = tg._lib.load(build_if_missing=False)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(L, n)]
    assert not missing, missing
    # the Python binding covers every declared symbol, too
    assert declared_symbols() <= set(tg._lib.SIGNATURES)


def test_create_without_device_or_with_bad_config_fails_cleanly(tg):
    L = tg._lib.load()
    cfg = tg._lib.TagConfig()
    h = ctypes.c_void_p()
    rc = L.tag_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc in (tg._lib.TAG_E_NO_DEVICE, tg._lib.TAG_E_INVALID)
    assert not h.value
    assert L.tag_create(None, ctypes.byref(h)) == tg._lib.TAG_E_INVALID
    assert L.tag_last_error()


def test_host_geometry_matches_oracle(tg, orc):
    b = tg.LobattoLegendreBasis(3)
    m = tg.StructuredMesh((16, 8), (0.0, 0.0), (20000.0, 10000.0), periodicity=(True, False))
    xy, Ja, invJ = m.geometry(b)
    o = orc.Euler2D(3, 16, 8, 0.0, 20000.0, 0.0, 10000.0, True, False)
    Jo, io, xo = o.geometry()
    assert np.allclose(xy, xo, rtol=1e-15, atol=1e-9)
    assert np.allclose(Ja, Jo, rtol=1e-13, atol=1e-9)
    assert np.allclose(invJ, io, rtol=1e-13, atol=0)


def test_host_connectivity(tg):
    m = tg.StructuredMesh((4, 3), (0.0, 0.0), (1.0, 1.0), periodicity=(True, False))
    c = m.connectivity()
    ie, ifc, fl, be, bf = c.arrays()
    # periodic in x: 4*3 x-interfaces; y: 4*2 interior interfaces; walls 4+4
    assert ie.shape == (12 + 8, 2) and be.shape == (8,)
    assert set(c.bd_names) == {"y_neg", "y_pos"}
    # every element face is used exactly once
    used = {}
    for (e0, e1), (f0, f1) in zip(ie, ifc):
        for e, f in ((e0, f0), (e1, f1)):
            used[(e, f)] = used.get((e, f), 0) + 1
    for e, f in zip(be, bf):
        used[(e, f)] = used.get((e, f), 0) + 1
    assert len(used) == 12 * 4 and set(used.values()) == {1}


def test_host_initial_condition_matches_oracle(tg, orc):
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    b = tg.LobattoLegendreBasis(3)
    m = tg.StructuredMesh((64, 32), (0.0, 0.0), (20000.0, 10000.0), periodicity=(True, False))
    xy, _, _ = m.geometry(b)
    u = tg.WarmBubble(dtheta=2.0)(xy, 0.0, eq)
    o = orc.Euler2D(3, 64, 32, 0.0, 20000.0, 0.0, 10000.0, True, False)
    uo = o.initial_condition(1, (10000.0, 2000.0, 2000.0, 2.0, 0.0))
    assert np.allclose(u, uo, rtol=1e-13, atol=1e-12)
    m2 = tg.StructuredMesh((60, 8), (0.0, 0.0), (300000.0, 10000.0), periodicity=(True, False))
    xy2, _, _ = m2.geometry(b)
    g = tg.initial_condition_gravity_waves(xy2, 0.0, eq)
    o2 = orc.Euler2D(3, 60, 8, 0.0, 300000.0, 0.0, 10000.0, True, False)
    assert np.allclose(g, o2.initial_condition(0), rtol=1e-13, atol=1e-12)


def test_semidiscretization_rejects_unsupported_setup(tg):
    eq = tg.CompressibleEulerEnergyEquationsWithGravity2D(c_p=1004, c_v=717, gravity=9.81)
    solver = tg.DGSEM(3, (tg.FluxLMARS(340.0), tg.flux_zero),
                      tg.VolumeIntegralFluxDifferencing((tg.flux_zero, tg.flux_zero)))
    mesh = tg.StructuredMesh((2, 2), (0.0, 0.0), (1.0, 1.0), periodicity=(True, True))
    with pytest.raises(ValueError):
        tg.SemidiscretizationHyperbolic(mesh, eq, None, solver)
