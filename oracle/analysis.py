"""ORACLE — test infrastructure only.

End-of-run error norms computed the way Trixi's AnalysisCallback reports
`l2` / `linf` (the quantities the reference's tests pin, e.g.
test/test_2d_euler_energy.jl:10-23): solution, node coordinates and the
Jacobian J = 1/inverse_jacobian are interpolated from the LGL nodes of degree
N to the LGL nodes of degree 2N (the default analysis polydeg); the exact
solution is evaluated there;
    l2   = sqrt( sum w_i w_j (w_k) J |u_exact - u|^2 / sum w_i w_j (w_k) J ),
    linf = max |u_exact - u|,
per variable.
"""
from __future__ import annotations

import numpy as np


def _lgl(N):
    import importlib
    import sys
    b = sys.modules.get("trixiatmo_gb300.basis") or importlib.import_module("trixiatmo_gb300.basis")
    return b


def error_norms(u, xyz, inv_jacobian, nodes, exact, ndims):
    """u[e, (k,) j, i, v], xyz[e, (k,) j, i, c], inv_jacobian[e, (k,) j, i];
    exact(x) -> u_exact[..., v]."""
    b = _lgl(None)
    N = len(nodes) - 1
    xa, wa = b.lgl_nodes_weights(2 * N)
    V = b.interpolation_matrix(np.asarray(nodes), xa)
    J = 1.0 / inv_jacobian
    if ndims == 2:
        def interp(f):
            return np.einsum("ai,bj,eji...->eba...", V, V, f, optimize=True)
        W = wa[:, None] * wa[None, :]
    else:
        def interp(f):
            return np.einsum("ai,bj,ck,ekji...->ecba...", V, V, V, f, optimize=True)
        W = wa[:, None, None] * wa[None, :, None] * wa[None, None, :]
    ua = interp(u)
    xa_ = interp(xyz)
    Ja = interp(J)
    diff = exact(xa_) - ua
    wJ = W[None] * Ja
    vol = wJ.sum()
    nv = u.shape[-1]
    l2 = np.sqrt((wJ[..., None] * diff * diff).reshape(-1, nv).sum(axis=0) / vol)
    linf = np.abs(diff).reshape(-1, u.shape[-1]).max(axis=0)
    return l2, linf
