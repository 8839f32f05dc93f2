"""ORACLE — test infrastructure only.

NumPy restatement of the output conversions that SaveSolutionCallback applies
before writing a solution file, for the covariant shallow-water equations:

* cons2cons  (h, h_vcon1, h_vcon2)   src/equations/covariant_shallow_water.jl:83-85
* cons2prim  (H, vcon1, vcon2), H = h + b     :88-90, :113-118
* contravariant2global (h, h_v1, h_v2, h_v3) = (h, A (h_vcon1, h_vcon2))   :97-100, :140-145
* cons2prim_and_vorticity (H, v1, v2, v3, b, zeta)
      src/callbacks_step/save_solution_covariant.jl:64-74, with the relative
      vorticity zeta = (d v_2/d xi^1 - d v_1/d xi^2) / J of
      calc_vorticity_node :93-118, v_k = G_kl v^l the covariant velocity,
      derivatives by the nodal derivative matrix along the node's grid lines.

The auxiliary slots follow src/equations/equations.jl:210-244 (0-based: 0-5
the covariant basis A with columns a_1 = slots 0-2 and a_2 = slots 3-5, 12 the
area element J, 13-15 the covariant metric G_11, G_12, G_22, 19 the bottom
topography b).  The derivative matrix is built here from the nodes with the
barycentric formula (D_ij = (l_j / l_i) / (x_i - x_j), D_ii = -sum_j D_ij;
Berrut & Trefethen, SIAM Review 46 (2004) 501-517), independently of the
product's basis.

Arrays: u[e, j, i, 3], aux[e, j, i, 26]; each result is [n_vars, E n n] with
rows in Julia node order (i fastest, then j, then element).
"""
from __future__ import annotations

import numpy as np


def derivative_matrix(nodes):
    x = np.asarray(nodes, dtype=np.float64)
    n = len(x)
    lam = np.array([1.0 / np.prod([x[i] - x[j] for j in range(n) if j != i]) for i in range(n)])
    D = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            if i != j:
                D[i, j] = (lam[j] / lam[i]) / (x[i] - x[j])
        D[i, i] = -D[i].sum()
    return D


def covariant_rows(u, aux, nodes, kind):
    """kind 0 cons2cons, 1 cons2prim, 2 contravariant2global,
    3 cons2prim_and_vorticity."""
    u = np.asarray(u, dtype=np.float64)
    a = np.asarray(aux, dtype=np.float64)
    h, m1, m2 = u[..., 0], u[..., 1], u[..., 2]
    b = a[..., 19]
    if kind == 0:
        rows = [h, m1, m2]
    elif kind == 1:
        rows = [h + b, m1 / h, m2 / h]
    elif kind == 2:
        rows = [h] + [a[..., c] * m1 + a[..., 3 + c] * m2 for c in range(3)]
    elif kind == 3:
        c1, c2 = m1 / h, m2 / h
        w1 = a[..., 13] * c1 + a[..., 14] * c2
        w2 = a[..., 14] * c1 + a[..., 15] * c2
        D = derivative_matrix(nodes)
        d21 = np.einsum("ik,ejk->eji", D, w2)   # along xi^1 (index i)
        d12 = np.einsum("jk,eki->eji", D, w1)   # along xi^2 (index j)
        zeta = (d21 - d12) / a[..., 12]
        rows = ([h + b] + [a[..., c] * c1 + a[..., 3 + c] * c2 for c in range(3)] + [b, zeta])
    else:
        raise ValueError(kind)
    return np.stack([r.reshape(-1) for r in rows])
