"""ORACLE — test infrastructure only.

CPU restatement of the differentiable layer's unrolled PDHG and of its adjoint, for the parity
tests of ``sg_batch_unroll`` / ``sg_batch_unroll_adjoint``. Only ``tests/`` import it.

The forward map is the reference's fixed-step PDHG (``src/lp/pdlp.cpp:574-641``: extrapolation
v_bar = 2 v - v_prev, dual step on [A -I] v_bar, projected primal step) with tau = sigma =
0.99 / L and primal weight 1, run for K iterations from zero on the problem equilibrated by the
reference's Ruiz scaling (``pdlp.cpp:109-187``) with L from its power iteration
(``pdlp.cpp:36-103``) — both taken from ``oracle.setup`` (the C restatement pinned to the
reference). The iterations themselves are ``oracle.pdhg_steps``. The adjoint is the transpose
of that map, restated here in numpy with scipy sparse products: per iteration, backwards,

    V = v_hat + 2 b_hat;  z_hat = [l < z < u] V;  l_hat += [z <= l] V;  u_hat += [z >= u] V
    v_hat <- z_hat - b_hat;  g_hat = -tau z_hat;  c_hat += g_hat
    y_hat <- y_hat + [A -I] g_hat;  b_hat <- [A -I]' (sigma y_hat)

for the state (v, v_bar, y) and the projection input z = v - tau (c + [A -I]' y+).
"""
from __future__ import annotations

import numpy as np

from . import oracle as _o


class UnrolledPdhg:
    """The unrolled map of one LpProblem (m, n, CSC colptr/rowidx/vals; cost/lower/upper of
    length n + m)."""

    def __init__(self, m, n, colptr, rowidx, vals):
        import scipy.sparse as sp
        self.m, self.n = m, n
        self.colptr = np.asarray(colptr, dtype=np.int64)
        self.rowidx = np.asarray(rowidx, dtype=np.int32)
        rs, cs, aeq, _ateq, L = _o.setup(m, n, self.colptr, self.rowidx, vals)
        self.rs, self.cs, self.aeq = rs, cs, aeq
        self.eta = 0.99 / L
        self.A = sp.csc_matrix((aeq, self.rowidx, self.colptr), shape=(m, n))

    def _scaled(self, cost, lower, upper):
        n = self.n
        s_c = np.concatenate([self.cs, self.rs])
        s_b = np.concatenate([1.0 / self.cs, self.rs])
        return cost * s_c, lower * s_b, upper * s_b

    def forward(self, cost, lower, upper, iterations):
        """v_K in the LpProblem's space (x = x_eq cs, r = r_eq / rs)."""
        m, n = self.m, self.n
        c, l, u = self._scaled(cost, lower, upper)
        st = {"v": np.zeros(n + m), "v_prev": np.zeros(n + m), "y": np.zeros(m),
              "v_erg": np.zeros(n + m), "y_erg": np.zeros(m)}
        st = _o.pdhg_steps(m, n, self.colptr, self.rowidx, self.aeq, c, l, u, self.eta,
                           self.eta, iterations, 0, st)
        v = st["v"]
        return np.concatenate([v[:n] * self.cs, v[n:] / self.rs])

    def _K(self, v):
        return self.A @ v[:self.n] - v[self.n:]

    def _Kt(self, y):
        return np.concatenate([self.A.T @ y, -y])

    def adjoint(self, cost, lower, upper, iterations, grad_v):
        """dL/dcost, dL/dlower, dL/dupper (LpProblem space) for dL/dv_K = grad_v."""
        m, n = self.m, self.n
        tau = sigma = self.eta
        c, l, u = self._scaled(cost, lower, upper)
        # Forward, keeping the projection inputs.
        v = np.zeros(n + m)
        vbar = np.zeros(n + m)
        y = np.zeros(m)
        zs = []
        for _ in range(iterations):
            y = y + sigma * self._K(vbar)
            z = v - tau * (c + self._Kt(y))
            zs.append(z)
            vn = np.minimum(np.maximum(z, l), u)
            vbar = 2.0 * vn - v
            v = vn
        vh = np.concatenate([grad_v[:n] * self.cs, grad_v[n:] / self.rs])
        bh = np.zeros(n + m)
        yh = np.zeros(m)
        gc = np.zeros(n + m)
        gl = np.zeros(n + m)
        gu = np.zeros(n + m)
        for z in reversed(zs):
            V = vh + 2.0 * bh
            at_l = z <= l
            at_u = (z >= u) & ~at_l
            inside = ~(at_l | at_u)
            zh = np.where(inside, V, 0.0)
            gl += np.where(at_l, V, 0.0)
            gu += np.where(at_u, V, 0.0)
            vh = zh - bh
            gh = -tau * zh
            gc += gh
            yh = yh + self._K(gh)
            bh = self._Kt(sigma * yh)
        s_c = np.concatenate([self.cs, self.rs])
        s_b = np.concatenate([1.0 / self.cs, self.rs])
        return gc * s_c, gl * s_b, gu * s_b
