"""Differentiable LP layer over the batched GPU engine.

``LpLayer`` solves a batch of LPs (one matrix per instance, or one shared matrix; each instance
its own cost and bounds) in one launch and makes two things differentiable with respect to
every instance's cost, lower and upper bounds (the LpProblem's computational form ``min c'v, [A -I] v = 0, l <= v <= u``; the
row entries of l and u are the row bounds, so for an equality row l = u = b):

* the optimal objective ``obj* = c'v*`` (PDLP to the requested tolerance, batched): by the
  envelope theorem ``dobj/dc = v*``, ``dobj/dl = max(d, 0)`` and ``dobj/du = min(d, 0)`` on
  finite bounds, with the reduced costs ``d = c + [A -I]' y*`` (so ``dobj/db = -y_i`` for an
  equality row: the reference's row dual, ``src/lp/pdlp.cpp:1167-1189``);
* the K-th iterate ``v_K`` of the fixed-step PDHG unrolled from zero (``sg_batch_unroll``),
  through the hand-written adjoint with checkpoints (``sg_batch_unroll_adjoint``).

Calling an ``LpLayer`` applies a ``torch.autograd.Function``: ``obj, v_star, v_K = layer(cost,
lower, upper)`` with (batch, n + m) float64 tensors; ``v_star`` is returned without a gradient.
The work runs in the CUDA library; torch carries the tensors and the chain rule.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .batch import BatchSolver
from .pdlp import FP64, OPTIMAL, REFERENCE, PdlpOptions


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class UnrolledPdhg:
    """K fixed-step PDHG iterations of every instance of a batch, and their adjoint.

    ``matrices`` and ``instances`` as for :class:`BatchSolver` (the batch must be FP64)."""

    def __init__(self, batch: BatchSolver, iterations: int = 2000, checkpoint_every: int = 64):
        if batch.options.precision != FP64:
            raise ValueError("the unrolled PDHG runs in FP64")
        self.batch = batch
        self.iterations = int(iterations)
        self.every = int(checkpoint_every)
        lib = batch._lib
        lib.sg_batch_unroll.restype = ctypes.c_int
        lib.sg_batch_unroll_adjoint.restype = ctypes.c_int
        self._lib = lib
        self.total = int(sum(batch.nt))

    def _check(self, rc, what):
        if rc != 0:
            self._lib.sg_batch_last_error.restype = ctypes.c_char_p
            raise _native.EngineError(rc, f"{what}: " +
                                      self._lib.sg_batch_last_error().decode())

    def forward(self) -> np.ndarray:
        """v_K of every instance, concatenated (n_i + m_i each), LpProblem space."""
        out = np.zeros(self.total)
        rc = self._lib.sg_batch_unroll(self.batch._h, ctypes.c_int(self.iterations),
                                       ctypes.c_int(self.every), _p(out))
        self._check(rc, "sg_batch_unroll")
        return out

    def adjoint(self, grad_v: np.ndarray):
        """(dL/dcost, dL/dlower, dL/dupper) for dL/dv_K = grad_v (concatenated layouts)."""
        g = np.ascontiguousarray(grad_v, dtype=np.float64)
        if g.size != self.total:
            raise ValueError(f"grad_v has {g.size} entries, expected {self.total}")
        gc = np.zeros(self.total)
        gl = np.zeros(self.total)
        gu = np.zeros(self.total)
        rc = self._lib.sg_batch_unroll_adjoint(self.batch._h, _p(g), _p(gc), _p(gl), _p(gu))
        self._check(rc, "sg_batch_unroll_adjoint")
        return gc, gl, gu


def reduced_costs(lp, cost, y):
    """d = c + [A -I]' y of an LpProblem (cost n + m, y m) = (c_x + A'y, c_r - y): the engine's
    PDHG is the saddle point of c'v + y'[A -I]v, so at the optimum d lies in minus the normal
    cone of the bounds at v*."""
    import scipy.sparse as sp
    A = sp.csc_matrix((lp.vals, lp.rowidx, lp.colptr), shape=(lp.m, lp.n))
    return np.concatenate([cost[:lp.n] + A.T @ y, cost[lp.n:] - y])


class LpLayer:
    """Batched LP layer. ``problems``: one LpProblem per instance (their matrices; every
    instance with the same n + m), or a single LpProblem whose matrix every instance shares.
    Each call brings every instance's cost, lower and upper. ``tol`` is the PDLP tolerance of
    the objective part; ``iterations`` / ``checkpoint_every`` define the unrolled part."""

    def __init__(self, problems, tol: float = 1e-8, iterations: int = 2000,
                 checkpoint_every: int = 64, algorithm: int = REFERENCE,
                 max_iterations: int = -1):
        self.shared = not isinstance(problems, (list, tuple))
        self.problems = [problems] if self.shared else list(problems)
        if len({p.n + p.m for p in self.problems}) != 1:
            raise ValueError("every instance must have the same n + m")
        self.tol = tol
        self.iterations = iterations
        self.every = checkpoint_every
        self.algorithm = algorithm
        self.max_iterations = max_iterations
        self._state = None
        self.last_status = None

    def _lp(self, b):
        return self.problems[0] if self.shared else self.problems[b]

    def _batch(self, cost, lower, upper):
        B = cost.shape[0]
        if not self.shared and B != len(self.problems):
            raise ValueError(f"{B} instances given, the layer has {len(self.problems)}")
        mats = [(p.m, p.n, p.colptr, p.rowidx, p.vals) for p in self.problems]
        inst = [(0 if self.shared else b, cost[b], lower[b], upper[b]) for b in range(B)]
        opts = PdlpOptions(tol=self.tol, precision=FP64, algorithm=self.algorithm,
                           max_iterations=self.max_iterations)
        return BatchSolver(mats, inst, opts)

    def evaluate(self, cost, lower, upper):
        """numpy forward: obj (B,), v* (B, n+m), y* (B, m), v_K (B, n+m), status (B,); keeps
        the batch for :meth:`vjp`."""
        cost = np.ascontiguousarray(cost, dtype=np.float64)
        lower = np.ascontiguousarray(lower, dtype=np.float64)
        upper = np.ascontiguousarray(upper, dtype=np.float64)
        B = cost.shape[0]
        self.close()
        batch = self._batch(cost, lower, upper)
        res = batch.solve()
        unroll = UnrolledPdhg(batch, self.iterations, self.every)
        vk = unroll.forward().reshape(B, -1)
        vstar = np.stack([r.x for r in res])
        ystar = np.stack([r.y for r in res])
        obj = np.einsum("bi,bi->b", cost, vstar)
        status = np.array([r.status for r in res])
        self.last_status = status
        self._state = (batch, unroll, cost, lower, upper, vstar, ystar)
        return obj, vstar, ystar, vk, status

    def vjp(self, grad_obj, grad_vk):
        """(dL/dcost, dL/dlower, dL/dupper), each (B, n+m), of the last :meth:`evaluate`."""
        batch, unroll, cost, lower, upper, vstar, ystar = self._state
        B = cost.shape[0]
        gobj = np.asarray(grad_obj, dtype=np.float64).reshape(B, 1)
        gc, gl, gu = unroll.adjoint(np.asarray(grad_vk, dtype=np.float64).reshape(-1))
        gc = gc.reshape(B, -1)
        gl = gl.reshape(B, -1)
        gu = gu.reshape(B, -1)
        d = np.stack([reduced_costs(self._lp(b), cost[b], ystar[b]) for b in range(B)])
        gc = gc + gobj * vstar
        gl = gl + gobj * np.where(np.isfinite(lower), np.maximum(d, 0.0), 0.0)
        gu = gu + gobj * np.where(np.isfinite(upper), np.minimum(d, 0.0), 0.0)
        return gc, gl, gu

    def close(self):
        st = getattr(self, "_state", None)
        if st is not None:
            st[0].close()
            self._state = None

    # torch front end --------------------------------------------------------------------
    def __call__(self, cost, lower, upper):
        import torch

        layer = self

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, c, lo, up):
                obj, vstar, _ystar, vk, _status = layer.evaluate(
                    c.detach().cpu().numpy(), lo.detach().cpu().numpy(),
                    up.detach().cpu().numpy())
                dev = c.device
                vstar_t = torch.from_numpy(vstar).to(dev)
                ctx.mark_non_differentiable(vstar_t)
                return (torch.from_numpy(obj).to(dev), vstar_t, torch.from_numpy(vk).to(dev))

            @staticmethod
            def backward(ctx, g_obj, _g_vstar, g_vk):
                B = g_vk.shape[0] if g_vk is not None else g_obj.shape[0]
                go = (g_obj.detach().cpu().numpy() if g_obj is not None
                      else np.zeros(B))
                gv = (g_vk.detach().cpu().numpy() if g_vk is not None
                      else np.zeros((B, layer._lp(0).n + layer._lp(0).m)))
                gc, gl, gu = layer.vjp(go, gv)
                dev = (g_vk if g_vk is not None else g_obj).device
                return (torch.from_numpy(gc).to(dev), torch.from_numpy(gl).to(dev),
                        torch.from_numpy(gu).to(dev))

        return _Fn.apply(cost, lower, upper)


def optimal(status) -> bool:
    return bool(np.all(np.asarray(status) == OPTIMAL))
