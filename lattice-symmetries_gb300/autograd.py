"""Differentiable Hamiltonian matvec: y = H(theta) x with H(theta) = sum_c theta_c H_c.

`ParametrizedOperator(basis, [expr_0, expr_1, ...])` keeps the terms of every coupling H_c apart
(tagged with their coupling id) and exposes `apply(theta, x)`, a torch.autograd.Function whose
hand-written backward computes

    dL/dx       = H(theta)^dagger g            (the adjoint matvec: same gather kernel, adjoint
                                                term table, no atomics)
    dL/dtheta_c = Re <g, H_c x>                 (one fused pass over all couplings,
                                                ls_gpu_coupling_inner_products)

for g = dL/dy in PyTorch's convention for complex tensors (dL/dRe y + i dL/dIm y).  x is
complex128 on the GPU, [D] or [D, k]; theta is real.  No reference counterpart: the reference
has no gradients (its matvec is DistributedMatrixVector.chpl:1045-1105).
"""

from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import numpy as np

from . import _native as N
from ._api import Basis, Operator, split_terms
from ._expr import Expr, terms_to_arrays


class ParametrizedOperator:
    """H(theta) = sum_c theta_c H_c on one built basis."""

    def __init__(self, basis: Basis, expressions: Sequence[Expr], theta: Optional[Sequence[float]] = None):
        if len(expressions) == 0:
            raise ValueError("need at least one coupling")
        self.basis = basis
        self.expressions = list(expressions)
        offs, diags, cid_off, cid_diag = [], [], [], []
        self._per_coupling = []
        for c, e in enumerate(self.expressions):
            o, d = split_terms(basis, e)
            offs += o
            diags += d
            cid_off += [c] * len(o)
            cid_diag += [c] * len(d)
            self._per_coupling.append((o, d))
        self.number_couplings = len(self.expressions)
        self._cid_off = np.asarray(cid_off, dtype=np.int64)
        self._cid_diag = np.asarray(cid_diag, dtype=np.int64)
        # coupling id of every term: off-diagonal terms first, then diagonal ones (table order)
        self.term_coupling = np.ascontiguousarray(np.concatenate([self._cid_off, self._cid_diag]).astype(np.int32))
        self._unit_off = terms_to_arrays(offs)
        self._unit_diag = terms_to_arrays(diags)
        # H_c with theta = 1 for every c (the generators used by the gradient), and H(theta)
        self.generator = Operator._from_arrays(basis, self._unit_off, self._unit_diag)
        self.operator = Operator._from_arrays(basis, [a.copy() for a in self._unit_off],
                                              [a.copy() for a in self._unit_diag])
        self._sub = None
        self._lib = N.lib()
        self.theta = None
        self.set_theta(np.ones(self.number_couplings) if theta is None else theta)

    def set_theta(self, theta) -> None:
        """Rescales the coefficients of H(theta) in place (the library re-uploads changed terms)."""
        t = np.asarray(theta, dtype=np.float64).reshape(-1)
        if t.shape[0] != self.number_couplings:
            raise ValueError("expected {} coupling constants".format(self.number_couplings))
        if self.theta is not None and np.array_equal(t, self.theta):
            return
        self.operator._off_arrays[0][:] = self._unit_off[0] * t[self._cid_off] if len(self._cid_off) else 0
        self.operator._diag_arrays[0][:] = self._unit_diag[0] * t[self._cid_diag] if len(self._cid_diag) else 0
        self.theta = t.copy()

    def _sub_operators(self) -> List[Operator]:
        if self._sub is None:
            self._sub = [Operator._from_arrays(self.basis, terms_to_arrays(o), terms_to_arrays(d))
                         for o, d in self._per_coupling]
        return self._sub

    def coupling_products(self, g, x, fused: bool = True):
        """<g, H_c x> for every coupling c (complex128 tensor [n_couplings]; columns of [D, k]
        inputs are summed).  fused=True uses one pass over all couplings (bases with lattice
        symmetries of at most 128 elements and at most 4 couplings); otherwise, or when the fused
        kernel does not apply, one matvec per coupling followed by inner products."""
        import torch

        D = self.basis.number_states
        G = g.reshape(D, -1)
        X = x.reshape(D, -1)
        out = torch.zeros(self.number_couplings, dtype=torch.complex128, device=x.device)
        if fused:
            stream = torch.cuda.current_stream(x.device).cuda_stream
            buf = torch.empty(self.number_couplings, dtype=torch.complex128, device=x.device)
            tc = self.term_coupling.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
            ok = True
            for j in range(X.shape[1]):
                gj = G[:, j].contiguous()
                xj = X[:, j].contiguous()
                rc = self._lib.ls_gpu_coupling_inner_products(self.generator._payload, self.number_couplings, tc,
                                                              gj.data_ptr(), xj.data_ptr(), buf.data_ptr(), stream)
                if rc != 0:
                    N.take_errors()
                    ok = False
                    break
                out += buf
            if ok:
                N.check(self._lib.ls_gpu_check_errors(stream), "coupling products")
                return out
            out.zero_()
        for c, op in enumerate(self._sub_operators()):
            y = op.apply_device(X.contiguous())
            out[c] = torch.sum(G.conj() * y)
        return out

    def apply(self, theta, x):
        """y = H(theta) x, differentiable with respect to theta (real, [n_couplings]) and x."""
        import torch

        if not isinstance(theta, torch.Tensor):
            theta = torch.as_tensor(theta, dtype=torch.float64)
        if theta.dtype != torch.float64:
            raise TypeError("theta must be float64 (got {}): the couplings are used in double precision".format(
                theta.dtype))
        return _HApply.apply(theta, x, self)


def _make_function():
    import torch

    class _HApplyImpl(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, x, pop):
            if x.dtype != torch.complex128 or not x.is_cuda:
                raise TypeError("x must be a complex128 CUDA tensor")
            pop.set_theta(theta.detach().cpu().numpy())
            y = pop.operator.apply_device(x.contiguous())
            ctx.pop = pop
            ctx.save_for_backward(theta, x)
            return y

        @staticmethod
        def backward(ctx, gy):
            theta, x = ctx.saved_tensors
            pop = ctx.pop
            gtheta = gx = None
            if ctx.needs_input_grad[1]:
                pop.set_theta(theta.detach().cpu().numpy())
                gx = pop.operator.apply_device(gy.contiguous(), adjoint=True)
            if ctx.needs_input_grad[0]:
                cp = pop.coupling_products(gy, x)
                gtheta = cp.real.to(dtype=theta.dtype, device=theta.device)
            return gtheta, gx, None

    return _HApplyImpl


class _LazyFunction:
    _impl = None

    def apply(self, *args):
        if _LazyFunction._impl is None:
            _LazyFunction._impl = _make_function()
        return _LazyFunction._impl.apply(*args)


_HApply = _LazyFunction()
