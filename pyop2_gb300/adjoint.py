"""Differentiable par_loops: a residual loop with a hand-written
vector-Jacobian product, exposed as a torch.autograd.Function.

The forward runs the user's residual kernel as an INC par_loop into the
output.  The backward, given the adjoint vector lambda (the incoming
gradient), runs the user's VJP kernel as a second par_loop: lambda is
*gathered* through the output's map (the forward's INC scatter, transposed),
the element data are gathered again (recomputed, not stored), and the VJP's
contributions are INC-scattered into the gradients of the inputs that live
behind a map, or written directly for per-cell inputs.  There is no
counterpart in the reference (it has no adjoint).

Kernel argument conventions:
    forward(F, *constants, *inputs)
    vjp(lambda, *constants, *inputs, *grads)      grads in the order of inputs
    fused(F, lambda, *constants, *inputs, *grads) (optional, both in one pass)
"""
import torch

from pyop2_gb300 import device
from pyop2_gb300.types.access import INC, READ, WRITE
from pyop2_gb300.types.dat import Dat


class AdjointParLoop:
    """``AdjointParLoop(iterset, kernel, vjp_kernel, output, inputs, constants=())``

    output: (dataset, map) of the residual;
    inputs: list of (dataset, map or None) of the differentiable inputs;
    constants: list of (Dat, map or None) read-only, not differentiated.
    Call it with one torch tensor per input; it returns the residual tensor
    and is differentiable with respect to every input.
    """

    def __init__(self, iterset, kernel, vjp_kernel, output, inputs, constants=(),
                 fused_kernel=None):
        self.iterset = iterset
        self.kernel = kernel
        self.vjp_kernel = vjp_kernel
        self.fused_kernel = fused_kernel
        self.output = output
        self.inputs = list(inputs)
        self.constants = list(constants)

    def _shape(self, dataset):
        return (dataset.total_size,) + (() if dataset.cdim == 1 else tuple(dataset.dim))

    def _wrap(self, dataset, t):
        return Dat.from_tensor(dataset, t.contiguous())

    def _const_args(self):
        return [d(READ, m) if m is not None else d(READ) for d, m in self.constants]

    def _input_args(self, xs):
        out = []
        for (ds, m), x in zip(self.inputs, xs):
            d = self._wrap(ds, x.detach())
            out.append(d(READ, m) if m is not None else d(READ))
        return out

    def _grad_args(self, grads):
        out = []
        for (ds, m), g in zip(self.inputs, grads):
            d = self._wrap(ds, g)
            out.append(d(INC, m) if m is not None else d(WRITE))
        return out

    def forward_values(self, *xs):
        """Residual for inputs xs (no autograd)."""
        from pyop2_gb300.parloop import par_loop
        ods, omap = self.output
        F = torch.zeros(self._shape(ods), dtype=torch.float64, device=device.device())
        Fd = self._wrap(ods, F)
        par_loop(self.kernel, self.iterset, Fd(INC, omap), *self._const_args(),
                 *self._input_args(xs))
        return F

    def vjp(self, lam, *xs):
        """Gradients of lam . F with respect to every input."""
        from pyop2_gb300.parloop import par_loop
        ods, omap = self.output
        grads = [torch.zeros(self._shape(ds), dtype=torch.float64, device=device.device())
                 for ds, _ in self.inputs]
        ld = self._wrap(ods, lam.detach())
        par_loop(self.vjp_kernel, self.iterset, ld(READ, omap), *self._const_args(),
                 *self._input_args(xs), *self._grad_args(grads))
        return grads

    def fused(self, lam, *xs):
        """Residual and the gradients of lam . F in one pass."""
        from pyop2_gb300.parloop import par_loop
        if self.fused_kernel is None:
            raise ValueError("no fused kernel given")
        ods, omap = self.output
        F = torch.zeros(self._shape(ods), dtype=torch.float64, device=device.device())
        grads = [torch.zeros(self._shape(ds), dtype=torch.float64, device=device.device())
                 for ds, _ in self.inputs]
        ld = self._wrap(ods, lam.detach())
        par_loop(self.fused_kernel, self.iterset, self._wrap(ods, F)(INC, omap), ld(READ, omap),
                 *self._const_args(), *self._input_args(xs), *self._grad_args(grads))
        return F, grads

    def __call__(self, *xs):
        return _ParLoopFunction.apply(self, *xs)


class _ParLoopFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, loop, *xs):
        ctx.loop = loop
        ctx.save_for_backward(*xs)
        return loop.forward_values(*xs)

    @staticmethod
    def backward(ctx, lam):
        xs = ctx.saved_tensors
        grads = ctx.loop.vjp(lam.contiguous(), *xs)
        return (None,) + tuple(grads)
