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

    The forward, VJP and fused loops are built once, on the first call that
    needs them, over Dats that wrap the call's tensors; later calls rebind
    those Dats to their own tensors (no copy) and launch the built loops, so
    a call costs a launch, not a loop construction.
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
        self._loops = {}       # "forward" / "vjp" / "fused" -> (ParLoop, Dats to rebind)

    def _shape(self, dataset):
        return (dataset.total_size,) + (() if dataset.cdim == 1 else tuple(dataset.dim))

    def _zeros(self, dataset):
        return torch.zeros(self._shape(dataset), dtype=torch.float64, device=device.device())

    def _const_args(self):
        return [d(READ, m) if m is not None else d(READ) for d, m in self.constants]

    def _run(self, which, tensors, build):
        """Launch loop `which` on `tensors` (one per Dat it rebinds, in the
        order `build` created them); `build(dats)` returns its arguments."""
        hit = self._loops.get(which)
        if hit is None:
            from pyop2_gb300.parloop import ParLoop
            specs = self._specs(which)
            dats = [Dat.from_tensor(ds, t) for (ds, _), t in zip(specs, tensors)]
            knl = {"forward": self.kernel, "vjp": self.vjp_kernel,
                   "fused": self.fused_kernel}[which]
            hit = (ParLoop(knl, self.iterset, *build(dats)), dats)
            self._loops[which] = hit
        else:
            for d, t in zip(hit[1], tensors):
                d._rebind(t)
        hit[0].compute()

    def _specs(self, which):
        """(dataset, map) of every rebound Dat of loop `which`, in order."""
        out = [self.output]
        if which == "fused":
            out = [self.output, self.output]          # F, lambda
        elif which == "vjp":
            out = [self.output]                       # lambda
        return out + self.inputs + ([] if which == "forward" else self.inputs)

    def _input_args(self, dats):
        return [d(READ, m) if m is not None else d(READ) for (_, m), d in zip(self.inputs, dats)]

    def _grad_args(self, dats):
        return [d(INC, m) if m is not None else d(WRITE) for (_, m), d in zip(self.inputs, dats)]

    def forward_values(self, *xs):
        """Residual for inputs xs (no autograd)."""
        F = self._zeros(self.output[0])
        omap = self.output[1]
        n = len(self.inputs)
        self._run("forward", [F] + [x.detach().contiguous() for x in xs],
                  lambda d: [d[0](INC, omap), *self._const_args(), *self._input_args(d[1:1 + n])])
        return F

    def vjp(self, lam, *xs):
        """Gradients of lam . F with respect to every input."""
        grads = [self._zeros(ds) for ds, _ in self.inputs]
        omap = self.output[1]
        n = len(self.inputs)
        self._run("vjp", [lam.detach().contiguous()] + [x.detach().contiguous() for x in xs] +
                  grads,
                  lambda d: [d[0](READ, omap), *self._const_args(),
                             *self._input_args(d[1:1 + n]), *self._grad_args(d[1 + n:])])
        return grads

    def fused(self, lam, *xs):
        """Residual and the gradients of lam . F in one pass."""
        if self.fused_kernel is None:
            raise ValueError("no fused kernel given")
        F = self._zeros(self.output[0])
        grads = [self._zeros(ds) for ds, _ in self.inputs]
        omap = self.output[1]
        n = len(self.inputs)
        self._run("fused", [F, lam.detach().contiguous()] +
                  [x.detach().contiguous() for x in xs] + grads,
                  lambda d: [d[0](INC, omap), d[1](READ, omap), *self._const_args(),
                             *self._input_args(d[2:2 + n]), *self._grad_args(d[2 + n:])])
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
