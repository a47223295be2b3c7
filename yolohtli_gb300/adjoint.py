"""Gradients of a probe loss with respect to the diffusion map D(x, y) and
the 13 FK3V parameters (yh_adjoint_* in include/yolohtli.h), and a
torch.autograd.Function over them: `loss = probe_loss(D, adjoint, state0,
fk)` then `loss.backward()` fills D.grad (and fk.grad, a float64 tensor of
the 13 parameters in yh_fk_params order) with the adjoint's gradients."""
import ctypes as C

import numpy as np

from . import _abi as A
from ._loader import load
from .ops import check


def _after_torch():
    """The handle runs on its own stream: inputs that torch is still
    writing on its current stream must be complete first."""
    try:
        import torch
        if torch.cuda.is_available() and torch.cuda.is_initialized():
            torch.cuda.current_stream().synchronize()
    except ImportError:
        pass


class Adjoint:
    """One FK3V problem: grid and parameters p (hx == hy), the FK3V
    parameters, nsteps steps, the loss on the states after every
    frame_steps steps at a probe lattice every probe_spacing cells,
    checkpoints every checkpoint_steps (default ~sqrt(nsteps); 1 keeps
    every state); smooth > 0 replaces the model's switches by tanh ramps of
    that width. batch > 1: that many instances with their own D, initial
    state and target, one launch per step for all (every per-instance
    tensor is then batch arrays one after another)."""

    def __init__(self, p, fk, nsteps, frame_steps, probe_spacing,
                 checkpoint_steps=None, fp64=False, smooth=0.0, stream=None,
                 batch=1):
        self.lib = load()
        self.p = p.copy()
        self.batch = int(batch)
        if checkpoint_steps is None:
            checkpoint_steps = max(1, int(round(np.sqrt(nsteps))))
        h = C.c_void_p()
        check("yh_adjoint_create_batch", self.lib.yh_adjoint_create_batch(
            C.byref(self.p), C.byref(fk), self.batch, int(nsteps),
            int(frame_steps), int(probe_spacing), int(checkpoint_steps),
            1 if fp64 else 0, float(smooth),
            C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h
        self.fk = A.FKParams.from_buffer_copy(fk)
        f, px, py = C.c_int(), C.c_int(), C.c_int()
        check("yh_adjoint_probes", self.lib.yh_adjoint_probes(
            h, C.byref(f), C.byref(px), C.byref(py)))
        self.frames, self.probes_x, self.probes_y = f.value, px.value, py.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.yh_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def target_shape(self):
        one = (self.frames, self.probes_y, self.probes_x)
        return one if self.batch == 1 else (self.batch,) + one

    def set_target(self, target):
        """target: a device tensor or host array of target_shape floats."""
        ptr = target.data_ptr() if hasattr(target, "data_ptr") else \
            np.ascontiguousarray(target, dtype=np.float32).ctypes.data
        _after_torch()
        check("yh_adjoint_set_target", self.lib.yh_adjoint_set_target(self.h, ptr))

    def record(self, D, state0, out):
        """Probe values of a forward run into `out` (device float32)."""
        _after_torch()
        check("yh_adjoint_record", self.lib.yh_adjoint_record(
            self.h, D.data_ptr(), *[x.data_ptr() for x in state0],
            out.data_ptr()))

    def set_fk(self, fk):
        """New FK3V parameters (an A.FKParams) for the following runs."""
        check("yh_adjoint_set_fk", self.lib.yh_adjoint_set_fk(self.h, C.byref(fk)))
        self.fk = A.FKParams.from_buffer_copy(fk)

    def run(self, D, state0, grad=None, grad_fk=None):
        """Loss and, with `grad` (device float32 like D), dLoss/dD; with
        grad_fk also dLoss/d(each FK parameter): an A.FKParams (batch 1) or
        an array of `batch` of them. The loss is a float (batch 1) or an
        array of one per instance."""
        loss = (C.c_double * self.batch)()
        _after_torch()
        g = grad.data_ptr() if grad is not None else None
        x = [D.data_ptr()] + [t.data_ptr() for t in state0]
        if grad_fk is not None:
            ref = C.byref(grad_fk) if isinstance(grad_fk, A.FKParams) else grad_fk
            check("yh_adjoint_run_fk", self.lib.yh_adjoint_run_fk(
                self.h, *x, loss, g, ref))
        else:
            check("yh_adjoint_run", self.lib.yh_adjoint_run(self.h, *x, loss, g))
        return loss[0] if self.batch == 1 else np.array(loss[:])


def fk_array(fk):
    """The 13 FK3V parameters of an A.FKParams as a float64 array."""
    return np.array([getattr(fk, n) for n in A.FK_NAMES], np.float64)


def fk_struct(x):
    """An A.FKParams from 13 values in yh_fk_params order."""
    f = A.FKParams()
    for n, v in zip(A.FK_NAMES, np.asarray(x, np.float64).tolist()):
        setattr(f, n, v)
    return f


def _make_function():
    import torch

    class ProbeLoss(torch.autograd.Function):
        """loss = ProbeLoss.apply(D, fk, adjoint, state0): D a float32 CUDA
        tensor of nx*ny, fk None or a float64 tensor of the 13 FK3V
        parameters (the handle is switched to them when they differ),
        state0 (u0, v0, w0) float32 CUDA tensors."""

        @staticmethod
        def forward(ctx, D, fk, adjoint, state0):
            D = D.contiguous()
            state0 = [x.contiguous() for x in state0]
            grad = torch.empty_like(D)
            gfk = None
            if fk is not None:
                want = fk.detach().cpu().double().numpy()
                if not np.array_equal(want, fk_array(adjoint.fk)):
                    adjoint.set_fk(fk_struct(want))
                gfk = A.FKParams()
            loss = adjoint.run(D, state0, grad, gfk)
            ctx.save_for_backward(grad)
            ctx.gfk = None if gfk is None else torch.tensor(
                fk_array(gfk), dtype=fk.dtype, device=fk.device)
            return torch.tensor(loss, dtype=torch.float64, device=D.device)

        @staticmethod
        def backward(ctx, g):
            (grad,) = ctx.saved_tensors
            gfk = None if ctx.gfk is None else g.to(ctx.gfk.dtype).to(ctx.gfk.device) * ctx.gfk
            return (g.to(grad.dtype) * grad, gfk, None, None)

    return ProbeLoss


_fn = None


def probe_loss(D, adjoint, state0, fk=None):
    """The probe loss as a differentiable function of D (and, when given,
    of the FK3V parameters fk: a float64 tensor of 13)."""
    global _fn
    if _fn is None:
        _fn = _make_function()
    return _fn.apply(D, fk, adjoint, state0)


def fit(adjoint, D, state0, fk, iters=20, lr=0.02, fit_fk=True,
        betas=(0.9, 0.999), eps=1e-8):
    """Parameter estimation with the adjoint's gradients: Adam on the
    logarithm of the diffusion map D (every cell of every instance) and of
    the 13 FK3V parameters, which the handle's instances share (their
    gradients are summed). The second moments are shared: one number per
    instance for its D field (the mean over its cells) and one for the 13
    parameters, so that a cell or a parameter moves in proportion to its
    gradient; a per-value second moment would move the cells the probes do
    not see, and the parameters the loss hardly depends on, as far as any
    other, which made the loss climb again at 10,000 steps. One iteration
    is one batched loss-and-gradient evaluation of all instances. D: float32 CUDA tensor (batch x cells),
    modified in place; fk: 13 values (yh_fk_params order). Returns
    (fk as an array, losses): losses[i] is the per-instance loss before
    iteration i, with one more row for the final estimate."""
    import torch
    b = adjoint.batch
    th = np.asarray(fk, np.float64).copy()
    logD = torch.log(D.double())
    mD = torch.zeros_like(logD)
    vD = torch.zeros(b, 1, dtype=torch.float64, device=D.device)
    mt, vt = np.zeros(13), 0.0
    g = torch.empty_like(D)
    gfk = (A.FKParams * b)()
    losses = []
    for it in range(iters + 1):
        adjoint.set_fk(fk_struct(th))
        D.copy_(torch.exp(logD).float())
        loss = adjoint.run(D, state0, g, gfk)
        losses.append(np.atleast_1d(loss).astype(np.float64))
        if it == iters:
            break
        # gradients with respect to the logarithms
        gD = g.double() * D.double()
        gt = sum(fk_array(gfk[k]) for k in range(b)) * th
        k1 = it + 1
        mD.mul_(betas[0]).add_(gD, alpha=1 - betas[0])
        vD.mul_(betas[1]).add_((gD * gD).view(b, -1).mean(dim=1, keepdim=True),
                               alpha=1 - betas[1])
        step = (mD / (1 - betas[0] ** k1)).view(b, -1) / (
            torch.sqrt(vD / (1 - betas[1] ** k1)) + eps)
        logD -= lr * step.view(-1)
        if fit_fk:
            mt = betas[0] * mt + (1 - betas[0]) * gt
            vt = betas[1] * vt + (1 - betas[1]) * float(np.mean(gt * gt))
            th = th * np.exp(-lr * (mt / (1 - betas[0] ** k1)) / (
                np.sqrt(vt / (1 - betas[1] ** k1)) + eps))
    return th, np.array(losses)
