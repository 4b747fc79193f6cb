"""Gradient of the stencil time loop: checkpointed forward, adjoint backward.

    uT = time_loop(u0, coef, "j2d5pt", timestep=1024, checkpoint_every=32)
    loss = (w * interior(uT, "j2d5pt")).sum()
    loss.backward()            # u0.grad (interior and halo), coef.grad

``u0`` is one time plane of shape ``dimsize`` (interior + halo) on the GPU,
float32 or float64; ``coef`` holds the update's coefficients as the source
writes them (before a divisor; gradient2d: its numerator), or None for the
source literals. Forward: gbs_adjoint_forward (the engine's time loop,
saving u_t every ``checkpoint_every`` steps). Backward: gbs_adjoint_backward
(recompute each chunk from its checkpoint with the engine, then the adjoint
step kernel backwards in time); with ``slots`` below 2 * checkpoint_every
(or a ``budget_bytes`` that forces it), gbs_adjoint_backward_slots reverses
each chunk by the binomial (revolve) schedule over that many snapshot
planes. ``forward_batch`` / ``backward_batch`` run many instances side by
side (gbs_adjoint_forward_batch / gbs_adjoint_backward_batch). There is no
CPU path: without the built engine every call raises.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi
from .grid import DeviceGrid


def _stream(device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class Checkpointed:
    """One forward run of the time loop with its checkpoints, ready for any
    number of backward passes (each with its own dL/du_T)."""

    def __init__(self, name: str, u0: torch.Tensor, timestep: int, checkpoint_every: int = 32,
                 coef=None, fp_mode: str = "fma", slots: int | None = None, budget_bytes: int | None = None,
                 run: bool = True):
        r = capi.info(name)["rad"]
        if u0.dtype not in (torch.float32, torch.float64):
            raise TypeError("u0 must be float32 or float64")
        dt = np.float32 if u0.dtype == torch.float32 else np.float64
        self.name = name
        self.grid = DeviceGrid(name, dt, [int(x) - 2 * r for x in u0.shape], device=u0.device)
        if list(u0.shape) != self.grid.dimsize:
            raise ValueError(f"u0 has shape {tuple(u0.shape)}, expected dimsize {tuple(self.grid.dimsize)}")
        self.grid.plane(0).copy_(u0.detach())
        self.grid.plane(1).copy_(self.grid.plane(0))
        if coef is not None and torch.is_tensor(coef):
            coef = coef.detach().cpu().numpy()
        self.desc, self._keep = self.grid.desc(int(timestep), fp_mode, coef=coef)
        L = capi.lib()
        if budget_bytes is not None:
            c, s = ctypes.c_int(0), ctypes.c_int(0)
            capi.check(L.gbs_adjoint_plan_budget(ctypes.byref(self.desc), int(budget_bytes), ctypes.byref(c),
                                                 ctypes.byref(s), None))
            checkpoint_every, slots = c.value, s.value
        self.checkpoint_every = int(checkpoint_every)
        self.slots = 2 * self.checkpoint_every if slots is None else int(slots)
        nbytes = ctypes.c_size_t(0)
        capi.check(L.gbs_adjoint_workspace_slots(ctypes.byref(self.desc), self.checkpoint_every, self.slots,
                                                 ctypes.byref(nbytes)))
        self.workspace_bytes = nbytes.value
        self.workspace = torch.empty(nbytes.value + 256, dtype=torch.uint8, device=u0.device)
        off = (-self.workspace.data_ptr()) % 256
        self._ws = ctypes.c_void_p(self.workspace.data_ptr() + off)
        if run:
            capi.check(L.gbs_adjoint_forward(ctypes.byref(self.desc), ctypes.c_void_p(self.grid.buf.data_ptr()),
                                             self.checkpoint_every, self._ws, _stream(u0.device)))

    @property
    def u_T(self) -> torch.Tensor:
        """View of u_T (shape dimsize) in the grid buffer."""
        return self.grid.plane(0)

    def _plane(self) -> tuple[torch.Tensor, torch.Tensor]:
        g = self.grid
        buf = torch.zeros(g.layout.plane, dtype=g.buf.dtype, device=g.device)
        L = g.layout
        v = buf.view(L.dimsize[0], L.pitch) if g.dim == 2 else buf.view(L.dimsize[0], L.dimsize[1], L.pitch)
        return buf, v[..., L.shift:L.shift + L.dimsize[g.dim - 1]]

    def backward(self, lam_T: torch.Tensor, want_coef: bool = True):
        """(dL/du_0, dL/dcoef or None) for dL/du_T = lam_T (shape dimsize;
        its halo is ignored). dL/dcoef is float64, one per term (gradient2d:
        one, for the numerator)."""
        g = self.grid
        lam_buf, lam_view = self._plane()
        lam_view.copy_(lam_T)
        out_buf, out_view = self._plane()
        cg = None
        if want_coef:
            s = capi.info(self.name)
            cg = torch.zeros(1 if s["kind"] == "gradient" else s["nterms"], dtype=torch.float64, device=g.device)
        capi.check(capi.lib().gbs_adjoint_backward_slots(
            ctypes.byref(self.desc), ctypes.c_void_p(lam_buf.data_ptr()), ctypes.c_void_p(out_buf.data_ptr()),
            ctypes.c_void_p(cg.data_ptr() if cg is not None else None),
            self.checkpoint_every, self.slots, self._ws, _stream(g.device)))
        return out_view, cg


def _ptrs(values):
    return (ctypes.c_void_p * len(values))(*[ctypes.c_void_p(v) if v else None for v in values])


def forward_batch(name_u0s, timestep, checkpoint_every=32, fp_mode="fma"):
    """Checkpointed forward runs of many instances at once
    (gbs_adjoint_forward_batch): ``name_u0s`` is a list of (stencil name,
    u0); one ``timestep`` and checkpoint interval for all. Returns the
    Checkpointed runs."""
    runs = [Checkpointed(n, u, timestep, checkpoint_every, fp_mode=fp_mode, run=False) for n, u in name_u0s]
    descs = (capi.Desc * len(runs))(*[r.desc for r in runs])
    capi.check(capi.lib().gbs_adjoint_forward_batch(
        descs, len(runs), _ptrs([r.grid.buf.data_ptr() for r in runs]), int(checkpoint_every),
        _ptrs([r._ws.value for r in runs]), _stream(runs[0].grid.device)))
    return runs


def backward_batch(runs, lam_Ts, want_coef=False):
    """dL/du_0 (and dL/dcoef) of every run at once
    (gbs_adjoint_backward_batch); one checkpoint interval for all."""
    planes, outs, cgs, keep = [], [], [], []
    for r, lam in zip(runs, lam_Ts):
        lb, lv = r._plane()
        lv.copy_(lam)
        ob, ov = r._plane()
        keep += [lb, ob]
        planes.append(lb.data_ptr())
        outs.append((ob, ov))
        if want_coef:
            s = capi.info(r.name)
            cgs.append(torch.zeros(1 if s["kind"] == "gradient" else s["nterms"], dtype=torch.float64,
                                   device=r.grid.device))
    descs = (capi.Desc * len(runs))(*[r.desc for r in runs])
    C = {r.checkpoint_every for r in runs}
    if len(C) != 1:
        raise ValueError("one checkpoint interval for the whole batch")
    capi.check(capi.lib().gbs_adjoint_backward_batch(
        descs, len(runs), _ptrs(planes), _ptrs([o[0].data_ptr() for o in outs]),
        _ptrs([c.data_ptr() for c in cgs]) if want_coef else None, C.pop(), _ptrs([r._ws.value for r in runs]),
        _stream(runs[0].grid.device)))
    return [o[1] for o in outs], (cgs if want_coef else None)


class TimeLoop(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, coef, name, timestep, checkpoint_every, fp_mode):
        run = Checkpointed(name, u0, timestep, checkpoint_every, coef=coef, fp_mode=fp_mode)
        ctx.run = run
        ctx.coef_dtype = None if coef is None else coef.dtype
        return run.u_T.clone()

    @staticmethod
    def backward(ctx, grad_uT):
        want = ctx.needs_input_grad[1]
        gu, gc = ctx.run.backward(grad_uT, want_coef=want)
        return gu.clone(), (gc.to(ctx.coef_dtype) if want else None), None, None, None, None


def time_loop(u0: torch.Tensor, coef: torch.Tensor | None, name: str, timestep: int,
              checkpoint_every: int = 32, fp_mode: str = "fma") -> torch.Tensor:
    """u_T of the stencil time loop from u_0 (one plane, interior + halo),
    differentiable with respect to u0 and coef."""
    return TimeLoop.apply(u0, coef, name, int(timestep), int(checkpoint_every), fp_mode)


def interior(x: torch.Tensor, name: str) -> torch.Tensor:
    r = capi.info(name)["rad"]
    return x[tuple(slice(r, -r) for _ in range(x.dim()))]
