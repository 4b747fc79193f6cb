"""Device-resident grids in the engine's layout.

PyTorch supplies the device memory and the stream; the engine
(``libgbstencil.so``) does the work. A ``DeviceGrid`` owns one two-plane
buffer laid out as ``gbs_get_layout`` prescribes (rows padded to ``pitch``
elements, column c at element ``shift + c``) and exposes each time plane as a
strided torch view of shape ``dimsize``.
"""
from __future__ import annotations

import numpy as np
import torch

from . import capi

TORCH_DT = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}


class DeviceGrid:
    def __init__(self, name: str, dtype, n, device=None):
        self.name = name
        self.dtype = np.dtype(dtype)
        s = capi.info(name)
        self.dim, self.rad = s["dim"], s["rad"]
        self.n = [int(n)] * self.dim if np.isscalar(n) else [int(x) for x in n]
        d, _ = capi.make_desc(name, self.dtype, self.n, 0)
        self.layout = capi.layout(d)
        es = self.dtype.itemsize
        self.device = torch.device(device or "cuda")
        self.buf = torch.zeros(self.layout.bytes // es, dtype=TORCH_DT[self.dtype], device=self.device)
        assert self.buf.data_ptr() % 128 == 0

    @property
    def dimsize(self):
        return [self.layout.dimsize[a] for a in range(self.dim)]

    def plane(self, p: int) -> torch.Tensor:
        """Strided view of time plane p with shape dimsize."""
        L = self.layout
        flat = self.buf[p * L.plane:(p + 1) * L.plane]
        if self.dim == 2:
            v = flat.view(L.dimsize[0], L.pitch)
        else:
            v = flat.view(L.dimsize[0], L.dimsize[1], L.pitch)
        return v[..., L.shift:L.shift + L.dimsize[self.dim - 1]]

    def desc(self, timestep, fp_mode="fma", bt=0, sl=0, coef=None, divisor=0.0, eps=0.0, bs1=0):
        return capi.make_desc(self.name, self.dtype, self.n, timestep, fp_mode, bt, sl, bs1=bs1,
                              coef=coef, divisor=divisor, eps=eps)

    def upload(self, host: np.ndarray, stream: int | None = None):
        d, _ = self.desc(0)
        host = np.ascontiguousarray(host, dtype=self.dtype)
        s = torch.cuda.current_stream(self.device).cuda_stream if stream is None else stream
        capi.upload(d, host.ctypes.data, self.buf.data_ptr(), s)
        torch.cuda.current_stream(self.device).synchronize() if stream is None else None

    def download(self, host: np.ndarray | None = None, stream: int | None = None) -> np.ndarray:
        d, _ = self.desc(0)
        if host is None:
            host = np.empty((2,) + tuple(self.dimsize), self.dtype)
        s = torch.cuda.current_stream(self.device).cuda_stream if stream is None else stream
        capi.download(d, self.buf.data_ptr(), host.ctypes.data, s)
        torch.cuda.current_stream(self.device).synchronize() if stream is None else None
        return host

    def fill_uniform(self, seed: int = 0):
        """Interior and halo i.i.d. U[0,1) (seeded), both planes equal."""
        g = torch.Generator(device=self.device)
        g.manual_seed(seed)
        p0 = self.plane(0)
        p0.copy_(torch.rand(p0.shape, generator=g, device=self.device, dtype=p0.dtype))
        self.plane(1).copy_(p0)

    def run(self, timestep: int, fp_mode="fma", bt=0, sl=0, coef=None, divisor=0.0, eps=0.0,
            stream: int | None = None, bs1=0):
        """Enqueues the time loop on ``stream`` (default: torch's current)."""
        d, keep = self.desc(timestep, fp_mode, bt, sl, coef, divisor, eps, bs1)
        s = torch.cuda.current_stream(self.device).cuda_stream if stream is None else stream
        capi.run_device(d, self.buf.data_ptr(), s)
        return keep
