"""Float64 numpy reference for the adjoint tests (test infrastructure).

The forward update follows the tap table that the generator extracted from
the artifact's scop regions (<stencil>.c, e.g. j2d5pt.c:14-21,
gradient2d.c:14-23); the adjoint is derived from it by hand:
  * linear u'(x) = sum_k c_k u(x + o_k) / d: lam_t(y) = sum_k c_k/d lam_{t+1}(y - o_k),
    dL/dc_k += sum_x lam_{t+1}(x) u_t(x + o_k) / d;
  * gradient2d u'(x) = u(x) + c (eps + s(x))^{-1/2}, s = sum_n (u(x) - u(x+n))^2:
    dF(x)/du(x) = 1 - c g sum_n d_n, dF(x)/du(x+n) = c g d_n, g = (eps+s)^{-3/2},
    dL/dc += sum_x lam_{t+1}(x) (eps + s(x))^{-1/2}.
The halo is fixed, so its gradient accumulates over all steps."""
import json
from pathlib import Path

import numpy as np

TABLE = json.loads((Path(__file__).resolve().parent.parent / "an5d-artifact_gb300" / "gbstencil" /
                    "stencils.json").read_text())["stencils"]
BY_NAME = {s["name"]: s for s in TABLE}


def _sl(r, shape, off):
    """The interior, shifted by ``off``."""
    return tuple(slice(r + o, n - r + o) for o, n in zip(off, shape))


def default_coef(name):
    s = BY_NAME[name]
    if s["kind"] == "gradient":
        return np.array([s["numerator"]])
    return np.array([t["value"] for t in s["terms"]])


def step(name, u, coef):
    s = BY_NAME[name]
    r = s["rad"]
    out = u.copy()
    inner = _sl(r, u.shape, [0] * u.ndim)
    if s["kind"] == "gradient":
        c = u[inner]
        acc = np.full(c.shape, s["eps"])
        for n in s["neighbours"]:
            d = c - u[_sl(r, u.shape, n)]
            acc = acc + d * d
        out[inner] = c + coef[0] / np.sqrt(acc)
        return out
    acc = np.zeros(u[inner].shape)
    for k, t in enumerate(s["terms"]):
        acc = acc + coef[k] * u[_sl(r, u.shape, t["off"])]
    out[inner] = acc / (s["divisor"] or 1.0)
    return out


def forward(name, u0, coef, T):
    states = [np.asarray(u0, np.float64)]
    for _ in range(T):
        states.append(step(name, states[-1], coef))
    return states


def adjoint(name, u0, coef, T, lamT):
    """(dL/du_0 over the whole grid, dL/dcoef) for dL/du_T = lamT (halo ignored)."""
    s = BY_NAME[name]
    r = s["rad"]
    states = forward(name, u0, coef, T)
    shape = u0.shape
    zero = [0] * u0.ndim
    inner = _sl(r, shape, zero)
    mask = np.zeros(shape, bool)
    mask[inner] = True
    lam = np.where(mask, np.asarray(lamT, np.float64), 0.0)
    hg = np.zeros(shape)
    cg = np.zeros(len(coef))
    div = s["divisor"] or 1.0
    for t in range(T - 1, -1, -1):
        u = states[t]
        new = np.zeros(shape)
        lin = lam[inner]
        if s["kind"] == "gradient":
            c = u[inner]
            acc = np.full(c.shape, s["eps"])
            ds = []
            for n in s["neighbours"]:
                d = c - u[_sl(r, shape, n)]
                ds.append(d)
                acc = acc + d * d
            q = acc ** -0.5
            g = q ** 3 * coef[0]
            new[inner] += lin * (1 - g * sum(ds))
            for n, d in zip(s["neighbours"], ds):
                new[_sl(r, shape, n)] += lin * g * d
            cg[0] += np.sum(lin * q)
        else:
            for k, term in enumerate(s["terms"]):
                off = term["off"]
                new[_sl(r, shape, off)] += coef[k] / div * lin
                cg[k] += np.sum(lin * u[_sl(r, shape, off)]) / div
        hg += np.where(mask, 0.0, new)
        lam = np.where(mask, new, 0.0)
    return np.where(mask, lam, hg), cg


def loss(name, u0, coef, T, w):
    """L = sum over the interior of w * u_T (so dL/du_T = w)."""
    r = BY_NAME[name]["rad"]
    uT = forward(name, u0, coef, T)[-1]
    inner = _sl(r, uT.shape, [0] * uT.ndim)
    return float(np.sum(w[inner] * uT[inner]))
