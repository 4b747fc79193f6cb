"""Adjoint of the time loop (gbs_adjoint_forward / gbs_adjoint_backward and
the torch.autograd.Function over them).

CPU: the float64 numpy adjoint (adjoint_ref.py) against central finite
differences of the numpy forward loop. GPU: the engine's adjoint against
that reference (normwise relative error <= 1e-4 for float32, 1e-9 for
float64), directional finite differences of the engine's own forward loop
in float64, the autograd wrapper, and argument checking."""
import ctypes

import numpy as np
import pytest

import adjoint_ref as ar

RNG = np.random.default_rng


def _inputs(name, n, seed):
    s = ar.BY_NAME[name]
    shape = [n + 2 * s["rad"]] * s["dim"]
    rng = RNG(seed)
    u0 = rng.random(shape)
    w = rng.standard_normal(shape)
    return u0, w


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


# ---------------------------------------------------------------- CPU -----
@pytest.mark.parametrize("name,n,T", [("j2d5pt", 10, 6), ("star2d2r", 9, 4), ("box2d1r", 8, 5),
                                      ("star3d1r", 6, 3), ("j3d27pt", 5, 3), ("gradient2d", 8, 4)])
def test_reference_adjoint_matches_finite_differences(name, n, T):
    u0, w = _inputs(name, n, 1)
    coef = ar.default_coef(name)
    gu, gc = ar.adjoint(name, u0, coef, T, w)
    rng = RNG(2)
    h = 1e-6
    for _ in range(3):
        du = rng.standard_normal(u0.shape)
        fd = (ar.loss(name, u0 + h * du, coef, T, w) - ar.loss(name, u0 - h * du, coef, T, w)) / (2 * h)
        assert abs(fd - np.sum(gu * du)) <= 1e-6 * max(1.0, abs(fd))
        dc = rng.standard_normal(coef.shape)
        fd = (ar.loss(name, u0, coef + h * dc, T, w) - ar.loss(name, u0, coef - h * dc, T, w)) / (2 * h)
        assert abs(fd - np.sum(gc * dc)) <= 1e-6 * max(1.0, abs(fd))


def test_adjoint_symbols_declared():
    text = (ar.Path(__file__).resolve().parent.parent / "include" / "gbstencil.h").read_text()
    for sym in ("gbs_adjoint_workspace", "gbs_adjoint_forward", "gbs_adjoint_backward"):
        assert sym + "(" in text


# ---------------------------------------------------------------- GPU -----
CASES = [
    # name, dtype, n, T, checkpoint interval
    ("j2d5pt", np.float32, 40, 10, 3),
    ("j2d5pt", np.float64, 33, 9, 1),
    ("j2d5pt", np.float64, 33, 9, 32),
    ("star2d1r", np.float32, 37, 8, 4),
    ("star2d3r", np.float64, 30, 7, 2),
    ("box2d2r", np.float32, 28, 6, 5),
    ("j2d9pt", np.float64, 31, 6, 4),
    ("j2d9pt-gol", np.float32, 29, 5, 2),
    ("star3d1r", np.float64, 14, 7, 3),
    ("star3d2r", np.float32, 15, 5, 2),
    ("j3d27pt", np.float32, 13, 5, 2),
    ("j3d27pt", np.float64, 12, 4, 3),
    ("gradient2d", np.float64, 24, 6, 4),
    ("gradient2d", np.float64, 20, 5, 1),
]


def _gpu_adjoint(name, dtype, u0, w, T, C, coef=None, want_coef=True, fp_mode="fma"):
    import torch
    from gbstencil.adjoint import Checkpointed
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    run = Checkpointed(name, torch.tensor(u0, dtype=tdt, device="cuda"), T, C, coef=coef, fp_mode=fp_mode)
    gu, gc = run.backward(torch.tensor(w, dtype=tdt, device="cuda"), want_coef=want_coef)
    torch.cuda.synchronize()
    return (run.u_T.double().cpu().numpy(), gu.double().cpu().numpy(),
            None if gc is None else gc.cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("name,dtype,n,T,C", CASES, ids=lambda v: getattr(v, "__name__", str(v)))
def test_adjoint_matches_reference(name, dtype, n, T, C):
    u0, w = _inputs(name, n, 3)
    u0 = u0.astype(dtype).astype(np.float64)
    coef = ar.default_coef(name)
    uT, gu, gc = _gpu_adjoint(name, dtype, u0, w, T, C)
    ref_gu, ref_gc = ar.adjoint(name, u0, coef, T, w)
    tol = 1e-4 if dtype == np.float32 else 1e-9
    assert _rel(uT, ar.forward(name, u0, coef, T)[-1]) <= tol
    assert _rel(gu, ref_gu) <= tol, name
    assert _rel(gc, ref_gc) <= tol, name


WIDE_CASES = [
    # rows wider than one lane segment (32 lanes x 16 bytes: 128 float or 64
    # double columns), so that in-row neighbours cross segments and warps
    # loop over several units; radius above the vector width (R > V)
    ("j2d5pt", np.float32, 300, 6, 4, True),
    ("j2d5pt", np.float32, 300, 6, 4, False),
    ("star2d3r", np.float64, 200, 5, 2, True),
    ("star2d3r", np.float64, 200, 5, 2, False),
    ("j2d9pt", np.float32, 300, 4, 3, True),
    ("box2d3r", np.float32, 170, 4, 2, False),
    ("box2d4r", np.float32, 150, 4, 2, False),
    ("box2d4r", np.float64, 150, 4, 3, False),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,dtype,n,T,C,want_coef", WIDE_CASES,
                         ids=lambda v: getattr(v, "__name__", str(v)))
def test_adjoint_matches_reference_wide_rows(name, dtype, n, T, C, want_coef):
    u0, w = _inputs(name, n, 4)
    u0 = u0.astype(dtype).astype(np.float64)
    coef = ar.default_coef(name)
    uT, gu, gc = _gpu_adjoint(name, dtype, u0, w, T, C, want_coef=want_coef)
    ref_gu, ref_gc = ar.adjoint(name, u0, coef, T, w)
    tol = 1e-4 if dtype == np.float32 else 1e-9
    assert _rel(gu, ref_gu) <= tol, name
    if want_coef:
        assert _rel(gc, ref_gc) <= tol, name
    else:
        assert gc is None


REVOLVE_CASES = [
    # name, dtype, n, T, checkpoint interval, snapshot slots (< 2C: binomial schedule)
    ("j2d5pt", np.float32, 40, 37, 8, 0),
    ("j2d5pt", np.float32, 40, 37, 8, 1),
    ("j2d5pt", np.float64, 33, 37, 13, 3),
    ("gradient2d", np.float64, 24, 20, 7, 2),
    ("star3d1r", np.float64, 12, 9, 9, 1),
    ("j3d27pt", np.float32, 11, 12, 12, 4),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,dtype,n,T,C,slots", REVOLVE_CASES, ids=lambda v: getattr(v, "__name__", str(v)))
def test_adjoint_binomial_schedule_matches_reference(name, dtype, n, T, C, slots):
    """A forced small budget: each chunk reversed by the revolve schedule."""
    import torch
    from gbstencil.adjoint import Checkpointed
    u0, w = _inputs(name, n, 11)
    u0 = u0.astype(dtype).astype(np.float64)
    coef = ar.default_coef(name)
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    run = Checkpointed(name, torch.tensor(u0, dtype=tdt, device="cuda"), T, C, slots=slots)
    gu, gc = run.backward(torch.tensor(w, dtype=tdt, device="cuda"), want_coef=True)
    full = Checkpointed(name, torch.tensor(u0, dtype=tdt, device="cuda"), T, C)
    fu, fc = full.backward(torch.tensor(w, dtype=tdt, device="cuda"), want_coef=True)
    torch.cuda.synchronize()
    # the recomputed states are the forward's, bit for bit: the same result as the full stash
    assert torch.equal(gu, fu) and torch.equal(gc, fc)
    ref_gu, ref_gc = ar.adjoint(name, u0, coef, T, w)
    tol = 1e-4 if dtype == np.float32 else 1e-9
    assert _rel(gu.double().cpu().numpy(), ref_gu) <= tol
    assert _rel(gc.cpu().numpy(), ref_gc) <= tol


@pytest.mark.gpu
def test_adjoint_budget_planner_run():
    import torch
    from gbstencil.adjoint import Checkpointed
    name, n, T = "j2d5pt", 64, 40
    u0, w = _inputs(name, n, 12)
    t0 = torch.tensor(u0, device="cuda")
    full = Checkpointed(name, t0, T, 8)
    small = Checkpointed(name, t0, T, budget_bytes=full.workspace_bytes // 3)
    assert small.workspace_bytes <= full.workspace_bytes // 3
    a, ca = full.backward(torch.tensor(w, device="cuda"))
    b, cb = small.backward(torch.tensor(w, device="cuda"))
    ref_gu, ref_gc = ar.adjoint(name, u0, ar.default_coef(name), T, w)
    assert _rel(b.cpu().numpy(), ref_gu) <= 1e-9 and _rel(cb.cpu().numpy(), ref_gc) <= 1e-9
    assert _rel(a.cpu().numpy(), b.cpu().numpy()) <= 1e-13


@pytest.mark.gpu
def test_adjoint_batch_matches_single_instances():
    """Uneven 3-D instances (and a 2-D one) at once through
    gbs_adjoint_forward_batch / gbs_adjoint_backward_batch."""
    import torch
    from gbstencil.adjoint import Checkpointed, backward_batch, forward_batch
    specs = [("j3d27pt", 10), ("j3d27pt", 14), ("j3d27pt", 17), ("star3d1r", 12)]
    T, C = 9, 4
    u0s, ws = [], []
    for i, (name, n) in enumerate(specs):
        u0, w = _inputs(name, n, 20 + i)
        u0s.append(torch.tensor(u0, dtype=torch.float32, device="cuda"))
        ws.append(torch.tensor(w, dtype=torch.float32, device="cuda"))
    runs = forward_batch([(nm, u) for (nm, _), u in zip(specs, u0s)], T, C)
    outs, _ = backward_batch(runs, ws)
    outs_c, cgs = backward_batch(runs, ws, want_coef=True)
    torch.cuda.synchronize()
    for (name, n), u, w, r, g, gc2, g2 in zip(specs, u0s, ws, runs, outs, cgs, outs_c):
        one = Checkpointed(name, u, T, C)
        gu, gc = one.backward(w, want_coef=True)
        torch.cuda.synchronize()
        assert torch.equal(r.u_T, one.u_T)
        assert torch.equal(g, gu) and torch.equal(g2, gu) and torch.equal(gc2, gc)
        ref_gu, ref_gc = ar.adjoint(name, u.double().cpu().numpy(), ar.default_coef(name), T, w.double().cpu().numpy())
        assert _rel(g.double().cpu().numpy(), ref_gu) <= 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["j2d5pt", "gradient2d", "star3d1r"])
def test_adjoint_directional_finite_difference(name):
    """<dL/du0, du> and <dL/dc, dc> against central differences of the
    engine's own float64 forward loop."""
    import torch
    from gbstencil.adjoint import Checkpointed
    n = {"j2d5pt": 48, "gradient2d": 40, "star3d1r": 16}[name]
    T = 8
    u0, w = _inputs(name, n, 5)
    coef = ar.default_coef(name)
    _, gu, gc = _gpu_adjoint(name, np.float64, u0, w, T, 3)
    r = ar.BY_NAME[name]["rad"]
    inner = tuple(slice(r, -r) for _ in range(u0.ndim))

    def L(u, c):
        run = Checkpointed(name, torch.tensor(u, device="cuda"), T, 64, coef=c)
        torch.cuda.synchronize()
        return float(np.sum(w[inner] * run.u_T.cpu().numpy()[inner]))

    def richardson(f, h=1e-5):
        # central differences at h and h/2, extrapolated: the h^2 error
        # term cancels (gradient2d's third derivatives are large where s is small)
        d1 = (f(h) - f(-h)) / (2 * h)
        d2 = (f(h / 2) - f(-h / 2)) / h
        return (4 * d2 - d1) / 3

    rng = RNG(6)
    du = rng.standard_normal(u0.shape)
    fd = richardson(lambda e: L(u0 + e * du, coef))
    assert abs(fd - np.sum(gu * du)) <= 1e-8 * max(1.0, abs(fd))
    dc = rng.standard_normal(coef.shape)
    fd = richardson(lambda e: L(u0, coef + e * dc))
    assert abs(fd - np.sum(gc * dc)) <= 1e-8 * max(1.0, abs(fd))


@pytest.mark.gpu
def test_adjoint_custom_coefficients_and_exact_mode():
    u0, w = _inputs("star2d2r", 26, 7)
    coef = RNG(8).random(len(ar.BY_NAME["star2d2r"]["terms"])) * 0.2
    uT, gu, gc = _gpu_adjoint("star2d2r", np.float64, u0, w, 6, 4, coef=coef, fp_mode="exact")
    ref_gu, ref_gc = ar.adjoint("star2d2r", u0, coef, 6, w)
    assert _rel(uT, ar.forward("star2d2r", u0, coef, 6)[-1]) <= 1e-12
    assert _rel(gu, ref_gu) <= 1e-9 and _rel(gc, ref_gc) <= 1e-9


@pytest.mark.gpu
def test_adjoint_backward_twice_and_many_terms():
    """Two backward passes from one forward give the same result; a stencil
    with more than 32 terms returns dL/du0 and refuses coefficient gradients."""
    import torch
    from gbstencil import capi
    from gbstencil.adjoint import Checkpointed
    u0, w = _inputs("box3d2r", 12, 9)
    run = Checkpointed("box3d2r", torch.tensor(u0, dtype=torch.float32, device="cuda"), 4, 2)
    lam = torch.tensor(w, dtype=torch.float32, device="cuda")
    a, _ = run.backward(lam, want_coef=False)
    a = a.clone()
    b, _ = run.backward(lam, want_coef=False)
    assert torch.equal(a, b)
    ref_gu, _ = ar.adjoint("box3d2r", u0.astype(np.float32).astype(np.float64), ar.default_coef("box3d2r"), 4, w)
    assert _rel(a.double().cpu().numpy(), ref_gu) <= 1e-4
    with pytest.raises(capi.GbsError) as e:
        run.backward(lam, want_coef=True)
    assert e.value.status == capi.GBS_ERR_UNSUPPORTED


@pytest.mark.gpu
def test_autograd_time_loop():
    import torch
    from gbstencil.adjoint import interior, time_loop
    name, T = "j2d5pt", 12
    u0, w = _inputs(name, 50, 10)
    coef = ar.default_coef(name)
    ut = torch.tensor(u0, device="cuda", requires_grad=True)
    ct = torch.tensor(coef, device="cuda", requires_grad=True)
    wt = torch.tensor(w, device="cuda")
    out = time_loop(ut, ct, name, T, checkpoint_every=5)
    loss = (interior(wt, name) * interior(out, name)).sum()
    loss.backward()
    ref_gu, ref_gc = ar.adjoint(name, u0, coef, T, w)
    assert _rel(ut.grad.cpu().numpy(), ref_gu) <= 1e-9
    assert _rel(ct.grad.cpu().numpy(), ref_gc) <= 1e-9
    assert abs(loss.item() - ar.loss(name, u0, coef, T, w)) <= 1e-9 * abs(loss.item())


@pytest.mark.gpu
def test_adjoint_argument_checks():
    import torch
    from gbstencil import capi
    d, _ = capi.make_desc("j2d5pt", np.float32, [32, 32], 4)
    L = capi.lib()
    nbytes = ctypes.c_size_t(0)
    assert L.gbs_adjoint_workspace(ctypes.byref(d), 0, ctypes.byref(nbytes)) == capi.GBS_ERR_INVALID
    assert L.gbs_adjoint_workspace(ctypes.byref(d), 2, ctypes.byref(nbytes)) == capi.GBS_OK
    ws = torch.empty(nbytes.value + 512, dtype=torch.uint8, device="cuda")
    base = ws.data_ptr() + (-ws.data_ptr()) % 256
    buf = torch.zeros(capi.layout(d).bytes // 4, dtype=torch.float32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.gbs_adjoint_forward(ctypes.byref(d), ctypes.c_void_p(buf.data_ptr()), 2,
                                 ctypes.c_void_p(base + 16), s) == capi.GBS_ERR_INVALID
    assert L.gbs_adjoint_forward(ctypes.byref(d), None, 2, ctypes.c_void_p(base), s) == capi.GBS_ERR_INVALID
    assert L.gbs_adjoint_backward(ctypes.byref(d), None, ctypes.c_void_p(buf.data_ptr()), None, 2,
                                  ctypes.c_void_p(base), s) == capi.GBS_ERR_INVALID


@pytest.mark.parametrize("name,dtype,n,T,C", [("j2d5pt", np.float32, 2048, 1024, 32),
                                               ("gradient2d", np.float64, 4096, 512, 32),
                                               ("j3d27pt", np.float32, 64, 20, 6)])
def test_adjoint_workspace_size(name, dtype, n, T, C):
    """Checkpoints (ceil(T/C) planes) + two stash buffers (2C) + two lam
    planes + the halo-gradient plane (+ q and sum-of-differences planes for
    gradient2d) + the partial-sum table, as the C ABI reports it (host
    arithmetic only)."""
    from gbstencil import capi
    d, _ = capi.make_desc(name, dtype, n, T, "fma")
    nbytes = ctypes.c_size_t(0)
    assert capi.lib().gbs_adjoint_workspace(ctypes.byref(d), C, ctypes.byref(nbytes)) == capi.GBS_OK
    L = capi.layout(d)
    plane = L.plane * np.dtype(dtype).itemsize
    s = capi.info(name)
    planes = -(-T // C) + 2 * C + 3 + (2 if s["kind"] == "gradient" else 0)
    assert nbytes.value >= planes * plane
    assert nbytes.value - planes * plane < 64 * 1024 * 1024   # the partial table and slack only
    # the 16 GB budget of the gradient2d configuration holds
    if name == "gradient2d":
        assert nbytes.value < 16e9


@pytest.mark.gpu
def test_adjoint_gradient_at_configuration_size():
    """j2d5pt float32 at the adjoint configuration's size (2048^2, T=1024,
    checkpoints every 32, loss 0.5 |u_T - target|^2, gradients of u_0 and of
    the five coefficients): directional derivatives of the engine's float32
    adjoint against Richardson-extrapolated central differences of the
    engine's float64 forward loop, relative error <= 1e-4."""
    import torch
    from gbstencil.adjoint import Checkpointed
    name, n, T, C = "j2d5pt", 2048, 1024, 32
    r = ar.BY_NAME[name]["rad"]
    shape = [n + 2 * r] * 2
    rng = RNG(31)
    u0 = rng.random(shape).astype(np.float32).astype(np.float64)
    target = rng.random(shape)
    coef = ar.default_coef(name)
    inner = (slice(r, -r), slice(r, -r))
    run = Checkpointed(name, torch.tensor(u0, dtype=torch.float32, device="cuda"), T, C)
    lam = (run.u_T.double() - torch.tensor(target, device="cuda")).float()
    gu, gc = run.backward(lam, want_coef=True)
    torch.cuda.synchronize()
    gu, gc = gu.double().cpu().numpy(), gc.cpu().numpy()
    tgt = torch.tensor(target[inner], device="cuda")

    def loss(u, c):
        # forward only: one checkpoint, no stash planes
        f = Checkpointed(name, torch.tensor(u, device="cuda"), T, T, coef=c, slots=0)
        torch.cuda.synchronize()
        return float(0.5 * ((f.u_T[inner] - tgt) ** 2).sum())

    def richardson(f, h):
        d1 = (f(h) - f(-h)) / (2 * h)
        d2 = (f(h / 2) - f(-h / 2)) / h
        return (4 * d2 - d1) / 3

    du = RNG(32).standard_normal(shape)
    fd = richardson(lambda e: loss(u0 + e * du, coef), 1e-3)
    assert abs(fd - np.sum(gu * du)) <= 1e-4 * abs(fd), (fd, np.sum(gu * du))
    dc = RNG(33).standard_normal(coef.shape)
    fd = richardson(lambda e: loss(u0, coef + e * dc), 1e-5)
    assert abs(fd - np.sum(gc * dc)) <= 1e-4 * abs(fd), (fd, np.sum(gc * dc))
