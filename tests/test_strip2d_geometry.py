"""Host replica of the 2-D kernels' column decomposition (make_layout and
geometry2d in csrc/engine.cu, the strip windows of warp_item2d in
csrc/kernel2d.cuh): for every radius, element size and fused degree and a
range of row widths, each interior column is stored by exactly one strip;
every stored column is exact after b levels (at least b*r columns inside
its 32*V-column window, or the window reaches past the grid edge, where the
fixed halo carries exact values); each window is 16-byte aligned and lies
inside the padded row. CPU only."""
import pytest


def layout(R, V, d1):
    shift = (V - R % V) % V
    need = shift + d1 + 32 * V
    align = 128 // (16 // V)
    return shift, -(-need // align) * align


def strips(R, V, B, d1):
    wout = ((32 * V - 2 * B * R - (V - 1)) // V) * V
    nj = d1 - 2 * R
    return wout, (-(-nj // wout) if wout > 0 else 1)


@pytest.mark.parametrize("V", [4, 2])
@pytest.mark.parametrize("R", [1, 2, 3, 4])
@pytest.mark.parametrize("B", range(1, 9))
def test_strip_windows_cover_each_column_once_exactly(V, R, B):
    ROW = 32 * V
    for n in list(range(1, 70)) + [127, 128, 129, 255, 300, 1000, 4096]:
        d1 = n + 2 * R
        shift, pitch = layout(R, V, d1)
        wout, ns = strips(R, V, B, d1)
        if wout <= 0:
            continue  # the planner refuses this degree (GBS_ERR_UNSUPPORTED)
        stored = [0] * d1
        for s in range(ns):
            cs = R + s * wout
            ce = min(cs + wout, d1 - R)
            need_lo = max(0, cs - B * R)
            ws = ((need_lo + shift) // V) * V       # element index of the window start
            assert ws % V == 0 and ws >= 0 and ws + ROW <= pitch
            w0 = ws - shift                          # grid column of window element 0
            for lane in range(32):
                col0 = w0 + lane * V
                for e in range(V):
                    c = col0 + e
                    if cs <= c < ce:
                        stored[c] += 1
                        assert w0 <= 0 or c - B * R >= w0, (n, s, c)
                        assert w0 + ROW >= d1 or c + B * R < w0 + ROW, (n, s, c)
        assert all(stored[c] == 1 for c in range(R, d1 - R)), n
        assert sum(stored) == d1 - 2 * R
