"""Host replica of the batched work-item schedule (csrc/batch.cu,
gbs_batch_build): the time blocks of each grid (batch_blocks: full blocks of
the family degree, then single steps, as many blocks as T has parity), the
items (grid, time block, strip, stream block) in time-block order, their
per-stream-block `need` counts, and the dependency rule of the persistent
kernel (an item waits for its own stream block and the two beside it to
finish every earlier time block of its grid). Checked on seeded mixes: every
read-after-write and write-after-read between consecutive time blocks of a
grid falls inside that rule, every waited-on item comes earlier in the list
(the order the CTAs take them in), and the result lands in plane T%2. CPU
only."""
import numpy as np
import pytest

from gbstencil import capi

MIX = ["star2d1r", "star2d2r", "star2d3r", "star2d4r", "box2d1r", "box2d2r", "box2d3r", "box2d4r", "j2d5pt",
       "j2d9pt", "j2d9pt-gol", "gradient2d"]


def degree(name):
    """batch_degree of csrc/batch.cu."""
    s = capi.info(name)
    if s["kind"] == "gradient":
        return 1
    r = s["rad"]
    if r == 1:
        return 6
    if r == 2:
        return 2 if s["nterms"] > 13 else 3
    if r == 3:
        return 1 if s["form"] == "assoc" else 2
    return 1


def batch_blocks(T, bs):
    if T <= 0:
        return []
    n, r = T // bs, T - (T // bs) * bs
    if ((n + r) - T) % 2 != 0 and n > 0:
        n -= 1
        r += bs
    return [bs] * n + [1] * r


def plan(grids, sl_max):
    """(items, per-grid geometry) as gbs_batch_build orders them."""
    geo = []
    for name, n, T in grids:
        r = capi.info(name)["rad"]
        d0, d1 = n[0] + 2 * r, n[1] + 2 * r
        ni = d0 - 2 * r
        sl = min(ni, sl_max)
        geo.append(dict(r=r, d0=d0, d1=d1, sl=sl, nblocks=-(-ni // sl), blocks=batch_blocks(T, degree(name))))
    items, done_before = [], [0] * len(grids)
    kmax = max((len(g["blocks"]) for g in geo), default=0)
    sids = {name: i for i, name in enumerate(capi.NAMES)}
    for k in range(kmax):
        for sid in range(len(capi.NAMES)):
            for gi, (name, n, T) in enumerate(grids):
                if sids[name] != sid or k >= len(geo[gi]["blocks"]):
                    continue
                g = geo[gi]
                b = g["blocks"][k]
                wout = ((128 - 2 * b * g["r"] - 3) // 4) * 4
                nstrips = -(-(g["d1"] - 2 * g["r"]) // wout)
                for blk in range(g["nblocks"]):
                    for st in range(nstrips):
                        items.append(dict(g=gi, k=k, b=b, strip=st, blk=blk, need=done_before[gi]))
                done_before[gi] += nstrips
    return items, geo


def rows(g, blk):
    i0 = g["r"] + blk * g["sl"]
    return i0, min(i0 + g["sl"], g["d0"] - g["r"])


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("sl_max", [96, 128])
def test_dependencies_cover_every_hazard(seed, sl_max):
    rng = np.random.default_rng(seed)
    grids = []
    for i in range(40):
        name = MIX[i % len(MIX)] if i < len(MIX) else MIX[int(rng.integers(len(MIX)))]
        n = [int(round(np.exp(rng.uniform(np.log(3), np.log(700))))) for _ in range(2)]
        grids.append((name, n, int(rng.integers(0, 40))))
    items, geo = plan(grids, sl_max)
    pos = {}
    for idx, it in enumerate(items):
        pos.setdefault((it["g"], it["k"], it["blk"]), []).append(idx)
    for gi, g in enumerate(geo):
        L = len(g["blocks"])
        # the result plane: one plane swap per time block
        assert L % 2 == grids[gi][2] % 2
        assert sum(g["blocks"]) == grids[gi][2]
        for k in range(1, L):
            ba, bb = g["blocks"][k - 1], g["blocks"][k]
            for blk_b in range(g["nblocks"]):
                b0, b1 = rows(g, blk_b)
                # the blocks item (k, blk_b) waits for, and what they must cover
                waited = {c for c in (blk_b - 1, blk_b, blk_b + 1) if 0 <= c < g["nblocks"]}
                for blk_a in range(g["nblocks"]):
                    a0, a1 = rows(g, blk_a)
                    raw = max(a0, b0 - bb * g["r"]) < min(a1, b1 + bb * g["r"])   # B reads what A wrote
                    war = max(b0, a0 - ba * g["r"]) < min(b1, a1 + ba * g["r"])   # B overwrites what A read
                    if raw or war:
                        assert blk_a in waited, (gi, k, blk_a, blk_b)
                # every waited-on item comes earlier in the list, and `need`
                # counts exactly the items of one block in earlier time blocks
                first_b = min(pos[(gi, k, blk_b)])
                for c in waited:
                    for kk in range(k):
                        assert max(pos[(gi, kk, c)]) < first_b
                need = items[first_b]["need"]
                assert need == sum(len(pos[(gi, kk, blk_b)]) for kk in range(k))
