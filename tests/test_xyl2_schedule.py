"""The work schedule of the L2-staged fused x+y pass (convfpga_gb300/csrc/xyl2.cuh), on CPU.

A restatement of the kernel's item order (xyl2_item) and dependency rules, with the
per-size constants read from the header, checks:
  - the order lists every (plane, tile, X/Y) item exactly once;
  - every item an item waits on comes earlier in the order (a Y item on the X items of its
    plane, an X item of plane p >= R on the Y items of plane p - R, which read the scratch
    slot it overwrites);
  - a randomised run of CTAs that claim items in order, hold the current item and the
    next index, and finish an item only when its dependencies are done always completes,
    whatever the number of resident CTAs (the kernel's no-deadlock argument).
"""
import os
import random
import re

import pytest

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "convfpga_gb300", "csrc",
                      "xyl2.cuh")


def _cfg(n):
    """C, LAG, RING of XyL2Cfg<n> as written in the header."""
    text = open(HEADER).read()
    m = re.search(r"struct XyL2Cfg<%d>\s*\{(.*?)\n\};" % n, text, re.S)
    assert m, f"XyL2Cfg<{n}> not found"
    body = m.group(1)
    vals = {k: int(v) for k, v in re.findall(r"\b(C|LAG|RING)\s*=\s*(\d+)", body)}
    return vals["C"], vals["LAG"], vals["RING"]


def _item(w, np_, lag, items):
    """(plane, tile, is_y) of item w: X items of plane b then Y items of plane b - lag."""
    head = lag * items
    body = (np_ - lag) * 2 * items
    if w < head:
        return w // items, w % items, False
    if w < head + body:
        v = w - head
        b = lag + v // (2 * items)
        r = v % (2 * items)
        is_y = r >= items
        return (b - lag if is_y else b), (r - items if is_y else r), is_y
    v = w - head - body
    return np_ - lag + v // items, v % items, True


def _schedule(n, ncubes):
    c, lag_max, ring = _cfg(n)
    items = n // c
    np_ = n * ncubes
    lag = min(np_, lag_max)
    order = [_item(w, np_, lag, items) for w in range(2 * np_ * items)]
    return order, items, ring


def _deps(it, items, ring):
    p, _, is_y = it
    if is_y:
        return [(p, r, False) for r in range(items)]
    if p >= ring:
        return [(p - ring, r, True) for r in range(items)]
    return []


@pytest.mark.parametrize("n,ncubes", [(256, 1), (256, 3), (128, 1), (128, 2), (128, 8)])
def test_order_is_complete_and_dependencies_come_first(n, ncubes):
    order, items, ring = _schedule(n, ncubes)
    pos = {it: w for w, it in enumerate(order)}
    assert len(pos) == len(order) == 2 * n * ncubes * items
    for w, it in enumerate(order):
        for d in _deps(it, items, ring):
            assert pos[d] < w, (it, d)


def _simulate(order, items, ring, ctas, rng):
    """CTAs claim indices in order; each holds its current item and the next index.
    Returns True when every item finished."""
    done = set()
    nxt = 0
    cur = []
    for _ in range(ctas):  # every CTA claims two indices at start
        if nxt < len(order):
            c = nxt
            nxt += 1
            n2 = nxt if nxt < len(order) else None
            if n2 is not None:
                nxt += 1
            cur.append([c, n2])
    active = [k for k in range(len(cur))]
    steps = 0
    while active:
        steps += 1
        if steps > 50 * len(order) + 1000:
            return False
        progressed = False
        rng.shuffle(active)
        for k in list(active):
            c, n2 = cur[k]
            if all(d in done for d in _deps(order[c], items, ring)):
                done.add(order[c])
                progressed = True
                if n2 is None:
                    active.remove(k)
                    continue
                # the next index becomes current; a new one is claimed during it
                c = n2
                if nxt < len(order):
                    n2 = nxt
                    nxt += 1
                else:
                    n2 = None
                cur[k] = [c, n2]
                if rng.random() < 0.5:
                    break  # let other CTAs move too
        if not progressed:
            return False
    return len(done) == len(order)


@pytest.mark.parametrize("n,ncubes", [(256, 1), (128, 2)])
@pytest.mark.parametrize("ctas", [1, 3, 64, 1216])
def test_any_number_of_resident_ctas_completes(n, ncubes, ctas):
    order, items, ring = _schedule(n, ncubes)
    rng = random.Random(ctas * 7 + n)
    assert _simulate(order, items, ring, ctas, rng)


def _tiled(n):
    """TILED of XyL2Cfg<n> as written in the header."""
    text = open(HEADER).read()
    body = re.search(r"struct XyL2Cfg<%d>\s*\{(.*?)\n\};" % n, text, re.S).group(1)
    return re.search(r"\bTILED\s*=\s*(true|false)", body).group(1) == "true"


@pytest.mark.parametrize("n", [128, 256, 512])
def test_ring_slot_layout(n):
    """The X items' stores and the Y items' loads address the same slot positions: every
    element of a plane is stored exactly once by the X items, and the Y item of column tile c
    reads exactly columns C*c .. C*c+C-1 of every row, row by row in the order its threads
    expect (position n of column j at n*C + j). Restates the index arithmetic of k_xy_l2: with
    column tiles (N = 128, 256) an X thread (row y, lane t) stores x = t + e*T at
    (x / C) * N * C + y * C + x % C and a Y item bulk-copies the N * C values from
    c * N * C; with row-major slots (N = 512) the store is at y * N + x and the Y item's TMA
    box lands row by row."""
    import numpy as np

    c_cols, _, _ = _cfg(n)
    e_pts = 16
    t_thr = n // e_pts
    tiled = _tiled(n)
    assert tiled == (n in (128, 256))
    slot = np.full(n * n, -1, np.int64)
    for tile in range(n // c_cols):            # X items of one plane
        for c in range(c_cols):                # rows of the item
            y = tile * c_cols + c
            for t in range(t_thr):
                for e in range(e_pts):
                    x = t + e * t_thr
                    addr = (x // c_cols) * n * c_cols + y * c_cols + x % c_cols if tiled else y * n + x
                    assert slot[addr] == -1, "two stores to one slot position"
                    slot[addr] = y * n + x     # which element lives there
    assert (slot >= 0).all()
    for tile in range(n // c_cols):            # Y items: what lands in shared memory
        if tiled:
            landed = slot[tile * n * c_cols:(tile + 1) * n * c_cols]
        else:
            landed = np.array([slot[r * n + tile * c_cols + j] for r in range(n) for j in range(c_cols)])
        want = np.array([r * n + tile * c_cols + j for r in range(n) for j in range(c_cols)])
        assert np.array_equal(landed, want)
