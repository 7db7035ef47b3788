"""The quad path's list construction (aggregate.cu: rlist_*, qlist_*,
gather_quad_kernel), restated on the CPU: for every pixel, merging the quad
lists of its origin frames and keeping the members that cover the pixel
yields exactly the pixel's own terms in slot order -- the order in which the
reference adds them (src/core/nldct.cpp:2259-2332) -- and no member takes more
than the list entries the chunk budget reserves (2 row-list and 8 quad-list
entries)."""
import numpy as np
import pytest

Q = 4   # pixels per quad, also the patch width


def build(w, h, F, pt, origins):
    """Row lists rl[(to, oy, q)] and quad lists ql[(to, y, q)] of (slot, ...)
    entries in slot order, from member origins (slot -> (ox, oy, to))."""
    nq = (w + Q - 1) // Q
    by_origin = {}
    for slot, (ox, oy, to) in enumerate(origins):
        by_origin.setdefault((to, oy, ox), []).append(slot)
    rl = {}
    for to in range(F):
        for oy in range(h):
            for q in range(nq):
                ent = []
                for ox in range(max(0, Q * q - 3), min(w - Q, Q * q + 3) + 1):
                    ent += [(s, ox - Q * q + 3) for s in by_origin.get((to, oy, ox), [])]
                if ent:
                    rl[(to, oy, q)] = sorted(ent)
    ql = {}
    for to in range(F):
        for y in range(h):
            for q in range(nq):
                ent = []
                for dy in range(Q):
                    ent += [(s, dy, s3) for s, s3 in rl.get((to, y - dy, q), [])]
                if ent:
                    ql[(to, y, q)] = sorted(ent)
    return rl, ql


@pytest.mark.parametrize("w,h,F,pt,seed", [(13, 9, 6, 4, 1), (16, 8, 5, 2, 2), (10, 7, 3, 1, 3), (21, 5, 7, 4, 4)])
def test_quad_lists_give_each_pixel_its_terms_in_slot_order(w, h, F, pt, seed):
    rng = np.random.default_rng(seed)
    n = 400
    origins = [(int(rng.integers(0, w - Q + 1)), int(rng.integers(0, h - Q + 1)), int(rng.integers(0, F - pt + 1)))
               for _ in range(n)]
    rl, ql = build(w, h, F, pt, origins)
    # list sizes against the chunk's reservation
    per_rl = np.zeros(n, int)
    per_ql = np.zeros(n, int)
    for v in rl.values():
        for s, _ in v:
            per_rl[s] += 1
    for v in ql.values():
        for s, _, _ in v:
            per_ql[s] += 1
    assert per_rl.max() <= 2 and per_ql.max() <= 8
    for t in range(F):
        for y in range(h):
            for x in range(w):
                # the reference's order: every member covering (x, y, t), by slot
                want = [(s, (t - to) * Q * Q + (y - oy) * Q + (x - ox)) for s, (ox, oy, to) in enumerate(origins)
                        if ox <= x < ox + Q and oy <= y < oy + Q and to <= t < to + pt]
                # the quad gather: merge the pt quad lists by slot, keep the covering members
                q, j = x // Q, x % Q
                merged = []
                for dt in range(pt):
                    merged += [(s, dt, dy, s3) for s, dy, s3 in ql.get((t - dt, y, q), [])]
                merged.sort()
                got = []
                for s, dt, dy, s3 in merged:
                    dx = j - (s3 - 3)
                    if 0 <= dx < Q:
                        got.append((s, (dt * Q + dy) * Q + dx))
                assert got == want, (x, y, t)
