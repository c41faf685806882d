"""The rule by which P2G merges its segment leaders' sums along z (mpm_substep_kernels.cuh,
p2g_warp_segments with kMerge and p2g_column_sums), restated over simulated warps: every lane's 27 node
contributions reach the grid exactly once, at the right node, whatever the warp's bases, group cuts and
invalid lanes. (The GPU test test_p2g_merge_along_z_matches_one_reduction_per_leader checks the kernel.)"""

from __future__ import annotations

import random

import pytest


def _warp(rng, group):
    lanes, (x, y, z) = [], (rng.randint(0, 5), rng.randint(0, 5), rng.randint(0, 5))
    for _ in range(32):
        r = rng.random()
        if r < 0.08:
            x, y, z = rng.randint(0, 5), rng.randint(0, 5), rng.randint(0, 5)
        elif r >= 0.5:
            z += rng.choice([1, 1, 1, 2, 3])
        lanes.append(((x, y, z), rng.random() > 0.03))
    key = [b if v else ("invalid", lane) for lane, (b, v) in enumerate(lanes)]
    first = [lane % group == 0 or key[lane - 1] != key[lane] for lane in range(32)]
    leader = [lanes[lane][1] and first[lane] for lane in range(32)]
    return lanes, first, leader


def _written(lanes, first, leader):
    """(lane, node) -> how many times the merged scatter adds that lane's contribution to that node."""
    owner, cur = [], None
    for lane in range(32):
        cur = lane if first[lane] else cur
        owner.append(cur)
    sums = {lane: {} for lane in range(32) if leader[lane]}  # leader -> (i, j, k) -> contributions
    for lane, ((bx, by, bz), valid) in enumerate(lanes):
        if valid and leader[owner[lane]]:
            for i in range(3):
                for j in range(3):
                    for k in range(3):
                        sums[owner[lane]].setdefault((i, j, k), []).append((lane, (bx + i, by + j, bz + k)))
    leaders = [lane for lane in range(32) if leader[lane]]
    xy = lambda q: lanes[q][0][:2] if lanes[q][1] else ("invalid", q)  # noqa: E731
    z = lambda q: lanes[q][0][2]  # noqa: E731
    out = {}
    for b in leaders:
        below = [q for q in leaders if q < b]
        p1 = below[-1] if below else b
        below2 = [q for q in leaders if q < p1]
        p2 = below2[-1] if below2 else b
        above = [q for q in leaders if q > b]
        s1 = above[0] if above else b
        d1 = z(b) - z(p1) if p1 != b and xy(p1) == xy(b) and z(b) - z(p1) in (1, 2) else 0
        ok2 = d1 == 1 and p2 != p1 and xy(p2) == xy(b) and z(b) - z(p2) == 2
        ws = z(s1) - z(b) if s1 != b and xy(s1) == xy(b) and z(s1) - z(b) in (1, 2) else 0
        bx, by, bz = lanes[b][0]
        for i in range(3):
            for j in range(3):
                o0 = list(sums[b].get((i, j, 0), []))
                if d1:
                    o0 += sums[p1].get((i, j, d1), [])
                if ok2:
                    o0 += sums[p2].get((i, j, 2), [])
                o1 = list(sums[b].get((i, j, 1), [])) + (sums[p1].get((i, j, 2), []) if d1 == 1 else [])
                outs = [(0, o0)] + ([(1, o1)] if ws != 1 else []) + ([(2, sums[b].get((i, j, 2), []))] if ws == 0 else [])
                for k, items in outs:
                    for lane, node in items:
                        assert node == (bx + i, by + j, bz + k)
                        out[(lane, node)] = out.get((lane, node), 0) + 1
    return out


@pytest.mark.parametrize("group", [32, 4, 1])
def test_every_contribution_is_written_once(group):
    rng = random.Random(group)
    for _ in range(2000):
        lanes, first, leader = _warp(rng, group)
        out = _written(lanes, first, leader)
        for lane, ((bx, by, bz), valid) in enumerate(lanes):
            if valid:
                for i in range(3):
                    for j in range(3):
                        for k in range(3):
                            assert out.get((lane, (bx + i, by + j, bz + k)), 0) == 1
        assert sum(out.values()) == 27 * sum(v for _, v in lanes)
