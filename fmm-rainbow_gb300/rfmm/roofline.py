"""Per-phase algorithmic work of one FMM step, counted from a moment tree.

The work of a step depends on the tree: which subtrees hold bodies, which
parents are listed (count > 16, src/rainbow_fmm.wgsl:472-476), which of their
children are targets, and how many stencil sources each target sees.  These
functions count it exactly from a downloaded moment buffer (reference layout,
levels 0..depth at offsets (8^l - 1) / 7, cells x-fastest), so a measured
phase time turns into an achieved rate.

Algorithmic bytes and flops per phase (the data each phase must move, each
item once, whatever the kernel's layout):

  upward     16 B read + 52 B written per leaf of a non-empty 8x8x8-leaf
             subtree (leaf moment in; source 16, record 16, sample cell 4,
             cleared next-deposit leaf 16 out), 48 B written per upper cell
             of such a subtree and per cell above the subtrees (moment,
             source, record), 48 B per field cleared for the previous
             step's targets
  m2l        flops: 51 binary32 operations per (target, source) pair
             (pair_field's 41 adds, multiplies, square root and division, and
             10 accumulating adds); bytes: the 216-cell source tile per
             listed parent (3,456 B) and 64 B per target (count in, 48 B
             M2L result out)
  l2l_near   112 B per target (its count, its M2L result, its final field;
             each ancestor's M2L result is another target's) + 16 B per
             adaptive-leaf target (its source record, read once by its
             neighbours)
  integrate  64 B per body (particle in and out) + 64 B per cell (field and
             moment gathered once) + 16 B per leaf (the next deposit)
  resort     72 B per body (particle and id in and out) + 36 B per leaf
             (leaf count read twice, start slot written)
  near_p2p   (exact near-field mode) flops: 20 per pair interaction, the
             usual N-body convention; bytes: 16 B position in and 16 B sums
             out per body
"""
from __future__ import annotations

import numpy as np

ADAPTIVE = 16
PAIR_FLOPS = 51


def level_offset(l: int) -> int:
    return (8 ** l - 1) // 7


def _grid(counts: np.ndarray, l: int) -> np.ndarray:
    d = 1 << l
    c = counts[level_offset(l): level_offset(l) + d ** 3]
    return c.reshape(d, d, d)  # [z, y, x]


def _box_sum(nonempty: np.ndarray, lo: np.ndarray, hi: np.ndarray) -> np.ndarray:
    """Sum of a level grid (occupancy or counts) over boxes [lo, hi]
    (inclusive, per axis, clipped).

    lo/hi are (k, 3) arrays of (z, y, x) corners."""
    d = nonempty.shape[0]
    s = np.zeros((d + 1, d + 1, d + 1), np.int64)
    s[1:, 1:, 1:] = nonempty.astype(np.int64).cumsum(0).cumsum(1).cumsum(2)
    a = np.clip(lo, 0, d)
    b = np.clip(hi + 1, 0, d)
    b = np.maximum(a, b)
    z0, y0, x0 = a[:, 0], a[:, 1], a[:, 2]
    z1, y1, x1 = b[:, 0], b[:, 1], b[:, 2]
    return (s[z1, y1, x1] - s[z0, y1, x1] - s[z1, y0, x1] - s[z1, y1, x0]
            + s[z0, y0, x1] + s[z0, y1, x0] + s[z1, y0, x0] - s[z0, y0, x0])


def tree_work(moments: np.ndarray, depth: int) -> dict:
    """Exact per-step work counts of the tree in `moments` (count column used)."""
    counts = np.ascontiguousarray(moments).view(np.uint32).reshape(-1, 4)[:, 0].astype(np.int64)
    D = depth
    cells = level_offset(D + 1)
    assert len(counts) >= cells
    parents = 0
    targets = 0
    leaf_targets = 0
    m2l_pairs = 0
    near_pairs = 0
    for lp in range(D):
        pg = _grid(counts, lp)
        listed = pg > ADAPTIVE
        parents += int(listed.sum())
        l = lp + 1
        cg = _grid(counts, l)
        nonempty = cg > 0
        # Targets: non-empty children of listed parents.
        child_of_listed = np.repeat(np.repeat(np.repeat(listed, 2, 0), 2, 1), 2, 2)
        tmask = child_of_listed & nonempty
        t = np.argwhere(tmask)  # (k, 3) z, y, x
        if len(t) == 0:
            continue
        targets += len(t)
        p2 = (t // 2) * 2
        window = _box_sum(nonempty, p2 - 2, p2 + 3)  # children of the parent's 3x3x3 block
        near = _box_sum(nonempty, t - 1, t + 1)      # the target's 3x3x3 block (itself included)
        m2l_pairs += int((window - near).sum())
        tc = cg[tmask]
        is_leaf = (tc <= ADAPTIVE) | (l == D)
        leaf_targets += int(is_leaf.sum())
        near_pairs += int((near[is_leaf] - 1).sum())  # 26 neighbours, empty ones skipped
    # Upward: subtrees of 8x8x8 leaves rooted at level D - 3 that hold bodies.
    r = D - 3
    live_sub = int((_grid(counts, r) > 0).sum())
    leaves_live = live_sub * 512
    upper_live = live_sub * (64 + 8 + 1) + level_offset(r)
    return {"depth": D, "cells": cells, "leaves": 8 ** D, "parents": parents, "targets": targets,
            "leaf_targets": leaf_targets, "m2l_pairs": m2l_pairs, "near_pairs": near_pairs,
            "live_subtrees": live_sub, "leaves_live": leaves_live, "upper_live": upper_live}


def p2p_pairs(moments: np.ndarray, depth: int) -> int:
    """Pair interactions of one exact near-field step (RFMM_NEAR_P2P): every
    body pairs with every other body of the 3x3x3 cells around its sample
    cell, the first level whose cell holds at most 16 bodies (else the leaf)."""
    counts = np.ascontiguousarray(moments).view(np.uint32).reshape(-1, 4)[:, 0].astype(np.int64)
    D = depth
    leaf = _grid(counts, D)
    lvl = np.full(leaf.shape, D, np.int64)
    for l in range(D - 1, 0, -1):  # coarser levels overwrite: the first level from the top wins
        f = 1 << (D - l)
        g = _grid(counts, l)
        up = np.repeat(np.repeat(np.repeat(g, f, 0), f, 1), f, 2)
        lvl = np.where(up <= ADAPTIVE, l, lvl)
    pairs = 0
    for l in range(1, D + 1):
        sel = (leaf > 0) & (lvl == l)
        if not sel.any():
            continue
        cell = np.argwhere(sel) >> (D - l)
        box = _box_sum(_grid(counts, l), cell - 1, cell + 1)  # bodies of the 3x3x3 block
        pairs += int((leaf[sel] * (box - 1)).sum())
    return pairs


def phase_work(n: int, w: dict) -> dict:
    """Algorithmic bytes (and flops) per launch of each phase for one scene."""
    return {
        "upward": {"bytes": 68 * w["leaves_live"] + 48 * w["upper_live"] + 48 * w["targets"]},
        "m2l": {"bytes": 3456 * w["parents"] + 64 * w["targets"],
                "flops": PAIR_FLOPS * w["m2l_pairs"]},
        "l2l_near": {"bytes": 112 * w["targets"] + 16 * w["leaf_targets"]},
        "integrate": {"bytes": 64 * n + 64 * w["cells"] + 16 * w["leaves"]},
        "resort": {"bytes": 72 * n + 36 * w["leaves"]},
    }


def add_work(total: dict | None, part: dict) -> dict:
    """Sum per-phase work over the scenes of a batch."""
    if total is None:
        return {k: dict(v) for k, v in part.items()}
    for k, v in part.items():
        for kk, vv in v.items():
            total[k][kk] = total[k].get(kk, 0) + vv
    return total


def fp32_peak_tflops(sms: int, sm_mhz: float) -> float:
    """Nominal FP32 rate: 128 lanes per SM, an FMA (2 flops) per lane per cycle."""
    return sms * 128 * 2 * sm_mhz * 1e6 / 1e12


def phases_roofline(work: dict, timeline: dict, hbm_peak_gbs: float, fp32_tflops: float,
                    peak_source: str) -> dict:
    """Per-phase achieved rates from the in-graph timeline (busy time per launch)."""
    out = {}
    for k, v in work.items():
        t = timeline["kinds"].get(k)
        if t is None or t["launches"] == 0:
            continue
        ms = t["busy_ms"] / t["launches"]
        gbs = v["bytes"] / (ms * 1e-3) / 1e9
        e = {"busy_ms_per_launch": ms, "gap_ms_per_launch": t["gap_ms"] / t["launches"],
             "launches": t["launches"], "algorithmic_bytes": v["bytes"], "achieved_gbs": gbs,
             "hbm_frac": gbs / hbm_peak_gbs}
        if "flops" in v:
            tf = v["flops"] / (ms * 1e-3) / 1e12
            e.update({"bound": "fp32", "flops": v["flops"], "achieved_tflops": tf,
                      "peak_tflops": fp32_tflops, "frac": tf / fp32_tflops,
                      "peak_source": "nominal: SMs x 128 lanes x 2 x sampled SM clock"})
        else:
            e.update({"bound": "hbm", "frac": gbs / hbm_peak_gbs, "peak_gbs": hbm_peak_gbs,
                      "peak_source": peak_source})
        out[k] = e
    return out
