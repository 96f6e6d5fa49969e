"""The per-phase work counts behind the bench's per-phase roofline: targets
against the oracle's target list, stencil pairs against a direct count over
the reference's M2L and near loops (src/rainbow_fmm.wgsl:457-572)."""
import numpy as np


def _brute(moments, depth):
    counts = moments["count"].astype(np.int64)
    off = lambda l: (8 ** l - 1) // 7  # noqa: E731
    m2l = near = 0
    for l in range(1, depth + 1):
        d = 1 << l
        g = counts[off(l): off(l) + d ** 3].reshape(d, d, d)
        pd = d // 2
        pg = counts[off(l - 1): off(l - 1) + pd ** 3].reshape(pd, pd, pd)
        for z, y, x in np.argwhere(g > 0):
            if pg[z // 2, y // 2, x // 2] <= 16:
                continue
            # m2l_all: children of the parent's 3x3x3 neighbours, not adjacent.
            for pz in range(z // 2 - 1, z // 2 + 2):
                for py in range(y // 2 - 1, y // 2 + 2):
                    for px in range(x // 2 - 1, x // 2 + 2):
                        if not (0 <= pz < pd and 0 <= py < pd and 0 <= px < pd):
                            continue
                        for cz in range(2):
                            for cy in range(2):
                                for cx in range(2):
                                    sz, sy, sx = 2 * pz + cz, 2 * py + cy, 2 * px + cx
                                    if max(abs(sz - z), abs(sy - y), abs(sx - x)) <= 1:
                                        continue
                                    m2l += int(g[sz, sy, sx] > 0)
            # near_all at adaptive leaves: the 26 neighbours.
            if g[z, y, x] <= 16 or l == depth:
                for dz in (-1, 0, 1):
                    for dy in (-1, 0, 1):
                        for dx in (-1, 0, 1):
                            if dz == dy == dx == 0:
                                continue
                            sz, sy, sx = z + dz, y + dy, x + dx
                            if 0 <= sz < d and 0 <= sy < d and 0 <= sx < d:
                                near += int(g[sz, sy, sx] > 0)
    return m2l, near


def test_tree_work_counts_match_reference_loops(oracle_mod):
    O = oracle_mod
    from rfmm import roofline, scenes
    for kind, n in (("plummer", 30000), ("clusters", 20000), ("uniform", 5000)):
        p = scenes.make(kind, n, 3)
        st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4))
        st.solve_fields()
        w = roofline.tree_work(st.moments, st.params.depth)
        assert w["targets"] == len(st.m2l_targets()), kind
        m2l, near = _brute(st.moments, st.params.depth)
        assert m2l > 0 and near > 0
        assert (w["m2l_pairs"], w["near_pairs"]) == (m2l, near), kind
        assert w["parents"] == int((st.moments["count"][: (8 ** st.params.depth - 1) // 7] > 16).sum())
        work = roofline.phase_work(n, w)
        assert work["m2l"]["flops"] == 51 * m2l and work["integrate"]["bytes"] > 64 * n


def test_p2p_pair_count_matches_direct_count(oracle_mod):
    """Exact near-field pairs: every body against the bodies of the 3x3x3
    cells around its sample cell, itself excluded."""
    O = oracle_mod
    from rfmm import roofline, scenes
    for kind, n in (("plummer", 20000), ("uniform", 6000)):
        p = scenes.make(kind, n, 4)
        st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4))
        st.solve_fields()
        D = st.params.depth
        samples = st.sample_cells().astype(np.int64)  # global cell index per body
        counts = st.moments["count"].astype(np.int64)
        off = lambda l: (8 ** l - 1) // 7  # noqa: E731
        want = 0
        for g in samples.tolist():
            l = next(k for k in range(D + 1) if off(k) <= g < off(k + 1))
            d = 1 << l
            c = g - off(l)
            x, y, z = c % d, (c // d) % d, c // (d * d)
            tot = 0
            for dz in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dx in (-1, 0, 1):
                        X, Y, Z = x + dx, y + dy, z + dz
                        if 0 <= X < d and 0 <= Y < d and 0 <= Z < d:
                            tot += int(counts[off(l) + X + d * (Y + d * Z)])
            want += tot - 1
        assert want > 0
        assert roofline.p2p_pairs(st.moments, D) == want, kind
