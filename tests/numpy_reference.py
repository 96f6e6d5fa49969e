"""Independent numpy restatement of the reference compute passes (test helper).

Written from src/rainbow_fmm.wgsl directly, vectorised over cells and bodies,
to cross-check the C oracle (oracle/rfmm_oracle.c) on small scenes.  It uses
the same floating-point definition as the oracle: float32 round-to-nearest
with one rounding per operation (numpy never fuses), IEEE division and sqrt,
left-to-right evaluation, fmin/fmax clamps, ties-to-even rounding, wrapping
32-bit moment sums.
"""
import numpy as np

F = np.float32
HALF = F(1.6)                      # WORLD_HALF_EXTENT (wgsl:12)
CAP = 16                           # ADAPTIVE_LEAF_CAPACITY (wgsl:10)


def level_offset(l):
    return ((1 << (3 * l)) - 1) // 7


def clamp(x, lo, hi):
    return np.fmin(np.fmax(x, F(lo)), F(hi))


def position_cell(pos, dim):  # wgsl:144-152
    n = clamp(pos / HALF, -0.99999, 0.99999)
    return np.floor((n * F(0.5) + F(0.5)) * F(dim)).astype(np.int64)


def cell_center(c, dim):  # wgsl:136-142
    w = F(2.0) / F(dim)
    return ((c.astype(F) + F(0.5)) * w - F(1.0)) * HALF


def lin(c, dim):
    return c[..., 0] + dim * (c[..., 1] + dim * c[..., 2])


def coords(local, dim):  # wgsl:128-134
    z = local // (dim * dim)
    rest = local - z * dim * dim
    y = rest // dim
    return np.stack([rest - y * dim, y, z], axis=-1)


def i32_round(x):
    r = np.rint(x.astype(F)).astype(np.float64)
    r = np.where(np.isnan(r), 0.0, r)
    return np.clip(r, -2147483648.0, 2147483647.0).astype(np.int64)


def deposit(pos, depth, scale):  # wgsl:408-422 (after clear_cells)
    cells = level_offset(depth + 1)
    mom = np.zeros((cells, 4), np.uint32)
    dim = 1 << depth
    idx = level_offset(depth) + lin(position_cell(pos, dim), dim)
    np.add.at(mom[:, 0], idx, np.uint32(1))
    for k in range(3):
        q = i32_round(pos[:, k] * F(scale)).astype(np.int32).view(np.uint32)
        np.add.at(mom[:, k + 1], idx, q)
    return mom


def upward(mom, depth):  # wgsl:424-455, levels depth-1 .. 0
    for l in range(depth - 1, -1, -1):
        dim = 1 << l
        c = coords(np.arange(1 << (3 * l)), dim)
        acc = np.zeros((len(c), 4), np.uint32)
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    ch = level_offset(l + 1) + lin(c * 2 + np.array([dx, dy, dz]), dim * 2)
                    acc += mom[ch]
        mom[level_offset(l): level_offset(l) + len(c)] = acc
    return mom


def sources(mom, n, scale, gravity):
    count = mom[:, 0]
    inv = F(1.0) / (F(scale) * count.astype(F))
    com = mom[:, 1:].view(np.int32).astype(F) * inv[:, None]
    gm = F(gravity) * (count.astype(F) / F(n))
    return count, com, gm


def pair_field(com, gm, tgt, eps):  # wgsl:170-203 (non-empty sources)
    r = com - tgt
    r2 = (r[:, 0] * r[:, 0] + r[:, 1] * r[:, 1]) + r[:, 2] * r[:, 2] + eps * eps
    inv_r = F(1.0) / np.sqrt(r2)
    inv_r3 = inv_r * inv_r * inv_r
    inv_r5 = inv_r3 * inv_r * inv_r
    diag = -gm * inv_r3
    tidal = F(3.0) * gm * inv_r5
    out = np.zeros((len(r), 12), F)
    for k in range(3):
        out[:, k] = gm * r[:, k] * inv_r3
    out[:, 3] = -gm * inv_r
    out[:, 4] = diag + tidal * r[:, 0] * r[:, 0]
    out[:, 5] = tidal * r[:, 0] * r[:, 1]
    out[:, 6] = tidal * r[:, 0] * r[:, 2]
    out[:, 7] = diag + tidal * r[:, 1] * r[:, 1]
    out[:, 8] = tidal * r[:, 1] * r[:, 2]
    out[:, 9] = diag + tidal * r[:, 2] * r[:, 2]
    return out


def accumulate(result, rows, sel, contrib):
    """result[rows[sel]] += contrib (float32, one add per row)."""
    idx = rows[sel]
    result[idx] = result[idx] + contrib


def solve_fields(pos, n, depth, scale, gravity, softening):
    """clear, deposit, upward, m2l_all, downward, near_all (native/main.rs:437-449)."""
    mom = upward(deposit(pos, depth, scale), depth)
    count, com, gm = sources(mom, n, scale, gravity)
    cells = level_offset(depth + 1)
    fields = np.zeros((cells, 12), F)
    for l in range(1, depth + 1):  # m2l_all (wgsl:457-519), all levels
        dim = 1 << l
        off = level_offset(l)
        local = np.arange(1 << (3 * l))
        tc = coords(local, dim)
        pc = tc // 2
        parent = level_offset(l - 1) + lin(pc, dim // 2)
        live = (count[off + local] != 0) & (count[parent].astype(np.int64) > CAP)
        rows = off + local[live]
        tcl, pcl = tc[live], pc[live]
        tgt = cell_center(tcl, dim)
        eps = F(0.06) * HALF / F(dim)
        res = np.zeros((len(rows), 12), F)
        for pz in (-1, 0, 1):
            for py in (-1, 0, 1):
                for px in (-1, 0, 1):
                    sp = pcl + np.array([px, py, pz])
                    okp = np.all((sp >= 0) & (sp < dim // 2), axis=1)
                    for cz in (0, 1):
                        for cy in (0, 1):
                            for cx in (0, 1):
                                sc = sp * 2 + np.array([cx, cy, cz])
                                ok = okp & np.all((sc >= 0) & (sc < dim), axis=1)
                                ok &= ~np.all(np.abs(sc - tcl) <= 1, axis=1)
                                src = off + lin(np.where(ok[:, None], sc, 0), dim)
                                ok &= count[src] != 0
                                sel = np.nonzero(ok)[0]
                                if len(sel):
                                    pf = pair_field(com[src[sel]], gm[src[sel]], tgt[sel], eps)
                                    res[sel] = res[sel] + pf
        fields[rows] = res
    for l in range(1, depth + 1):  # downward (wgsl:585-611)
        dim = 1 << l
        off = level_offset(l)
        local = np.arange(1 << (3 * l))
        c = coords(local, dim)
        pc = c // 2
        parent = level_offset(l - 1) + lin(pc, dim // 2)
        live = (count[off + local] != 0) & (count[parent].astype(np.int64) > CAP)
        rows = off + local[live]
        pf = fields[parent[live]]
        delta = cell_center(c[live], dim) - cell_center(pc[live], dim // 2)
        inh = pf.copy()
        j = pf
        jd0 = j[:, 4] * delta[:, 0] + j[:, 5] * delta[:, 1] + j[:, 6] * delta[:, 2]
        jd1 = j[:, 5] * delta[:, 0] + j[:, 7] * delta[:, 1] + j[:, 8] * delta[:, 2]
        jd2 = j[:, 6] * delta[:, 0] + j[:, 8] * delta[:, 1] + j[:, 9] * delta[:, 2]
        inh[:, 0] = pf[:, 0] + jd0
        inh[:, 1] = pf[:, 1] + jd1
        inh[:, 2] = pf[:, 2] + jd2
        inh[:, 3] = pf[:, 3] - ((pf[:, 0] * delta[:, 0] + pf[:, 1] * delta[:, 1]) + pf[:, 2] * delta[:, 2])
        fields[rows] = fields[rows] + inh
    for l in range(1, depth + 1):  # near_all (wgsl:521-572)
        dim = 1 << l
        off = level_offset(l)
        local = np.arange(1 << (3 * l))
        tc = coords(local, dim)
        parent = level_offset(l - 1) + lin(tc // 2, dim // 2)
        tcount = count[off + local]
        live = (tcount != 0) & (count[parent].astype(np.int64) > CAP) & ((tcount <= CAP) | (l == depth))
        rows = off + local[live]
        tcl = tc[live]
        tgt = cell_center(tcl, dim)
        eps = np.fmax(F(softening), F(0.72) * HALF / F(dim))
        res = fields[rows].copy()
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    if dx == 0 and dy == 0 and dz == 0:
                        continue
                    sc = tcl + np.array([dx, dy, dz])
                    ok = np.all((sc >= 0) & (sc < dim), axis=1)
                    src = off + lin(np.where(ok[:, None], sc, 0), dim)
                    ok &= count[src] != 0
                    sel = np.nonzero(ok)[0]
                    if len(sel):
                        res[sel] = res[sel] + pair_field(com[src[sel]], gm[src[sel]], tgt[sel], eps)
        fields[rows] = res
    return mom, fields


def integrate(part, mom, fields, n, depth, scale, gravity, softening, dt, speed=1.0):
    """wgsl:613-771 with the control field off."""
    pos = part[:, 0:3].astype(F)
    vel = part[:, 4:7].astype(F)
    count_all = mom[:, 0]
    chosen = np.full(n, -1, np.int64)
    cdim = np.zeros(n, np.int64)
    for l in range(1, depth + 1):
        dim = 1 << l
        idx = level_offset(l) + lin(position_cell(pos, dim), dim)
        ok = (chosen < 0) & ((count_all[idx].astype(np.int64).astype(np.int32) <= CAP) | (l == depth))
        chosen[ok] = idx[ok]
        cdim[ok] = dim
    cc = np.zeros((n, 3), np.int64)
    for dim in np.unique(cdim):
        sel = cdim == dim
        cc[sel] = position_cell(pos[sel], int(dim))
    center = np.zeros((n, 3), F)
    for dim in np.unique(cdim):
        sel = cdim == dim
        center[sel] = cell_center(cc[sel], int(dim))
    f = fields[chosen]
    d = pos - center
    acc = np.stack([
        f[:, 0] + (f[:, 4] * d[:, 0] + f[:, 5] * d[:, 1] + f[:, 6] * d[:, 2]),
        f[:, 1] + (f[:, 5] * d[:, 0] + f[:, 7] * d[:, 1] + f[:, 8] * d[:, 2]),
        f[:, 2] + (f[:, 6] * d[:, 0] + f[:, 8] * d[:, 1] + f[:, 9] * d[:, 2]),
    ], axis=1)
    count = count_all[chosen]
    many = count > 1
    inv = F(1.0) / (F(scale) * count.astype(F))
    com = mom[chosen, 1:].view(np.int32).astype(F) * inv[:, None]
    delta = com - pos
    eps = np.fmax(F(softening), (F(0.62) * HALF) / cdim.astype(F))
    inv_r = F(1.0) / np.sqrt((delta[:, 0] * delta[:, 0] + delta[:, 1] * delta[:, 1]) + delta[:, 2] * delta[:, 2] + eps * eps)
    self_mass = (count.astype(np.int64) - 1).clip(0).astype(F) / F(n)
    for k in range(3):
        add = F(gravity) * self_mass * delta[:, k] * inv_r * inv_r * inv_r
        acc[:, k] = np.where(many, acc[:, k] + add, acc[:, k])
    dtv = F(dt) * F(speed)

    def length(v):
        return np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2])

    radius = np.fmax(length(pos), F(0.0001))
    vlen = np.fmax(length(vel), F(0.0001))
    pv = (pos[:, 0] * vel[:, 0] + pos[:, 1] * vel[:, 1]) + pos[:, 2] * vel[:, 2]
    srm = clamp(pv / (radius * vlen), -1.0, 1.0)
    rf = np.abs(srm)
    shock = rf * rf * rf
    pulse = clamp((count.astype(F) - F(CAP)) / F(72.0), 0.0, 1.0)
    strength = clamp(length(acc) * (radius + F(0.12)) * F(0.58), 0.0, 1.0)
    ci = F(0.0)
    target = clamp(F(0.025) + shock * F(0.56) + pulse * F(0.26) + strength * F(0.13) + ci * F(0.42), 0.0, 1.0)
    exc = part[:, 7].astype(F)
    response = np.where(target > exc, F(10.0), F(1.05)).astype(F)
    t = clamp(dtv * response, 0.0, 1.0)
    exc = exc * (F(1.0) - t) + target * t
    vel = vel + acc * dtv
    pos = pos + vel * dtv
    edge = HALF * F(0.985)
    band = F(0.12) * HALF
    for k in range(3):
        over = np.abs(pos[:, k]) - (edge - band)
        absorb = clamp(over / band, 0.0, 1.0)
        vel[:, k] = np.where(over > F(0), vel[:, k] * (F(1.0) - absorb * F(0.16)), vel[:, k])
        out = np.abs(pos[:, k]) > edge
        pos[:, k] = np.where(out, clamp(pos[:, k], -float(edge), float(edge)), pos[:, k])
        vel[:, k] = np.where(out, vel[:, k] * F(-0.55), vel[:, k])
    st = clamp((exc - F(0.30)) / (F(0.70) - F(0.30)), 0.0, 1.0)
    drift = F(1.0) - st * st * (F(3.0) - F(2.0) * st)
    h = part[:, 3].astype(F) + dtv * drift * (F(0.012) + srm * F(0.030) + exc * F(0.036) + ci * F(0.080))
    hue = h - np.floor(h)
    out = np.empty_like(part)
    out[:, 0:3], out[:, 3], out[:, 4:7], out[:, 7] = pos, hue, vel, exc
    return out
