/*
 * rfmm_oracle.c -- CPU oracle for the p=1 Cartesian FMM step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only the tests, the
 * smoke check and the CPU-baseline leg of bench.py load it.  The product
 * library never links, loads or calls it.
 *
 * It restates, pass by pass and in the reference's loop order, the compute
 * shader of iskamag/fmm-rainbow:
 *   planner            src/lib.rs:10-86
 *   helper functions   src/rainbow_fmm.wgsl:100-203
 *   initialize         src/rainbow_fmm.wgsl:205-374
 *   clear_cells        src/rainbow_fmm.wgsl:394-406
 *   deposit (P2M)      src/rainbow_fmm.wgsl:408-422
 *   upward (M2M)       src/rainbow_fmm.wgsl:424-455
 *   m2l_all            src/rainbow_fmm.wgsl:457-519
 *   near_all           src/rainbow_fmm.wgsl:521-572
 *   downward (L2L)     src/rainbow_fmm.wgsl:574-611
 *   integrate          src/rainbow_fmm.wgsl:613-771
 * and the native harness's frame order and content digest
 * (native/main.rs:362-421 and 152-163).
 *
 * Floating-point definition (the reference leaves these to the WebGPU
 * implementation, so this oracle fixes them; the CUDA kernels follow the
 * same definition):
 *   - IEEE-754 binary32, round to nearest even, no fused multiply-add
 *     (build with -ffp-contract=off), denormals preserved;
 *   - vector expressions evaluate left to right, component by component;
 *     dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z;
 *   - inverseSqrt(x) = 1 / sqrt(x), both correctly rounded;
 *   - round() is ties-to-even (rintf); i32(f32) saturates, NaN -> 0;
 *   - clamp(x, lo, hi) = fminf(fmaxf(x, lo), hi); mix(a, b, t) =
 *     a*(1-t) + b*t; smoothstep(l, h, x) with t = clamp((x-l)/(h-l), 0, 1)
 *     and t*t*(3-2t); fract(x) = x - floor(x);
 *   - integer moment sums wrap modulo 2^32 (i32 atomics in the reference).
 * The transcendentals of `initialize`, of the control field and of the display
 * passes are not the reference's (WGSL leaves them implementation-defined) but
 * the contract's own binary32 functions (fmm-rainbow_gb300/csrc/rfmm_math.h,
 * shared with the kernels; their accuracy against libm is tested separately),
 * so those paths match the GPU bit for bit too.
 *
 * Pinning: the planner is pinned to the reference's own unit tests
 * (src/lib.rs:163-217).  The passes are pinned to the reference's own shader
 * code: oracle/wgsl_transpile.py translates the compute entry points of
 * src/rainbow_fmm.wgsl into C++, oracle/wgsl_ref_harness.cpp runs them in the
 * native harness's dispatch order, and this oracle reproduces the digests of
 * that execution bit for bit (tests/test_reference_golden.py against
 * tests/golden/reference_wgsl_digests.json).  The float definitions above are
 * the one thing the two share: WGSL leaves them to the implementation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "rfmm_math.h" /* the contract's sin/cos/exp/pow/atan2, shared with the kernels */

#ifdef _OPENMP
#include <omp.h>
#endif

#define O_MIN_DEPTH 4u
#define O_MAX_DEPTH 6u
#define O_MIN_PARTICLES (1u << 14)
#define O_MAX_PARTICLES (1u << 23)
#define O_LEAF_TARGET 8u
#define O_HALF 1.60f                      /* WORLD_HALF_EXTENT, wgsl:12 */
#define O_ADAPTIVE 16u                    /* ADAPTIVE_LEAF_CAPACITY, wgsl:10 */
#define O_TAU 6.28318530718f              /* wgsl:9 */

typedef struct {
  float px, py, pz, hue; /* pos_light */
  float vx, vy, vz, exc; /* vel_hue */
} OParticle;

typedef struct {
  uint32_t count;
  int32_t sx, sy, sz;
} OMoment;

typedef struct {
  float a[4];  /* acceleration xyz, potential */
  float j0[4]; /* Jxx Jxy Jxz Jyy */
  float j1[4]; /* Jyz Jzz pad pad */
} OField;

/* The compute-relevant subset of `struct Params` (wgsl:18-50). */
typedef struct {
  uint32_t n;      /* particle_count */
  uint32_t depth;  /* depth */
  float scale;     /* control_settings.z */
  float dt;
  float gravity;
  float softening;
  float speed;
  float control_point[4];
  float control_axis_mode[4];
  float control_strength; /* control_settings.x */
  float control_radius;   /* control_settings.y */
  uint32_t near_mode;     /* 0: reference near field; 1: exact P2P (no reference counterpart) */
} OParams;

#define O_NEAR_P2P 1u

/* ---------------------------------------------------------------- planner */

static uint32_t o_level_cells(uint32_t l) { return 1u << (3u * l); }
static uint32_t o_level_offset(uint32_t l) { return (o_level_cells(l) - 1u) / 7u; }

uint32_t oracle_level_cells(uint32_t l) { return o_level_cells(l); }
uint32_t oracle_level_offset(uint32_t l) { return o_level_offset(l); }
uint32_t oracle_total_cells(uint32_t depth) { return o_level_offset(depth + 1u); }

uint32_t oracle_depth_for_particles(uint32_t particles) { /* lib.rs:45-52 */
  uint32_t target = (uint32_t)(((uint64_t)particles + O_LEAF_TARGET - 1u) / O_LEAF_TARGET);
  uint32_t d = O_MIN_DEPTH;
  while (d < O_MAX_DEPTH && o_level_cells(d) < target) d++;
  return d;
}

float oracle_fixed_point_scale(uint32_t particles) { /* lib.rs:59-69 */
  double worst = (double)particles * (double)O_HALF;
  double max_scale = 0.82 * 2147483647.0 / (worst > 1.0 ? worst : 1.0);
  return (float)pow(2.0, floor(log2(max_scale)));
}

uint32_t oracle_clamp_particle_count(uint32_t r) { /* lib.rs:71-79 */
  return r < O_MIN_PARTICLES ? O_MIN_PARTICLES : (r > O_MAX_PARTICLES ? O_MAX_PARTICLES : r);
}

uint64_t oracle_linear_work_bound(uint32_t particles, uint32_t depth) { /* lib.rs:83-86 */
  return (uint64_t)particles * 3u + (uint64_t)oracle_total_cells(depth) * 199u;
}

/* -------------------------------------------------------------- helpers */

static float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

static int32_t f2i_sat(float x) { /* i32(round(x)) with saturation */
  float r = rintf(x);
  if (r != r) return 0;
  if (r >= 2147483648.0f) return INT32_MAX;
  if (r < -2147483648.0f) return INT32_MIN;
  return (int32_t)r;
}

static void cell_coord(uint32_t index, uint32_t dim, uint32_t c[3]) { /* wgsl:128-134 */
  uint32_t plane = dim * dim;
  uint32_t z = index / plane;
  uint32_t rest = index - z * plane;
  uint32_t y = rest / dim;
  c[0] = rest - y * dim;
  c[1] = y;
  c[2] = z;
}

static uint32_t linear_index(const uint32_t c[3], uint32_t dim) { /* wgsl:120-122 */
  return c[0] + dim * (c[1] + dim * c[2]);
}

static void cell_center(const uint32_t c[3], uint32_t dim, float out[3]) { /* wgsl:136-142 */
  float w = 2.0f / (float)dim;
  for (int k = 0; k < 3; k++) out[k] = (((float)c[k] + 0.5f) * w - 1.0f) * O_HALF;
}

static void position_cell(const float p[3], uint32_t dim, uint32_t c[3]) { /* wgsl:144-152 */
  for (int k = 0; k < 3; k++) {
    float n = clampf(p[k] / O_HALF, -0.99999f, 0.99999f);
    c[k] = (uint32_t)floorf((n * 0.5f + 0.5f) * (float)dim);
  }
}

static uint32_t level_of(uint32_t g) { /* wgsl:380-392 */
  uint32_t level = 1u, start = 1u;
  for (;;) {
    uint32_t cells = 1u << (3u * level);
    if (g < start + cells) break;
    start += cells;
    level++;
  }
  return level;
}

static void moment_com(const OMoment *m, uint32_t count, float scale, float out[3]) { /* wgsl:163-168 */
  float inv = 1.0f / (scale * (float)count);
  out[0] = (float)m->sx * inv;
  out[1] = (float)m->sy * inv;
  out[2] = (float)m->sz * inv;
}

static void zero_field(OField *f) { memset(f, 0, sizeof(*f)); }

static void add_field(OField *acc, const OField *b) { /* wgsl:108-110 */
  for (int k = 0; k < 4; k++) {
    acc->a[k] = acc->a[k] + b->a[k];
    acc->j0[k] = acc->j0[k] + b->j0[k];
    acc->j1[k] = acc->j1[k] + b->j1[k];
  }
}

static void field_j_mul(const OField *f, const float v[3], float out[3]) { /* wgsl:112-118 */
  out[0] = f->j0[0] * v[0] + f->j0[1] * v[1] + f->j0[2] * v[2];
  out[1] = f->j0[1] * v[0] + f->j0[3] * v[1] + f->j1[0] * v[2];
  out[2] = f->j0[2] * v[0] + f->j1[0] * v[1] + f->j1[1] * v[2];
}

static void pair_field(const OMoment *moments, uint32_t source, const float tgt[3], float eps,
                       const OParams *P, OField *out) { /* wgsl:170-203 */
  uint32_t count = moments[source].count;
  if (count == 0u) {
    zero_field(out);
    return;
  }
  float src[3], r[3];
  moment_com(&moments[source], count, P->scale, src);
  for (int k = 0; k < 3; k++) r[k] = src[k] - tgt[k];
  float r2 = (r[0] * r[0] + r[1] * r[1]) + r[2] * r[2] + eps * eps;
  float inv_r = 1.0f / sqrtf(r2);
  float inv_r3 = inv_r * inv_r * inv_r;
  float inv_r5 = inv_r3 * inv_r * inv_r;
  float mass = (float)count / (float)P->n;
  float gm = P->gravity * mass;
  float diagonal = -gm * inv_r3;
  float tidal = 3.0f * gm * inv_r5;
  out->a[0] = gm * r[0] * inv_r3;
  out->a[1] = gm * r[1] * inv_r3;
  out->a[2] = gm * r[2] * inv_r3;
  out->a[3] = -gm * inv_r;
  out->j0[0] = diagonal + tidal * r[0] * r[0];
  out->j0[1] = tidal * r[0] * r[1];
  out->j0[2] = tidal * r[0] * r[2];
  out->j0[3] = diagonal + tidal * r[1] * r[1];
  out->j1[0] = tidal * r[1] * r[2];
  out->j1[1] = diagonal + tidal * r[2] * r[2];
  out->j1[2] = 0.0f;
  out->j1[3] = 0.0f;
}

/* ------------------------------------------------------------ the passes */

void oracle_clear(OMoment *moments, uint32_t cells) { /* wgsl:394-406 */
  memset(moments, 0, (size_t)cells * sizeof(OMoment));
}

/* Leaf cell (global index) of a body, and its fixed-point position. */
static uint32_t deposit_cell(const OParticle *p, uint32_t depth) {
  uint32_t dim = 1u << depth, c[3];
  float pos[3] = {p->px, p->py, p->pz};
  position_cell(pos, dim, c);
  return o_level_offset(depth) + linear_index(c, dim);
}

uint32_t oracle_leaf_of(const OParticle *p, uint32_t depth) { return deposit_cell(p, depth); }

void oracle_deposit(const OParticle *particles, OMoment *moments, const OParams *P) { /* wgsl:408-422 */
  const uint32_t n = P->n, depth = P->depth;
  const uint32_t leaf0 = o_level_offset(depth), leaves = o_level_cells(depth);
#ifdef _OPENMP
  int nt = omp_get_max_threads();
#else
  int nt = 1;
#endif
  if (nt > 1 && n >= 65536u) {
    /* Integer sums are exact modulo 2^32, so per-thread partial histograms
     * summed in any order equal the reference's atomics bit for bit. */
    uint32_t *part = (uint32_t *)calloc((size_t)nt * leaves * 4u, sizeof(uint32_t));
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
      int t = omp_get_thread_num();
#else
      int t = 0;
#endif
      uint32_t *mine = part + (size_t)t * leaves * 4u;
#pragma omp for schedule(static)
      for (int64_t i = 0; i < (int64_t)n; i++) {
        const OParticle *p = &particles[i];
        uint32_t cell = deposit_cell(p, depth) - leaf0;
        float fp = P->scale;
        mine[cell * 4u + 0] += 1u;
        mine[cell * 4u + 1] += (uint32_t)f2i_sat(p->px * fp);
        mine[cell * 4u + 2] += (uint32_t)f2i_sat(p->py * fp);
        mine[cell * 4u + 3] += (uint32_t)f2i_sat(p->pz * fp);
      }
#pragma omp for schedule(static)
      for (int64_t c = 0; c < (int64_t)leaves; c++) {
        uint32_t acc[4] = {0, 0, 0, 0};
        for (int s = 0; s < nt; s++)
          for (int k = 0; k < 4; k++) acc[k] += part[((size_t)s * leaves + (size_t)c) * 4u + k];
        OMoment *m = &moments[leaf0 + c];
        m->count += acc[0];
        m->sx = (int32_t)((uint32_t)m->sx + acc[1]);
        m->sy = (int32_t)((uint32_t)m->sy + acc[2]);
        m->sz = (int32_t)((uint32_t)m->sz + acc[3]);
      }
    }
    free(part);
    return;
  }
  for (uint32_t i = 0; i < n; i++) {
    const OParticle *p = &particles[i];
    OMoment *m = &moments[deposit_cell(p, depth)];
    float fp = P->scale;
    m->count += 1u;
    m->sx = (int32_t)((uint32_t)m->sx + (uint32_t)f2i_sat(p->px * fp));
    m->sy = (int32_t)((uint32_t)m->sy + (uint32_t)f2i_sat(p->py * fp));
    m->sz = (int32_t)((uint32_t)m->sz + (uint32_t)f2i_sat(p->pz * fp));
  }
}

static void upward_level(OMoment *moments, uint32_t level) { /* wgsl:424-455, one dispatch */
  const uint32_t dim = 1u << level, pdim = dim << 1;
  const uint32_t off = o_level_offset(level), coff = o_level_offset(level + 1u);
  const uint32_t cells = o_level_cells(level);
#pragma omp parallel for schedule(static) if (cells >= 4096u)
  for (int64_t li = 0; li < (int64_t)cells; li++) {
    uint32_t c[3];
    cell_coord((uint32_t)li, dim, c);
    uint32_t count = 0u, sx = 0u, sy = 0u, sz = 0u;
    for (uint32_t dz = 0; dz < 2u; dz++)
      for (uint32_t dy = 0; dy < 2u; dy++)
        for (uint32_t dx = 0; dx < 2u; dx++) {
          uint32_t cc[3] = {c[0] * 2u + dx, c[1] * 2u + dy, c[2] * 2u + dz};
          const OMoment *ch = &moments[coff + linear_index(cc, pdim)];
          count += ch->count;
          sx += (uint32_t)ch->sx;
          sy += (uint32_t)ch->sy;
          sz += (uint32_t)ch->sz;
        }
    OMoment *t = &moments[off + (uint32_t)li];
    t->count = count;
    t->sx = (int32_t)sx;
    t->sy = (int32_t)sy;
    t->sz = (int32_t)sz;
  }
}

void oracle_upward(OMoment *moments, const OParams *P) { /* levels depth-1 .. 0 */
  for (int l = (int)P->depth - 1; l >= 0; l--) upward_level(moments, (uint32_t)l);
}

void oracle_m2l_all(const OMoment *moments, OField *fields, const OParams *P) { /* wgsl:457-519 */
  const uint32_t total = oracle_total_cells(P->depth);
#pragma omp parallel for schedule(dynamic, 512)
  for (int64_t gg = 1; gg < (int64_t)total; gg++) {
    const uint32_t g = (uint32_t)gg;
    const uint32_t level = level_of(g);
    const uint32_t start = o_level_offset(level);
    const uint32_t local = g - start;
    const uint32_t dim = 1u << level, pdim = dim >> 1;
    uint32_t tc[3], pc[3];
    cell_coord(local, dim, tc);
    pc[0] = tc[0] / 2u;
    pc[1] = tc[1] / 2u;
    pc[2] = tc[2] / 2u;
    const uint32_t parent_index = o_level_offset(level - 1u) + linear_index(pc, pdim);
    if (moments[g].count == 0u || (int32_t)moments[parent_index].count <= (int32_t)O_ADAPTIVE) {
      zero_field(&fields[g]);
      continue;
    }
    float tgt[3];
    cell_center(tc, dim, tgt);
    const float cell_eps = 0.06f * O_HALF / (float)dim;
    OField result, pf;
    zero_field(&result);
    for (int pz = -1; pz <= 1; pz++)
      for (int py = -1; py <= 1; py++)
        for (int px = -1; px <= 1; px++) {
          int sp[3] = {(int)pc[0] + px, (int)pc[1] + py, (int)pc[2] + pz};
          if (sp[0] < 0 || sp[1] < 0 || sp[2] < 0 || sp[0] >= (int)pdim || sp[1] >= (int)pdim ||
              sp[2] >= (int)pdim)
            continue;
          for (int cz = 0; cz < 2; cz++)
            for (int cy = 0; cy < 2; cy++)
              for (int cx = 0; cx < 2; cx++) {
                int sc[3] = {sp[0] * 2 + cx, sp[1] * 2 + cy, sp[2] * 2 + cz};
                if (sc[0] < 0 || sc[1] < 0 || sc[2] < 0 || sc[0] >= (int)dim ||
                    sc[1] >= (int)dim || sc[2] >= (int)dim)
                  continue;
                if (abs(sc[0] - (int)tc[0]) <= 1 && abs(sc[1] - (int)tc[1]) <= 1 &&
                    abs(sc[2] - (int)tc[2]) <= 1)
                  continue;
                uint32_t scu[3] = {(uint32_t)sc[0], (uint32_t)sc[1], (uint32_t)sc[2]};
                pair_field(moments, start + linear_index(scu, dim), tgt, cell_eps, P, &pf);
                add_field(&result, &pf);
              }
        }
    fields[g] = result;
  }
}

void oracle_near_all(const OMoment *moments, OField *fields, const OParams *P) { /* wgsl:521-572 */
  const uint32_t total = oracle_total_cells(P->depth);
#pragma omp parallel for schedule(dynamic, 512)
  for (int64_t gg = 1; gg < (int64_t)total; gg++) {
    const uint32_t g = (uint32_t)gg;
    const uint32_t level = level_of(g);
    const uint32_t start = o_level_offset(level);
    const uint32_t dim = 1u << level, pdim = dim >> 1;
    const uint32_t target_count = moments[g].count;
    uint32_t tc[3], pc[3];
    cell_coord(g - start, dim, tc);
    pc[0] = tc[0] / 2u;
    pc[1] = tc[1] / 2u;
    pc[2] = tc[2] / 2u;
    const uint32_t parent_index = o_level_offset(level - 1u) + linear_index(pc, pdim);
    const int on_path = (int32_t)moments[parent_index].count > (int32_t)O_ADAPTIVE;
    if (target_count == 0u || !on_path || !(target_count <= O_ADAPTIVE || level == P->depth))
      continue;
    float tgt[3];
    cell_center(tc, dim, tgt);
    OField result = fields[g], pf;
    const float ce = 0.72f * O_HALF / (float)dim;
    const float near_eps = fmaxf(P->softening, ce);
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          if (dx == 0 && dy == 0 && dz == 0) continue;
          int sc[3] = {(int)tc[0] + dx, (int)tc[1] + dy, (int)tc[2] + dz};
          if (sc[0] < 0 || sc[1] < 0 || sc[2] < 0 || sc[0] >= (int)dim || sc[1] >= (int)dim ||
              sc[2] >= (int)dim)
            continue;
          uint32_t scu[3] = {(uint32_t)sc[0], (uint32_t)sc[1], (uint32_t)sc[2]};
          pair_field(moments, start + linear_index(scu, dim), tgt, near_eps, P, &pf);
          add_field(&result, &pf);
        }
    fields[g] = result;
  }
}

static void downward_level(const OMoment *moments, OField *fields, uint32_t level) { /* wgsl:574-611 */
  const uint32_t dim = 1u << level, pdim = dim >> 1;
  const uint32_t off = o_level_offset(level), poff = o_level_offset(level - 1u);
  const uint32_t cells = o_level_cells(level);
#pragma omp parallel for schedule(static) if (cells >= 4096u)
  for (int64_t li = 0; li < (int64_t)cells; li++) {
    const uint32_t t = off + (uint32_t)li;
    uint32_t c[3], pc[3];
    cell_coord((uint32_t)li, dim, c);
    pc[0] = c[0] / 2u;
    pc[1] = c[1] / 2u;
    pc[2] = c[2] / 2u;
    const uint32_t parent_index = poff + linear_index(pc, pdim);
    /* level >= 1 always here, so target_is_on_adaptive_path reads the parent */
    if (moments[t].count == 0u || !((int32_t)moments[parent_index].count > (int32_t)O_ADAPTIVE))
      continue;
    const OField pf = fields[parent_index];
    float cc[3], cp[3], delta[3], jd[3];
    cell_center(c, dim, cc);
    cell_center(pc, pdim, cp);
    for (int k = 0; k < 3; k++) delta[k] = cc[k] - cp[k];
    OField inherited = pf;
    field_j_mul(&pf, delta, jd);
    for (int k = 0; k < 3; k++) inherited.a[k] = pf.a[k] + jd[k];
    inherited.a[3] = pf.a[3] - ((pf.a[0] * delta[0] + pf.a[1] * delta[1]) + pf.a[2] * delta[2]);
    add_field(&fields[t], &inherited);
  }
}

void oracle_downward(const OMoment *moments, OField *fields, const OParams *P) {
  for (uint32_t l = 1u; l <= P->depth; l++) downward_level(moments, fields, l);
}

static float smoothstepf(float lo, float hi, float x) {
  float t = clampf((x - lo) / (hi - lo), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}

static float fractf(float x) { return x - floorf(x); }

static float length3(const float v[3]) { return sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]); }

/* ---------------------------------------------------- P2P near field */

/* The near-field P2P mode (no reference counterpart): the fields carry M2L
 * and L2L only, and each body adds the exact softened pair forces of every
 * body in the 3x3x3 cells around its sample cell.  Bodies are visited cell by
 * cell (z-, y-, x-major offsets -1..1) and, inside a cell, by the Morton code
 * of their leaf (x in bit 0) and then by index. */
typedef struct {
  const OParticle *snap; /* positions the sums read (the state before the step) */
  uint32_t *order;       /* body indices sorted by (leaf Morton code, index) */
  uint32_t *starts;      /* 8^depth + 1 entries: first rank of each leaf code */
} ONear;

static uint32_t spread3(uint32_t v) {
  uint32_t r = 0;
  for (uint32_t b = 0; b < 10u; b++) r |= ((v >> b) & 1u) << (3u * b);
  return r;
}

static uint32_t morton3(const uint32_t c[3]) {
  return spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2);
}

static void near_build(const OParticle *particles, const OParams *P, ONear *nr) {
  const uint32_t n = P->n, depth = P->depth, dim = 1u << depth, leaves = 1u << (3u * depth);
  uint32_t *code = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1u));
  nr->snap = particles;
  nr->order = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1u));
  nr->starts = (uint32_t *)calloc(leaves + 1u, sizeof(uint32_t));
  for (uint32_t i = 0; i < n; i++) {
    float pos[3] = {particles[i].px, particles[i].py, particles[i].pz};
    uint32_t c[3];
    position_cell(pos, dim, c);
    code[i] = morton3(c);
    nr->starts[code[i] + 1u]++;
  }
  for (uint32_t m = 0; m < leaves; m++) nr->starts[m + 1u] += nr->starts[m];
  uint32_t *fill = (uint32_t *)malloc(sizeof(uint32_t) * leaves);
  memcpy(fill, nr->starts, sizeof(uint32_t) * leaves);
  for (uint32_t i = 0; i < n; i++) nr->order[fill[code[i]]++] = i; /* stable: by index */
  free(fill);
  free(code);
}

static void near_free(ONear *nr) {
  free(nr->order);
  free(nr->starts);
}

/* Sums over the 3x3x3 cells at `level` around cell c; gm * sum is added. */
static void near_p2p(const ONear *nr, const OParams *P, uint32_t self, const float pos[3],
                     uint32_t level, const uint32_t c[3], float s[3]) {
  const int dim = 1 << level;
  const uint32_t sh3 = 3u * (P->depth - level);
  const float eps2 = P->softening * P->softening;
  s[0] = s[1] = s[2] = 0.0f;
  for (int oz = -1; oz <= 1; oz++)
    for (int oy = -1; oy <= 1; oy++)
      for (int ox = -1; ox <= 1; ox++) {
        const int nx = (int)c[0] + ox, ny = (int)c[1] + oy, nz = (int)c[2] + oz;
        if (nx < 0 || ny < 0 || nz < 0 || nx >= dim || ny >= dim || nz >= dim) continue;
        const uint32_t nc[3] = {(uint32_t)nx, (uint32_t)ny, (uint32_t)nz};
        const uint32_t m = morton3(nc);
        const uint32_t lo = nr->starts[m << sh3], hi = nr->starts[(m + 1u) << sh3];
        for (uint32_t k = lo; k < hi; k++) {
          const uint32_t j = nr->order[k];
          if (j == self) continue;
          const OParticle *q = &nr->snap[j];
          const float d[3] = {q->px - pos[0], q->py - pos[1], q->pz - pos[2]};
          const float r2 = ((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) + eps2;
          const float inv = 1.0f / sqrtf(r2);
          const float w = (inv * inv) * inv;
          for (int a = 0; a < 3; a++) s[a] = s[a] + d[a] * w;
        }
      }
}

/* The FMM acceleration integrate applies before the control field
 * (wgsl:619-657): adaptive descent, local expansion, self-leaf monopole (or,
 * with `nr`, the P2P near field of body `self`).  Returns the chosen cell's
 * count. */
static uint32_t fmm_acceleration(const OParticle *particle, const OMoment *moments,
                                 const OField *fields, const OParams *P, float acc[3],
                                 const ONear *nr, uint32_t self) {
  const uint32_t depth = P->depth;
  float pos[3] = {particle->px, particle->py, particle->pz};
  uint32_t chosen_dim = 1u << depth, chosen_cell[3], cell_index;
  position_cell(pos, chosen_dim, chosen_cell);
  cell_index = o_level_offset(depth) + linear_index(chosen_cell, chosen_dim);
  for (uint32_t level = 1u; level <= depth; level++) {
    uint32_t dim = 1u << level, c[3];
    position_cell(pos, dim, c);
    uint32_t index = o_level_offset(level) + linear_index(c, dim);
    int32_t count_at_level = (int32_t)moments[index].count;
    if (count_at_level <= (int32_t)O_ADAPTIVE || level == depth) {
      chosen_dim = dim;
      chosen_cell[0] = c[0];
      chosen_cell[1] = c[1];
      chosen_cell[2] = c[2];
      cell_index = index;
      break;
    }
  }
  float center[3], rel[3], jm[3];
  cell_center(chosen_cell, chosen_dim, center);
  const OField *field = &fields[cell_index];
  for (int k = 0; k < 3; k++) rel[k] = pos[k] - center[k];
  field_j_mul(field, rel, jm);
  for (int k = 0; k < 3; k++) acc[k] = field->a[k] + jm[k];

  const uint32_t count = moments[cell_index].count;
  if (nr != NULL) {
    uint32_t level = 0;
    while ((1u << level) != chosen_dim) level++;
    float s[3];
    near_p2p(nr, P, self, pos, level, chosen_cell, s);
    const float gm = P->gravity / (float)P->n;
    for (int k = 0; k < 3; k++) acc[k] = acc[k] + gm * s[k];
    return count;
  }
  if (count > 1u) {
    float com[3], delta[3];
    moment_com(&moments[cell_index], count, P->scale, com);
    for (int k = 0; k < 3; k++) delta[k] = com[k] - pos[k];
    const float ce = 0.62f * O_HALF / (float)chosen_dim;
    const float eps = fmaxf(P->softening, ce);
    const float inv_r =
        1.0f / sqrtf((delta[0] * delta[0] + delta[1] * delta[1]) + delta[2] * delta[2] + eps * eps);
    const float self_mass = (float)(count - 1u) / (float)P->n;
    for (int k = 0; k < 3; k++)
      acc[k] = acc[k] + P->gravity * self_mass * delta[k] * inv_r * inv_r * inv_r;
  }
  return count;
}

/* FMM accelerations of every body (no update). */
void oracle_accelerations(const OParticle *particles, const OMoment *moments, const OField *fields,
                          const OParams *P, float *acc_out) {
  ONear nr;
  const int p2p = P->near_mode == O_NEAR_P2P;
  if (p2p) near_build(particles, P, &nr);
#pragma omp parallel for schedule(dynamic, 256) if (P->n >= 8192u)
  for (int64_t i = 0; i < (int64_t)P->n; i++)
    fmm_acceleration(&particles[i], moments, fields, P, &acc_out[3 * i], p2p ? &nr : NULL,
                     (uint32_t)i);
  if (p2p) near_free(&nr);
}

void oracle_integrate(OParticle *particles, const OMoment *moments, const OField *fields,
                      const OParams *P) { /* wgsl:613-771 */
  const uint32_t n = P->n;
  /* P2P reads every body's pre-step position: sums run on a snapshot. */
  ONear nr;
  OParticle *snap = NULL;
  const int p2p = P->near_mode == O_NEAR_P2P;
  if (p2p) {
    snap = (OParticle *)malloc(sizeof(OParticle) * (n ? n : 1u));
    memcpy(snap, particles, sizeof(OParticle) * n);
    near_build(snap, P, &nr);
  }
#pragma omp parallel for schedule(dynamic, 256) if (n >= 8192u)
  for (int64_t ii = 0; ii < (int64_t)n; ii++) {
    OParticle particle = particles[ii];
    float pos[3] = {particle.px, particle.py, particle.pz};
    float velocity[3] = {particle.vx, particle.vy, particle.vz};
    float acc[3];
    const uint32_t count =
        fmm_acceleration(&particle, moments, fields, P, acc, p2p ? &nr : NULL, (uint32_t)ii);

    float control_influence = 0.0f;
    if (P->control_point[3] > 0.5f) { /* wgsl:659-689 */
      float cd[3];
      for (int k = 0; k < 3; k++) cd[k] = P->control_point[k] - pos[k];
      const float d2 = (cd[0] * cd[0] + cd[1] * cd[1]) + cd[2] * cd[2];
      const float cr = fmaxf(P->control_radius, 0.02f);
      control_influence = rf_expf(-2.0f * d2 / (cr * cr));
      const float strength = P->control_strength;
      const float inv = 1.0f / sqrtf(d2 + cr * cr * 0.018f);
      float dir[3] = {cd[0] * inv, cd[1] * inv, cd[2] * inv};
      const float mode = P->control_axis_mode[3];
      if (mode < 1.5f) {
        for (int k = 0; k < 3; k++) acc[k] = acc[k] + dir[k] * strength * control_influence;
      } else if (mode < 2.5f) {
        for (int k = 0; k < 3; k++) acc[k] = acc[k] - dir[k] * strength * control_influence;
      } else {
        float ax[3] = {P->control_axis_mode[0], P->control_axis_mode[1], P->control_axis_mode[2]};
        const float al = length3(ax);
        for (int k = 0; k < 3; k++) ax[k] = ax[k] / al;
        float tg[3] = {ax[1] * cd[2] - ax[2] * cd[1], ax[2] * cd[0] - ax[0] * cd[2],
                       ax[0] * cd[1] - ax[1] * cd[0]};
        const float tl = length3(tg);
        if (tl > 0.00001f)
          for (int k = 0; k < 3; k++) acc[k] = acc[k] + tg[k] / tl * strength * control_influence;
      }
    }

    const float dt = P->dt * P->speed; /* wgsl:693 */
    const float radius = fmaxf(length3(pos), 0.0001f);
    const float velocity_length = fmaxf(length3(velocity), 0.0001f);
    const float pv = (pos[0] * velocity[0] + pos[1] * velocity[1]) + pos[2] * velocity[2];
    const float signed_radial = clampf(pv / (radius * velocity_length), -1.0f, 1.0f);
    const float radial_fraction = fabsf(signed_radial);
    const float radial_shock = radial_fraction * radial_fraction * radial_fraction;
    const float density_pulse = clampf(((float)count - (float)O_ADAPTIVE) / 72.0f, 0.0f, 1.0f);
    const float field_strength = clampf(length3(acc) * (radius + 0.12f) * 0.58f, 0.0f, 1.0f);
    const float target_exc =
        clampf(0.025f + radial_shock * 0.56f + density_pulse * 0.26f + field_strength * 0.13f +
                   control_influence * 0.42f,
               0.0f, 1.0f);
    float excitation = particle.exc;
    const float response = target_exc > excitation ? 10.0f : 1.05f;
    const float t = clampf(dt * response, 0.0f, 1.0f);
    excitation = excitation * (1.0f - t) + target_exc * t;

    for (int k = 0; k < 3; k++) velocity[k] = velocity[k] + acc[k] * dt;
    for (int k = 0; k < 3; k++) pos[k] = pos[k] + velocity[k] * dt;

    const float world_edge = O_HALF * 0.985f;
    const float edge_band = 0.12f * O_HALF;
    for (int axis = 0; axis < 3; axis++) {
      const float over = fabsf(pos[axis]) - (world_edge - edge_band);
      if (over > 0.0f) {
        const float absorb = clampf(over / edge_band, 0.0f, 1.0f);
        velocity[axis] = velocity[axis] * (1.0f - absorb * 0.16f);
      }
      if (fabsf(pos[axis]) > world_edge) {
        pos[axis] = clampf(pos[axis], -world_edge, world_edge);
        velocity[axis] = velocity[axis] * -0.55f;
      }
    }
    const float hue_drift = 1.0f - smoothstepf(0.30f, 0.70f, excitation);
    const float hue = fractf(particle.hue + dt * hue_drift *
                                                (0.012f + signed_radial * 0.030f +
                                                 excitation * 0.036f + control_influence * 0.080f));
    particle.px = pos[0];
    particle.py = pos[1];
    particle.pz = pos[2];
    particle.hue = hue;
    particle.vx = velocity[0];
    particle.vy = velocity[1];
    particle.vz = velocity[2];
    particle.exc = excitation;
    particles[ii] = particle;
  }
  if (p2p) {
    near_free(&nr);
    free(snap);
  }
}

/* ------------------------------------------------------------ seeding */

static uint32_t hash32(uint32_t x) { /* wgsl:205-210 */
  x = ((x >> 16) ^ x) * 0x45d9f3bu;
  x = ((x >> 16) ^ x) * 0x45d9f3bu;
  return (x >> 16) ^ x;
}

static float random01(uint32_t seed) { return (float)hash32(seed) * (1.0f / 4294967296.0f); }

static float seeded_enclosed_mass(float radius) { /* wgsl:216-230 */
  float bulge = 0.05f * rf_powf(clampf(radius / 0.11f, 0.0f, 1.0f), 3.0f);
  float halo = 0.70f * rf_powf(clampf(radius / 0.70f, 0.0f, 1.0f), 3.0f);
  float disc = 0.18f * rf_powf(clampf((radius - 0.055f) / 0.60f, 0.0f, 1.0f), 1.0f / 0.72f);
  float polar = 0.07f * rf_powf(clampf((radius - 0.22f) / 0.31f, 0.0f, 1.0f), 1.0f / 0.86f);
  return fmaxf(bulge + halo + disc + polar, 0.0001f);
}

static void cross3(const float a[3], const float b[3], float o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

void oracle_initialize(OParticle *particles, const OParams *P) { /* wgsl:232-374 */
  const uint32_t n = P->n;
#pragma omp parallel for schedule(static) if (n >= 8192u)
  for (int64_t ii = 0; ii < (int64_t)n; ii++) {
    const uint32_t i = (uint32_t)ii;
    float u0 = random01(i * 11u + 1u), u1 = random01(i * 11u + 2u), u2 = random01(i * 11u + 3u);
    float u3 = random01(i * 11u + 4u), u4 = random01(i * 11u + 5u), u5 = random01(i * 11u + 6u);
    float pos[3], vel[3], excitation;
    if (u5 < 0.75f) {
      float z = u0 * 2.0f - 1.0f, phi = O_TAU * u1;
      float outer = u5 < 0.05f ? 0.11f : 0.70f;
      float radius = outer * rf_powf(u2, 0.3333333f);
      float ring = sqrtf(fmaxf(0.0f, 1.0f - z * z));
      float rd[3] = {ring * rf_cosf(phi), z, ring * rf_sinf(phi)};
      for (int k = 0; k < 3; k++) pos[k] = radius * rd[k];
      float tz = u3 * 2.0f - 1.0f, tphi = O_TAU * u4;
      float tring = sqrtf(fmaxf(0.0f, 1.0f - tz * tz));
      float rnd[3] = {tring * rf_cosf(tphi), tz, tring * rf_sinf(tphi)};
      float tangent[3];
      cross3(rd, rnd, tangent);
      if (length3(tangent) < 0.001f) {
        float up[3] = {0.0f, 1.0f, 0.0f};
        cross3(rd, up, tangent);
      }
      if (length3(tangent) < 0.001f) {
        float ex[3] = {1.0f, 0.0f, 0.0f};
        cross3(rd, ex, tangent);
      }
      float orbital = 0.985f * sqrtf(P->gravity * seeded_enclosed_mass(radius) / (radius + 0.018f));
      float tl = length3(tangent);
      for (int k = 0; k < 3; k++) vel[k] = orbital * (tangent[k] / tl);
      excitation = u5 < 0.05f ? 0.09f : 0.025f + u4 * 0.025f;
    } else if (u5 < 0.93f) {
      float radius = 0.055f + 0.60f * rf_powf(u0, 0.72f);
      float arm = (float)(i & 3u) * (O_TAU / 4.0f);
      float angle = arm + radius * 7.8f + (u1 - 0.5f) * (0.045f + radius * 0.055f);
      float thickness = (u2 + u3 + u4 - 1.5f) * (0.0035f + radius * 0.010f);
      float flat[3] = {radius * rf_cosf(angle), radius * rf_sinf(angle) * 0.72f, thickness};
      float tilt = 0.20f;
      pos[0] = flat[0];
      pos[1] = flat[1] * rf_cosf(tilt) - flat[2] * rf_sinf(tilt);
      pos[2] = flat[1] * rf_sinf(tilt) + flat[2] * rf_cosf(tilt);
      float orbital = 0.99f * sqrtf(P->gravity * seeded_enclosed_mass(radius) / (radius + 0.018f));
      float tangent[3] = {-rf_sinf(angle), rf_cosf(angle) * 0.72f * rf_cosf(tilt),
                          rf_cosf(angle) * 0.72f * rf_sinf(tilt)};
      float pl = length3(pos), tl = length3(tangent);
      float sw = rf_sinf(angle * 3.0f - radius * 13.0f);
      for (int k = 0; k < 3; k++)
        vel[k] = orbital * (tangent[k] / tl) + (pos[k] / pl) * orbital * 0.035f * sw;
      excitation = 0.08f + u3 * 0.05f;
    } else {
      float lineage = (float)(i & 3u);
      float radius = 0.22f + 0.31f * rf_powf(u0, 0.86f) + (lineage - 1.5f) * 0.007f;
      float angle = O_TAU * u1 + radius * 3.5f;
      float thickness = (u2 + u3 + u4 - 1.5f) * (0.004f + radius * 0.009f);
      float flat[3] = {radius * rf_cosf(angle), thickness, radius * rf_sinf(angle)};
      float tilt = -0.54f + lineage * 0.36f;
      pos[0] = flat[0] * rf_cosf(tilt) - flat[1] * rf_sinf(tilt);
      pos[1] = flat[0] * rf_sinf(tilt) + flat[1] * rf_cosf(tilt);
      pos[2] = flat[2];
      float tangent[3] = {-rf_sinf(angle) * rf_cosf(tilt), -rf_sinf(angle) * rf_sinf(tilt), rf_cosf(angle)};
      float orbital = 0.99f * sqrtf(P->gravity * seeded_enclosed_mass(radius) / (radius + 0.018f));
      float tl = length3(tangent);
      for (int k = 0; k < 3; k++) vel[k] = -orbital * (tangent[k] / tl);
      excitation = 0.20f + u4 * 0.08f;
    }
    float hue = 0.0f;
    if (u5 >= 0.75f) {
      float speed = fmaxf(length3(vel), 0.0001f);
      float radius = fmaxf(length3(pos), 0.0001f);
      float pv = (pos[0] * vel[0] + pos[1] * vel[1]) + pos[2] * vel[2];
      float radial_motion = clampf(pv / (radius * speed), -1.0f, 1.0f);
      float am[3];
      cross3(pos, vel, am);
      float spin = am[1] / fmaxf(length3(am), 0.0001f);
      hue = fractf(rf_atan2f(vel[1], vel[0]) / O_TAU + (vel[2] / speed) * 0.14f + spin * 0.075f +
                   radial_motion * 0.065f + excitation * 0.085f + (float)(i & 3u) * 0.018f);
    }
    OParticle *p = &particles[ii];
    p->px = pos[0];
    p->py = pos[1];
    p->pz = pos[2];
    p->hue = hue;
    p->vx = vel[0];
    p->vy = vel[1];
    p->vz = vel[2];
    p->exc = excitation;
  }
}

/* ---------------------------------------------------------- frame order */

/* clear, deposit, upward, m2l, downward, near: one field solve without
 * integrate (native/main.rs:437-449). */
void oracle_solve_fields(const OParticle *particles, OMoment *moments, OField *fields,
                         const OParams *P) {
  oracle_clear(moments, oracle_total_cells(P->depth));
  oracle_deposit(particles, moments, P);
  oracle_upward(moments, P);
  oracle_m2l_all(moments, fields, P);
  oracle_downward(moments, fields, P);
  if (P->near_mode != O_NEAR_P2P) oracle_near_all(moments, fields, P);
}

/* `steps` full solver frames (native/main.rs:411-421). */
void oracle_step(OParticle *particles, OMoment *moments, OField *fields, const OParams *P,
                 uint32_t steps) {
  for (uint32_t s = 0; s < steps; s++) {
    oracle_solve_fields(particles, moments, fields, P);
    oracle_integrate(particles, moments, fields, P);
  }
}

/* FNV-1a over little-endian bytes (native/main.rs:152-163). */
uint32_t oracle_fnv1a(const void *data, size_t bytes) {
  const uint8_t *b = (const uint8_t *)data;
  uint32_t h = 2166136261u;
  for (size_t i = 0; i < bytes; i++) {
    h ^= b[i];
    h *= 16777619u;
  }
  return h;
}

/* ------------------------------------------- interaction-list exports */

/* On-path M2L targets (wgsl:472-476): non-empty cells whose parent holds more
 * than ADAPTIVE_LEAF_CAPACITY bodies.  Writes global cell ids in ascending
 * order; returns how many. */
uint32_t oracle_m2l_targets(const OMoment *moments, const OParams *P, uint32_t *out,
                            uint32_t cap) {
  const uint32_t total = oracle_total_cells(P->depth);
  uint32_t k = 0;
  for (uint32_t g = 1; g < total; g++) {
    uint32_t level = level_of(g), start = o_level_offset(level), dim = 1u << level, tc[3], pc[3];
    cell_coord(g - start, dim, tc);
    pc[0] = tc[0] / 2u;
    pc[1] = tc[1] / 2u;
    pc[2] = tc[2] / 2u;
    uint32_t parent = o_level_offset(level - 1u) + linear_index(pc, dim >> 1);
    if (moments[g].count != 0u && (int32_t)moments[parent].count > (int32_t)O_ADAPTIVE) {
      if (k < cap) out[k] = g;
      k++;
    }
  }
  return k;
}

/* The cell each body samples its field from in integrate (wgsl:625-639). */
void oracle_sample_cells(const OParticle *particles, const OMoment *moments, const OParams *P,
                         uint32_t *out) {
#pragma omp parallel for schedule(static) if (P->n >= 8192u)
  for (int64_t i = 0; i < (int64_t)P->n; i++) {
    float pos[3] = {particles[i].px, particles[i].py, particles[i].pz};
    uint32_t res = 0;
    for (uint32_t level = 1u; level <= P->depth; level++) {
      uint32_t dim = 1u << level, c[3];
      position_cell(pos, dim, c);
      uint32_t index = o_level_offset(level) + linear_index(c, dim);
      if ((int32_t)moments[index].count <= (int32_t)O_ADAPTIVE || level == P->depth) {
        res = index;
        break;
      }
    }
    out[i] = res;
  }
}

/* ----------------------------------------------- FP64 direct-sum check */

/* Softened Newtonian acceleration on selected targets from all bodies, in
 * double precision (the force-error reference for the FMM). Equal masses 1/n. */
void oracle_direct_sum_f64(const OParticle *particles, uint32_t n, const uint32_t *targets,
                           uint32_t nt, double gravity, double eps, double *acc_out) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t t = 0; t < (int64_t)nt; t++) {
    const OParticle *pt = &particles[targets[t]];
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (uint32_t j = 0; j < n; j++) {
      if (j == targets[t]) continue;
      double dx = (double)particles[j].px - pt->px;
      double dy = (double)particles[j].py - pt->py;
      double dz = (double)particles[j].pz - pt->pz;
      double r2 = dx * dx + dy * dy + dz * dz + eps * eps;
      double inv = 1.0 / sqrt(r2);
      double w = inv * inv * inv;
      ax += dx * w;
      ay += dy * w;
      az += dz * w;
    }
    double gm = gravity / (double)n;
    acc_out[3 * t + 0] = ax * gm;
    acc_out[3 * t + 1] = ay * gm;
    acc_out[3 * t + 2] = az * gm;
  }
}

int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

/* ------------------------------------------------------------------ render */

/* Headless restatement of the display passes (wgsl:780-1009, app.js:650-710)
 * with the product's definitions: per-pixel fixed-point accumulation at 2^24
 * units per 1.0 (order-independent), binary32 blur and resolve intermediates,
 * exact bilinear weights, RGBA8 output with row 0 at the top. */
typedef struct {
  uint32_t width, height, instances;
  float yaw, pitch, zoom, point_size, exposure;
} ORenderParams;

static float o_mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }

static void o_fetch_acc(const uint64_t *acc, uint32_t w, uint32_t h, int x, int y, float out[4]) {
  if (x < 0) x = 0;
  if (y < 0) y = 0;
  if (x > (int)w - 1) x = (int)w - 1;
  if (y > (int)h - 1) y = (int)h - 1;
  const uint64_t *p = acc + 4u * ((size_t)y * w + (size_t)x);
  for (int k = 0; k < 4; k++) out[k] = (float)p[k] * (1.0f / 16777216.0f);
}

static void o_fetch_tex(const float *tex, uint32_t w, uint32_t h, int x, int y, float out[4]) {
  if (x < 0) x = 0;
  if (y < 0) y = 0;
  if (x > (int)w - 1) x = (int)w - 1;
  if (y > (int)h - 1) y = (int)h - 1;
  const float *p = tex + 4u * ((size_t)y * w + (size_t)x);
  for (int k = 0; k < 4; k++) out[k] = p[k];
}

void oracle_render(const OParticle *particles, const OParams *P, const ORenderParams *R,
                   uint8_t *rgba, uint64_t *acc_out) {
  const uint32_t W = R->width, H = R->height, aw = (W + 1u) / 2u, ah = (H + 1u) / 2u;
  const uint32_t instances = R->instances ? R->instances : P->n;
  const float cyw = (float)cos((double)R->yaw), syw = (float)sin((double)R->yaw);
  const float cpt = (float)cos((double)R->pitch), spt = (float)sin((double)R->pitch);
  const float aspect = (float)((double)W / (double)(H > 1u ? H : 1u));
  const float pop = 0.62f * rf_powf(1048576.0f / fmaxf((float)instances, 1.0f), 0.14f);
  uint64_t *acc = (uint64_t *)calloc((size_t)aw * ah * 4u, sizeof(uint64_t));
  for (uint32_t i = 0; i < instances && P->n > 0u; i++) {
    const OParticle *pt = &particles[(i * 747796405u + 2891336453u) % P->n];
    const float yx = cyw * pt->px + syw * pt->pz, yy = pt->py, yz = -syw * pt->px + cyw * pt->pz;
    const float rx = yx, ry = cpt * yy - spt * yz, rz = spt * yy + cpt * yz;
    const float view_z = R->zoom * O_HALF - rz;
    const float perspective = (1.92f * O_HALF) / view_z;
    const float cx = rx * perspective / aspect, cy = ry * perspective;
    const float depth = 0.46f + rz * 0.08f;
    const float vel[3] = {pt->vx, pt->vy, pt->vz}, pos[3] = {pt->px, pt->py, pt->pz};
    const float velocity = length3(vel);
    const float speed = fmaxf(velocity, 0.0001f);
    const float excitation = clampf(pt->exc, 0.0f, 1.0f);
    const float signed_radial =
        clampf(((pos[0] * vel[0] + pos[1] * vel[1]) + pos[2] * vel[2]) / (fmaxf(length3(pos), 0.0001f) * speed),
               -1.0f, 1.0f);
    const float infall = clampf(-signed_radial, 0.0f, 1.0f), outflow = clampf(signed_radial, 0.0f, 1.0f);
    float sp[3] = {o_mix(0.50f, 0.24f, infall), o_mix(0.42f, 0.56f, infall), o_mix(0.58f, 1.00f, infall)};
    sp[0] = o_mix(sp[0], 1.00f, outflow);
    sp[1] = o_mix(sp[1], 0.50f, outflow);
    sp[2] = o_mix(sp[2], 0.20f, outflow);
    const float heat = smoothstepf(0.18f, 0.85f, excitation);
    const float phase[3] = {0.00f, 0.67f, 0.33f};
    const float luminosity = 0.30f + excitation * 0.90f;
    const float speed_gain = 0.62f + fminf(velocity * 1.4f, 1.0f) * 0.30f;
    float col[3];
    for (int k = 0; k < 3; k++) {
      const float rainbow = 0.5f + 0.5f * rf_cosf(O_TAU * (pt->hue + phase[k]));
      const float tint = rf_powf(rainbow, 0.85f);
      const float s = o_mix(sp[k] * tint, sp[k], heat);
      col[k] = s * (speed_gain + excitation * 0.90f) + heat * heat * 0.55f;
    }
    float influence = 0.0f, cc[3] = {0.82f, 1.0f, 0.28f};
    if (P->control_point[3] > 0.5f) {
      const float dx = P->control_point[0] - pos[0], dy = P->control_point[1] - pos[1],
                  dz = P->control_point[2] - pos[2];
      const float radius = fmaxf(P->control_radius, 0.02f);
      influence = rf_expf(-2.0f * ((dx * dx + dy * dy) + dz * dz) / (radius * radius));
      const float mode = P->control_axis_mode[3];
      if (mode > 1.5f && mode < 2.5f) {
        cc[0] = 1.0f; cc[1] = 0.38f; cc[2] = 0.18f;
      } else if (mode >= 2.5f) {
        cc[0] = 0.82f; cc[1] = 0.34f; cc[2] = 1.0f;
      }
    }
    for (int k = 0; k < 3; k++) col[k] = o_mix(col[k], cc[k], influence * 0.68f);
    const float depth_fade = clampf(0.62f + rz * 0.25f, 0.28f, 1.0f) * (0.76f + excitation * 0.48f) *
                             luminosity * (1.0f + influence * 0.72f);
    if (!(cx >= -1.0f && cx <= 1.0f && cy >= -1.0f && cy <= 1.0f && depth >= 0.0f && depth <= 1.0f)) continue;
    const float fx = (cx + 1.0f) * 0.5f * (float)aw, fy = (1.0f - cy) * 0.5f * (float)ah;
    int px = (int)floorf(fx), py = (int)floorf(fy);
    if (px > (int)aw - 1) px = (int)aw - 1;
    if (py > (int)ah - 1) py = (int)ah - 1;
    const float weight = R->exposure * depth_fade * pop;
    uint64_t *d = acc + 4u * ((size_t)py * aw + (size_t)px);
    for (int k = 0; k < 3; k++) d[k] += (uint64_t)llrintf(col[k] * weight * 16777216.0f);
    d[3] += (uint64_t)llrintf(weight * 16777216.0f);
  }
  if (acc_out) memcpy(acc_out, acc, sizeof(uint64_t) * 4u * (size_t)aw * ah);
  /* Two separable passes (wgsl:914-970). */
  float *ta = (float *)malloc(sizeof(float) * 4u * (size_t)aw * ah);
  float *tb = (float *)malloc(sizeof(float) * 4u * (size_t)aw * ah);
  for (int axis = 0; axis < 2; axis++) {
    const float dim = axis == 0 ? (float)aw : (float)ah;
    const float out_dim = axis == 0 ? (float)W : (float)H;
    const float step = fmaxf(R->point_size, 1.0f) / (out_dim * 3.230769f);
    const float offs[5] = {0.0f, step * 1.384615f, -(step * 1.384615f), step * 3.230769f, -(step * 3.230769f)};
    const float wts[5] = {0.227027f, 0.316216f, 0.316216f, 0.070270f, 0.070270f};
    float *dst = axis == 0 ? ta : tb;
    for (uint32_t y = 0; y < ah; y++)
      for (uint32_t x = 0; x < aw; x++) {
        const float uv = ((axis == 0 ? (float)x : (float)y) + 0.5f) / dim;
        float field[4] = {0, 0, 0, 0};
        for (int t = 0; t < 5; t++) {
          const float u = t == 0 ? uv : uv + offs[t];
          const float tc = u * dim - 0.5f, f0 = floorf(tc), f = tc - f0;
          const int i0 = (int)f0;
          float a[4], b[4];
          if (axis == 0) {
            o_fetch_acc(acc, aw, ah, i0, (int)y, a);
            o_fetch_acc(acc, aw, ah, i0 + 1, (int)y, b);
          } else {
            o_fetch_tex(ta, aw, ah, (int)x, i0, a);
            o_fetch_tex(ta, aw, ah, (int)x, i0 + 1, b);
          }
          for (int k = 0; k < 4; k++) {
            const float v = (a[k] * (1.0f - f) + b[k] * f) * wts[t];
            field[k] = t == 0 ? v : field[k] + v;
          }
        }
        memcpy(dst + 4u * ((size_t)y * aw + x), field, sizeof(field));
      }
  }
  /* Resolve (wgsl:972-1009). */
  const float bg[3] = {0.006f, 0.008f, 0.015f};
  for (uint32_t y = 0; y < H; y++)
    for (uint32_t x = 0; x < W; x++) {
      const float u = ((float)x + 0.5f) / (float)W, v = ((float)y + 0.5f) / (float)H;
      const float tx = u * (float)aw - 0.5f, ty = v * (float)ah - 0.5f;
      const float fx0 = floorf(tx), fy0 = floorf(ty), fx = tx - fx0, fy = ty - fy0;
      const int ix = (int)fx0, iy = (int)fy0;
      float c00[4], c10[4], c01[4], c11[4], a[4];
      o_fetch_tex(tb, aw, ah, ix, iy, c00);
      o_fetch_tex(tb, aw, ah, ix + 1, iy, c10);
      o_fetch_tex(tb, aw, ah, ix, iy + 1, c01);
      o_fetch_tex(tb, aw, ah, ix + 1, iy + 1, c11);
      for (int k = 0; k < 4; k++) {
        const float top = c00[k] * (1.0f - fx) + c10[k] * fx;
        const float bot = c01[k] * (1.0f - fx) + c11[k] * fx;
        a[k] = top * (1.0f - fy) + bot * fy;
      }
      float rgb[3] = {bg[0], bg[1], bg[2]};
      if (!(a[3] < 0.00001f)) {
        const float avg[3] = {a[0] / a[3], a[1] / a[3], a[2] / a[3]};
        const float luma = (avg[0] * 0.2126f + avg[1] * 0.7152f) + avg[2] * 0.0722f;
        const float density = sqrtf(a[3] / (a[3] + 1.0f));
        for (int k = 0; k < 3; k++) {
          const float vivid = fmaxf(0.0f, o_mix(luma, avg[k], 1.16f));
          const float mapped = 1.0f - rf_expf(-vivid * density * 1.58f);
          rgb[k] = rf_powf(clampf(mapped + bg[k], 0.0f, 1.0f), 0.82f);
        }
      }
      uint8_t *o = rgba + 4u * ((size_t)y * W + x);
      for (int k = 0; k < 3; k++) o[k] = (uint8_t)lrintf(rgb[k] * 255.0f);
      o[3] = 255;
    }
  free(ta);
  free(tb);
  free(acc);
}
