// Host harness for the reference shader translated to C++ (test
// infrastructure only).  It replays the native wgpu harness's dispatch
// sequence (native/main.rs) on the host: per-level uniform blocks written as
// `write_params` writes them (native/main.rs:39-86, 89-128), then
//   seed   = initialize                                  (main.rs:423-433)
//   solve  = clear_cells, deposit, upward (levels depth-1..0), m2l_all,
//            downward (levels 1..depth), near_all        (main.rs:436-451)
//   frame  = solve + integrate                           (main.rs:411-421)
// with the same workgroup counts.  A dispatch's invocations may run on
// several host threads (OpenMP), which the passes allow: no pass reads what
// another invocation of the same dispatch writes, and the deposit's integer
// atomics commute, so results do not depend on the thread count.
//
// The translated shader (oracle/_ref/rainbow_fmm_wgsl.gen.cpp, written by
// wgsl_transpile.py) is force-included ahead of this file by the build
// (g++ -include); it defines the T_* structs, the w_* bindings and
// functions, and the wgsl_entries table used below.
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "wgsl_runtime.hpp"

namespace {

// The values `write_params` fixes, made settable so the control field and
// other parameters can be exercised (defaults: native/main.rs:55-81).
struct RefConfig {
  uint32_t count, depth, cells;
  float scale;
  float dt, gravity, softening, speed;
  float control_point[4];
  float control_axis_mode[4];
  float control_strength, control_radius;
};

constexpr uint32_t kParticleRow = 65535u * 256u;

uint32_t level_offset(uint32_t l) { return ((1u << (3u * l)) - 1u) / 7u; }

// One uniform block in the Params layout: eight u32s then twenty-four f32s.
T_Params block(const RefConfig &c, uint32_t level, uint32_t lo, uint32_t ldim, uint32_t po,
               uint32_t pdim) {
  const uint32_t u[8] = {c.count, c.depth, level, lo, ldim, po, pdim, c.cells};
  const float f[24] = {c.dt, c.gravity, c.softening, 5.0f, 0.0f, 1.0f, 0.0f, 0.0f,
                       0.0f, 0.0f, 0.84f, c.speed,
                       c.control_point[0], c.control_point[1], c.control_point[2],
                       c.control_point[3],
                       c.control_axis_mode[0], c.control_axis_mode[1], c.control_axis_mode[2],
                       c.control_axis_mode[3],
                       c.control_strength, c.control_radius, c.scale, 0.0f};
  static_assert(sizeof(T_Params) == 128, "Params block is 128 bytes");
  unsigned char raw[128];
  std::memcpy(raw, u, 32);
  std::memcpy(raw + 32, f, 96);
  T_Params p;
  std::memcpy(&p, raw, 128);
  return p;
}

// Per-level blocks (slot l, l = 0..depth) and upward blocks (l = 0..depth-1).
struct Plans {
  std::vector<T_Params> level, upward;
};

Plans plans(const RefConfig &c) {
  Plans P;
  for (uint32_t l = 0; l <= c.depth; l++) {
    const uint32_t pl = l > 0 ? l - 1u : 0u;
    P.level.push_back(block(c, l, level_offset(l), 1u << l, level_offset(pl), 1u << pl));
  }
  for (uint32_t l = 0; l < c.depth; l++)
    P.upward.push_back(block(c, l, level_offset(l), 1u << l, level_offset(l + 1u), 1u << (l + 1u)));
  return P;
}

const wgsl_entry *entry(const char *name) {
  for (const auto &e : wgsl_entries)
    if (std::strcmp(e.name, name) == 0) return &e;
  return nullptr;
}

// Set when a dispatch names an entry point the translation does not have
// (the shader changed): the calls below then return -1.
bool g_missing = false;

void dispatch(const char *name, uint32_t gx, uint32_t gy) {
  const wgsl_entry *e = entry(name);
  if (e == nullptr) {
    g_missing = true;
    return;
  }
  const int64_t row = (int64_t)gx * e->wg, total = row * gy;
#pragma omp parallel for schedule(static, 4096) if (total >= 16384)
  for (int64_t i = 0; i < total; i++)
    e->fn(wgsl::make<uint32_t, 3>((uint32_t)(i % row), (uint32_t)(i / row), 0u));
}

uint32_t div_ceil(uint32_t a, uint32_t b) { return (a + b - 1u) / b; }

void particle_grid(uint32_t n, uint32_t &gx, uint32_t &gy) {
  gx = div_ceil(n < kParticleRow ? n : kParticleRow, 256u);
  gy = div_ceil(n, kParticleRow);
}

void bind(void *particles, void *moments, void *fields) {
  w_particles = static_cast<T_Particle *>(particles);
  w_tree_particles = static_cast<T_Particle *>(particles);
  w_moments = static_cast<T_Moment *>(moments);
  w_moments_read = static_cast<wgsl::vec<int32_t, 4> *>(moments);
  w_fields = static_cast<T_Field *>(fields);
  w_tree_fields = static_cast<T_Field *>(fields);
}

void solve(const RefConfig &c, const Plans &P) {
  const T_Params &base = P.level[c.depth];
  uint32_t gx, gy;
  particle_grid(c.count, gx, gy);
  w_params = base;
  dispatch("clear_cells", div_ceil(c.cells, 256u), 1u);
  dispatch("deposit", gx, gy);
  for (uint32_t l = c.depth; l-- > 0;) {
    w_params = P.upward[l];
    dispatch("upward", div_ceil(1u << (3u * l), 64u), 1u);
  }
  w_tree_params = P.level[0];
  dispatch("m2l_all", div_ceil(c.cells - 1u, 64u), 1u);
  for (uint32_t l = 1; l <= c.depth; l++) {
    w_tree_params = P.level[l];
    dispatch("downward", div_ceil(1u << (3u * l), 64u), 1u);
  }
  w_tree_params = P.level[0];
  dispatch("near_all", div_ceil(c.cells - 1u, 64u), 1u);
}

}  // namespace

extern "C" {

// Host threads for the dispatches (<= 0: all); returns the count in use.
int wref_set_threads(int n) {
#ifdef _OPENMP
  if (n <= 0) n = omp_get_num_procs();
  omp_set_num_threads(n);
  return n;
#else
  (void)n;
  return 1;
#endif
}

// The reference galaxy (`initialize`) into `particles` (count x 32 bytes).
int wref_seed(void *particles, const RefConfig *c) {
  const Plans P = plans(*c);
  bind(particles, nullptr, nullptr);
  w_params = P.level[c->depth];
  uint32_t gx, gy;
  particle_grid(c->count, gx, gy);
  g_missing = false;
  dispatch("initialize", gx, gy);
  return g_missing ? -1 : 0;
}

// One field solve (the harness's digest block): moments and fields.
int wref_solve_fields(void *particles, void *moments, void *fields, const RefConfig *c) {
  const Plans P = plans(*c);
  bind(particles, moments, fields);
  g_missing = false;
  solve(*c, P);
  return g_missing ? -1 : 0;
}

// `frames` full frames (solve + integrate).
int wref_frames(void *particles, void *moments, void *fields, const RefConfig *c,
                uint32_t frames) {
  const Plans P = plans(*c);
  bind(particles, moments, fields);
  uint32_t gx, gy;
  particle_grid(c->count, gx, gy);
  g_missing = false;
  for (uint32_t f = 0; f < frames && !g_missing; f++) {
    solve(*c, P);
    w_tree_params = P.level[c->depth];
    dispatch("integrate", gx, gy);
  }
  return g_missing ? -1 : 0;
}

}  // extern "C"
