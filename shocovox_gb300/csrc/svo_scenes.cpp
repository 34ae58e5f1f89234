// svo_scenes.cpp -- seeded synthetic workloads: scene construction recipes
// (lists of svo_op in the reference tests' x -> y -> z insert order) and ray
// batches.  Everything is built from integer hashing and IEEE-754 basic
// operations (no libm transcendental calls; sin/cos are evaluated with a
// fixed polynomial in double precision), and compiled with
// -ffp-contract=off, so x86_64 and aarch64 produce identical bits.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "svo_internal.h"

namespace svo {
namespace {

// splitmix64 (seeding) -> PCG32 (XSH RR) stream
uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
struct Pcg32 {
  uint64_t state, inc;
  explicit Pcg32(uint64_t seed) {
    uint64_t s = seed;
    state = splitmix64(s);
    inc = splitmix64(s) | 1u;
  }
  uint32_t next() {
    uint64_t old = state;
    state = old * 6364136223846793005ull + inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  float unit() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }  // [0, 1)
  uint32_t range(uint32_t lo, uint32_t hi) { return lo + next() % (hi - lo); }
};

// integer lattice hash -> [0, 1)
inline float lattice(int32_t x, int32_t y, int32_t z, uint32_t seed) {
  uint32_t h = (uint32_t)x * 0x8DA6B343u ^ (uint32_t)y * 0xD8163841u ^ (uint32_t)z * 0xCB1AB31Fu ^ seed * 0x9E3779B9u;
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  h ^= h >> 16;
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}
inline float smooth(float t) { return t * t * (3.0f - 2.0f * t); }
inline float lerp(float a, float b, float t) { return a + (b - a) * t; }

float value_noise2(float x, float z, uint32_t seed) {
  const float fx = std::floor(x), fz = std::floor(z);
  const int32_t ix = (int32_t)fx, iz = (int32_t)fz;
  const float tx = smooth(x - fx), tz = smooth(z - fz);
  const float a = lerp(lattice(ix, 0, iz, seed), lattice(ix + 1, 0, iz, seed), tx);
  const float b = lerp(lattice(ix, 0, iz + 1, seed), lattice(ix + 1, 0, iz + 1, seed), tx);
  return lerp(a, b, tz);
}
float value_noise3(float x, float y, float z, uint32_t seed) {
  const float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  const int32_t ix = (int32_t)fx, iy = (int32_t)fy, iz = (int32_t)fz;
  const float tx = smooth(x - fx), ty = smooth(y - fy), tz = smooth(z - fz);
  float c[2][2];
  for (int dy = 0; dy < 2; ++dy)
    for (int dz = 0; dz < 2; ++dz)
      c[dy][dz] = lerp(lattice(ix, iy + dy, iz + dz, seed), lattice(ix + 1, iy + dy, iz + dz, seed), tx);
  return lerp(lerp(c[0][0], c[1][0], ty), lerp(c[0][1], c[1][1], ty), tz);
}
// fractal sum: amplitude x0.5, frequency x2 per octave, normalised to [0, 1)
float fbm2(float x, float z, uint32_t octaves, uint32_t seed) {
  float sum = 0.0f, amp = 1.0f, norm = 0.0f, f = 1.0f;
  for (uint32_t o = 0; o < octaves; ++o) {
    sum = sum + amp * value_noise2(x * f, z * f, seed + o * 101u);
    norm = norm + amp;
    amp = amp * 0.5f;
    f = f * 2.0f;
  }
  return sum / norm;
}
float fbm3(float x, float y, float z, uint32_t octaves, uint32_t seed) {
  float sum = 0.0f, amp = 1.0f, norm = 0.0f, f = 1.0f;
  for (uint32_t o = 0; o < octaves; ++o) {
    sum = sum + amp * value_noise3(x * f, y * f, z * f, seed + o * 131u);
    norm = norm + amp;
    amp = amp * 0.5f;
    f = f * 2.0f;
  }
  return sum / norm;
}

// sin/cos of |x| <= 4 pi by range reduction to [-pi/4, pi/4] and Taylor polynomials (double)
const double kPi = 3.14159265358979323846;
void det_sincos(double x, double* s, double* c) {
  const double k = std::floor(x / (kPi / 2.0) + 0.5);
  const double r = x - k * (kPi / 2.0);
  const double r2 = r * r;
  double ps = 0.0, pc = 0.0, term_s = r, term_c = 1.0;
  for (int n = 0; n < 12; ++n) {
    ps = ps + term_s;
    pc = pc + term_c;
    term_s = -term_s * r2 / (double)((2 * n + 2) * (2 * n + 3));
    term_c = -term_c * r2 / (double)((2 * n + 1) * (2 * n + 2));
  }
  const int q = ((int)k % 4 + 4) % 4;
  switch (q) {
    case 0: *s = ps; *c = pc; break;
    case 1: *s = pc; *c = -ps; break;
    case 2: *s = -ps; *c = -pc; break;
    default: *s = -pc; *c = ps; break;
  }
}

struct V3 {
  float x, y, z;
};
inline V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
// V3c::<f32>::normalized (src/spatial/math/vector.rs:75-81)
inline V3 normalized(V3 v) {
  const float l = std::sqrt((v.x * v.x + v.y * v.y) + v.z * v.z);
  return V3{v.x / l, v.y / l, v.z / l};
}
// V3c::cross (vector.rs:186-192)
inline V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

inline uint32_t pack(uint32_t r, uint32_t g, uint32_t b) { return (r << 24) | (g << 16) | (b << 8) | 0xFFu; }
// 64 height bands: a fixed earth-tone ramp
inline uint32_t band_color(uint32_t band) {
  return pack(60 + (band * 3) % 160, 90 + (band * 5) % 140, 40 + (band * 7) % 120);
}
// 5-6-5 quantised random colour
inline uint32_t q565(Pcg32& g) {
  const uint32_t v = g.next();
  return pack(((v >> 0) & 31u) << 3, ((v >> 5) & 63u) << 2, ((v >> 11) & 31u) << 3);
}

struct Sphere {
  float cx, cy, cz, r2;
  uint32_t color, user;
};

class OpSink {
 public:
  OpSink(svo_op* ops, uint64_t max) : ops_(ops), max_(max) {}
  void add(uint8_t op, uint32_t x, uint32_t y, uint32_t z, uint32_t size, uint32_t rgba, uint32_t user) {
    if (n_ < max_ && ops_) {
      svo_op& o = ops_[n_];
      o.x = (uint16_t)x;
      o.y = (uint16_t)y;
      o.z = (uint16_t)z;
      o.op = op;
      o.kind = SVO_ENTRY_COMPLEX;
      o.size = size;
      o.rgba = rgba;
      o.user = user;
    }
    ++n_;
  }
  uint64_t count() const { return n_; }

 private:
  svo_op* ops_;
  uint64_t max_, n_ = 0;
};

void gen_spheres(Pcg32& g, const svo_scene_recipe& r, std::vector<Sphere>& out) {
  const float S = (float)r.size;
  for (uint32_t i = 0; i < r.spheres; ++i) {
    Sphere s;
    const float rad = 4.0f + g.unit() * 12.0f * (S / 128.0f > 1.0f ? S / 128.0f : 1.0f);
    s.cx = g.unit() * S;
    s.cy = g.unit() * S;
    s.cz = g.unit() * S;
    s.r2 = rad * rad;
    s.color = q565(g);
    s.user = 1000u + i;
    out.push_back(s);
  }
}

// kind 0: value-noise heightfield plus random solid spheres
// kind 1: terrain with caves carved by 3D noise
// kind 3: 3D noise field thresholded to the target occupancy plus spheres
void gen_dense(const svo_scene_recipe& r, OpSink& sink) {
  const uint32_t S = r.size;
  Pcg32 g(r.seed);
  std::vector<Sphere> spheres;
  gen_spheres(g, r, spheres);
  const uint32_t seed = (uint32_t)(r.seed * 2654435761ull);
  std::vector<float> height((size_t)S * S);
  for (uint32_t x = 0; x < S; ++x)
    for (uint32_t z = 0; z < S; ++z)
      height[(size_t)x * S + z] =
          r.height_lo + (r.height_hi - r.height_lo) * fbm2((float)x * r.base_freq, (float)z * r.base_freq,
                                                           r.octaves ? r.octaves : 1, seed);
  // kind 3 threshold: the fbm3 value whose upper tail matches the occupancy (coarse estimate)
  float thr = 1.0f - r.occupancy;
  if (r.kind == 3) {
    std::vector<float> sample;
    Pcg32 gs(r.seed ^ 0xABCDull);
    for (int i = 0; i < 8192; ++i) {
      // drawn z, y, x: the order is spelled out so that every compiler makes the same sample
      const float uz = gs.unit(), uy = gs.unit(), ux = gs.unit();
      sample.push_back(fbm3(ux * (float)S * r.base_freq, uy * (float)S * r.base_freq, uz * (float)S * r.base_freq,
                            r.octaves ? r.octaves : 1, seed + 7u));
    }
    std::sort(sample.begin(), sample.end());
    size_t idx = (size_t)((1.0f - r.occupancy) * 8191.0f);
    thr = sample[idx < 8191 ? idx : 8191];
  }
  // x slabs are generated in parallel into per-slab buffers and emitted in x order
  const unsigned hw = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  const uint32_t slabs = std::min<uint32_t>(S, hw * 4);
  std::vector<std::vector<svo_op>> parts(slabs);
  std::atomic<uint32_t> next{0};
  auto worker = [&]() {
    for (uint32_t sl; (sl = next.fetch_add(1)) < slabs;) {
      const uint32_t x0 = (uint32_t)((uint64_t)S * sl / slabs), x1 = (uint32_t)((uint64_t)S * (sl + 1) / slabs);
      std::vector<svo_op>& out = parts[sl];
      auto add = [&](uint32_t x, uint32_t y, uint32_t z, uint32_t rgba, uint32_t user) {
        svo_op o;
        o.x = (uint16_t)x;
        o.y = (uint16_t)y;
        o.z = (uint16_t)z;
        o.op = SVO_OP_INSERT;
        o.kind = SVO_ENTRY_COMPLEX;
        o.size = 1;
        o.rgba = rgba;
        o.user = user;
        out.push_back(o);
      };
      for (uint32_t x = x0; x < x1; ++x)
        for (uint32_t y = 0; y < S; ++y)
          for (uint32_t z = 0; z < S; ++z) {
            const float fx = (float)x + 0.5f, fy = (float)y + 0.5f, fz = (float)z + 0.5f;
            bool placed = false;
            for (const Sphere& s : spheres) {
              const float ddx = fx - s.cx, ddy = fy - s.cy, ddz = fz - s.cz;
              if ((ddx * ddx + ddy * ddy) + ddz * ddz <= s.r2) {
                add(x, y, z, s.color, s.user);
                placed = true;
                break;
              }
            }
            if (placed) continue;
            bool solid = false;
            if (r.kind == 0 || r.kind == 1) {
              solid = (float)y <= height[(size_t)x * S + z];
              if (solid && r.kind == 1 && y > 0) {
                const float c =
                    fbm3(fx * r.base_freq * 4.0f, fy * r.base_freq * 4.0f, fz * r.base_freq * 4.0f, 2, seed + 3u);
                solid = !(c > r.cave_threshold);
              }
            } else if (r.kind == 3) {
              solid = fbm3(fx * r.base_freq, fy * r.base_freq, fz * r.base_freq, r.octaves ? r.octaves : 1, seed + 7u) >
                      thr;
            }
            if (solid) {
              const uint32_t band = y * 64u / S;
              add(x, y, z, band_color(band), 1u + band);
            }
          }
    }
  };
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < hw; ++t) pool.emplace_back(worker);
  for (auto& t : pool) t.join();
  for (const auto& part : parts)
    for (const svo_op& o : part) sink.add(o.op, o.x, o.y, o.z, o.size, o.rgba, o.user);
}

// kind 2: sparse 16^3 cells: 30% uniform solid blocks (insert_at_lod), the rest noise-carved mixed bricks
void gen_sparse_blocks(const svo_scene_recipe& r, OpSink& sink) {
  const uint32_t S = r.size, cell = 2 * r.brick_dim, n = S / cell;
  Pcg32 g(r.seed);
  const uint32_t seed = (uint32_t)(r.seed * 2246822519ull);
  // mean voxels per occupied cell: 0.3 * cell^3 + 0.7 * cell^3 * ~0.25
  const float per_cell = (float)cell * cell * cell * (0.3f + 0.7f * 0.25f);
  const float total = (float)S * S * S * r.occupancy;
  const float p_cell = std::min(1.0f, total / per_cell / ((float)n * n * n));
  for (uint32_t cx = 0; cx < n; ++cx)
    for (uint32_t cy = 0; cy < n; ++cy)
      for (uint32_t cz = 0; cz < n; ++cz) {
        if (!(g.unit() < p_cell)) continue;
        const uint32_t color = q565(g), user = 1u + g.range(0, 64);
        if (g.unit() < 0.3f) {
          sink.add(SVO_OP_INSERT_AT_LOD, cx * cell, cy * cell, cz * cell, cell, color, user);
          continue;
        }
        for (uint32_t x = 0; x < cell; ++x)
          for (uint32_t y = 0; y < cell; ++y)
            for (uint32_t z = 0; z < cell; ++z) {
              const uint32_t X = cx * cell + x, Y = cy * cell + y, Z = cz * cell + z;
              if (value_noise3((float)X * 0.25f, (float)Y * 0.25f, (float)Z * 0.25f, seed) > 0.68f)
                sink.add(SVO_OP_INSERT, X, Y, Z, 1, color, user);
            }
      }
}

// kind 4: axis-aligned boxes on a 2*brick_dim cell grid, each filled with insert_at_lod cubes of one
// cell, until the target occupancy; every 20th box gets a noise-carved detail cell of single voxels
// on top (mixed bricks).  Builds large sparse scenes with few operations.
void gen_boxes(const svo_scene_recipe& r, OpSink& sink) {
  const uint32_t S = r.size, cell = 2 * r.brick_dim, n = S / cell;
  Pcg32 g(r.seed);
  const uint32_t seed = (uint32_t)(r.seed * 3266489917ull);
  const double target = (double)S * S * S * r.occupancy;
  double placed = 0;
  uint32_t box = 0;
  while (placed < target && n >= 2) {
    const uint32_t span = std::max(2u, n / 14);  // box sides of 1..span cells (1..9 at 2048^3, brick 8)
    const uint32_t w = std::min(n, 1u + g.range(0, span)), h = std::min(n, 1u + g.range(0, span)),
                   d = std::min(n, 1u + g.range(0, span));
    const uint32_t x0 = g.range(0, n - w + 1), y0 = g.range(0, n - h + 1), z0 = g.range(0, n - d + 1);
    const uint32_t color = q565(g), user = 1u + g.range(0, 255);
    for (uint32_t x = x0; x < x0 + w; ++x)
      for (uint32_t y = y0; y < y0 + h; ++y)
        for (uint32_t z = z0; z < z0 + d; ++z) sink.add(SVO_OP_INSERT_AT_LOD, x * cell, y * cell, z * cell, cell, color, user);
    placed += (double)w * h * d * cell * cell * cell;
    if (box % 20 == 0 && y0 + h < n) {
      const uint32_t cx = x0 * cell, cy = (y0 + h) * cell, cz = z0 * cell;
      for (uint32_t x = 0; x < cell; ++x)
        for (uint32_t y = 0; y < cell; ++y)
          for (uint32_t z = 0; z < cell; ++z)
            if (value_noise3((float)(cx + x) * 0.3f, (float)(cy + y) * 0.3f, (float)(cz + z) * 0.3f, seed) > 0.6f)
              sink.add(SVO_OP_INSERT, cx + x, cy + y, cz + z, 1, color, user + 1);
    }
    ++box;
  }
}

}  // namespace

// Pinhole frame shared by the host and device ray generators: forward and right
// axes (V3c::normalized, V3c::cross order of operations), tan(fov / 2) from the
// fixed double-precision sin/cos above, and the aspect ratio.
void camera_frame(const float eye[3], const float target[3], float fov_deg, uint32_t width, uint32_t height,
                  CameraFrame* out) {
  const V3 e{eye[0], eye[1], eye[2]};
  const V3 fwd = normalized(sub(V3{target[0], target[1], target[2]}, e));
  const V3 up{0.0f, 1.0f, 0.0f};  // examples/cpu_render.rs:83-86
  const V3 right = normalized(cross(up, fwd));
  double s, c;
  det_sincos((double)fov_deg * kPi / 360.0, &s, &c);
  out->fwd[0] = fwd.x;
  out->fwd[1] = fwd.y;
  out->fwd[2] = fwd.z;
  out->right[0] = right.x;
  out->right[1] = right.y;
  out->right[2] = right.z;
  out->tan_half = (float)(s / c);
  out->aspect = (float)width / (float)height;
}
}  // namespace svo

using namespace svo;

extern "C" {

svo_status svo_gen_scene(const svo_scene_recipe* r, svo_op* ops, uint64_t max_ops, uint64_t* n_ops) {
  if (!r || !n_ops) return fail(SVO_ERR_ARGUMENT, "svo_gen_scene: NULL argument");
  if (r->size == 0 || r->size > 65536 || r->brick_dim == 0) return fail(SVO_ERR_ARGUMENT, "svo_gen_scene: bad size");
  OpSink sink(ops, max_ops);
  if (r->kind == 2)
    gen_sparse_blocks(*r, sink);
  else if (r->kind == 4)
    gen_boxes(*r, sink);
  else
    gen_dense(*r, sink);
  *n_ops = sink.count();
  return SVO_OK;
}

svo_status svo_gen_camera_rays(const float eye[3], const float target[3], float fov_deg, uint32_t width,
                               uint32_t height, float* ox, float* oy, float* oz, float* dx, float* dy, float* dz) {
  if (!eye || !target || !ox || !oy || !oz || !dx || !dy || !dz || !width || !height)
    return fail(SVO_ERR_ARGUMENT, "svo_gen_camera_rays: bad argument");
  CameraFrame f;
  camera_frame(eye, target, fov_deg, width, height, &f);
  const V3 fwd{f.fwd[0], f.fwd[1], f.fwd[2]}, right{f.right[0], f.right[1], f.right[2]};
  const V3 up{0.0f, 1.0f, 0.0f};  // examples/cpu_render.rs:83-86
  for (uint32_t py = 0; py < height; ++py)
    for (uint32_t px = 0; px < width; ++px) {
      const float u = (2.0f * ((float)px + 0.5f) / (float)width - 1.0f) * f.tan_half * f.aspect;
      const float v = (1.0f - 2.0f * ((float)py + 0.5f) / (float)height) * f.tan_half;
      const V3 d = normalized(add(add(fwd, mul(right, u)), mul(up, v)));
      const size_t i = (size_t)py * width + px;
      ox[i] = eye[0];
      oy[i] = eye[1];
      oz[i] = eye[2];
      dx[i] = d.x;
      dy[i] = d.y;
      dz[i] = d.z;
    }
  return SVO_OK;
}

svo_status svo_gen_sphere_rays(const float center[3], float radius, uint64_t n, uint64_t seed, float* ox, float* oy,
                               float* oz, float* dx, float* dy, float* dz) {
  if (!center || !ox || !oy || !oz || !dx || !dy || !dz) return fail(SVO_ERR_ARGUMENT, "svo_gen_sphere_rays: NULL");
  Pcg32 g(seed);
  auto on_sphere = [&](V3& out) {
    const double z = 2.0 * (double)g.unit() - 1.0;
    const double phi = 2.0 * kPi * (double)g.unit();
    double s, c;
    det_sincos(phi, &s, &c);
    const double rr = std::sqrt(std::max(0.0, 1.0 - z * z));
    out = V3{(float)(rr * c), (float)(rr * s), (float)z};
  };
  for (uint64_t i = 0; i < n; ++i) {
    V3 a, b;
    on_sphere(a);
    on_sphere(b);
    ox[i] = center[0] + radius * a.x;
    oy[i] = center[1] + radius * a.y;
    oz[i] = center[2] + radius * a.z;
    const V3 d = normalized(b);
    dx[i] = d.x;
    dy[i] = d.y;
    dz[i] = d.z;
  }
  return SVO_OK;
}

}  // extern "C"
