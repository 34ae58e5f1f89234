// workloads.cpp -- TEST INFRASTRUCTURE ONLY.
//
// The benchmark's seeded synthetic workloads (scene construction op lists and
// ray batches), restated on the oracle side so that the CPU baseline of the
// benchmark's reference arm builds its scene and rays without loading any
// product code.  The recipes are this project's own definitions (the reference
// ships no datasets): PCG32 streams seeded through splitmix64, value noise on an
// integer lattice with smoothstep weights, fractal sums, pinhole cameras and
// rays uniform on a sphere.  Their op lists and rays must equal the product's
// generators bit for bit, which tests/test_oracle_workloads.py checks, so every
// f32/f64 operation below is spelled out in a fixed order (compiled with
// -ffp-contract=off; sin/cos by a fixed Taylor evaluation, no libm calls
// besides floor and sqrt, which IEEE-754 rounds exactly).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "svo_oracle.h"

namespace {

constexpr uint8_t kOpInsert = 0, kOpInsertAtLod = 2, kEntryComplex = 3;
constexpr double kPi = 3.14159265358979323846;

// ---- random streams -------------------------------------------------------
class Stream {
 public:
  explicit Stream(uint64_t seed) : mix_(seed) {
    state_ = mix();
    inc_ = mix() | 1u;
  }
  uint32_t next() {  // PCG32, XSH RR output
    const uint64_t s = state_;
    state_ = s * 6364136223846793005ull + inc_;
    const uint32_t x = (uint32_t)(((s >> 18u) ^ s) >> 27u);
    const uint32_t r = (uint32_t)(s >> 59u);
    return (x >> r) | (x << ((32u - r) & 31u));
  }
  float unit() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
  uint32_t below(uint32_t lo, uint32_t hi) { return lo + next() % (hi - lo); }

 private:
  uint64_t mix() {  // splitmix64
    mix_ += 0x9E3779B97F4A7C15ull;
    uint64_t z = mix_;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  uint64_t mix_, state_ = 0, inc_ = 0;
};

// ---- value noise ----------------------------------------------------------
float corner(int32_t x, int32_t y, int32_t z, uint32_t seed) {
  uint32_t h = ((uint32_t)x * 0x8DA6B343u) ^ ((uint32_t)y * 0xD8163841u) ^ ((uint32_t)z * 0xCB1AB31Fu) ^
               (seed * 0x9E3779B9u);
  h = (h ^ (h >> 16)) * 0x7FEB352Du;
  h = (h ^ (h >> 15)) * 0x846CA68Bu;
  h = h ^ (h >> 16);
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}
float fade(float t) { return (t * t) * (3.0f - 2.0f * t); }
float mixf(float a, float b, float t) { return a + (b - a) * t; }

float noise2(float x, float z, uint32_t seed) {
  const float x0 = std::floor(x), z0 = std::floor(z);
  const int32_t i = (int32_t)x0, k = (int32_t)z0;
  const float wx = fade(x - x0), wz = fade(z - z0);
  const float near = mixf(corner(i, 0, k, seed), corner(i + 1, 0, k, seed), wx);
  const float far = mixf(corner(i, 0, k + 1, seed), corner(i + 1, 0, k + 1, seed), wx);
  return mixf(near, far, wz);
}
float noise3(float x, float y, float z, uint32_t seed) {
  const float x0 = std::floor(x), y0 = std::floor(y), z0 = std::floor(z);
  const int32_t i = (int32_t)x0, j = (int32_t)y0, k = (int32_t)z0;
  const float wx = fade(x - x0), wy = fade(y - y0), wz = fade(z - z0);
  // edges along x at (y, z) = (j, k), (j+1, k), (j, k+1), (j+1, k+1)
  const float e00 = mixf(corner(i, j, k, seed), corner(i + 1, j, k, seed), wx);
  const float e01 = mixf(corner(i, j, k + 1, seed), corner(i + 1, j, k + 1, seed), wx);
  const float e10 = mixf(corner(i, j + 1, k, seed), corner(i + 1, j + 1, k, seed), wx);
  const float e11 = mixf(corner(i, j + 1, k + 1, seed), corner(i + 1, j + 1, k + 1, seed), wx);
  return mixf(mixf(e00, e10, wy), mixf(e01, e11, wy), wz);
}
// octave o: amplitude 2^-o, frequency 2^o, seed + o * step; the sum is divided by the amplitudes' sum
float fractal2(float x, float z, uint32_t octaves, uint32_t seed) {
  float acc = 0.0f, amps = 0.0f, amp = 1.0f, freq = 1.0f;
  for (uint32_t o = 0; o < octaves; ++o) {
    acc = acc + amp * noise2(x * freq, z * freq, seed + o * 101u);
    amps = amps + amp;
    amp = amp * 0.5f;
    freq = freq * 2.0f;
  }
  return acc / amps;
}
float fractal3(float x, float y, float z, uint32_t octaves, uint32_t seed) {
  float acc = 0.0f, amps = 0.0f, amp = 1.0f, freq = 1.0f;
  for (uint32_t o = 0; o < octaves; ++o) {
    acc = acc + amp * noise3(x * freq, y * freq, z * freq, seed + o * 131u);
    amps = amps + amp;
    amp = amp * 0.5f;
    freq = freq * 2.0f;
  }
  return acc / amps;
}

// sin and cos of x by reduction to [-pi/4, pi/4] (nearest multiple of pi/2) and 12 Taylor terms each
void sin_cos(double x, double* s_out, double* c_out) {
  const double q = std::floor(x / (kPi / 2.0) + 0.5);
  const double r = x - q * (kPi / 2.0);
  const double r2 = r * r;
  double s = 0.0, c = 0.0, ts = r, tc = 1.0;
  for (int n = 0; n < 12; ++n) {
    s = s + ts;
    c = c + tc;
    ts = -ts * r2 / (double)((2 * n + 2) * (2 * n + 3));
    tc = -tc * r2 / (double)((2 * n + 1) * (2 * n + 2));
  }
  switch ((((int)q % 4) + 4) % 4) {
    case 0: *s_out = s; *c_out = c; break;
    case 1: *s_out = c; *c_out = -s; break;
    case 2: *s_out = -s; *c_out = -c; break;
    default: *s_out = -c; *c_out = s; break;
  }
}

// ---- colours --------------------------------------------------------------
uint32_t rgba8(uint32_t r, uint32_t g, uint32_t b) { return (r << 24) | (g << 16) | (b << 8) | 0xFFu; }
uint32_t height_band_color(uint32_t band) {
  return rgba8(60 + (band * 3) % 160, 90 + (band * 5) % 140, 40 + (band * 7) % 120);
}
uint32_t color_565(Stream& g) {
  const uint32_t v = g.next();
  return rgba8((v & 31u) << 3, ((v >> 5) & 63u) << 2, ((v >> 11) & 31u) << 3);
}

orc_op make_op(uint8_t op, uint32_t x, uint32_t y, uint32_t z, uint32_t size, uint32_t rgba, uint32_t user) {
  orc_op o;
  o.x = (uint16_t)x;
  o.y = (uint16_t)y;
  o.z = (uint16_t)z;
  o.op = op;
  o.kind = kEntryComplex;
  o.size = size;
  o.rgba = rgba;
  o.user = user;
  return o;
}

struct Ball {
  float x, y, z, r2;
  uint32_t rgba, user;
};

// kinds 0 (heightfield + spheres), 1 (terrain with caves) and 3 (thresholded 3D noise + spheres):
// every voxel in x -> y -> z order; the first sphere containing the voxel centre wins
void dense_scene(const orc_recipe& r, std::vector<orc_op>& out) {
  const uint32_t S = r.size;
  const uint32_t oct = r.octaves ? r.octaves : 1;
  Stream g(r.seed);
  std::vector<Ball> balls;
  for (uint32_t i = 0; i < r.spheres; ++i) {
    Ball b;
    const float grow = (float)S / 128.0f > 1.0f ? (float)S / 128.0f : 1.0f;
    const float radius = 4.0f + g.unit() * 12.0f * grow;
    b.x = g.unit() * (float)S;
    b.y = g.unit() * (float)S;
    b.z = g.unit() * (float)S;
    b.r2 = radius * radius;
    b.rgba = color_565(g);
    b.user = 1000u + i;
    balls.push_back(b);
  }
  const uint32_t nseed = (uint32_t)(r.seed * 2654435761ull);
  std::vector<float> ground((size_t)S * S);
  for (uint32_t x = 0; x < S; ++x)
    for (uint32_t z = 0; z < S; ++z)
      ground[(size_t)x * S + z] =
          r.height_lo + (r.height_hi - r.height_lo) * fractal2((float)x * r.base_freq, (float)z * r.base_freq, oct, nseed);
  float level = 1.0f - r.occupancy;
  if (r.kind == 3) {  // the noise value with the target occupancy above it, from 8192 samples
    Stream gs(r.seed ^ 0xABCDull);
    std::vector<float> v(8192);
    for (float& s : v) {
      const float uz = gs.unit(), uy = gs.unit(), ux = gs.unit();
      s = fractal3(ux * (float)S * r.base_freq, uy * (float)S * r.base_freq, uz * (float)S * r.base_freq, oct,
                   nseed + 7u);
    }
    std::sort(v.begin(), v.end());
    const size_t at = (size_t)((1.0f - r.occupancy) * 8191.0f);
    level = v[std::min<size_t>(at, 8191)];
  }
  auto voxels_of_slab = [&](uint32_t x_lo, uint32_t x_hi, std::vector<orc_op>& ops) {
    for (uint32_t x = x_lo; x < x_hi; ++x)
      for (uint32_t y = 0; y < S; ++y)
        for (uint32_t z = 0; z < S; ++z) {
          const float cx = (float)x + 0.5f, cy = (float)y + 0.5f, cz = (float)z + 0.5f;
          const Ball* in = nullptr;
          for (const Ball& b : balls) {
            const float dx = cx - b.x, dy = cy - b.y, dz = cz - b.z;
            if ((dx * dx + dy * dy) + dz * dz <= b.r2) {
              in = &b;
              break;
            }
          }
          if (in) {
            ops.push_back(make_op(kOpInsert, x, y, z, 1, in->rgba, in->user));
            continue;
          }
          bool fill = false;
          if (r.kind == 3) {
            fill = fractal3(cx * r.base_freq, cy * r.base_freq, cz * r.base_freq, oct, nseed + 7u) > level;
          } else if (r.kind == 0 || r.kind == 1) {
            fill = (float)y <= ground[(size_t)x * S + z];
            if (fill && r.kind == 1 && y > 0) {
              fill = !(fractal3(cx * r.base_freq * 4.0f, cy * r.base_freq * 4.0f, cz * r.base_freq * 4.0f, 2, nseed + 3u) >
                       r.cave_threshold);
            }
          }
          if (fill) {
            const uint32_t band = y * 64u / S;
            ops.push_back(make_op(kOpInsert, x, y, z, 1, height_band_color(band), 1u + band));
          }
        }
  };
  const uint32_t threads = std::max(1u, std::min(S, std::min(64u, std::thread::hardware_concurrency())));
  std::vector<std::vector<orc_op>> part(threads);
  std::vector<std::thread> pool;
  for (uint32_t t = 0; t < threads; ++t)
    pool.emplace_back(voxels_of_slab, (uint32_t)((uint64_t)S * t / threads), (uint32_t)((uint64_t)S * (t + 1) / threads),
                      std::ref(part[t]));
  for (std::thread& t : pool) t.join();
  for (const auto& p : part) out.insert(out.end(), p.begin(), p.end());
}

// kind 2: cells of 2*brick_dim voxels occupied at random; 30% of them one insert_at_lod of the whole
// cell, the rest single voxels where 3D noise (lattice step 4 voxels) exceeds 0.68
void block_scene(const orc_recipe& r, std::vector<orc_op>& out) {
  const uint32_t S = r.size, cell = 2 * r.brick_dim, n = S / cell;
  Stream g(r.seed);
  const uint32_t nseed = (uint32_t)(r.seed * 2246822519ull);
  const float voxels_per_cell = (float)cell * cell * cell * (0.3f + 0.7f * 0.25f);
  const float wanted = (float)S * S * S * r.occupancy;
  const float p = std::min(1.0f, wanted / voxels_per_cell / ((float)n * n * n));
  for (uint32_t i = 0; i < n; ++i)
    for (uint32_t j = 0; j < n; ++j)
      for (uint32_t k = 0; k < n; ++k) {
        if (!(g.unit() < p)) continue;
        const uint32_t rgba = color_565(g);
        const uint32_t user = 1u + g.below(0, 64);
        if (g.unit() < 0.3f) {
          out.push_back(make_op(kOpInsertAtLod, i * cell, j * cell, k * cell, cell, rgba, user));
          continue;
        }
        for (uint32_t x = i * cell; x < (i + 1) * cell; ++x)
          for (uint32_t y = j * cell; y < (j + 1) * cell; ++y)
            for (uint32_t z = k * cell; z < (k + 1) * cell; ++z)
              if (noise3((float)x * 0.25f, (float)y * 0.25f, (float)z * 0.25f, nseed) > 0.68f)
                out.push_back(make_op(kOpInsert, x, y, z, 1, rgba, user));
      }
}

// kind 4: random axis-aligned boxes of whole cells (one insert_at_lod per cell) until the target
// occupancy is placed; every 20th box gets a noise-carved cell of single voxels on its top face
void box_scene(const orc_recipe& r, std::vector<orc_op>& out) {
  const uint32_t S = r.size, cell = 2 * r.brick_dim, n = S / cell;
  Stream g(r.seed);
  const uint32_t nseed = (uint32_t)(r.seed * 3266489917ull);
  const double wanted = (double)S * S * S * r.occupancy;
  double placed = 0.0;
  for (uint32_t box = 0; placed < wanted && n >= 2; ++box) {
    const uint32_t span = std::max(2u, n / 14);
    const uint32_t w = std::min(n, 1u + g.below(0, span));
    const uint32_t h = std::min(n, 1u + g.below(0, span));
    const uint32_t d = std::min(n, 1u + g.below(0, span));
    const uint32_t x0 = g.below(0, n - w + 1);
    const uint32_t y0 = g.below(0, n - h + 1);
    const uint32_t z0 = g.below(0, n - d + 1);
    const uint32_t rgba = color_565(g);
    const uint32_t user = 1u + g.below(0, 255);
    for (uint32_t x = x0; x < x0 + w; ++x)
      for (uint32_t y = y0; y < y0 + h; ++y)
        for (uint32_t z = z0; z < z0 + d; ++z)
          out.push_back(make_op(kOpInsertAtLod, x * cell, y * cell, z * cell, cell, rgba, user));
    placed += (double)w * h * d * cell * cell * cell;
    if (box % 20 == 0 && y0 + h < n) {
      const uint32_t bx = x0 * cell, by = (y0 + h) * cell, bz = z0 * cell;
      for (uint32_t x = bx; x < bx + cell; ++x)
        for (uint32_t y = by; y < by + cell; ++y)
          for (uint32_t z = bz; z < bz + cell; ++z)
            if (noise3((float)x * 0.3f, (float)y * 0.3f, (float)z * 0.3f, nseed) > 0.6f)
              out.push_back(make_op(kOpInsert, x, y, z, 1, rgba, user + 1));
    }
  }
}

struct Vec {
  float x, y, z;
};
// V3c::<f32>::normalized (src/spatial/math/vector.rs:75-81): divide by sqrt((x*x + y*y) + z*z)
Vec unit_vec(Vec v) {
  const float len = std::sqrt((v.x * v.x + v.y * v.y) + v.z * v.z);
  return Vec{v.x / len, v.y / len, v.z / len};
}

}  // namespace

extern "C" {

int orc_gen_scene(const orc_recipe* r, orc_op* ops, uint64_t max_ops, uint64_t* n_ops) {
  if (!r || !n_ops || r->size == 0 || r->size > 65536 || r->brick_dim == 0) return ORC_ERR_ARGUMENT;
  std::vector<orc_op> out;
  if (r->kind == 2)
    block_scene(*r, out);
  else if (r->kind == 4)
    box_scene(*r, out);
  else
    dense_scene(*r, out);
  *n_ops = out.size();
  if (ops) std::copy(out.begin(), out.begin() + (ptrdiff_t)std::min<uint64_t>(max_ops, out.size()), ops);
  return ORC_OK;
}

int orc_gen_camera_rays_strided(const float eye[3], const float target[3], float fov_deg, uint32_t width,
                                uint32_t height, uint64_t first, uint64_t stride, uint64_t n, float* ox, float* oy,
                                float* oz, float* dx, float* dy, float* dz) {
  if (!eye || !target || !ox || !oy || !oz || !dx || !dy || !dz || !width || !height || !stride) return ORC_ERR_ARGUMENT;
  if (n && first + (n - 1) * stride >= (uint64_t)width * height) return ORC_ERR_ARGUMENT;
  const Vec fwd = unit_vec(Vec{target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]});
  const Vec up{0.0f, 1.0f, 0.0f};  // examples/cpu_render.rs:83-86
  // up x fwd (V3c::cross, vector.rs:186-192)
  const Vec right = unit_vec(Vec{up.y * fwd.z - up.z * fwd.y, up.z * fwd.x - up.x * fwd.z, up.x * fwd.y - up.y * fwd.x});
  double s, c;
  sin_cos((double)fov_deg * kPi / 360.0, &s, &c);
  const float t = (float)(s / c), aspect = (float)width / (float)height;
  for (uint64_t k = 0; k < n; ++k) {
    const uint64_t pixel = first + k * stride;
    const uint32_t px = (uint32_t)(pixel % width), py = (uint32_t)(pixel / width);
    const float v = (1.0f - 2.0f * ((float)py + 0.5f) / (float)height) * t;
    const float u = (2.0f * ((float)px + 0.5f) / (float)width - 1.0f) * t * aspect;
    const Vec sum{(fwd.x + right.x * u) + up.x * v, (fwd.y + right.y * u) + up.y * v, (fwd.z + right.z * u) + up.z * v};
    const Vec d = unit_vec(sum);
    ox[k] = eye[0];
    oy[k] = eye[1];
    oz[k] = eye[2];
    dx[k] = d.x;
    dy[k] = d.y;
    dz[k] = d.z;
  }
  return ORC_OK;
}

int orc_gen_camera_rays(const float eye[3], const float target[3], float fov_deg, uint32_t width, uint32_t height,
                        float* ox, float* oy, float* oz, float* dx, float* dy, float* dz) {
  return orc_gen_camera_rays_strided(eye, target, fov_deg, width, height, 0, 1, (uint64_t)width * height, ox, oy, oz,
                                     dx, dy, dz);
}

int orc_gen_sphere_rays(const float center[3], float radius, uint64_t n, uint64_t seed, float* ox, float* oy, float* oz,
                        float* dx, float* dy, float* dz) {
  if (!center || !ox || !oy || !oz || !dx || !dy || !dz) return ORC_ERR_ARGUMENT;
  Stream g(seed);
  auto uniform_on_sphere = [&]() {  // z uniform in [-1, 1), longitude uniform
    const double z = 2.0 * (double)g.unit() - 1.0;
    const double lon = 2.0 * kPi * (double)g.unit();
    double s, c;
    sin_cos(lon, &s, &c);
    const double ring = std::sqrt(std::max(0.0, 1.0 - z * z));
    return Vec{(float)(ring * c), (float)(ring * s), (float)z};
  };
  for (uint64_t i = 0; i < n; ++i) {
    const Vec a = uniform_on_sphere();
    const Vec b = uniform_on_sphere();
    ox[i] = center[0] + radius * a.x;
    oy[i] = center[1] + radius * a.y;
    oz[i] = center[2] + radius * a.z;
    const Vec d = unit_vec(b);
    dx[i] = d.x;
    dy[i] = d.y;
    dz[i] = d.z;
  }
  return ORC_OK;
}

}  // extern "C"
