// Checks svo::nudge_run and svo::restart_cells_run (shocovox_gb300/csrc/svo_restart.h) against
// performing every addition p <- fl(p + c).  Built and run by tests/test_restart_run.py with
// -ffp-contract=off; exits 0 when every case agrees and prints the first disagreement otherwise.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "../shocovox_gb300/csrc/svo_restart.h"

using svo::f32_bits;
using svo::f32_from;
using svo::kRunNever;

static uint64_t g_state = 0x9E3779B97F4A7C15ull;
static uint64_t next_u64() {
  g_state += 0x9E3779B97F4A7C15ull;
  uint64_t z = g_state;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double uni() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

// one addition at a time
static uint32_t brute(float& p, float c, float lo, float hi, uint32_t n_max) {
  uint32_t k = 0;
  while (k < n_max) {
    const float q = p + c;
    if (q == p) return kRunNever;
    ++k;
    p = q;
    if (svo::run_left(p, c, lo, hi)) return k;
  }
  return k;
}

static int check_run(float p0, float c, float lo, float hi, uint32_t n_max, long& cases) {
  float a = p0, b = p0;
  const uint32_t ka = svo::nudge_run(a, c, lo, hi, n_max);
  const uint32_t kb = brute(b, c, lo, hi, n_max);
  ++cases;
  if (ka != kb || f32_bits(a) != f32_bits(b)) {
    printf("MISMATCH nudge_run p=%a c=%a lo=%a hi=%a n_max=%u: got k=%u p=%a, additions give k=%u p=%a\n", p0, c, lo,
           hi, n_max, ka, a, kb, b);
    return 1;
  }
  return 0;
}

// cell interval [j w, (j + 1) w) of p for an octree of size s
static void cell(float p, float s, float& lo, float& hi) {
  const float w = s * 0.25f;
  uint32_t j = (uint32_t)(p * (4.0f / s));
  j = j > 3u ? 3u : j;
  lo = (float)j * w;
  hi = (float)(j + 1u) * w;
}

int main(int argc, char** argv) {
  const long n_random = argc > 1 ? atol(argv[1]) : 200000;
  const float sizes[] = {16.0f, 64.0f, 512.0f, 2048.0f, 4096.0f, 65536.0f};
  long cases = 0;
  const uint32_t kBruteLimit = 1u << 17;  // additions the brute force may take per case
  for (long i = 0; i < n_random; ++i) {
    const float s = sizes[next_u64() % 6];
    // points spread over many binades, including very small ones
    const double mode = uni();
    float p;
    if (mode < 0.6) {
      p = (float)(uni() * s);
    } else if (mode < 0.8) {
      p = (float)std::ldexp(1.0 + uni(), -(int)(next_u64() % 30));
    } else {  // at or next to a binade edge or a cell boundary
      const float edge = mode < 0.9 ? std::ldexp(1.0f, (int)(next_u64() % 12) - 2) : (float)(next_u64() % 4) * s * 0.25f;
      const int off = (int)(next_u64() % 9) - 4;
      p = f32_from(f32_bits(edge) + off);
    }
    if (!(p > 0.0f) || !(p < s)) continue;
    // direction component times 0.1, magnitudes from 1 down to 1e-9, both signs and zeros
    const double mag = std::pow(10.0, -9.0 * uni() * uni());
    float d = (float)(mag * (uni() < 0.5 ? -1.0 : 1.0));
    const uint64_t z = next_u64() % 64;
    if (z == 0) d = 0.0f;
    if (z == 1) d = -0.0f;
    float c = d * 0.1f;
    if (next_u64() % 8 == 0) {  // a tie: c an odd multiple of half the spacing of p's binade
      const float u = f32_from(f32_bits(p) & 0x7F800000u) * std::ldexp(1.0f, -23);
      const int j = (int)(next_u64() % 7);
      c = (float)((j + 0.5) * u) * (uni() < 0.5 ? -1.0f : 1.0f);
      if (next_u64() % 2) c = (float)((j + 0.5) * u * 2.0) * (c < 0 ? -1.0f : 1.0f);  // tie one binade up
    }
    float lo, hi;
    cell(p, s, lo, hi);
    const uint32_t limits[] = {kBruteLimit, 1u + (uint32_t)(next_u64() % 64), 1u + (uint32_t)(next_u64() % 100000)};
    for (uint32_t n_max : limits)
      if (check_run(p, c, lo, hi, n_max, cases)) return 1;
  }
  // whole restart runs: three axes, the first cell change of any of them
  for (long i = 0; i < n_random / 4; ++i) {
    const float s = sizes[next_u64() % 6];
    float x = (float)(uni() * s), y = (float)(uni() * s), zz = (float)(uni() * s);
    if (!(x > 0.0f && y > 0.0f && zz > 0.0f)) continue;
    float dx = (float)(uni() * 2 - 1), dy = (float)(uni() * 2 - 1), dz = (float)(uni() * 2 - 1);
    const float nn = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (!(nn > 0.0f)) continue;
    dx /= nn;
    dy /= nn;
    dz /= nn;
    if (next_u64() % 4 == 0) dy = 0.0f;
    const float cx = dx * 0.1f, cy = dy * 0.1f, cz = dz * 0.1f;
    const float q4 = 4.0f / s;
    auto cell_of = [&](float v) {
      uint32_t j = (uint32_t)(v * q4);
      return j > 3u ? 3u : j;
    };
    const uint32_t flat = cell_of(x) + 4u * cell_of(y) + 16u * cell_of(zz);
    const uint32_t n_max = next_u64() % 3 == 0 ? 1u + (uint32_t)(next_u64() % 2000) : kBruteLimit;
    float ax = x, ay = y, az = zz;
    const uint32_t k = svo::restart_cells_run(ax, ay, az, cx, cy, cz, flat, s * 0.25f, n_max);
    // brute force: add until the cell changes or the point leaves the octree
    float bx = x, by = y, bz = zz;
    uint32_t kb = 0;
    for (;;) {
      if (kb + 1 >= n_max + 1) {
        kb = kRunNever;
        break;
      }
      const float nx = bx + cx, ny = by + cy, nz = bz + cz;
      if (nx == bx && ny == by && nz == bz) {
        kb = kRunNever;
        break;
      }
      ++kb;
      bx = nx;
      by = ny;
      bz = nz;
      const bool inside = bx < s && by < s && bz < s && bx > 0.0f && by > 0.0f && bz > 0.0f;
      if (!inside || cell_of(bx) + 4u * cell_of(by) + 16u * cell_of(bz) != flat) break;
    }
    ++cases;
    if (kb == kRunNever || kb >= n_max) {
      if (k != kRunNever || f32_bits(ax) != f32_bits(x) || f32_bits(ay) != f32_bits(y) ||
          f32_bits(az) != f32_bits(zz)) {
        printf("MISMATCH restart_cells_run (no change expected) s=%g p=(%a,%a,%a) c=(%a,%a,%a) n_max=%u k=%u\n", s, x,
               y, zz, cx, cy, cz, n_max, k);
        return 1;
      }
    } else if (k != kb || f32_bits(ax) != f32_bits(bx) || f32_bits(ay) != f32_bits(by) ||
               f32_bits(az) != f32_bits(bz)) {
      printf("MISMATCH restart_cells_run s=%g p=(%a,%a,%a) c=(%a,%a,%a) n_max=%u: got k=%u (%a,%a,%a), additions "
             "give k=%u (%a,%a,%a)\n",
             s, x, y, zz, cx, cy, cz, n_max, k, ax, ay, az, kb, bx, by, bz);
      return 1;
    }
  }
  // runs until the point leaves the octree
  for (long i = 0; i < n_random / 4; ++i) {
    const float s = sizes[next_u64() % 6];
    const float x = (float)(uni() * s), y = (float)(uni() * s), zz = (float)(uni() * s);
    if (!(x > 0.0f && y > 0.0f && zz > 0.0f)) continue;
    float d[3] = {(float)(uni() * 2 - 1), (float)(uni() * 2 - 1), (float)(uni() * 2 - 1)};
    const float nn = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (!(nn > 0.0f)) continue;
    for (float& v : d) v /= nn;
    if (next_u64() % 5 == 0) d[next_u64() % 3] = 0.0f;
    if (next_u64() % 7 == 0) d[next_u64() % 3] *= 1e-6f;
    const float cx = d[0] * 0.1f, cy = d[1] * 0.1f, cz = d[2] * 0.1f;
    const uint32_t n_max = next_u64() % 3 == 0 ? 1u + (uint32_t)(next_u64() % 5000) : kBruteLimit;
    float ax = x, ay = y, az = zz;
    const uint32_t k = svo::restart_exit_run(ax, ay, az, cx, cy, cz, s, n_max);
    float bx = x, by = y, bz = zz;
    uint32_t kb = 0;
    for (;;) {
      if (kb >= n_max) {
        kb = kRunNever;
        break;
      }
      const float nx = bx + cx, ny = by + cy, nz = bz + cz;
      if (nx == bx && ny == by && nz == bz) {
        kb = kRunNever;
        break;
      }
      ++kb;
      bx = nx;
      by = ny;
      bz = nz;
      if (!(bx < s && by < s && bz < s && bx > 0.0f && by > 0.0f && bz > 0.0f)) break;
    }
    ++cases;
    if (kb != kRunNever && kb >= n_max) kb = kRunNever;
    const bool same = kb == kRunNever ? (k == kRunNever && f32_bits(ax) == f32_bits(x) && f32_bits(ay) == f32_bits(y) &&
                                         f32_bits(az) == f32_bits(zz))
                                      : (k == kb && f32_bits(ax) == f32_bits(bx) && f32_bits(ay) == f32_bits(by) &&
                                         f32_bits(az) == f32_bits(bz));
    if (!same) {
      printf("MISMATCH restart_exit_run s=%g p=(%a,%a,%a) c=(%a,%a,%a) n_max=%u: got k=%u, additions give k=%u\n", s, x,
             y, zz, cx, cy, cz, n_max, k, kb);
      return 1;
    }
  }
  printf("OK %ld cases\n", cases);
  return 0;
}
