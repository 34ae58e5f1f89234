// svo_restart.h -- restart runs of Octree::get_by_ray without one addition per restart.
//
// When the 4-entry node stack empties, get_by_ray moves the current point by
// direction * 0.1 and starts again from the root (src/raytracing/raytracing_on_cpu.rs:548-562).
// While the root's occupancy test fails (:430-446) every restart visits only the root and pops,
// so a ray crossing empty root cells repeats p <- fl(p + c), c = direction * 0.1, per axis, up
// to thousands of times.  The test depends only on the root bitmap cell of p, so every visit
// between two changes of that cell fails alike; nudge_run finds the number of additions until
// an axis leaves its cell, and the value they produce, bit for bit, without performing each one:
//
//  * In one binade [2^e, 2^(e+1)) the floats are the multiples of u = 2^(e-23).  When the exact
//    sum p + c lies in the binade, fl(p + c) is the multiple of u nearest to it.  If c / u is not
//    an odd multiple of 1/2 that is p + round(c / u) * u for every p of the binade; if it is (a
//    tie), round-to-even makes the result's significand even, and from an even significand the
//    step is again the same even number of u.
//  * So once two consecutive additions start and end in one binade, the second one's step D
//    (in units of u) repeats for as long as the exact sums stay in the binade, which holds while
//    each result's significand stays within [2^23 + 1, 2^24 - 1]; the run over those additions is
//    one multiply-add on the integer significand.  Additions near binade edges are performed one
//    by one.
//
// The header compiles for the device (nvcc) and the host (a C++ test checks it against
// performing every addition).
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define SVO_HD __host__ __device__ __forceinline__
#else
#define SVO_HD inline
#endif

namespace svo {

SVO_HD uint32_t f32_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
SVO_HD float f32_from(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

constexpr uint32_t kRunNever = 0xFFFFFFFFu;

// Leaves [lo, hi) in the direction of c: upward at hi, downward below lo or at 0 and below
// (the restart's `p > 0.` bound).
SVO_HD bool run_left(float p, float c, float lo, float hi) { return c > 0.0f ? p >= hi : (p < lo || p <= 0.0f); }

// Performs up to n_max additions p <- fl(p + c) and returns how many were made when p first left
// [lo, hi) (see run_left), n_max when it had not left by then, or kRunNever when an addition left
// p unchanged first (p then never changes again).  p holds the value after the additions made.
// Requires p in [lo, hi), p > 0, lo >= 0 and c not NaN.
SVO_HD uint32_t nudge_run(float& p, float c, float lo, float hi, uint32_t n_max) {
  uint32_t k = 0;
  bool prev_in_binade = false;  // the addition that produced p started and ended in one binade
  while (k < n_max) {
    const float q = p + c;
    if (q == p) return kRunNever;
    ++k;
    const uint32_t pb = f32_bits(p), qb = f32_bits(q);
    const bool in_binade = (pb >> 23) == (qb >> 23);  // same sign and exponent
    p = q;
    if (run_left(q, c, lo, hi)) return k;
    const uint32_t E = qb >> 23;
    if (in_binade && prev_in_binade && k < n_max && E >= 24u && E <= 253u) {
      const int32_t M = (int32_t)((qb & 0x7FFFFFu) | 0x800000u);
      const int32_t D = M - (int32_t)((pb & 0x7FFFFFu) | 0x800000u);
      // additions whose results keep the significand within [2^23 + 1, 2^24 - 1]
      int32_t t = D > 0 ? (0xFFFFFF - M) / D : (M - 0x800001) / (-D);
      if (D > 0) {
        if (hi < f32_from((E + 1u) << 23)) {  // hi lies in this binade: first t with M + t D >= H
          const int32_t H = (int32_t)((f32_bits(hi) & 0x7FFFFFu) | 0x800000u);
          const int32_t tl = (H - M + D - 1) / D;
          t = tl < t ? tl : t;
        }
      } else if (lo >= f32_from(E << 23)) {  // lo lies in this binade: first t with M + t D < L
        const int32_t L = (int32_t)((f32_bits(lo) & 0x7FFFFFu) | 0x800000u);
        const int32_t tl = (M - L) / (-D) + 1;
        t = tl < t ? tl : t;
      }
      if (t > 0 && (uint32_t)t > n_max - k) t = (int32_t)(n_max - k);
      if (t > 0) {
        p = f32_from((E << 23) | ((uint32_t)(M + t * D) & 0x7FFFFFu));
        k += (uint32_t)t;
        if (run_left(p, c, lo, hi)) return k;
      }
    }
    prev_in_binade = in_binade;
  }
  return k;
}

// Number of restarts k >= 1 after which the point (x, y, z), inside the box [lx, hx) x [ly, hy) x
// [lz, hz), first leaves it (see run_left), moving it by (cx, cy, cz) per restart to its value
// after those k restarts.  Returns kRunNever (the point is left unchanged) when that takes n_max
// restarts or more, or never happens.
SVO_HD uint32_t restart_box_run(float& x, float& y, float& z, float cx, float cy, float cz, float lx, float hx,
                                float ly, float hy, float lz, float hz, uint32_t n_max) {
  float ax = x, ay = y, az = z;
  const uint32_t kx = nudge_run(ax, cx, lx, hx, n_max);
  const uint32_t ky = nudge_run(ay, cy, ly, hy, n_max);
  const uint32_t kz = nudge_run(az, cz, lz, hz, n_max);
  uint32_t k = kx < ky ? kx : ky;
  k = k < kz ? k : kz;
  if (k >= n_max) return kRunNever;
  if (kx != k) {
    ax = x;
    nudge_run(ax, cx, lx, hx, k);
  }
  if (ky != k) {
    ay = y;
    nudge_run(ay, cy, ly, hy, k);
  }
  if (kz != k) {
    az = z;
    nudge_run(az, cz, lz, hz, k);
  }
  x = ax;
  y = ay;
  z = az;
  return k;
}

// The run until the point -- inside the octree, in root bitmap cell `flat` (x + 4 y + 16 z) --
// lies in another cell or outside the octree.  w = size / 4.
SVO_HD uint32_t restart_cells_run(float& x, float& y, float& z, float cx, float cy, float cz, uint32_t flat,
                                  float w, uint32_t n_max) {
  const float jx = (float)(flat & 3u), jy = (float)((flat >> 2) & 3u), jz = (float)(flat >> 4);
  return restart_box_run(x, y, z, cx, cy, cz, jx * w, (jx + 1.0f) * w, jy * w, (jy + 1.0f) * w, jz * w,
                         (jz + 1.0f) * w, n_max);
}

// The run until the point leaves the octree [0, S)^3.
SVO_HD uint32_t restart_exit_run(float& x, float& y, float& z, float cx, float cy, float cz, float S,
                                 uint32_t n_max) {
  return restart_box_run(x, y, z, cx, cy, cz, 0.0f, S, 0.0f, S, 0.0f, S, n_max);
}

}  // namespace svo
