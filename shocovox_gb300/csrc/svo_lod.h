// svo_lod.h -- the MIP condition of Octree::get_by_ray_at_lod, for the device cast and a host check.
//
// get_by_ray_at_lod reads a node's MIP brick when
//   level < (origin - round(p / (2 level)) * 2 level).length() / viewing_distance
// (src/raytracing/raytracing_on_cpu.rs:366-375), evaluated in f32 at every node visit.  The grid
// point lies within sqrt(3) (level + 2^-20 (|p| + level)) of p: rounding to the grid moves each
// coordinate by at most level, the f32 division and product by far less.  So where |origin - p| is
// farther than that from level * viewing_distance the outcome is decided without the three
// divisions; margins of 2^-16 of level * viewing_distance cover every rounding of either
// evaluation.  Only level > 0 and viewing_distance > 0 take the shortcut.  The header compiles for
// the device (nvcc) and the host (a C++ test compares the two forms on random and boundary cases).
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define SVO_LOD_HD __host__ __device__ __forceinline__
#else
#define SVO_LOD_HD inline
#endif

namespace svo {

// the reference's f32 operations
SVO_LOD_HD bool lod_reads_mip_exact(float ox, float oy, float oz, float px, float py, float pz, float level,
                                    float viewing_distance) {
  const float m2 = level * 2.0f;
  const float ax = ox - roundf(px / m2) * m2, ay = oy - roundf(py / m2) * m2, az = oz - roundf(pz / m2) * m2;
  return level < sqrtf((ax * ax + ay * ay) + az * az) / viewing_distance;
}

SVO_LOD_HD bool lod_reads_mip(float ox, float oy, float oz, float px, float py, float pz, float level,
                              float viewing_distance) {
  if (level > 0.0f && viewing_distance > 0.0f) {
    const float ex = ox - px, ey = oy - py, ez = oz - pz;
    const float r2 = (ex * ex + ey * ey) + ez * ez;
    const float k = 1.7321f * (level + 0x1p-20f * (((fabsf(px) + fabsf(py)) + fabsf(pz)) + level));
    const float lv = level * viewing_distance;
    const float lo = lv * (1.0f - 0x1p-16f) - k, hi = lv * (1.0f + 0x1p-16f) + k;
    if (lo > 0.0f && r2 < (lo * lo) * (1.0f - 0x1p-16f)) return false;  // |origin - p| < lo: too close
    if (r2 > (hi * hi) * (1.0f + 0x1p-16f)) return true;                 // |origin - p| > hi: far enough
  }
  return lod_reads_mip_exact(ox, oy, oz, px, py, pz, level, viewing_distance);
}

}  // namespace svo
