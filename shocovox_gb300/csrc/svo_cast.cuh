// svo_cast.cuh -- device-side restatement of Octree::get_by_ray shared by the
// plain (one thread per ray) and the batched persistent cast kernels.
//
// The cast follows src/raytracing/raytracing_on_cpu.rs:99-565 of shocovox-rs
// v0.11.1 (MIP maps disabled) operation by operation; compiled with
// -fmad=false -prec-div=true -prec-sqrt=true -ftz=false so each f32
// operation rounds exactly like the Rust code.  The look-up tables of
// src/spatial/lut.rs are evaluated with bit arithmetic (svo_selftest_luts
// compares them with the reference constants).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "svo_internal.h"
#include "svo_lod.h"
#include "svo_restart.h"

namespace svo {

#define SVO_CUDA_TRY(call)                                                                  \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return fail(e_ == cudaErrorMemoryAllocation ? SVO_ERR_OUT_OF_MEMORY : SVO_ERR_CUDA,   \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                      \
  } while (0)

constexpr uint32_t kOob = 8;
constexpr uint32_t kWorkCap = 1u << 22;  // traversal steps per ray; the reference loops forever past it
constexpr float kTol = 0.00001f;         // FLOAT_ERROR_TOLERANCE (src/spatial/raytracing/mod.rs:5)

// ------------------------------------------------------------------ work claims
// Which rays a warp's claim covers.  Rays laid out as rows of `row` rays (a camera image, or
// several stacked) are claimed as blocks of 32 neighbouring rays, 2^shift wide and 32 / 2^shift
// rows high, whose traversals stay in step far longer than 32 rays of one row; the rays past the
// last full band of rows, and every ray of a batch without a row layout, are claimed 32
// consecutive rays at a time.  Any order gives the same hits: rays are independent.
struct ClaimOrder {
  uint64_t row = 0;       // rays per row; 0: no row layout
  uint64_t per_band = 0;  // blocks per band of rows
  uint64_t blocks = 0;    // claims that are blocks
  uint64_t tail = 0;      // first ray claimed 32 consecutive rays at a time
  uint64_t claims = 0;    // claims in all
  uint32_t shift = 3;     // log2 of the block width (3: 8 x 4, 4: 16 x 2)
};

inline ClaimOrder claim_order(uint64_t n, uint64_t row, uint32_t shift = 3) {
  ClaimOrder o;
  o.shift = shift;
  const uint64_t width = 1ull << shift, band = (32ull >> shift) * row;
  if (row >= width && n >= band) {
    o.row = row;
    o.per_band = (row + width - 1) / width;
    o.blocks = (n / band) * o.per_band;
    o.tail = (n / band) * band;
  }
  o.claims = o.blocks + (n - o.tail + 31) / 32;
  return o;
}

// the ray of `lane` in claim c, or n when the lane has none
__device__ __forceinline__ uint64_t claimed_ray(const ClaimOrder& o, uint64_t c, uint32_t lane, uint64_t n) {
  if (c < o.blocks) {
    const uint64_t band = c / o.per_band;
    const uint64_t col = ((c - band * o.per_band) << o.shift) + (lane & ((1u << o.shift) - 1u));
    return col < o.row ? ((band << (5 - o.shift)) + (lane >> o.shift)) * o.row + col : n;
  }
  const uint64_t i = o.tail + (c - o.blocks) * 32 + lane;
  return i < n ? i : n;
}

// ------------------------------------------------------------------ Rust f32 semantics
__device__ __forceinline__ float rmin(float a, float b) { return isnan(a) ? b : (isnan(b) ? a : (b < a ? b : a)); }
__device__ __forceinline__ float rmax(float a, float b) { return isnan(a) ? b : (isnan(b) ? a : (b > a ? b : a)); }
__device__ __forceinline__ float rsignum(float x) { return isnan(x) ? x : copysignf(1.0f, x); }
__device__ __forceinline__ float rclamp(float x, float lo, float hi) {
  x = (x < lo) ? lo : x;
  return (x > hi) ? hi : x;
}
// `f as i32` (truncate, saturate, NaN -> 0): exactly cvt.rzi.s32.f32
__device__ __forceinline__ int as_i32(float x) { return __float2int_rz(x); }
__device__ __forceinline__ int isignum(int v) { return (v > 0) - (v < 0); }

// ------------------------------------------------------------------ look-up tables as arithmetic
// RAY_TO_NODE_OCCUPANCY_BITMASK_LUT[pos][dir] (src/spatial/lut.rs:33-84, 255-896): the 4x4x4 box
// between cell pos = x + 4y + 16z and the far corner in direction octant dir.
__host__ __device__ constexpr uint64_t ray_to_node_mask(uint32_t pos, uint32_t dir) {
  const uint32_t x = pos & 3u, y = (pos >> 2) & 3u, z = (pos >> 4) & 3u;
  const uint32_t xm = (dir & 1u) ? ((0xFu << x) & 0xFu) : (0xFu >> (3u - x));
  const uint32_t ym = (dir & 4u) ? ((0xFu << y) & 0xFu) : (0xFu >> (3u - y));
  const uint32_t zm = (dir & 2u) ? ((0xFu << z) & 0xFu) : (0xFu >> (3u - z));
  const uint64_t X = (uint64_t)xm * 0x1111111111111111ull;
  const uint32_t y16 = (ym & 1u) * 0xFu | (ym & 2u) * 0x78u | (ym & 4u) * 0x3C0u | (ym & 8u) * 0x1E00u;
  const uint64_t Y = (uint64_t)y16 * 0x0001000100010001ull;
  const uint64_t Z = ((zm & 1u) ? 0xFFFFull : 0ull) | ((zm & 2u) ? 0xFFFF0000ull : 0ull) |
                     ((zm & 4u) ? 0xFFFF00000000ull : 0ull) | ((zm & 8u) ? 0xFFFF000000000000ull : 0ull);
  return X & Y & Z;
}
// BITMAP_MASK_FOR_OCTANT_LUT (lut.rs:199-208): the 2x2x2 block of octant o
__host__ __device__ constexpr uint64_t octant_mask(uint32_t o) {
  const uint64_t X = (uint64_t)(3u << (2u * (o & 1u))) * 0x1111111111111111ull;
  const uint64_t Y = (uint64_t)(0xFFu << (8u * ((o >> 2) & 1u))) * 0x0001000100010001ull;
  const uint64_t Z = 0xFFFFFFFFull << (32u * ((o >> 1) & 1u));
  return X & Y & Z;
}
// step_octant + OCTANT_STEP_RESULT_LUT (src/spatial/raytracing/mod.rs:68-80, lut.rs:237-253)
__device__ __forceinline__ uint32_t step_octant(uint32_t o, float sx, float sy, float sz) {
  const int nx = (int)(o & 1u) + isignum(as_i32(sx));
  const int ny = (int)((o >> 2) & 1u) + isignum(as_i32(sy));
  const int nz = (int)((o >> 1) & 1u) + isignum(as_i32(sz));
  if ((unsigned)nx > 1u || (unsigned)ny > 1u || (unsigned)nz > 1u) return kOob;
  return (uint32_t)(nx + 2 * nz + 4 * ny);
}
// hash_region (src/spatial/math/mod.rs:11-19)
__device__ __forceinline__ uint32_t hash_region(float ox, float oy, float oz, float half) {
  return (uint32_t)(ox >= half) + 2u * (uint32_t)(oz >= half) + 4u * (uint32_t)(oy >= half);
}
// OCTANT_OFFSET_REGION_LUT (lut.rs:156-197)
__device__ __forceinline__ float offx(uint32_t o) { return (float)(o & 1u); }
__device__ __forceinline__ float offy(uint32_t o) { return (float)((o >> 2) & 1u); }
__device__ __forceinline__ float offz(uint32_t o) { return (float)((o >> 1) & 1u); }

// Every bounds size of the traversal is a power of two (the octree size is
// brick_dim * 2^k and sizes only halve or double), so `inv` = 1 / s is exact
// and x / s == x * inv bit for bit (both round the same exact value).
struct Bounds {
  float x, y, z, s, inv;
};
// Cube::child_bounds_for (src/spatial/mod.rs:32-39).  offset * half is half or +0 (offsets are 0 or 1)
// and minima are >= 0, so selecting the addend gives the reference's sums bit for bit.
__device__ __forceinline__ Bounds child_bounds(const Bounds& b, uint32_t o) {
  const float h = b.s * 0.5f;
  return Bounds{b.x + ((o & 1u) ? h : 0.0f), b.y + ((o & 4u) ? h : 0.0f), b.z + ((o & 2u) ? h : 0.0f), h,
                b.inv * 2.0f};
}

struct RayState {
  float dx, dy, dz;     // direction
  float gx, gy, gz;     // signum(direction)
  float fx, fy, fz;     // dda scale factors
  float px, py, pz;     // current point
};

// dda_step_to_next_sibling (raytracing_on_cpu.rs:124-152).
// kFast (direction without NaN, so signum is +-1): `size * max(g, 0) - g * e`
// is `size - e` for g = +1 and `0 - (-e)` = e (up to the sign of a zero,
// which the following abs() removes) for g = -1; the distances are >= 0 or
// NaN, where fminf equals the NaN-ignoring Rust f32::min.
template <bool kFast>
__device__ __forceinline__ void dda_step(RayState& r, const Bounds& b, float& sx, float& sy, float& sz) {
  const float ex = r.px - b.x, ey = r.py - b.y, ez = r.pz - b.z;
  float nx, ny, nz;
  if (kFast) {
    nx = r.gx > 0.0f ? b.s - ex : ex;
    ny = r.gy > 0.0f ? b.s - ey : ey;
    nz = r.gz > 0.0f ? b.s - ez : ez;
  } else {
    nx = b.s * rmax(r.gx, 0.0f) - r.gx * ex;
    ny = b.s * rmax(r.gy, 0.0f) - r.gy * ey;
    nz = b.s * rmax(r.gz, 0.0f) - r.gz * ez;
  }
  const float ax = fabsf(nx * r.fx), ay = fabsf(ny * r.fy), az = fabsf(nz * r.fz);
  const float m = kFast ? fminf(fminf(ax, ay), az) : rmin(rmin(ax, ay), az);
  r.px = r.px + r.dx * m;
  r.py = r.py + r.dy * m;
  r.pz = r.pz + r.dz * m;
  sx = (m == ax) ? r.gx : 0.0f;
  sy = (m == ay) ? r.gy : 0.0f;
  sz = (m == az) ? r.gz : 0.0f;
}

// cube_impact_normal (src/spatial/raytracing/mod.rs:106-134)
__device__ __forceinline__ void impact_normal(const Bounds& c, float px, float py, float pz, float& nx, float& ny,
                                              float& nz) {
  const float h = c.s * 0.5f;
  const float mx = (c.x + h) - px, my = (c.y + h) - py, mz = (c.z + h) - pz;
  const float m = rmax(rmax(fabsf(mx), fabsf(my)), fabsf(mz));
  const float vx = fabsf(mx) == m ? -mx : 0.0f;
  const float vy = fabsf(my) == m ? -my : 0.0f;
  const float vz = fabsf(mz) == m ? -mz : 0.0f;
  const float len = sqrtf((vx * vx + vy * vy) + vz * vz);
  nx = vx / len;
  ny = vy / len;
  nz = vz / len;
}

struct HitRecord {
  uint32_t status, octant, node, voxel, pix;
  float px, py, pz, nx, ny, nz;
  uint32_t visits, creads, vreads, runs;  // counters, kept only by the instrumented cast
};

enum : uint32_t { kKindNothing = 0, kKindInternal = 1, kKindLeaf = 2, kKindUniform = 3 };
enum : uint32_t { kBkEmpty = 0, kBkSolid = 1, kBkParted = 2 };

// Outcome of probe_brick: 0 miss, 1 hit, 2 work cap, 3 reference panic.
template <bool kCount, bool kFast>
__device__ __forceinline__ uint32_t probe_brick(const SceneView& s, RayState& r, uint32_t bk, uint32_t value,
                                                const Bounds& bb, HitRecord& h, uint32_t& work) {
  if (bk == kBkEmpty) return 0;
  if (bk == kBkSolid) {  // raytracing_on_cpu.rs:269-280
    h.pix = value;
    h.voxel = 0xFFFFFFFFu;
    h.px = r.px;
    h.py = r.py;
    h.pz = r.pz;
    impact_normal(bb, r.px, r.py, r.pz, h.nx, h.ny, h.nz);
    return 1;
  }
  // traverse_brick (raytracing_on_cpu.rs:156-252)
  const int D = (int)s.dim;
  const float Df = (float)s.dim;
  // x * D / size == (x * D) * (1 / size): size is a power of two
  int cx = min(max(as_i32((r.px - bb.x) * Df * bb.inv), 0), D - 1);
  int cy = min(max(as_i32((r.py - bb.y) * Df * bb.inv), 0), D - 1);
  int cz = min(max(as_i32((r.pz - bb.z) * Df * bb.inv), 0), D - 1);
  int flat = cx + cy * D + cz * D * D;
  const int D3 = D * D * D;
  const float unit = bb.s * s.inv_dim;  // brick_bounds.size / brick_dim, exact
  Bounds cur{bb.x + (float)cx * unit, bb.y + (float)cy * unit, bb.z + (float)cz * unit, unit, bb.inv * Df};
  const uint32_t* bits = s.vbits + (size_t)value * s.vwords;
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
  for (;;) {
    if (cx < 0 || cx >= D || cy < 0 || cy >= D || cz < 0 || cz >= D) return 0;
    flat += as_i32(sx) + as_i32(sy) * D + as_i32(sz) * D * D;
    if (flat < 0 || flat >= D3) return 3;
    if (kCount) h.vreads++;
    if (++work > kWorkCap) return 2;
    if ((__ldg(bits + (flat >> 5)) >> (flat & 31)) & 1u) {
      const Bounds hb{bb.x + (float)cx * bb.s * s.inv_dim, bb.y + (float)cy * bb.s * s.inv_dim,
                      bb.z + (float)cz * bb.s * s.inv_dim, unit, bb.inv * Df};
      h.pix = __ldg(s.voxels + (size_t)value * (size_t)D3 + (size_t)flat);
      h.voxel = (uint32_t)flat;
      h.px = r.px;
      h.py = r.py;
      h.pz = r.pz;
      impact_normal(hb, r.px, r.py, r.pz, h.nx, h.ny, h.nz);
      return 1;
    }
    dda_step<kFast>(r, cur, sx, sy, sz);
    cur.x = cur.x + sx * unit;
    cur.y = cur.y + sy * unit;
    cur.z = cur.z + sz * unit;
    cx += as_i32(roundf(sx));
    cy += as_i32(roundf(sy));
    cz += as_i32(roundf(sz));
  }
}

// BITMAP_INDEX_LUT lookup of a clamped bitmap position; false when the reference would index out of bounds.
__device__ __forceinline__ bool bitmap_index(float bx, float by, float bz, uint32_t& out) {
  const float fx = floorf(bx), fy = floorf(by), fz = floorf(bz);
  if (fx >= 4.0f || fy >= 4.0f || fz >= 4.0f) return false;
  const uint32_t ix = fx > 0.0f ? (uint32_t)fx : 0u;  // `as usize`: NaN and negatives become 0
  const uint32_t iy = fy > 0.0f ? (uint32_t)fy : 0u;
  const uint32_t iz = fz > 0.0f ? (uint32_t)fz : 0u;
  out = ix + 4u * iy + 16u * iz;
  return true;
}

// RAY_TO_NODE_OCCUPANCY_BITMASK_LUT and BITMAP_MASK_FOR_OCTANT_LUT staged in
// shared memory by each block (computed with the arithmetic above).
struct alignas(16) SharedLuts {
  uint64_t ray_to_node[512];  // [pos * 8 + dir]
  uint64_t octant[8];
};
// The tables, evaluated at compile time into each module's global memory; a block copies them
// into shared memory with 16-byte loads (two per thread at 128 threads).
constexpr SharedLuts make_luts() {
  SharedLuts t{};
  for (uint32_t i = 0; i < 512; ++i) t.ray_to_node[i] = ray_to_node_mask(i >> 3, i & 7u);
  for (uint32_t o = 0; o < 8; ++o) t.octant[o] = octant_mask(o);
  return t;
}
static __device__ const SharedLuts kLuts = make_luts();
__device__ __forceinline__ void fill_shared_luts(SharedLuts& L) {
  const uint4* src = reinterpret_cast<const uint4*>(&kLuts);
  uint4* dst = reinterpret_cast<uint4*>(&L);
  for (uint32_t i = threadIdx.x; i < sizeof(SharedLuts) / 16; i += blockDim.x) dst[i] = __ldg(src + i);
}

// Octree::get_by_ray (raytracing_on_cpu.rs:316-565, MIP maps disabled)
// kLod: get_by_ray_at_lod with MIP maps enabled (s.mips), reading a node's MIP brick when its
// level is below the one the travelled distance asks for (:366-386).
template <bool kCount, bool kFast, bool kLod = false>
__device__ void cast_ray(const SceneView& s, const SharedLuts& L, float ox, float oy, float oz, float dx, float dy,
                         float dz, HitRecord& h, float viewing_distance = 0.0f) {
  h.status = 0;
  h.octant = 0;
  h.node = 0;
  h.voxel = 0xFFFFFFFFu;
  h.pix = 0;
  h.px = h.py = h.pz = h.nx = h.ny = h.nz = 0.0f;
  if (kCount) h.visits = h.creads = h.vreads = h.runs = 0;

  RayState r;
  r.dx = dx;
  r.dy = dy;
  r.dz = dz;
  r.gx = rsignum(dx);
  r.gy = rsignum(dy);
  r.gz = rsignum(dz);
  {  // get_dda_scale_factors (:99-112); powf(q, 2.) == q * q
    const float a = dz / dx, b = dy / dx, c = dx / dy, d = dz / dy, e = dx / dz, f = dy / dz;
    r.fx = sqrtf((1.0f + a * a) + b * b);
    r.fy = sqrtf((c * c + 1.0f) + d * d);
    r.fz = sqrtf((e * e + 1.0f) + f * f);
  }
  const uint32_t dir = hash_region(1.0f + dx, 1.0f + dy, 1.0f + dz, 1.0f);  // hash_direction
  const uint64_t* rtn = L.ray_to_node + dir;
  const float S = s.size;
  Bounds cb{0.0f, 0.0f, 0.0f, S, s.inv_size};
  uint32_t target;
  {  // Cube::intersect_ray (src/spatial/raytracing/mod.rs:32-61) on the root bounds
    const float t1 = (0.0f - ox) / dx, t2 = ((0.0f + S) - ox) / dx;
    const float t3 = (0.0f - oy) / dy, t4 = ((0.0f + S) - oy) / dy;
    const float t5 = (0.0f - oz) / dz, t6 = ((0.0f + S) - oz) / dz;
    const float tmin = rmax(rmax(rmin(t1, t2), rmin(t3, t4)), rmin(t5, t6));
    const float tmax = rmin(rmin(rmax(t1, t2), rmax(t3, t4)), rmax(t5, t6));
    if (tmax < 0.0f || tmin > tmax) return;  // miss: target_octant = OOB
    const float t = tmin < 0.0f ? 0.0f : tmin;
    r.px = ox + dx * t;
    r.py = oy + dy * t;
    r.pz = oz + dz * t;
    target = hash_region(r.px - 0.0f, r.py - 0.0f, r.pz - 0.0f, S * 0.5f);
  }
  uint32_t work = 0;
  float mip_level = s.mip_top;  // (:350) kept across restarts
  while (target != kOob) {
    uint32_t cur = 0;
    cb = Bounds{0.0f, 0.0f, 0.0f, S, s.inv_size};
    // NodeStack<u32, 4> (:20-82) as a shift register: the newest entry in s0
    uint32_t s0 = 0, s1 = 0, s2 = 0, s3 = 0, count = 1;
    while (count > 0) {
      if (++work > kWorkCap) {
        h.status = 2;
        return;
      }
      if (kCount) h.visits++;
      const DevNode* nd = s.nodes + cur;
      const uint4 head = __ldg(reinterpret_cast<const uint4*>(nd));
      const uint64_t occ = ((uint64_t)head.y << 32) | head.x;
      const uint32_t meta = head.z;
      const uint32_t kind = meta & 3u;
      bool backtrack = kind == kKindUniform;
      if (kLod && s.mips) {
        // mip_level < (origin - round(p / (2 mip_level)) * 2 mip_level).length() / viewing_distance
        const float m2 = mip_level * 2.0f;
        const float ax = ox - roundf(r.px / m2) * m2, ay = oy - roundf(r.py / m2) * m2, az = oz - roundf(r.pz / m2) * m2;
        if (mip_level < sqrtf((ax * ax + ay * ay) + az * az) / viewing_distance) {
          const uint32_t mk = (meta >> 24) & 3u;
          if (mk == 3u) {  // node_mips[key] past the vector: the reference panics
            h.status = 3;
            return;
          }
          const uint32_t rc = probe_brick<kCount, kFast>(s, r, mk, head.w, cb, h, work);
          if (rc) {
            h.status = rc;
            h.node = cur;
            h.octant = 8;  // the node's MIP brick
            return;
          }
        }
      }
      if (target != kOob) {
        if (kind == kKindUniform) {
          const uint32_t rc = probe_brick<kCount, kFast>(s, r, (meta >> 8) & 3u, __ldg(&nd->slot[0]), cb, h, work);
          if (rc) {
            h.status = rc;
            h.node = cur;
            h.octant = 0;
            return;
          }
          backtrack = true;
        } else if (kind == kKindLeaf) {
          const uint32_t rc = probe_brick<kCount, kFast>(s, r, (meta >> (8 + 2 * target)) & 3u,
                                                         __ldg(&nd->slot[target]), child_bounds(cb, target), h, work);
          if (rc) {
            h.status = rc;
            h.node = cur;
            h.octant = target;
            return;
          }
        }
      }
      // bitmap position of the point in the node; floor(clamp(v, 1e-5, 4 - 1e-5)) as usize equals
      // min(trunc_to_u32(v), 3) for every v including NaN and +-inf, so the clamped values
      // themselves are only formed when ADVANCE needs them
      const float rx = (r.px - cb.x) * 4.0f * cb.inv;
      const float ry = (r.py - cb.y) * 4.0f * cb.inv;
      const float rz = (r.pz - cb.z) * 4.0f * cb.inv;
      uint32_t flat = min(__float2uint_rz(rx), 3u) + 4u * min(__float2uint_rz(ry), 3u) +
                      16u * min(__float2uint_rz(rz), 3u);
      if (backtrack || target == kOob || occ == 0 || (occ & rtn[flat * 8u]) == 0) {
        // POP (:445-473)
        s0 = s1;
        s1 = s2;
        s2 = s3;
        --count;
        if (kLod) mip_level += 1.0f;
        if (count > 0) {
          cur = s0;
          // min - fmod(min, 2s): bounds minima are non-negative multiples of s and 2s is a power of
          // two, so fmod(x, 2s) == x - floor(x / 2s) * 2s exactly and the parent minimum is floor(x / 2s) * 2s
          const float h2 = cb.s * 0.5f, s2x = cb.s * 2.0f, i2x = cb.inv * 0.5f;
          const float pmx = floorf(cb.x * i2x) * s2x, pmy = floorf(cb.y * i2x) * s2x, pmz = floorf(cb.z * i2x) * s2x;
          const uint32_t ho = hash_region((cb.x + h2) - pmx, (cb.y + h2) - pmy, (cb.z + h2) - pmz, cb.s);
          float sx, sy, sz;
          dda_step<kFast>(r, cb, sx, sy, sz);
          target = step_octant(ho, sx, sy, sz);
          cb = Bounds{pmx, pmy, pmz, s2x, i2x};
        }
        continue;
      }
      Bounds tb = child_bounds(cb, target);
      uint32_t ck = kind == kKindInternal ? __ldg(&nd->slot[target]) : kInvalidChild;
      if (kCount) h.creads++;
      if (ck != kInvalidChild && (occ & L.octant[target]) != 0) {
        // PUSH (:484-492)
        cur = ck;
        cb = tb;
        target = hash_region(r.px - tb.x, r.py - tb.y, r.pz - tb.z, tb.s * 0.5f);
        s3 = s2;
        s2 = s1;
        s1 = s0;
        s0 = ck;
        count = count < 4 ? count + 1 : 4;
        if (kLod) mip_level -= 1.0f;
      } else {
        // ADVANCE (:494-544)
        float bx = rclamp(rx, kTol, 4.0f - kTol);
        float by = rclamp(ry, kTol, 4.0f - kTol);
        float bz = rclamp(rz, kTol, 4.0f - kTol);
        for (;;) {
          if (++work > kWorkCap) {
            h.status = 2;
            return;
          }
          float sx, sy, sz;
          dda_step<kFast>(r, tb, sx, sy, sz);
          target = step_octant(target, sx, sy, sz);
          if (target != kOob) {
            tb = child_bounds(cb, target);
            ck = kind == kKindInternal ? __ldg(&nd->slot[target]) : kInvalidChild;
            if (kCount) h.creads++;
            bx = bx + sx * 4.0f * cb.inv;
            by = by + sy * 4.0f * cb.inv;
            bz = bz + sz * 4.0f * cb.inv;
            if (!bitmap_index(bx, by, bz, flat)) {
              h.status = 3;
              return;
            }
          }
          if (target == kOob) break;
          if (ck != kInvalidChild && (occ & L.octant[target]) != 0 && (rtn[flat * 8u] & occ) != 0) break;
          if (kind == kKindLeaf && ((meta >> (8 + 2 * target)) & 3u) != kBkEmpty) break;
        }
      }
    }
    // restart from the root with a 0.1 nudge (:548-562)
    r.px = r.px + dx * 0.1f;
    r.py = r.py + dy * 0.1f;
    r.pz = r.pz + dz * 0.1f;
    target = (r.px < S && r.py < S && r.pz < S && r.px > 0.0f && r.py > 0.0f && r.pz > 0.0f)
                 ? hash_region(r.px, r.py, r.pz, S * 0.5f)
                 : kOob;
  }
}


// True when no restart visit from the next one on can read a MIP: the visit after j nudges has
// level L + j - 1 (L > 0, each visit POPs) and point p_j with |o - p_j| <= |o - p| + j g, g = |c| plus
// the rounding of one nudge, and the grid point it is rounded to lies within sqrt(3) (level +
// 2^-22 |p|) of p_j, so the condition is false while (L + j - 1)(vd - sqrt(3)) exceeds
// |o - p| + j g + sqrt(3) 2^-21 S, padded by 2^-20 for the f32 evaluation.  Both sides grow
// linearly in j, so the first visit and the slopes decide.  Evaluated in f64.
static __device__ __noinline__ bool lod_runs_clear(float ox, float oy, float oz, float px, float py, float pz, float cx,
                                            float cy, float cz, float level, float viewing_distance, float S) {
  if (!(level > 0.0f) || !(viewing_distance > 0.0f)) return false;
  const double pad = 1.0 + 0x1p-20, r3 = 1.7320508075688772 * pad;
  const double vd = (double)viewing_distance, L = (double)level;
  const double dx = (double)ox - px, dy = (double)oy - py, dz = (double)oz - pz;
  const double d0 = sqrt(dx * dx + dy * dy + dz * dz) * pad;
  const double g = sqrt((double)cx * cx + (double)cy * cy + (double)cz * cz) * pad + 0x1p-22 * S * r3;
  const double slack = r3 * 0x1p-21 * S + 1e-6;
  if ((vd - r3) < g * pad) return false;                  // the right-hand side could catch up
  return L * (vd - r3) >= (d0 + g + slack) * pad;         // the first visit (j = 1)
}


// restart_cells_run out of line: it runs a few times per ray at most, and inlined it would add to
// the register allocation of the whole traversal loop.
struct RestartRun {
  float x, y, z;
  uint32_t k;
};
static __device__ __noinline__ RestartRun restart_exit(float x, float y, float z, float cx, float cy, float cz,
                                                       float S, uint32_t n_max) {
  RestartRun o;
  o.k = restart_exit_run(x, y, z, cx, cy, cz, S, n_max);
  o.x = x;
  o.y = y;
  o.z = z;
  return o;
}
static __device__ __noinline__ RestartRun restart_run(float x, float y, float z, float cx, float cy, float cz, uint32_t flat,
                                                      float w, uint32_t n_max) {
  RestartRun o;
  o.k = restart_cells_run(x, y, z, cx, cy, cz, flat, w, n_max);
  o.x = x;
  o.y = y;
  o.z = z;
  return o;
}

// ---------------------------------------------------------------------------
// Fast form of the same cast for directions without NaN (signum is +-1 on every
// axis).  It performs the reference's operations on every value it keeps; only
// the bookkeeping around them is cheaper, each step justified where it appears:
//  * a DDA step returns the 3-bit set of axes that advance (octant bit layout:
//    x = 1, z = 2, y = 4) instead of a float step vector whose entries are
//    +-1 or 0, so step_octant's LUT becomes `o ^ move`, out of bounds when a
//    moved axis is already on the far side in the ray's direction;
//  * `x + step * k` with step in {+-1, +0} is `moved ? x + sign * k : x`;
//  * POP's parent octant: a node minimum is either the parent minimum or the
//    parent minimum + size, so hash_region(center - parent_min, size) tests
//    `min != parent_min` per axis.
struct FastRay {
  float dx, dy, dz;  // direction
  float fx, fy, fz;  // dda scale factors
  float px, py, pz;  // current point
  uint32_t pos;      // axes with a positive direction, octant bit layout
};

// dda_step_to_next_sibling (raytracing_on_cpu.rs:124-152), returning the moved axes
__device__ __forceinline__ uint32_t dda_move(FastRay& r, float bx, float by, float bz, float bs) {
  const float ex = r.px - bx, ey = r.py - by, ez = r.pz - bz;
  const float nx = (r.pos & 1u) ? bs - ex : ex;
  const float ny = (r.pos & 4u) ? bs - ey : ey;
  const float nz = (r.pos & 2u) ? bs - ez : ez;
  const float ax = fabsf(nx * r.fx), ay = fabsf(ny * r.fy), az = fabsf(nz * r.fz);
  const float m = fminf(fminf(ax, ay), az);
  r.px = r.px + r.dx * m;
  r.py = r.py + r.dy * m;
  r.pz = r.pz + r.dz * m;
  return (m == ax ? 1u : 0u) | (m == az ? 2u : 0u) | (m == ay ? 4u : 0u);
}

// step_octant for a step along the moved axes in the ray's direction
__device__ __forceinline__ uint32_t step_fast(uint32_t o, uint32_t move, uint32_t pos) {
  return (((o ^ pos) ^ 7u) & move) ? kOob : (o ^ move);
}

// probe_brick / traverse_brick (raytracing_on_cpu.rs:156-312), fast form
template <bool kCount>
__device__ __forceinline__ uint32_t probe_brick_fast(const SceneView& s, FastRay& r, uint32_t bk, uint32_t value,
                                                     const Bounds& bb, HitRecord& h, uint32_t& work) {
  if (bk == kBkEmpty) return 0;
  if (bk == kBkSolid) {
    h.pix = value;
    h.voxel = 0xFFFFFFFFu;
    h.px = r.px;
    h.py = r.py;
    h.pz = r.pz;
    impact_normal(bb, r.px, r.py, r.pz, h.nx, h.ny, h.nz);
    return 1;
  }
  const int D = (int)s.dim;
  const float Df = (float)s.dim;
  int cx = min(max(as_i32((r.px - bb.x) * Df * bb.inv), 0), D - 1);
  int cy = min(max(as_i32((r.py - bb.y) * Df * bb.inv), 0), D - 1);
  int cz = min(max(as_i32((r.pz - bb.z) * Df * bb.inv), 0), D - 1);
  int flat = cx + cy * D + cz * D * D;
  const int D3 = D * D * D;
  const float unit = bb.s * s.inv_dim;
  float ux = bb.x + (float)cx * unit, uy = bb.y + (float)cy * unit, uz = bb.z + (float)cz * unit;
  const float gux = (r.pos & 1u) ? unit : -unit, guy = (r.pos & 4u) ? unit : -unit, guz = (r.pos & 2u) ? unit : -unit;
  const int ix = (r.pos & 1u) ? 1 : -1, iy = (r.pos & 4u) ? 1 : -1, iz = (r.pos & 2u) ? 1 : -1;
  const int fdx = ix, fdy = iy * D, fdz = iz * D * D;
  const uint32_t* bits = s.vbits + (size_t)value * s.vwords;
  uint32_t move = 0;
  for (;;) {
    if ((unsigned)cx >= (unsigned)D || (unsigned)cy >= (unsigned)D || (unsigned)cz >= (unsigned)D) return 0;
    // flat == cx + cy D + cz D^2 (moved with the index), inside the brick like the index
    flat += ((move & 1u) ? fdx : 0) + ((move & 4u) ? fdy : 0) + ((move & 2u) ? fdz : 0);
    if (kCount) h.vreads++;
    if (++work > kWorkCap) return 2;
    if ((__ldg(bits + (flat >> 5)) >> (flat & 31)) & 1u) {
      const Bounds hb{bb.x + (float)cx * bb.s * s.inv_dim, bb.y + (float)cy * bb.s * s.inv_dim,
                      bb.z + (float)cz * bb.s * s.inv_dim, unit, bb.inv * Df};
      h.pix = __ldg(s.voxels + (size_t)value * (size_t)D3 + (size_t)flat);
      h.voxel = (uint32_t)flat;
      h.px = r.px;
      h.py = r.py;
      h.pz = r.pz;
      impact_normal(hb, r.px, r.py, r.pz, h.nx, h.ny, h.nz);
      return 1;
    }
    move = dda_move(r, ux, uy, uz, unit);
    if (move & 1u) {
      ux = ux + gux;
      cx += ix;
    }
    if (move & 4u) {
      uy = uy + guy;
      cy += iy;
    }
    if (move & 2u) {
      uz = uz + guz;
      cz += iz;
    }
  }
}

// probe of a node's MIP brick (kind in meta[25:24]; kind 3: no node_mips entry, where the reference panics)
template <bool kCount>
__device__ __forceinline__ uint32_t probe_mip(const SceneView& s, FastRay& r, uint32_t meta, uint32_t value,
                                              const Bounds& b, HitRecord& h, uint32_t& work) {
  const uint32_t mk = (meta >> 24) & 3u;
  if (mk == 3u) return 3;
  return probe_brick_fast<kCount>(s, r, mk, value, b, h, work);
}

// kLod: get_by_ray_at_lod with MIP maps (s.mips): the MIP reads of the literal form, and restart
// runs taken in closed form only where lod_runs_clear proves that none of their visits reads a MIP.
// The record of a ray that hits nothing.
__device__ __forceinline__ void miss_record(HitRecord& h) {
  h.status = 0;
  h.octant = 0;
  h.node = 0;
  h.voxel = 0xFFFFFFFFu;
  h.pix = 0;
  h.px = h.py = h.pz = h.nx = h.ny = h.nz = 0.0f;
  h.visits = h.creads = h.vreads = h.runs = 0;
}

// The fast form's way into the octree (get_by_ray's root intersection, :330-348): false when the ray
// misses the root box; else the point where it enters (its origin when inside) and that point's
// octant of the root.
__device__ __forceinline__ bool fast_entry(const SceneView& s, float ox, float oy, float oz, float dx, float dy,
                                           float dz, float& px, float& py, float& pz, uint32_t& target) {
  const float S = s.size;
  // A ray whose origin lies outside the octree on some axis and that moves further away on it has
  // both of that axis' slab distances negative, so tmax < 0 and the slab test below rejects it.
  // The quotients are strictly negative when the origin is finite, at least 2^-100 below 0 (or
  // above S) and the direction component at most 2^20 in size: no quotient rounds to -0.
  {
    const float lo = -0x1p-100f, big = 0x1p20f;
    const bool fin = isfinite(ox) && isfinite(oy) && isfinite(oz) && fabsf(dx) <= big && fabsf(dy) <= big &&
                     fabsf(dz) <= big;
    if (fin && ((ox < lo && dx < 0.0f) || (ox > S && dx > 0.0f) || (oy < lo && dy < 0.0f) || (oy > S && dy > 0.0f) ||
                (oz < lo && dz < 0.0f) || (oz > S && dz > 0.0f)))
      return false;
  }
  const float t1 = (0.0f - ox) / dx, t2 = ((0.0f + S) - ox) / dx;
  const float t3 = (0.0f - oy) / dy, t4 = ((0.0f + S) - oy) / dy;
  const float t5 = (0.0f - oz) / dz, t6 = ((0.0f + S) - oz) / dz;
  const float tmin = rmax(rmax(rmin(t1, t2), rmin(t3, t4)), rmin(t5, t6));
  const float tmax = rmin(rmin(rmax(t1, t2), rmax(t3, t4)), rmax(t5, t6));
  if (tmax < 0.0f || tmin > tmax) return false;
  const float t = tmin < 0.0f ? 0.0f : tmin;
  px = ox + dx * t;
  py = oy + dy * t;
  pz = oz + dz * t;
  target = hash_region(px - 0.0f, py - 0.0f, pz - 0.0f, S * 0.5f);
  return true;
}

// The fast form's traversal of a ray that entered the root at (px, py, pz), in its octant `target`.
// kStage: the first stg_n records of the scene's top table are staged at `stg` (shared memory); a
// node key with kStagedBit set names one of them.  Only Internal nodes are staged, so the key of a
// node that holds a hit never carries the bit.
template <bool kCount, bool kLod = false, bool kStage = false>
__device__ void cast_ray_fast_from(const SceneView& s, const SharedLuts& L, float ox, float oy, float oz, float dx,
                                   float dy, float dz, float px, float py, float pz, uint32_t target, HitRecord& h,
                                   float viewing_distance = 0.0f, const DevNode* stg = nullptr, uint32_t stg_n = 0) {
  static_assert(!(kStage && kLod), "a MIP hit reports its node's key: the LOD cast reads no staged copy");
  miss_record(h);
  FastRay r;
  r.dx = dx;
  r.dy = dy;
  r.dz = dz;
  // signum(d) > 0 <=> d > 0 or d == +0
  r.pos = (rsignum(dx) > 0.0f ? 1u : 0u) | (rsignum(dz) > 0.0f ? 2u : 0u) | (rsignum(dy) > 0.0f ? 4u : 0u);
  const float g4x = (r.pos & 1u) ? 4.0f : -4.0f, g4y = (r.pos & 4u) ? 4.0f : -4.0f, g4z = (r.pos & 2u) ? 4.0f : -4.0f;
  const uint32_t dir = hash_region(1.0f + dx, 1.0f + dy, 1.0f + dz, 1.0f);
  const uint64_t* rtn = L.ray_to_node + dir;
  const float S = s.size;
  Bounds cb{0.0f, 0.0f, 0.0f, S, s.inv_size};
  r.px = px;
  r.py = py;
  r.pz = pz;
  {  // get_dda_scale_factors (:99-112), a function of the direction only, so formed after the
     // root's slab test has let the ray in; powf(q, 2.) == q * q
    const float a = dz / dx, b = dy / dx, c = dx / dy, d = dz / dy, e = dx / dz, f = dy / dz;
    r.fx = sqrtf((1.0f + a * a) + b * b);
    r.fy = sqrtf((c * c + 1.0f) + d * d);
    r.fz = sqrtf((e * e + 1.0f) + f * f);
  }
  uint32_t work = 0;
  float mip_level = s.mip_top;  // (:350) kept across restarts
  const bool lod = kLod && s.mips;
  const uint32_t root = (kStage && stg_n) ? kStagedBit : 0u;
  while (target != kOob) {
    uint32_t cur = root;
    cb = Bounds{0.0f, 0.0f, 0.0f, S, s.inv_size};
    uint32_t s0 = root, s1 = 0, s2 = 0, s3 = 0, count = 1;
    uint32_t oct = 0;  // octant of each stack entry in its parent, newest in the low 3 bits
    while (count > 0) {
      if (++work > kWorkCap) {
        h.status = 2;
        return;
      }
      if (kCount) h.visits++;
      const bool staged = kStage && (cur & kStagedBit) != 0u;
      const DevNode* nd = s.nodes + cur;
      const DevNode* sn = kStage ? stg + (cur & ~kStagedBit) : nd;
      const uint4 head = staged ? *reinterpret_cast<const uint4*>(sn) : __ldg(reinterpret_cast<const uint4*>(nd));
      const uint64_t occ = ((uint64_t)head.y << 32) | head.x;
      const uint32_t meta = head.z;
      const uint32_t kind = meta & 3u;
      const bool uniform = kind == kKindUniform;
      const bool backtrack = uniform;  // a UniformLeaf is always left after its probe
      if (lod && lod_reads_mip(ox, oy, oz, r.px, r.py, r.pz, mip_level, viewing_distance)) {
        const uint32_t rc = probe_mip<kCount>(s, r, meta, head.w, cb, h, work);
        if (rc) {
          h.status = rc;
          h.node = cur;
          h.octant = 8;  // the node's MIP brick
          return;
        }
      }
      if (target != kOob && (uniform || kind == kKindLeaf)) {
        // probe the UniformLeaf's brick over the node bounds, or the Leaf's brick under target_octant
        const uint32_t slot = uniform ? 0u : target;
        const uint32_t bk = (meta >> (8 + 2 * slot)) & 3u;
        if (bk != kBkEmpty) {
          const uint32_t rc = probe_brick_fast<kCount>(s, r, bk, __ldg(&nd->slot[slot]),
                                                       uniform ? cb : child_bounds(cb, target), h, work);
          if (rc) {
            h.status = rc;
            h.node = cur;
            h.octant = slot;
            return;
          }
        }
      }
      // (x * 4) / size == x * (4 / size): both only rescale x by powers of two
      const float q4 = cb.inv * 4.0f;
      const float rx = (r.px - cb.x) * q4;
      const float ry = (r.py - cb.y) * q4;
      const float rz = (r.pz - cb.z) * q4;
      uint32_t flat = min(__float2uint_rz(rx), 3u) + 4u * min(__float2uint_rz(ry), 3u) +
                      16u * min(__float2uint_rz(rz), 3u);
      if (backtrack || target == kOob || occ == 0 || (occ & rtn[flat * 8u]) == 0) {
        // POP.  The popped node was pushed as child `ho` of the new top, so its bounds are
        // child_bounds_for(parent, ho): the reference's parent minimum min - fmod(min, 2 size) is
        // min - offset(ho) * size and hash_region(center - parent_min, size) is ho (both exact).
        const uint32_t ho = oct & 7u;
        s0 = s1;
        s1 = s2;
        s2 = s3;
        oct >>= 3;
        --count;
        if (kLod) mip_level += 1.0f;
        if (count > 0) {
          cur = s0;
          const float pmx = (ho & 1u) ? cb.x - cb.s : cb.x;
          const float pmy = (ho & 4u) ? cb.y - cb.s : cb.y;
          const float pmz = (ho & 2u) ? cb.z - cb.s : cb.z;
          const uint32_t move = dda_move(r, cb.x, cb.y, cb.z, cb.s);
          target = step_fast(ho, move, r.pos);
          cb = Bounds{pmx, pmy, pmz, cb.s * 2.0f, cb.inv * 0.5f};
        }
        continue;
      }
      Bounds tb = child_bounds(cb, target);
      if (kCount) h.creads++;
      // the child key is read only where the octant is occupied: an empty octant neither pushes nor
      // stops an ADVANCE, whatever its key
      uint32_t ck = kInvalidChild;
      if (kind == kKindInternal && (occ & L.octant[target]) != 0) ck = staged ? sn->slot[target] : __ldg(&nd->slot[target]);
      if (ck != kInvalidChild) {
        // PUSH (the child's octant in its parent rides along: 3 bits per stack entry); a staged
        // node's staged child is entered through its copy
        if (staged) {
          const uint32_t si = sn->stage[target];
          if (si < stg_n) ck = kStagedBit | si;
        }
        oct = ((oct << 3) | target) & 0xFFFu;
        cur = ck;
        cb = tb;
        target = hash_region(r.px - tb.x, r.py - tb.y, r.pz - tb.z, tb.s * 0.5f);
        s3 = s2;
        s2 = s1;
        s1 = s0;
        s0 = ck;
        count = count < 4 ? count + 1 : 4;
        if (kLod) mip_level -= 1.0f;
      } else {
        // ADVANCE
        float bx = rclamp(rx, kTol, 4.0f - kTol);
        float by = rclamp(ry, kTol, 4.0f - kTol);
        float bz = rclamp(rz, kTol, 4.0f - kTol);
        const float dbx = (g4x > 0.0f) ? q4 : -q4, dby = (g4y > 0.0f) ? q4 : -q4, dbz = (g4z > 0.0f) ? q4 : -q4;
        for (;;) {
          if (++work > kWorkCap) {
            h.status = 2;
            return;
          }
          const uint32_t move = dda_move(r, tb.x, tb.y, tb.z, tb.s);
          target = step_fast(target, move, r.pos);
          if (target == kOob) break;
          tb = child_bounds(cb, target);
          if (kCount) h.creads++;
          if (move & 1u) bx = bx + dbx;
          if (move & 4u) by = by + dby;
          if (move & 2u) bz = bz + dbz;
          // floor(bp) as usize: the reference panics at 4 and above
          const uint32_t ux = __float2uint_rz(bx), uy = __float2uint_rz(by), uz = __float2uint_rz(bz);
          if (ux >= 4u || uy >= 4u || uz >= 4u) {
            h.status = 3;
            return;
          }
          flat = ux + 4u * uy + 16u * uz;
          if (kind == kKindInternal && (occ & L.octant[target]) != 0 && (rtn[flat * 8u] & occ) != 0) {
            ck = staged ? sn->slot[target] : __ldg(&nd->slot[target]);
            if (ck != kInvalidChild) break;
          }
          if (kind == kKindLeaf && ((meta >> (8 + 2 * target)) & 3u) != kBkEmpty) break;
        }
      }
    }
    const float c01x = dx * 0.1f, c01y = dy * 0.1f, c01z = dz * 0.1f;  // the same product on every restart
    r.px = r.px + c01x;
    r.py = r.py + c01y;
    r.pz = r.pz + c01z;
    // Restarts whose root visit fails its occupancy test (an Internal or empty root, whose visit
    // neither probes nor pushes) repeat visit, POP and nudge until the point changes root bitmap
    // cell; each such run is taken in closed form, counting its visits.
    const uint4 root = __ldg(reinterpret_cast<const uint4*>(s.nodes));
    const uint64_t occ_root = ((uint64_t)root.y << 32) | root.x;
    const bool root_runs = (root.z & 3u) == kKindInternal || (root.z & 3u) == kKindNothing;
    const float q4r = s.inv_size * 4.0f;
    while (root_runs && r.px < S && r.py < S && r.pz < S && r.px > 0.0f && r.py > 0.0f && r.pz > 0.0f) {
      // a root visit that reads the root's MIP (which may move the point before the occupancy
      // test) is left to the traversal loop
      if (lod && lod_reads_mip(ox, oy, oz, r.px, r.py, r.pz, mip_level, viewing_distance)) break;
      const float rx = (r.px - 0.0f) * q4r, ry = (r.py - 0.0f) * q4r, rz = (r.pz - 0.0f) * q4r;
      const uint32_t flat = min(__float2uint_rz(rx), 3u) + 4u * min(__float2uint_rz(ry), 3u) +
                            16u * min(__float2uint_rz(rz), 3u);
      if (occ_root != 0 && (occ_root & rtn[flat * 8u]) != 0) break;
      if (++work > kWorkCap) {
        h.status = 2;
        return;
      }
      if (kCount) h.visits++;
      if (kLod) mip_level += 1.0f;  // the root's POP
      if (lod && !lod_runs_clear(ox, oy, oz, r.px, r.py, r.pz, c01x, c01y, c01z, mip_level, viewing_distance, S)) {
        // a later restart visit may read the root's MIP: one restart at a time
        r.px = r.px + c01x;
        r.py = r.py + c01y;
        r.pz = r.pz + c01z;
        continue;
      }
      // When every axis moves the way the direction octant of the LUT says (only a negative
      // component so small that 1 + d rounds to 1 breaks this), every later cell lies inside this
      // cell's box towards the far corner, whose occupancy bits are empty: all later root tests fail
      // and the ray leaves the octree without a hit.  Without counters only the work cap matters:
      // an axis with |c| >= 2^-22 S advances by at least 3|c|/4 per restart (|c| >= 2 ulp), so at
      // most S / (|c| / 2) + 2 restarts remain.  The counted cast takes the run to the exit exactly.
      if (!((dx < 0.0f && 1.0f + dx >= 1.0f) || (dy < 0.0f && 1.0f + dy >= 1.0f) || (dz < 0.0f && 1.0f + dz >= 1.0f))) {
        if (!kCount) {
          const float cmax = fmaxf(fmaxf(fabsf(c01x), fabsf(c01y)), fabsf(c01z));
          if (cmax >= S * 0x1p-22f && (float)work + S / (0.5f * cmax) + 2.0f < (float)kWorkCap) return;
        }
        const RestartRun run = restart_exit(r.px, r.py, r.pz, c01x, c01y, c01z, S, kWorkCap - work + 2u);
        if (run.k == kRunNever) {
          h.status = 2;
          return;
        }
        if (kCount) {
          h.visits += run.k - 1u;
          h.runs += run.k - 1u;
        }
        return;
      }
      // the visits before the next cell change fail alike; the cap holds if they fit in it
      const RestartRun run = restart_run(r.px, r.py, r.pz, c01x, c01y, c01z, flat, S * 0.25f, kWorkCap - work + 2u);
      const uint32_t k = run.k;
      r.px = run.x;
      r.py = run.y;
      r.pz = run.z;
      if (k == kRunNever) {
        h.status = 2;
        return;
      }
      work += k - 1u;
      if (kLod) mip_level += (float)(k - 1u);  // the skipped visits' POPs
      if (kCount) {
        h.visits += k - 1u;
        h.runs += k - 1u;
      }
    }
    target = (r.px < S && r.py < S && r.pz < S && r.px > 0.0f && r.py > 0.0f && r.pz > 0.0f)
                 ? hash_region(r.px, r.py, r.pz, S * 0.5f)
                 : kOob;
  }
}

template <bool kCount, bool kLod = false>
__device__ __forceinline__ void cast_ray_fast(const SceneView& s, const SharedLuts& L, float ox, float oy, float oz,
                                              float dx, float dy, float dz, HitRecord& h,
                                              float viewing_distance = 0.0f) {
  float px, py, pz;
  uint32_t target;
  if (fast_entry(s, ox, oy, oz, dx, dy, dz, px, py, pz, target))
    cast_ray_fast_from<kCount, kLod>(s, L, ox, oy, oz, dx, dy, dz, px, py, pz, target, h, viewing_distance);
  else
    miss_record(h);
}

// Rays whose direction holds a NaN take the literal form, out of line so that
// it does not add to the fast path's register allocation.
template <bool kCount>
__device__ __noinline__ void cast_ray_literal(const SceneView& s, const SharedLuts& L, float ox, float oy, float oz,
                                              float dx, float dy, float dz, HitRecord& h) {
  cast_ray<kCount, false>(s, L, ox, oy, oz, dx, dy, dz, h);
}

// get_by_ray_at_lod for rays whose direction holds a NaN, out of line like cast_ray_literal.
template <bool kCount>
__device__ __noinline__ void cast_ray_literal_lod(const SceneView& s, const SharedLuts& L, float ox, float oy, float oz,
                                                  float dx, float dy, float dz, HitRecord& h, float viewing_distance) {
  cast_ray<kCount, false, true>(s, L, ox, oy, oz, dx, dy, dz, h, viewing_distance);
}

// cast_one for a ray whose way in is known: `fast` with its fast_entry (px, py, pz, target), else the
// literal form (a NaN in the direction, or literal mode).  kStage: the fast form reads the first stg_n
// top-table records from their copy at `stg` (shared memory).
template <bool kCount, bool kLod = false, bool kStage = false>
__device__ __forceinline__ void cast_entered(const SceneView& s, const SharedLuts& L, float ox, float oy, float oz,
                                             float dx, float dy, float dz, bool fast, float px, float py, float pz,
                                             uint32_t target, HitRecord& h, float viewing_distance = 0.0f,
                                             const DevNode* stg = nullptr, uint32_t stg_n = 0) {
  if (fast)
    cast_ray_fast_from<kCount, kLod, kStage>(s, L, ox, oy, oz, dx, dy, dz, px, py, pz, target, h, viewing_distance,
                                             stg, stg_n);
  else if (kLod)
    cast_ray_literal_lod<kCount>(s, L, ox, oy, oz, dx, dy, dz, h, viewing_distance);
  else
    cast_ray_literal<kCount>(s, L, ox, oy, oz, dx, dy, dz, h);
}

// One ray: the exact fast form when the direction holds no NaN, the literal form otherwise; kLod
// casts get_by_ray_at_lod at the viewing distance.
template <bool kCount, bool kLod = false>
__device__ __forceinline__ void cast_one(const SceneView& s, const SharedLuts& L, float ox, float oy, float oz,
                                         float dx, float dy, float dz, HitRecord& h, float viewing_distance = 0.0f) {
  if (!s.literal && !isnan(dx) && !isnan(dy) && !isnan(dz))
    cast_ray_fast<kCount, kLod>(s, L, ox, oy, oz, dx, dy, dz, h, viewing_distance);
  else if (kLod)
    cast_ray_literal_lod<kCount>(s, L, ox, oy, oz, dx, dy, dz, h, viewing_distance);
  else
    cast_ray_literal<kCount>(s, L, ox, oy, oz, dx, dy, dz, h);
}

struct HitsView {
  uint8_t *status, *octant, *kind;
  uint32_t *node, *voxel, *pix, *albedo, *user;
  float *px, *py, *pz, *nx, *ny, *nz;
  uint32_t *visits, *creads, *vreads, *runs;
};

__host__ __device__ inline HitsView hits_view_of(const svo_hits& h) {
  HitsView v;
  v.status = h.status;
  v.octant = h.brick_octant;
  v.kind = h.entry_kind;
  v.node = h.node_key;
  v.voxel = h.voxel_index;
  v.pix = h.pix;
  v.albedo = h.albedo;
  v.user = h.user;
  v.px = h.px;
  v.py = h.py;
  v.pz = h.pz;
  v.nx = h.nx;
  v.ny = h.ny;
  v.nz = h.nz;
  v.visits = h.node_visits;
  v.creads = h.child_reads;
  v.vreads = h.voxel_reads;
  v.runs = h.run_visits;
  return v;
}

// pix_get_ref (src/octree/node.rs:381-419): the hit's entry kind and payload from its palette
// indices; an index past a palette panics in the reference (status 3).
__device__ __forceinline__ void resolve_entry(const SceneView& s, HitRecord& h, uint32_t& kind, uint32_t& albedo,
                                              uint32_t& user) {
  kind = albedo = user = 0;
  if (h.status != 1) return;
  const uint32_t c = h.pix & 0xFFFFu, d = h.pix >> 16;
  if (c < 0xFFFFu) {
    if (c >= s.n_colors) {
      h.status = 3;
    } else {
      kind |= 1u;
      albedo = __ldg(s.colors + c);
    }
  }
  if (d != 0xFFFFu) {
    if (d >= s.n_datas) {
      h.status = 3;
    } else {
      kind |= 2u;
      user = __ldg(s.datas + d);
    }
  }
}

__device__ __forceinline__ void write_hit(const SceneView& s, const HitsView& o, uint64_t i, HitRecord& h) {
  uint32_t kind, albedo, user;
  resolve_entry(s, h, kind, albedo, user);
  if (h.status != 1) {
    h.octant = h.node = h.pix = 0;
    h.voxel = 0xFFFFFFFFu;
    h.px = h.py = h.pz = h.nx = h.ny = h.nz = 0.0f;
    kind = albedo = user = 0;
  }
  if (h.status >= 2) h.visits = h.creads = h.vreads = h.runs = 0;  // no defined counts past a cap or panic
  if (o.status) o.status[i] = (uint8_t)h.status;
  if (o.octant) o.octant[i] = (uint8_t)h.octant;
  if (o.kind) o.kind[i] = (uint8_t)kind;
  if (o.node) o.node[i] = h.node;
  if (o.voxel) o.voxel[i] = h.voxel;
  if (o.pix) o.pix[i] = h.pix;
  if (o.albedo) o.albedo[i] = albedo;
  if (o.user) o.user[i] = user;
  if (o.px) o.px[i] = h.px;
  if (o.py) o.py[i] = h.py;
  if (o.pz) o.pz[i] = h.pz;
  if (o.nx) o.nx[i] = h.nx;
  if (o.ny) o.ny[i] = h.ny;
  if (o.nz) o.nz[i] = h.nz;
}

__device__ __forceinline__ void write_counters(const HitsView& o, uint64_t i, const HitRecord& h) {
  if (o.visits) o.visits[i] = h.visits;
  if (o.creads) o.creads[i] = h.creads;
  if (o.vreads) o.vreads[i] = h.vreads;
  if (o.runs) o.runs[i] = h.runs;
}


struct RaysView {
  const float *ox, *oy, *oz, *dx, *dy, *dz;
};

// Lets `kernel` take `bytes` of dynamic shared memory: with its static shared memory a block may pass
// 48 KB only after the opt-in, which is raised when a launch asks for more than allowed so far (never
// lowered).  Host-side attributes only: nothing is enqueued.
template <class K>
inline cudaError_t allow_dynamic_smem(K kernel, size_t bytes) {
  if (bytes == 0) return cudaSuccess;
  cudaFuncAttributes a{};
  cudaError_t e = cudaFuncGetAttributes(&a, (const void*)kernel);
  if (e != cudaSuccess) return e;
  if ((size_t)a.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
  return cudaFuncSetAttribute((const void*)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Copies `n` top-table records from `src` (global) to `dst` (shared memory) with the block's threads,
// 16 bytes per load.  The caller synchronises the block before the copy is read.
__device__ __forceinline__ void stage_records(DevNode* dst, const DevNode* src, uint32_t n) {
  const uint4* a = reinterpret_cast<const uint4*>(src);
  uint4* b = reinterpret_cast<uint4*>(dst);
  for (uint32_t i = threadIdx.x; i < n * (uint32_t)(sizeof(DevNode) / 16); i += blockDim.x) b[i] = __ldg(a + i);
}

}  // namespace svo
