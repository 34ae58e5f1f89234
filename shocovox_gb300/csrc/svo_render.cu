// svo_render.cu -- fused viewport render: the per-pixel loop of examples/cpu_render.rs:77-138
// (viewport ray, Octree::get_by_ray, diffuse shading) as one kernel writing RGBA8.
//
// Rays are generated where they are cast, so no ray or hit buffer touches memory: a pixel costs
// its 4 output bytes plus the scene reads of its traversal.  A warp renders 8 x 4 pixel tiles, so
// its rays are neighbours in both image directions and take similar paths through the octree;
// warps claim tiles from the scene's work counter for the stream (svo_queue.h), so a warp that
// drew sky tiles goes on to take more.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

#include "svo_cast.cuh"
#include "svo_queue.h"
#include "svo_trace.h"

namespace svo {
namespace {

// The frame of one viewport, computed on the host with the example's f32 operations.
struct ViewFrame {
  float ox, oy, oz;  // viewport_ray.origin
  float rx, ry, rz;  // viewport_right_direction
  float ux, uy, uz;  // viewport_up_direction
  float bx, by, bz;  // viewport_bottom_left
  float pw, ph;      // pixel_width, pixel_height
  float lx, ly, lz;  // diffuse_light_normal
  uint32_t background;
};

// The frames of one launch (kernel parameters): several viewports of one scene render in one launch.
constexpr uint32_t kMaxViews = 16;
struct ViewFrames {
  ViewFrame f[kMaxViews];
};

// `f32 as u8`: truncate, saturate, NaN -> 0
__device__ __forceinline__ uint32_t f32_as_u8(float v) {
  return v > 0.0f ? (v >= 255.0f ? 255u : (uint32_t)v) : 0u;
}

// The example's viewport ray through pixel (x, y): direction (glass_point - origin).normalized().
__device__ __forceinline__ void pixel_ray(const ViewFrame& f, uint32_t x, uint32_t y, float& dx, float& dy, float& dz) {
  // glass_point = bottom_left + right * x * pixel_width + up * y * pixel_height
  const float fx = (float)x, fy = (float)y;
  const float gx = (f.bx + (f.rx * fx) * f.pw) + (f.ux * fy) * f.ph;
  const float gy = (f.by + (f.ry * fx) * f.pw) + (f.uy * fy) * f.ph;
  const float gz = (f.bz + (f.rz * fx) * f.pw) + (f.uz * fy) * f.ph;
  // (vector.rs:75-81)
  const float vx = gx - f.ox, vy = gy - f.oy, vz = gz - f.oz;
  const float len = sqrtf((vx * vx + vy * vy) + vz * vz);
  dx = vx / len;
  dy = vy / len;
  dz = vz / len;
}

// The example's colour for a cast result; returns true where the example would panic or loop forever.
__device__ __forceinline__ bool shade_pixel(const SceneView& s, const ViewFrame& f, uint32_t W, uint32_t H, uint32_t x,
                                            uint32_t y, HitRecord& h, uchar4* __restrict__ out) {
  uint32_t kind, albedo, user;
  resolve_entry(s, h, kind, albedo, user);
  uchar4 px;
  bool bad = false;
  if (h.status == 0) {
    px = make_uchar4(f.background >> 24, (f.background >> 16) & 0xFFu, (f.background >> 8) & 0xFFu,
                     f.background & 0xFFu);
  } else if (h.status == 1 && (kind & 1u)) {
    // 1. - (normal.dot(&diffuse_light_normal) / 2. + 0.5)
    const float strength = 1.0f - (((h.nx * f.lx + h.ny * f.ly) + h.nz * f.lz) / 2.0f + 0.5f);
    px = make_uchar4(f32_as_u8((float)(albedo >> 24) * strength), f32_as_u8((float)((albedo >> 16) & 0xFFu) * strength),
                     f32_as_u8((float)((albedo >> 8) & 0xFFu) * strength), 255u);
  } else {
    px = make_uchar4(0, 0, 0, 0);
    bad = true;
  }
  out[(size_t)(H - y - 1) * W + x] = px;
  return bad;
}

// One pixel of the example's loop; returns true where the example would panic or loop forever.
__device__ __forceinline__ bool render_pixel(const SceneView& s, const SharedLuts& L, const ViewFrame& f, uint32_t W,
                                             uint32_t H, uint32_t x, uint32_t y, uchar4* __restrict__ out) {
  float dx, dy, dz;
  pixel_ray(f, x, y, dx, dy, dz);
  HitRecord h;
  cast_one<false>(s, L, f.ox, f.oy, f.oz, dx, dy, dz, h);
  return shade_pixel(s, f, W, H, x, y, h, out);
}

__device__ __forceinline__ void count_unshaded(bool bad, unsigned long long* unshaded) {
  const uint32_t m = __ballot_sync(0xFFFFFFFFu, bad);
  if (unshaded && (threadIdx.x & 31u) == 0 && m) atomicAdd(unshaded, (unsigned long long)__popc(m));
}

// Warps claim 8 x 4 pixel tiles (row-major over the image) from the stream's work counter.  Pixels
// whose ray misses the root box are coloured at once; the entering rays of a tile that has some
// wait in the warp's slice of shared memory (direction, entry point, pixel) until 32 of them fill
// the warp, so that sky pixels do not leave lanes idle.
struct WaitingPixels {
  float d[3][64], p[3][64];
  uint32_t target[64];  // octant of the entry point | view << 8; bit 31: fast form
  uint32_t xy[64];      // x | y << 16
};

__global__ void __launch_bounds__(128, 7)
    render_queue_kernel(SceneView s, ViewFrames fs, uint32_t W, uint32_t H, uchar4* __restrict__ out,
                        unsigned long long* __restrict__ unshaded, unsigned long long* __restrict__ counter,
                        uint32_t tiles_x, uint32_t tiles_per_view, uint32_t tiles) {
  __shared__ SharedLuts L;
  __shared__ WaitingPixels waiting[4];
  fill_shared_luts(L);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  WaitingPixels& w = waiting[threadIdx.x >> 5];
  const size_t frame = (size_t)W * H;
  uint32_t count = 0;  // pixels waiting (the same in every lane)
  bool more = true;    // tiles left
  for (;;) {
    bool have = false, fast = false;
    uint32_t x = 0, y = 0, target = 0, view = 0;
    float dx = 0.0f, dy = 0.0f, dz = 0.0f, px = 0.0f, py = 0.0f, pz = 0.0f;
    while (more && count < 32) {
      unsigned long long t = 0;
      if (lane == 0) t = atomicAdd(counter, 1ull);
      t = __shfl_sync(0xFFFFFFFFu, t, 0);
      if (t >= tiles) {
        more = false;
        break;
      }
      view = (uint32_t)(t / tiles_per_view);
      const uint32_t tv = (uint32_t)(t - (unsigned long long)view * tiles_per_view);
      x = (tv % tiles_x) * 8u + (lane & 7u);
      y = (tv / tiles_x) * 4u + (lane >> 3);
      bool enters = false;
      if (x < W && y < H) {
        const ViewFrame& f = fs.f[view];
        pixel_ray(f, x, y, dx, dy, dz);
        fast = !s.literal && !isnan(dx) && !isnan(dy) && !isnan(dz);
        enters = !fast || fast_entry(s, f.ox, f.oy, f.oz, dx, dy, dz, px, py, pz, target);
        if (!enters) {
          HitRecord h;
          miss_record(h);
          shade_pixel(s, f, W, H, x, y, h, out + view * frame);
        }
      }
      const unsigned m = __ballot_sync(0xFFFFFFFFu, enters);
      if (m == 0xFFFFFFFFu && count == 0) {  // a tile whose rays all enter: cast in place
        have = true;
        break;
      }
      if (enters) {
        const uint32_t k = count + __popc(m & ((1u << lane) - 1u));
        w.d[0][k] = dx;
        w.d[1][k] = dy;
        w.d[2][k] = dz;
        w.p[0][k] = px;
        w.p[1][k] = py;
        w.p[2][k] = pz;
        w.target[k] = target | (view << 8) | (fast ? 0x80000000u : 0u);
        w.xy[k] = x | (y << 16);
      }
      count += __popc(m);
      __syncwarp();
    }
    if (!have) {
      if (count == 0) break;  // no tiles left and nothing waiting
      const uint32_t take = count < 32 ? count : 32;
      if (lane < take) {
        const uint32_t k = count - take + lane;
        dx = w.d[0][k];
        dy = w.d[1][k];
        dz = w.d[2][k];
        px = w.p[0][k];
        py = w.p[1][k];
        pz = w.p[2][k];
        target = w.target[k] & 7u;
        view = (w.target[k] >> 8) & 0xFFu;
        fast = (w.target[k] >> 31) != 0u;
        x = w.xy[k] & 0xFFFFu;
        y = w.xy[k] >> 16;
        have = true;
      }
      count -= take;
      __syncwarp();
    }
    bool bad = false;
    if (have) {
      const ViewFrame& f = fs.f[view];
      HitRecord h;
      cast_entered<false>(s, L, f.ox, f.oy, f.oz, dx, dy, dz, fast, px, py, pz, target, h);
      bad = shade_pixel(s, f, W, H, x, y, h, out + view * frame);
    }
    count_unshaded(bad, unshaded);
  }
}

// One 16 x 8 tile per block (8 x 4 per warp), blockIdx.z the view, for streams without a work counter.
__global__ void __launch_bounds__(128, 7)
    render_grid_kernel(SceneView s, ViewFrames fs, uint32_t W, uint32_t H, uchar4* __restrict__ out,
                       unsigned long long* __restrict__ unshaded) {
  __shared__ SharedLuts L;
  fill_shared_luts(L);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t x = blockIdx.x * 16u + (warp & 1u) * 8u + (lane & 7u);
  const uint32_t y = blockIdx.y * 8u + (warp >> 1) * 4u + (lane >> 3);
  const bool bad = x < W && y < H && render_pixel(s, L, fs.f[blockIdx.z], W, H, x, y, out + (size_t)blockIdx.z * W * H);
  count_unshaded(bad, unshaded);
}

struct V3 {
  float x, y, z;
};
V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 mul(V3 a, float k) { return V3{a.x * k, a.y * k, a.z * k}; }
V3 normalized(V3 a) {
  const float len = std::sqrt((a.x * a.x + a.y * a.y) + a.z * a.z);
  return V3{a.x / len, a.y / len, a.z / len};
}
V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

}  // namespace
}  // namespace svo

using namespace svo;

namespace {
// cpu_render.rs:82-98, host f32 operations in the example's order
ViewFrame frame_of(const svo_viewport* vp, uint32_t W, uint32_t H) {
  const V3 origin{vp->origin[0], vp->origin[1], vp->origin[2]};
  const V3 dir{vp->direction[0], vp->direction[1], vp->direction[2]};
  const V3 up{vp->up[0], vp->up[1], vp->up[2]};
  const V3 right = normalized(cross(up, dir));
  const V3 bl = sub(sub(add(origin, mul(dir, vp->fov)), mul(up, vp->height / 2.0f)), mul(right, vp->width / 2.0f));
  ViewFrame f;
  f.ox = origin.x, f.oy = origin.y, f.oz = origin.z;
  f.rx = right.x, f.ry = right.y, f.rz = right.z;
  f.ux = up.x, f.uy = up.y, f.uz = up.z;
  f.bx = bl.x, f.by = bl.y, f.bz = bl.z;
  f.pw = vp->width / (float)W;
  f.ph = vp->height / (float)H;
  f.lx = vp->light[0], f.ly = vp->light[1], f.lz = vp->light[2];
  f.background = vp->background;
  return f;
}

// up to kMaxViews views in one launch
svo_status render_views(svo_scene* sc, const svo_viewport* vps, uint32_t n_views, uint32_t W, uint32_t H,
                        uchar4* out, unsigned long long* unshaded, cudaStream_t st) {
  ViewFrames fs;
  for (uint32_t k = 0; k < n_views; ++k) fs.f[k] = frame_of(vps + k, W, H);
  const uint64_t tiles_per_view = (uint64_t)((W + 7) / 8) * ((H + 3) / 4);
  const uint64_t tiles = tiles_per_view * n_views;
  CastQueues* q = sc->dev.queues;
  if (q && tiles < 0xFFFFFFFFull && W < 65536u && H < 65536u) {  // the queue packs a pixel's x and y in 16 bits each
    std::lock_guard<std::mutex> lock(q->m);
    if (unsigned long long* ctr = queue_counter(q, st)) {
      static const int per_sm = [] {  // resident blocks per SM: the same kernel on every GPU of a process
        int v = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, render_queue_kernel, 128, 0) == cudaSuccess ? v : 1;
      }();
      const uint64_t grid = std::min<uint64_t>((uint64_t)q->sm_count * std::max(per_sm, 1), (tiles + 3) / 4);
      SVO_CUDA_TRY(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), st));
      render_queue_kernel<<<(unsigned)grid, 128, 0, st>>>(scene_view(sc), fs, W, H, out, unshaded, ctr, (W + 7) / 8,
                                                           (uint32_t)tiles_per_view, (uint32_t)tiles);
      SVO_CUDA_TRY(cudaGetLastError());
      return SVO_OK;
    }
  }
  render_grid_kernel<<<dim3((W + 15) / 16, (H + 7) / 8, n_views), 128, 0, st>>>(scene_view(sc), fs, W, H, out,
                                                                                unshaded);
  SVO_CUDA_TRY(cudaGetLastError());
  return SVO_OK;
}
}  // namespace

extern "C" svo_status svo_render_viewports(svo_scene* sc, const svo_viewport* vps, uint32_t n_views, uint32_t W,
                                           uint32_t H, uint8_t* rgba, unsigned long long* unshaded, void* stream) {
  TraceRange range("svo_render_viewports");
  if (!sc || (!vps && n_views)) return fail(SVO_ERR_ARGUMENT, "svo_render_viewports: NULL argument");
  if (W == 0 || H == 0 || n_views == 0) return SVO_OK;
  if (!rgba) return fail(SVO_ERR_ARGUMENT, "svo_render_viewports: NULL output");
  if (!sc->dev.valid) return fail(SVO_ERR_NOT_UPLOADED, "svo_render_viewports: scene not uploaded");
  if ((H + 7) / 8 > 65535u) return fail(SVO_ERR_ARGUMENT, "svo_render_viewports: image too tall");
  if (reinterpret_cast<uintptr_t>(rgba) % 4 != 0)
    return fail(SVO_ERR_ARGUMENT, "svo_render_viewports: rgba must be 4-byte aligned");
  const cudaStream_t st = (cudaStream_t)stream;
  uchar4* out = reinterpret_cast<uchar4*>(rgba);
  for (uint32_t k = 0; k < n_views; k += kMaxViews) {
    const svo_status rc = render_views(sc, vps + k, std::min(kMaxViews, n_views - k), W, H,
                                       out + (size_t)k * W * H, unshaded, st);
    if (rc != SVO_OK) return rc;
  }
  return SVO_OK;
}

extern "C" svo_status svo_render_viewport(svo_scene* sc, const svo_viewport* vp, uint32_t W, uint32_t H,
                                          uint8_t* rgba, unsigned long long* unshaded, void* stream) {
  if (!sc || !vp) return fail(SVO_ERR_ARGUMENT, "svo_render_viewport: NULL argument");
  return svo_render_viewports(sc, vp, 1, W, H, rgba, unshaded, stream);
}
