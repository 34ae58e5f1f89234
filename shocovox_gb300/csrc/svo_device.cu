// svo_device.cu -- device image of a scene and the plain get_by_ray cast of libsvo (sm_103a).
//
// The device image: 64-byte node records, a brick arena of
// PaletteIndexValues, one occupancy bit per voxel and the two palettes,
// uploaded once and then synced in place from the host octree's dirty
// flags.  The plain cast runs one thread per ray (svo_cast.cuh holds the
// per-ray restatement of Octree::get_by_ray).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>

#include "svo_cast.cuh"
#include "svo_queue.h"
#include "svo_refill.cuh"
#include "svo_trace.h"

namespace svo {

// Device memory of scene images: cudaMalloc / cudaFree, or the caller's allocator
// (svo_set_device_allocator).
struct ImageAllocator {
  svo_alloc_fn alloc = nullptr;
  svo_free_fn release = nullptr;
  void* user = nullptr;
};
ImageAllocator g_image_alloc;
std::mutex g_image_alloc_mutex;

bool caller_allocator() {
  std::lock_guard<std::mutex> lock(g_image_alloc_mutex);
  return g_image_alloc.alloc != nullptr;
}

// `ordered`: from the stream-ordered pool on st (used only without the caller's allocator)
svo_status image_alloc(void** p, size_t bytes, cudaStream_t st, bool ordered = false) {
  ImageAllocator a;
  {
    std::lock_guard<std::mutex> lock(g_image_alloc_mutex);
    a = g_image_alloc;
  }
  *p = nullptr;
  if (a.alloc) {
    *p = a.alloc(bytes, (void*)st, a.user);
    if (!*p) return fail(SVO_ERR_OUT_OF_MEMORY, "scene image: the device allocator returned no memory");
    return SVO_OK;
  }
  if (ordered) {
    SVO_CUDA_TRY(cudaMallocAsync(p, bytes, st));
  } else {
    SVO_CUDA_TRY(cudaMalloc(p, bytes));
  }
  return SVO_OK;
}

void image_free(void* p) {
  if (!p) return;
  ImageAllocator a;
  {
    std::lock_guard<std::mutex> lock(g_image_alloc_mutex);
    a = g_image_alloc;
  }
  if (a.release)
    a.release(p, a.user);
  else
    cudaFree(p);
}

template <bool kCount>
__global__ void __launch_bounds__(128, 7) cast_kernel(SceneView s, RaysView rays, HitsView out, uint64_t n) {
  __shared__ SharedLuts L;
  fill_shared_luts(L);
  __syncthreads();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  HitRecord h;
  cast_one<kCount>(s, L, __ldg(rays.ox + i), __ldg(rays.oy + i), __ldg(rays.oz + i), __ldg(rays.dx + i),
                   __ldg(rays.dy + i), __ldg(rays.dz + i), h);
  write_hit(s, out, i, h);
  if (kCount) write_counters(out, i, h);
}

// Queued cast: a persistent grid whose warps claim 32 rays at a time from a work counter.  The
// cost of a ray varies by orders of magnitude (a sky ray leaves after a few node visits, a
// grazing ray walks a whole cave), and a warp that finishes early takes more work instead of
// idling until its block's slowest warp is done.  The counter (claims taken) starts at 0.
//
// Rays that miss the octree's root box get their miss written at once.  A claim whose rays all
// enter is cast as it is; the entering rays of other claims wait in the warp's slice of shared
// memory, with the point where they enter, until 32 of them fill the warp, so that rays from
// outside the octree (most of them missing it) do not leave most lanes idle.
struct WaitingRays {  // the ray's origin and direction are read again from the ray arrays
  float p[3][64];
  uint32_t target[64];  // octant of the entry point; bit 31: fast form
  unsigned long long i[64];
};

// kStage: the block first copies the scene's top table's first stage_n records into dynamic shared
// memory, and the fast form reads those nodes there.
template <bool kCount, bool kLod = false, bool kStage = false>
__global__ void __launch_bounds__(128, 7)
    queue_kernel(SceneView s, RaysView rays, HitsView out, uint64_t n, ClaimOrder order,
                 unsigned long long* __restrict__ counter, float viewing_distance = 0.0f, uint32_t stage_n = 0) {
  __shared__ SharedLuts L;
  __shared__ WaitingRays waiting[4];
  extern __shared__ uint4 staged_smem[];
  DevNode* stg = reinterpret_cast<DevNode*>(staged_smem);
  fill_shared_luts(L);
  if (kStage) stage_records(stg, s.top, stage_n);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  WaitingRays& w = waiting[threadIdx.x >> 5];
  uint32_t count = 0;  // rays waiting (the same in every lane)
  bool more = true;    // claims left
  for (;;) {
    bool have = false, fast = false;
    uint64_t i = 0;
    float ox = 0.0f, oy = 0.0f, oz = 0.0f, dx = 0.0f, dy = 0.0f, dz = 0.0f, px = 0.0f, py = 0.0f, pz = 0.0f;
    uint32_t target = 0;
    while (more && count < 32) {
      unsigned long long c = 0;
      if (lane == 0) c = atomicAdd(counter, 1ull);
      c = __shfl_sync(0xFFFFFFFFu, c, 0);
      if (c >= order.claims) {
        more = false;
        break;
      }
      const uint64_t j = claimed_ray(order, c, lane, n);
      bool enters = false;
      if (j < n) {
        ox = __ldg(rays.ox + j);
        oy = __ldg(rays.oy + j);
        oz = __ldg(rays.oz + j);
        dx = __ldg(rays.dx + j);
        dy = __ldg(rays.dy + j);
        dz = __ldg(rays.dz + j);
        fast = !s.literal && !isnan(dx) && !isnan(dy) && !isnan(dz);
        enters = !fast || fast_entry(s, ox, oy, oz, dx, dy, dz, px, py, pz, target);
        if (!enters) {
          HitRecord h;
          miss_record(h);
          write_hit(s, out, j, h);
          if (kCount) write_counters(out, j, h);
        }
      }
      const unsigned m = __ballot_sync(0xFFFFFFFFu, enters);
      if (m == 0xFFFFFFFFu && count == 0) {  // a full claim: cast in place
        have = true;
        i = j;
        break;
      }
      if (enters) {
        const uint32_t k = count + __popc(m & ((1u << lane) - 1u));
        w.p[0][k] = px;
        w.p[1][k] = py;
        w.p[2][k] = pz;
        w.target[k] = target | (fast ? 0x80000000u : 0u);
        w.i[k] = j;
      }
      count += __popc(m);
      __syncwarp();
    }
    if (!have) {
      if (count == 0) break;  // no claims left and nothing waiting
      const uint32_t take = count < 32 ? count : 32;
      if (lane < take) {
        const uint32_t k = count - take + lane;
        i = w.i[k];
        ox = __ldg(rays.ox + i);
        oy = __ldg(rays.oy + i);
        oz = __ldg(rays.oz + i);
        dx = __ldg(rays.dx + i);
        dy = __ldg(rays.dy + i);
        dz = __ldg(rays.dz + i);
        px = w.p[0][k];
        py = w.p[1][k];
        pz = w.p[2][k];
        target = w.target[k] & 0x7FFFFFFFu;
        fast = (w.target[k] >> 31) != 0u;
        have = true;
      }
      count -= take;
      __syncwarp();
    }
    if (!have) continue;
    HitRecord h;
    cast_entered<kCount, kLod, kStage>(s, L, ox, oy, oz, dx, dy, dz, fast, px, py, pz, target, h, viewing_distance,
                                       stg, stage_n);
    write_hit(s, out, i, h);
    if (kCount) write_counters(out, i, h);
  }
}

// Refilling cast: the work queue of queue_kernel, where a warp also parks its rays at a node visit
// once fewer than park_below of them are in flight, hands its idle lanes new entering rays from its
// waiting list (refilled from the work counter) and resumes all of them together.  Rays in no
// particular order then keep the lanes busy where a warp would otherwise run its few longest rays
// alone; park_below = 0 never parks (each warp's rays run to their end, as in queue_kernel).
template <bool kCount, bool kStage = false>
__global__ void __launch_bounds__(128, 7)
    refill_kernel(SceneView s, RaysView rays, HitsView out, uint64_t n, ClaimOrder order,
                  unsigned long long* __restrict__ counter, uint32_t park_below, uint32_t stage_n = 0) {
  __shared__ SharedLuts L;
  __shared__ WaitingRays waiting[4];
  __shared__ uint32_t in_flight[4];  // rays of each warp in flight (parked ones included)
  // each thread's ray between two runs: 23 words a thread, an odd stride, so the 32 lanes of a warp
  // touch 32 different banks; registers hold the state only while the ray runs
  __shared__ FastState parked[128];
  extern __shared__ uint4 staged_smem[];
  DevNode* stg = reinterpret_cast<DevNode*>(staged_smem);
  fill_shared_luts(L);
  if (kStage) stage_records(stg, s.top, stage_n);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  WaitingRays& w = waiting[threadIdx.x >> 5];
  volatile uint32_t* live = in_flight + (threadIdx.x >> 5);
  uint32_t count = 0;  // rays waiting (the same in every lane)
  bool more = true;    // claims left
  uint32_t park = park_below;
  bool alive = false;
  uint64_t i = 0;
  for (;;) {
    const unsigned idle = __ballot_sync(0xFFFFFFFFu, !alive);
    const uint32_t need = __popc(idle);
    if (need) {
      // claims until `need` entering rays wait or no claims are left (misses written at once)
      while (more && count < need) {
        unsigned long long c = 0;
        if (lane == 0) c = atomicAdd(counter, 1ull);
        c = __shfl_sync(0xFFFFFFFFu, c, 0);
        if (c >= order.claims) {
          more = false;
          break;
        }
        const uint64_t j = claimed_ray(order, c, lane, n);
        bool enters = false, fast = false;
        float px = 0.0f, py = 0.0f, pz = 0.0f;
        uint32_t target = 0;
        if (j < n) {
          const float ox = __ldg(rays.ox + j), oy = __ldg(rays.oy + j), oz = __ldg(rays.oz + j);
          const float dx = __ldg(rays.dx + j), dy = __ldg(rays.dy + j), dz = __ldg(rays.dz + j);
          fast = !s.literal && !isnan(dx) && !isnan(dy) && !isnan(dz);
          enters = !fast || fast_entry(s, ox, oy, oz, dx, dy, dz, px, py, pz, target);
          if (!enters) {
            HitRecord m;
            miss_record(m);
            write_hit(s, out, j, m);
            if (kCount) write_counters(out, j, m);
          }
        }
        const unsigned m = __ballot_sync(0xFFFFFFFFu, enters);
        if (enters) {
          const uint32_t k = count + __popc(m & ((1u << lane) - 1u));
          w.p[0][k] = px;
          w.p[1][k] = py;
          w.p[2][k] = pz;
          w.target[k] = target | (fast ? 0x80000000u : 0u);
          w.i[k] = j;
        }
        count += __popc(m);
        __syncwarp();
      }
      // the k-th idle lane takes the k-th of the last `take` waiting rays
      const uint32_t take = count < need ? count : need;
      if (!alive) {
        const uint32_t k = __popc(idle & ((1u << lane) - 1u));
        if (k < take) {
          const uint32_t at = count - take + k;
          i = w.i[at];
          const uint32_t tg = w.target[at];
          const float px = w.p[0][at], py = w.p[1][at], pz = w.p[2][at];
          const float ox = __ldg(rays.ox + i), oy = __ldg(rays.oy + i), oz = __ldg(rays.oz + i);
          const float dx = __ldg(rays.dx + i), dy = __ldg(rays.dy + i), dz = __ldg(rays.dz + i);
          if ((tg >> 31) == 0u) {  // a NaN direction (or literal mode): the literal form, in one go
            HitRecord h;
            cast_ray_literal<kCount>(s, L, ox, oy, oz, dx, dy, dz, h);
            write_hit(s, out, i, h);
            if (kCount) write_counters(out, i, h);
          } else {
            fast_start(parked[threadIdx.x], dx, dy, dz, px, py, pz, tg & 0x7FFFFFFFu);
            alive = true;
          }
        }
      }
      count -= take;
      if (take == 0 && !more) park = 0;  // nothing left to hand out: rays in flight run to their end
      __syncwarp();
      const unsigned now = __ballot_sync(0xFFFFFFFFu, alive);
      if (lane == 0) *live = __popc(now);
      __syncwarp();
      if (now == 0) {
        if (!more && count == 0) break;
        continue;
      }
    }
    if (alive) {
      HitRecord h;
      if (fast_run<kCount, kStage>(parked + threadIdx.x, s, L, h, live, park, stg, stage_n)) {
        write_hit(s, out, i, h);
        if (kCount) write_counters(out, i, h);
        alive = false;
      }
    }
    __syncwarp();
  }
}

// Host-buffer cast that reads its rays from and writes its hits to host memory in place (over the CPU
// link).  Stores to host memory cost by the piece, and a warp's 16 x 2 ray block gives pieces of 64
// bytes (4-byte fields) and 16 bytes (1-byte fields) per row.  Here a warp claims two neighbouring
// 16 x 2 blocks (a 32 x 2 block of the image), casts them one after the other -- so that it keeps the
// lock-step of 16 x 2 blocks -- keeps their records in shared memory, and then writes each field row
// by row: 32 neighbouring rays, pieces of 128 and 32 bytes.  The records are those of queue_kernel.
struct PairStage {  // one warp's two blocks, a field at a time (no bank conflicts)
  uint32_t node[64], voxel[64], pix[64], albedo[64], user[64];
  float px[64], py[64], pz[64], nx[64], ny[64], nz[64];
  uint32_t small[64];  // status | octant << 8 | entry kind << 16
};

__global__ void __launch_bounds__(128, 7)
    pair_rows_kernel(SceneView s, RaysView rays, HitsView out, uint64_t n, ClaimOrder order,
                     unsigned long long* __restrict__ counter) {
  __shared__ SharedLuts L;
  __shared__ PairStage stage[4];
  fill_shared_luts(L);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  PairStage& ps = stage[threadIdx.x >> 5];
  for (;;) {
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(counter, 2ull);
    c = __shfl_sync(0xFFFFFFFFu, c, 0);
    if (c >= order.claims) break;
    for (uint32_t half = 0; half < 2; ++half) {
      const uint64_t cc = c + half;
      const uint64_t j = cc < order.claims ? claimed_ray(order, cc, lane, n) : n;
      HitRecord h;
      miss_record(h);
      if (j < n) {
        const float ox = __ldg(rays.ox + j), oy = __ldg(rays.oy + j), oz = __ldg(rays.oz + j);
        const float dx = __ldg(rays.dx + j), dy = __ldg(rays.dy + j), dz = __ldg(rays.dz + j);
        const bool fast = !s.literal && !isnan(dx) && !isnan(dy) && !isnan(dz);
        float px = 0.0f, py = 0.0f, pz = 0.0f;
        uint32_t target = 0;
        if (!fast || fast_entry(s, ox, oy, oz, dx, dy, dz, px, py, pz, target))
          cast_entered<false>(s, L, ox, oy, oz, dx, dy, dz, fast, px, py, pz, target, h);
      }
      // write_hit's record, kept for the rows below
      uint32_t kind, albedo, user;
      resolve_entry(s, h, kind, albedo, user);
      if (h.status != 1) {
        h.octant = h.node = h.pix = 0;
        h.voxel = 0xFFFFFFFFu;
        h.px = h.py = h.pz = h.nx = h.ny = h.nz = 0.0f;
        kind = albedo = user = 0;
      }
      const uint32_t k = half * 32u + lane;
      ps.node[k] = h.node;
      ps.voxel[k] = h.voxel;
      ps.pix[k] = h.pix;
      ps.albedo[k] = albedo;
      ps.user[k] = user;
      ps.px[k] = h.px;
      ps.py[k] = h.py;
      ps.pz[k] = h.pz;
      ps.nx[k] = h.nx;
      ps.ny[k] = h.ny;
      ps.nz[k] = h.nz;
      ps.small[k] = (h.status & 0xFFu) | ((h.octant & 0xFFu) << 8) | ((kind & 0xFFu) << 16);
    }
    __syncwarp();
    // row r of the 32 x 2 block: lanes 0-15 the first block's columns, lanes 16-31 the second's
    for (uint32_t r = 0; r < 2; ++r) {
      const uint32_t half = lane >> 4, bl = (r << 4) | (lane & 15u);
      const uint64_t cc = c + half;
      const uint64_t j = cc < order.claims ? claimed_ray(order, cc, bl, n) : n;
      if (j < n) {
        const uint32_t k = half * 32u + bl;
        const uint32_t sm = ps.small[k];
        if (out.status) out.status[j] = (uint8_t)sm;
        if (out.octant) out.octant[j] = (uint8_t)(sm >> 8);
        if (out.kind) out.kind[j] = (uint8_t)(sm >> 16);
        if (out.node) out.node[j] = ps.node[k];
        if (out.voxel) out.voxel[j] = ps.voxel[k];
        if (out.pix) out.pix[j] = ps.pix[k];
        if (out.albedo) out.albedo[j] = ps.albedo[k];
        if (out.user) out.user[j] = ps.user[k];
        if (out.px) out.px[j] = ps.px[k];
        if (out.py) out.py[j] = ps.py[k];
        if (out.pz) out.pz[j] = ps.pz[k];
        if (out.nx) out.nx[j] = ps.nx[k];
        if (out.ny) out.ny[j] = ps.ny[k];
        if (out.nz) out.nz[j] = ps.nz[k];
      }
    }
    __syncwarp();
  }
}

constexpr uint64_t kQueueMinRays = 1u << 15;  // below this the one-thread-per-ray grid is as fast

void destroy_queues(DeviceImage& d) {
  if (!d.queues) return;
  cudaFree(d.queues->counters);
  delete d.queues;
  d.queues = nullptr;
}

svo_status create_queues(DeviceImage& d) {
  if (d.queues) return SVO_OK;
  CastQueues* q = new CastQueues();
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&q->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q->blocks_per_sm, queue_kernel<false>, 128, 0);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q->blocks_per_sm_count, queue_kernel<true>, 128, 0);
  if (e == cudaSuccess) e = cudaMalloc(&q->counters, kQueueSlots * sizeof(unsigned long long));
  if (e != cudaSuccess) {
    cudaFree(q->counters);
    delete q;
    return fail(e == cudaErrorMemoryAllocation ? SVO_ERR_OUT_OF_MEMORY : SVO_ERR_CUDA,
                std::string("work counters: ") + cudaGetErrorString(e));
  }
  d.queues = q;
  return SVO_OK;
}

// get_by_ray_at_lod one thread per ray, for streams without a work counter.
template <bool kCount>
__global__ void __launch_bounds__(128) lod_grid_kernel(SceneView s, RaysView rays, HitsView out, uint64_t n,
                                                       float viewing_distance) {
  __shared__ SharedLuts L;
  fill_shared_luts(L);
  __syncthreads();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  HitRecord h;
  cast_one<kCount, true>(s, L, __ldg(rays.ox + i), __ldg(rays.oy + i), __ldg(rays.oz + i), __ldg(rays.dx + i),
                         __ldg(rays.dy + i), __ldg(rays.dz + i), h, viewing_distance);
  write_hit(s, out, i, h);
  if (kCount) write_counters(out, i, h);
}

int g_cast_mode = 0;
int g_host_transfer = 0;  // svo_set_host_transfer: 0 auto, 1 staged copies, 2 direct access
int g_stage_depth = 0;    // svo_set_staging_depth: top levels the plain casts stage in shared memory
int g_refill_below = 0;   // svo_set_refill: a warp parks and refills below this many rays in flight
int g_pair_rows = 1;      // host buffers read and written in place: 32 x 2 blocks written row by row

// ------------------------------------------------------------------ device image
uint64_t device_image_bytes(const svo_scene* sc) {
  const DeviceImage& d = sc->dev;
  if (!d.valid) return 0;
  const uint64_t len = sc->tree.arena.len(), W = len >= 32 ? len / 32 : 1;
  return d.node_cap * sizeof(DevNode) + d.brick_cap * (len + W) * 4 + (d.color_cap + d.data_cap) * 4 +
         kMaxStaged * sizeof(DevNode);
}
uint64_t device_image_bytes_estimate(const svo_scene* sc) {
  const HostOctree& t = sc->tree;
  const uint64_t nn = t.nodes(), nb = std::max<uint64_t>(1, t.arena.slots());
  const uint64_t nc = std::max<uint64_t>(1, t.colors.size()), nd = std::max<uint64_t>(1, t.datas.size());
  const uint64_t len = t.arena.len(), W = len >= 32 ? len / 32 : 1;
  return (nn + nn / 4 + 64) * sizeof(DevNode) + (nb + nb / 4 + 16) * (len + W) * 4 + (nc + nc / 4 + 64 + nd + nd / 4 + 64) * 4 +
         kMaxStaged * sizeof(DevNode);
}

SceneView scene_view(const svo_scene* sc) {
  const DeviceImage& d = sc->dev;
  SceneView v;
  v.nodes = d.nodes;
  v.voxels = d.voxels;
  v.vbits = d.vbits;
  v.colors = d.colors;
  v.datas = d.datas;
  v.n_nodes = (uint32_t)d.n_nodes;
  v.n_colors = (uint32_t)d.n_colors;
  v.n_datas = (uint32_t)d.n_datas;
  v.dim = sc->tree.dim;
  const uint32_t len = sc->tree.arena.len();
  v.vwords = len >= 32 ? len / 32 : 1;
  v.size = (float)sc->tree.size;
  v.inv_size = 1.0f / v.size;
  v.inv_dim = 1.0f / (float)v.dim;
  v.literal = g_cast_mode == 1 ? 1u : 0u;
  v.mips = sc->tree.mips_enabled ? 1u : 0u;
  uint32_t levels = 0;
  for (uint32_t r = sc->tree.size / sc->tree.dim; r > 1; r >>= 1) ++levels;
  v.mip_top = (float)levels;
  v.top = d.top;
  return v;
}

uint32_t staged_records(const svo_scene* sc, uint32_t depth) {
  const DeviceImage& d = sc->dev;
  return d.top ? d.top_count[std::min(depth, kMaxStageDepth)] : 0u;
}

namespace {

uint32_t vwords_of(const HostOctree& t) { return t.arena.len() >= 32 ? t.arena.len() / 32 : 1; }

void build_node(const HostOctree& t, size_t k, DevNode& n) {
  std::memset(&n, 0, sizeof(n));
  for (auto& v : n.slot) v = kInvalidChild;
  for (auto& v : n.stage) v = kNotStaged;  // set by stage_top for the nodes of the top table
  if (!t.reserved[k]) return;
  const uint32_t kind = t.kind[k];
  n.ocbits = t.stored_occupied_bits(k);
  n.meta = kind | (1u << 2);
  if (kind == kInternal) {
    if (t.ch_kind[k] == kChildren)
      for (int i = 0; i < 8; ++i) {
        const uint32_t c = t.ch[k * 8 + i];
        n.slot[i] = t.key_valid(c) ? c : kInvalidChild;
      }
  } else if (kind == kLeaf || kind == kUniform) {
    const int nb = kind == kLeaf ? 8 : 1;
    for (int i = 0; i < nb; ++i) {
      const BrickRef& b = t.bricks[k * 8 + i];
      n.meta |= (uint32_t)b.kind << (8 + 2 * i);
      n.slot[i] = b.kind == kBrickEmpty ? 0u : b.v;
    }
  }
  if (k >= t.mips.size()) {
    n.meta |= 3u << 24;
  } else {
    const BrickRef& m = t.mips[k];
    n.meta |= (uint32_t)m.kind << 24;
    n.mip = m.kind == kBrickEmpty ? 0u : m.v;
  }
}

void build_vbits(const HostOctree& t, uint32_t slot, uint32_t* out) {
  const uint32_t W = vwords_of(t), len = t.arena.len();
  std::memset(out, 0, sizeof(uint32_t) * W);
  if (!t.arena.live(slot)) return;
  const uint32_t* v = t.arena.at(slot);
  for (uint32_t f = 0; f < len; ++f)
    if (!t.pix_empty(v[f])) out[f >> 5] |= 1u << (f & 31);
}

// The top table (breadth-first Internal nodes of depth < kMaxStageDepth) from the node records, and
// every record's stage[] naming its staged children.  Records whose stage[] changes are marked dirty.
void stage_top(HostOctree& t, DeviceImage& d) {
  const uint64_t nn = d.host_nodes.size();
  auto internal = [&](uint32_t k) {
    return k < nn && (d.host_nodes[k].meta & 3u) == kInternal && (d.host_nodes[k].meta & 4u) != 0;
  };
  std::vector<uint32_t> keys;
  std::unordered_map<uint32_t, uint32_t> index;  // node key -> its place in the table
  std::vector<uint32_t> count(kMaxStageDepth + 1, 0);
  if (internal(0)) {
    keys.push_back(0);
    index[0] = 0;
  }
  count[1] = (uint32_t)keys.size();
  size_t level = 0;
  for (uint32_t depth = 1; depth < kMaxStageDepth; ++depth) {
    const size_t end = keys.size();
    for (size_t i = level; i < end; ++i)
      for (int c = 0; c < 8; ++c) {
        const uint32_t ck = d.host_nodes[keys[i]].slot[c];
        if (ck != kInvalidChild && internal(ck) && index.emplace(ck, (uint32_t)keys.size()).second) keys.push_back(ck);
      }
    level = end;
    count[depth + 1] = (uint32_t)keys.size();
  }
  auto set_stage = [&](uint32_t k, const uint16_t (&st)[8]) {
    if (std::memcmp(d.host_nodes[k].stage, st, sizeof(st)) != 0) {
      std::memcpy(d.host_nodes[k].stage, st, sizeof(st));
      if (k < t.node_dirty.size()) t.node_dirty[k] = 1;
    }
  };
  const uint16_t none[8] = {kNotStaged, kNotStaged, kNotStaged, kNotStaged,
                            kNotStaged, kNotStaged, kNotStaged, kNotStaged};
  for (uint32_t k : d.top_keys)
    if (k < nn && !index.count(k)) set_stage(k, none);
  for (uint32_t k : keys) {
    uint16_t st[8];
    for (int c = 0; c < 8; ++c) {
      const auto at = index.find(d.host_nodes[k].slot[c]);
      st[c] = at == index.end() ? kNotStaged : (uint16_t)at->second;
    }
    set_stage(k, st);
  }
  d.top_keys = keys;
  for (uint32_t k = 0; k <= kMaxStageDepth; ++k) d.top_count[k] = count[k];
}

// Copies the top table's records from the node mirror to the device.
svo_status upload_top(DeviceImage& d, cudaStream_t st) {
  if (!d.top) {
    void* p = nullptr;
    const svo_status rc = image_alloc(&p, kMaxStaged * sizeof(DevNode), st, d.ordered);
    if (rc != SVO_OK) return rc;
    d.top = static_cast<DevNode*>(p);
  }
  d.host_top.resize(d.top_keys.size());
  for (size_t i = 0; i < d.top_keys.size(); ++i) d.host_top[i] = d.host_nodes[d.top_keys[i]];
  if (!d.host_top.empty())
    SVO_CUDA_TRY(cudaMemcpyAsync(d.top, d.host_top.data(), d.host_top.size() * sizeof(DevNode),
                                 cudaMemcpyHostToDevice, st));
  return SVO_OK;
}

void free_blob(DeviceImage& d) {
  if (d.blob_done) {
    cudaEventSynchronize(d.blob_done);  // no copy still reads the blob
    cudaEventDestroy(d.blob_done);
    d.blob_done = nullptr;
  }
  if (d.blob) cudaFreeHost(d.blob);
  d.blob = nullptr;
  d.blob_bytes = 0;
  d.blob_ok = false;
}

void free_device(DeviceImage& d) {
  // cudaFree waits for no cast on memory from the stream-ordered pool: wait for the device here, as
  // cudaFree does for other memory, so that releasing a scene keeps the same meaning either way
  if (d.ordered && (d.top || d.nodes || d.block)) cudaDeviceSynchronize();
  if (d.block) {
    cudaFree(d.block);
    d.block = nullptr;
  } else if (d.ordered) {
    cudaFree(d.top);
    cudaFree(d.nodes);
    cudaFree(d.voxels);
    cudaFree(d.vbits);
    cudaFree(d.colors);
    cudaFree(d.datas);
  } else {
    image_free(d.top);
    image_free(d.nodes);
    image_free(d.voxels);
    image_free(d.vbits);
    image_free(d.colors);
    image_free(d.datas);
  }
  d.ordered = false;
  d.top = nullptr;
  for (auto& c : d.top_count) c = 0;  // top_keys describe the host mirror, which stays
  d.nodes = nullptr;
  d.voxels = d.vbits = d.colors = d.datas = nullptr;
  d.node_cap = d.brick_cap = d.color_cap = d.data_cap = 0;
  d.valid = false;
}

// The tree has changed in nothing since the device image was last made or synced.
bool tree_clean(HostOctree& t) {
  auto none = [](const std::vector<uint8_t>& f) { return std::find(f.begin(), f.end(), 1) == f.end(); };
  return !t.structure_grew && t.colors_synced == t.colors.size() && t.datas_synced == t.datas.size() &&
         none(t.node_dirty) && none(t.arena.dirty());
}

// Marks the device image in step with the tree.
void image_synced(HostOctree& t, DeviceImage& d) {
  d.n_nodes = t.nodes();
  d.n_bricks = t.arena.slots();
  d.n_colors = t.colors.size();
  d.n_datas = t.datas.size();
  std::fill(t.node_dirty.begin(), t.node_dirty.end(), 0);
  std::fill(t.arena.dirty().begin(), t.arena.dirty().end(), 0);
  t.colors_synced = t.colors.size();
  t.datas_synced = t.datas.size();
  t.structure_grew = false;
  d.valid = true;
}

// The stream-ordered image of a server's scene: one block of the pool, filled from the pinned blob
// (the arrays in the order nodes, top table, voxels, voxel bits, colors, user data; each at a
// 256-byte boundary).  `fill`: the host mirror changed, copy it into the blob first.
svo_status upload_block(svo_scene* sc, cudaStream_t st, bool fill) {
  HostOctree& t = sc->tree;
  DeviceImage& d = sc->dev;
  const uint64_t W = vwords_of(t), len = t.arena.len(), nb = t.arena.slots();
  const uint64_t cap[6] = {d.node_cap * sizeof(DevNode), kMaxStaged * sizeof(DevNode), d.brick_cap * len * 4,
                           d.brick_cap * W * 4, d.color_cap * 4, d.data_cap * 4};
  uint64_t off[6], total = 0;
  for (int i = 0; i < 6; ++i) {
    off[i] = total;
    total += (cap[i] + 255) / 256 * 256;
  }
  if (!fill && d.blob_bytes != total) {
    stage_top(t, d);  // the top table of the (unchanged) mirror, for the blob made again below
    fill = true;
  }
  if (fill) {
    if (d.blob_bytes != total) {
      free_blob(d);
      void* h = nullptr;
      if (cudaMallocHost(&h, total) != cudaSuccess) {
        cudaGetLastError();
        d.ordered = false;
        free_device(d);
        return fail(SVO_ERR_OUT_OF_MEMORY, "scene image: no pinned host memory for the upload copy");
      }
      d.blob = static_cast<uint8_t*>(h);
      d.blob_bytes = total;
    } else if (d.blob_done) {
      SVO_CUDA_TRY(cudaEventSynchronize(d.blob_done));  // the last upload has finished reading the blob
    }
    d.host_top.resize(d.top_keys.size());
    for (size_t i = 0; i < d.top_keys.size(); ++i) d.host_top[i] = d.host_nodes[d.top_keys[i]];
    const void* src[6] = {d.host_nodes.data(), d.host_top.data(), t.arena.raw().data(), d.host_vbits.data(),
                          t.colors.data(), t.datas.data()};
    const uint64_t used[6] = {d.host_nodes.size() * sizeof(DevNode), d.host_top.size() * sizeof(DevNode),
                              nb * len * 4, nb * W * 4, t.colors.size() * 4, t.datas.size() * 4};
    for (int i = 0; i < 6; ++i)
      if (used[i]) std::memcpy(d.blob + off[i], src[i], used[i]);
    for (uint32_t k = 0; k <= kMaxStageDepth; ++k) d.blob_top_count[k] = d.top_count[k];
    d.blob_ok = true;
  } else {
    for (uint32_t k = 0; k <= kMaxStageDepth; ++k) d.top_count[k] = d.blob_top_count[k];
  }
  void* p = nullptr;
  {
    const svo_status rc = image_alloc(&p, total, st, true);
    if (rc != SVO_OK) {
      d.ordered = false;
      free_device(d);
      return rc;
    }
  }
  uint8_t* base = static_cast<uint8_t*>(p);
  d.block = p;
  d.nodes = reinterpret_cast<DevNode*>(base + off[0]);
  d.top = reinterpret_cast<DevNode*>(base + off[1]);
  d.voxels = reinterpret_cast<uint32_t*>(base + off[2]);
  d.vbits = reinterpret_cast<uint32_t*>(base + off[3]);
  d.colors = reinterpret_cast<uint32_t*>(base + off[4]);
  d.datas = reinterpret_cast<uint32_t*>(base + off[5]);
  const uint64_t used[6] = {t.nodes() * sizeof(DevNode), d.host_top.size() * sizeof(DevNode), nb * len * 4,
                            nb * W * 4, t.colors.size() * 4, t.datas.size() * 4};
  for (int i = 0; i < 6; ++i)
    if (used[i]) SVO_CUDA_TRY(cudaMemcpyAsync(base + off[i], d.blob + off[i], used[i], cudaMemcpyHostToDevice, st));
  if (!d.blob_done) SVO_CUDA_TRY(cudaEventCreateWithFlags(&d.blob_done, cudaEventDisableTiming));
  SVO_CUDA_TRY(cudaEventRecord(d.blob_done, st));
  image_synced(t, d);
  return SVO_OK;
}

svo_status full_upload(svo_scene* sc, cudaStream_t st, bool ordered = false) {
  HostOctree& t = sc->tree;
  DeviceImage& d = sc->dev;
  free_device(d);
  d.ordered = ordered && !caller_allocator();
  {
    const svo_status qs = create_queues(d);
    if (qs != SVO_OK) return qs;
  }
  const uint64_t nn = t.nodes(), nb = std::max<uint64_t>(1, t.arena.slots());
  const uint64_t nc = std::max<uint64_t>(1, t.colors.size()), ndt = std::max<uint64_t>(1, t.datas.size());
  // headroom so that later in-place syncs rarely need a new allocation
  d.node_cap = nn + nn / 4 + 64;
  d.brick_cap = nb + nb / 4 + 16;
  d.color_cap = nc + nc / 4 + 64;
  d.data_cap = ndt + ndt / 4 + 64;
  const uint32_t W = vwords_of(t), len = t.arena.len();
  // a server's scene evicted and uploaded again unchanged: the blob already holds its image
  if (d.ordered && d.blob_ok && d.mirror_ok && tree_clean(t)) return upload_block(sc, st, false);
  if (!d.ordered) d.blob_ok = false;  // in-place syncs of this image do not reach the blob
  try {
    // the host mirror of the records is rebuilt where the tree changed since it was last built (all of
    // it the first time, or after svo_scene_release_device); a scene evicted by a server and uploaded
    // again unchanged only copies
    const bool reuse = d.mirror_ok && d.host_nodes.size() <= nn && d.host_vbits.size() <= t.arena.slots() * (size_t)W;
    if (!reuse) {
      d.host_nodes.assign(nn, DevNode{});
      d.host_vbits.assign(t.arena.slots() * (size_t)W, 0u);
    }
    d.host_nodes.resize(nn);
    d.host_vbits.resize(t.arena.slots() * (size_t)W, 0u);
    auto& bd = t.arena.dirty();
    for (uint64_t k = 0; k < nn; ++k)
      if (!reuse || t.node_dirty[k]) build_node(t, k, d.host_nodes[k]);
    for (uint32_t sl = 0; sl < t.arena.slots(); ++sl)
      if (!reuse || bd[sl]) build_vbits(t, sl, &d.host_vbits[(size_t)sl * W]);
    stage_top(t, d);
    d.mirror_ok = true;
  } catch (const ReferencePanic& p) {
    d.mirror_ok = false;
    d.blob_ok = false;
    return fail(SVO_ERR_REFERENCE_PANIC, std::string("upload: ") + p.what());
  }
  if (d.ordered) return upload_block(sc, st, true);
  {
    // a failed allocation releases what the upload holds: the scene is left without a device image
    void* p[5] = {};
    const size_t bytes[5] = {d.node_cap * sizeof(DevNode), d.brick_cap * (size_t)len * 4, d.brick_cap * (size_t)W * 4,
                             d.color_cap * 4, d.data_cap * 4};
    for (int i = 0; i < 5; ++i) {
      const svo_status rc = image_alloc(&p[i], bytes[i], st, d.ordered);
      if (rc != SVO_OK) {
        for (int j = 0; j < i; ++j) {
          if (d.ordered)
            cudaFreeAsync(p[j], st);
          else
            image_free(p[j]);
        }
        d.ordered = false;
        free_device(d);
        return rc;
      }
    }
    d.nodes = static_cast<DevNode*>(p[0]);
    d.voxels = static_cast<uint32_t*>(p[1]);
    d.vbits = static_cast<uint32_t*>(p[2]);
    d.colors = static_cast<uint32_t*>(p[3]);
    d.datas = static_cast<uint32_t*>(p[4]);
  }
  SVO_CUDA_TRY(cudaMemcpyAsync(d.nodes, d.host_nodes.data(), nn * sizeof(DevNode), cudaMemcpyHostToDevice, st));
  {
    const svo_status ts = upload_top(d, st);
    if (ts != SVO_OK) {
      free_device(d);
      return ts;
    }
  }
  if (t.arena.slots()) {
    SVO_CUDA_TRY(cudaMemcpyAsync(d.voxels, t.arena.raw().data(), (size_t)t.arena.slots() * len * 4,
                                 cudaMemcpyHostToDevice, st));
    SVO_CUDA_TRY(cudaMemcpyAsync(d.vbits, d.host_vbits.data(), d.host_vbits.size() * 4, cudaMemcpyHostToDevice, st));
  }
  if (!t.colors.empty())
    SVO_CUDA_TRY(cudaMemcpyAsync(d.colors, t.colors.data(), t.colors.size() * 4, cudaMemcpyHostToDevice, st));
  if (!t.datas.empty())
    SVO_CUDA_TRY(cudaMemcpyAsync(d.datas, t.datas.data(), t.datas.size() * 4, cudaMemcpyHostToDevice, st));
  // pageable sources: the copies are staged before cudaMemcpyAsync returns, but
  // the mirrors must stay valid until then, which they do (they live in the scene)
  image_synced(t, d);
  return SVO_OK;
}

// Copies runs of flagged elements [i, j) with one cudaMemcpyAsync per run.
template <class F>
svo_status copy_runs(std::vector<uint8_t>& flags, uint64_t limit, F&& copy) {
  uint64_t i = 0;
  while (i < limit) {
    if (!flags[i]) {
      ++i;
      continue;
    }
    uint64_t j = i;
    while (j < limit && flags[j]) flags[j++] = 0;
    svo_status rc = copy(i, j);
    if (rc != SVO_OK) return rc;
    i = j;
  }
  return SVO_OK;
}

svo_status incremental_sync(svo_scene* sc, cudaStream_t st) {
  HostOctree& t = sc->tree;
  DeviceImage& d = sc->dev;
  const uint64_t nn = t.nodes();
  if (nn > d.node_cap || t.arena.slots() > d.brick_cap || t.colors.size() > d.color_cap || t.datas.size() > d.data_cap)
    return full_upload(sc, st);
  const uint32_t W = vwords_of(t), len = t.arena.len();
  if (!tree_clean(t)) d.blob_ok = false;  // the image changes in place, the blob keeps the old one
  try {
    d.host_nodes.resize(nn);
    for (uint64_t k = 0; k < nn; ++k)
      if (t.node_dirty[k]) build_node(t, k, d.host_nodes[k]);
    stage_top(t, d);  // rebuilt records lost their stage indices, and the top levels may have changed
    d.host_vbits.resize((size_t)t.arena.slots() * W, 0u);
    auto& bd = t.arena.dirty();
    for (uint32_t sl = 0; sl < t.arena.slots(); ++sl)
      if (bd[sl]) build_vbits(t, sl, &d.host_vbits[(size_t)sl * W]);
  } catch (const ReferencePanic& p) {
    return fail(SVO_ERR_REFERENCE_PANIC, std::string("sync: ") + p.what());
  }
  svo_status rc = copy_runs(t.node_dirty, nn, [&](uint64_t a, uint64_t b) -> svo_status {
    SVO_CUDA_TRY(cudaMemcpyAsync(d.nodes + a, d.host_nodes.data() + a, (b - a) * sizeof(DevNode),
                                 cudaMemcpyHostToDevice, st));
    return SVO_OK;
  });
  if (rc != SVO_OK) return rc;
  rc = upload_top(d, st);
  if (rc != SVO_OK) return rc;
  rc = copy_runs(t.arena.dirty(), t.arena.slots(), [&](uint64_t a, uint64_t b) -> svo_status {
    SVO_CUDA_TRY(cudaMemcpyAsync(d.voxels + a * len, t.arena.raw().data() + a * len, (b - a) * len * 4,
                                 cudaMemcpyHostToDevice, st));
    SVO_CUDA_TRY(cudaMemcpyAsync(d.vbits + a * W, d.host_vbits.data() + a * W, (b - a) * W * 4,
                                 cudaMemcpyHostToDevice, st));
    return SVO_OK;
  });
  if (rc != SVO_OK) return rc;
  if (t.colors.size() > t.colors_synced)
    SVO_CUDA_TRY(cudaMemcpyAsync(d.colors + t.colors_synced, t.colors.data() + t.colors_synced,
                                 (t.colors.size() - t.colors_synced) * 4, cudaMemcpyHostToDevice, st));
  if (t.datas.size() > t.datas_synced)
    SVO_CUDA_TRY(cudaMemcpyAsync(d.datas + t.datas_synced, t.datas.data() + t.datas_synced,
                                 (t.datas.size() - t.datas_synced) * 4, cudaMemcpyHostToDevice, st));
  t.colors_synced = t.colors.size();
  t.datas_synced = t.datas.size();
  d.n_nodes = nn;
  d.n_bricks = t.arena.slots();
  d.n_colors = t.colors.size();
  d.n_datas = t.datas.size();
  return SVO_OK;
}


// `in_place`: rays and hits are host memory the device reads and writes through the CPU's page
// tables; the claims are then 16 x 2 blocks (two 64-byte pieces of each array per warp instead of
// four 32-byte ones), which the host link serves faster than 8 x 4 blocks.
svo_status launch_cast(svo_scene* sc, const svo_rays* rays, uint64_t n, const svo_hits* hits, cudaStream_t st,
                       uint64_t row = 0, bool in_place = false) {
  if (n == 0) return SVO_OK;
  const SceneView v = scene_view(sc);
  RaysView rv{rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz};
  const HitsView hv = hits_view_of(*hits);
  const bool count = counts_requested(*hits);
  const unsigned block = 128;
  CastQueues* q = sc->dev.queues;
  if (q && n >= kQueueMinRays) {
    std::lock_guard<std::mutex> lock(q->m);
    if (unsigned long long* ctr = queue_counter(q, st)) {
      const int per_sm = std::max(1, count ? q->blocks_per_sm_count : q->blocks_per_sm);
      const uint64_t grid = std::min<uint64_t>((uint64_t)q->sm_count * per_sm, (n + block - 1) / block);
      SVO_CUDA_TRY(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), st));
      const ClaimOrder order = claim_order(n, row, in_place ? 4 : 3);
      const uint32_t stage_n = g_cast_mode == 1 ? 0u : staged_records(sc, (uint32_t)g_stage_depth);
      // two blocks per claim halve the units of work: only where every resident warp gets at least four
      // of them (a small batch keeps the per-block claims, whose tail is shorter)
      const uint64_t warps = (uint64_t)q->sm_count * (uint64_t)per_sm * (block / 32);
      if (in_place && !count && stage_n == 0 && g_refill_below == 0 && g_pair_rows && n >= warps * 64 * 4) {
        pair_rows_kernel<<<(unsigned)grid, block, 0, st>>>(v, rv, hv, n, order, ctr);
      } else if (g_refill_below > 0) {
        const size_t smem = (size_t)stage_n * sizeof(DevNode);
        auto kern = stage_n ? (count ? refill_kernel<true, true> : refill_kernel<false, true>)
                            : (count ? refill_kernel<true> : refill_kernel<false>);
        SVO_CUDA_TRY(allow_dynamic_smem(kern, smem));
        int per = 0;
        SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, block, smem));
        const uint64_t rgrid = std::min<uint64_t>((uint64_t)q->sm_count * std::max(per, 1), (n + block - 1) / block);
        kern<<<(unsigned)rgrid, block, smem, st>>>(v, rv, hv, n, order, ctr, (uint32_t)g_refill_below, stage_n);
      } else if (stage_n) {
        // the staged records take dynamic shared memory: resident blocks from this launch's size
        const size_t smem = (size_t)stage_n * sizeof(DevNode);
        auto kern = count ? queue_kernel<true, false, true> : queue_kernel<false, false, true>;
        SVO_CUDA_TRY(allow_dynamic_smem(kern, smem));
        int per = 0;
        SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, block, smem));
        const uint64_t sgrid = std::min<uint64_t>((uint64_t)q->sm_count * std::max(per, 1), (n + block - 1) / block);
        kern<<<(unsigned)sgrid, block, smem, st>>>(v, rv, hv, n, order, ctr, 0.0f, stage_n);
      } else if (count) {
        queue_kernel<true><<<(unsigned)grid, block, 0, st>>>(v, rv, hv, n, order, ctr);
      } else {
        queue_kernel<false><<<(unsigned)grid, block, 0, st>>>(v, rv, hv, n, order, ctr);
      }
      SVO_CUDA_TRY(cudaGetLastError());
      return SVO_OK;
    }
  }
  const uint64_t grid = (n + block - 1) / block;
  if (grid > 0x7FFFFFFFull) return fail(SVO_ERR_ARGUMENT, "svo_cast: too many rays for one launch");
  if (count)
    cast_kernel<true><<<(unsigned)grid, block, 0, st>>>(v, rv, hv, n);
  else
    cast_kernel<false><<<(unsigned)grid, block, 0, st>>>(v, rv, hv, n);
  SVO_CUDA_TRY(cudaGetLastError());
  return SVO_OK;
}

// Host-buffer cast, pipelined: the batch is cut into chunks cast on three
// streams in turn, so chunk i+1's host->device copy and chunk i-1's
// device->host copy overlap chunk i's kernel (with pinned host memory; with
// pageable memory the copies still run, only without overlap).
constexpr int kPipeStreams = 3;

struct HostPipeline {
  cudaStream_t st[kPipeStreams] = {};
  cudaEvent_t ready = nullptr;                 // caller's stream reached the call
  cudaEvent_t done[kPipeStreams] = {};         // a pipeline stream finished its chunks
  char* buf[kPipeStreams] = {};
  size_t buf_bytes = 0;
};

void destroy_pipeline(DeviceImage& d) {
  HostPipeline* p = static_cast<HostPipeline*>(d.ws);
  if (!p) return;
  for (int i = 0; i < kPipeStreams; ++i) {
    if (p->st[i]) cudaStreamSynchronize(p->st[i]);
    cudaFree(p->buf[i]);
    if (p->st[i]) cudaStreamDestroy(p->st[i]);
    if (p->done[i]) cudaEventDestroy(p->done[i]);
  }
  if (p->ready) cudaEventDestroy(p->ready);
  delete p;
  d.ws = nullptr;
  d.ws_bytes = 0;
}

svo_status cast_host_pipelined(svo_scene* sc, const svo_rays* rays, uint64_t n, const svo_hits* hits,
                               cudaStream_t caller, uint64_t row) {
  DeviceImage& d = sc->dev;
  void* const* host_fields = reinterpret_cast<void* const*>(hits);
  size_t per_ray = 24;
  for (int f = 0; f < kHitFields; ++f)
    if (host_fields[f]) per_ray += kHitFieldBytes[f];
  uint64_t chunk = std::min<uint64_t>(n, std::max<uint64_t>(262144, ((n / 6 + 255) / 256) * 256));
  if (row) chunk = std::min<uint64_t>(n, ((chunk + 4 * row - 1) / (4 * row)) * 4 * row);  // whole bands of rows
  const size_t need = (size_t)chunk * per_ray + 32 * 256;
  HostPipeline* p = static_cast<HostPipeline*>(d.ws);
  if (!p) {
    p = new HostPipeline();
    d.ws = p;
    for (int i = 0; i < kPipeStreams; ++i) {
      SVO_CUDA_TRY(cudaStreamCreateWithFlags(&p->st[i], cudaStreamNonBlocking));
      SVO_CUDA_TRY(cudaEventCreateWithFlags(&p->done[i], cudaEventDisableTiming));
    }
    SVO_CUDA_TRY(cudaEventCreateWithFlags(&p->ready, cudaEventDisableTiming));
  }
  if (need > p->buf_bytes) {
    for (int i = 0; i < kPipeStreams; ++i) {
      SVO_CUDA_TRY(cudaStreamSynchronize(p->st[i]));
      cudaFree(p->buf[i]);
      p->buf[i] = nullptr;
    }
    p->buf_bytes = 0;
    for (int i = 0; i < kPipeStreams; ++i) SVO_CUDA_TRY(cudaMalloc(&p->buf[i], need));
    p->buf_bytes = need;
    d.ws_bytes = need * kPipeStreams;
  }
  // the pipeline streams start after the work already queued on the caller's stream
  SVO_CUDA_TRY(cudaEventRecord(p->ready, caller));
  for (int i = 0; i < kPipeStreams; ++i) SVO_CUDA_TRY(cudaStreamWaitEvent(p->st[i], p->ready, 0));
  const float* hr[6] = {rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz};
  uint64_t c = 0;
  for (uint64_t off = 0; off < n; off += chunk, ++c) {
    const uint64_t m = std::min<uint64_t>(chunk, n - off);
    const int k = (int)(c % kPipeStreams);
    cudaStream_t st = p->st[k];
    char* base = p->buf[k];
    size_t o = 0;
    float* dr[6];
    for (int a = 0; a < 6; ++a) {
      dr[a] = reinterpret_cast<float*>(base + o);
      o += ((chunk * 4 + 255) / 256) * 256;
      SVO_CUDA_TRY(cudaMemcpyAsync(dr[a], hr[a] + off, m * 4, cudaMemcpyHostToDevice, st));
    }
    svo_hits dh;
    std::memset(&dh, 0, sizeof(dh));
    void** dev_fields = reinterpret_cast<void**>(&dh);
    for (int f = 0; f < kHitFields; ++f)
      if (host_fields[f]) {
        dev_fields[f] = base + o;
        o += ((kHitFieldBytes[f] * chunk + 255) / 256) * 256;
      }
    svo_rays drays{dr[0], dr[1], dr[2], dr[3], dr[4], dr[5]};
    svo_status rc = launch_cast(sc, &drays, m, &dh, st, row);
    if (rc != SVO_OK) return rc;
    for (int f = 0; f < kHitFields; ++f)
      if (host_fields[f])
        SVO_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(host_fields[f]) + off * kHitFieldBytes[f], dev_fields[f],
                                     kHitFieldBytes[f] * m, cudaMemcpyDeviceToHost, st));
  }
  for (int i = 0; i < kPipeStreams; ++i) {
    SVO_CUDA_TRY(cudaEventRecord(p->done[i], p->st[i]));
    SVO_CUDA_TRY(cudaStreamWaitEvent(caller, p->done[i], 0));
  }
  SVO_CUDA_TRY(cudaStreamSynchronize(caller));
  return SVO_OK;
}

}  // namespace

// ------------------------------------------------------------------ LUT self-test kernel
// Reports the tables exactly as a cast block holds them in shared memory.
__global__ void lut_kernel(uint64_t* rtn, uint32_t* step, uint64_t* mask) {
  __shared__ SharedLuts L;
  fill_shared_luts(L);
  __syncthreads();
  const uint32_t t = threadIdx.x;
  if (t < 512) rtn[t] = L.ray_to_node[t];
  if (t < 8) mask[t] = L.octant[t];
  if (t < 27) {  // OCTANT_STEP_RESULT_LUT[x][y][z] packs 8 octants x 4 bits
    const int x = (int)(t / 9) - 1, y = (int)((t / 3) % 3) - 1, z = (int)(t % 3) - 1;
    uint32_t packed = 0;
    for (uint32_t o = 0; o < 8; ++o) packed |= (step_octant(o, (float)x, (float)y, (float)z) & 0xFu) << (4 * o);
    step[t] = packed;
  }
}

}  // namespace svo

using namespace svo;

extern "C" {

}  // extern "C"

namespace svo {
svo_status upload_ordered(svo_scene* sc, cudaStream_t st) {
  TraceRange range("svo_scene_upload (stream-ordered)");
  const svo_status rc = full_upload(sc, st, true);
  if (rc != SVO_OK) return rc;
  DeviceImage& d = sc->dev;
  if (!d.ready) SVO_CUDA_TRY(cudaEventCreateWithFlags(&d.ready, cudaEventDisableTiming));
  SVO_CUDA_TRY(cudaEventRecord(d.ready, st));
  return SVO_OK;
}

svo_status evict_ordered(svo_scene* sc, cudaStream_t st) {
  TraceRange range("svo_scene_evict");
  DeviceImage& d = sc->dev;
  if (!d.ordered) return svo_scene_release_device(sc);
  if (d.block) {
    SVO_CUDA_TRY(cudaFreeAsync(d.block, st));
    d.block = nullptr;
  } else {
    void* arrays[6] = {d.top, d.nodes, d.voxels, d.vbits, d.colors, d.datas};
    for (void* p : arrays)
      if (p) SVO_CUDA_TRY(cudaFreeAsync(p, st));
  }
  d.top = d.nodes = nullptr;
  d.voxels = d.vbits = d.colors = d.datas = nullptr;
  for (auto& c : d.top_count) c = 0;  // top_keys describe the host mirror, which stays
  d.node_cap = d.brick_cap = d.color_cap = d.data_cap = 0;
  d.valid = false;
  d.ordered = false;
  // the host mirror, the blob and the dirty flags stay: uploading the scene again copies the blob if
  // nothing changed meanwhile, else rebuilds what changed and refills the blob
  return SVO_OK;
}
}  // namespace svo

extern "C" {

svo_status svo_set_device_allocator(svo_alloc_fn alloc, svo_free_fn release, void* user) {
  if ((alloc == nullptr) != (release == nullptr))
    return fail(SVO_ERR_ARGUMENT, "svo_set_device_allocator: give both functions or neither");
  std::lock_guard<std::mutex> lock(g_image_alloc_mutex);
  g_image_alloc = ImageAllocator{alloc, release, user};
  return SVO_OK;
}

svo_status svo_scene_upload(svo_scene* sc, void* stream) {
  TraceRange range("svo_scene_upload");
  if (!sc) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  return full_upload(sc, (cudaStream_t)stream);
}

svo_status svo_scene_sync(svo_scene* sc, void* stream) {
  TraceRange range("svo_scene_sync");
  if (!sc) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  if (!sc->dev.valid) return full_upload(sc, (cudaStream_t)stream);
  return incremental_sync(sc, (cudaStream_t)stream);
}

svo_status svo_scene_release_device(svo_scene* sc) {
  TraceRange range("svo_scene_release_device");
  if (!sc) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  destroy_pipeline(sc->dev);
  free_device(sc->dev);
  destroy_queues(sc->dev);
  std::fill(sc->tree.node_dirty.begin(), sc->tree.node_dirty.end(), 1);
  std::fill(sc->tree.arena.dirty().begin(), sc->tree.arena.dirty().end(), 1);
  return SVO_OK;
}

void svo_scene_destroy(svo_scene* sc) {
  if (!sc) return;
  destroy_pipeline(sc->dev);
  free_device(sc->dev);
  free_blob(sc->dev);
  if (sc->dev.ready) cudaEventDestroy(sc->dev.ready);
  destroy_queues(sc->dev);
  delete sc;
}

svo_status svo_cast_rows(svo_scene* sc, const svo_rays* rays, uint64_t n, uint32_t row_length, const svo_hits* hits,
                         void* stream) {
  TraceRange range("svo_cast");
  if (!sc || !rays || !hits) return fail(SVO_ERR_ARGUMENT, "svo_cast: NULL argument");
  if (!sc->dev.valid) return fail(SVO_ERR_NOT_UPLOADED, "svo_cast: scene has no device image (svo_scene_upload)");
  if (n && (!rays->ox || !rays->oy || !rays->oz || !rays->dx || !rays->dy || !rays->dz))
    return fail(SVO_ERR_ARGUMENT, "svo_cast: NULL ray array");
  return launch_cast(sc, rays, n, hits, (cudaStream_t)stream, row_length);
}

svo_status svo_cast(svo_scene* sc, const svo_rays* rays, uint64_t n, const svo_hits* hits, void* stream) {
  return svo_cast_rows(sc, rays, n, 0, hits, stream);
}

svo_status svo_cast_lod_rows(svo_scene* sc, const svo_rays* rays, uint64_t n, uint32_t row, const svo_hits* hits,
                             float viewing_distance, void* stream) {
  TraceRange range("svo_cast_lod");
  if (!sc || !rays || !hits) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  if (!sc->dev.valid) return fail(SVO_ERR_NOT_UPLOADED, "svo_cast_lod: scene not uploaded");
  if (n == 0) return SVO_OK;
  if (!rays->ox || !rays->oy || !rays->oz || !rays->dx || !rays->dy || !rays->dz)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_lod: NULL ray array");
  const cudaStream_t st = (cudaStream_t)stream;
  // without MIP maps get_by_ray_at_lod is get_by_ray
  if (!sc->tree.mips_enabled) return launch_cast(sc, rays, n, hits, st, row);
  CastQueues* q = sc->dev.queues;
  const SceneView v = scene_view(sc);
  const RaysView rv{rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz};
  const HitsView hv = hits_view_of(*hits);
  const bool count = counts_requested(*hits);
  std::lock_guard<std::mutex> lock(q->m);
  unsigned long long* ctr = queue_counter(q, st);
  if (!ctr) {
    const uint64_t blocks = (n + 127) / 128;
    if (blocks > 0x7FFFFFFFull) return fail(SVO_ERR_ARGUMENT, "svo_cast_lod: too many rays for one launch");
    if (count)
      lod_grid_kernel<true><<<(unsigned)blocks, 128, 0, st>>>(v, rv, hv, n, viewing_distance);
    else
      lod_grid_kernel<false><<<(unsigned)blocks, 128, 0, st>>>(v, rv, hv, n, viewing_distance);
    SVO_CUDA_TRY(cudaGetLastError());
    return SVO_OK;
  }
  static const int per_sm_lod[2] = {  // resident blocks of the two LOD queue kernels
      [] { int v = 0; return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, queue_kernel<false, true>, 128, 0) == cudaSuccess ? v : 1; }(),
      [] { int v = 0; return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, queue_kernel<true, true>, 128, 0) == cudaSuccess ? v : 1; }()};
  const int per_sm = std::max(1, per_sm_lod[count ? 1 : 0]);
  const uint64_t grid = std::min<uint64_t>((uint64_t)q->sm_count * per_sm, (n + 127) / 128);
  SVO_CUDA_TRY(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), st));
  const ClaimOrder order = claim_order(n, row);
  if (count)
    queue_kernel<true, true><<<(unsigned)grid, 128, 0, st>>>(v, rv, hv, n, order, ctr, viewing_distance);
  else
    queue_kernel<false, true><<<(unsigned)grid, 128, 0, st>>>(v, rv, hv, n, order, ctr, viewing_distance);
  SVO_CUDA_TRY(cudaGetLastError());
  return SVO_OK;
}

svo_status svo_cast_lod(svo_scene* sc, const svo_rays* rays, uint64_t n, const svo_hits* hits, float viewing_distance,
                        void* stream) {
  return svo_cast_lod_rows(sc, rays, n, 0, hits, viewing_distance, stream);
}

svo_status svo_cast_host_rows(svo_scene* sc, const svo_rays* rays, uint64_t n, uint32_t row_length,
                              const svo_hits* hits, void* stream) {
  TraceRange range("svo_cast_host");
  if (!sc || !rays || !hits) return fail(SVO_ERR_ARGUMENT, "svo_cast_host: NULL argument");
  if (!sc->dev.valid) return fail(SVO_ERR_NOT_UPLOADED, "svo_cast_host: scene has no device image");
  if (n == 0) return SVO_OK;
  if (!rays->ox || !rays->oy || !rays->oz || !rays->dx || !rays->dy || !rays->dz)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_host: NULL ray array");
  const cudaStream_t st = (cudaStream_t)stream;
  // Where the device reads host memory through the CPU's page tables (Grace: NVLink-C2C with
  // address translation), the kernel reads the rays and writes the hits in place; elsewhere the
  // batch goes through staged copies.
  // By default only batches with a row layout (camera images) are read in place: the work queue
  // casts the rays that enter the octree out of order (packed into full warps), and where many rays
  // miss the octree their hits would reach host memory in small scattered pieces.
  int direct = 0;
  if (g_host_transfer != 1) {
    int dev = 0;
    SVO_CUDA_TRY(cudaGetDevice(&dev));
    SVO_CUDA_TRY(cudaDeviceGetAttribute(&direct, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
    if (g_host_transfer == 2 && !direct)
      return fail(SVO_ERR_ARGUMENT, "svo_cast_host: this device cannot access host memory directly");
    if (g_host_transfer == 0 && row_length < 16) direct = 0;
  }
  if (!direct) return cast_host_pipelined(sc, rays, n, hits, st, row_length);
  const svo_status rc = launch_cast(sc, rays, n, hits, st, row_length, true);
  if (rc != SVO_OK) return rc;
  SVO_CUDA_TRY(cudaStreamSynchronize(st));
  return SVO_OK;
}

svo_status svo_cast_host(svo_scene* sc, const svo_rays* rays, uint64_t n, const svo_hits* hits, void* stream) {
  return svo_cast_host_rows(sc, rays, n, 0, hits, stream);
}

svo_status svo_set_host_transfer(int32_t mode) {
  if (mode < 0 || mode > 3) return fail(SVO_ERR_ARGUMENT, "svo_set_host_transfer: mode must be 0, 1, 2 or 3");
  g_host_transfer = mode == 3 ? 2 : mode;
  g_pair_rows = mode == 3 ? 0 : 1;
  return SVO_OK;
}

svo_status svo_set_refill(int32_t park_below) {
  if (park_below < 0 || park_below > 32) return fail(SVO_ERR_ARGUMENT, "svo_set_refill: park_below must be 0..32");
  g_refill_below = park_below;
  return SVO_OK;
}

svo_status svo_set_staging_depth(int32_t depth) {
  if (depth < 0 || depth > (int32_t)kMaxStageDepth)
    return fail(SVO_ERR_ARGUMENT, "svo_set_staging_depth: depth must be 0.." + std::to_string(kMaxStageDepth));
  g_stage_depth = depth;
  return SVO_OK;
}

svo_status svo_set_cast_mode(int32_t mode) {
  if (mode != 0 && mode != 1) return fail(SVO_ERR_ARGUMENT, "svo_set_cast_mode: mode must be 0 or 1");
  g_cast_mode = mode;
  return SVO_OK;
}

// Runs the device-side look-up-table arithmetic and copies the tables back
// (RAY_TO_NODE_OCCUPANCY_BITMASK_LUT [64][8], OCTANT_STEP_RESULT_LUT [3][3][3],
// BITMAP_MASK_FOR_OCTANT_LUT [8]) so tests can compare them with the reference.
svo_status svo_selftest_luts(uint64_t* ray_to_node, uint32_t* octant_step, uint64_t* octant_masks) {
  if (!ray_to_node || !octant_step || !octant_masks) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  uint64_t *d_rtn = nullptr, *d_mask = nullptr;
  uint32_t* d_step = nullptr;
  SVO_CUDA_TRY(cudaMalloc(&d_rtn, 512 * 8));
  SVO_CUDA_TRY(cudaMalloc(&d_mask, 8 * 8));
  SVO_CUDA_TRY(cudaMalloc(&d_step, 27 * 4));
  lut_kernel<<<1, 512>>>(d_rtn, d_step, d_mask);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(ray_to_node, d_rtn, 512 * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(octant_step, d_step, 27 * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(octant_masks, d_mask, 8 * 8, cudaMemcpyDeviceToHost);
  cudaFree(d_rtn);
  cudaFree(d_mask);
  cudaFree(d_step);
  if (e != cudaSuccess) return fail(SVO_ERR_CUDA, std::string("svo_selftest_luts: ") + cudaGetErrorString(e));
  return SVO_OK;
}

}  // extern "C"
