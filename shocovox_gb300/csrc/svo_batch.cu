// svo_batch.cu -- batched multi-scene cast: one persistent launch over many
// (scene, ray batch) items.
//
// Work distribution: the claims of all items form one global index space
// (item prefix sums; an item spans 32 indices per claim of its ClaimOrder, so
// an item of camera rays with a row length is cast in 8 x 4 ray blocks).  Each
// warp repeatedly claims `rays_per_chunk` consecutive indices from a device
// work counter with one atomicAdd, maps every lane's index to its item by
// binary search over the prefix sums held in shared memory, and casts with the
// shared per-ray restatement of Octree::get_by_ray (svo_cast.cuh).  Items of
// different octree sizes and brick dimensions mix freely; a ray's result does
// not depend on which warp or launch casts it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "svo_cast.cuh"
#include "svo_refill.cuh"
#include "svo_trace.h"

namespace svo {

struct BatchItemDev {
  SceneView scene;
  RaysView rays;
  HitsView hits;
  ClaimOrder order;  // the item's rays by claim and lane
  uint64_t begin;    // first global index of the item (a multiple of 32)
  uint64_t n;
  const DevNode* stage_src;  // the first item of each staged scene: its top table, which blocks copy
  uint32_t stage_off;        // the scene's staged records in the block's copy: [stage_off, + stage_n)
  uint32_t stage_n;          // 0: the scene's nodes are read from L1/L2
};

constexpr uint32_t kBatchStageRecords = 768;  // 48 KB of staged records per block at most

// Shares the staged records out among the scenes of a call, in order of first appearance, at staging
// depth `depth` while they fit kBatchStageRecords; returns the records a block copies.
inline uint32_t assign_staging(BatchItemDev* table, const svo_batch_item* items, uint32_t n_items, uint32_t depth) {
  uint32_t total = 0;
  for (uint32_t i = 0; i < n_items; ++i) {
    table[i].stage_src = nullptr;
    table[i].stage_off = 0;
    table[i].stage_n = 0;
  }
  if (depth == 0) return 0;
  for (uint32_t i = 0; i < n_items; ++i) {
    uint32_t first = i;
    for (uint32_t j = 0; j < i; ++j)
      if (items[j].scene == items[i].scene) {
        first = j;
        break;
      }
    if (first < i) {  // a later item of a scene seen before: the same staged records
      table[i].stage_off = table[first].stage_off;
      table[i].stage_n = table[first].stage_n;
      continue;
    }
    const uint32_t n = table[i].scene.literal ? 0u : staged_records(items[i].scene, depth);
    if (n == 0 || total + n > kBatchStageRecords) continue;
    table[i].stage_src = table[i].scene.top;
    table[i].stage_off = total;
    table[i].stage_n = n;
    total += n;
  }
  return total;
}

// The staged records of every scene of the table into the block's shared-memory copy.
__device__ __forceinline__ void stage_items(DevNode* stg, const BatchItemDev* items, uint32_t n_items) {
  for (uint32_t i = 0; i < n_items; ++i) {
    const DevNode* src = items[i].stage_src;
    if (src) stage_records(stg + items[i].stage_off, src, items[i].stage_n);
  }
}

// fills the device form of one item at global index `begin`; returns the indices it spans
// (none when the item's rays are cast through the ray sort instead: `claimed` false)
uint64_t item_dev(const svo_batch_item& it, uint64_t begin, uint32_t shape, BatchItemDev& d, bool claimed = true) {
  d.scene = scene_view(it.scene);
  d.rays = RaysView{it.rays.ox, it.rays.oy, it.rays.oz, it.rays.dx, it.rays.dy, it.rays.dz};
  d.hits = hits_view_of(it.hits);
  d.n = claimed ? it.n : 0;
  d.order = claim_order(d.n, it.row_length, shape);
  d.begin = begin;
  return 32 * d.order.claims;
}

constexpr uint32_t kMaxSharedItems = 256;  // prefix sums staged in shared memory (the rest read from the table)

// At most kBatchMaxBlock threads per block with 7 resident blocks per SM (72 registers, a few
// spilled bytes); the launch configuration is checked against the block limit.
constexpr uint32_t kBatchMaxBlock = 128;

// Rays that miss their octree's root box get their miss written at once; the entering rays of a
// partly entering round of 32 indices wait in the warp's slice of shared memory (their index, item,
// the point where they enter and its octant) until 32 of them fill the warp; their origin and
// direction are read again when they are cast (less shared memory per block leaves more L1).
struct WaitingBatchRays {
  float p[3][64];
  uint32_t target[64];  // octant of the entry point; bit 31: fast form
  uint32_t item[64];
  unsigned long long i[64];
};

template <bool kCount, bool kStage = false>
__global__ void __launch_bounds__(kBatchMaxBlock, 7)
    batched_kernel(const BatchItemDev* __restrict__ items, uint32_t n_items, uint64_t total,
                   unsigned long long* __restrict__ counter, uint32_t chunk) {
  __shared__ uint64_t s_begin[kMaxSharedItems];
  __shared__ SharedLuts L;
  __shared__ WaitingBatchRays waiting[kBatchMaxBlock / 32];
  extern __shared__ uint4 staged_smem[];
  DevNode* stg = reinterpret_cast<DevNode*>(staged_smem);
  const uint32_t staged = n_items < kMaxSharedItems ? n_items : kMaxSharedItems;
  for (uint32_t i = threadIdx.x; i < staged; i += blockDim.x) s_begin[i] = items[i].begin;
  fill_shared_luts(L);
  if (kStage) stage_items(stg, items, n_items);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  WaitingBatchRays& w = waiting[threadIdx.x >> 5];
  uint32_t count = 0;                 // rays waiting (the same in every lane)
  bool more = true;                   // chunks left
  unsigned long long base = 0;        // the warp's chunk
  uint32_t next = chunk;              // offset of the next round of 32 indices in it
  for (;;) {
    bool have = false, fast = false, waited = false;
    uint64_t i = 0;
    uint32_t item = 0, target = 0;
    float ox = 0.0f, oy = 0.0f, oz = 0.0f, dx = 0.0f, dy = 0.0f, dz = 0.0f, px = 0.0f, py = 0.0f, pz = 0.0f;
    while (count < 32) {
      if (next >= chunk) {
        if (!more) break;
        if (lane == 0) base = atomicAdd(counter, (unsigned long long)chunk);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= total) {
          more = false;
          break;
        }
        next = 0;
      }
      const uint64_t g = base + next + lane;
      const bool in_chunk = next + lane < chunk;
      next += 32;
      bool enters = false;
      if (in_chunk && g < total) {
        // largest item with begin <= g (items are sorted by begin)
        uint32_t lo = 0, hi = n_items - 1;
        while (lo < hi) {
          const uint32_t mid = (lo + hi + 1) >> 1;
          const uint64_t b = mid < kMaxSharedItems ? s_begin[mid] : items[mid].begin;
          if (b <= g)
            lo = mid;
          else
            hi = mid - 1;
        }
        const BatchItemDev& it = items[lo];
        const uint64_t x = g - it.begin;  // an empty item shares its begin with the next one
        const uint64_t j =
            x < 32 * it.order.claims ? claimed_ray(it.order, x >> 5, (uint32_t)(x & 31u), it.n) : it.n;
        if (j < it.n) {
          const RaysView& r = it.rays;
          ox = __ldg(r.ox + j);
          oy = __ldg(r.oy + j);
          oz = __ldg(r.oz + j);
          dx = __ldg(r.dx + j);
          dy = __ldg(r.dy + j);
          dz = __ldg(r.dz + j);
          fast = !it.scene.literal && !isnan(dx) && !isnan(dy) && !isnan(dz);
          enters = !fast || fast_entry(it.scene, ox, oy, oz, dx, dy, dz, px, py, pz, target);
          if (!enters) {
            HitRecord h;
            miss_record(h);
            write_hit(it.scene, it.hits, j, h);
            if (kCount) write_counters(it.hits, j, h);
          }
          i = j;
          item = lo;
        }
      }
      const unsigned m = __ballot_sync(0xFFFFFFFFu, enters);
      if (m == 0xFFFFFFFFu && count == 0) {  // a full round: cast in place
        have = true;
        break;
      }
      if (enters) {
        const uint32_t k = count + __popc(m & ((1u << lane) - 1u));
        w.p[0][k] = px;
        w.p[1][k] = py;
        w.p[2][k] = pz;
        w.target[k] = target | (fast ? 0x80000000u : 0u);
        w.item[k] = item;
        w.i[k] = i;
      }
      count += __popc(m);
      __syncwarp();
    }
    if (!have) {
      if (count == 0) break;  // no chunks left and nothing waiting
      const uint32_t take = count < 32 ? count : 32;
      if (lane < take) {
        const uint32_t k = count - take + lane;
        px = w.p[0][k];
        py = w.p[1][k];
        pz = w.p[2][k];
        target = w.target[k] & 0x7FFFFFFFu;
        fast = (w.target[k] >> 31) != 0u;
        item = w.item[k];
        i = w.i[k];
        have = true;
        waited = true;
      }
      count -= take;
      __syncwarp();
    }
    if (!have) continue;
    const BatchItemDev& it = items[item];
    if (waited) {  // origin and direction again from the item's arrays
      const RaysView& r = it.rays;
      ox = __ldg(r.ox + i);
      oy = __ldg(r.oy + i);
      oz = __ldg(r.oz + i);
      dx = __ldg(r.dx + i);
      dy = __ldg(r.dy + i);
      dz = __ldg(r.dz + i);
    }
    HitRecord h;
    cast_entered<kCount, false, kStage>(it.scene, L, ox, oy, oz, dx, dy, dz, fast, px, py, pz, target, h, 0.0f,
                                        stg + it.stage_off, it.stage_n);
    write_hit(it.scene, it.hits, i, h);
    if (kCount) write_counters(it.hits, i, h);
  }
}

// ---- ray sort (svo_launch_config.sort_key = 1) -------------------------------------------------
//
// The rays of the items without a row length (rays in no particular order, such as rays from random
// points in random directions) are cast in the order of a key instead of their index order, so that
// a warp's 32 rays start near one another and head the same way and walk much the same nodes:
//   1. bin_kernel: a ray that misses its octree's root box gets its miss written at once; an entering
//      ray gets its bucket (item, octant of its direction, Morton code of its entry point at `bits`
//      bits an axis), counted into the bucket's count, and is appended, with the point where it
//      enters, to an unsorted list;
//   2. the bucket counts are turned into bucket offsets (exclusive scan: scan_reduce, scan_top,
//      scan_down);
//   3. scatter_kernel moves every listed ray to the next free place of its bucket (atomicAdd on the
//      bucket's offset);
//   4. sorted_cast_kernel casts the sorted list, warps claiming `rays_per_chunk` rays at a time.
// The order of the rays inside a bucket depends on the atomics' order; a ray's result does not.
struct SortItemDev {
  uint64_t begin;         // first index of the item in the sort's index space (plain order)
  uint64_t n;             // the item's rays in it (0: the item is cast in claim order)
  uint32_t bucket_base;   // first bucket of the item
  uint32_t bits;          // bits of the entry point's Morton code per axis
};

// One entering ray of the sort, 64 bytes (four 16-byte pieces).
struct __align__(16) SortedRay {
  float o[3], d[3], p[3];
  uint32_t target;  // octant of the entry point; bit 31: fast form
  uint32_t item;
  uint32_t bucket;
  uint32_t pad[2];
  unsigned long long i;  // ray index in the item
};
static_assert(sizeof(SortedRay) == 64, "SortedRay is four 16-byte pieces");
// the kernels read a SortedRay as four float4 (a, b, c, d): o = a.xyz, d = (a.w, b.x, b.y),
// p = (b.z, b.w, c.x), target = c.y, item = c.z, bucket = c.w, i = d.zw
static_assert(offsetof(SortedRay, d) == 12 && offsetof(SortedRay, p) == 24 && offsetof(SortedRay, target) == 36 &&
                  offsetof(SortedRay, item) == 40 && offsetof(SortedRay, bucket) == 44 && offsetof(SortedRay, i) == 56,
              "SortedRay layout");

// bits of the entry point's Morton code per axis for an item of n rays: about 16 rays a bucket
inline uint32_t sort_bits(uint64_t n) {
  uint32_t len = 0;
  while (len < 64 && (n >> len)) ++len;
  const int b = ((int)len - 7) / 3;
  return (uint32_t)std::min(std::max(b, 0), 6);
}

__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // bit k of v to bit 3k (v < 2^7)
  uint32_t r = 0;
#pragma unroll
  for (int k = 0; k < 7; ++k) r |= ((v >> k) & 1u) << (3 * k);
  return r;
}

constexpr uint32_t kSortBlock = 256;

// The one sorted item of a call whose sort holds a single item: its views ride in the kernel
// parameters (read from the constant bank) instead of the item table in global memory.
struct OneItem {
  SceneView scene;
  RaysView rays;
  HitsView hits;
  SortItemDev sort;
  uint32_t index;
};

// Ray j of an item (origin o, direction d): its miss written at once (a miss is written for an
// entering ray too, until the cast overwrites it), and for an entering ray its record (with its
// bucket) in r.
template <bool kCount>
__device__ __forceinline__ bool bin_ray(const SceneView& sc, const HitsView& hv, const SortItemDev& si,
                                        uint32_t item, uint64_t j, const float (&o)[3], const float (&d)[3],
                                        SortedRay& r) {
  const float ox = o[0], oy = o[1], oz = o[2], dx = d[0], dy = d[1], dz = d[2];
  const bool fast = !sc.literal && !isnan(dx) && !isnan(dy) && !isnan(dz);
  float px = ox, py = oy, pz = oz;
  uint32_t target = 0;
  const bool enters = !fast || fast_entry(sc, ox, oy, oz, dx, dy, dz, px, py, pz, target);
  // every lane writes a miss, the entering rays' ones to be overwritten by the cast: whole sectors of
  // the hit arrays are written at once instead of sectors with holes that DRAM must read back
  HitRecord h;
  miss_record(h);
  write_hit(sc, hv, j, h);
  if (kCount) write_counters(hv, j, h);
  if (!enters) return false;
  // the key: only an order, so any rounding will do (a literal ray keys on its origin)
  const uint32_t q = 1u << si.bits;
  const float scale = (float)q * sc.inv_size;
  const uint32_t qx = (uint32_t)fminf(fmaxf(px * scale, 0.0f), (float)(q - 1));
  const uint32_t qy = (uint32_t)fminf(fmaxf(py * scale, 0.0f), (float)(q - 1));
  const uint32_t qz = (uint32_t)fminf(fmaxf(pz * scale, 0.0f), (float)(q - 1));
  const uint32_t oct = (uint32_t)(dx >= 0.0f) | ((uint32_t)(dy >= 0.0f) << 1) | ((uint32_t)(dz >= 0.0f) << 2);
  r.o[0] = ox;
  r.o[1] = oy;
  r.o[2] = oz;
  r.d[0] = dx;
  r.d[1] = dy;
  r.d[2] = dz;
  r.p[0] = px;
  r.p[1] = py;
  r.p[2] = pz;
  r.target = target | (fast ? 0x80000000u : 0u);
  r.item = item;
  r.bucket = si.bucket_base + (oct << (3 * si.bits)) + (spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2));
  r.pad[0] = r.pad[1] = 0;
  r.i = j;
  return true;
}

constexpr uint32_t kBinRays = 2;  // rays per lane per round of the binning

template <bool kCount, bool kOne>
__global__ void __launch_bounds__(kSortBlock)
    bin_kernel(const BatchItemDev* __restrict__ items, const SortItemDev* __restrict__ sort, uint32_t n_items,
               uint64_t total, uint32_t* __restrict__ hist, SortedRay* __restrict__ list,
               unsigned long long* __restrict__ n_list, const OneItem one) {
  __shared__ uint64_t s_begin[kMaxSharedItems];
  if (!kOne) {
    const uint32_t staged = n_items < kMaxSharedItems ? n_items : kMaxSharedItems;
    for (uint32_t i = threadIdx.x; i < staged; i += blockDim.x) s_begin[i] = sort[i].begin;
    __syncthreads();
  }
  // each warp bins kBinRays rays per round, its loads issued before any of them is binned
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * kBinRays;
  for (uint64_t g0 = ((uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) * kBinRays; g0 < total; g0 += stride) {
    float o[kBinRays][3], d[kBinRays][3];
    uint64_t jj[kBinRays];
    uint32_t at[kBinRays];
#pragma unroll
    for (uint32_t u = 0; u < kBinRays; ++u) {
      const uint64_t g = g0 + 32 * u + lane;
      at[u] = 0xFFFFFFFFu;  // no ray
      jj[u] = 0;
      if (g < total) {
        if (kOne) {
          const uint64_t j = g - one.sort.begin;
          if (j < one.sort.n) {
            at[u] = one.index;
            jj[u] = j;
          }
        } else {
          uint32_t lo = 0, hi = n_items - 1;  // the item: largest with begin <= g
          while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            const uint64_t b = mid < kMaxSharedItems ? s_begin[mid] : sort[mid].begin;
            if (b <= g)
              lo = mid;
            else
              hi = mid - 1;
          }
          const uint64_t j = g - sort[lo].begin;  // an empty item shares its begin with the next one
          if (j < sort[lo].n) {
            at[u] = lo;
            jj[u] = j;
          }
        }
      }
      if (at[u] != 0xFFFFFFFFu) {
        const RaysView& rv = kOne ? one.rays : items[at[u]].rays;
        const uint64_t j = jj[u];
        o[u][0] = __ldg(rv.ox + j);
        o[u][1] = __ldg(rv.oy + j);
        o[u][2] = __ldg(rv.oz + j);
        d[u][0] = __ldg(rv.dx + j);
        d[u][1] = __ldg(rv.dy + j);
        d[u][2] = __ldg(rv.dz + j);
      }
    }
    bool enters[kBinRays];
    SortedRay r[kBinRays];
#pragma unroll
    for (uint32_t u = 0; u < kBinRays; ++u) {
      enters[u] = false;
      if (at[u] != 0xFFFFFFFFu) {
        if (kOne)
          enters[u] = bin_ray<kCount>(one.scene, one.hits, one.sort, at[u], jj[u], o[u], d[u], r[u]);
        else
          enters[u] = bin_ray<kCount>(items[at[u]].scene, items[at[u]].hits, sort[at[u]], at[u], jj[u], o[u], d[u], r[u]);
      }
      if (enters[u]) atomicAdd(hist + r[u].bucket, 1u);  // a reduction: nothing waits for it
    }
    unsigned m[kBinRays];
    uint32_t entering = 0;
#pragma unroll
    for (uint32_t u = 0; u < kBinRays; ++u) {
      m[u] = __ballot_sync(0xFFFFFFFFu, enters[u]);
      entering += __popc(m[u]);
    }
    if (entering == 0) continue;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(n_list, (unsigned long long)entering);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
#pragma unroll
    for (uint32_t u = 0; u < kBinRays; ++u) {
      if (enters[u]) {
        float4* dst = reinterpret_cast<float4*>(list + base + __popc(m[u] & ((1u << lane) - 1u)));
        const float4* src = reinterpret_cast<const float4*>(&r[u]);
#pragma unroll
        for (int k = 0; k < 4; ++k) dst[k] = src[k];
      }
      base += __popc(m[u]);
    }
  }
}

// Exclusive scan of the bucket counts in place, kScanTile counts per block.
constexpr uint32_t kScanTile = 4096;
constexpr uint32_t kScanPerThread = kScanTile / kSortBlock;  // 16

// exclusive prefix of v over the block's threads; *block_sum gets the total
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* warp_sums, uint32_t* block_sum) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const uint32_t nw = blockDim.x >> 5;
    uint32_t w = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= (uint32_t)o) w += y;
    }
    if (lane < nw) warp_sums[lane] = w;  // inclusive
  }
  __syncthreads();
  const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
  *block_sum = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();  // warp_sums is reused by the next call
  return before + x - v;
}

__global__ void __launch_bounds__(kSortBlock) scan_reduce(const uint32_t* __restrict__ hist, uint64_t nb,
                                                          uint32_t* __restrict__ sums) {
  __shared__ uint32_t warp_sums[32];
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  uint32_t v = 0;
  for (uint32_t k = 0; k < kScanPerThread; ++k) {
    const uint64_t b = base + k * kSortBlock + threadIdx.x;
    if (b < nb) v += hist[b];
  }
  uint32_t total = 0;
  block_exclusive(v, warp_sums, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) scan_top(uint32_t* __restrict__ sums, uint32_t n) {
  __shared__ uint32_t warp_sums[32];
  uint32_t carry = 0;
  for (uint32_t b0 = 0; b0 < n; b0 += blockDim.x) {
    const uint32_t b = b0 + threadIdx.x;
    const uint32_t v = b < n ? sums[b] : 0u;
    uint32_t total = 0;
    const uint32_t ex = block_exclusive(v, warp_sums, &total);
    if (b < n) sums[b] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(kSortBlock) scan_down(uint32_t* __restrict__ hist, uint64_t nb,
                                                        const uint32_t* __restrict__ sums) {
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t tile[kScanTile];
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  for (uint32_t k = 0; k < kScanPerThread; ++k) {
    const uint32_t t = k * kSortBlock + threadIdx.x;
    tile[t] = base + t < nb ? hist[base + t] : 0u;
  }
  __syncthreads();
  uint32_t v = 0;
  for (uint32_t k = 0; k < kScanPerThread; ++k) v += tile[threadIdx.x * kScanPerThread + k];
  uint32_t total = 0;
  uint32_t run = sums[blockIdx.x] + block_exclusive(v, warp_sums, &total);
  for (uint32_t k = 0; k < kScanPerThread; ++k) {
    const uint32_t t = threadIdx.x * kScanPerThread + k;
    const uint32_t c = tile[t];
    tile[t] = run;
    run += c;
  }
  __syncthreads();
  for (uint32_t k = 0; k < kScanPerThread; ++k) {
    const uint32_t t = k * kSortBlock + threadIdx.x;
    if (base + t < nb) hist[base + t] = tile[t];
  }
}

__global__ void __launch_bounds__(kSortBlock)
    scatter_kernel(const SortedRay* __restrict__ list, const unsigned long long* __restrict__ n_list,
                   uint32_t* __restrict__ offsets, SortedRay* __restrict__ sorted) {
  const uint64_t n = *n_list;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
    const float4* src = reinterpret_cast<const float4*>(list + k);
    const float4 a = __ldg(src), b = __ldg(src + 1), c = __ldg(src + 2), d = __ldg(src + 3);
    const uint32_t bucket = __float_as_uint(c.w);  // SortedRay::bucket
    float4* dst = reinterpret_cast<float4*>(sorted + atomicAdd(offsets + bucket, 1u));
    dst[0] = a;
    dst[1] = b;
    dst[2] = c;
    dst[3] = d;
  }
}

template <bool kCount, bool kOne, bool kStage = false>
__global__ void __launch_bounds__(kBatchMaxBlock, 7)
    sorted_cast_kernel(const BatchItemDev* __restrict__ items, const SortedRay* __restrict__ sorted,
                       const unsigned long long* __restrict__ n_list, unsigned long long* __restrict__ counter,
                       uint32_t chunk, const SceneView one_scene, const HitsView one_hits, uint32_t n_items,
                       uint32_t one_stage_n) {
  __shared__ SharedLuts L;
  extern __shared__ uint4 staged_smem[];
  DevNode* stg = reinterpret_cast<DevNode*>(staged_smem);
  fill_shared_luts(L);
  if (kStage) {
    if (kOne)
      stage_records(stg, one_scene.top, one_stage_n);
    else
      stage_items(stg, items, n_items);
  }
  __syncthreads();
  const uint64_t n = *n_list;
  const uint32_t lane = threadIdx.x & 31u;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(counter, (unsigned long long)chunk);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (base >= n) break;
    for (uint32_t off = 0; off < chunk; off += 32) {
      const uint64_t k = base + off + lane;
      if (off + lane >= chunk || k >= n) continue;
      const float4* src = reinterpret_cast<const float4*>(sorted + k);
      const float4 a = __ldg(src), b = __ldg(src + 1), c = __ldg(src + 2), d = __ldg(src + 3);
      const uint32_t target = __float_as_uint(c.y);
      const uint64_t i = (uint64_t)__float_as_uint(d.z) | ((uint64_t)__float_as_uint(d.w) << 32);
      const bool fast = (target >> 31) != 0u;
      HitRecord h;
      if (kOne) {
        cast_entered<kCount, false, kStage>(one_scene, L, a.x, a.y, a.z, a.w, b.x, b.y, fast, b.z, b.w, c.x,
                                            target & 0x7FFFFFFFu, h, 0.0f, stg, one_stage_n);
        write_hit(one_scene, one_hits, i, h);
        if (kCount) write_counters(one_hits, i, h);
      } else {
        const BatchItemDev& it = items[__float_as_uint(c.z)];
        cast_entered<kCount, false, kStage>(it.scene, L, a.x, a.y, a.z, a.w, b.x, b.y, fast, b.z, b.w, c.x,
                                            target & 0x7FFFFFFFu, h, 0.0f, stg + it.stage_off, it.stage_n);
        write_hit(it.scene, it.hits, i, h);
        if (kCount) write_counters(it.hits, i, h);
      }
    }
  }
}

// The sorted cast with lane refill (svo_launch_config.refill_below): a warp parks its rays at a node
// visit once fewer than park_below are in flight (refill_kernel, svo_device.cu) and its idle lanes
// take the next sorted records, claimed exactly as many as there are idle lanes, so the list's order
// (neighbouring entry points, one direction octant) carries over into the refilled warp.
template <bool kCount, bool kOne, bool kStage = false>
__global__ void __launch_bounds__(kBatchMaxBlock, 7)
    sorted_refill_kernel(const BatchItemDev* __restrict__ items, const SortedRay* __restrict__ sorted,
                         const unsigned long long* __restrict__ n_list, unsigned long long* __restrict__ counter,
                         const SceneView one_scene, const HitsView one_hits, uint32_t n_items, uint32_t one_stage_n,
                         uint32_t park_below) {
  __shared__ SharedLuts L;
  __shared__ uint32_t in_flight[kBatchMaxBlock / 32];
  __shared__ FastState parked[kBatchMaxBlock];  // a thread's ray between runs (23 words: no bank conflicts)
  extern __shared__ uint4 staged_smem[];
  DevNode* stg = reinterpret_cast<DevNode*>(staged_smem);
  fill_shared_luts(L);
  if (kStage) {
    if (kOne)
      stage_records(stg, one_scene.top, one_stage_n);
    else
      stage_items(stg, items, n_items);
  }
  __syncthreads();
  const uint64_t n = *n_list;
  const uint32_t lane = threadIdx.x & 31u;
  volatile uint32_t* live = in_flight + (threadIdx.x >> 5);
  uint32_t park = park_below;
  bool more = true, alive = false;
  uint64_t i = 0;    // the ray's index in its item
  uint32_t item = 0;
  for (;;) {
    const unsigned idle = __ballot_sync(0xFFFFFFFFu, !alive);
    const uint32_t need = __popc(idle);
    if (need && more) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(counter, (unsigned long long)need);
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base + need >= n) more = false;
      if (!alive) {
        const uint64_t k = base + __popc(idle & ((1u << lane) - 1u));
        if (k < n) {
          const float4* src = reinterpret_cast<const float4*>(sorted + k);
          const float4 a = __ldg(src), b = __ldg(src + 1), c = __ldg(src + 2), d = __ldg(src + 3);
          const uint32_t target = __float_as_uint(c.y);
          i = (uint64_t)__float_as_uint(d.z) | ((uint64_t)__float_as_uint(d.w) << 32);
          item = kOne ? 0u : __float_as_uint(c.z);
          if ((target >> 31) == 0u) {  // a NaN direction (or literal mode): the literal form, in one go
            HitRecord h;
            const SceneView& sc = kOne ? one_scene : items[item].scene;
            const HitsView& hv = kOne ? one_hits : items[item].hits;
            cast_entered<kCount>(sc, L, a.x, a.y, a.z, a.w, b.x, b.y, false, b.z, b.w, c.x, 0u, h);
            write_hit(sc, hv, i, h);
            if (kCount) write_counters(hv, i, h);
          } else {
            fast_start(parked[threadIdx.x], a.w, b.x, b.y, b.z, b.w, c.x, target & 0x7FFFFFFFu);
            alive = true;
          }
        }
      }
      if (!more) park = 0;  // nothing left to hand out: rays in flight run to their end
      __syncwarp();
      const unsigned now = __ballot_sync(0xFFFFFFFFu, alive);
      if (lane == 0) *live = __popc(now);
      __syncwarp();
      if (now == 0) continue;
    } else if (!__any_sync(0xFFFFFFFFu, alive)) {
      break;
    }
    if (alive) {
      HitRecord h;
      if (kOne) {
        if (fast_run<kCount, kStage>(parked + threadIdx.x, one_scene, L, h, live, park, stg, one_stage_n)) {
          write_hit(one_scene, one_hits, i, h);
          if (kCount) write_counters(one_hits, i, h);
          alive = false;
        }
      } else {
        const BatchItemDev& it = items[item];
        if (fast_run<kCount, kStage>(parked + threadIdx.x, it.scene, L, h, live, park, stg + it.stage_off,
                                     it.stage_n)) {
          write_hit(it.scene, it.hits, i, h);
          if (kCount) write_counters(it.hits, i, h);
          alive = false;
        }
      }
    }
    __syncwarp();
  }
}

}  // namespace svo

namespace svo {
// The claim-order persistent launch of a prepared item table (device copy at d_items), with
// staged_n records of the call's top tables staged by every block.
svo_status launch_claimed(const BatchItemDev* d_items, uint32_t n_items, uint64_t total,
                          unsigned long long* d_counter, uint32_t chunk, uint32_t block, const svo_launch_config* cfg,
                          bool count, uint32_t staged_n, int sm_count, cudaStream_t st) {
  const size_t smem = (size_t)staged_n * sizeof(DevNode);
  auto kern = staged_n ? (count ? batched_kernel<true, true> : batched_kernel<false, true>)
                       : (count ? batched_kernel<true> : batched_kernel<false>);
  SVO_CUDA_TRY(allow_dynamic_smem(kern, smem));
  int per_sm = (cfg && cfg->blocks_per_sm) ? (int)cfg->blocks_per_sm : 0;
  if (per_sm == 0) {
    SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem));
    per_sm = std::max(per_sm, 1);
  }
  const uint64_t warps_needed = (total + chunk - 1) / chunk;
  uint64_t grid = (uint64_t)sm_count * (uint64_t)per_sm;
  grid = std::min<uint64_t>(grid, (warps_needed * 32 + block - 1) / block);
  grid = std::max<uint64_t>(grid, 1);
  SVO_CUDA_TRY(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st));
  kern<<<(unsigned)grid, block, smem, st>>>(d_items, n_items, total, d_counter, chunk);
  SVO_CUDA_TRY(cudaGetLastError());
  return SVO_OK;
}
}  // namespace svo

// Workspace of the batched cast: device item table + work counter, and a
// pinned host staging copy of the table.  Grows only when the item count grows.
struct svo_batch_workspace {
  svo::BatchItemDev* d_items = nullptr;
  unsigned long long* d_counter = nullptr;  // [0] work counter, [1] length of the ray sort's list
  svo::BatchItemDev* h_items = nullptr;     // pinned
  svo::SortItemDev* d_sort = nullptr;       // the ray sort's item table
  svo::SortItemDev* h_sort = nullptr;       // pinned
  cudaEvent_t copied = nullptr;             // the last table upload has left h_items and h_sort
  uint32_t cap = 0;
  int sm_count = 0;
  // ray sort buffers (sort_key 1), grown on demand
  uint32_t* d_hist = nullptr;  // bucket counts, then bucket offsets
  uint32_t* d_sums = nullptr;  // per scan tile
  uint64_t hist_cap = 0;
  svo::SortedRay* d_list = nullptr;    // entering rays as binned
  svo::SortedRay* d_sorted = nullptr;  // entering rays in bucket order
  uint64_t list_cap = 0;
};

using namespace svo;

extern "C" {

svo_status svo_batch_workspace_create(svo_batch_workspace** out) {
  if (!out) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  svo_batch_workspace* ws = new svo_batch_workspace();
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ws->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMalloc(&ws->d_counter, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ws->copied, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    cudaFree(ws->d_counter);
    if (ws->copied) cudaEventDestroy(ws->copied);
    delete ws;
    return fail(SVO_ERR_CUDA, std::string("svo_batch_workspace_create: ") + cudaGetErrorString(e));
  }
  *out = ws;
  return SVO_OK;
}

void svo_batch_workspace_destroy(svo_batch_workspace* ws) {
  if (!ws) return;
  cudaFree(ws->d_items);
  cudaFree(ws->d_counter);
  cudaFreeHost(ws->h_items);
  cudaFree(ws->d_sort);
  cudaFreeHost(ws->h_sort);
  cudaFree(ws->d_hist);
  cudaFree(ws->d_sums);
  cudaFree(ws->d_list);
  cudaFree(ws->d_sorted);
  if (ws->copied) cudaEventDestroy(ws->copied);
  delete ws;
}

svo_status svo_cast_batched(svo_batch_workspace* ws, const svo_batch_item* items, uint32_t n_items,
                            const svo_launch_config* cfg, void* stream) {
  TraceRange range("svo_cast_batched");
  if (!ws || (!items && n_items)) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: NULL argument");
  if (n_items == 0) return SVO_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
  SVO_CUDA_TRY(cudaStreamIsCapturing(st, &capturing));
  const bool in_capture = capturing != cudaStreamCaptureStatusNone;
  if (n_items > ws->cap) {
    if (in_capture) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: workspace must be sized before stream capture");
    // the previous table may still be read by an in-flight launch on this stream
    SVO_CUDA_TRY(cudaStreamSynchronize(st));
    cudaFree(ws->d_items);
    cudaFreeHost(ws->h_items);
    cudaFree(ws->d_sort);
    cudaFreeHost(ws->h_sort);
    ws->d_items = nullptr;
    ws->h_items = nullptr;
    ws->d_sort = nullptr;
    ws->h_sort = nullptr;
    ws->cap = 0;
    const uint32_t cap = std::max<uint32_t>(n_items, 16);
    SVO_CUDA_TRY(cudaMalloc(&ws->d_items, cap * sizeof(BatchItemDev)));
    SVO_CUDA_TRY(cudaMallocHost(&ws->h_items, cap * sizeof(BatchItemDev)));
    SVO_CUDA_TRY(cudaMalloc(&ws->d_sort, cap * sizeof(SortItemDev)));
    SVO_CUDA_TRY(cudaMallocHost(&ws->h_sort, cap * sizeof(SortItemDev)));
    ws->cap = cap;
  } else if (!in_capture) {
    // the pinned staging tables are reused: wait until their previous upload has left them
    SVO_CUDA_TRY(cudaEventSynchronize(ws->copied));
  }
  const uint32_t shape = (cfg && cfg->block_shape) ? cfg->block_shape : 3;
  if (shape < 3 || shape > 5) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: block_shape must be 0, 3, 4 or 5");
  const uint32_t sort_key = cfg ? cfg->sort_key : 0;
  if (sort_key > 1) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: sort_key must be 0 or 1");
  const uint32_t depth = cfg ? cfg->staging_depth : 0;
  if (depth > kMaxStageDepth)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: staging_depth must be 0.." + std::to_string(kMaxStageDepth));
  const uint32_t refill = cfg ? cfg->refill_below : 0;
  if (refill > 32) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: refill_below must be 0..32");
  uint64_t total = 0, sort_total = 0, buckets = 0;
  bool count = false;
  for (uint32_t i = 0; i < n_items; ++i) {
    const svo_batch_item& it = items[i];
    if (!it.scene) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: NULL scene");
    if (!it.scene->dev.valid) return fail(SVO_ERR_NOT_UPLOADED, "svo_cast_batched: scene not uploaded");
    if (it.n && (!it.rays.ox || !it.rays.oy || !it.rays.oz || !it.rays.dx || !it.rays.dy || !it.rays.dz))
      return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: NULL ray array");
    const bool sorted = sort_key == 1 && it.row_length == 0 && it.n > 0;
    total += item_dev(it, total, shape, ws->h_items[i], !sorted);
    SortItemDev& si = ws->h_sort[i];
    si.begin = sort_total;
    si.n = sorted ? it.n : 0;
    si.bits = sorted ? sort_bits(it.n) : 0;
    si.bucket_base = (uint32_t)buckets;
    if (sorted) {
      sort_total += it.n;
      buckets += 8ull << (3 * si.bits);
    }
    count |= counts_requested(it.hits);
  }
  if (total == 0 && sort_total == 0) return SVO_OK;
  if (sort_total >= (1ull << 32) || buckets >= (1ull << 32))
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: the ray sort takes fewer than 2^32 rays per call");
  const uint32_t staged_n = assign_staging(ws->h_items, items, n_items, depth);
  const size_t stage_smem = (size_t)staged_n * sizeof(DevNode);
  const uint32_t block = (cfg && cfg->block) ? cfg->block : 128;
  const uint32_t chunk = (cfg && cfg->rays_per_chunk) ? cfg->rays_per_chunk : 64;
  if (block % 32 != 0 || block > kBatchMaxBlock || chunk == 0)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: block must be a multiple of 32 and at most 128");
  if (sort_total > ws->list_cap || buckets > ws->hist_cap) {
    if (in_capture)
      return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: the ray sort's buffers must be sized before stream capture");
    SVO_CUDA_TRY(cudaStreamSynchronize(st));
    if (sort_total > ws->list_cap) {
      cudaFree(ws->d_list);
      cudaFree(ws->d_sorted);
      ws->d_list = ws->d_sorted = nullptr;
      ws->list_cap = 0;
      SVO_CUDA_TRY(cudaMalloc(&ws->d_list, sort_total * sizeof(SortedRay)));
      SVO_CUDA_TRY(cudaMalloc(&ws->d_sorted, sort_total * sizeof(SortedRay)));
      ws->list_cap = sort_total;
    }
    if (buckets > ws->hist_cap) {
      cudaFree(ws->d_hist);
      cudaFree(ws->d_sums);
      ws->d_hist = ws->d_sums = nullptr;
      ws->hist_cap = 0;
      SVO_CUDA_TRY(cudaMalloc(&ws->d_hist, buckets * sizeof(uint32_t)));
      SVO_CUDA_TRY(cudaMalloc(&ws->d_sums, (buckets / kScanTile + 1) * sizeof(uint32_t)));
      ws->hist_cap = buckets;
    }
  }
  // a single sorted item rides in the kernel parameters
  uint32_t n_sorted = 0;
  OneItem one{};
  for (uint32_t i = 0; i < n_items; ++i)
    if (ws->h_sort[i].n) {
      if (n_sorted++ == 0) {
        one.scene = ws->h_items[i].scene;
        one.rays = ws->h_items[i].rays;
        one.hits = ws->h_items[i].hits;
        one.sort = ws->h_sort[i];
        one.index = i;
      }
    }
  const bool single = n_sorted == 1;
  // the tables are read by the claim-order kernel and by the sort's kernels of several items
  if (total > 0 || (sort_total > 0 && !single))
    SVO_CUDA_TRY(cudaMemcpyAsync(ws->d_items, ws->h_items, n_items * sizeof(BatchItemDev), cudaMemcpyHostToDevice, st));
  if (sort_total > 0 && !single)
    SVO_CUDA_TRY(cudaMemcpyAsync(ws->d_sort, ws->h_sort, n_items * sizeof(SortItemDev), cudaMemcpyHostToDevice, st));
  if (!in_capture) SVO_CUDA_TRY(cudaEventRecord(ws->copied, st));
  if (sort_total) {
    unsigned long long* n_list = ws->d_counter + 1;
    SVO_CUDA_TRY(cudaMemsetAsync(ws->d_counter, 0, 2 * sizeof(unsigned long long), st));
    SVO_CUDA_TRY(cudaMemsetAsync(ws->d_hist, 0, buckets * sizeof(uint32_t), st));
    int bin_per_sm = 0;
    SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &bin_per_sm, single ? (count ? bin_kernel<true, true> : bin_kernel<false, true>)
                            : (count ? bin_kernel<true, false> : bin_kernel<false, false>),
        kSortBlock, 0));
    const uint64_t fill = (uint64_t)ws->sm_count * (uint64_t)std::max(bin_per_sm, 1);
    const unsigned bin_grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(fill, (sort_total + kSortBlock - 1) / kSortBlock));
    auto bin = single ? (count ? bin_kernel<true, true> : bin_kernel<false, true>)
                      : (count ? bin_kernel<true, false> : bin_kernel<false, false>);
    bin<<<bin_grid, kSortBlock, 0, st>>>(ws->d_items, ws->d_sort, n_items, sort_total, ws->d_hist, ws->d_list, n_list, one);
    const uint32_t tiles = (uint32_t)((buckets + kScanTile - 1) / kScanTile);
    scan_reduce<<<tiles, kSortBlock, 0, st>>>(ws->d_hist, buckets, ws->d_sums);
    scan_top<<<1, 1024, 0, st>>>(ws->d_sums, tiles);
    scan_down<<<tiles, kSortBlock, 0, st>>>(ws->d_hist, buckets, ws->d_sums);
    scatter_kernel<<<bin_grid, kSortBlock, 0, st>>>(ws->d_list, n_list, ws->d_hist, ws->d_sorted);
    // the one sorted item's staged records sit at the start of the block's copy
    const uint32_t one_stage = single ? ws->h_items[one.index].stage_n : 0u;
    const bool stage = single ? one_stage > 0 : staged_n > 0;
    const size_t smem = single ? (size_t)one_stage * sizeof(DevNode) : stage_smem;
    if (refill) {
      auto rk = stage ? (single ? (count ? sorted_refill_kernel<true, true, true> : sorted_refill_kernel<false, true, true>)
                                : (count ? sorted_refill_kernel<true, false, true> : sorted_refill_kernel<false, false, true>))
                      : (single ? (count ? sorted_refill_kernel<true, true> : sorted_refill_kernel<false, true>)
                                : (count ? sorted_refill_kernel<true, false> : sorted_refill_kernel<false, false>));
      SVO_CUDA_TRY(allow_dynamic_smem(rk, smem));
      int per_sm = (cfg && cfg->blocks_per_sm) ? (int)cfg->blocks_per_sm : 0;
      if (per_sm == 0) {
        SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rk, block, smem));
        per_sm = std::max(per_sm, 1);
      }
      uint64_t grid = (uint64_t)ws->sm_count * (uint64_t)per_sm;
      grid = std::max<uint64_t>(1, std::min<uint64_t>(grid, (sort_total + block - 1) / block));
      rk<<<(unsigned)grid, block, smem, st>>>(ws->d_items, ws->d_sorted, n_list, ws->d_counter, one.scene, one.hits,
                                               n_items, one_stage, refill);
      SVO_CUDA_TRY(cudaGetLastError());
    } else {
    auto cast = stage ? (single ? (count ? sorted_cast_kernel<true, true, true> : sorted_cast_kernel<false, true, true>)
                                : (count ? sorted_cast_kernel<true, false, true> : sorted_cast_kernel<false, false, true>))
                      : (single ? (count ? sorted_cast_kernel<true, true> : sorted_cast_kernel<false, true>)
                                : (count ? sorted_cast_kernel<true, false> : sorted_cast_kernel<false, false>));
    SVO_CUDA_TRY(allow_dynamic_smem(cast, smem));
    int per_sm = (cfg && cfg->blocks_per_sm) ? (int)cfg->blocks_per_sm : 0;
    if (per_sm == 0) {
      SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cast, block, smem));
      per_sm = std::max(per_sm, 1);
    }
    const uint64_t warps_needed = (sort_total + chunk - 1) / chunk;
    uint64_t grid = (uint64_t)ws->sm_count * (uint64_t)per_sm;
    grid = std::max<uint64_t>(1, std::min<uint64_t>(grid, (warps_needed * 32 + block - 1) / block));
    cast<<<(unsigned)grid, block, smem, st>>>(ws->d_items, ws->d_sorted, n_list, ws->d_counter, chunk, one.scene,
                                               one.hits, n_items, one_stage);
    SVO_CUDA_TRY(cudaGetLastError());
    }
  }
  if (total == 0) return SVO_OK;
  return launch_claimed(ws->d_items, n_items, total, ws->d_counter, chunk, block, cfg, count, staged_n, ws->sm_count, st);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free batched cast.
//
// Some callers of this library cannot allocate device memory at the moment they
// cast: an engine that hands the library a fixed memory budget and forbids
// allocation after start-up, or code running inside a frame loop or a graph of
// its own where a cudaMalloc would synchronise the device.  For them the item
// table and the work counter of the batched cast live in the fixed scratch
// array below instead of an svo_batch_workspace.  The array is reserved on
// every GPU that loads the library, for as long as the process lives.
constexpr uint32_t kNoAllocMaxItems = 128;  // items per call
constexpr size_t kNoAllocTableBytes = kNoAllocMaxItems * sizeof(svo::BatchItemDev);
constexpr size_t kNoAllocCounterOffset = (kNoAllocTableBytes + 255) / 256 * 256;
constexpr size_t kNoAllocBytes = kNoAllocCounterOffset + 256;
static_assert(kNoAllocBytes == 47360, "include/svo.h documents the scratch array's size");
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};
int g_noalloc_sms[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once per device.
svo_status noalloc_scratch(void** out, int* sms) {
  int dev = 0;
  SVO_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: device ordinal too large");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* ptr = nullptr;
    SVO_CUDA_TRY(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    int n = 0;
    SVO_CUDA_TRY(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    g_noalloc_ptr[dev] = ptr;
    g_noalloc_sms[dev] = n;
  }
  *out = g_noalloc_ptr[dev];
  *sms = g_noalloc_sms[dev];
  return SVO_OK;
}
}  // namespace

extern "C" {

svo_status svo_cast_batched_noalloc(const svo_batch_item* items, uint32_t n_items, const svo_launch_config* cfg,
                                    void* stream) {
  TraceRange range("svo_cast_batched_noalloc");
  if (!items && n_items) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: NULL items");
  if (n_items > kNoAllocMaxItems)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: " + std::to_string(n_items) + " items exceed the maximum of " +
                                      std::to_string(kNoAllocMaxItems) + " per call");
  if (n_items == 0) return SVO_OK;
  cudaStream_t st = (cudaStream_t)stream;
  // The item table below is copied from this call's stack frame.  Inside a stream capture the copy
  // would become a graph node that reads that frame again at every replay, long after it is gone, so
  // a capturing stream is refused before anything is enqueued.
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  SVO_CUDA_TRY(cudaStreamIsCapturing(st, &capture));
  if (capture != cudaStreamCaptureStatusNone)
    return fail(SVO_ERR_ARGUMENT,
                "svo_cast_batched_noalloc: the stream is capturing; its item table is copied from the caller's "
                "stack and cannot be replayed (capture svo_cast_batched with a workspace instead)");
  void* scratch = nullptr;
  int sms = 0;
  svo_status rc = noalloc_scratch(&scratch, &sms);
  if (rc != SVO_OK) return rc;
  BatchItemDev table[kNoAllocMaxItems];
  const uint32_t shape = (cfg && cfg->block_shape) ? cfg->block_shape : 3;
  if (shape < 3 || shape > 5)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: block_shape must be 0, 3, 4 or 5");
  if (cfg && cfg->sort_key)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: the ray sort (sort_key) needs a batch workspace");
  uint64_t total = 0;
  bool count = false;
  for (uint32_t i = 0; i < n_items; ++i) {
    const svo_batch_item& it = items[i];
    if (!it.scene) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: NULL scene");
    if (!it.scene->dev.valid) return fail(SVO_ERR_NOT_UPLOADED, "svo_cast_batched_noalloc: scene not uploaded");
    if (it.n && (!it.rays.ox || !it.rays.oy || !it.rays.oz || !it.rays.dx || !it.rays.dy || !it.rays.dz))
      return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: NULL ray array");
    total += item_dev(it, total, shape, table[i]);
    count |= counts_requested(it.hits);
  }
  if (total == 0) return SVO_OK;
  const uint32_t block = (cfg && cfg->block) ? cfg->block : 128;
  const uint32_t chunk = (cfg && cfg->rays_per_chunk) ? cfg->rays_per_chunk : 64;
  if (block % 32 != 0 || block > kBatchMaxBlock || chunk == 0)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: block must be a multiple of 32 and at most 128");
  const uint32_t depth = cfg ? cfg->staging_depth : 0;
  if (depth > kMaxStageDepth)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: staging_depth must be 0.." + std::to_string(kMaxStageDepth));
  const uint32_t staged_n = assign_staging(table, items, n_items, depth);
  BatchItemDev* d_items = static_cast<BatchItemDev*>(scratch);
  unsigned long long* d_counter =
      reinterpret_cast<unsigned long long*>(static_cast<unsigned char*>(scratch) + kNoAllocCounterOffset);
  // the table is copied from this stack frame: a pageable source is staged before cudaMemcpyAsync returns;
  // the counter keeps the previous call's final value and is reset for this launch by launch_claimed
  SVO_CUDA_TRY(cudaMemcpyAsync(d_items, table, n_items * sizeof(BatchItemDev), cudaMemcpyHostToDevice, st));
  return launch_claimed(d_items, n_items, total, d_counter, chunk, block, cfg, count, staged_n, sms, st);
}

}  // extern "C"
