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
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "svo_cast.cuh"

namespace svo {

struct BatchItemDev {
  SceneView scene;
  RaysView rays;
  HitsView hits;
  ClaimOrder order;  // the item's rays by claim and lane
  uint64_t begin;    // first global index of the item (a multiple of 32)
  uint64_t n;
};

// fills the device form of one item at global index `begin`; returns the indices it spans
uint64_t item_dev(const svo_batch_item& it, uint64_t begin, uint32_t shape, BatchItemDev& d) {
  d.scene = scene_view(it.scene);
  d.rays = RaysView{it.rays.ox, it.rays.oy, it.rays.oz, it.rays.dx, it.rays.dy, it.rays.dz};
  d.hits = hits_view_of(it.hits);
  d.order = claim_order(it.n, it.row_length, shape);
  d.begin = begin;
  d.n = it.n;
  return 32 * d.order.claims;
}

constexpr uint32_t kMaxSharedItems = 1024;  // prefix sums staged in shared memory

// At most kBatchMaxBlock threads per block with 7 resident blocks per SM (72 registers, a few
// spilled bytes); the launch configuration is checked against the block limit.
constexpr uint32_t kBatchMaxBlock = 128;

// Rays that miss their octree's root box get their miss written at once; the entering rays of a
// partly entering round of 32 indices wait in the warp's slice of shared memory (with the point where
// they enter and their item) until 32 of them fill the warp.
struct WaitingBatchRays {
  float o[3][64], d[3][64], p[3][64];
  uint32_t target[64];  // octant of the entry point; bit 31: fast form
  uint32_t item[64];
  unsigned long long i[64];
};

template <bool kCount>
__global__ void __launch_bounds__(kBatchMaxBlock, 7)
    batched_kernel(const BatchItemDev* __restrict__ items, uint32_t n_items, uint64_t total,
                   unsigned long long* __restrict__ counter, uint32_t chunk) {
  __shared__ uint64_t s_begin[kMaxSharedItems];
  __shared__ SharedLuts L;
  __shared__ WaitingBatchRays waiting[kBatchMaxBlock / 32];
  const uint32_t staged = n_items < kMaxSharedItems ? n_items : kMaxSharedItems;
  for (uint32_t i = threadIdx.x; i < staged; i += blockDim.x) s_begin[i] = items[i].begin;
  fill_shared_luts(L);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  WaitingBatchRays& w = waiting[threadIdx.x >> 5];
  uint32_t count = 0;                 // rays waiting (the same in every lane)
  bool more = true;                   // chunks left
  unsigned long long base = 0;        // the warp's chunk
  uint32_t next = chunk;              // offset of the next round of 32 indices in it
  for (;;) {
    bool have = false, fast = false;
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
        w.o[0][k] = ox;
        w.o[1][k] = oy;
        w.o[2][k] = oz;
        w.d[0][k] = dx;
        w.d[1][k] = dy;
        w.d[2][k] = dz;
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
        ox = w.o[0][k];
        oy = w.o[1][k];
        oz = w.o[2][k];
        dx = w.d[0][k];
        dy = w.d[1][k];
        dz = w.d[2][k];
        px = w.p[0][k];
        py = w.p[1][k];
        pz = w.p[2][k];
        target = w.target[k] & 0x7FFFFFFFu;
        fast = (w.target[k] >> 31) != 0u;
        item = w.item[k];
        i = w.i[k];
        have = true;
      }
      count -= take;
      __syncwarp();
    }
    if (!have) continue;
    const BatchItemDev& it = items[item];
    HitRecord h;
    cast_entered<kCount>(it.scene, L, ox, oy, oz, dx, dy, dz, fast, px, py, pz, target, h);
    write_hit(it.scene, it.hits, i, h);
    if (kCount) write_counters(it.hits, i, h);
  }
}

}  // namespace svo

// Workspace of the batched cast: device item table + work counter, and a
// pinned host staging copy of the table.  Grows only when the item count grows.
struct svo_batch_workspace {
  svo::BatchItemDev* d_items = nullptr;
  unsigned long long* d_counter = nullptr;
  svo::BatchItemDev* h_items = nullptr;  // pinned
  cudaEvent_t copied = nullptr;           // the last table upload has left h_items
  uint32_t cap = 0;
  int sm_count = 0;
};

using namespace svo;

extern "C" {

svo_status svo_batch_workspace_create(svo_batch_workspace** out) {
  if (!out) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  svo_batch_workspace* ws = new svo_batch_workspace();
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ws->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMalloc(&ws->d_counter, sizeof(unsigned long long));
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
  if (ws->copied) cudaEventDestroy(ws->copied);
  delete ws;
}

svo_status svo_cast_batched(svo_batch_workspace* ws, const svo_batch_item* items, uint32_t n_items,
                            const svo_launch_config* cfg, void* stream) {
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
    ws->d_items = nullptr;
    ws->h_items = nullptr;
    ws->cap = 0;
    const uint32_t cap = std::max<uint32_t>(n_items, 16);
    SVO_CUDA_TRY(cudaMalloc(&ws->d_items, cap * sizeof(BatchItemDev)));
    SVO_CUDA_TRY(cudaMallocHost(&ws->h_items, cap * sizeof(BatchItemDev)));
    ws->cap = cap;
  } else if (!in_capture) {
    // the pinned staging table is reused: wait until its previous upload has left it
    SVO_CUDA_TRY(cudaEventSynchronize(ws->copied));
  }
  const uint32_t shape = (cfg && cfg->block_shape) ? cfg->block_shape : 3;
  if (shape < 3 || shape > 5) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: block_shape must be 0, 3, 4 or 5");
  uint64_t total = 0;
  bool count = false;
  for (uint32_t i = 0; i < n_items; ++i) {
    const svo_batch_item& it = items[i];
    if (!it.scene) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: NULL scene");
    if (!it.scene->dev.valid) return fail(SVO_ERR_NOT_UPLOADED, "svo_cast_batched: scene not uploaded");
    if (it.n && (!it.rays.ox || !it.rays.oy || !it.rays.oz || !it.rays.dx || !it.rays.dy || !it.rays.dz))
      return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: NULL ray array");
    total += item_dev(it, total, shape, ws->h_items[i]);
    count |= counts_requested(it.hits);
  }
  if (total == 0) return SVO_OK;
  const uint32_t block = (cfg && cfg->block) ? cfg->block : 128;
  const uint32_t chunk = (cfg && cfg->rays_per_chunk) ? cfg->rays_per_chunk : 64;
  if (block % 32 != 0 || block > kBatchMaxBlock || chunk == 0)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched: block must be a multiple of 32 and at most 128");
  int per_sm = (cfg && cfg->blocks_per_sm) ? (int)cfg->blocks_per_sm : 0;
  if (per_sm == 0) {
    if (count)
      SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_kernel<true>, block, 0));
    else
      SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_kernel<false>, block, 0));
    per_sm = std::max(per_sm, 1);
  }
  const uint64_t warps_needed = (total + chunk - 1) / chunk;
  uint64_t grid = (uint64_t)ws->sm_count * (uint64_t)per_sm;
  grid = std::min<uint64_t>(grid, (warps_needed * 32 + block - 1) / block);
  grid = std::max<uint64_t>(grid, 1);
  SVO_CUDA_TRY(cudaMemcpyAsync(ws->d_items, ws->h_items, n_items * sizeof(BatchItemDev), cudaMemcpyHostToDevice, st));
  if (!in_capture) SVO_CUDA_TRY(cudaEventRecord(ws->copied, st));
  SVO_CUDA_TRY(cudaMemsetAsync(ws->d_counter, 0, sizeof(unsigned long long), st));
  if (count)
    batched_kernel<true><<<(unsigned)grid, block, 0, st>>>(ws->d_items, n_items, total, ws->d_counter, chunk);
  else
    batched_kernel<false><<<(unsigned)grid, block, 0, st>>>(ws->d_items, n_items, total, ws->d_counter, chunk);
  SVO_CUDA_TRY(cudaGetLastError());
  return SVO_OK;
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
  if (!items && n_items) return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: NULL items");
  if (n_items > kNoAllocMaxItems)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: " + std::to_string(n_items) + " items exceed the maximum of " +
                                      std::to_string(kNoAllocMaxItems) + " per call");
  if (n_items == 0) return SVO_OK;
  void* scratch = nullptr;
  int sms = 0;
  svo_status rc = noalloc_scratch(&scratch, &sms);
  if (rc != SVO_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  BatchItemDev table[kNoAllocMaxItems];
  const uint32_t shape = (cfg && cfg->block_shape) ? cfg->block_shape : 3;
  if (shape < 3 || shape > 5)
    return fail(SVO_ERR_ARGUMENT, "svo_cast_batched_noalloc: block_shape must be 0, 3, 4 or 5");
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
  int per_sm = (cfg && cfg->blocks_per_sm) ? (int)cfg->blocks_per_sm : 0;
  if (per_sm == 0) {
    if (count)
      SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_kernel<true>, block, 0));
    else
      SVO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_kernel<false>, block, 0));
    per_sm = std::max(per_sm, 1);
  }
  const uint64_t warps_needed = (total + chunk - 1) / chunk;
  uint64_t grid = (uint64_t)sms * (uint64_t)per_sm;
  grid = std::min<uint64_t>(grid, (warps_needed * 32 + block - 1) / block);
  grid = std::max<uint64_t>(grid, 1);
  BatchItemDev* d_items = static_cast<BatchItemDev*>(scratch);
  unsigned long long* d_counter =
      reinterpret_cast<unsigned long long*>(static_cast<unsigned char*>(scratch) + kNoAllocCounterOffset);
  // the table is copied from this stack frame: a pageable source is staged before cudaMemcpyAsync returns
  SVO_CUDA_TRY(cudaMemcpyAsync(d_items, table, n_items * sizeof(BatchItemDev), cudaMemcpyHostToDevice, st));
  // the counter keeps the previous call's final value: reset it for this launch
  SVO_CUDA_TRY(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st));
  if (count)
    batched_kernel<true><<<(unsigned)grid, block, 0, st>>>(d_items, n_items, total, d_counter, chunk);
  else
    batched_kernel<false><<<(unsigned)grid, block, 0, st>>>(d_items, n_items, total, d_counter, chunk);
  SVO_CUDA_TRY(cudaGetLastError());
  return SVO_OK;
}

}  // extern "C"
