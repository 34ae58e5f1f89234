// svo_queue.h -- the per-stream work counters of a scene, shared by the queued cast
// (svo_device.cu) and the fused render (svo_render.cu).
//
// A queued kernel's warps claim work from a counter that starts at 0.  Launches on one stream run
// one after another, so a stream can reuse its counter (zeroed on the stream before each launch);
// launches on different streams may overlap, so every stream that uses the scene gets a counter
// of its own.  The zeroing and the launch are enqueued together under the mutex, so two host
// threads sharing a stream cannot interleave them.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "svo_internal.h"

namespace svo {

constexpr uint32_t kQueueSlots = 64;

struct CastQueues {
  std::mutex m;
  cudaStream_t streams[kQueueSlots] = {};
  uint32_t used = 0;
  unsigned long long* counters = nullptr;  // kQueueSlots device words
  int sm_count = 0, blocks_per_sm = 0, blocks_per_sm_count = 0;
};

// The counter of stream `st` (claimed on first use), or nullptr when the scene has none for it:
// all slots taken, or the per-thread default stream, which names a different stream in every
// host thread.  Call with q->m held.
inline unsigned long long* queue_counter(CastQueues* q, cudaStream_t st) {
  if (!q || st == cudaStreamPerThread) return nullptr;
  uint32_t slot = 0;
  while (slot < q->used && q->streams[slot] != st) ++slot;
  if (slot == q->used) {
    if (q->used == kQueueSlots) return nullptr;
    q->streams[q->used++] = st;
  }
  return q->counters + slot;
}

}  // namespace svo
