// svo_server.cu -- serving loop: continuous batching of camera requests over
// resident scenes.
//
// One worker thread owns the device side.  Each iteration it retires launches
// whose completion event has fired (results are then in the callers' host
// buffers), and, while a launch slot is free, admits the oldest pending
// requests into a new launch: scenes the batch needs are made resident under
// the device-memory budget (least recently used idle scenes are evicted),
// rays are generated on the device (bit for bit what svo_gen_camera_rays
// computes on the host), all requests of the batch are cast by one persistent
// batched launch, and each request's requested fields are copied back.  Up to
// max_inflight launches run at once on separate streams, so requests arriving
// while others are on the GPU start as soon as a slot frees up and overlap the
// work already running.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "svo_cast.cuh"
#include "svo_trace.h"

namespace svo {
namespace {

#define SRV_CUDA(call)                                                                            \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) {                                                                      \
      set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                             \
      return e_ == cudaErrorMemoryAllocation ? SVO_ERR_OUT_OF_MEMORY : SVO_ERR_CUDA;              \
    }                                                                                             \
  } while (0)


struct CamParams {
  float ex, ey, ez;
  float fx, fy, fz, rx, ry, rz;
  float tan_half, aspect;
  uint32_t width, height;
};

// The per-pixel part of svo_gen_camera_rays, same operations in the same order.
__global__ void camera_rays_kernel(CamParams c, float* ox, float* oy, float* oz, float* dx, float* dy, float* dz) {
  const uint64_t n = (uint64_t)c.width * c.height;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t px = (uint32_t)(i % c.width), py = (uint32_t)(i / c.width);
    const float u = (2.0f * ((float)px + 0.5f) / (float)c.width - 1.0f) * c.tan_half * c.aspect;
    const float v = (1.0f - 2.0f * ((float)py + 0.5f) / (float)c.height) * c.tan_half;
    // add(add(fwd, mul(right, u)), mul(up, v)) with up = (0, 1, 0)
    const float ax = c.fx + c.rx * u, ay = c.fy + c.ry * u, az = c.fz + c.rz * u;
    const float vx = ax + 0.0f * v, vy = ay + 1.0f * v, vz = az + 0.0f * v;
    const float l = sqrtf((vx * vx + vy * vy) + vz * vz);
    ox[i] = c.ex;
    oy[i] = c.ey;
    oz[i] = c.ez;
    dx[i] = vx / l;
    dy[i] = vy / l;
    dz[i] = vz / l;
  }
}

double now_s() {
  using namespace std::chrono;
  return duration_cast<duration<double>>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  svo_request r;
  uint64_t id = 0, n = 0;
  int32_t status = SVO_OK;
  double t_submit = 0, t_start = 0, t_done = 0;
  uint32_t batch_n = 0;
  bool done = false;
};

struct SceneSlot {
  svo_scene* scene = nullptr;
  uint64_t last_used = 0;
  int users = 0;  // launches in flight that read it
};

struct LaunchSlot {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  svo_batch_workspace* ws = nullptr;
  char* buf = nullptr;
  size_t bytes = 0;
  bool busy = false;
  std::vector<Request*> reqs;
  std::vector<uint32_t> scenes;
};

}  // namespace
}  // namespace svo

// Locking: `mu` guards the request queue, the request table, `stats` and the
// scene count.  Launch slots, scene residency bookkeeping (last_used, users)
// and every CUDA call belong to the worker thread alone, which drops the lock
// while it launches so that submissions never wait for a launch.
struct svo_server {
  static constexpr size_t kMaxScenes = 4096;  // scene slots never move: the vector is reserved once
  svo_server_config cfg{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<svo::Request*> pending;
  std::unordered_map<uint64_t, svo::Request*> requests;
  std::vector<svo::SceneSlot> scenes;
  std::vector<svo::LaunchSlot> slots;
  uint64_t next_id = 1, tick = 0;
  svo_server_stats stats{};
  bool stop = false;
  std::thread worker;
};

namespace svo {
namespace {

struct LaunchCounts {
  uint64_t uploads = 0, evictions = 0, launches = 0;
};

uint64_t resident_bytes(const svo_server* sv, size_t n_scenes) {
  uint64_t b = 0;
  for (size_t j = 0; j < n_scenes; ++j) b += device_image_bytes(sv->scenes[j].scene);
  return b;
}

// Makes every scene of the batch resident, evicting idle least-recently-used ones above the budget.
svo_status make_resident(svo_server* sv, const std::vector<uint32_t>& need, size_t n_scenes, cudaStream_t st,
                         LaunchCounts& cnt) {
  TraceRange range("svo_server residency");
  for (uint32_t id : need) {
    SceneSlot& sc = sv->scenes[id];
    sc.last_used = ++sv->tick;
    if (sc.scene->dev.valid) continue;
    const uint64_t want = device_image_bytes_estimate(sc.scene);
    while (resident_bytes(sv, n_scenes) + want > sv->cfg.budget_bytes) {
      int victim = -1;
      for (size_t j = 0; j < n_scenes; ++j) {
        const SceneSlot& c = sv->scenes[j];
        if (!c.scene->dev.valid || c.users > 0) continue;
        if (std::find(need.begin(), need.end(), (uint32_t)j) != need.end()) continue;
        if (victim < 0 || c.last_used < sv->scenes[victim].last_used) victim = (int)j;
      }
      if (victim < 0) break;  // nothing idle left to evict: admit over budget rather than deadlock
      // the victim's last launch has retired: its image goes back to the pool in stream order
      svo_status rc = evict_ordered(sv->scenes[victim].scene, st);
      if (rc != SVO_OK) return rc;
      cnt.evictions++;
    }
    svo_status rc = upload_ordered(sc.scene, st);
    if (rc != SVO_OK) return rc;
    cnt.uploads++;
  }
  return SVO_OK;
}

// Evicts idle least-recently-used scenes while the resident images exceed the budget: an admission
// goes over it when every resident scene is in use, and this brings residency back as launches
// retire.  `st` is a stream with nothing in flight (a retired launch's).
svo_status trim_residency(svo_server* sv, size_t n_scenes, cudaStream_t st, LaunchCounts& cnt) {
  while (resident_bytes(sv, n_scenes) > sv->cfg.budget_bytes) {
    int victim = -1;
    for (size_t j = 0; j < n_scenes; ++j) {
      const SceneSlot& c = sv->scenes[j];
      if (!c.scene->dev.valid || c.users > 0) continue;
      if (victim < 0 || c.last_used < sv->scenes[victim].last_used) victim = (int)j;
    }
    if (victim < 0) break;
    svo_status rc = evict_ordered(sv->scenes[victim].scene, st);
    if (rc != SVO_OK) return rc;
    cnt.evictions++;
  }
  return SVO_OK;
}

svo_status launch(svo_server* sv, LaunchSlot& ls, size_t n_scenes, LaunchCounts& cnt) {
  TraceRange range("svo_server launch");
  uint64_t total = 0;
  size_t need = 0;
  for (Request* q : ls.reqs) {
    total += q->n;
    need += ((q->n * 24 + 255) / 256) * 256 + 6 * 256;
    void* const* hf = reinterpret_cast<void* const*>(&q->r.hits);
    for (int f = 0; f < kHitFields; ++f)
      if (hf[f]) need += ((kHitFieldBytes[f] * q->n + 255) / 256) * 256;
  }
  if (need > ls.bytes) {
    SRV_CUDA(cudaStreamSynchronize(ls.st));
    cudaFree(ls.buf);
    ls.buf = nullptr;
    ls.bytes = 0;
    SRV_CUDA(cudaMalloc(&ls.buf, need));
    ls.bytes = need;
  }
  svo_status rc = make_resident(sv, ls.scenes, n_scenes, ls.st, cnt);
  if (rc != SVO_OK) return rc;
  // a scene uploaded for another slot may still be in its copies on that slot's stream
  for (uint32_t id : ls.scenes) {
    const cudaEvent_t ready = sv->scenes[id].scene->dev.ready;
    if (ready) SRV_CUDA(cudaStreamWaitEvent(ls.st, ready, 0));
  }
  std::vector<svo_batch_item> items(ls.reqs.size());
  size_t o = 0;
  for (size_t i = 0; i < ls.reqs.size(); ++i) {
    Request* q = ls.reqs[i];
    float* r[6];
    for (int a = 0; a < 6; ++a) {
      r[a] = reinterpret_cast<float*>(ls.buf + o);
      o += ((q->n * 4 + 255) / 256) * 256;
    }
    CameraFrame f;
    camera_frame(q->r.eye, q->r.target, q->r.fov_deg, q->r.width, q->r.height, &f);
    CamParams c{q->r.eye[0], q->r.eye[1], q->r.eye[2], f.fwd[0], f.fwd[1], f.fwd[2], f.right[0], f.right[1],
                f.right[2], f.tan_half, f.aspect, q->r.width, q->r.height};
    const unsigned blocks = (unsigned)std::min<uint64_t>((q->n + 255) / 256, 4096);
    camera_rays_kernel<<<blocks, 256, 0, ls.st>>>(c, r[0], r[1], r[2], r[3], r[4], r[5]);
    SRV_CUDA(cudaGetLastError());
    svo_batch_item& it = items[i];
    std::memset(&it, 0, sizeof(it));
    it.scene = sv->scenes[q->r.scene_id].scene;
    it.rays = svo_rays{r[0], r[1], r[2], r[3], r[4], r[5]};
    it.n = q->n;
    it.row_length = q->r.width;  // camera rays in raster order
    void* const* hf = reinterpret_cast<void* const*>(&q->r.hits);
    void** df = reinterpret_cast<void**>(&it.hits);
    for (int fi = 0; fi < kHitFields; ++fi)
      if (hf[fi]) {
        df[fi] = ls.buf + o;
        o += ((kHitFieldBytes[fi] * q->n + 255) / 256) * 256;
      }
  }
  rc = svo_cast_batched(ls.ws, items.data(), (uint32_t)items.size(), &sv->cfg.launch, ls.st);
  if (rc != SVO_OK) return rc;
  for (size_t i = 0; i < ls.reqs.size(); ++i) {
    Request* q = ls.reqs[i];
    void* const* hf = reinterpret_cast<void* const*>(&q->r.hits);
    void** df = reinterpret_cast<void**>(&items[i].hits);
    for (int f = 0; f < kHitFields; ++f)
      if (hf[f]) SRV_CUDA(cudaMemcpyAsync(hf[f], df[f], kHitFieldBytes[f] * q->n, cudaMemcpyDeviceToHost, ls.st));
  }
  SRV_CUDA(cudaEventRecord(ls.done, ls.st));
  cnt.launches++;
  return SVO_OK;
}

void worker_main(svo_server* sv) {
  cudaSetDevice(sv->device);
  std::unique_lock<std::mutex> lk(sv->mu);
  for (;;) {
    bool progressed = false;
    // retire finished launches
    cudaStream_t idle_stream = nullptr;
    for (LaunchSlot& ls : sv->slots) {
      if (!ls.busy) continue;
      const cudaError_t e = cudaEventQuery(ls.done);
      if (e == cudaErrorNotReady) continue;
      idle_stream = ls.st;
      TraceRange range("svo_server retire");
      const double t = now_s();
      if (e != cudaSuccess) {  // the launch failed on the device: its requests fail, none waits forever
        set_error(std::string("svo_server: launch failed: ") + cudaGetErrorString(e));
        idle_stream = nullptr;
      }
      for (Request* q : ls.reqs) {
        q->t_done = t;
        q->done = true;
        if (e != cudaSuccess) {
          q->status = SVO_ERR_CUDA;
          continue;
        }
        sv->stats.requests_done++;
        sv->stats.rays_done += q->n;
      }
      for (uint32_t id : ls.scenes) sv->scenes[id].users--;
      ls.reqs.clear();
      ls.scenes.clear();
      ls.busy = false;
      progressed = true;
      sv->cv_done.notify_all();
    }
    if (idle_stream) {  // scenes admitted over the budget while all were in use leave as they go idle
      const size_t n_scenes = sv->scenes.size();
      LaunchCounts cnt;
      lk.unlock();
      trim_residency(sv, n_scenes, idle_stream, cnt);
      lk.lock();
      sv->stats.evictions += cnt.evictions;
    }
    // admit pending requests into free launch slots
    for (LaunchSlot& ls : sv->slots) {
      if (ls.busy || sv->pending.empty()) continue;
      uint64_t rays = 0;
      while (!sv->pending.empty() && ls.reqs.size() < sv->cfg.max_batch_requests) {
        Request* q = sv->pending.front();
        if (!ls.reqs.empty() && rays + q->n > sv->cfg.max_batch_rays) break;
        sv->pending.pop_front();
        ls.reqs.push_back(q);
        rays += q->n;
        if (std::find(ls.scenes.begin(), ls.scenes.end(), q->r.scene_id) == ls.scenes.end())
          ls.scenes.push_back(q->r.scene_id);
      }
      const double t = now_s();
      for (Request* q : ls.reqs) {
        q->t_start = t;
        q->batch_n = (uint32_t)ls.reqs.size();
      }
      for (uint32_t id : ls.scenes) sv->scenes[id].users++;
      const size_t n_scenes = sv->scenes.size();
      LaunchCounts cnt;
      lk.unlock();
      svo_status rc = launch(sv, ls, n_scenes, cnt);
      lk.lock();
      sv->stats.uploads += cnt.uploads;
      sv->stats.evictions += cnt.evictions;
      sv->stats.launches += cnt.launches;
      if (rc != SVO_OK) {  // the launch failed: fail its requests, keep serving
        cudaStreamSynchronize(ls.st);
        for (Request* q : ls.reqs) {
          q->status = rc;
          q->t_done = now_s();
          q->done = true;
        }
        for (uint32_t id : ls.scenes) sv->scenes[id].users--;
        ls.reqs.clear();
        ls.scenes.clear();
        sv->cv_done.notify_all();
      } else {
        ls.busy = true;
      }
      progressed = true;
    }
    bool any_busy = false;
    for (const LaunchSlot& ls : sv->slots) any_busy |= ls.busy;
    if (sv->stop && sv->pending.empty() && !any_busy) break;
    if (progressed) continue;
    if (any_busy)
      sv->cv_work.wait_for(lk, std::chrono::microseconds(50));
    else
      sv->cv_work.wait(lk, [&] { return sv->stop || !sv->pending.empty(); });
  }
}

}  // namespace
}  // namespace svo

using namespace svo;

extern "C" {

svo_status svo_server_create(const svo_server_config* cfg, svo_server** out) {
  if (!cfg || !out) return fail(SVO_ERR_ARGUMENT, "svo_server_create: NULL argument");
  *out = nullptr;
  svo_server_config c = *cfg;
  if (c.max_batch_requests == 0) c.max_batch_requests = 64;
  if (c.max_batch_requests > 128) return fail(SVO_ERR_ARGUMENT, "svo_server_create: max_batch_requests > 128");
  if (c.max_batch_rays == 0) c.max_batch_rays = 1u << 25;
  if (c.max_inflight == 0) c.max_inflight = 2;
  if (c.max_inflight > 4) return fail(SVO_ERR_ARGUMENT, "svo_server_create: max_inflight > 4");
  if (c.budget_bytes == 0) c.budget_bytes = 60ull << 30;
  svo_server* sv = new svo_server();
  sv->cfg = c;
  sv->scenes.reserve(svo_server::kMaxScenes);
  cudaGetDevice(&sv->device);
  sv->slots.resize(c.max_inflight);
  for (LaunchSlot& ls : sv->slots) {
    cudaError_t e = cudaStreamCreateWithFlags(&ls.st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ls.done, cudaEventDisableTiming);
    svo_status rc = e == cudaSuccess ? svo_batch_workspace_create(&ls.ws)
                                     : fail(SVO_ERR_CUDA, std::string("svo_server_create: ") + cudaGetErrorString(e));
    if (rc != SVO_OK) {
      svo_server_destroy(sv);
      return rc;
    }
  }
  sv->worker = std::thread(worker_main, sv);
  *out = sv;
  return SVO_OK;
}

void svo_server_destroy(svo_server* sv) {
  if (!sv) return;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  if (sv->worker.joinable()) sv->worker.join();
  for (LaunchSlot& ls : sv->slots) {
    if (ls.st) cudaStreamSynchronize(ls.st);
    cudaFree(ls.buf);
    if (ls.ws) svo_batch_workspace_destroy(ls.ws);
    if (ls.done) cudaEventDestroy(ls.done);
    if (ls.st) cudaStreamDestroy(ls.st);
  }
  for (auto& kv : sv->requests) delete kv.second;
  delete sv;
}

svo_status svo_server_add_scene(svo_server* sv, svo_scene* scene, uint32_t* scene_id) {
  if (!sv || !scene || !scene_id) return fail(SVO_ERR_ARGUMENT, "svo_server_add_scene: NULL argument");
  std::lock_guard<std::mutex> lk(sv->mu);
  if (sv->scenes.size() >= svo_server::kMaxScenes) return fail(SVO_ERR_ARGUMENT, "svo_server_add_scene: too many scenes");
  SceneSlot s;
  s.scene = scene;
  sv->scenes.push_back(s);
  *scene_id = (uint32_t)(sv->scenes.size() - 1);
  return SVO_OK;
}

svo_status svo_server_submit(svo_server* sv, const svo_request* r, uint64_t* request_id) {
  if (!sv || !r || !request_id) return fail(SVO_ERR_ARGUMENT, "svo_server_submit: NULL argument");
  if (r->width == 0 || r->height == 0) return fail(SVO_ERR_ARGUMENT, "svo_server_submit: empty image");
  Request* q = new Request();
  q->r = *r;
  q->n = (uint64_t)r->width * r->height;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (r->scene_id >= sv->scenes.size()) {
      delete q;
      return fail(SVO_ERR_NOT_FOUND, "svo_server_submit: unknown scene id");
    }
    q->id = sv->next_id++;
    q->t_submit = now_s();
    sv->requests[q->id] = q;
    sv->pending.push_back(q);
    *request_id = q->id;
  }
  sv->cv_work.notify_one();
  return SVO_OK;
}

svo_status svo_server_wait(svo_server* sv, uint64_t request_id, double timeout_s, svo_request_result* out) {
  if (!sv) return fail(SVO_ERR_ARGUMENT, "svo_server_wait: NULL server");
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->requests.find(request_id);
  if (it == sv->requests.end()) return fail(SVO_ERR_NOT_FOUND, "svo_server_wait: unknown request id");
  Request* q = it->second;
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
  if (!sv->cv_done.wait_until(lk, deadline, [&] { return q->done; }))
    return fail(SVO_ERR_BUSY, "svo_server_wait: request not complete before the timeout");
  if (out) {
    out->status = q->status;
    out->submit_s = q->t_submit;
    out->start_s = q->t_start;
    out->done_s = q->t_done;
    out->batch_requests = q->batch_n;
  }
  sv->requests.erase(it);
  const int32_t st = q->status;
  delete q;
  if (st != SVO_OK) return fail(st, "svo_server_wait: the request failed");
  return SVO_OK;
}

svo_status svo_server_stats_get(svo_server* sv, svo_server_stats* out) {
  if (!sv || !out) return fail(SVO_ERR_ARGUMENT, "svo_server_stats_get: NULL argument");
  std::lock_guard<std::mutex> lk(sv->mu);
  *out = sv->stats;
  // device images change only on the worker thread between launches: a racy read here is only a snapshot
  out->resident_bytes = resident_bytes(sv, sv->scenes.size());
  return SVO_OK;
}

double svo_server_now(svo_server* sv) { return now_s(); }

}  // extern "C"
