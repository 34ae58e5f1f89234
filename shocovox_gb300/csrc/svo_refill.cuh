// svo_refill.cuh -- the fast form of the cast as a resumable traversal, for kernels that refill a
// warp's idle lanes while its other rays are still in flight.
//
// Rays in no particular order walk paths of very different lengths (a ray that enters the octree may
// leave after two node visits or walk a hundred), so a warp that casts 32 of them runs at the pace of
// its longest ray and most lanes idle at its end.  Here a ray's whole traversal state lives in a
// FastState the kernel keeps in registers; the traversal can stop ("park") at the top of a node visit
// and later continue from there exactly, because a node visit is a point where the state is complete
// (the position, the node and its bounds, the ring stack, the target octant, the step count).  A warp
// parks its rays when fewer than `park_below` of them are still in flight (a per-warp counter in
// shared memory that every finishing ray decrements, so that all lanes see the same count), hands new
// rays to the idle lanes and resumes.  Parking changes when a ray's steps run, never which steps:
// the results and counters are those of cast_ray_fast_from (svo_cast.cuh), whose operations the
// function below repeats one for one (without the LOD branches, which this form does not serve).
#pragma once

#include "svo_cast.cuh"

namespace svo {

// What a parked ray keeps: the rest (scale factors, direction octant, 1 / node size) is formed again
// from these, exactly, when it resumes.  The counters live here only in the instrumented cast.
struct FastState {
  float dx, dy, dz, px, py, pz;
  float bx, by, bz, bs;  // bounds of the current node
  uint32_t cur, target, s0, s1, s2, s3, count, oct, work;
  uint32_t visits, creads, vreads, runs;
};
static_assert(sizeof(FastState) == 23 * 4, "23 words: an odd stride in shared memory");

// Starts the state of a ray that entered the root at p in its octant `target` (fast_entry).
__device__ __forceinline__ void fast_start(FastState& st, float dx, float dy, float dz, float px, float py, float pz,
                                           uint32_t target) {
  st.dx = dx;
  st.dy = dy;
  st.dz = dz;
  st.px = px;
  st.py = py;
  st.pz = pz;
  st.target = target;
  st.count = 0;  // at the head of the restart loop: the next run starts from the root
  st.work = 0;
  st.visits = st.creads = st.vreads = st.runs = 0;
}

// Runs the ray until it is done (true: `h` holds its record) or parks at a node visit (false) because
// `*live` (rays of the warp still in flight) fell below park_below (0: never park).  A ray that ends
// decrements *live.
// The ray's state stays in its slot `ps` (shared memory) between runs: a run reads it, keeps it in
// registers while the ray moves, and writes back only what changed when the ray parks.
template <bool kCount, bool kStage = false>
__device__ __forceinline__ bool fast_run(FastState* ps, const SceneView& s, const SharedLuts& L, HitRecord& h,
                                         volatile uint32_t* live, uint32_t park_below, const DevNode* stg = nullptr,
                                         uint32_t stg_n = 0) {
  miss_record(h);
  struct {
    uint32_t cur, target, s0, s1, s2, s3, count, oct, work;
  } st = {ps->cur, ps->target, ps->s0, ps->s1, ps->s2, ps->s3, ps->count, ps->oct, ps->work};
  FastRay r;
  r.dx = ps->dx;
  r.dy = ps->dy;
  r.dz = ps->dz;
  r.px = ps->px;
  r.py = ps->py;
  r.pz = ps->pz;
  r.pos = (rsignum(r.dx) > 0.0f ? 1u : 0u) | (rsignum(r.dz) > 0.0f ? 2u : 0u) | (rsignum(r.dy) > 0.0f ? 4u : 0u);
  {  // get_dda_scale_factors (raytracing_on_cpu.rs:99-112); powf(q, 2.) == q * q
    const float a = r.dz / r.dx, b = r.dy / r.dx, c = r.dx / r.dy, d = r.dz / r.dy, e = r.dx / r.dz, f = r.dy / r.dz;
    r.fx = sqrtf((1.0f + a * a) + b * b);
    r.fy = sqrtf((c * c + 1.0f) + d * d);
    r.fz = sqrtf((e * e + 1.0f) + f * f);
  }
  if (kCount) {
    h.visits = ps->visits;
    h.creads = ps->creads;
    h.vreads = ps->vreads;
    h.runs = ps->runs;
  }
  // node bounds: sizes are powers of two, so 1 / size is exact
  Bounds cb{ps->bx, ps->by, ps->bz, ps->bs, st.count ? 1.0f / ps->bs : 0.0f};
  const float g4x = (r.pos & 1u) ? 4.0f : -4.0f, g4y = (r.pos & 4u) ? 4.0f : -4.0f, g4z = (r.pos & 2u) ? 4.0f : -4.0f;
  const uint32_t dir = hash_region(1.0f + r.dx, 1.0f + r.dy, 1.0f + r.dz, 1.0f);
  const uint64_t* rtn = L.ray_to_node + dir;
  const float S = s.size;
  const uint32_t root = (kStage && stg_n) ? kStagedBit : 0u;
  bool done = false;
  for (;;) {
    if (st.count == 0) {  // the head of the restart loop
      if (st.target == kOob) {
        done = true;
        break;
      }
      st.cur = root;
      cb = Bounds{0.0f, 0.0f, 0.0f, S, s.inv_size};
      st.s0 = root;
      st.s1 = st.s2 = st.s3 = 0;
      st.count = 1;
      st.oct = 0;
    }
    while (st.count > 0) {
      if (park_below && *live < park_below) {  // parked at the top of a node visit
        ps->px = r.px;
        ps->py = r.py;
        ps->pz = r.pz;
        ps->bx = cb.x;
        ps->by = cb.y;
        ps->bz = cb.z;
        ps->bs = cb.s;
        ps->cur = st.cur;
        ps->target = st.target;
        ps->s0 = st.s0;
        ps->s1 = st.s1;
        ps->s2 = st.s2;
        ps->s3 = st.s3;
        ps->count = st.count;
        ps->oct = st.oct;
        ps->work = st.work;
        if (kCount) {
          ps->visits = h.visits;
          ps->creads = h.creads;
          ps->vreads = h.vreads;
          ps->runs = h.runs;
        }
        return false;
      }
      if (++st.work > kWorkCap) {
        h.status = 2;
        done = true;
        break;
      }
      if (kCount) h.visits++;
      const uint32_t cur = st.cur;
      const bool staged = kStage && (cur & kStagedBit) != 0u;
      const DevNode* nd = s.nodes + cur;
      const DevNode* sn = kStage ? stg + (cur & ~kStagedBit) : nd;
      const uint4 head = staged ? *reinterpret_cast<const uint4*>(sn) : __ldg(reinterpret_cast<const uint4*>(nd));
      const uint64_t occ = ((uint64_t)head.y << 32) | head.x;
      const uint32_t meta = head.z;
      const uint32_t kind = meta & 3u;
      const bool uniform = kind == kKindUniform;
      uint32_t target = st.target;
      if (target != kOob && (uniform || kind == kKindLeaf)) {
        const uint32_t slot = uniform ? 0u : target;
        const uint32_t bk = (meta >> (8 + 2 * slot)) & 3u;
        if (bk != kBkEmpty) {
          const uint32_t rc = probe_brick_fast<kCount>(s, r, bk, __ldg(&nd->slot[slot]),
                                                       uniform ? cb : child_bounds(cb, target), h, st.work);
          if (rc) {
            h.status = rc;
            h.node = cur;
            h.octant = slot;
            done = true;
            break;
          }
        }
      }
      const float q4 = cb.inv * 4.0f;
      const float rx = (r.px - cb.x) * q4;
      const float ry = (r.py - cb.y) * q4;
      const float rz = (r.pz - cb.z) * q4;
      uint32_t flat = min(__float2uint_rz(rx), 3u) + 4u * min(__float2uint_rz(ry), 3u) +
                      16u * min(__float2uint_rz(rz), 3u);
      if (uniform || target == kOob || occ == 0 || (occ & rtn[flat * 8u]) == 0) {
        // POP: the popped node was pushed as child `ho` of the new top
        const uint32_t ho = st.oct & 7u;
        st.s0 = st.s1;
        st.s1 = st.s2;
        st.s2 = st.s3;
        st.oct >>= 3;
        --st.count;
        if (st.count > 0) {
          st.cur = st.s0;
          const float pmx = (ho & 1u) ? cb.x - cb.s : cb.x;
          const float pmy = (ho & 4u) ? cb.y - cb.s : cb.y;
          const float pmz = (ho & 2u) ? cb.z - cb.s : cb.z;
          const uint32_t move = dda_move(r, cb.x, cb.y, cb.z, cb.s);
          st.target = step_fast(ho, move, r.pos);
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
        // PUSH
        if (staged) {
          const uint32_t si = sn->stage[target];
          if (si < stg_n) ck = kStagedBit | si;
        }
        st.oct = ((st.oct << 3) | target) & 0xFFFu;
        st.cur = ck;
        cb = tb;
        st.target = hash_region(r.px - tb.x, r.py - tb.y, r.pz - tb.z, tb.s * 0.5f);
        st.s3 = st.s2;
        st.s2 = st.s1;
        st.s1 = st.s0;
        st.s0 = ck;
        st.count = st.count < 4 ? st.count + 1 : 4;
      } else {
        // ADVANCE
        float bx = rclamp(rx, kTol, 4.0f - kTol);
        float by = rclamp(ry, kTol, 4.0f - kTol);
        float bz = rclamp(rz, kTol, 4.0f - kTol);
        const float dbx = (g4x > 0.0f) ? q4 : -q4, dby = (g4y > 0.0f) ? q4 : -q4, dbz = (g4z > 0.0f) ? q4 : -q4;
        bool stop = false;
        for (;;) {
          if (++st.work > kWorkCap) {
            h.status = 2;
            stop = true;
            break;
          }
          const uint32_t move = dda_move(r, tb.x, tb.y, tb.z, tb.s);
          target = step_fast(target, move, r.pos);
          if (target == kOob) break;
          tb = child_bounds(cb, target);
          if (kCount) h.creads++;
          if (move & 1u) bx = bx + dbx;
          if (move & 4u) by = by + dby;
          if (move & 2u) bz = bz + dbz;
          const uint32_t ux = __float2uint_rz(bx), uy = __float2uint_rz(by), uz = __float2uint_rz(bz);
          if (ux >= 4u || uy >= 4u || uz >= 4u) {
            h.status = 3;
            stop = true;
            break;
          }
          flat = ux + 4u * uy + 16u * uz;
          if (kind == kKindInternal && (occ & L.octant[target]) != 0 && (rtn[flat * 8u] & occ) != 0) {
            ck = staged ? sn->slot[target] : __ldg(&nd->slot[target]);
            if (ck != kInvalidChild) break;
          }
          if (kind == kKindLeaf && ((meta >> (8 + 2 * target)) & 3u) != kBkEmpty) break;
        }
        st.target = target;
        if (stop) {
          done = true;
          break;
        }
      }
    }
    if (done) break;
    // the stack is empty: restart from the root with a 0.1 nudge, root runs in closed form
    const float c01x = r.dx * 0.1f, c01y = r.dy * 0.1f, c01z = r.dz * 0.1f;
    r.px = r.px + c01x;
    r.py = r.py + c01y;
    r.pz = r.pz + c01z;
    const uint4 rootrec = __ldg(reinterpret_cast<const uint4*>(s.nodes));
    const uint64_t occ_root = ((uint64_t)rootrec.y << 32) | rootrec.x;
    const bool root_runs = (rootrec.z & 3u) == kKindInternal || (rootrec.z & 3u) == kKindNothing;
    const float q4r = s.inv_size * 4.0f;
    bool ended = false;
    while (root_runs && r.px < S && r.py < S && r.pz < S && r.px > 0.0f && r.py > 0.0f && r.pz > 0.0f) {
      const float rx = (r.px - 0.0f) * q4r, ry = (r.py - 0.0f) * q4r, rz = (r.pz - 0.0f) * q4r;
      const uint32_t flat = min(__float2uint_rz(rx), 3u) + 4u * min(__float2uint_rz(ry), 3u) +
                            16u * min(__float2uint_rz(rz), 3u);
      if (occ_root != 0 && (occ_root & rtn[flat * 8u]) != 0) break;
      if (++st.work > kWorkCap) {
        h.status = 2;
        ended = true;
        break;
      }
      if (kCount) h.visits++;
      if (!((r.dx < 0.0f && 1.0f + r.dx >= 1.0f) || (r.dy < 0.0f && 1.0f + r.dy >= 1.0f) ||
            (r.dz < 0.0f && 1.0f + r.dz >= 1.0f))) {
        ended = true;
        if (!kCount) {
          const float cmax = fmaxf(fmaxf(fabsf(c01x), fabsf(c01y)), fabsf(c01z));
          if (cmax >= S * 0x1p-22f && (float)st.work + S / (0.5f * cmax) + 2.0f < (float)kWorkCap) break;
        }
        const RestartRun run = restart_exit(r.px, r.py, r.pz, c01x, c01y, c01z, S, kWorkCap - st.work + 2u);
        if (run.k == kRunNever) {
          h.status = 2;
          break;
        }
        if (kCount) {
          h.visits += run.k - 1u;
          h.runs += run.k - 1u;
        }
        break;
      }
      const RestartRun run = restart_run(r.px, r.py, r.pz, c01x, c01y, c01z, flat, S * 0.25f, kWorkCap - st.work + 2u);
      const uint32_t k = run.k;
      r.px = run.x;
      r.py = run.y;
      r.pz = run.z;
      if (k == kRunNever) {
        h.status = 2;
        ended = true;
        break;
      }
      st.work += k - 1u;
      if (kCount) {
        h.visits += k - 1u;
        h.runs += k - 1u;
      }
    }
    if (ended) {
      done = true;
      break;
    }
    st.target = (r.px < S && r.py < S && r.pz < S && r.px > 0.0f && r.py > 0.0f && r.pz > 0.0f)
                    ? hash_region(r.px, r.py, r.pz, S * 0.5f)
                    : kOob;
    // st.count is 0: the loop head restarts from the root or ends the ray
  }
  atomicSub((uint32_t*)live, 1u);
  return done;
}

}  // namespace svo
