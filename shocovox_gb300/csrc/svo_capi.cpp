// svo_capi.cpp -- host-side C ABI of libsvo (construction, update, queries).
// No exception or panic crosses the boundary: ReferencePanic becomes
// SVO_ERR_REFERENCE_PANIC, allocation failure SVO_ERR_OUT_OF_MEMORY.
#include <cstring>
#include <new>
#include <cstdio>
#include <memory>
#include <string>

#include "svo_internal.h"
#include "svo_trace.h"

namespace svo {
namespace {
thread_local std::string g_last_error;

Entry make_entry(uint32_t kind, uint32_t rgba, uint32_t user) {
  Entry e;
  e.kind = kind & 3u;
  e.rgba = (kind & 1u) ? rgba : 0;
  e.user = (kind & 2u) ? user : 0;
  return e;
}

template <class F>
svo_status guarded(const char* what, F&& f) {
  try {
    return f();
  } catch (const ReferencePanic& p) {
    return fail(SVO_ERR_REFERENCE_PANIC, std::string(what) + ": the reference panics here (" + p.what() + ")");
  } catch (const std::bad_alloc&) {
    return fail(SVO_ERR_OUT_OF_MEMORY, std::string(what) + ": host allocation failed");
  }
}

svo_status op_status(int rc, const char* what) {
  if (rc == 0) return SVO_OK;
  static const char* names[] = {"ok", "InvalidSize", "InvalidBrickDimension", "InvalidStructure", "InvalidPosition"};
  return fail(rc, std::string(what) + ": " + (rc < 5 ? names[rc] : "error"));
}
}  // namespace

void set_error(const std::string& msg) { g_last_error = msg; }
svo_status fail(svo_status code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
}  // namespace svo

using namespace svo;

extern "C" {

const char* svo_last_error(void) { return g_last_error.c_str(); }
int32_t svo_version(void) { return 100; }

svo_status svo_scene_create(uint32_t size, uint32_t brick_dim, svo_scene** out) {
  if (!out) return fail(SVO_ERR_ARGUMENT, "svo_scene_create: out is NULL");
  *out = nullptr;
  return guarded("svo_scene_create", [&]() -> svo_status {
    svo_scene* s = new svo_scene();
    int rc = HostOctree::create(size, brick_dim, &s->tree);
    if (rc != 0) {
      delete s;
      return op_status(rc, "Octree::new");
    }
    *out = s;
    return SVO_OK;
  });
}

svo_status svo_set_auto_simplify(svo_scene* s, int32_t enabled) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  s->tree.auto_simplify = enabled != 0;
  return SVO_OK;
}

// ---- persistence: Octree::to_bytes / from_bytes / save / load (src/octree/mod.rs:138-168) ----
svo_status svo_scene_to_bytes(svo_scene* s, uint8_t* out, uint64_t capacity, uint64_t* length) {
  if (!s || !length) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  return guarded("svo_scene_to_bytes", [&]() -> svo_status {
    std::string bytes;
    s->tree.encode(bytes);
    *length = bytes.size();
    if (!out) return SVO_OK;
    if (capacity < bytes.size()) return fail(SVO_ERR_ARGUMENT, "svo_scene_to_bytes: buffer too small");
    std::memcpy(out, bytes.data(), bytes.size());
    return SVO_OK;
  });
}

svo_status svo_scene_from_bytes(const uint8_t* bytes, uint64_t length, svo_scene** out) {
  if (!out || (!bytes && length)) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  *out = nullptr;
  return guarded("svo_scene_from_bytes", [&]() -> svo_status {
    std::unique_ptr<svo_scene> s(new svo_scene());
    std::string err;
    const int rc = HostOctree::decode(bytes, (size_t)length, &s->tree, &err);
    if (rc != 0) return err.empty() ? op_status(rc, "Octree::from_bytes") : fail((svo_status)rc, "svo_scene_from_bytes: " + err);
    *out = s.release();
    return SVO_OK;
  });
}

svo_status svo_scene_save(svo_scene* s, const char* path) {
  if (!s || !path) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  return guarded("svo_scene_save", [&]() -> svo_status {
    std::string bytes;
    s->tree.encode(bytes);
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(SVO_ERR_IO, std::string("svo_scene_save: cannot open ") + path);
    const bool ok = std::fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
    if (std::fclose(f) != 0 || !ok) return fail(SVO_ERR_IO, std::string("svo_scene_save: cannot write ") + path);
    return SVO_OK;
  });
}

svo_status svo_scene_load(const char* path, svo_scene** out) {
  if (!path || !out) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  *out = nullptr;
  std::string bytes;
  {
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(SVO_ERR_IO, std::string("svo_scene_load: cannot open ") + path);
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) bytes.append(buf, n);
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    if (err) return fail(SVO_ERR_IO, std::string("svo_scene_load: cannot read ") + path);
  }
  return svo_scene_from_bytes(reinterpret_cast<const uint8_t*>(bytes.data()), bytes.size(), out);
}

// ---- MIP maps: Octree::albedo_mip_map_resampling_strategy() (src/octree/mipmap.rs) ----
svo_status svo_mip_switch(svo_scene* s, int32_t enabled) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  return guarded("svo_mip_switch", [&] {
    s->tree.switch_albedo_mip_maps(enabled != 0);
    return SVO_OK;
  });
}

svo_status svo_mip_set_method(svo_scene* s, uint32_t level, uint32_t method, float threshold) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  if (method > SVO_MIP_POSTERIZE_BD) return fail(SVO_ERR_ARGUMENT, "svo_mip_set_method: unknown method");
  s->tree.set_mip_method(level, method, threshold);
  return SVO_OK;
}

svo_status svo_mip_set_color_threshold(svo_scene* s, uint32_t level, float threshold) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  s->tree.set_mip_color_threshold(level, threshold);
  return SVO_OK;
}

svo_status svo_mip_recalculate(svo_scene* s) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  return guarded("svo_mip_recalculate", [&] {
    s->tree.recalculate_mips();
    return SVO_OK;
  });
}

svo_status svo_mip_sample_root(svo_scene* s, uint32_t octant, uint32_t x, uint32_t y, uint32_t z, uint32_t* kind,
                               uint32_t* rgba, uint32_t* user) {
  if (!s || !kind || !rgba || !user) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  if (octant > 8) return fail(SVO_ERR_ARGUMENT, "svo_mip_sample_root: octant must be 0..8");
  const uint32_t p[3] = {x, y, z};
  return guarded("svo_mip_sample_root", [&] {
    const Entry e = s->tree.sample_root_mip((uint8_t)octant, p);
    *kind = e.kind;
    *rgba = e.rgba;
    *user = e.user;
    return SVO_OK;
  });
}

svo_status svo_insert(svo_scene* s, uint32_t x, uint32_t y, uint32_t z, uint32_t kind, uint32_t rgba, uint32_t user) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  const uint32_t p[3] = {x, y, z};
  return guarded("insert", [&] { return op_status(s->tree.insert_at_lod(true, p, 1, make_entry(kind, rgba, user)), "insert"); });
}
svo_status svo_update(svo_scene* s, uint32_t x, uint32_t y, uint32_t z, uint32_t kind, uint32_t rgba, uint32_t user) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  const uint32_t p[3] = {x, y, z};
  return guarded("update", [&] { return op_status(s->tree.insert_at_lod(false, p, 1, make_entry(kind, rgba, user)), "update"); });
}
svo_status svo_insert_at_lod(svo_scene* s, uint32_t x, uint32_t y, uint32_t z, uint32_t size, uint32_t kind,
                             uint32_t rgba, uint32_t user) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  const uint32_t p[3] = {x, y, z};
  return guarded("insert_at_lod", [&] {
    return op_status(s->tree.insert_at_lod(true, p, size, make_entry(kind, rgba, user)), "insert_at_lod");
  });
}
svo_status svo_clear(svo_scene* s, uint32_t x, uint32_t y, uint32_t z) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  const uint32_t p[3] = {x, y, z};
  return guarded("clear", [&] { return op_status(s->tree.clear_at_lod(p, 1), "clear"); });
}
svo_status svo_clear_at_lod(svo_scene* s, uint32_t x, uint32_t y, uint32_t z, uint32_t size) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  const uint32_t p[3] = {x, y, z};
  return guarded("clear_at_lod", [&] { return op_status(s->tree.clear_at_lod(p, size), "clear_at_lod"); });
}

svo_status svo_apply_ops(svo_scene* s, const svo_op* ops, uint64_t n, uint64_t* n_done) {
  TraceRange range("svo_apply_ops");
  if (!s || (!ops && n)) return fail(SVO_ERR_ARGUMENT, "svo_apply_ops: NULL argument");
  uint64_t i = 0;
  svo_status rc = SVO_OK;
  for (; i < n; ++i) {
    const svo_op& o = ops[i];
    switch (o.op) {
      case SVO_OP_INSERT: rc = svo_insert(s, o.x, o.y, o.z, o.kind, o.rgba, o.user); break;
      case SVO_OP_UPDATE: rc = svo_update(s, o.x, o.y, o.z, o.kind, o.rgba, o.user); break;
      case SVO_OP_INSERT_AT_LOD: rc = svo_insert_at_lod(s, o.x, o.y, o.z, o.size, o.kind, o.rgba, o.user); break;
      case SVO_OP_CLEAR: rc = svo_clear(s, o.x, o.y, o.z); break;
      case SVO_OP_CLEAR_AT_LOD: rc = svo_clear_at_lod(s, o.x, o.y, o.z, o.size); break;
      default: rc = fail(SVO_ERR_ARGUMENT, "svo_apply_ops: unknown op");
    }
    if (rc != SVO_OK) break;
  }
  if (n_done) *n_done = i;
  return rc;
}

svo_status svo_insert_dense(svo_scene* s, uint32_t x0, uint32_t y0, uint32_t z0, uint32_t w, uint32_t h, uint32_t d,
                            const uint32_t* rgba, const uint32_t* user, uint64_t* n_done) {
  if (!s || (!rgba && !user)) return fail(SVO_ERR_ARGUMENT, "svo_insert_dense: NULL argument");
  uint64_t done = 0;
  svo_status rc = SVO_OK;
  // the nesting of the reference's fill loops: x outermost, z innermost
  for (uint32_t i = 0; i < w && rc == SVO_OK; ++i)
    for (uint32_t j = 0; j < h && rc == SVO_OK; ++j)
      for (uint32_t k = 0; k < d; ++k) {
        const uint64_t f = (uint64_t)i + (uint64_t)w * ((uint64_t)j + (uint64_t)h * k);
        const uint32_t c = rgba ? rgba[f] : 0, u = user ? user[f] : 0;
        const uint32_t kind = (rgba ? SVO_ENTRY_VISUAL : 0) | (user ? SVO_ENTRY_INFORMATIVE : 0);
        rc = svo_insert(s, x0 + i, y0 + j, z0 + k, kind, c, u);
        if (rc != SVO_OK) break;
        ++done;
      }
  if (n_done) *n_done = done;
  return rc;
}

svo_status svo_get(svo_scene* s, uint32_t x, uint32_t y, uint32_t z, uint32_t* kind, uint32_t* rgba, uint32_t* user) {
  if (!s) return fail(SVO_ERR_ARGUMENT, "NULL scene");
  const uint32_t p[3] = {x, y, z};
  return guarded("get", [&] {
    Entry e = s->tree.get(p);
    if (kind) *kind = e.kind;
    if (rgba) *rgba = e.rgba;
    if (user) *user = e.user;
    return SVO_OK;
  });
}

svo_status svo_scene_stats_get(svo_scene* s, svo_scene_stats* out) {
  if (!s || !out) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  std::memset(out, 0, sizeof(*out));
  const HostOctree& t = s->tree;
  out->nodes = t.nodes();
  for (auto r : t.reserved) out->reserved_nodes += r;
  out->parted_bricks = t.arena.live_count();
  out->colors = t.colors.size();
  out->datas = t.datas.size();
  out->size = t.size;
  out->brick_dim = t.dim;
  out->device_bytes = device_image_bytes(s);  // what a server counts against its budget
  return SVO_OK;
}

svo_status svo_node_record(svo_scene* s, uint64_t key, uint64_t rec[40]) {
  if (!s || !rec) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  if (key >= s->tree.nodes()) return fail(SVO_ERR_ARGUMENT, "svo_node_record: key out of range");
  s->tree.node_record(key, rec);
  return SVO_OK;
}

uint64_t svo_palette(svo_scene* s, int32_t which, uint32_t* out, uint64_t max) {
  if (!s) return 0;
  const auto& p = which == 0 ? s->tree.colors : s->tree.datas;
  if (out)
    for (uint64_t i = 0; i < max && i < p.size(); ++i) out[i] = p[i];
  return p.size();
}

}  // extern "C"
