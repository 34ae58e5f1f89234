// svo_vox.cpp -- MagicaVoxel .vox import: Octree::load_vox_file and
// MIPMapStrategy::load_vox_file (src/convert/magicavoxel.rs:204-345 of
// shocovox-rs v0.11.1).
//
// The reference parses the file with the dot_vox 5.1.1 crate and then walks its
// scene graph (iterate_vox_tree, magicavoxel.rs:104-202) twice: once for the
// bounds that fix the octree size, once inserting every voxel of frame 0 in
// file order.  The parser here restates the published chunk format (RIFF-like
// chunks "SIZE", "XYZI", "RGBA", "nTRN", "nGRP", "nSHP" under "MAIN"; the rest
// skipped) with dot_vox's conventions: models in SIZE/XYZI order, scene nodes
// in order of appearance (a child id indexes that order), a voxel's colour
// index one less than the stored one (clamped at 0) selecting entry i of the
// RGBA chunk.  A file without an RGBA chunk is refused (dot_vox substitutes the
// format's default palette, which is not restated here).
//
// Every place where the reference panics (a malformed file, a missing root
// transform, an unparsable attribute, an Octree::new or insert error) returns
// a status instead; malformed bytes are SVO_ERR_ARGUMENT, the rest
// SVO_ERR_REFERENCE_PANIC.  Integer arithmetic wraps like the reference's
// release build.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "svo_internal.h"

namespace svo {
namespace {

using Dict = std::vector<std::pair<std::string, std::string>>;

struct VoxModel {
  int32_t size[3];
  std::vector<uint8_t> xyzi;  // 4 bytes per voxel: x, y, z, colour index as stored
};

struct VoxNode {
  enum Kind : uint8_t { kTransform, kGroup, kShape } kind;
  uint32_t child = 0;                               // kTransform
  std::vector<Dict> frames;                         // kTransform
  std::vector<uint32_t> children;                   // kGroup
  std::vector<std::pair<uint32_t, Dict>> models;    // kShape: model id, attributes
};

struct VoxFile {
  std::vector<VoxModel> models;
  std::vector<VoxNode> nodes;
  uint32_t palette[256];  // RRGGBBAA
  bool has_palette = false;
};

struct VoxError {
  int code;
  std::string msg;
};

// ---- chunk reader ----------------------------------------------------------------------
struct Cursor {
  const uint8_t* p;
  size_t n, i;
  uint32_t u32() {
    if (n - i < 4) throw VoxError{SVO_ERR_ARGUMENT, "truncated chunk"};
    const uint32_t v = (uint32_t)p[i] | ((uint32_t)p[i + 1] << 8) | ((uint32_t)p[i + 2] << 16) | ((uint32_t)p[i + 3] << 24);
    i += 4;
    return v;
  }
  int32_t i32() { return (int32_t)u32(); }
  std::string str() {
    const uint32_t len = u32();
    if (n - i < len) throw VoxError{SVO_ERR_ARGUMENT, "truncated string"};
    std::string s(reinterpret_cast<const char*>(p + i), len);
    i += len;
    return s;
  }
  Dict dict() {
    const uint32_t count = u32();
    if (count > (n - i) / 8) throw VoxError{SVO_ERR_ARGUMENT, "truncated dictionary"};
    Dict d;
    d.reserve(count);
    for (uint32_t k = 0; k < count; ++k) {
      std::string key = str();
      d.emplace_back(std::move(key), str());
    }
    return d;
  }
};

const std::string* lookup(const Dict& d, const char* key) {
  // dot_vox keeps attributes in a map: the last of repeated keys wins
  const std::string* out = nullptr;
  for (const auto& kv : d)
    if (kv.first == key) out = &kv.second;
  return out;
}

void parse(const uint8_t* bytes, size_t length, VoxFile* f) {
  if (length < 8 || std::memcmp(bytes, "VOX ", 4) != 0) throw VoxError{SVO_ERR_ARGUMENT, "not a .vox file"};
  Cursor c{bytes, length, 8};
  if (length - c.i < 12 || std::memcmp(bytes + c.i, "MAIN", 4) != 0) throw VoxError{SVO_ERR_ARGUMENT, "no MAIN chunk"};
  c.i += 4;
  const uint32_t main_content = c.u32(), main_children = c.u32();
  if (length - c.i < (uint64_t)main_content + main_children) throw VoxError{SVO_ERR_ARGUMENT, "truncated MAIN chunk"};
  size_t at = c.i + main_content;
  const size_t end = at + main_children;
  bool open_model = false;  // a SIZE chunk waiting for its XYZI
  while (at < end) {
    if (end - at < 12) throw VoxError{SVO_ERR_ARGUMENT, "truncated chunk header"};
    char id[5] = {0};
    std::memcpy(id, bytes + at, 4);
    Cursor h{bytes, end, at + 4};
    const uint32_t content = h.u32(), children = h.u32();
    if (end - h.i < (uint64_t)content + children) throw VoxError{SVO_ERR_ARGUMENT, std::string("truncated ") + id + " chunk"};
    Cursor b{bytes, h.i + content, h.i};  // the chunk's content only
    if (!std::strcmp(id, "SIZE")) {
      VoxModel m;
      for (int k = 0; k < 3; ++k) m.size[k] = b.i32();
      f->models.push_back(std::move(m));
      open_model = true;
    } else if (!std::strcmp(id, "XYZI")) {
      if (!open_model) throw VoxError{SVO_ERR_ARGUMENT, "XYZI chunk without a SIZE chunk"};
      const uint32_t count = b.u32();
      if (count > (b.n - b.i) / 4) throw VoxError{SVO_ERR_ARGUMENT, "truncated XYZI chunk"};
      f->models.back().xyzi.assign(bytes + b.i, bytes + b.i + (size_t)count * 4);
      open_model = false;
    } else if (!std::strcmp(id, "RGBA")) {
      if (content < 1024) throw VoxError{SVO_ERR_ARGUMENT, "truncated RGBA chunk"};
      for (int k = 0; k < 256; ++k) {
        const uint8_t* q = bytes + b.i + 4 * k;
        f->palette[k] = ((uint32_t)q[0] << 24) | ((uint32_t)q[1] << 16) | ((uint32_t)q[2] << 8) | q[3];
      }
      f->has_palette = true;
    } else if (!std::strcmp(id, "nTRN")) {
      VoxNode n;
      n.kind = VoxNode::kTransform;
      b.i32();  // node id (dot_vox keeps nodes in order of appearance)
      b.dict();
      n.child = b.u32();
      b.i32();  // reserved id
      b.i32();  // layer id
      const uint32_t frames = b.u32();
      if (frames > (b.n - b.i) / 4) throw VoxError{SVO_ERR_ARGUMENT, "truncated nTRN chunk"};
      for (uint32_t k = 0; k < frames; ++k) n.frames.push_back(b.dict());
      f->nodes.push_back(std::move(n));
    } else if (!std::strcmp(id, "nGRP")) {
      VoxNode n;
      n.kind = VoxNode::kGroup;
      b.i32();
      b.dict();
      const uint32_t count = b.u32();
      if (count > (b.n - b.i) / 4) throw VoxError{SVO_ERR_ARGUMENT, "truncated nGRP chunk"};
      for (uint32_t k = 0; k < count; ++k) n.children.push_back(b.u32());
      f->nodes.push_back(std::move(n));
    } else if (!std::strcmp(id, "nSHP")) {
      VoxNode n;
      n.kind = VoxNode::kShape;
      b.i32();
      b.dict();
      const uint32_t count = b.u32();
      if (count > (b.n - b.i) / 8) throw VoxError{SVO_ERR_ARGUMENT, "truncated nSHP chunk"};
      for (uint32_t k = 0; k < count; ++k) {
        const uint32_t model = b.u32();
        n.models.emplace_back(model, b.dict());
      }
      f->nodes.push_back(std::move(n));
    }
    at = h.i + content + children;
  }
}

// ---- Rust's integer parsing (core::num::from_str_radix, radix 10) ----------------------
// An optional '+' (or '-' for a signed type) and at least one decimal digit; overflow is an error.
bool parse_digits(const std::string& s, size_t i, uint64_t max, uint64_t* out) {
  if (i >= s.size()) return false;
  uint64_t v = 0;
  for (; i < s.size(); ++i) {
    if (s[i] < '0' || s[i] > '9') return false;
    const uint64_t d = (uint64_t)(s[i] - '0');
    if (v > (max - d) / 10) return false;
    v = v * 10 + d;
  }
  *out = v;
  return true;
}

bool parse_unsigned(const std::string& s, uint64_t max, uint64_t* out) {
  return parse_digits(s, !s.empty() && s[0] == '+' ? 1 : 0, max, out);
}

bool parse_i32(const std::string& s, int32_t* out) {
  const bool neg = !s.empty() && s[0] == '-';
  uint64_t v;
  if (!parse_digits(s, !s.empty() && (s[0] == '+' || s[0] == '-') ? 1 : 0, neg ? 2147483648ull : 2147483647ull, &v))
    return false;
  *out = neg ? (int32_t)(0u - (uint32_t)v) : (int32_t)v;
  return true;
}

int32_t wrap(int64_t v) { return (int32_t)(uint32_t)(uint64_t)v; }

// ---- magicavoxel.rs ------------------------------------------------------------------------
struct Mat {
  int32_t m[3][3];  // row, column
};
const Mat kIdentity{{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}};

// parse_rotation_matrix (magicavoxel.rs:61-90): row r holds its single non-zero entry in the
// column given by bits 2r..2r+1 (the third row's column is the one the first two leave), with
// the sign of bit 4 + r.  An index of 3, or two rows on one column, indexes past the matrix.
bool rotation_of(uint8_t b, Mat* out) {
  const uint32_t c0 = b & 3u, c1 = (b >> 2) & 3u, c2 = ~(c0 ^ c1) & 3u;
  if (c0 > 2 || c1 > 2 || c2 > 2) return false;
  Mat r{};
  r.m[0][c0] = (b & 0x10) ? -1 : 1;
  r.m[1][c1] = (b & 0x20) ? -1 : 1;
  r.m[2][c2] = (b & 0x40) ? -1 : 1;
  *out = r;
  return true;
}

Mat mul(const Mat& a, const Mat& b) {
  Mat o{};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) o.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
  return o;
}

// V3c::transformed (magicavoxel.rs:96-102): matrix times column vector, i32 wrapping
void transformed(const int32_t v[3], const Mat& m, int32_t out[3]) {
  for (int i = 0; i < 3; ++i)
    out[i] = (int32_t)((uint32_t)v[0] * (uint32_t)m.m[i][0] + (uint32_t)v[1] * (uint32_t)m.m[i][1] +
                       (uint32_t)v[2] * (uint32_t)m.m[i][2]);
}

// iterate_vox_tree (magicavoxel.rs:104-202) for frame 0, calling fun(model, translation, rotation)
// for every model of a shape whose "_f" attribute is 0.  Kept exactly: the root transform's own
// attributes are not applied; translations add up without rotation; a transform without "_r"
// resets the orientation to the identity; a shape raises its parent's child index on leaving.
template <class F>
void iterate(const VoxFile& f, F&& fun) {
  struct Entry {
    uint32_t node;
    int32_t t[3];
    Mat r;
    uint32_t index;
  };
  if (f.nodes.empty() || f.nodes[0].kind != VoxNode::kTransform)
    throw VoxError{SVO_ERR_REFERENCE_PANIC, "the root node of the scene graph is not a transform"};
  std::vector<Entry> stack{{f.nodes[0].child, {0, 0, 0}, kIdentity, 0}};
  uint64_t steps = 0;
  while (!stack.empty()) {
    // a cycle in the graph grows the reference's stack without end
    if (stack.size() > f.nodes.size() + 1 || ++steps > (1ull << 28))
      throw VoxError{SVO_ERR_REFERENCE_PANIC, "the scene graph does not terminate"};
    const Entry e = stack.back();
    if (e.node >= f.nodes.size()) throw VoxError{SVO_ERR_REFERENCE_PANIC, "scene node index out of bounds"};
    const VoxNode& n = f.nodes[e.node];
    if (n.kind == VoxNode::kTransform) {
      if (n.frames.empty()) throw VoxError{SVO_ERR_REFERENCE_PANIC, "transform without frames"};
      const Dict& fr = n.frames[0];
      int32_t t[3] = {e.t[0], e.t[1], e.t[2]};
      if (const std::string* ts = lookup(fr, "_t")) {
        // split(" ") then every piece parsed as i32, the first three used
        std::vector<int32_t> parts;
        size_t start = 0;
        for (;;) {
          const size_t sp = ts->find(' ', start);
          const std::string piece = ts->substr(start, sp == std::string::npos ? std::string::npos : sp - start);
          int32_t v;
          if (!parse_i32(piece, &v))
            throw VoxError{SVO_ERR_REFERENCE_PANIC, "translation \"" + *ts + "\" is not integers"};
          parts.push_back(v);
          if (sp == std::string::npos) break;
          start = sp + 1;
        }
        if (parts.size() < 3) throw VoxError{SVO_ERR_REFERENCE_PANIC, "translation with fewer than 3 values"};
        for (int k = 0; k < 3; ++k) t[k] = wrap((int64_t)e.t[k] + parts[k]);
      }
      Mat r = kIdentity;
      if (const std::string* rs = lookup(fr, "_r")) {
        uint64_t v;
        Mat p;
        if (!parse_unsigned(*rs, 255, &v)) throw VoxError{SVO_ERR_REFERENCE_PANIC, "rotation \"" + *rs + "\" is not a u8"};
        if (!rotation_of((uint8_t)v, &p)) throw VoxError{SVO_ERR_REFERENCE_PANIC, "invalid rotation byte " + *rs};
        r = mul(e.r, p);
      }
      if (e.index == 0) {
        stack.back().index += 1;
        stack.push_back({n.child, {t[0], t[1], t[2]}, r, 0});
      } else {
        stack.pop_back();
      }
    } else if (n.kind == VoxNode::kGroup) {
      if (e.index < n.children.size()) {
        stack.back().index += 1;
        stack.push_back({n.children[e.index], {e.t[0], e.t[1], e.t[2]}, e.r, 0});
      } else {
        stack.pop_back();
      }
    } else {
      for (const auto& m : n.models) {
        uint64_t frame = 0;
        if (const std::string* fs = lookup(m.second, "_f"))
          if (!parse_unsigned(*fs, UINT64_MAX, &frame))
            throw VoxError{SVO_ERR_REFERENCE_PANIC, "frame attribute \"" + *fs + "\" is not an integer"};
        if (frame == 0) {
          if (m.first >= f.models.size()) throw VoxError{SVO_ERR_REFERENCE_PANIC, "model index out of bounds"};
          fun(f.models[m.first], e.t, e.r);
        }
      }
      stack.pop_back();
      if (!stack.empty()) stack.back().index += 1;
    }
  }
}

void half_size(const VoxModel& m, const Mat& r, int32_t h[3]) {
  transformed(m.size, r, h);
  for (int k = 0; k < 3; ++k) h[k] /= 2;  // i32 division truncates towards zero
}

// load_vox_file_internal (magicavoxel.rs:278-335): the voxel bounds in the file's right-handed
// z-up frame
void bounds_rzup(const VoxFile& f, int32_t lo[3], int32_t hi[3]) {
  for (int k = 0; k < 3; ++k) {
    lo[k] = INT32_MAX;
    hi[k] = INT32_MIN;
  }
  iterate(f, [&](const VoxModel& m, const int32_t p[3], const Mat& r) {
    int32_t h[3];
    half_size(m, r, h);
    for (int k = 0; k < 3; ++k) {
      const int32_t a = wrap((int64_t)p[k] - h[k]), b = wrap((int64_t)p[k] + h[k]);
      lo[k] = std::min(std::min(lo[k], a), b);
      hi[k] = std::max(std::max(hi[k], b), a);
    }
  });
}

// convert_coordinate Rzup <-> Lyup (src/spatial/math/mod.rs:196-199): y and z swap
void swap_yz(int32_t v[3]) { std::swap(v[1], v[2]); }

// Octree::load_vox_file's size (magicavoxel.rs:265-270): 2^ceil(log2(largest extent)), the
// extent max - min of the bounds in the octree's left-handed y-up frame
uint32_t tree_size_of(const VoxFile& f) {
  int32_t lo[3], hi[3];
  bounds_rzup(f, lo, hi);
  swap_yz(lo);
  swap_yz(hi);
  int32_t ext[3];
  for (int k = 0; k < 3; ++k) ext[k] = wrap((int64_t)hi[k] - lo[k]);
  const int32_t e = std::max(std::max(ext[0], ext[1]), ext[2]);
  const float l = std::ceil(std::log2((float)e));
  // `as u32` saturates (NaN to 0); 2_u32.pow wraps past 2^31 in a release build
  const uint32_t x = std::isnan(l) || l <= 0.0f ? 0u : (l >= 4294967295.0f ? 4294967295u : (uint32_t)l);
  return x >= 32 ? 0u : (1u << x);
}

// load_vox_data_internal (magicavoxel.rs:337-385): every voxel of frame 0, in file order,
// inserted as its palette colour
void insert_all(const VoxFile& f, HostOctree& t) {
  int32_t lo[3], hi[3];
  bounds_rzup(f, lo, hi);
  if (!f.has_palette) throw VoxError{SVO_ERR_ARGUMENT, "no RGBA palette chunk (the format's default palette is not supported)"};
  iterate(f, [&](const VoxModel& m, const int32_t p[3], const Mat& r) {
    int32_t h[3], bl[3];
    half_size(m, r, h);
    for (int k = 0; k < 3; ++k) bl[k] = wrap((int64_t)p[k] - h[k] - lo[k] + (h[k] < 0 ? -1 : 0));
    const size_t count = m.xyzi.size() / 4;
    for (size_t v = 0; v < count; ++v) {
      const uint8_t* q = &m.xyzi[4 * v];
      const int32_t local[3] = {q[0], q[1], q[2]};
      int32_t d[3], pos[3];
      transformed(local, r, d);
      for (int k = 0; k < 3; ++k) pos[k] = wrap((int64_t)bl[k] + d[k]);
      swap_yz(pos);
      const uint32_t up[3] = {(uint32_t)pos[0], (uint32_t)pos[1], (uint32_t)pos[2]};
      Entry e;
      e.kind = 1;
      e.rgba = f.palette[q[3] == 0 ? 0 : q[3] - 1];
      const int rc = t.insert_at_lod(true, up, 1, e);
      if (rc != 0) {
        static const char* names[] = {"ok", "InvalidSize", "InvalidBrickDimension", "InvalidStructure", "InvalidPosition"};
        char where[96];
        std::snprintf(where, sizeof where, " inserting voxel (%u, %u, %u)", up[0], up[1], up[2]);
        throw VoxError{SVO_ERR_REFERENCE_PANIC, std::string(rc < 5 ? names[rc] : "error") + where};
      }
    }
  });
}

template <class F>
svo_status vox_guarded(const char* what, F&& f) {
  try {
    return f();
  } catch (const VoxError& e) {
    return fail(e.code, std::string(what) + ": " + e.msg);
  } catch (const ReferencePanic& p) {
    return fail(SVO_ERR_REFERENCE_PANIC, std::string(what) + ": the reference panics here (" + p.what() + ")");
  } catch (const std::bad_alloc&) {
    return fail(SVO_ERR_OUT_OF_MEMORY, std::string(what) + ": host allocation failed");
  }
}

}  // namespace
}  // namespace svo

using namespace svo;

extern "C" {

svo_status svo_vox_rotation(uint8_t byte, int8_t out[9]) {
  if (!out) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  Mat m;
  if (!rotation_of(byte, &m)) return fail(SVO_ERR_REFERENCE_PANIC, "svo_vox_rotation: invalid rotation byte");
  for (int i = 0; i < 9; ++i) out[i] = (int8_t)m.m[i / 3][i % 3];
  return SVO_OK;
}

svo_status svo_vox_tree_size(const uint8_t* bytes, uint64_t length, uint32_t* size) {
  if (!size || (!bytes && length)) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  return vox_guarded("svo_vox_tree_size", [&]() -> svo_status {
    VoxFile f;
    parse(bytes, (size_t)length, &f);
    *size = tree_size_of(f);
    return SVO_OK;
  });
}

svo_status svo_vox_insert(svo_scene* s, const uint8_t* bytes, uint64_t length) {
  if (!s || (!bytes && length)) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  return vox_guarded("svo_vox_insert", [&]() -> svo_status {
    VoxFile f;
    parse(bytes, (size_t)length, &f);
    insert_all(f, s->tree);
    return SVO_OK;
  });
}

svo_status svo_scene_from_vox(const uint8_t* bytes, uint64_t length, uint32_t brick_dim, svo_scene** out) {
  if (!out || (!bytes && length)) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  *out = nullptr;
  return vox_guarded("svo_scene_from_vox", [&]() -> svo_status {
    VoxFile f;
    parse(bytes, (size_t)length, &f);
    const uint32_t size = tree_size_of(f);
    std::unique_ptr<svo_scene> s(new svo_scene());
    const int rc = HostOctree::create(size, brick_dim, &s->tree);
    if (rc != 0) {
      static const char* names[] = {"ok", "InvalidSize", "InvalidBrickDimension", "InvalidStructure", "InvalidPosition"};
      throw VoxError{SVO_ERR_REFERENCE_PANIC, std::string("Octree::new(") + std::to_string(size) + ", " +
                                                  std::to_string(brick_dim) + "): " + (rc < 5 ? names[rc] : "error")};
    }
    insert_all(f, s->tree);
    *out = s.release();
    return SVO_OK;
  });
}

svo_status svo_scene_load_vox(const char* path, uint32_t brick_dim, svo_scene** out) {
  if (!path || !out) return fail(SVO_ERR_ARGUMENT, "NULL argument");
  *out = nullptr;
  std::string bytes;
  {
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(SVO_ERR_IO, std::string("svo_scene_load_vox: cannot open ") + path);
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) bytes.append(buf, n);
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    if (err) return fail(SVO_ERR_IO, std::string("svo_scene_load_vox: cannot read ") + path);
  }
  return svo_scene_from_vox(reinterpret_cast<const uint8_t*>(bytes.data()), bytes.size(), brick_dim, out);
}

}  // extern "C"
