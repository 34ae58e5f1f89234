// svo_octree.cpp -- host octree of libsvo (construction, update, get).
//
// Structure decisions follow shocovox-rs v0.11.1 line by line (cited per
// function) so node keys, palettes and brick contents equal the reference's;
// storage is flat: per-node arrays plus a brick arena, each change marking
// the node/brick dirty for in-place device sync.  Compiled with
// -ffp-contract=off: every f32 operation rounds on its own, as in Rust.
#include "svo_octree.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace svo {
namespace {

// ---- Rust scalar semantics used by the construction code ----
inline uint64_t sat_usize(float x) {  // `x as usize`
  if (std::isnan(x) || x <= 0.0f) return 0;
  if (x >= 18446744073709551616.0f) return UINT64_MAX;
  return (uint64_t)x;
}
inline uint32_t sat_u32(float x) {  // `x as u32`
  if (std::isnan(x) || x <= 0.0f) return 0;
  if (x >= 4294967296.0f) return UINT32_MAX;
  return (uint32_t)x;
}
inline uint64_t round_usize(float x) { return sat_usize(std::round(x)); }  // From<V3c<f32>> for V3c<usize>

// OCTANT_OFFSET_REGION_LUT (src/spatial/lut.rs:156-197): x = bit 0, z = bit 1, y = bit 2
inline float off_x(uint32_t o) { return (float)(o & 1u); }
inline float off_y(uint32_t o) { return (float)((o >> 2) & 1u); }
inline float off_z(uint32_t o) { return (float)((o >> 1) & 1u); }

inline uint64_t flat3(uint64_t x, uint64_t y, uint64_t z, uint64_t d) { return x + y * d + z * d * d; }

// hash_region (src/spatial/math/mod.rs:11-19)
inline uint8_t octant_of(float ox, float oy, float oz, float half) {
  return (uint8_t)((ox >= half) + (oz >= half) * 2 + (oy >= half) * 4);
}

// set_occupancy_in_bitmap_64bits (src/spatial/math/mod.rs:114-162)
void set_occupancy(const uint64_t p[3], uint64_t size, uint64_t brick_dim, bool occupied, uint64_t* bitmap) {
  if (brick_dim == 1) {
    *bitmap = occupied ? UINT64_MAX : 0;
    return;
  }
  const uint64_t count = sat_usize(std::ceil((float)size * 4.0f / (float)brick_dim));
  uint64_t s[3];
  for (int a = 0; a < 3; ++a) s[a] = round_usize(std::floor((float)(p[a] * 4) / (float)brick_dim));
  for (uint64_t x = s[0]; x < std::min<uint64_t>(s[0] + count, 4); ++x)
    for (uint64_t y = s[1]; y < std::min<uint64_t>(s[1] + count, 4); ++y)
      for (uint64_t z = s[2]; z < std::min<uint64_t>(s[2] + count, 4); ++z) {
        const uint64_t m = 1ull << (x + 4 * y + 16 * z);
        *bitmap = occupied ? (*bitmap | m) : (*bitmap & ~m);
      }
}

// matrix_index_for (src/spatial/math/mod.rs:44-78)
inline void matrix_index(const Cube& b, const uint32_t pos[3], uint32_t dim, uint64_t out[3]) {
  out[0] = round_usize(std::floor(((float)pos[0] - b.x) * (float)dim / b.size));
  out[1] = round_usize(std::floor(((float)pos[1] - b.y) * (float)dim / b.size));
  out[2] = round_usize(std::floor(((float)pos[2] - b.z) * (float)dim / b.size));
}

// bound_contains / child_octant_for (src/octree/detail.rs:20-38)
inline bool contains(const Cube& b, float x, float y, float z) {
  return x >= b.x && x < b.x + b.size && y >= b.y && y < b.y + b.size && z >= b.z && z < b.z + b.size;
}
inline uint8_t child_octant(const Cube& b, float x, float y, float z) {
  return octant_of(x - b.x, y - b.y, z - b.z, b.size / 2.0f);
}
// target bounds as written in insert.rs:129-134 / clear.rs:69-74: min + (offset * size) / 2
inline Cube target_cube(const Cube& b, uint8_t o) {
  return Cube{b.x + off_x(o) * b.size / 2.0f, b.y + off_y(o) * b.size / 2.0f, b.z + off_z(o) * b.size / 2.0f,
              b.size / 2.0f};
}
// derived PartialOrd on V3c: lexicographic (x, y, z)
inline bool lex_le(float ax, float ay, float az, float bx, float by, float bz) {
  if (ax != bx) return ax < bx;
  if (ay != by) return ay < by;
  return az <= bz;
}

inline bool transparent(uint32_t rgba) { return (rgba & 0xFFu) == 0; }
inline uint32_t pix_color(uint32_t p) { return p & 0xFFFFu; }
inline uint32_t pix_data(uint32_t p) { return p >> 16; }

struct DepthGuard {
  int& d;
  explicit DepthGuard(int& v) : d(v) {
    if (++d > 4096) throw ReferencePanic("unbounded recursion");
  }
  ~DepthGuard() { --d; }
};

}  // namespace

// ---------------------------------------------------------------- arena
void BrickArena::init(uint32_t dim) { len_ = dim * dim * dim; }
uint32_t BrickArena::alloc() {
  uint32_t s;
  if (!free_.empty()) {
    s = free_.back();
    free_.pop_back();
  } else {
    s = (uint32_t)live_.size();
    live_.push_back(0);
    dirty_.push_back(0);
    hint_.push_back(0);
    hint_.push_back(0);
    data_.resize(data_.size() + len_);
  }
  live_[s] = 1;
  dirty_[s] = 1;
  ++live_count_;
  return s;
}
uint32_t BrickArena::alloc_fill(uint32_t value) {
  uint32_t s = alloc();
  std::fill(at(s), at(s) + len_, value);
  return s;
}
uint32_t BrickArena::clone(uint32_t slot) {
  uint32_t s = alloc();
  std::memcpy(at(s), at(slot), sizeof(uint32_t) * len_);
  return s;
}
void BrickArena::release(uint32_t slot) {
  if (slot < live_.size() && live_[slot]) {
    live_[slot] = 0;
    free_.push_back(slot);
    --live_count_;
  }
}

// ---------------------------------------------------------------- pool
int HostOctree::create(uint32_t size, uint32_t dim, HostOctree* t) {
  // Octree::new (src/octree/mod.rs:173-186); the f32 log2().fract() tests are exact power-of-two tests.
  auto pow2 = [](uint32_t v) { return v != 0 && (v & (v - 1)) == 0; };
  if (size == 0 || !pow2(dim)) return 2;
  if (dim > size || size % dim != 0 || !pow2(size / dim)) return 1;
  if (size < dim * 2) return 3;
  t->size = size;
  t->dim = dim;
  t->arena.init(dim);
  t->push(Content{});  // root key 0 (mod.rs:190)
  t->mips.assign(1, BrickRef{});  // node_mips: vec![BrickData::Empty] (mod.rs:198)
  // MIPMapStrategy::default (mipmap.rs:580-595)
  t->mip_methods = {{1, {kMipPoint, 0.0f}}, {2, {kMipBox, 0.0f}}, {3, {kMipBox, 0.0f}}, {4, {kMipBox, 0.0f}}};
  t->mip_color_thr = {{2, 0.1f}, {3, 0.05f}, {4, 0.02f}};
  return 0;
}

void HostOctree::grow_nodes(size_t n) {
  reserved.resize(n, 0);
  kind.resize(n, kNothing);
  ocbits.resize(n, 0);
  bricks.resize(n * 8);
  ch_kind.resize(n, kNoChildren);
  ch.resize(n * 8, 0);
  ch_bitmap.resize(n, 0);
  node_dirty.resize(n, 1);
  structure_grew = true;
}

// ObjectPool::allocate (src/object_pool.rs:151-202).  The reference keeps
// node_children exactly as long as the pool, so one length serves both.
size_t HostOctree::pool_allocate() {
  const size_t len = reserved.size();
  auto next_free = [&] { return first_available + 1 < reserved.size() && !reserved[first_available + 1]; };
  size_t key;
  bool found;
  if (first_available < len && !reserved[first_available]) {
    found = true;
  } else if (next_free()) {
    first_available += 1;
    found = true;
  } else {
    first_available = len;
    found = false;
  }
  if (found) {
    key = first_available;
  } else {
    grow_nodes(len + 1);
    key = len;
  }
  reserved[key] = 1;
  touch(key);
  if (next_free()) first_available += 1;
  return key;
}

size_t HostOctree::push(Content&& c) {
  size_t k = pool_allocate();
  store(k, std::move(c));
  return k;
}

// ObjectPool::free (object_pool.rs:214-222).  A freed node's content is never
// read again by the reference (every read is behind key_is_valid), so its
// bricks are returned to the arena right away.
void HostOctree::pool_free(size_t k) {
  if (!key_valid(k)) return;
  reserved[k] = 0;
  first_available = std::min(first_available, k);
  Content dead = take(k);
  release(dead);
  touch(k);
}

void HostOctree::pool_swap(size_t a, size_t b) {  // object_pool.rs:234-236 swaps the whole item
  check_key(a);
  check_key(b);
  std::swap(reserved[a], reserved[b]);
  std::swap(kind[a], kind[b]);
  std::swap(ocbits[a], ocbits[b]);
  for (int i = 0; i < 8; ++i) std::swap(bricks[a * 8 + i], bricks[b * 8 + i]);
  touch(a);
  touch(b);
}

Content HostOctree::take(size_t k) {
  check_key(k);
  Content c;
  c.kind = kind[k];
  c.ocbits = ocbits[k];
  for (int i = 0; i < 8; ++i) {
    c.b[i] = bricks[k * 8 + i];
    bricks[k * 8 + i] = BrickRef{};
  }
  kind[k] = kNothing;
  ocbits[k] = 0;
  touch(k);
  return c;
}

void HostOctree::release(Content& c) {
  for (auto& b : c.b) {
    if (b.kind == kBrickParted) arena.release(b.v);
    b = BrickRef{};
  }
  c.kind = kNothing;
}

void HostOctree::store(size_t k, Content&& c) {
  Content old = take(k);
  release(old);
  kind[k] = c.kind;
  ocbits[k] = c.kind == kInternal ? c.ocbits : 0;
  const int n = c.kind == kLeaf ? 8 : (c.kind == kUniform ? 1 : 0);
  for (int i = 0; i < 8; ++i) {
    if (i < n) {
      bricks[k * 8 + i] = c.b[i];
    } else if (c.b[i].kind == kBrickParted) {
      arena.release(c.b[i].v);
    }
    c.b[i] = BrickRef{};
  }
  touch(k);
}

BrickRef HostOctree::clone_brick(const BrickRef& b) {
  BrickRef r = b;
  if (b.kind == kBrickParted) r.v = arena.clone(b.v);
  return r;
}

Content HostOctree::clone_content(size_t k) {
  Content c;
  c.kind = kind[k];
  c.ocbits = ocbits[k];
  const int n = c.kind == kLeaf ? 8 : (c.kind == kUniform ? 1 : 0);
  for (int i = 0; i < n; ++i) c.b[i] = clone_brick(bricks[k * 8 + i]);
  return c;
}

void HostOctree::set_children_none(size_t k) {
  ch_kind[k] = kNoChildren;
  ch_bitmap[k] = 0;
  touch(k);
}
void HostOctree::set_children_bitmap(size_t k, uint64_t bits) {
  ch_kind[k] = kBitmap;
  ch_bitmap[k] = bits;
  touch(k);
}
// NodeChildren::child_mut (src/octree/node.rs:40-48)
uint32_t* HostOctree::child_mut(size_t k, size_t index) {
  if (ch_kind[k] == kNoChildren) {
    ch_kind[k] = kChildren;
    for (int i = 0; i < 8; ++i) ch[k * 8 + i] = kEmpty32;
  }
  if (ch_kind[k] != kChildren) throw ReferencePanic("child_mut on an occupancy bitmap");
  touch(k);
  return &ch[k * 8 + index];
}
// NodeChildren::clear (node.rs:59-67)
void HostOctree::children_clear(size_t k, size_t index) {
  if (ch_kind[k] != kChildren) return;
  ch[k * 8 + index] = kEmpty32;
  bool all = true;
  for (int i = 0; i < 8; ++i) all &= ch[k * 8 + i] == kEmpty32;
  if (all) {
    ch_kind[k] = kNoChildren;
    for (int i = 0; i < 8; ++i) ch[k * 8 + i] = 0;
  }
  touch(k);
}

// ---------------------------------------------------------------- palettes
// pix_points_to_empty (src/octree/node.rs:357-379)
bool HostOctree::pix_empty(uint32_t p) const {
  const uint32_t c = pix_color(p), d = pix_data(p);
  if (c < kEmpty16) {
    if (c >= colors.size()) throw ReferencePanic("colour palette index out of bounds");
    if (!transparent(colors[c])) return false;
  }
  if (d == kEmpty16) return true;
  if (d >= datas.size()) throw ReferencePanic("data palette index out of bounds");
  return datas[d] == 0;
}

// pix_get_ref (node.rs:381-419)
Entry HostOctree::pix_entry(uint32_t p) const {
  Entry e;
  const uint32_t c = pix_color(p), d = pix_data(p);
  if (c < kEmpty16) {
    if (c >= colors.size()) throw ReferencePanic("colour palette index out of bounds");
    e.kind |= 1;
    e.rgba = colors[c];
  }
  if (d != kEmpty16) {
    if (d >= datas.size()) throw ReferencePanic("data palette index out of bounds");
    e.kind |= 2;
    e.user = datas[d];
  }
  return e;
}

uint32_t HostOctree::add_color(uint32_t rgba) {
  auto it = color_index_.find(rgba);
  if (it != color_index_.end()) return it->second;
  uint32_t i = (uint32_t)color_index_.size();
  color_index_.emplace(rgba, i);
  colors.push_back(rgba);
  return i;
}
uint32_t HostOctree::add_data(uint32_t v) {
  auto it = data_index_.find(v);
  if (it != data_index_.end()) return it->second;
  uint32_t i = (uint32_t)data_index_.size();
  data_index_.emplace(v, i);
  datas.push_back(v);
  return i;
}
// add_to_palette (src/octree/update/mod.rs:55-136)
uint32_t HostOctree::add_to_palette(const Entry& e) {
  switch (e.kind) {
    case 0:
      return kEmpty32;
    case 1:
      if (e.rgba == 0) return kEmpty32;
      return (add_color(e.rgba) & 0xFFFFu) | (kEmpty16 << 16);
    case 2:
      if (e.user == 0) return kEmpty32;
      return kEmpty16 | ((add_data(e.user) & 0xFFFFu) << 16);
    default:
      if (e.rgba == 0) return add_to_palette(Entry{2, 0, e.user});
      if (e.user == 0) return add_to_palette(Entry{1, e.rgba, 0});
      {
        uint32_t c = add_color(e.rgba);
        uint32_t d = add_data(e.user);
        return (c & 0xFFFFu) | ((d & 0xFFFFu) << 16);
      }
  }
}

// ---------------------------------------------------------------- bricks
// BrickData::get_homogeneous_data (node.rs:268-281)
bool HostOctree::brick_homogeneous(const BrickRef& b, uint32_t* out) const {
  if (b.kind == kBrickEmpty) return false;
  if (b.kind == kBrickSolid) {
    *out = b.v;
    return true;
  }
  const uint32_t* v = arena.at(b.v);
  const uint32_t first = v[0];
  uint32_t& hint = arena.differs_at(b.v);  // most bricks stay mixed across the checks of many inserts
  if (hint < arena.len() && v[hint] != first) return false;
  for (uint32_t i = 1; i < arena.len(); ++i)
    if (v[i] != first) {
      hint = i;
      return false;
    }
  *out = first;
  return true;
}
// BrickData::simplify (node.rs:284-299)
bool HostOctree::brick_simplify(BrickRef& b) {
  uint32_t h;
  if (!brick_homogeneous(b, &h)) return false;
  if (b.kind == kBrickParted) arena.release(b.v);
  if (pix_empty(h))
    b = BrickRef{};
  else
    b = BrickRef{kBrickSolid, h};
  return true;
}
bool HostOctree::brick_equal(const BrickRef& a, const BrickRef& b) const {  // derived PartialEq
  if (a.kind != b.kind) return false;
  if (a.kind == kBrickSolid) return a.v == b.v;
  if (a.kind == kBrickParted) return std::memcmp(arena.at(a.v), arena.at(b.v), sizeof(uint32_t) * arena.len()) == 0;
  return true;
}
// BrickData::is_empty_throughout (node.rs:75-146)
bool HostOctree::brick_empty_throughout(const BrickRef& b, uint8_t octant) const {
  if (b.kind == kBrickEmpty) return true;
  if (b.kind == kBrickSolid) return pix_empty(b.v);
  const uint32_t* v = arena.at(b.v);
  if (dim == 1) return pix_empty(v[0]);
  if (dim == 2) return pix_empty(v[flat3((uint64_t)off_x(octant), (uint64_t)off_y(octant), (uint64_t)off_z(octant), 2)]);
  const uint64_t e = dim / 2;
  const uint64_t ox = (uint64_t)off_x(octant) * e, oy = (uint64_t)off_y(octant) * e, oz = (uint64_t)off_z(octant) * e;
  for (uint64_t x = ox; x < ox + e; ++x)
    for (uint64_t y = oy; y < oy + e; ++y)
      for (uint64_t z = oz; z < oz + e; ++z)
        if (!pix_empty(v[flat3(x, y, z, dim)])) return false;
  return true;
}
// BrickData::is_part_empty_throughout (node.rs:152-209)
bool HostOctree::brick_part_empty_throughout(const BrickRef& b, uint8_t part, uint8_t target) const {
  if (b.kind == kBrickEmpty) return true;
  if (b.kind == kBrickSolid) return pix_empty(b.v);
  const uint32_t* v = arena.at(b.v);
  if (dim == 1) return pix_empty(v[0]);
  if (dim == 2) return pix_empty(v[flat3((uint64_t)off_x(part), (uint64_t)off_y(part), (uint64_t)off_z(part), 2)]);
  const float outer = (float)dim / 2.0f, inner = (float)dim / 4.0f;
  const uint64_t ox = round_usize(off_x(part) * outer + off_x(target) * inner);
  const uint64_t oy = round_usize(off_y(part) * outer + off_y(target) * inner);
  const uint64_t oz = round_usize(off_z(part) * outer + off_z(target) * inner);
  const uint64_t n = sat_usize(inner);
  for (uint64_t x = 0; x < n; ++x)
    for (uint64_t y = 0; y < n; ++y)
      for (uint64_t z = 0; z < n; ++z) {
        const uint64_t i = flat3(ox + x, oy + y, oz + z, dim);
        if (i >= arena.len()) throw ReferencePanic("brick index out of bounds");
        if (!pix_empty(v[i])) return false;
      }
  return true;
}
// BrickData::calculate_brick_occupied_bits (node.rs:212-240)
uint64_t HostOctree::brick_occupied_bits(const uint32_t* v) const {
  uint64_t bits = 0;
  for (uint64_t x = 0; x < dim; ++x)
    for (uint64_t y = 0; y < dim; ++y)
      for (uint64_t z = 0; z < dim; ++z)
        if (!pix_empty(v[flat3(x, y, z, dim)])) {
          const uint64_t p[3] = {x, y, z};
          set_occupancy(p, 1, dim, true, &bits);
        }
  return bits;
}
// BrickData::calculate_occupied_bits (node.rs:243-265)
uint64_t HostOctree::brick_ref_occupied_bits(const BrickRef& b) const {
  if (b.kind == kBrickEmpty) return 0;
  if (b.kind == kBrickSolid) return pix_empty(b.v) ? 0 : UINT64_MAX;
  return brick_occupied_bits(arena.at(b.v));
}

// dilute_brick_data (src/octree/update/mod.rs:531-596).  The source offset is
// `OCTANT_OFFSET * 2` for every brick size, as in the reference.
void HostOctree::dilute(uint32_t src_slot, uint32_t out[8]) {
  const uint32_t D = dim;
  // copy the source first: allocating the new slots may move the arena storage
  dilute_src_.assign(arena.at(src_slot), arena.at(src_slot) + arena.len());
  const uint32_t* src = dilute_src_.data();
  if (D == 1) {
    for (int o = 0; o < 8; ++o) out[o] = arena.alloc_fill(src[0]);
    return;
  }
  uint32_t first[8];
  for (int o = 0; o < 8; ++o) first[o] = src[o];
  for (int o = 0; o < 8; ++o) out[o] = arena.alloc_fill(first[o]);
  if (D == 2) return;
  for (uint32_t o = 0; o < 8; ++o) {
    const uint64_t bx = (uint64_t)off_x(o) * 2, by = (uint64_t)off_y(o) * 2, bz = (uint64_t)off_z(o) * 2;
    uint32_t* dst = arena.at(out[o]);
    const uint32_t fill = src[flat3(bx, by, bz, D)];
    std::fill(dst, dst + arena.len(), fill);
    for (uint64_t x = 0; x < D; ++x)
      for (uint64_t y = 0; y < D; ++y)
        for (uint64_t z = 0; z < D; ++z) {
          if (x < 2 && y < 2 && z < 2) continue;
          const uint64_t s = flat3(bx + x / 2, by + y / 2, bz + z / 2, D);
          if (s >= arena.len()) throw ReferencePanic("brick index out of bounds");
          dst[flat3(x, y, z, D)] = src[s];
        }
  }
}

// update_brick (src/octree/update/mod.rs:605-643)
size_t HostOctree::update_brick(bool overwrite, uint32_t slot, const Cube& bounds, const uint32_t pos[3],
                                uint32_t size_, uint32_t data) {
  uint64_t mi[3];
  matrix_index(bounds, pos, dim, mi);
  const size_t update_size = std::min<size_t>((size_t)dim - (size_t)mi[0], size_);
  uint32_t* v = arena.at(slot);
  arena.mark(slot);
  for (uint64_t x = mi[0]; x < std::min<uint64_t>(mi[0] + size_, dim); ++x)
    for (uint64_t y = mi[1]; y < std::min<uint64_t>(mi[1] + size_, dim); ++y)
      for (uint64_t z = mi[2]; z < std::min<uint64_t>(mi[2] + size_, dim); ++z) {
        uint32_t& cell = v[flat3(x, y, z, dim)];
        if (overwrite) {
          cell = data;
        } else {
          if (pix_color(data) < kEmpty16) cell = (cell & 0xFFFF0000u) | (data & 0xFFFFu);
          if (pix_data(data) != kEmpty16) cell = (cell & 0xFFFFu) | (data & 0xFFFF0000u);
        }
      }
  return update_size;
}

// ---------------------------------------------------------------- structure queries
// NodeContent::is_empty (node.rs:422-467)
bool HostOctree::content_is_empty(size_t k) const {
  auto brick_all_empty = [&](const BrickRef& b) {
    if (b.kind == kBrickEmpty) return true;
    if (b.kind == kBrickSolid) return pix_empty(b.v);
    const uint32_t* v = arena.at(b.v);
    for (uint32_t i = 0; i < arena.len(); ++i)
      if (!pix_empty(v[i])) return false;
    return true;
  };
  switch (kind[k]) {
    case kUniform: return brick_all_empty(bricks[k * 8]);
    case kLeaf:
      for (int i = 0; i < 8; ++i)
        if (!brick_all_empty(bricks[k * 8 + i])) return false;
      return true;
    case kInternal: return false;
    default: return true;
  }
}
// NodeContent::is_all (node.rs:470-504)
bool HostOctree::content_is_all(size_t k, uint32_t data) const {
  auto brick_all = [&](const BrickRef& b) {
    if (b.kind == kBrickEmpty) return false;
    if (b.kind == kBrickSolid) return b.v == data;
    uint32_t h;
    return brick_homogeneous(b, &h) && h == data;
  };
  if (kind[k] == kUniform) return brick_all(bricks[k * 8]);
  if (kind[k] == kLeaf) {
    for (int i = 0; i < 8; ++i)
      if (!brick_all(bricks[k * 8 + i])) return false;
    return true;
  }
  return false;
}
// NodeContent::compare (node.rs:506-525)
bool HostOctree::content_compare(size_t a, size_t b) const {
  switch (kind[a]) {
    case kNothing: return kind[b] == kNothing;
    case kInternal: return false;
    case kUniform: return kind[b] == kUniform && brick_equal(bricks[a * 8], bricks[b * 8]);
    default:
      if (kind[b] != kLeaf) return false;
      for (int i = 0; i < 8; ++i)
        if (!brick_equal(bricks[a * 8 + i], bricks[b * 8 + i])) return false;
      return true;
  }
}

// should_bitmap_be_empty_at_bitmap_index (src/octree/detail.rs:165-180)
bool HostOctree::should_bitmap_be_empty_at_index(size_t k, const uint64_t idx[3]) {
  const float px = 0.5f + (float)idx[0], py = 0.5f + (float)idx[1], pz = 0.5f + (float)idx[2];
  const uint8_t t = octant_of(px, py, pz, 4.0f / 2.0f);
  const uint8_t tc = octant_of(px - off_x(t) * 4.0f / 2.0f, py - off_y(t) * 4.0f / 2.0f, pz - off_z(t) * 4.0f / 2.0f,
                               4.0f / 4.0f);
  return should_bitmap_be_empty_at_octants(k, t, tc);
}
// should_bitmap_be_empty_at_octants (detail.rs:206-236)
bool HostOctree::should_bitmap_be_empty_at_octants(size_t k, uint8_t oct, uint8_t child_oct) {
  check_key(k);
  switch (kind[k]) {
    case kNothing: return true;
    case kInternal: {
      const uint64_t c = child(k, oct);
      return key_valid(c) ? node_empty_at(c, child_oct) : true;
    }
    case kUniform: return brick_part_empty_throughout(bricks[k * 8], oct, child_oct);
    default: return brick_empty_throughout(bricks[k * 8 + oct], child_oct);
  }
}
// node_empty_at (detail.rs:239-300)
bool HostOctree::node_empty_at(size_t k, uint8_t oct) {
  check_key(k);
  auto brick_empty = [&](const BrickRef& b) {
    if (b.kind == kBrickEmpty) return true;
    uint32_t h;
    if (brick_homogeneous(b, &h)) return pix_empty(h);
    return false;
  };
  switch (kind[k]) {
    case kNothing: return true;
    case kLeaf: return brick_empty(bricks[k * 8 + oct]);
    case kUniform: return brick_empty(bricks[k * 8]);
    default: {
      DepthGuard g(depth_);
      // detail.rs:289-296 queries child(target_octant) on every iteration
      for (uint8_t co = 0; co < 8; ++co) {
        const uint64_t c = child(k, oct);
        if (key_valid(c) && !node_empty_at(c, co)) return false;
      }
      return true;
    }
  }
}

// subdivide_leaf_to_nodes (detail.rs:305-470)
void HostOctree::subdivide_leaf_to_nodes(size_t k, size_t target_octant) {
  check_key(k);
  if (ch_kind[k] != kBitmap) throw ReferencePanic("subdivide: node has no occupancy bitmap");
  Content old = take(k);
  {
    Content internal;
    internal.kind = kInternal;
    internal.ocbits = ch_bitmap[k];
    store(k, std::move(internal));
  }
  uint32_t nn[8];
  std::fill(nn, nn + 8, kEmpty32);
  if (old.kind == kNothing || old.kind == kInternal) throw ReferencePanic("subdivide: node is not a leaf");
  if (old.kind == kLeaf) {
    for (size_t o = 0; o < 8; ++o) {
      BrickRef b = old.b[o];
      old.b[o] = BrickRef{};
      if (b.kind == kBrickEmpty) {
        if (o == target_octant) {
          nn[o] = (uint32_t)push(Content{});
          mips_resize();
        }
      } else if (b.kind == kBrickSolid) {
        Content u;
        u.kind = kUniform;
        u.b[0] = b;
        nn[o] = (uint32_t)push(std::move(u));
        mips_resize();
        set_children_bitmap(nn[o], UINT64_MAX);
      } else {
        // detail.rs:387-394 computes the bitmap from bricks[octant], already swapped out to Empty
        Content u;
        u.kind = kUniform;
        u.b[0] = b;
        nn[o] = (uint32_t)push(std::move(u));
        mips_resize();
        set_children_bitmap(nn[o], 0);
      }
    }
  } else {  // UniformLeaf
    BrickRef b = old.b[0];
    old.b[0] = BrickRef{};
    if (b.kind == kBrickEmpty) {
      nn[target_octant] = (uint32_t)push(Content{});
      mips_resize();
      set_children_bitmap(nn[target_octant], 0);
    } else if (b.kind == kBrickSolid) {
      for (size_t o = 0; o < 8; ++o) {
        Content u;
        u.kind = kUniform;
        u.b[0] = BrickRef{kBrickSolid, b.v};
        nn[o] = (uint32_t)push(std::move(u));  // node_mips is not resized here (detail.rs:432-447)
        set_children_bitmap(nn[o], UINT64_MAX);
      }
    } else {
      uint32_t slots[8];
      dilute(b.v, slots);
      arena.release(b.v);
      for (size_t o = 0; o < 8; ++o) {
        const uint64_t bits = brick_occupied_bits(arena.at(slots[o]));
        Content u;
        u.kind = kUniform;
        u.b[0] = BrickRef{kBrickParted, slots[o]};
        nn[o] = (uint32_t)push(std::move(u));
        mips_resize();
        set_children_bitmap(nn[o], bits);
      }
    }
  }
  release(old);
  ch_kind[k] = kChildren;
  for (int i = 0; i < 8; ++i) ch[k * 8 + i] = nn[i];
  touch(k);
}

// try_brick_from_node (detail.rs:473-484)
BrickRef HostOctree::try_brick_from_node(uint64_t k) {
  if (!key_valid(k)) return BrickRef{};
  if (kind[k] == kUniform) return clone_brick(bricks[k * 8]);
  return BrickRef{};
}

// deallocate_children_of (detail.rs:487-504)
void HostOctree::deallocate_children_of(uint64_t k) {
  if (!key_valid(k) || ch_kind[k] != kChildren) return;
  DepthGuard g(depth_);
  uint64_t kids[8];
  int n = 0;
  for (int i = 0; i < 8; ++i)
    if (key_valid(ch[k * 8 + i])) kids[n++] = ch[k * 8 + i];
  for (int i = 0; i < n; ++i) {
    deallocate_children_of(kids[i]);
    pool_free(kids[i]);
    set_children_none(kids[i]);
  }
}

// stored_occupied_bits (detail.rs:508-528)
uint64_t HostOctree::stored_occupied_bits(size_t k) const {
  check_key(k);
  switch (kind[k]) {
    case kLeaf:
    case kUniform: return ch_kind[k] == kBitmap ? ch_bitmap[k] : 0;
    case kNothing: return 0;
    default: return ocbits[k];
  }
}
// store_occupied_bits (detail.rs:531-553)
void HostOctree::store_occupied_bits(size_t k, uint64_t bits) {
  check_key(k);
  switch (kind[k]) {
    case kInternal:
      ocbits[k] = bits;
      touch(k);
      break;
    case kNothing: set_children_bitmap(k, bits); break;
    default:
      if (ch_kind[k] == kChildren) throw ReferencePanic("leaf node with children");
      set_children_bitmap(k, bits);
  }
}

// ---------------------------------------------------------------- leaf_update (update/mod.rs:136-525)
size_t HostOctree::leaf_update(bool overwrite, size_t k, const Cube& nb, const Cube& tb, size_t to,
                               const uint32_t pos[3], uint32_t sz, uint32_t target) {
  DepthGuard g(depth_);
  check_key(k);
  const uint32_t blen = arena.len();
  switch (kind[k]) {
    case kLeaf: {
      BrickRef& b = bricks[k * 8 + to];
      if (b.kind == kBrickEmpty) {
        uint32_t s = arena.alloc_fill(kEmpty32);
        size_t us = update_brick(overwrite, s, tb, pos, sz, target);
        bricks[k * 8 + to] = BrickRef{kBrickParted, s};
        touch(k);
        return us;
      }
      if (b.kind == kBrickSolid) {
        const uint32_t voxel = b.v;
        const bool te = pix_empty(target);
        if ((te && !pix_empty(voxel)) || (!te && voxel != target)) {
          uint32_t s = arena.alloc_fill(voxel);
          size_t us = update_brick(overwrite, s, tb, pos, sz, target);
          bricks[k * 8 + to] = BrickRef{kBrickParted, s};
          touch(k);
          return us;
        }
        return 0;
      }
      return update_brick(overwrite, b.v, tb, pos, sz, target);
    }
    case kUniform: {
      BrickRef& mat = bricks[k * 8];
      if (mat.kind == kBrickEmpty) {
        if (!pix_empty(target)) {
          Content leaf;
          leaf.kind = kLeaf;
          uint32_t s = arena.alloc_fill(add_to_palette(Entry{}));
          size_t us = update_brick(overwrite, s, tb, pos, sz, target);
          leaf.b[to] = BrickRef{kBrickParted, s};
          store(k, std::move(leaf));
          return us;
        }
        return leaf_update(overwrite, k, nb, tb, to, pos, sz, target);
      }
      if (mat.kind == kBrickSolid) {
        const uint32_t voxel = mat.v;
        const bool te = pix_empty(target);
        if (te && pix_empty(voxel)) {
          store(k, Content{});
          return 0;
        }
        if ((!te && voxel != target) || (te && !pix_empty(voxel))) {
          bricks[k * 8] = BrickRef{kBrickParted, arena.alloc_fill(voxel)};
          touch(k);
          return leaf_update(overwrite, k, nb, tb, to, pos, sz, target);
        }
        return 0;
      }
      // Parted
      const uint32_t slot = mat.v;
      uint64_t mi[3];
      matrix_index(nb, pos, dim, mi);
      const uint64_t fi = flat3(mi[0], mi[1], mi[2], dim);
      const bool te = pix_empty(target);
      if (1 < dim) {
        if (fi >= blen) throw ReferencePanic("brick index out of bounds");
        const uint32_t cur = arena.at(slot)[fi];
        if ((te && pix_empty(cur)) || (!te && cur == target)) return 0;
      }
      if (nb.size <= (float)dim && dim > 1) return update_brick(overwrite, slot, nb, pos, sz, target);
      Content leaf;
      leaf.kind = kLeaf;
      size_t us = 0;
      if (dim == 1) {
        for (int i = 0; i < 8; ++i) leaf.b[i] = BrickRef{kBrickParted, arena.clone(slot)};
        const uint32_t s = arena.clone(slot);
        us = update_brick(overwrite, s, tb, pos, sz, target);
        arena.release(leaf.b[to].v);
        leaf.b[to] = BrickRef{kBrickParted, s};
      } else {
        uint32_t kids[8];
        dilute(slot, kids);
        for (size_t o = 0; o < 8; ++o) {
          if (o == to) us = update_brick(overwrite, kids[o], tb, pos, sz, target);
          leaf.b[o] = BrickRef{kBrickParted, kids[o]};
        }
      }
      store(k, std::move(leaf));
      return us;
    }
    case kInternal: {
      // update/mod.rs:473-497: the children entry becomes the bitmap first, so
      // every gathered brick is Empty and the old children stay allocated.
      set_children_bitmap(k, ocbits[k]);
      Content leaf;
      leaf.kind = kLeaf;
      for (int i = 0; i < 8; ++i) leaf.b[i] = try_brick_from_node(child(k, (uint8_t)i));
      store(k, std::move(leaf));
      deallocate_children_of(k);
      return leaf_update(overwrite, k, nb, tb, to, pos, sz, target);
    }
    default: {  // Nothing (update/mod.rs:498-523)
      Content leaf;
      leaf.kind = kLeaf;
      for (int i = 0; i < 8; ++i) leaf.b[i] = try_brick_from_node(child(k, (uint8_t)i));
      store(k, std::move(leaf));
      deallocate_children_of(k);
      return leaf_update(overwrite, k, nb, tb, to, pos, sz, target);
    }
  }
}

// ---------------------------------------------------------------- simplify (update/mod.rs:649-1028)
bool HostOctree::simplify(uint64_t k) {
  if (!key_valid(k)) return false;
  DepthGuard g(depth_);
  switch (kind[k]) {
    case kNothing: return true;
    case kUniform: {
      BrickRef& b = bricks[k * 8];
      if (b.kind == kBrickEmpty) return true;
      if (b.kind == kBrickSolid) {
        if (pix_empty(b.v)) {
          store(k, Content{});
          set_children_none(k);
          return true;
        }
        return false;
      }
      bool s = brick_simplify(b);
      if (s) touch(k);
      return s;
    }
    case kLeaf: {
      bool simplified = false, uniform_solid = true, have = false;
      uint32_t value = 0;
      for (int o = 0; o < 8; ++o) {
        BrickRef& b = bricks[k * 8 + o];
        if (brick_simplify(b)) {
          simplified = true;
          touch(k);
        }
        if (uniform_solid) {
          if (b.kind == kBrickSolid) {
            if (have) {
              if (value != b.v) uniform_solid = false;
            } else {
              have = true;
              value = b.v;
            }
          } else {
            uniform_solid = false;
          }
        }
      }
      if (uniform_solid) {
        Content u;
        u.kind = kUniform;
        u.b[0] = BrickRef{kBrickSolid, value};
        store(k, std::move(u));
        return true;
      }
      // Leaf -> UniformLeaf when every brick downsamples losslessly (:860-995): first the test
      // alone (it fails for most leaves), then the downsampled brick
      const uint32_t D = dim, half = D / 2;
      bool uniform = true;
      for (uint32_t o = 0; o < 8 && uniform; ++o) {
        const BrickRef& b = bricks[k * 8 + o];
        if (b.kind != kBrickParted) {
          uniform &= brick_equal(b, bricks[k * 8]);
          continue;
        }
        const uint32_t* v = arena.at(b.v);
        auto cell_uniform = [&](uint64_t x, uint64_t y, uint64_t z) {
          const uint32_t c = v[flat3(x * 2, y * 2, z * 2, D)];
          return c == v[flat3(x * 2 + 1, y * 2, z * 2, D)] && c == v[flat3(x * 2, y * 2 + 1, z * 2, D)] &&
                 c == v[flat3(x * 2, y * 2, z * 2 + 1, D)] && c == v[flat3(x * 2 + 1, y * 2 + 1, z * 2, D)] &&
                 c == v[flat3(x * 2, y * 2 + 1, z * 2 + 1, D)] && c == v[flat3(x * 2 + 1, y * 2, z * 2 + 1, D)] &&
                 c == v[flat3(x * 2 + 1, y * 2 + 1, z * 2 + 1, D)];
        };
        uint32_t& hint = arena.mixed_cell(b.v);  // most bricks stay mixed across the checks of many inserts
        if (hint < half * half * half && !cell_uniform(hint % half, (hint / half) % half, hint / (half * half))) {
          uniform = false;
          continue;
        }
        for (uint64_t x = 0; x < half && uniform; ++x)
          for (uint64_t y = 0; y < half && uniform; ++y)
            for (uint64_t z = 0; z < half && uniform; ++z)
              if (!cell_uniform(x, y, z)) {
                uniform = false;
                hint = (uint32_t)(x + half * (y + half * z));
              }
      }
      if (uniform) {
        unified_.assign(arena.len(), kEmpty32);
        uint32_t* uv = unified_.data();
        for (uint32_t o = 0; o < 8; ++o) {
          const uint64_t ox = round_usize(off_x(o) * (float)half), oy = round_usize(off_y(o) * (float)half),
                         oz = round_usize(off_z(o) * (float)half);
          const BrickRef& b = bricks[k * 8 + o];
          if (b.kind == kBrickSolid) {
            for (uint64_t x = ox; x < ox + half; ++x)
              for (uint64_t y = oy; y < oy + half; ++y)
                for (uint64_t z = oz; z < oz + half; ++z) uv[flat3(x, y, z, D)] = b.v;
          } else if (b.kind == kBrickParted) {
            const uint32_t* v = arena.at(b.v);
            for (uint64_t x = 0; x < half; ++x)
              for (uint64_t y = 0; y < half; ++y)
                for (uint64_t z = 0; z < half; ++z) uv[flat3(ox + x, oy + y, oz + z, D)] = v[flat3(x * 2, y * 2, z * 2, D)];
          }
        }
        const uint32_t slot = arena.alloc();
        std::memcpy(arena.at(slot), unified_.data(), sizeof(uint32_t) * arena.len());
        Content u;
        u.kind = kUniform;
        u.b[0] = BrickRef{kBrickParted, slot};
        store(k, std::move(u));
        return true;
      }
      return simplified;
    }
    default: {  // Internal
      if (ocbits[k] == 0 || ch_kind[k] == kNoChildren) {
        store(k, Content{});
        return true;
      }
      if (ch_kind[k] != kChildren) return false;
      uint32_t kids[8];
      std::memcpy(kids, &ch[k * 8], sizeof(kids));
      simplify(kids[0]);
      if (!key_valid(kids[0])) {
        for (int i = 1; i < 8; ++i) simplify(kids[i]);
        return false;
      }
      for (int o = 1; o < 8; ++o) {
        simplify(kids[o]);
        if (!key_valid(kids[o]) || !content_compare(kids[0], kids[o])) return false;
      }
      pool_swap(k, kids[0]);
      const uint8_t nk = ch_kind[kids[0]];
      const uint64_t nbm = ch_bitmap[kids[0]];
      uint32_t nch[8];
      std::memcpy(nch, &ch[(size_t)kids[0] * 8], sizeof(nch));
      deallocate_children_of(k);
      ch_kind[k] = nk;
      ch_bitmap[k] = nbm;
      std::memcpy(&ch[k * 8], nch, sizeof(nch));
      touch(k);
      return true;
    }
  }
}

// ---------------------------------------------------------------- insert (update/insert.rs:99-388)
int HostOctree::insert_at_lod(bool overwrite, const uint32_t up[3], uint32_t isz, const Entry& data) {
  const Cube root{0.0f, 0.0f, 0.0f, (float)size};
  const float px = (float)up[0], py = (float)up[1], pz = (float)up[2];
  if (!contains(root, px, py, pz)) return 4;
  bool none;  // OctreeEntry::is_none (src/octree/mod.rs:97-104)
  switch (data.kind & 3) {
    case 0: none = true; break;
    case 1: none = transparent(data.rgba); break;
    case 2: none = data.user == 0; break;
    default: none = transparent(data.rgba) && data.user == 0;
  }
  if (none) return 0;
  std::vector<PathFrame>& stack = path_;  // reused: no allocation per operation
  stack.clear();
  stack.push_back({0u, root});
  size_t actual = 0;
  const uint32_t target = add_to_palette(data);
  for (;;) {
    const size_t cur = stack.back().key;
    const Cube cb = stack.back().b;
    check_key(cur);
    const uint8_t to = child_octant(cb, px, py, pz);
    const Cube tb = target_cube(cb, to);
    uint64_t tck = child(cur, to);
    if (isz > 1 && tb.size <= (float)isz && lex_le(px, py, pz, tb.x, tb.y, tb.z)) {
      if (kind[cur] == kLeaf || kind[cur] == kUniform) {
        subdivide_leaf_to_nodes(cur, to);
        tck = child(cur, to);
      }
      Content u;
      u.kind = kUniform;
      u.b[0] = BrickRef{kBrickSolid, target};
      if (key_valid(tck)) {
        deallocate_children_of(tck);
        store(tck, std::move(u));
        set_children_bitmap(tck, UINT64_MAX);
      } else {
        const uint32_t nk = (uint32_t)push(std::move(u));
        mips_resize();
        *child_mut(cur, to) = nk;
        set_children_bitmap(nk, UINT64_MAX);
      }
      actual = sat_usize(tb.size);
      break;
    }
    const Cube data_b = kind[cur] == kUniform ? cb : tb;
    if (data_b.size > (float)dim || key_valid(tck)) {
      if (key_valid(tck)) {
        stack.push_back({(uint32_t)child(cur, to), tb});
      } else if (kind[cur] == kLeaf || kind[cur] == kUniform) {
        bool match = false;
        const BrickRef& b = kind[cur] == kUniform ? bricks[cur * 8] : bricks[cur * 8 + to];
        if (b.kind == kBrickSolid) {
          match = b.v == target;
        } else if (b.kind == kBrickParted) {
          uint64_t mi[3];
          matrix_index(kind[cur] == kUniform ? cb : tb, up, dim, mi);
          const uint64_t fi = flat3(mi[0], mi[1], mi[2], dim);
          if (fi >= arena.len()) throw ReferencePanic("brick index out of bounds");
          match = arena.at(b.v)[fi] == target;
        }
        if (match || content_is_all(cur, target)) break;
        subdivide_leaf_to_nodes(cur, to);
        stack.push_back({(uint32_t)child(cur, to), tb});
      } else {
        if (kind[cur] == kNothing) {
          kind[cur] = kInternal;
          ocbits[cur] = 0;
          touch(cur);
        }
        const uint32_t nk = (uint32_t)push(Content{});
        mips_resize();
        *child_mut(cur, to) = nk;
        stack.push_back({nk, tb});
      }
    } else {
      actual = leaf_update(overwrite, cur, cb, tb, to, up, isz, target);
      break;
    }
  }
  // post-processing (insert.rs:318-386)
  bool simplifyable = auto_simplify;
  for (auto it = stack.rbegin(); it != stack.rend(); ++it) {
    const uint32_t k = it->key;
    const Cube nb = it->b;
    if (!key_valid(k)) continue;
    if (kind[k] == kNothing) {
      kind[k] = kInternal;
      ocbits[k] = 0;
      touch(k);
    }
    uint64_t bits = stored_occupied_bits(k);
    if (sat_usize(nb.size) == actual) {
      bits = UINT64_MAX;
    } else {
      const uint64_t rel[3] = {round_usize(px - nb.x), round_usize(py - nb.y), round_usize(pz - nb.z)};
      set_occupancy(rel, actual, sat_usize(nb.size), true, &bits);
    }
    store_occupied_bits(k, bits);
    update_mip(k, nb, up);  // insert.rs:370-371
    if (kind[k] == kLeaf || kind[k] == kUniform) {
      simplifyable = simplify(k);
      continue;
    }
    if (simplifyable) simplifyable = simplify(k);
  }
  return 0;
}

// ---------------------------------------------------------------- clear (update/clear.rs:47-340)
int HostOctree::clear_at_lod(const uint32_t up[3], uint32_t csz) {
  const Cube root{0.0f, 0.0f, 0.0f, (float)size};
  const float px = (float)up[0], py = (float)up[1], pz = (float)up[2];
  if (!contains(root, px, py, pz)) return 4;
  std::vector<PathFrame>& stack = path_;  // reused: no allocation per operation
  stack.clear();
  stack.push_back({0u, root});
  size_t actual = 0;
  for (;;) {
    const size_t cur = stack.back().key;
    const Cube cb = stack.back().b;
    check_key(cur);
    const uint8_t to = child_octant(cb, px, py, pz);
    const Cube tb = target_cube(cb, to);
    const uint64_t tck = child(cur, to);
    const uint32_t tmin[3] = {sat_u32(std::round(tb.x)), sat_u32(std::round(tb.y)), sat_u32(std::round(tb.z))};
    bool pos_le;
    if (up[0] != tmin[0])
      pos_le = up[0] < tmin[0];
    else if (up[1] != tmin[1])
      pos_le = up[1] < tmin[1];
    else
      pos_le = up[2] <= tmin[2];
    if (csz > 1 && tb.size <= (float)csz && pos_le && key_valid(tck)) {
      deallocate_children_of(tck);
      store(tck, Content{});
      set_children_none(tck);
      actual = sat_usize(tb.size);
      stack.push_back({(uint32_t)child(cur, to), tb});
      break;
    }
    if (tb.size > (float)std::max(csz, dim) || key_valid(tck)) {
      if (key_valid(tck)) {
        stack.push_back({(uint32_t)child(cur, to), tb});
      } else if (kind[cur] == kLeaf || kind[cur] == kUniform) {
        const BrickRef& b = kind[cur] == kUniform ? bricks[cur * 8] : bricks[cur * 8 + to];
        bool match;
        if (b.kind == kBrickEmpty) {
          match = true;
        } else if (b.kind == kBrickSolid) {
          match = pix_empty(b.v);
        } else {
          // clear.rs:128-140: index = position - round(current_bounds.min) in u32, unscaled
          const uint32_t ix = up[0] - sat_u32(std::round(cb.x)), iy = up[1] - sat_u32(std::round(cb.y)),
                         iz = up[2] - sat_u32(std::round(cb.z));
          const uint64_t fi = flat3(ix, iy, iz, dim);
          if (fi >= arena.len()) throw ReferencePanic("brick index out of bounds");
          match = pix_empty(arena.at(b.v)[fi]);
        }
        if (match || content_is_empty(cur)) break;
        subdivide_leaf_to_nodes(cur, to);
        stack.push_back({(uint32_t)child(cur, to), tb});
      } else {
        break;
      }
    } else {
      actual = leaf_update(true, cur, cb, tb, to, up, csz, kEmpty32);
      break;
    }
  }
  // post-processing (clear.rs:224-339)
  bool have_removed = false;
  PathFrame removed{0, Cube{0, 0, 0, 0}};
  if (!stack.empty()) {
    PathFrame last = stack.back();
    stack.pop_back();
    if (sat_usize(last.b.size) <= actual) {
      have_removed = true;
      removed = last;
    }
  }
  bool simplifyable = auto_simplify;
  for (auto it = stack.rbegin(); it != stack.rend(); ++it) {
    const uint32_t k = it->key;
    const Cube nb = it->b;
    check_key(k);
    if (have_removed) {
      const uint8_t co = octant_of((removed.b.x - nb.x) + removed.b.size / 2.0f,
                                   (removed.b.y - nb.y) + removed.b.size / 2.0f,
                                   (removed.b.z - nb.z) + removed.b.size / 2.0f, nb.size / 2.0f);
      children_clear(k, co);
      pool_free(removed.key);
      have_removed = false;
    }
    const uint64_t previous = stored_occupied_bits(k);
    uint64_t bits = ch_kind[k] == kNoChildren ? 0 : previous;
    if (sat_usize(nb.size) == actual) {
      bits = 0;
    } else {
      uint64_t s[3];
      matrix_index(nb, up, 4, s);
      const uint64_t n = sat_usize(std::ceil((float)actual * 4.0f / nb.size));
      for (uint64_t x = s[0]; x < std::min<uint64_t>(s[0] + n, 4); ++x)
        for (uint64_t y = s[1]; y < std::min<uint64_t>(s[1] + n, 4); ++y)
          for (uint64_t z = s[2]; z < std::min<uint64_t>(s[2] + n, 4); ++z) {
            const uint64_t idx[3] = {x, y, z};
            if (should_bitmap_be_empty_at_index(k, idx)) set_occupancy(idx, 1, 4, false, &bits);
          }
    }
    if (bits != 0 && ch_kind[k] == kChildren) {
      Content c;
      c.kind = kInternal;
      c.ocbits = bits;
      store(k, std::move(c));
    } else {
      deallocate_children_of(k);
      set_children_none(k);
      have_removed = true;
      removed = PathFrame{k, nb};
      store(k, Content{});
    }
    if (bits == 0)
      set_children_none(k);
    else
      store_occupied_bits(k, bits);
    update_mip(k, nb, up);  // clear.rs:334-335
    if (simplifyable) simplifyable = simplify(k);
    if (previous == bits) break;
  }
  return 0;
}

// ---------------------------------------------------------------- get (src/octree/mod.rs:209-371)
Entry HostOctree::get(const uint32_t up[3]) { return get_internal(0, Cube{0.0f, 0.0f, 0.0f, (float)size}, up); }

// get_internal (mod.rs:219-371): the entry at a position within node k's bounds
Entry HostOctree::get_internal(size_t cur, Cube cb, const uint32_t up[3]) {
  const float px = (float)up[0], py = (float)up[1], pz = (float)up[2];
  if (!contains(cb, px, py, pz)) return Entry{};
  for (;;) {
    check_key(cur);
    switch (kind[cur]) {
      case kNothing: return Entry{};
      case kLeaf: {
        const uint8_t o = child_octant(cb, px, py, pz);
        const BrickRef& b = bricks[cur * 8 + o];
        if (b.kind == kBrickEmpty) return Entry{};
        if (b.kind == kBrickSolid) return pix_entry(b.v);
        const float h = cb.size / 2.0f;
        const Cube c{cb.x + off_x(o) * h, cb.y + off_y(o) * h, cb.z + off_z(o) * h, h};
        uint64_t mi[3];
        matrix_index(c, up, dim, mi);
        const uint64_t fi = flat3(mi[0], mi[1], mi[2], dim);
        if (fi >= arena.len()) throw ReferencePanic("brick index out of bounds");
        const uint32_t p = arena.at(b.v)[fi];
        return pix_empty(p) ? Entry{} : pix_entry(p);
      }
      case kUniform: {
        const BrickRef& b = bricks[cur * 8];
        if (b.kind == kBrickEmpty) return Entry{};
        uint32_t p = b.v;
        if (b.kind == kBrickParted) {
          uint64_t mi[3];
          matrix_index(cb, up, dim, mi);
          const uint64_t fi = flat3(mi[0], mi[1], mi[2], dim);
          if (fi >= arena.len()) throw ReferencePanic("brick index out of bounds");
          p = arena.at(b.v)[fi];
        }
        return pix_empty(p) ? Entry{} : pix_entry(p);
      }
      default: {
        const uint8_t o = child_octant(cb, px, py, pz);
        const uint64_t c = child(cur, o);
        if (!key_valid(c)) return Entry{};
        cur = c;
        const float h = cb.size / 2.0f;
        cb = Cube{cb.x + off_x(o) * h, cb.y + off_y(o) * h, cb.z + off_z(o) * h, h};
      }
    }
  }
}


// ---------------------------------------------------------------- MIP maps (src/octree/mipmap.rs)
namespace {

uint32_t sat_u8(float v) {  // `f32 as u8`
  if (!(v > 0.0f)) return 0;
  if (v >= 255.0f) return 255;
  return (uint32_t)v;
}
uint32_t round_u32(float v) { return sat_u32(std::round(v)); }  // `f32.round() as u32`

// Albedo::distance_from (detail.rs:82-89)
float albedo_distance(uint32_t a, uint32_t b) {
  const float dr = (float)(a >> 24) - (float)(b >> 24), dg = (float)((a >> 16) & 0xFFu) - (float)((b >> 16) & 0xFFu);
  const float db = (float)((a >> 8) & 0xFFu) - (float)((b >> 8) & 0xFFu), da = (float)(a & 0xFFu) - (float)(b & 0xFFu);
  return std::sqrt(((dr * dr + dg * dg) + db * db) + da * da);
}

// MIPResaplingFunction::execute (mipmap.rs:131-273) over size^3 cells from start, x outermost.  The
// reference keeps PointFilter and Posterize candidates in a HashMap whose iteration order Rust
// randomises per process, so the winner among equally frequent colours (and, for Posterize, which
// of several matching groups a colour joins) is not defined by it; candidates are kept here in
// first-seen order and the first one with the highest count wins.
template <class F>
bool mip_resample(HostOctree::MipSampler sampler, const uint32_t start[3], uint32_t size, F&& sample, uint32_t* out) {
  const uint32_t method = sampler.method;
  if (method == HostOctree::kMipBox) {
    bool any = false;
    uint32_t count = 0;
    float acc[4] = {0, 0, 0, 0};
    for (uint32_t x = start[0]; x < start[0] + size; ++x)
      for (uint32_t y = start[1]; y < start[1] + size; ++y)
        for (uint32_t z = start[2]; z < start[2] + size; ++z) {
          uint32_t c;
          if (!sample(x, y, z, &c)) continue;
          const float v[4] = {(float)(c >> 24), (float)((c >> 16) & 0xFFu), (float)((c >> 8) & 0xFFu), (float)(c & 0xFFu)};
          ++count;
          for (int k = 0; k < 4; ++k) acc[k] = any ? acc[k] + v[k] * v[k] : v[k] * v[k];  // powf(2.) == v * v
          any = true;
        }
    if (!any) return false;
    uint32_t ch[4];
    for (int k = 0; k < 4; ++k) ch[k] = sat_u8(std::fmin(std::sqrt(acc[k] / (float)count), 255.0f));
    *out = (ch[0] << 24) | (ch[1] << 16) | (ch[2] << 8) | ch[3];
    return true;
  }
  if (method == HostOctree::kMipPoint || method == HostOctree::kMipPointBD) {
    std::vector<std::pair<uint32_t, uint32_t>> counts;
    for (uint32_t x = start[0]; x < start[0] + size; ++x)
      for (uint32_t y = start[1]; y < start[1] + size; ++y)
        for (uint32_t z = start[2]; z < start[2] + size; ++z) {
          uint32_t c;
          if (!sample(x, y, z, &c)) continue;
          auto it = std::find_if(counts.begin(), counts.end(), [&](const std::pair<uint32_t, uint32_t>& e) { return e.first == c; });
          if (it == counts.end())
            counts.push_back({c, 1});
          else
            ++it->second;
        }
    if (counts.empty()) return false;
    size_t best = 0;
    for (size_t i = 1; i < counts.size(); ++i)
      if (counts[i].second > counts[best].second) best = i;
    *out = counts[best].first;
    return true;
  }
  // Posterize / PosterizeBD: groups of squared channel sums (Albedou32, u32 arithmetic wrapping
  // like the release build)
  struct Group {
    uint32_t sum[4];
    uint32_t count;
  };
  auto poster = [](const Group& g, int k) { return round_u32(std::sqrt((float)round_u32((float)g.sum[k] / (float)g.count))); };
  std::vector<Group> groups;
  for (uint32_t x = start[0]; x < start[0] + size; ++x)
    for (uint32_t y = start[1]; y < start[1] + size; ++y)
      for (uint32_t z = start[2]; z < start[2] + size; ++z) {
        uint32_t c;
        if (!sample(x, y, z, &c)) continue;
        const uint32_t v[4] = {c >> 24, (c >> 16) & 0xFFu, (c >> 8) & 0xFFu, c & 0xFFu};
        bool joined = false;
        for (Group& g : groups) {
          uint32_t d[4];
          for (int k = 0; k < 4; ++k) d[k] = poster(g, k) - v[k];
          if (std::sqrt((float)(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + d[3] * d[3])) < sampler.thr * 255.0f) {
            for (int k = 0; k < 4; ++k) g.sum[k] += v[k] * v[k];
            ++g.count;
            joined = true;
            break;
          }
        }
        if (!joined) groups.push_back(Group{{v[0] * v[0], v[1] * v[1], v[2] * v[2], v[3] * v[3]}, 1});
      }
  if (groups.empty()) return false;
  size_t best = 0;
  for (size_t i = 1; i < groups.size(); ++i)
    if (groups[i].count > groups[best].count) best = i;
  uint32_t ch[4];
  for (int k = 0; k < 4; ++k) ch[k] = std::min<uint32_t>(poster(groups[best], k), 255);
  *out = (ch[0] << 24) | (ch[1] << 16) | (ch[2] << 8) | ch[3];
  return true;
}

}  // namespace

void HostOctree::set_mip(size_t k, BrickRef b) {
  BrickRef& m = mip(k);
  if (m.kind == kBrickParted && !(b.kind == kBrickParted && b.v == m.v)) arena.release(m.v);
  m = b;
  touch(k);
}

// Octree::update_mip (mipmap.rs:309-577)
void HostOctree::update_mip(size_t k, const Cube& nb, const uint32_t up[3]) {
  if (!mips_enabled) return;
  const size_t level = sat_usize(std::log2(nb.size / (float)dim));
  const MipSampler* found = nullptr;
  for (const auto& e : mip_methods)
    if (e.first == level) found = &e.second;
  const bool dominant_bottom = found && found->method == kMipPointBD;
  const MipSampler sampler = found ? *found : MipSampler{kMipBox, 0.0f};
  check_key(k);
  uint32_t start[3] = {0, 0, 0}, ssize = 0;
  switch (kind[k]) {
    case kNothing: return;
    case kUniform:  // a UniformLeaf's content is its own MIP
      if (mip(k).kind != kBrickEmpty) set_mip(k, BrickRef{});
      return;
    case kLeaf: {
      ssize = std::min<uint32_t>(sat_u32(nb.size) / dim, dim * 2);
      for (int a = 0; a < 3; ++a)
        start[a] = round_u32(std::floor((float)((up[a] - up[a] % ssize) * 2 * dim) / nb.size));
      break;
    }
    default:
      if (dominant_bottom) {
        ssize = sat_u32(nb.size) / dim;
        for (int a = 0; a < 3; ++a) start[a] = up[a] - up[a] % ssize;
      } else {
        ssize = 2;
        const float mn[3] = {nb.x, nb.y, nb.z};
        for (int a = 0; a < 3; ++a) {
          const uint32_t v = round_u32(std::floor(((float)up[a] - mn[a]) * 2.0f * (float)dim / nb.size));
          start[a] = v - v % 2;
        }
      }
  }
  uint32_t color = 0;
  bool sampled = false;
  if (kind[k] == kLeaf || dominant_bottom) {
    sampled = mip_resample(sampler, start, ssize, [&](uint32_t x, uint32_t y, uint32_t z, uint32_t* c) {
      const uint32_t p[3] = {x, y, z};
      const Entry e = get_internal(k, nb, p);
      if (!(e.kind & 1u)) return false;
      *c = e.rgba;
      return true;
    }, &color);
  } else {
    const float D = (float)dim;
    if (child(k, octant_of((float)start[0], (float)start[1], (float)start[2], D)) != kEmpty32) {
      sampled = mip_resample(sampler, start, ssize, [&](uint32_t x, uint32_t y, uint32_t z, uint32_t* c) {
        const uint8_t o = octant_of((float)x, (float)y, (float)z, D);
        const uint64_t ck = child(k, o);
        if (ck == kEmpty32) return false;
        const uint32_t q[3] = {x - round_u32(off_x(o) * D), y - round_u32(off_y(o) * D), z - round_u32(off_z(o) * D)};
        const BrickRef& m = mip(ck);
        uint32_t p;
        if (m.kind == kBrickEmpty) return false;
        if (m.kind == kBrickSolid) {
          p = m.v;
        } else {
          const uint64_t fi = flat3(q[0], q[1], q[2], dim);
          if (fi >= arena.len()) throw ReferencePanic("MIP brick index out of bounds");
          p = arena.at(m.v)[fi];
        }
        const Entry e = pix_entry(p);
        if (!(e.kind & 1u)) return false;
        *c = e.rgba;
        return true;
      }, &color);
    }
  }
  if (!sampled) return;
  // the MIP entry: a similar palette colour, or the colour added to the palette (:519-545)
  uint32_t entry = kEmpty32;
  const float* thr = nullptr;
  for (const auto& e : mip_color_thr)
    if (e.first == level) thr = &e.second;
  bool similar = false;
  if (thr) {
    const float limit = *thr * 255.0f;
    for (size_t i = 0; i < colors.size(); ++i)
      if (albedo_distance(color, colors[i]) < limit) {
        entry = (uint32_t)(uint16_t)i | (kEmpty16 << 16);  // pix_visual
        similar = true;
        break;
      }
  }
  if (!similar) {
    Entry e;
    e.kind = 1;
    e.rgba = color;
    entry = add_to_palette(e);
  }
  uint64_t mi[3];
  matrix_index(nb, up, dim, mi);
  const uint64_t fi = flat3(mi[0], mi[1], mi[2], dim);
  BrickRef& m = mip(k);
  if (fi >= arena.len()) throw ReferencePanic("MIP brick index out of bounds");
  if (m.kind == kBrickParted) {
    arena.at(m.v)[fi] = entry;
    arena.mark(m.v);
  } else {
    const uint32_t slot = arena.alloc_fill(m.kind == kBrickSolid ? m.v : kEmpty32);
    arena.at(slot)[fi] = entry;
    set_mip(k, BrickRef{kBrickParted, slot});
  }
  touch(k);
}

// StrategyUpdater::recalculate_mip (mipmap.rs:882-899)
void HostOctree::recalculate_mip(size_t k, const Cube& b) {
  if (!mips_enabled) return;
  const float D = (float)dim;
  for (uint32_t x = 0; x < dim; ++x)
    for (uint32_t y = 0; y < dim; ++y)
      for (uint32_t z = 0; z < dim; ++z) {
        const uint32_t p[3] = {round_u32(b.x + std::round((float)x * b.size / D)),
                               round_u32(b.y + std::round((float)y * b.size / D)),
                               round_u32(b.z + std::round((float)z * b.size / D))};
        update_mip(k, b, p);
      }
}

// StrategyUpdater::recalculate_mips (mipmap.rs:798-856)
void HostOctree::recalculate_mips() {
  for (BrickRef& m : mips)
    if (m.kind == kBrickParted) arena.release(m.v);
  mips.assign(nodes(), BrickRef{});
  std::fill(node_dirty.begin(), node_dirty.end(), 1);
  struct Frame {
    size_t key;
    Cube b;
    uint32_t octant;
  };
  std::vector<Frame> st{{0, Cube{0.0f, 0.0f, 0.0f, (float)size}, 0}};
  while (!st.empty()) {
    Frame& top = st.back();
    if (top.octant == 8) {
      const Frame done = top;
      recalculate_mip(done.key, done.b);
      st.pop_back();
      if (!st.empty()) st.back().octant += 1;
      continue;
    }
    check_key(top.key);
    if (kind[top.key] == kNothing) throw ReferencePanic("BFS shouldn't evaluate empty children");
    if (kind[top.key] == kInternal) {
      const uint64_t ck = child(top.key, (uint8_t)top.octant);
      if (key_valid(ck) && kind[ck] != kNothing) {
        const float h = top.b.size / 2.0f;
        const uint8_t o = (uint8_t)top.octant;
        const Frame next{(size_t)ck, Cube{top.b.x + off_x(o) * h, top.b.y + off_y(o) * h, top.b.z + off_z(o) * h, h}, 0};
        st.push_back(next);
      } else {
        top.octant += 1;
      }
    } else {
      top.octant = 8;
    }
  }
}

// StrategyUpdater::switch_albedo_mip_maps (mipmap.rs:858-880)
void HostOctree::switch_albedo_mip_maps(bool enabled) {
  const bool before = mips_enabled;
  mips_enabled = enabled;
  if (mips_enabled && before != enabled && kind[0] != kNothing) recalculate_mips();
}

void HostOctree::set_mip_method(uint32_t level, uint32_t method, float thr) {
  if (method >= kMipPosterize) thr = std::min(std::max(thr, 0.0f), 1.0f);  // set_method_at_internal
  for (auto& e : mip_methods)
    if (e.first == level) {
      e.second = MipSampler{method, thr};
      return;
    }
  mip_methods.push_back({level, MipSampler{method, thr}});
}

void HostOctree::set_mip_color_threshold(uint32_t level, float thr) {
  thr = std::min(std::max(thr, 0.0f), 1.0f);  // set_color_similarity_thr_internal
  for (auto& e : mip_color_thr)
    if (e.first == level) {
      e.second = thr;
      return;
    }
  mip_color_thr.push_back({level, thr});
}

// StrategyUpdater::sample_root_mip (mipmap.rs:905-937)
Entry HostOctree::sample_root_mip(uint8_t octant, const uint32_t p[3]) {
  const uint64_t key = octant == 8 ? 0 : child(0, octant);
  if (!key_valid(key)) return Entry{};
  const BrickRef& m = mip(key);
  if (m.kind == kBrickEmpty) return Entry{};
  if (m.kind == kBrickSolid) return pix_entry(m.v);
  const uint64_t fi = flat3(p[0], p[1], p[2], dim);
  if (fi >= arena.len()) throw ReferencePanic("MIP brick index out of bounds");
  return pix_entry(arena.at(m.v)[fi]);
}

// Canonical per-node record (same layout as the oracle's orc_node_record).
void HostOctree::node_record(uint64_t key, uint64_t rec[40]) const {
  std::memset(rec, 0, sizeof(uint64_t) * 40);
  if (key >= reserved.size()) return;
  rec[0] = reserved[key];
  rec[1] = kind[key];
  rec[2] = kind[key] == kInternal ? ocbits[key] : 0;
  rec[3] = ch_kind[key];
  for (int i = 0; i < 8; ++i) rec[4 + i] = ch_kind[key] == kChildren ? ch[key * 8 + i] : 0;
  rec[12] = ch_kind[key] == kBitmap ? ch_bitmap[key] : 0;
  const int n = kind[key] == kLeaf ? 8 : (kind[key] == kUniform ? 1 : 0);
  for (int i = 0; i < n; ++i) {
    const BrickRef& b = bricks[key * 8 + i];
    // the oracle numbers brick kinds Empty 0, Parted 1, Solid 2 (declaration order of BrickData)
    rec[13 + i] = b.kind == kBrickEmpty ? 0 : (b.kind == kBrickParted ? 1 : 2);
    rec[21 + i] = b.kind == kBrickSolid ? b.v : 0;
    if (b.kind == kBrickParted) {
      uint64_t h = 1469598103934665603ull;
      const uint32_t* v = arena.at(b.v);
      for (uint32_t j = 0; j < arena.len(); ++j)
        for (int s = 0; s < 4; ++s) {
          h ^= (v[j] >> (8 * s)) & 0xFFu;
          h *= 1099511628211ull;
        }
      rec[29 + i] = h ^ arena.len();
    }
  }
  // the node's MIP brick: kind (numbered like the bricks, 3 = past node_mips), solid value, hash
  if (key >= mips.size()) {
    rec[37] = 3;
  } else {
    const BrickRef& m = mips[key];
    rec[37] = m.kind == kBrickEmpty ? 0 : (m.kind == kBrickParted ? 1 : 2);
    rec[38] = m.kind == kBrickSolid ? m.v : 0;
    if (m.kind == kBrickParted) {
      uint64_t h = 1469598103934665603ull;
      const uint32_t* v = arena.at(m.v);
      for (uint32_t j = 0; j < arena.len(); ++j)
        for (int s = 0; s < 4; ++s) {
          h ^= (v[j] >> (8 * s)) & 0xFFu;
          h *= 1099511628211ull;
        }
      rec[39] = h ^ arena.len();
    }
  }
}

}  // namespace svo
