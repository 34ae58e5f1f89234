// svo_oracle.cpp -- TEST INFRASTRUCTURE ONLY: CPU oracle for the sparse voxel
// octree ray cast.
//
// A plain restatement of shocovox-rs v0.11.1 (Rust) in C++17, release
// semantics (debug_assert! disabled, MIP maps disabled, user data T = u32).
// Every function cites the reference file:line it follows.  Where the
// reference would panic (slice index out of bounds, unbounded recursion) the
// oracle throws `Panic`, which the C interface reports as
// ORC_ERR_REFERENCE_PANIC (or ray status 3 inside the cast).
//
// Build flags matter: -O2 -ffp-contract=off -fno-fast-math so that every f32
// operation rounds exactly like the Rust code (Rust never contracts a*b+c).

#include "svo_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <atomic>
#include <map>
#include <thread>
#include <unordered_map>
#include <vector>

namespace orc {

struct Panic : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct OctreeError {
  int code;
};

constexpr uint32_t EMPTY_U32 = 0xFFFFFFFFu;  // object_pool.rs:14-16 empty_marker::<u32>()
constexpr uint32_t EMPTY_U16 = 0xFFFFu;      // empty_marker::<u16>()
constexpr float FLOAT_ERROR_TOLERANCE = 0.00001f;  // spatial/raytracing/mod.rs:5
constexpr uint8_t OOB_OCTANT = 8;                  // spatial/lut.rs:154
constexpr uint64_t BITMAP_DIMENSION = 4;           // spatial/math/mod.rs:39

// ---------------------------------------------------------------------------
// Rust f32 / integer semantics (Rust core library behaviour, restated)
// ---------------------------------------------------------------------------
// f32::min / f32::max ignore a NaN operand.  Ties (including +0/-0) keep the
// first operand.
static inline float rmin(float a, float b) {
  if (std::isnan(a)) return b;
  if (std::isnan(b)) return a;
  return (b < a) ? b : a;
}
static inline float rmax(float a, float b) {
  if (std::isnan(a)) return b;
  if (std::isnan(b)) return a;
  return (b > a) ? b : a;
}
// f32::signum: +-1 with the sign of the operand (also for +-0 and +-inf), NaN for NaN.
static inline float rsignum(float x) { return std::isnan(x) ? x : std::copysign(1.0f, x); }
// f32::clamp(min, max)
static inline float rclamp(float x, float lo, float hi) {
  if (x < lo) x = lo;
  if (x > hi) x = hi;
  return x;
}
// `x as i32`: truncation toward zero, saturating, NaN -> 0.
static inline int32_t as_i32(float x) {
  if (std::isnan(x)) return 0;
  if (x >= 2147483648.0f) return INT32_MAX;
  if (x <= -2147483648.0f) return INT32_MIN;
  return (int32_t)x;
}
// `x as usize` / `x as u32`: truncation, saturating at 0 and the type max, NaN -> 0.
static inline uint64_t as_usize(float x) {
  if (std::isnan(x) || x <= 0.0f) return 0;
  if (x >= 18446744073709551616.0f) return UINT64_MAX;
  return (uint64_t)x;
}
static inline uint32_t as_u32(float x) {
  if (std::isnan(x) || x <= 0.0f) return 0;
  if (x >= 4294967296.0f) return UINT32_MAX;
  return (uint32_t)x;
}
static inline int32_t isignum(int32_t v) { return (v > 0) - (v < 0); }

// ---------------------------------------------------------------------------
// V3c<f32> (spatial/math/vector.rs)
// ---------------------------------------------------------------------------
struct V3f {
  float x, y, z;
};
static inline V3f v3(float x, float y, float z) { return V3f{x, y, z}; }
static inline V3f unit(float s) { return V3f{s, s, s}; }                                   // vector.rs:21-27
static inline V3f operator+(V3f a, V3f b) { return V3f{a.x + b.x, a.y + b.y, a.z + b.z}; }  // :195-205
static inline V3f operator-(V3f a, V3f b) { return V3f{a.x - b.x, a.y - b.y, a.z - b.z}; }  // :207-220
static inline V3f operator*(V3f a, float s) { return V3f{a.x * s, a.y * s, a.z * s}; }      // :222-232
static inline V3f operator*(V3f a, V3f b) { return V3f{a.x * b.x, a.y * b.y, a.z * b.z}; }  // :234-244
static inline V3f operator/(V3f a, float s) { return V3f{a.x / s, a.y / s, a.z / s}; }      // :246-256
static inline float length(V3f v) { return std::sqrt((v.x * v.x) + (v.y * v.y) + (v.z * v.z)); }  // :75-77
static inline V3f normalized(V3f v) { return v / length(v); }                                     // :79-81
static inline V3f vfloor(V3f v) { return V3f{std::floor(v.x), std::floor(v.y), std::floor(v.z)}; }
// vector.rs:66-71 modulo (f32 `%` is fmod)
static inline V3f vmodulo(V3f v, float m) { return V3f{std::fmod(v.x, m), std::fmod(v.y, m), std::fmod(v.z, m)}; }

struct V3u {
  uint64_t x, y, z;
};
// From<V3c<f32>> for V3c<usize> rounds half away from zero (vector.rs:306-316)
static inline V3u to_usize_round(V3f v) {
  return V3u{as_usize(std::round(v.x)), as_usize(std::round(v.y)), as_usize(std::round(v.z))};
}
// From<V3c<f32>> for V3c<u32> (vector.rs:326-336)
static inline void to_u32_round(V3f v, uint32_t out[3]) {
  out[0] = as_u32(std::round(v.x));
  out[1] = as_u32(std::round(v.y));
  out[2] = as_u32(std::round(v.z));
}
// derived PartialOrd on V3c compares fields lexicographically (x, y, z)
static inline bool lex_le(V3f a, V3f b) {
  if (a.x != b.x) return a.x < b.x;
  if (a.y != b.y) return a.y < b.y;
  return a.z <= b.z;
}
static inline bool lex_le_u32(const uint32_t a[3], const uint32_t b[3]) {
  if (a[0] != b[0]) return a[0] < b[0];
  if (a[1] != b[1]) return a[1] < b[1];
  return a[2] <= b[2];
}

// ---------------------------------------------------------------------------
// Look-up tables (spatial/lut.rs); generated with the reference's generators
// ---------------------------------------------------------------------------
// lut.rs:156-197
static const V3f OCTANT_OFFSET_REGION_LUT[8] = {{0, 0, 0}, {1, 0, 0}, {0, 0, 1}, {1, 0, 1},
                                                {0, 1, 0}, {1, 1, 0}, {0, 1, 1}, {1, 1, 1}};

static uint64_t flat_projection(uint64_t x, uint64_t y, uint64_t z, uint64_t size) {  // math/mod.rs:35-37
  return x + (y * size) + (z * size * size);
}
// math/mod.rs:82-106
static uint64_t position_in_bitmap_64bits(V3u i, uint64_t brick_size) {
  return flat_projection(i.x * BITMAP_DIMENSION / brick_size, i.y * BITMAP_DIMENSION / brick_size,
                         i.z * BITMAP_DIMENSION / brick_size, BITMAP_DIMENSION);
}
// math/mod.rs:114-162
static void set_occupancy_in_bitmap_64bits(V3u position, uint64_t size, uint64_t brick_dim, bool occupied,
                                           uint64_t* bitmap) {
  if (brick_dim == 1) {
    *bitmap = occupied ? UINT64_MAX : 0;
    return;
  }
  uint64_t update_count = as_usize(std::ceil((float)size * (float)BITMAP_DIMENSION / (float)brick_dim));
  V3f start_f = vfloor(V3f{(float)(position.x * BITMAP_DIMENSION), (float)(position.y * BITMAP_DIMENSION),
                           (float)(position.z * BITMAP_DIMENSION)} /
                       (float)brick_dim);
  V3u start = to_usize_round(start_f);
  for (uint64_t x = start.x; x < std::min(start.x + update_count, BITMAP_DIMENSION); ++x)
    for (uint64_t y = start.y; y < std::min(start.y + update_count, BITMAP_DIMENSION); ++y)
      for (uint64_t z = start.z; z < std::min(start.z + update_count, BITMAP_DIMENSION); ++z) {
        uint64_t pos_mask = 1ull << position_in_bitmap_64bits(V3u{x, y, z}, BITMAP_DIMENSION);
        if (occupied)
          *bitmap |= pos_mask;
        else
          *bitmap &= ~pos_mask;
      }
}

// math/mod.rs:11-19
static uint8_t hash_region(V3f offset, float size_half) {
  return (uint8_t)((offset.x >= size_half) + (offset.z >= size_half) * 2 + (offset.y >= size_half) * 4);
}
// math/mod.rs:22-26
static uint8_t hash_direction(V3f direction) { return hash_region(unit(1.0f) + direction, 1.0f); }

struct Luts {
  uint64_t ray_to_node[64][8];
  uint32_t octant_step[3][3][3];
  uint64_t octant_mask[8];
  uint8_t bitmap_index[4][4][4];
  Luts() {
    // generate_lut_64_bits (lut.rs:33-84)
    std::memset(ray_to_node, 0, sizeof(ray_to_node));
    for (int x = 0; x < 4; ++x)
      for (int y = 0; y < 4; ++y)
        for (int z = 0; z < 4; ++z) {
          uint64_t pos = position_in_bitmap_64bits(V3u{(uint64_t)x, (uint64_t)y, (uint64_t)z}, 4);
          for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
              for (int dz = -1; dz <= 1; ++dz) {
                if (dx == 0 || dy == 0 || dz == 0) continue;
                uint8_t dir = hash_direction(V3f{(float)dx, (float)dy, (float)dz});
                int mx = std::clamp(x + dx * 4, 0, 3), my = std::clamp(y + dy * 4, 0, 3),
                    mz = std::clamp(z + dz * 4, 0, 3);
                uint64_t mask = 0;
                for (int bx = std::min(mx, x); bx <= std::max(mx, x); ++bx)
                  for (int by = std::min(my, y); by <= std::max(my, y); ++by)
                    for (int bz = std::min(mz, z); bz <= std::max(mz, z); ++bz)
                      set_occupancy_in_bitmap_64bits(V3u{(uint64_t)bx, (uint64_t)by, (uint64_t)bz}, 1, 4, true,
                                                     &mask);
                ray_to_node[pos][dir] = mask;
              }
        }
    // generate_octant_step_result_lut (lut.rs:86-139)
    std::memset(octant_step, 0, sizeof(octant_step));
    for (int octant = 0; octant < 8; ++octant) {
      for (int z = -1; z <= 1; ++z)
        for (int y = -1; y <= 1; ++y)
          for (int x = -1; x <= 1; ++x) {
            const float SPACE = 12.0f;
            V3f off = OCTANT_OFFSET_REGION_LUT[octant];
            V3f center{SPACE / 4.0f + off.x * (SPACE / 2.0f), SPACE / 4.0f + off.y * (SPACE / 2.0f),
                       SPACE / 4.0f + off.z * (SPACE / 2.0f)};
            V3f after{center.x + (float)isignum(x) * (SPACE / 2.0f), center.y + (float)isignum(y) * (SPACE / 2.0f),
                      center.z + (float)isignum(z) * (SPACE / 2.0f)};
            uint8_t result;
            if (after.x < 0 || after.x > SPACE || after.y < 0 || after.y > SPACE || after.z < 0 || after.z > SPACE)
              result = OOB_OCTANT;
            else
              result = hash_region(after, SPACE / 2.0f);
            octant_step[x + 1][y + 1][z + 1] |= ((uint32_t)result & 0x0F) << (4 * octant);
          }
    }
    // convert_8bit_bitmap_to_64bit (lut.rs:6-30): the per-octant 2x2x2 masks
    for (int octant = 0; octant < 8; ++octant) {
      V3f mp = OCTANT_OFFSET_REGION_LUT[octant];
      uint64_t bm = 0;
      for (uint64_t x = (uint64_t)mp.x * 2; x < (uint64_t)mp.x * 2 + 2; ++x)
        for (uint64_t y = (uint64_t)mp.y * 2; y < (uint64_t)mp.y * 2 + 2; ++y)
          for (uint64_t z = (uint64_t)mp.z * 2; z < (uint64_t)mp.z * 2 + 2; ++z)
            set_occupancy_in_bitmap_64bits(V3u{x, y, z}, 1, 4, true, &bm);
      octant_mask[octant] = bm;
    }
    // generate_bitmap_flat_index_lut (lut.rs:141-152)
    for (int x = 0; x < 4; ++x)
      for (int y = 0; y < 4; ++y)
        for (int z = 0; z < 4; ++z)
          bitmap_index[x][y][z] = (uint8_t)position_in_bitmap_64bits(V3u{(uint64_t)x, (uint64_t)y, (uint64_t)z}, 4);
  }
};
static const Luts& luts() {
  static const Luts L;
  return L;
}

// ---------------------------------------------------------------------------
// Cube / Ray (spatial/mod.rs, spatial/raytracing/mod.rs)
// ---------------------------------------------------------------------------
struct Cube {
  V3f min_position;
  float size;
};
static inline Cube root_bounds(float size) { return Cube{unit(0.0f), size}; }  // spatial/mod.rs:24-29
static inline Cube child_bounds_for(const Cube& c, uint8_t octant) {          // spatial/mod.rs:32-39
  float child_size = c.size / 2.0f;
  return Cube{c.min_position + (OCTANT_OFFSET_REGION_LUT[octant] * child_size), child_size};
}
struct Ray {
  V3f origin, direction;
};
static inline V3f point_at(const Ray& r, float d) { return r.origin + r.direction * d; }  // raytracing/mod.rs:20-22

// spatial/raytracing/mod.rs:32-61.  Returns 0 for None, 1 for Some(None), 2 for Some(Some(d)).
static int intersect_ray(const Cube& c, const Ray& ray, float* dist) {
  V3f max_position = c.min_position + unit(c.size);
  float t1 = (c.min_position.x - ray.origin.x) / ray.direction.x;
  float t2 = (max_position.x - ray.origin.x) / ray.direction.x;
  float t3 = (c.min_position.y - ray.origin.y) / ray.direction.y;
  float t4 = (max_position.y - ray.origin.y) / ray.direction.y;
  float t5 = (c.min_position.z - ray.origin.z) / ray.direction.z;
  float t6 = (max_position.z - ray.origin.z) / ray.direction.z;
  float tmin = rmax(rmax(rmin(t1, t2), rmin(t3, t4)), rmin(t5, t6));
  float tmax = rmin(rmin(rmax(t1, t2), rmax(t3, t4)), rmax(t5, t6));
  if (tmax < 0.0f || tmin > tmax) return 0;
  if (tmin < 0.0f) return 1;
  *dist = tmin;
  return 2;
}

// spatial/raytracing/mod.rs:68-80
static uint8_t step_octant(uint8_t octant, V3f step) {
  uint32_t pos = 4u * octant;
  uint32_t v = luts().octant_step[isignum(as_i32(step.x)) + 1][isignum(as_i32(step.y)) + 1][isignum(as_i32(step.z)) + 1];
  return (uint8_t)((v & (0x0Fu << pos)) >> pos);
}

// spatial/raytracing/mod.rs:86-104
static bool plane_line_intersection(V3f plane_point, V3f plane_normal, V3f line_origin, V3f line_direction,
                                    float* out) {
  V3f od = plane_point - line_origin;
  auto dot = [](V3f a, V3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; };
  float pl = dot(od, plane_normal);
  float dd = dot(line_direction, plane_normal);
  if (0.0f == dd) {
    if (0.0f == dot(od, plane_normal)) {
      *out = 0.0f;
      return true;
    }
    return false;
  }
  *out = pl / dd;
  return true;
}

// spatial/raytracing/mod.rs:106-134
static V3f cube_impact_normal(const Cube& cube, V3f impact_point) {
  V3f mid_to_impact = cube.min_position + unit(cube.size / 2.0f) - impact_point;
  float max_component = rmax(rmax(std::fabs(mid_to_impact.x), std::fabs(mid_to_impact.y)), std::fabs(mid_to_impact.z));
  V3f n{std::fabs(mid_to_impact.x) == max_component ? -mid_to_impact.x : 0.0f,
        std::fabs(mid_to_impact.y) == max_component ? -mid_to_impact.y : 0.0f,
        std::fabs(mid_to_impact.z) == max_component ? -mid_to_impact.z : 0.0f};
  return normalized(n);
}

// ---------------------------------------------------------------------------
// Octree data model (octree/types.rs:40-81, object_pool.rs)
// ---------------------------------------------------------------------------
enum BrickKind : uint8_t { B_EMPTY = 0, B_PARTED = 1, B_SOLID = 2 };
struct BrickData {  // types.rs:40-52
  BrickKind kind = B_EMPTY;
  uint32_t solid = 0;
  std::vector<uint32_t> parted;
  bool operator==(const BrickData& o) const {
    if (kind != o.kind) return false;
    if (kind == B_SOLID) return solid == o.solid;
    if (kind == B_PARTED) return parted == o.parted;
    return true;
  }
  static BrickData Empty() { return BrickData{}; }
  static BrickData Solid(uint32_t v) {
    BrickData b;
    b.kind = B_SOLID;
    b.solid = v;
    return b;
  }
  static BrickData Parted(std::vector<uint32_t> v) {
    BrickData b;
    b.kind = B_PARTED;
    b.parted = std::move(v);
    return b;
  }
};
enum ContentKind : uint8_t { C_NOTHING = 0, C_INTERNAL = 1, C_LEAF = 2, C_UNIFORM = 3 };
struct NodeContent {  // types.rs:54-72; UniformLeaf stores its brick in bricks[0]
  ContentKind kind = C_NOTHING;
  uint64_t ocbits = 0;
  BrickData bricks[8];
};
enum ChildrenKind : uint8_t { CH_NONE = 0, CH_CHILDREN = 1, CH_BITMAP = 2 };
struct NodeChildren {  // types.rs:74-81
  ChildrenKind kind = CH_NONE;
  uint32_t c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  uint64_t bitmap = 0;
  // node.rs:33-38
  uint64_t child(uint8_t octant) const { return kind == CH_CHILDREN ? (uint64_t)c[octant] : (uint64_t)EMPTY_U32; }
  // node.rs:40-48
  uint32_t* child_mut(size_t index) {
    if (kind == CH_NONE) {
      kind = CH_CHILDREN;
      for (auto& e : c) e = EMPTY_U32;
    }
    if (kind != CH_CHILDREN) throw Panic("child_mut on OccupancyBitmap");
    return &c[index];
  }
  // node.rs:59-67
  void clear(size_t child_index) {
    if (kind == CH_CHILDREN) {
      c[child_index] = EMPTY_U32;
      int n = 0;
      for (auto e : c) n += (e == EMPTY_U32);
      if (n == 8) *this = NodeChildren{};
    }
  }
  static NodeChildren Bitmap(uint64_t b) {
    NodeChildren n;
    n.kind = CH_BITMAP;
    n.bitmap = b;
    return n;
  }
};

struct PoolItem {
  bool reserved = false;
  NodeContent item;
};
struct ObjectPool {  // object_pool.rs:91-241
  std::vector<PoolItem> buffer;
  size_t first_available = 0;
  bool is_next_available() const {  // :151-154
    return first_available + 1 < buffer.size() && !buffer[first_available + 1].reserved;
  }
  bool check_first_available() {  // :156-166
    if (first_available < buffer.size() && !buffer[first_available].reserved) return true;
    if (is_next_available()) {
      first_available += 1;
      return true;
    }
    first_available = buffer.size();
    return false;
  }
  size_t len() const { return buffer.size(); }
  size_t allocate() {  // :178-202
    size_t key;
    if (check_first_available()) {
      buffer[first_available].reserved = true;
      key = first_available;
    } else {
      buffer.push_back(PoolItem{true, NodeContent{}});
      key = buffer.size() - 1;
    }
    if (is_next_available()) first_available += 1;
    return key;
  }
  size_t push(NodeContent item) {  // :172-176
    size_t key = allocate();
    buffer[key].item = std::move(item);
    return key;
  }
  bool free(size_t key) {  // :214-222
    if (key_is_valid(key)) {
      buffer[key].reserved = false;
      first_available = std::min(first_available, key);
      return true;
    }
    return false;
  }
  NodeContent& get(size_t key) {  // :224-232 (release: slice index only)
    if (key >= buffer.size()) throw Panic("pool index out of bounds");
    return buffer[key].item;
  }
  void swap(size_t a, size_t b) {  // :234-236
    if (a >= buffer.size() || b >= buffer.size()) throw Panic("pool swap out of bounds");
    std::swap(buffer[a], buffer[b]);
  }
  bool key_is_valid(uint64_t key) const { return key < buffer.size() && buffer[key].reserved; }  // :238-240
};

// Palette index codec (node.rs:306-379)
static inline uint32_t pix_visual(uint32_t c) { return (c & 0xFFFF) | (EMPTY_U16 << 16); }
static inline uint32_t pix_informal(uint32_t d) { return EMPTY_U16 | ((d & 0xFFFF) << 16); }
static inline uint32_t pix_complex(uint32_t c, uint32_t d) { return (c & 0xFFFF) | ((d & 0xFFFF) << 16); }
static inline uint32_t pix_color_index(uint32_t p) { return p & 0x0000FFFF; }
static inline uint32_t pix_data_index(uint32_t p) { return (p & 0xFFFF0000) >> 16; }
static inline bool pix_color_is_some(uint32_t p) { return pix_color_index(p) < EMPTY_U16; }
static inline bool pix_color_is_none(uint32_t p) { return !pix_color_is_some(p); }
static inline bool pix_data_is_none(uint32_t p) { return pix_data_index(p) == EMPTY_U16; }
static inline bool pix_data_is_some(uint32_t p) { return !pix_data_is_none(p); }
static inline uint32_t pix_overwrite_color(uint32_t i, uint32_t d) { return (i & 0xFFFF0000) | (d & 0x0000FFFF); }
static inline uint32_t pix_overwrite_data(uint32_t i, uint32_t d) { return (i & 0x0000FFFF) | (d & 0xFFFF0000); }

struct Entry {  // types.rs:23-36 OctreeEntry; kind bit0 = albedo, bit1 = data
  uint32_t kind = 0;
  uint32_t rgba = 0;
  uint32_t user = 0;
};
static inline bool albedo_transparent(uint32_t rgba) { return (rgba & 0xFF) == 0; }  // detail.rs:70-72
// octree/mod.rs:97-104 OctreeEntry::is_none
static bool entry_is_none(const Entry& e) {
  switch (e.kind) {
    case 0: return true;
    case 1: return albedo_transparent(e.rgba);
    case 2: return e.user == 0;
    default: return albedo_transparent(e.rgba) && e.user == 0;
  }
}

struct Octree {
  uint32_t brick_dim = 0;
  uint32_t octree_size = 0;
  ObjectPool nodes;
  std::vector<NodeChildren> node_children;
  std::vector<uint32_t> color_palette;  // Albedo packed 0xRRGGBBAA
  std::vector<uint32_t> data_palette;
  std::unordered_map<uint32_t, size_t> color_map, data_map;
  bool auto_simplify = true;
  int recursion = 0;
  // MIP maps (types.rs:146-160, mipmap.rs:578-595): disabled by default
  enum MipMethod : uint32_t { MIP_BOX = 0, MIP_POINT = 1, MIP_POINT_BD = 2, MIP_POSTERIZE = 3, MIP_POSTERIZE_BD = 4 };
  struct MipSampler {
    MipMethod method;
    float thr;
  };
  bool mips_enabled = false;
  std::map<size_t, MipSampler> mip_methods{
      {1, {MIP_POINT, 0.0f}}, {2, {MIP_BOX, 0.0f}}, {3, {MIP_BOX, 0.0f}}, {4, {MIP_BOX, 0.0f}}};
  std::map<size_t, float> mip_color_thr{{2, 0.1f}, {3, 0.05f}, {4, 0.02f}};
  std::vector<BrickData> node_mips{BrickData{}};  // mod.rs:198
  BrickData& mip(size_t key) {
    if (key >= node_mips.size()) throw Panic("node_mips index out of bounds");
    return node_mips[key];
  }
  const BrickData& mip(size_t key) const {
    if (key >= node_mips.size()) throw Panic("node_mips index out of bounds");
    return node_mips[key];
  }
  // `node_mips.resize(node_mips.len().max(nodes.len()), BrickData::Empty)`, which the reference
  // does beside most node_children resizes
  void mips_resize() {
    if (node_mips.size() < nodes.len()) node_mips.resize(nodes.len());
  }

  NodeChildren& nc(uint64_t key) {
    if (key >= node_children.size()) throw Panic("node_children index out of bounds");
    return node_children[key];
  }
  void nc_resize(size_t n) {
    if (node_children.size() < n) node_children.resize(n);
  }

  // node.rs:357-379
  bool pix_points_to_empty(uint32_t p) const {
    bool color_empty = pix_color_is_none(p);
    if (!color_empty) {
      uint32_t c = pix_color_index(p);
      if (c >= color_palette.size()) throw Panic("color palette index out of bounds");
      color_empty = albedo_transparent(color_palette[c]);
    }
    if (!color_empty) return false;
    if (pix_data_is_none(p)) return true;
    uint32_t d = pix_data_index(p);
    if (d >= data_palette.size()) throw Panic("data palette index out of bounds");
    return data_palette[d] == 0;
  }
  // node.rs:381-419
  Entry pix_get_ref(uint32_t p) const {
    Entry e;
    if (pix_data_is_none(p) && pix_color_is_none(p)) return e;
    if (pix_color_is_some(p)) {
      if (pix_color_index(p) >= color_palette.size()) throw Panic("color palette index out of bounds");
      e.kind |= 1;
      e.rgba = color_palette[pix_color_index(p)];
    }
    if (pix_data_is_some(p)) {
      if (pix_data_index(p) >= data_palette.size()) throw Panic("data palette index out of bounds");
      e.kind |= 2;
      e.user = data_palette[pix_data_index(p)];
    }
    return e;
  }

  // ---------------- construction (octree/mod.rs:173-206) ----------------
  static bool is_pow2(uint32_t v) { return v != 0 && (v & (v - 1)) == 0; }
  static int create(uint32_t size, uint32_t dim, Octree* t) {
    // `(x as f32).log(2.0).fract() != 0.0` checks are restated as exact power-of-two tests.
    if (size == 0 || !is_pow2(dim)) return ORC_ERR_INVALID_BRICK_DIM;
    if (dim > size || size % dim != 0 || !is_pow2(size / dim)) return ORC_ERR_INVALID_SIZE;
    if (size < dim * 2) return ORC_ERR_INVALID_STRUCTURE;
    t->brick_dim = dim;
    t->octree_size = size;
    t->nodes.push(NodeContent{});
    t->node_children.assign(1, NodeChildren{});
    return ORC_OK;
  }

  // ---------------- BrickData helpers (node.rs:72-300) ----------------
  bool is_empty_throughout(const BrickData& b, uint8_t octant, size_t dim) const {  // node.rs:75-146
    switch (b.kind) {
      case B_EMPTY: return true;
      case B_SOLID: return pix_points_to_empty(b.solid);
      default: break;
    }
    const auto& brick = b.parted;
    auto at = [&](size_t i) -> uint32_t {
      if (i >= brick.size()) throw Panic("brick index out of bounds");
      return brick[i];
    };
    if (dim == 1) return pix_points_to_empty(at(0));
    if (dim == 2) {
      V3u o = to_usize_round(OCTANT_OFFSET_REGION_LUT[octant]);
      return pix_points_to_empty(at(flat_projection(o.x, o.y, o.z, 2)));
    }
    size_t ext = dim / 2;
    V3u o = to_usize_round(OCTANT_OFFSET_REGION_LUT[octant]);
    o = V3u{o.x * ext, o.y * ext, o.z * ext};
    for (size_t x = o.x; x < o.x + ext; ++x)
      for (size_t y = o.y; y < o.y + ext; ++y)
        for (size_t z = o.z; z < o.z + ext; ++z)
          if (!pix_points_to_empty(at(flat_projection(x, y, z, dim)))) return false;
    return true;
  }
  bool is_part_empty_throughout(const BrickData& b, uint8_t part_octant, uint8_t target_octant,
                                size_t dim) const {  // node.rs:152-209
    switch (b.kind) {
      case B_EMPTY: return true;
      case B_SOLID: return pix_points_to_empty(b.solid);
      default: break;
    }
    const auto& brick = b.parted;
    auto at = [&](size_t i) -> uint32_t {
      if (i >= brick.size()) throw Panic("brick index out of bounds");
      return brick[i];
    };
    if (dim == 1) return pix_points_to_empty(at(0));
    if (dim == 2) {
      V3u o = to_usize_round(OCTANT_OFFSET_REGION_LUT[part_octant]);
      return pix_points_to_empty(at(flat_projection(o.x, o.y, o.z, 2)));
    }
    float outer = (float)dim / 2.0f, inner = (float)dim / 4.0f;
    V3u o = to_usize_round(OCTANT_OFFSET_REGION_LUT[part_octant] * outer +
                           OCTANT_OFFSET_REGION_LUT[target_octant] * inner);
    size_t n = as_usize(inner);
    for (size_t x = 0; x < n; ++x)
      for (size_t y = 0; y < n; ++y)
        for (size_t z = 0; z < n; ++z)
          if (!pix_points_to_empty(at(flat_projection(o.x + x, o.y + y, o.z + z, dim)))) return false;
    return true;
  }
  uint64_t calculate_brick_occupied_bits(const std::vector<uint32_t>& brick, size_t dim) const {  // node.rs:212-240
    uint64_t bitmap = 0;
    for (size_t x = 0; x < dim; ++x)
      for (size_t y = 0; y < dim; ++y)
        for (size_t z = 0; z < dim; ++z) {
          size_t fi = flat_projection(x, y, z, dim);
          if (fi >= brick.size()) throw Panic("brick index out of bounds");
          if (!pix_points_to_empty(brick[fi])) set_occupancy_in_bitmap_64bits(V3u{x, y, z}, 1, dim, true, &bitmap);
        }
    return bitmap;
  }
  uint64_t calculate_occupied_bits(const BrickData& b, size_t dim) const {  // node.rs:243-265
    switch (b.kind) {
      case B_EMPTY: return 0;
      case B_SOLID: return pix_points_to_empty(b.solid) ? 0 : UINT64_MAX;
      default: return calculate_brick_occupied_bits(b.parted, dim);
    }
  }
  // node.rs:268-281; returns false for None
  static bool get_homogeneous_data(const BrickData& b, uint32_t* out) {
    switch (b.kind) {
      case B_EMPTY: return false;
      case B_SOLID: *out = b.solid; return true;
      default:
        if (b.parted.empty()) throw Panic("brick index out of bounds");
        for (auto v : b.parted)
          if (v != b.parted[0]) return false;
        *out = b.parted[0];
        return true;
    }
  }
  bool brick_simplify(BrickData& b) const {  // node.rs:284-299
    uint32_t h;
    if (get_homogeneous_data(b, &h)) {
      if (pix_points_to_empty(h))
        b = BrickData::Empty();
      else
        b = BrickData::Solid(h);
      return true;
    }
    return false;
  }

  // ---------------- NodeContent helpers (node.rs:421-525) ----------------
  bool content_is_empty(const NodeContent& n) const {  // node.rs:422-467
    switch (n.kind) {
      case C_UNIFORM: {
        const BrickData& b = n.bricks[0];
        if (b.kind == B_EMPTY) return true;
        if (b.kind == B_SOLID) return pix_points_to_empty(b.solid);
        for (auto v : b.parted)
          if (!pix_points_to_empty(v)) return false;
        return true;
      }
      case C_LEAF:
        for (const auto& b : n.bricks) {
          if (b.kind == B_EMPTY) continue;
          if (b.kind == B_SOLID) {
            if (!pix_points_to_empty(b.solid)) return false;
          } else {
            for (auto v : b.parted)
              if (!pix_points_to_empty(v)) return false;
          }
        }
        return true;
      case C_INTERNAL: return false;
      default: return true;
    }
  }
  static bool content_is_all(const NodeContent& n, uint32_t data) {  // node.rs:470-504
    auto brick_is_all = [&](const BrickData& b) {
      if (b.kind == B_EMPTY) return false;
      if (b.kind == B_SOLID) return b.solid == data;
      uint32_t h;
      return get_homogeneous_data(b, &h) && h == data;
    };
    if (n.kind == C_UNIFORM) return brick_is_all(n.bricks[0]);
    if (n.kind == C_LEAF) {
      for (const auto& b : n.bricks)
        if (!brick_is_all(b)) return false;
      return true;
    }
    return false;
  }
  static bool content_compare(const NodeContent& a, const NodeContent& b) {  // node.rs:506-525
    switch (a.kind) {
      case C_NOTHING: return b.kind == C_NOTHING;
      case C_INTERNAL: return false;
      case C_UNIFORM: return b.kind == C_UNIFORM && a.bricks[0] == b.bricks[0];
      default:
        if (b.kind != C_LEAF) return false;
        for (int i = 0; i < 8; ++i)
          if (!(a.bricks[i] == b.bricks[i])) return false;
        return true;
    }
  }

  // ---------------- detail.rs ----------------
  bool should_bitmap_be_empty_at_bitmap_index(size_t node_key, V3u index) {  // detail.rs:165-180
    V3f position = v3(0.5f, 0.5f, 0.5f) + v3((float)index.x, (float)index.y, (float)index.z);
    uint8_t target_octant = hash_region(position, (float)BITMAP_DIMENSION / 2.0f);
    uint8_t target_octant_for_child = hash_region(
        position - (OCTANT_OFFSET_REGION_LUT[target_octant] * (float)BITMAP_DIMENSION / 2.0f),
        (float)BITMAP_DIMENSION / 4.0f);
    return should_bitmap_be_empty_at_octants(node_key, target_octant, target_octant_for_child);
  }
  bool should_bitmap_be_empty_at_octants(size_t node_key, uint8_t target_octant,
                                         uint8_t target_octant_for_child) {  // detail.rs:206-236
    NodeContent& n = nodes.get(node_key);
    switch (n.kind) {
      case C_NOTHING: return true;
      case C_INTERNAL: {
        uint64_t child_key = nc(node_key).child(target_octant);
        if (nodes.key_is_valid(child_key)) return node_empty_at(child_key, target_octant_for_child);
        return true;
      }
      case C_UNIFORM:
        return is_part_empty_throughout(n.bricks[0], target_octant, target_octant_for_child, brick_dim);
      default: return is_empty_throughout(n.bricks[target_octant], target_octant_for_child, brick_dim);
    }
  }
  bool node_empty_at(size_t node_key, uint8_t target_octant) {  // detail.rs:239-300
    NodeContent& n = nodes.get(node_key);
    auto brick_empty = [&](const BrickData& b) {
      if (b.kind == B_EMPTY) return true;
      if (b.kind == B_SOLID) return pix_points_to_empty(b.solid);
      uint32_t h;
      if (get_homogeneous_data(b, &h)) return pix_points_to_empty(h);
      return false;
    };
    switch (n.kind) {
      case C_NOTHING: return true;
      case C_LEAF: return brick_empty(n.bricks[target_octant]);
      case C_UNIFORM: return brick_empty(n.bricks[0]);
      default:
        // detail.rs:289-296: the loop variable is unused, the same child is checked 8 times
        for (int child_octant = 0; child_octant < 8; ++child_octant) {
          uint64_t child_key = nc(node_key).child(target_octant);
          if (nodes.key_is_valid(child_key) && !node_empty_at(child_key, (uint8_t)child_octant)) return false;
        }
        return true;
    }
  }

  size_t push_node(NodeContent c) { return nodes.push(std::move(c)); }

  void subdivide_leaf_to_nodes(size_t node_key, size_t target_octant) {  // detail.rs:305-470
    if (nc(node_key).kind != CH_BITMAP) throw Panic("Expected node to have OccupancyBitmap(_)");
    NodeContent node_content;
    node_content.kind = C_INTERNAL;
    node_content.ocbits = nc(node_key).bitmap;
    std::swap(node_content, nodes.get(node_key));
    uint32_t nn[8];
    for (auto& e : nn) e = EMPTY_U32;
    if (node_content.kind == C_NOTHING || node_content.kind == C_INTERNAL) throw Panic("Non-leaf node expected");
    if (node_content.kind == C_LEAF) {
      for (size_t octant = 0; octant < 8; ++octant) {
        BrickData brick;
        std::swap(brick, node_content.bricks[octant]);
        if (brick.kind == B_EMPTY) {
          if (octant == target_octant) {
            nn[octant] = (uint32_t)push_node(NodeContent{});
            nc_resize(std::max(node_children.size(), (size_t)nn[octant] + 1));
            mips_resize();
          }
        } else if (brick.kind == B_SOLID) {
          NodeContent c;
          c.kind = C_UNIFORM;
          c.bricks[0] = BrickData::Solid(brick.solid);
          nn[octant] = (uint32_t)push_node(std::move(c));
          nc_resize(std::max(node_children.size(), (size_t)nn[octant] + 1));
          mips_resize();
          nc(nn[octant]) = NodeChildren::Bitmap(UINT64_MAX);
        } else {
          NodeContent c;
          c.kind = C_UNIFORM;
          c.bricks[0] = BrickData::Parted(brick.parted);
          nn[octant] = (uint32_t)push_node(std::move(c));
          nc_resize(std::max(node_children.size(), (size_t)nn[octant] + 1));
          mips_resize();
          // detail.rs:387-394: computed from bricks[octant], which was swapped out to Empty above
          nc(nn[octant]) = NodeChildren::Bitmap(calculate_occupied_bits(node_content.bricks[octant], brick_dim));
        }
      }
    } else {  // UniformLeaf
      BrickData& brick = node_content.bricks[0];
      if (brick.kind == B_EMPTY) {
        nn[target_octant] = (uint32_t)push_node(NodeContent{});
        nc_resize(std::max(node_children.size(), (size_t)nn[target_octant] + 1));
        mips_resize();
        nc(nn[target_octant]) = NodeChildren::Bitmap(0);
      } else if (brick.kind == B_SOLID) {
        for (size_t octant = 0; octant < 8; ++octant) {
          NodeContent c;
          c.kind = C_UNIFORM;
          c.bricks[0] = BrickData::Solid(brick.solid);
          nn[octant] = (uint32_t)push_node(std::move(c));
          nc_resize(std::max(node_children.size(), (size_t)nn[octant] + 1));  // node_mips not resized (:439-446)
          nc(nn[octant]) = NodeChildren::Bitmap(UINT64_MAX);
        }
      } else {
        auto children_bricks = dilute_brick_data(brick.parted, brick_dim);
        for (size_t octant = 0; octant < 8; ++octant) {
          uint64_t bits = calculate_brick_occupied_bits(children_bricks[octant], brick_dim);
          NodeContent c;
          c.kind = C_UNIFORM;
          c.bricks[0] = BrickData::Parted(std::move(children_bricks[octant]));
          nn[octant] = (uint32_t)push_node(std::move(c));
          nc_resize(std::max(node_children.size(), (size_t)nn[octant] + 1));
          mips_resize();
          nc(nn[octant]) = NodeChildren::Bitmap(bits);
        }
      }
    }
    NodeChildren ch;
    ch.kind = CH_CHILDREN;
    for (int i = 0; i < 8; ++i) ch.c[i] = nn[i];
    nc(node_key) = ch;
  }

  BrickData try_brick_from_node(uint64_t node_key) {  // detail.rs:473-484
    if (!nodes.key_is_valid(node_key)) return BrickData::Empty();
    NodeContent& n = nodes.get(node_key);
    if (n.kind == C_UNIFORM) return n.bricks[0];
    return BrickData::Empty();
  }

  void deallocate_children_of(uint64_t node) {  // detail.rs:487-504
    if (!nodes.key_is_valid(node)) return;
    if (nc(node).kind != CH_CHILDREN) return;
    std::vector<uint64_t> to_deallocate;
    for (auto child : nc(node).c)
      if (nodes.key_is_valid(child)) to_deallocate.push_back(child);
    if (++recursion > 4096) throw Panic("recursion");
    for (auto child : to_deallocate) {
      deallocate_children_of(child);
      nodes.free(child);
      nc(child) = NodeChildren{};
    }
    --recursion;
  }

  uint64_t stored_occupied_bits(size_t node_key) {  // detail.rs:508-528
    NodeContent& n = nodes.get(node_key);
    switch (n.kind) {
      case C_LEAF:
      case C_UNIFORM: {
        const NodeChildren& ch = nc(node_key);
        return ch.kind == CH_BITMAP ? ch.bitmap : 0;
      }
      case C_NOTHING: return 0;
      default: return n.ocbits;
    }
  }
  void store_occupied_bits(size_t node_key, uint64_t bits) {  // detail.rs:531-553
    NodeContent& n = nodes.get(node_key);
    switch (n.kind) {
      case C_INTERNAL: n.ocbits = bits; break;
      case C_NOTHING: nc(node_key) = NodeChildren::Bitmap(bits); break;
      default: {
        NodeChildren& ch = nc(node_key);
        if (ch.kind == CH_NONE)
          ch = NodeChildren::Bitmap(bits);
        else if (ch.kind == CH_BITMAP)
          ch.bitmap = bits;
        else
          throw Panic("Expected Leaf node to have OccupancyBitmap");
      }
    }
  }

  // ---------------- update/mod.rs ----------------
  uint32_t add_color(uint32_t rgba) {
    auto it = color_map.find(rgba);
    if (it != color_map.end()) return (uint32_t)it->second;
    size_t idx = color_map.size();
    color_map.emplace(rgba, idx);
    color_palette.push_back(rgba);
    return (uint32_t)idx;
  }
  uint32_t add_data(uint32_t v) {
    auto it = data_map.find(v);
    if (it != data_map.end()) return (uint32_t)it->second;
    size_t idx = data_map.size();
    data_map.emplace(v, idx);
    data_palette.push_back(v);
    return (uint32_t)idx;
  }
  uint32_t add_to_palette(const Entry& e) {  // update/mod.rs:55-136
    switch (e.kind) {
      case 0: return EMPTY_U32;
      case 1:
        if (e.rgba == 0) return EMPTY_U32;
        return pix_visual(add_color(e.rgba));
      case 2:
        if (e.user == 0) return EMPTY_U32;
        return pix_informal(add_data(e.user));
      default: {
        if (e.rgba == 0) return add_to_palette(Entry{2, 0, e.user});
        if (e.user == 0) return add_to_palette(Entry{1, e.rgba, 0});
        uint32_t c = add_color(e.rgba);
        uint32_t d = add_data(e.user);
        return pix_complex(c, d);
      }
    }
  }

  V3u matrix_index_for(const Cube& bounds, const uint32_t position[3], uint32_t dim) const {  // math/mod.rs:44-78
    V3f p{(float)position[0], (float)position[1], (float)position[2]};
    return to_usize_round(vfloor((p - bounds.min_position) * (float)dim / bounds.size));
  }

  // update/mod.rs:531-596
  static std::vector<std::vector<uint32_t>> dilute_brick_data(const std::vector<uint32_t>& data, uint32_t dim) {
    size_t n = (size_t)dim * dim * dim;
    if (data.size() != n) throw Panic("brick size mismatch");
    std::vector<std::vector<uint32_t>> result(8);
    if (dim == 1) {
      for (auto& r : result) r = data;
      return result;
    }
    for (size_t o = 0; o < 8; ++o) result[o] = std::vector<uint32_t>(n, data[o]);
    if (dim == 2) return result;
    for (size_t octant = 0; octant < 8; ++octant) {
      V3u off = to_usize_round(OCTANT_OFFSET_REGION_LUT[octant]);
      off = V3u{off.x * 2, off.y * 2, off.z * 2};
      size_t f0 = flat_projection(off.x, off.y, off.z, dim);
      std::vector<uint32_t> nb(n, data.at(f0));
      for (size_t x = 0; x < dim; ++x)
        for (size_t y = 0; y < dim; ++y)
          for (size_t z = 0; z < dim; ++z) {
            if (x < 2 && y < 2 && z < 2) continue;
            size_t src = flat_projection(off.x + x / 2, off.y + y / 2, off.z + z / 2, dim);
            if (src >= n) throw Panic("brick index out of bounds");
            nb[flat_projection(x, y, z, dim)] = data[src];
          }
      result[octant] = std::move(nb);
    }
    return result;
  }

  // update/mod.rs:605-643
  size_t update_brick(bool overwrite_if_empty, std::vector<uint32_t>& brick, const Cube& brick_bounds, uint32_t dim,
                      const uint32_t position[3], uint32_t size, uint32_t data) const {
    V3u mi = matrix_index_for(brick_bounds, position, dim);
    size_t update_size = std::min((size_t)dim - (size_t)mi.x, (size_t)size);
    for (size_t x = mi.x; x < std::min(mi.x + size, (uint64_t)dim); ++x)
      for (size_t y = mi.y; y < std::min(mi.y + size, (uint64_t)dim); ++y)
        for (size_t z = mi.z; z < std::min(mi.z + size, (uint64_t)dim); ++z) {
          size_t fi = flat_projection(x, y, z, dim);
          if (fi >= brick.size()) throw Panic("brick index out of bounds");
          if (overwrite_if_empty) {
            brick[fi] = data;
          } else {
            if (pix_color_is_some(data)) brick[fi] = pix_overwrite_color(brick[fi], data);
            if (pix_data_is_some(data)) brick[fi] = pix_overwrite_data(brick[fi], data);
          }
        }
    return update_size;
  }

  // update/mod.rs:136-525
  size_t leaf_update(bool overwrite_if_empty, size_t node_key, const Cube& node_bounds, const Cube& target_bounds,
                     size_t target_child_octant, const uint32_t position[3], uint32_t size, uint32_t target_content) {
    struct Guard {
      int& r;
      Guard(int& r_) : r(r_) {
        if (++r > 4096) throw Panic("unbounded recursion in leaf_update");
      }
      ~Guard() { --r; }
    } guard(recursion);
    const size_t brick_len = (size_t)brick_dim * brick_dim * brick_dim;
    NodeContent& node = nodes.get(node_key);
    switch (node.kind) {
      case C_LEAF: {
        BrickData& b = node.bricks[target_child_octant];
        if (b.kind == B_EMPTY) {
          std::vector<uint32_t> nb(brick_len, EMPTY_U32);
          size_t us = update_brick(overwrite_if_empty, nb, target_bounds, brick_dim, position, size, target_content);
          b = BrickData::Parted(std::move(nb));
          return us;
        }
        if (b.kind == B_SOLID) {
          uint32_t voxel = b.solid;
          bool te = pix_points_to_empty(target_content);
          if ((te && !pix_points_to_empty(voxel)) || (!te && voxel != target_content)) {
            std::vector<uint32_t> nb(brick_len, voxel);
            size_t us = update_brick(overwrite_if_empty, nb, target_bounds, brick_dim, position, size, target_content);
            nodes.get(node_key).bricks[target_child_octant] = BrickData::Parted(std::move(nb));
            return us;
          }
          return 0;
        }
        return update_brick(overwrite_if_empty, b.parted, target_bounds, brick_dim, position, size, target_content);
      }
      case C_UNIFORM: {
        BrickData& mat = node.bricks[0];
        if (mat.kind == B_EMPTY) {
          if (!pix_points_to_empty(target_content)) {
            NodeContent leaf;
            leaf.kind = C_LEAF;
            std::vector<uint32_t> nb(brick_len, add_to_palette(Entry{}));
            size_t us = update_brick(overwrite_if_empty, nb, target_bounds, brick_dim, position, size, target_content);
            leaf.bricks[target_child_octant] = BrickData::Parted(std::move(nb));
            nodes.get(node_key) = std::move(leaf);
            return us;
          }
        } else if (mat.kind == B_SOLID) {
          uint32_t voxel = mat.solid;
          bool te = pix_points_to_empty(target_content);
          if (te && pix_points_to_empty(voxel)) {
            nodes.get(node_key) = NodeContent{};
            return 0;
          }
          if ((!te && voxel != target_content) || (te && !pix_points_to_empty(voxel))) {
            mat = BrickData::Parted(std::vector<uint32_t>(brick_len, voxel));
            return leaf_update(overwrite_if_empty, node_key, node_bounds, target_bounds, target_child_octant, position,
                               size, target_content);
          }
          return 0;
        } else {
          std::vector<uint32_t>& brick = mat.parted;
          V3u mi = matrix_index_for(node_bounds, position, brick_dim);
          size_t fi = flat_projection(mi.x, mi.y, mi.z, brick_dim);
          if (fi >= brick.size()) throw Panic("brick index out of bounds");
          bool te = pix_points_to_empty(target_content);
          if (1 < brick_dim && ((te && pix_points_to_empty(brick[fi])) || (!te && brick[fi] == target_content)))
            return 0;
          if (node_bounds.size <= (float)brick_dim && brick_dim > 1)
            return update_brick(overwrite_if_empty, brick, node_bounds, brick_dim, position, size, target_content);
          NodeContent leaf;
          leaf.kind = C_LEAF;
          size_t us = 0;
          if (brick_dim == 1) {
            for (int i = 0; i < 8; ++i) leaf.bricks[i] = BrickData::Parted(brick);
            std::vector<uint32_t> nb = brick;
            us = update_brick(overwrite_if_empty, nb, target_bounds, brick_dim, position, size, target_content);
            leaf.bricks[target_child_octant] = BrickData::Parted(std::move(nb));
          } else {
            std::vector<uint32_t> taken;
            std::swap(taken, brick);
            auto child_bricks = dilute_brick_data(taken, brick_dim);
            for (size_t octant = 0; octant < 8; ++octant) {
              if (octant == target_child_octant)
                us = update_brick(overwrite_if_empty, child_bricks[octant], target_bounds, brick_dim, position, size,
                                  target_content);
              leaf.bricks[octant] = BrickData::Parted(std::move(child_bricks[octant]));
            }
          }
          nodes.get(node_key) = std::move(leaf);
          return us;
        }
        return leaf_update(overwrite_if_empty, node_key, node_bounds, target_bounds, target_child_octant, position, size,
                           target_content);
      }
      case C_INTERNAL: {
        // update/mod.rs:473-497 -- node_children is switched to the bitmap before the
        // bricks are gathered, so every try_brick_from_node below sees an invalid key.
        nc(node_key) = NodeChildren::Bitmap(node.ocbits);
        NodeContent leaf;
        leaf.kind = C_LEAF;
        for (int i = 0; i < 8; ++i) leaf.bricks[i] = try_brick_from_node(nc(node_key).child((uint8_t)i));
        nodes.get(node_key) = std::move(leaf);
        deallocate_children_of(node_key);
        return leaf_update(overwrite_if_empty, node_key, node_bounds, target_bounds, target_child_octant, position, size,
                           target_content);
      }
      default: {  // Nothing, update/mod.rs:498-523
        NodeContent leaf;
        leaf.kind = C_LEAF;
        for (int i = 0; i < 8; ++i) leaf.bricks[i] = try_brick_from_node(nc(node_key).child((uint8_t)i));
        nodes.get(node_key) = std::move(leaf);
        deallocate_children_of(node_key);
        return leaf_update(overwrite_if_empty, node_key, node_bounds, target_bounds, target_child_octant, position, size,
                           target_content);
      }
    }
  }

  // update/mod.rs:649-1028
  bool simplify(uint64_t node_key) {
    if (!nodes.key_is_valid(node_key)) return false;
    struct Guard {
      int& r;
      Guard(int& r_) : r(r_) {
        if (++r > 4096) throw Panic("unbounded recursion in simplify");
      }
      ~Guard() { --r; }
    } guard(recursion);
    NodeContent& node = nodes.get(node_key);
    switch (node.kind) {
      case C_NOTHING: return true;
      case C_UNIFORM: {
        BrickData& brick = node.bricks[0];
        if (brick.kind == B_EMPTY) return true;
        if (brick.kind == B_SOLID) {
          if (pix_points_to_empty(brick.solid)) {
            nodes.get(node_key) = NodeContent{};
            nc(node_key) = NodeChildren{};
            return true;
          }
          return false;
        }
        return brick_simplify(brick);
      }
      case C_LEAF: {
        bool simplified = false;
        bool is_leaf_uniform_solid = true;
        bool have_uniform = false;
        uint32_t uniform_solid_value = 0;
        for (int octant = 0; octant < 8; ++octant) {
          simplified |= brick_simplify(node.bricks[octant]);
          if (is_leaf_uniform_solid) {
            if (node.bricks[octant].kind == B_SOLID) {
              if (have_uniform) {
                if (uniform_solid_value != node.bricks[octant].solid) is_leaf_uniform_solid = false;
              } else {
                have_uniform = true;
                uniform_solid_value = node.bricks[octant].solid;
              }
            } else {
              is_leaf_uniform_solid = false;
            }
          }
        }
        if (is_leaf_uniform_solid) {
          NodeContent u;
          u.kind = C_UNIFORM;
          u.bricks[0] = BrickData::Solid(uniform_solid_value);
          nodes.get(node_key) = std::move(u);
          return true;
        }
        const size_t D = brick_dim;
        std::vector<uint32_t> unified(D * D * D, EMPTY_U32);
        bool is_leaf_uniform = true;
        for (int octant = 0; octant < 8; ++octant) {
          size_t half = D / 2;
          V3u off = to_usize_round(OCTANT_OFFSET_REGION_LUT[octant] * (float)half);
          const BrickData& b = node.bricks[octant];
          if (b.kind == B_EMPTY) {
            is_leaf_uniform &= (b == node.bricks[0]);
          } else if (b.kind == B_SOLID) {
            is_leaf_uniform &= (b == node.bricks[0]);
            for (size_t x = off.x; x < off.x + half; ++x)
              for (size_t y = off.y; y < off.y + half; ++y)
                for (size_t z = off.z; z < off.z + half; ++z) unified[flat_projection(x, y, z, D)] = b.solid;
          } else {
            const auto& br = b.parted;
            auto at = [&](size_t x, size_t y, size_t z) -> uint32_t {
              size_t i = flat_projection(x, y, z, D);
              if (i >= br.size()) throw Panic("brick index out of bounds");
              return br[i];
            };
            for (size_t x = 0; x < half; ++x)
              for (size_t y = 0; y < half; ++y)
                for (size_t z = 0; z < half; ++z) {
                  if (!is_leaf_uniform) break;
                  uint32_t v = at(x * 2, y * 2, z * 2);
                  if (v == at(x * 2 + 1, y * 2, z * 2) && v == at(x * 2, y * 2 + 1, z * 2) &&
                      v == at(x * 2, y * 2, z * 2 + 1) && v == at(x * 2 + 1, y * 2 + 1, z * 2) &&
                      v == at(x * 2, y * 2 + 1, z * 2 + 1) && v == at(x * 2 + 1, y * 2, z * 2 + 1) &&
                      v == at(x * 2 + 1, y * 2 + 1, z * 2 + 1)) {
                    unified[flat_projection(off.x + x, off.y + y, off.z + z, D)] = v;
                  } else {
                    is_leaf_uniform = false;
                  }
                }
          }
          if (!is_leaf_uniform) break;
        }
        if (is_leaf_uniform) {
          NodeContent u;
          u.kind = C_UNIFORM;
          u.bricks[0] = BrickData::Parted(std::move(unified));
          nodes.get(node_key) = std::move(u);
          simplified = true;
        }
        return simplified;
      }
      default: {  // Internal
        if (node.ocbits == 0 || nc(node_key).kind == CH_NONE) {
          nodes.get(node_key) = NodeContent{};
          return true;
        }
        if (nc(node_key).kind != CH_CHILDREN) return false;
        uint32_t child_keys[8];
        std::memcpy(child_keys, nc(node_key).c, sizeof(child_keys));
        simplify(child_keys[0]);
        if (!nodes.key_is_valid(child_keys[0])) {
          for (int i = 1; i < 8; ++i) simplify(child_keys[i]);
          return false;
        }
        for (int octant = 1; octant < 8; ++octant) {
          simplify(child_keys[octant]);
          if (!nodes.key_is_valid(child_keys[octant]) ||
              !content_compare(nodes.get(child_keys[0]), nodes.get(child_keys[octant])))
            return false;
        }
        nodes.swap(node_key, child_keys[0]);
        NodeChildren new_node_children = nc(child_keys[0]);
        deallocate_children_of(node_key);
        nc(node_key) = new_node_children;
        return true;
      }
    }
  }

  // update/insert.rs:99-388
  int insert_at_lod_internal(bool overwrite_if_empty, const uint32_t upos[3], uint32_t insert_size,
                             const Entry& data) {
    Cube root = root_bounds((float)octree_size);
    V3f position{(float)upos[0], (float)upos[1], (float)upos[2]};
    if (!bound_contains(root, position)) return ORC_ERR_INVALID_POSITION;
    if (entry_is_none(data)) return ORC_OK;
    struct SE {
      uint32_t key;
      Cube b;
    };
    std::vector<SE> node_stack{{0u, root}};
    size_t actual_update_size = 0;
    uint32_t target_content = add_to_palette(data);
    for (;;) {
      size_t cur = node_stack.back().key;
      Cube cb = node_stack.back().b;
      uint8_t tco = child_octant_for(cb, position);
      Cube tb{cb.min_position + OCTANT_OFFSET_REGION_LUT[tco] * cb.size / 2.0f, cb.size / 2.0f};
      uint64_t target_child_key = nc(cur).child(tco);
      if (insert_size > 1 && tb.size <= (float)insert_size && lex_le(position, tb.min_position)) {
        ContentKind k = nodes.get(cur).kind;
        if (k == C_LEAF || k == C_UNIFORM) {
          subdivide_leaf_to_nodes(cur, tco);
          target_child_key = nc(cur).child(tco);
        }
        if (nodes.key_is_valid(target_child_key)) {
          deallocate_children_of(target_child_key);
          NodeContent u;
          u.kind = C_UNIFORM;
          u.bricks[0] = BrickData::Solid(target_content);
          nodes.get(target_child_key) = std::move(u);
          nc(target_child_key) = NodeChildren::Bitmap(UINT64_MAX);
        } else {
          NodeContent u;
          u.kind = C_UNIFORM;
          u.bricks[0] = BrickData::Solid(target_content);
          uint32_t nk = (uint32_t)push_node(std::move(u));
          nc_resize(std::max(node_children.size(), (size_t)nk + 1));
          mips_resize();
          *nc(cur).child_mut(tco) = nk;
          nc(nk) = NodeChildren::Bitmap(UINT64_MAX);
        }
        actual_update_size = as_usize(tb.size);
        break;
      }
      Cube data_bounds = (nodes.get(cur).kind == C_UNIFORM) ? cb : tb;
      if (data_bounds.size > (float)brick_dim || nodes.key_is_valid(target_child_key)) {
        if (nodes.key_is_valid(target_child_key)) {
          node_stack.push_back({(uint32_t)nc(cur).child(tco), tb});
        } else {
          ContentKind k = nodes.get(cur).kind;
          if (k == C_LEAF || k == C_UNIFORM) {
            bool target_match = false;
            NodeContent& n = nodes.get(cur);
            if (n.kind == C_UNIFORM) {
              const BrickData& b = n.bricks[0];
              if (b.kind == B_SOLID)
                target_match = b.solid == target_content;
              else if (b.kind == B_PARTED) {
                V3u mi = matrix_index_for(cb, upos, brick_dim);
                size_t fi = flat_projection(mi.x, mi.y, mi.z, brick_dim);
                if (fi >= b.parted.size()) throw Panic("brick index out of bounds");
                target_match = b.parted[fi] == target_content;
              }
            } else {
              const BrickData& b = n.bricks[tco];
              if (b.kind == B_SOLID)
                target_match = b.solid == target_content;
              else if (b.kind == B_PARTED) {
                V3u mi = matrix_index_for(tb, upos, brick_dim);
                size_t fi = flat_projection(mi.x, mi.y, mi.z, brick_dim);
                if (fi >= b.parted.size()) throw Panic("brick index out of bounds");
                target_match = b.parted[fi] == target_content;
              }
            }
            if (target_match || content_is_all(nodes.get(cur), target_content)) break;
            subdivide_leaf_to_nodes(cur, tco);
            node_stack.push_back({(uint32_t)nc(cur).child(tco), tb});
          } else {
            NodeContent& n = nodes.get(cur);
            if (n.kind == C_NOTHING) {
              n.kind = C_INTERNAL;
              n.ocbits = 0;
            }
            uint32_t nk = (uint32_t)push_node(NodeContent{});
            nc_resize(std::max(node_children.size(), nodes.len()));
            mips_resize();
            *nc(cur).child_mut(tco) = nk;
            node_stack.push_back({nk, tb});
          }
        }
      } else {
        actual_update_size = leaf_update(overwrite_if_empty, cur, cb, tb, tco, upos, insert_size, target_content);
        break;
      }
    }
    // post-processing (insert.rs:318-386)
    bool simplifyable = auto_simplify;
    for (auto it = node_stack.rbegin(); it != node_stack.rend(); ++it) {
      uint32_t node_key = it->key;
      const Cube nb = it->b;
      if (!nodes.key_is_valid(node_key)) continue;
      if (nodes.get(node_key).kind == C_NOTHING) {
        NodeContent& n = nodes.get(node_key);
        n.kind = C_INTERNAL;
        n.ocbits = 0;
      }
      uint64_t bits = stored_occupied_bits(node_key);
      if (as_usize(nb.size) == actual_update_size)
        bits = UINT64_MAX;
      else
        set_occupancy_in_bitmap_64bits(to_usize_round(position - nb.min_position), actual_update_size,
                                       as_usize(nb.size), true, &bits);
      store_occupied_bits(node_key, bits);
      update_mip(node_key, nb, upos);  // insert.rs:370-371
      ContentKind k = nodes.get(node_key).kind;
      if (k == C_LEAF || k == C_UNIFORM) {
        simplifyable = simplify(node_key);
        continue;
      }
      if (simplifyable) simplifyable = simplify(node_key);
    }
    return ORC_OK;
  }

  // update/clear.rs:47-340
  int clear_at_lod(const uint32_t position[3], uint32_t clear_size) {
    Cube root = root_bounds((float)octree_size);
    V3f fpos{(float)position[0], (float)position[1], (float)position[2]};
    if (!bound_contains(root, fpos)) return ORC_ERR_INVALID_POSITION;
    struct SE {
      uint32_t key;
      Cube b;
    };
    std::vector<SE> node_stack{{0u, root}};
    size_t actual_update_size = 0;
    for (;;) {
      size_t cur = node_stack.back().key;
      Cube cb = node_stack.back().b;
      uint8_t tco = child_octant_for(cb, fpos);
      Cube tb{cb.min_position + OCTANT_OFFSET_REGION_LUT[tco] * cb.size / 2.0f, cb.size / 2.0f};
      uint64_t target_child_key = nc(cur).child(tco);
      uint32_t tmin_u[3];
      to_u32_round(tb.min_position, tmin_u);
      if (clear_size > 1 && tb.size <= (float)clear_size && lex_le_u32(position, tmin_u) &&
          nodes.key_is_valid(target_child_key)) {
        deallocate_children_of(target_child_key);
        nodes.get(target_child_key) = NodeContent{};
        nc(target_child_key) = NodeChildren{};
        actual_update_size = as_usize(tb.size);
        node_stack.push_back({(uint32_t)nc(cur).child(tco), tb});
        break;
      }
      if (tb.size > (float)std::max(clear_size, brick_dim) || nodes.key_is_valid(target_child_key)) {
        if (nodes.key_is_valid(target_child_key)) {
          node_stack.push_back({(uint32_t)nc(cur).child(tco), tb});
        } else {
          ContentKind k = nodes.get(cur).kind;
          if (k == C_LEAF || k == C_UNIFORM) {
            bool target_match;
            NodeContent& n = nodes.get(cur);
            const BrickData& b = (n.kind == C_UNIFORM) ? n.bricks[0] : n.bricks[tco];
            if (b.kind == B_EMPTY)
              target_match = true;
            else if (b.kind == B_SOLID)
              target_match = pix_points_to_empty(b.solid);
            else {
              // clear.rs:128-140 / 152-164: `*position - V3c::from(current_bounds.min_position)` in u32
              uint32_t mn[3];
              to_u32_round(cb.min_position, mn);
              uint32_t ix = position[0] - mn[0], iy = position[1] - mn[1], iz = position[2] - mn[2];
              size_t fi = flat_projection(ix, iy, iz, brick_dim);
              if (fi >= b.parted.size()) throw Panic("brick index out of bounds");
              target_match = pix_points_to_empty(b.parted[fi]);
            }
            if (target_match || content_is_empty(nodes.get(cur))) break;
            subdivide_leaf_to_nodes(cur, tco);
            node_stack.push_back({(uint32_t)nc(cur).child(tco), tb});
          } else {
            break;
          }
        }
      } else {
        actual_update_size = leaf_update(true, cur, cb, tb, tco, position, clear_size, EMPTY_U32);
        break;
      }
    }
    // post-processing (clear.rs:224-339)
    bool have_removed = false;
    SE removed{0, Cube{}};
    if (!node_stack.empty()) {
      SE last = node_stack.back();
      node_stack.pop_back();
      if (as_usize(last.b.size) <= actual_update_size) {
        have_removed = true;
        removed = last;
      }
    }
    bool simplifyable = auto_simplify;
    for (auto it = node_stack.rbegin(); it != node_stack.rend(); ++it) {
      uint32_t node_key = it->key;
      const Cube nb = it->b;
      if (have_removed) {
        uint8_t child_octant = hash_region((removed.b.min_position - nb.min_position) + unit(removed.b.size / 2.0f),
                                           nb.size / 2.0f);
        nc(node_key).clear(child_octant);
        nodes.free(removed.key);
        have_removed = false;
      }
      uint64_t previous = stored_occupied_bits(node_key);
      uint64_t bits = (nc(node_key).kind == CH_NONE) ? 0 : previous;
      if (as_usize(nb.size) == actual_update_size) {
        bits = 0;
      } else {
        V3u start = matrix_index_for(nb, position, (uint32_t)BITMAP_DIMENSION);
        uint64_t us = as_usize(std::ceil((float)actual_update_size * (float)BITMAP_DIMENSION / nb.size));
        for (uint64_t x = start.x; x < std::min(start.x + us, BITMAP_DIMENSION); ++x)
          for (uint64_t y = start.y; y < std::min(start.y + us, BITMAP_DIMENSION); ++y)
            for (uint64_t z = start.z; z < std::min(start.z + us, BITMAP_DIMENSION); ++z)
              if (should_bitmap_be_empty_at_bitmap_index(node_key, V3u{x, y, z}))
                set_occupancy_in_bitmap_64bits(V3u{x, y, z}, 1, BITMAP_DIMENSION, false, &bits);
      }
      if (bits != 0 && nc(node_key).kind == CH_CHILDREN) {
        NodeContent n;
        n.kind = C_INTERNAL;
        n.ocbits = bits;
        nodes.get(node_key) = std::move(n);
      } else {
        deallocate_children_of(node_key);
        nc(node_key) = NodeChildren{};
        have_removed = true;
        removed = SE{node_key, nb};
        nodes.get(node_key) = NodeContent{};
      }
      if (bits == 0)
        nc(node_key) = NodeChildren{};
      else
        store_occupied_bits(node_key, bits);
      update_mip(node_key, nb, position);  // clear.rs:334-335
      if (simplifyable) simplifyable = simplify(node_key);
      if (previous == bits) break;
    }
    return ORC_OK;
  }

  // detail.rs:20-27, 30-38
  static bool bound_contains(const Cube& b, V3f p) {
    return p.x >= b.min_position.x && p.x < b.min_position.x + b.size && p.y >= b.min_position.y &&
           p.y < b.min_position.y + b.size && p.z >= b.min_position.z && p.z < b.min_position.z + b.size;
  }
  static uint8_t child_octant_for(const Cube& b, V3f p) { return hash_region(p - b.min_position, b.size / 2.0f); }

  // octree/mod.rs:209-371 (get = get_internal from the root)
  Entry get(const uint32_t upos[3]) { return get_internal(0, root_bounds((float)octree_size), upos); }
  Entry get_internal(size_t cur, Cube cb, const uint32_t upos[3]) {
    V3f position{(float)upos[0], (float)upos[1], (float)upos[2]};
    if (!bound_contains(cb, position)) return Entry{};
    for (;;) {
      NodeContent& n = nodes.get(cur);
      switch (n.kind) {
        case C_NOTHING: return Entry{};
        case C_LEAF: {
          uint8_t o = child_octant_for(cb, position);
          const BrickData& b = n.bricks[o];
          if (b.kind == B_EMPTY) return Entry{};
          if (b.kind == B_SOLID) return pix_get_ref(b.solid);
          cb = child_bounds_for(cb, o);
          V3u mi = matrix_index_for(cb, upos, brick_dim);
          size_t fi = flat_projection(mi.x, mi.y, mi.z, brick_dim);
          if (fi >= b.parted.size()) throw Panic("brick index out of bounds");
          if (!pix_points_to_empty(b.parted[fi])) return pix_get_ref(b.parted[fi]);
          return Entry{};
        }
        case C_UNIFORM: {
          const BrickData& b = n.bricks[0];
          if (b.kind == B_EMPTY) return Entry{};
          if (b.kind == B_PARTED) {
            V3u mi = matrix_index_for(cb, upos, brick_dim);
            size_t fi = flat_projection(mi.x, mi.y, mi.z, brick_dim);
            if (fi >= b.parted.size()) throw Panic("brick index out of bounds");
            if (pix_points_to_empty(b.parted[fi])) return Entry{};
            return pix_get_ref(b.parted[fi]);
          }
          if (pix_points_to_empty(b.solid)) return Entry{};
          return pix_get_ref(b.solid);
        }
        default: {
          uint8_t o = child_octant_for(cb, position);
          uint64_t ck = nc(cur).child(o);
          if (!nodes.key_is_valid(ck)) return Entry{};
          cur = ck;
          cb = child_bounds_for(cb, o);
        }
      }
    }
  }


  // ---------------- MIP maps (octree/mipmap.rs) ----------------
  // MIPResaplingFunction::execute (:131-273) over the sample_size^3 cells from sample_start, x
  // outermost.  PointFilter and Posterize keep their candidates in a HashMap whose iteration order
  // Rust randomises per process: the winner among equally frequent colours (and, for Posterize,
  // which of several matching groups a colour joins) is not defined by the reference; here the
  // groups are kept in first-seen order and the first group with the highest count wins.
  template <class F>
  static bool mip_resample(MipSampler sampler, V3u start, uint32_t size, F sample, uint32_t* out) {
    switch (sampler.method) {
      case MIP_BOX: {
        bool any = false;
        uint32_t count = 0;
        float acc[4] = {0, 0, 0, 0};
        for (uint64_t x = start.x; x < start.x + size; ++x)
          for (uint64_t y = start.y; y < start.y + size; ++y)
            for (uint64_t z = start.z; z < start.z + size; ++z) {
              uint32_t c;
              if (!sample(V3u{x, y, z}, &c)) continue;
              const float v[4] = {(float)(c >> 24), (float)((c >> 16) & 0xFF), (float)((c >> 8) & 0xFF), (float)(c & 0xFF)};
              if (!any) {
                any = true;
                count = 1;
                for (int k = 0; k < 4; ++k) acc[k] = v[k] * v[k];  // powf(2.) is exact as v * v
              } else {
                ++count;
                for (int k = 0; k < 4; ++k) acc[k] += v[k] * v[k];
              }
            }
        if (!any) return false;
        uint32_t ch[4];
        for (int k = 0; k < 4; ++k) ch[k] = sat_u8(std::fmin(std::sqrt(acc[k] / (float)count), 255.0f));
        *out = (ch[0] << 24) | (ch[1] << 16) | (ch[2] << 8) | ch[3];
        return true;
      }
      case MIP_POINT:
      case MIP_POINT_BD: {
        std::vector<std::pair<uint32_t, uint32_t>> counts;  // (colour, occurrences), first-seen order
        for (uint64_t x = start.x; x < start.x + size; ++x)
          for (uint64_t y = start.y; y < start.y + size; ++y)
            for (uint64_t z = start.z; z < start.z + size; ++z) {
              uint32_t c;
              if (!sample(V3u{x, y, z}, &c)) continue;
              bool found = false;
              for (auto& e : counts)
                if (e.first == c) {
                  ++e.second;
                  found = true;
                  break;
                }
              if (!found) counts.push_back({c, 1});
            }
        if (counts.empty()) return false;
        size_t best = 0;
        for (size_t i = 1; i < counts.size(); ++i)
          if (counts[i].second > counts[best].second) best = i;
        *out = counts[best].first;
        return true;
      }
      default: {  // Posterize, PosterizeBD
        struct Group {
          uint32_t sum[4];  // squared channel sums (Albedou32)
          uint32_t count;
        };
        std::vector<Group> groups;
        auto poster = [](const Group& g, uint32_t k) {  // (sum / count).sqrt(), channel k
          const uint32_t avg = round_u32((float)g.sum[k] / (float)g.count);
          return round_u32(std::sqrt((float)avg));
        };
        for (uint64_t x = start.x; x < start.x + size; ++x)
          for (uint64_t y = start.y; y < start.y + size; ++y)
            for (uint64_t z = start.z; z < start.z + size; ++z) {
              uint32_t c;
              if (!sample(V3u{x, y, z}, &c)) continue;
              const uint32_t v[4] = {c >> 24, (c >> 16) & 0xFF, (c >> 8) & 0xFF, c & 0xFF};
              bool joined = false;
              for (auto& g : groups) {
                uint32_t d[4];
                for (int k = 0; k < 4; ++k) d[k] = poster(g, k) - v[k];  // u32 wrap-around like the reference's Sub
                const float len = std::sqrt((float)(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + d[3] * d[3]));
                if (len < sampler.thr * 255.0f) {
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
    }
  }
  static uint32_t sat_u8(float v) {  // `f32 as u8`
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint32_t)v;
  }
  static uint32_t round_u32(float v) {  // `f32.round() as u32`
    return as_u32(std::round(v));
  }
  // Albedo::distance_from (detail.rs:82-89)
  static float albedo_distance(uint32_t a, uint32_t b) {
    const float dr = (float)(a >> 24) - (float)(b >> 24), dg = (float)((a >> 16) & 0xFF) - (float)((b >> 16) & 0xFF);
    const float db = (float)((a >> 8) & 0xFF) - (float)((b >> 8) & 0xFF), da = (float)(a & 0xFF) - (float)(b & 0xFF);
    return std::sqrt(((dr * dr + dg * dg) + db * db) + da * da);
  }

  // Octree::update_mip (mipmap.rs:309-577)
  void update_mip(size_t node_key, const Cube& node_bounds, const uint32_t upos[3]) {
    if (!mips_enabled) return;
    const V3u position{upos[0], upos[1], upos[2]};
    const size_t mip_level = as_usize(std::log2(node_bounds.size / (float)brick_dim));
    auto mit = mip_methods.find(mip_level);
    const bool dominant_bottom = mit != mip_methods.end() && mit->second.method == MIP_POINT_BD;
    const MipSampler sampler = mit != mip_methods.end() ? mit->second : MipSampler{MIP_BOX, 0.0f};
    const NodeContent& n = nodes.get(node_key);
    V3u sample_start{0, 0, 0};
    uint32_t sample_size = 0;
    switch (n.kind) {
      case C_NOTHING: return;
      case C_UNIFORM:
        // a UniformLeaf's content is its own MIP
        if (mip(node_key).kind != B_EMPTY) mip(node_key) = BrickData::Empty();
        return;
      case C_LEAF: {
        sample_size = std::min<uint32_t>(as_u32(node_bounds.size) / brick_dim, brick_dim * 2);
        const float f = node_bounds.size;
        const uint64_t px = (position.x - position.x % sample_size) * 2 * brick_dim;
        const uint64_t py = (position.y - position.y % sample_size) * 2 * brick_dim;
        const uint64_t pz = (position.z - position.z % sample_size) * 2 * brick_dim;
        sample_start = V3u{round_u32(std::floor((float)(uint32_t)px / f)), round_u32(std::floor((float)(uint32_t)py / f)),
                           round_u32(std::floor((float)(uint32_t)pz / f))};
        break;
      }
      default:
        if (dominant_bottom) {
          sample_size = as_u32(node_bounds.size) / brick_dim;
          sample_start = V3u{position.x - position.x % sample_size, position.y - position.y % sample_size,
                             position.z - position.z % sample_size};
        } else {
          sample_size = 2;
          const V3f pib{(float)position.x - node_bounds.min_position.x, (float)position.y - node_bounds.min_position.y,
                        (float)position.z - node_bounds.min_position.z};
          const float D = (float)brick_dim;
          V3u ss{round_u32(std::floor(pib.x * 2.0f * D / node_bounds.size)),
                 round_u32(std::floor(pib.y * 2.0f * D / node_bounds.size)),
                 round_u32(std::floor(pib.z * 2.0f * D / node_bounds.size))};
          sample_start = V3u{ss.x - ss.x % 2, ss.y - ss.y % 2, ss.z - ss.z % 2};
        }
    }
    uint32_t color = 0;
    bool sampled = false;
    if (n.kind == C_LEAF || dominant_bottom) {
      sampled = mip_resample(sampler, sample_start, sample_size, [&](V3u p, uint32_t* c) {
        const uint32_t up[3] = {(uint32_t)p.x, (uint32_t)p.y, (uint32_t)p.z};
        const Entry e = get_internal(node_key, node_bounds, up);
        if (!(e.kind & 1u)) return false;
        *c = e.rgba;
        return true;
      }, &color);
    } else {
      // the sampling range spans 0 .. 2 * brick_dim over the children's MIPs
      const float D = (float)brick_dim;
      const uint8_t first = hash_region(V3f{(float)sample_start.x, (float)sample_start.y, (float)sample_start.z}, D);
      if (nc(node_key).child(first) != EMPTY_U32) {
        sampled = mip_resample(sampler, sample_start, sample_size, [&](V3u p, uint32_t* c) {
          const uint8_t o = hash_region(V3f{(float)p.x, (float)p.y, (float)p.z}, D);
          const uint64_t ck = nc(node_key).child(o);
          if (ck == EMPTY_U32) return false;
          const V3f off = OCTANT_OFFSET_REGION_LUT[o] * D;
          const V3u q{p.x - round_u32(off.x), p.y - round_u32(off.y), p.z - round_u32(off.z)};
          const BrickData& m = mip(ck);
          Entry e;
          if (m.kind == B_EMPTY) return false;
          if (m.kind == B_SOLID) {
            e = pix_get_ref(m.solid);
          } else {
            const size_t fi = flat_projection(q.x, q.y, q.z, brick_dim);
            if (fi >= m.parted.size()) throw Panic("MIP brick index out of bounds");
            e = pix_get_ref(m.parted[fi]);
          }
          if (!(e.kind & 1u)) return false;
          *c = e.rgba;
          return true;
        }, &color);
      }
    }
    if (!sampled) return;
    // assemble the MIP entry (:519-545)
    uint32_t entry;
    auto thr = mip_color_thr.find(mip_level);
    if (thr != mip_color_thr.end()) {
      const float limit = thr->second * 255.0f;
      size_t similar = SIZE_MAX;
      for (size_t i = 0; i < color_palette.size(); ++i)
        if (albedo_distance(color, color_palette[i]) < limit) {
          similar = i;
          break;
        }
      entry = similar != SIZE_MAX ? pix_visual((uint32_t)(uint16_t)similar) : add_to_palette(Entry{1, color, 0});
    } else {
      entry = add_to_palette(Entry{1, color, 0});
    }
    const V3u pim = matrix_index_for(node_bounds, upos, brick_dim);
    const size_t fi = flat_projection(pim.x, pim.y, pim.z, brick_dim);
    const size_t len = (size_t)brick_dim * brick_dim * brick_dim;
    BrickData& m = mip(node_key);
    if (m.kind == B_EMPTY) {
      std::vector<uint32_t> b(len, EMPTY_U32);
      b[fi] = entry;
      m = BrickData::Parted(std::move(b));
    } else if (m.kind == B_SOLID) {
      std::vector<uint32_t> b(len, m.solid);
      b[fi] = entry;
      m = BrickData::Parted(std::move(b));
    } else {
      if (fi >= m.parted.size()) throw Panic("MIP brick index out of bounds");
      m.parted[fi] = entry;
    }
  }

  // StrategyUpdater::recalculate_mip (mipmap.rs:882-899)
  void recalculate_mip(size_t node_key, const Cube& b) {
    if (!mips_enabled) return;
    const float D = (float)brick_dim;
    for (uint32_t x = 0; x < brick_dim; ++x)
      for (uint32_t y = 0; y < brick_dim; ++y)
        for (uint32_t z = 0; z < brick_dim; ++z) {
          const V3f off{std::round((float)x * b.size / D), std::round((float)y * b.size / D),
                        std::round((float)z * b.size / D)};
          const V3f pos = b.min_position + off;
          const uint32_t up[3] = {round_u32(pos.x), round_u32(pos.y), round_u32(pos.z)};
          update_mip(node_key, b, up);
        }
  }
  // StrategyUpdater::recalculate_mips (mipmap.rs:798-856)
  void recalculate_mips() {
    node_mips.assign(nodes.len(), BrickData{});
    struct SE {
      size_t key;
      Cube b;
      uint32_t octant;
    };
    std::vector<SE> st{{0, root_bounds((float)octree_size), 0}};
    while (!st.empty()) {
      SE& top = st.back();
      if (top.octant == OOB_OCTANT) {
        recalculate_mip(top.key, top.b);
        st.pop_back();
        if (!st.empty()) st.back().octant += 1;
        continue;
      }
      const NodeContent& n = nodes.get(top.key);
      if (n.kind == C_NOTHING) throw Panic("BFS shouldn't evaluate empty children");
      if (n.kind == C_INTERNAL) {
        const uint64_t ck = nc(top.key).child((uint8_t)top.octant);
        if (nodes.key_is_valid(ck) && nodes.get(ck).kind != C_NOTHING) {
          const SE child{(size_t)ck, child_bounds_for(top.b, (uint8_t)top.octant), 0};
          st.push_back(child);
        } else {
          top.octant += 1;
        }
      } else {
        top.octant = OOB_OCTANT;
      }
    }
  }
  // StrategyUpdater::switch_albedo_mip_maps (mipmap.rs:858-880)
  void switch_albedo_mip_maps(bool enabled) {
    const bool before = mips_enabled;
    mips_enabled = enabled;
    if (mips_enabled && before != enabled && nodes.get(0).kind != C_NOTHING) recalculate_mips();
  }
  // StrategyUpdater::sample_root_mip (mipmap.rs:905-937)
  Entry sample_root_mip(uint8_t octant, const uint32_t p[3]) {
    const uint64_t key = octant == OOB_OCTANT ? 0 : nc(0).child(octant);
    if (!nodes.key_is_valid(key)) return Entry{};
    const BrickData& m = mip(key);
    if (m.kind == B_EMPTY) return Entry{};
    if (m.kind == B_SOLID) return pix_get_ref(m.solid);
    const size_t fi = flat_projection(p[0], p[1], p[2], brick_dim);
    if (fi >= m.parted.size()) throw Panic("MIP brick index out of bounds");
    return pix_get_ref(m.parted[fi]);
  }

  // ---------------- the cast (raytracing/raytracing_on_cpu.rs) ----------------
  struct CastResult {
    uint8_t status = 0, brick_octant = 0;
    uint32_t node_key = 0, voxel_index = EMPTY_U32, pix = 0;
    Entry entry;
    V3f point{0, 0, 0}, normal{0, 0, 0};
    uint32_t visits = 0, child_reads = 0, voxel_reads = 0;
  };
  // Work cap: the reference has none; any ray reaching it would loop forever there.
  static constexpr uint64_t WORK_CAP = 1u << 22;

  // :99-112
  static V3f get_dda_scale_factors(const Ray& r) {
    auto sq = [](float v) { return v * v; };  // powf(v, 2.) is exactly v*v
    const V3f d = r.direction;
    return V3f{std::sqrt(1.0f + sq(d.z / d.x) + sq(d.y / d.x)), std::sqrt(sq(d.x / d.y) + 1.0f + sq(d.z / d.y)),
               std::sqrt((sq(d.x / d.z) + 1.0f) + sq(d.y / d.z))};
  }
  // :124-152
  static V3f dda_step_to_next_sibling(const Ray& ray, V3f& p, const Cube& b, V3f sf) {
    V3f sg{rsignum(ray.direction.x), rsignum(ray.direction.y), rsignum(ray.direction.z)};
    V3f diff = p - b.min_position;
    V3f steps{b.size * rmax(sg.x, 0.0f) - sg.x * diff.x, b.size * rmax(sg.y, 0.0f) - sg.y * diff.y,
              b.size * rmax(sg.z, 0.0f) - sg.z * diff.z};
    float d_x = std::fabs(steps.x * sf.x), d_y = std::fabs(steps.y * sf.y), d_z = std::fabs(steps.z * sf.z);
    float m = rmin(rmin(d_x, d_y), d_z);
    p = p + ray.direction * m;
    return V3f{m == d_x ? sg.x : 0.0f, m == d_y ? sg.y : 0.0f, m == d_z ? sg.z : 0.0f};
  }
  // :156-252; returns -1 for no hit, else the flat index (and writes the 3D index)
  int64_t traverse_brick(const Ray& ray, V3f& p, const std::vector<uint32_t>& brick, const Cube& bb, uint32_t D,
                         V3f sf, int32_t idx_out[3], CastResult& res, uint64_t& work) const {
    V3f pib = (p - bb.min_position) * (float)D / bb.size;
    int32_t ci[3] = {std::clamp(as_i32(pib.x), 0, (int32_t)D - 1), std::clamp(as_i32(pib.y), 0, (int32_t)D - 1),
                     std::clamp(as_i32(pib.z), 0, (int32_t)D - 1)};
    const int32_t fdx = 1, fdy = (int32_t)D, fdz = (int32_t)(D * D);
    int32_t flat = (int32_t)flat_projection((uint64_t)ci[0], (uint64_t)ci[1], (uint64_t)ci[2], D);
    float unit_ = bb.size / (float)D;
    Cube cur{bb.min_position + V3f{(float)ci[0], (float)ci[1], (float)ci[2]} * unit_, unit_};
    V3f step{0, 0, 0};
    for (;;) {
      if (ci[0] < 0 || ci[0] >= (int32_t)D || ci[1] < 0 || ci[1] >= (int32_t)D || ci[2] < 0 || ci[2] >= (int32_t)D)
        return -1;
      flat += as_i32(step.x) * fdx + as_i32(step.y) * fdy + as_i32(step.z) * fdz;
      if (flat < 0 || (size_t)flat >= brick.size()) throw Panic("brick index out of bounds");
      res.voxel_reads++;
      if (++work > WORK_CAP) throw std::length_error("cap");
      if (!pix_points_to_empty(brick[(size_t)flat])) {
        idx_out[0] = ci[0];
        idx_out[1] = ci[1];
        idx_out[2] = ci[2];
        return flat;
      }
      step = dda_step_to_next_sibling(ray, p, cur, sf);
      cur.min_position = cur.min_position + step * unit_;
      // V3c::<i32>::from(step) rounds each component
      ci[0] += as_i32(std::round(step.x));
      ci[1] += as_i32(std::round(step.y));
      ci[2] += as_i32(std::round(step.z));
    }
  }
  // :256-312
  bool probe_brick(const Ray& ray, V3f& p, const BrickData& brick, const Cube& bb, V3f sf, CastResult& res,
                   uint64_t& work) const {
    if (brick.kind == B_EMPTY) return false;
    if (brick.kind == B_SOLID) {
      res.entry = pix_get_ref(brick.solid);
      res.pix = brick.solid;
      res.voxel_index = EMPTY_U32;
      res.point = p;
      res.normal = cube_impact_normal(bb, p);
      return true;
    }
    int32_t hit[3];
    int64_t fi = traverse_brick(ray, p, brick.parted, bb, brick_dim, sf, hit, res, work);
    if (fi < 0) return false;
    Cube hb{bb.min_position + V3f{(float)hit[0], (float)hit[1], (float)hit[2]} * bb.size / (float)brick_dim,
            bb.size / (float)brick_dim};
    res.point = p;
    res.normal = cube_impact_normal(hb, p);
    res.pix = brick.parted[(size_t)fi];
    res.entry = pix_get_ref(res.pix);
    res.voxel_index = (uint32_t)fi;
    return true;
  }

  // NodeStack<u32, 4> (:20-82)
  struct NodeStack {
    uint32_t data[4] = {0, 0, 0, 0};
    size_t head = 0;
    uint8_t count = 0;
    bool empty() const { return count == 0; }
    void push(uint32_t v) {
      head = (head + 1) % 4;
      count = (uint8_t)std::min<int>(count + 1, 4);
      data[head] = v;
    }
    bool pop() {
      if (count == 0) return false;
      count -= 1;
      head = (head == 0) ? 3 : head - 1;
      return true;
    }
    bool last(uint32_t* out) const {
      if (count == 0) return false;
      *out = data[head];
      return true;
    }
  };

  // :316-565 (get_by_ray -> get_by_ray_at_lod with MIPs disabled)
  // get_by_ray is get_by_ray_at_lod(ray, f32::MAX) (:316-318)
  CastResult get_by_ray(const Ray& ray, float viewing_distance = FLT_MAX) const {
    CastResult res;
    uint64_t work = 0;
    try {
      if (cast_inner(ray, viewing_distance, res, work))
        res.status = 1;
      else
        res.status = 0;
    } catch (const std::length_error&) {
      res = CastResult{};
      res.status = 2;
    } catch (const Panic&) {
      res = CastResult{};
      res.status = 3;
    }
    return res;
  }

  bool cast_inner(const Ray& ray, float viewing_distance, CastResult& res, uint64_t& work) const {
    const Luts& L = luts();
    const V3f sf = get_dda_scale_factors(ray);
    const uint8_t dir_idx = hash_direction(ray.direction);
    NodeStack stack;
    Cube cb = root_bounds((float)octree_size);
    V3f p;
    uint8_t target_octant;
    float dist = 0.0f;
    int ih = intersect_ray(cb, ray, &dist);
    if (ih != 0) {
      p = point_at(ray, ih == 2 ? dist : 0.0f);
      target_octant = hash_region(p - cb.min_position, cb.size / 2.0f);
    } else {
      p = ray.origin;
      target_octant = OOB_OCTANT;
    }
    size_t cur;
    const float S = (float)octree_size;
    auto node = [&](size_t k) -> const NodeContent& {
      if (k >= nodes.buffer.size()) throw Panic("pool index out of bounds");
      return nodes.buffer[k].item;
    };
    auto lut_index = [&](V3f bp) -> uint8_t {
      uint64_t ix = as_usize(std::floor(bp.x)), iy = as_usize(std::floor(bp.y)), iz = as_usize(std::floor(bp.z));
      if (ix >= 4 || iy >= 4 || iz >= 4) throw Panic("BITMAP_INDEX_LUT index out of bounds");
      return L.bitmap_index[ix][iy][iz];
    };
    float mip_level = std::log2((float)octree_size / (float)brick_dim);  // :350, kept across restarts
    while (target_octant != OOB_OCTANT) {
      cur = 0;
      cb = root_bounds(S);
      stack.push(0);
      while (!stack.empty()) {
        if (++work > WORK_CAP) throw std::length_error("cap");
        res.visits++;
        uint32_t top;
        stack.last(&top);
        // stored_occupied_bits (detail.rs:508-528) on the stack top
        uint64_t occ;
        {
          const NodeContent& tn = node(top);
          if (tn.kind == C_LEAF || tn.kind == C_UNIFORM) {
            if (top >= node_children.size()) throw Panic("node_children index out of bounds");
            occ = node_children[top].kind == CH_BITMAP ? node_children[top].bitmap : 0;
          } else if (tn.kind == C_NOTHING) {
            occ = 0;
          } else {
            occ = tn.ocbits;
          }
        }
        const NodeContent& cn = node(cur);
        bool backtrack = cn.kind == C_UNIFORM;
        // the node's MIP when its level is below the one the travelled distance asks for (:366-386)
        if (mips_enabled) {
          const float m2 = mip_level * 2.0f;
          const V3f al{std::round(p.x / m2) * m2, std::round(p.y / m2) * m2, std::round(p.z / m2) * m2};
          if (mip_level < length(ray.origin - al) / viewing_distance) {
            if (probe_brick(ray, p, mip(cur), cb, sf, res, work)) {
              res.node_key = (uint32_t)cur;
              res.brick_octant = 8;  // the node's MIP brick
              return true;
            }
          }
        }
        if (target_octant != OOB_OCTANT) {
          if (cn.kind == C_UNIFORM) {
            if (probe_brick(ray, p, cn.bricks[0], cb, sf, res, work)) {
              res.node_key = (uint32_t)cur;
              res.brick_octant = 0;
              return true;
            }
            backtrack = true;
          } else if (cn.kind == C_LEAF) {
            if (probe_brick(ray, p, cn.bricks[target_octant], child_bounds_for(cb, target_octant), sf, res, work)) {
              res.node_key = (uint32_t)cur;
              res.brick_octant = target_octant;
              return true;
            }
          }
        }
        V3f bp = (p - cb.min_position) * (float)BITMAP_DIMENSION / cb.size;
        bp = V3f{rclamp(bp.x, FLOAT_ERROR_TOLERANCE, 4.0f - FLOAT_ERROR_TOLERANCE),
                 rclamp(bp.y, FLOAT_ERROR_TOLERANCE, 4.0f - FLOAT_ERROR_TOLERANCE),
                 rclamp(bp.z, FLOAT_ERROR_TOLERANCE, 4.0f - FLOAT_ERROR_TOLERANCE)};
        uint8_t flat_pos = lut_index(bp);
        if (backtrack || target_octant == OOB_OCTANT || occ == 0 || (occ & L.ray_to_node[flat_pos][dir_idx]) == 0) {
          // POP (:445-473)
          stack.pop();
          mip_level += 1.0f;
          uint32_t parent;
          if (stack.last(&parent)) {
            cur = parent;
            V3f center = cb.min_position + unit(cb.size / 2.0f);
            V3f parent_min = cb.min_position - vmodulo(cb.min_position, cb.size * 2.0f);
            uint8_t h = hash_region(center - parent_min, cb.size);
            V3f st = dda_step_to_next_sibling(ray, p, cb, sf);
            target_octant = step_octant(h, st);
            cb.size *= 2.0f;
            cb.min_position = parent_min;
          }
          continue;
        }
        Cube tb = child_bounds_for(cb, target_octant);
        if (cur >= node_children.size()) throw Panic("node_children index out of bounds");
        uint64_t tck = node_children[cur].child(target_octant);
        res.child_reads++;
        if (nodes.key_is_valid(tck) && (occ & L.octant_mask[target_octant]) != 0) {
          // PUSH (:484-492)
          cur = (size_t)tck;
          cb = tb;
          target_octant = hash_region(p - tb.min_position, tb.size / 2.0f);
          stack.push((uint32_t)tck);
          mip_level -= 1.0f;
        } else {
          // ADVANCE (:494-544)
          for (;;) {
            if (++work > WORK_CAP) throw std::length_error("cap");
            V3f sv = dda_step_to_next_sibling(ray, p, tb, sf);
            target_octant = step_octant(target_octant, sv);
            if (target_octant != OOB_OCTANT) {
              tb = child_bounds_for(cb, target_octant);
              tck = node_children[cur].child(target_octant);
              res.child_reads++;
              bp = bp + sv * 4.0f / cb.size;
              flat_pos = lut_index(bp);
            }
            if (target_octant == OOB_OCTANT) break;
            if (nodes.key_is_valid(tck) && (occ & L.octant_mask[target_octant]) != 0 &&
                (L.ray_to_node[flat_pos][dir_idx] & occ) != 0)
              break;
            if (cn.kind == C_LEAF && cn.bricks[target_octant].kind != B_EMPTY) break;
          }
        }
      }
      // restart from the root (:548-562)
      p = p + ray.direction * 0.1f;
      if (p.x < S && p.y < S && p.z < S && p.x > 0.0f && p.y > 0.0f && p.z > 0.0f)
        target_octant = hash_region(p, S / 2.0f);
      else
        target_octant = OOB_OCTANT;
    }
    return false;
  }
};

}  // namespace orc

using namespace orc;

static Entry make_entry(uint32_t kind, uint32_t rgba, uint32_t user) {
  Entry e;
  e.kind = kind & 3;
  e.rgba = (kind & 1) ? rgba : 0;
  e.user = (kind & 2) ? user : 0;
  return e;
}

template <class F>
static int guarded(F&& f) {
  try {
    return f();
  } catch (const Panic&) {
    return ORC_ERR_REFERENCE_PANIC;
  } catch (const std::bad_alloc&) {
    return ORC_ERR_REFERENCE_PANIC;
  }
}

extern "C" {

int orc_new(uint32_t size, uint32_t brick_dim, void** out) {
  if (!out) return ORC_ERR_ARGUMENT;
  Octree* t = new Octree();
  int rc = Octree::create(size, brick_dim, t);
  if (rc != ORC_OK) {
    delete t;
    *out = nullptr;
    return rc;
  }
  *out = t;
  return ORC_OK;
}
void orc_free(void* tree) { delete static_cast<Octree*>(tree); }
void orc_set_auto_simplify(void* tree, int enabled) { static_cast<Octree*>(tree)->auto_simplify = enabled != 0; }

int orc_insert(void* tree, uint32_t x, uint32_t y, uint32_t z, uint32_t kind, uint32_t rgba, uint32_t user) {
  uint32_t p[3] = {x, y, z};
  return guarded([&] { return static_cast<Octree*>(tree)->insert_at_lod_internal(true, p, 1, make_entry(kind, rgba, user)); });
}
int orc_update(void* tree, uint32_t x, uint32_t y, uint32_t z, uint32_t kind, uint32_t rgba, uint32_t user) {
  uint32_t p[3] = {x, y, z};
  return guarded([&] { return static_cast<Octree*>(tree)->insert_at_lod_internal(false, p, 1, make_entry(kind, rgba, user)); });
}
int orc_insert_at_lod(void* tree, uint32_t x, uint32_t y, uint32_t z, uint32_t size, uint32_t kind, uint32_t rgba,
                      uint32_t user) {
  uint32_t p[3] = {x, y, z};
  return guarded(
      [&] { return static_cast<Octree*>(tree)->insert_at_lod_internal(true, p, size, make_entry(kind, rgba, user)); });
}
int orc_clear(void* tree, uint32_t x, uint32_t y, uint32_t z) {
  uint32_t p[3] = {x, y, z};
  return guarded([&] { return static_cast<Octree*>(tree)->clear_at_lod(p, 1); });
}
int orc_clear_at_lod(void* tree, uint32_t x, uint32_t y, uint32_t z, uint32_t size) {
  uint32_t p[3] = {x, y, z};
  return guarded([&] { return static_cast<Octree*>(tree)->clear_at_lod(p, size); });
}
int orc_apply_ops(void* tree, const orc_op* ops, uint64_t n, uint64_t* n_done) {
  uint64_t i = 0;
  int rc = ORC_OK;
  for (; i < n; ++i) {
    const orc_op& o = ops[i];
    switch (o.op) {
      case 0: rc = orc_insert(tree, o.x, o.y, o.z, o.kind, o.rgba, o.user); break;
      case 1: rc = orc_update(tree, o.x, o.y, o.z, o.kind, o.rgba, o.user); break;
      case 2: rc = orc_insert_at_lod(tree, o.x, o.y, o.z, o.size, o.kind, o.rgba, o.user); break;
      case 3: rc = orc_clear(tree, o.x, o.y, o.z); break;
      case 4: rc = orc_clear_at_lod(tree, o.x, o.y, o.z, o.size); break;
      default: rc = ORC_ERR_ARGUMENT;
    }
    if (rc != ORC_OK) break;
  }
  if (n_done) *n_done = i;
  return rc;
}
int orc_get(void* tree, uint32_t x, uint32_t y, uint32_t z, uint32_t out[3]) {
  uint32_t p[3] = {x, y, z};
  return guarded([&] {
    Entry e = static_cast<Octree*>(tree)->get(p);
    out[0] = e.kind;
    out[1] = e.rgba;
    out[2] = e.user;
    return ORC_OK;
  });
}

int orc_cast(void* tree, uint64_t n, const float* ox, const float* oy, const float* oz, const float* dx,
             const float* dy, const float* dz, const orc_hits* out, int threads) {
  return orc_cast_lod(tree, n, ox, oy, oz, dx, dy, dz, FLT_MAX, out, threads);
}

int orc_cast_lod(void* tree, uint64_t n, const float* ox, const float* oy, const float* oz, const float* dx,
                 const float* dy, const float* dz, float viewing_distance, const orc_hits* out, int threads) {
  const Octree* t = static_cast<const Octree*>(tree);
  if (!t || !out) return ORC_ERR_ARGUMENT;
  auto work = [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; ++i) {
      Ray r{V3f{ox[i], oy[i], oz[i]}, V3f{dx[i], dy[i], dz[i]}};
      Octree::CastResult h = t->get_by_ray(r, viewing_distance);
      if (out->status) out->status[i] = h.status;
      if (out->brick_octant) out->brick_octant[i] = h.brick_octant;
      if (out->entry_kind) out->entry_kind[i] = (uint8_t)h.entry.kind;
      if (out->node_key) out->node_key[i] = h.node_key;
      if (out->voxel_index) out->voxel_index[i] = h.voxel_index;
      if (out->pix) out->pix[i] = h.pix;
      if (out->albedo) out->albedo[i] = h.entry.rgba;
      if (out->user) out->user[i] = h.entry.user;
      if (out->px) out->px[i] = h.point.x;
      if (out->py) out->py[i] = h.point.y;
      if (out->pz) out->pz[i] = h.point.z;
      if (out->nx) out->nx[i] = h.normal.x;
      if (out->ny) out->ny[i] = h.normal.y;
      if (out->nz) out->nz[i] = h.normal.z;
      if (out->node_visits) out->node_visits[i] = h.visits;
      if (out->child_reads) out->child_reads[i] = h.child_reads;
      if (out->voxel_reads) out->voxel_reads[i] = h.voxel_reads;
    }
  };
  if (threads <= 1 || n < 1024) {
    work(0, n);
    return ORC_OK;
  }
  std::vector<std::thread> pool;
  uint64_t chunk = (n + threads - 1) / threads;
  for (int k = 0; k < threads; ++k) {
    uint64_t b = (uint64_t)k * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    pool.emplace_back(work, b, e);
  }
  for (auto& th : pool) th.join();
  return ORC_OK;
}

// examples/cpu_render.rs:77-138 (one iteration of its render loop; the viewport, light and
// background are parameters instead of the example's constants)
static inline V3f cross(V3f a, V3f b) {  // vector.rs:186-192
  return V3f{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline float dot(V3f a, V3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }  // vector.rs:182-184
static inline uint8_t as_u8(float v) {  // `f32 as u8`: truncate, saturate, NaN -> 0
  if (!(v > 0.0f)) return 0;
  if (v >= 255.0f) return 255;
  return (uint8_t)v;
}

int orc_render_viewport(void* tree, const orc_viewport* vp, uint32_t W, uint32_t H, uint8_t* rgba,
                        uint64_t* unshaded, int threads) {
  const Octree* t = static_cast<const Octree*>(tree);
  if (!t || !vp || !rgba) return ORC_ERR_ARGUMENT;
  const V3f origin{vp->origin[0], vp->origin[1], vp->origin[2]};
  const V3f dir{vp->direction[0], vp->direction[1], vp->direction[2]};
  const V3f up{vp->up[0], vp->up[1], vp->up[2]};
  const V3f light{vp->light[0], vp->light[1], vp->light[2]};
  const V3f right = normalized(cross(up, dir));
  const float pixel_width = vp->width / (float)W, pixel_height = vp->height / (float)H;
  const V3f bottom_left = origin + dir * vp->fov - up * (vp->height / 2.0f) - right * (vp->width / 2.0f);
  std::atomic<uint64_t> bad{0};
  auto work = [&](uint32_t x0, uint32_t x1) {
    uint64_t local = 0;
    for (uint32_t x = x0; x < x1; ++x)
      for (uint32_t y = 0; y < H; ++y) {
        const V3f glass = bottom_left + right * (float)x * pixel_width + up * (float)y * pixel_height;
        const Ray ray{origin, normalized(glass - origin)};
        const Octree::CastResult h = t->get_by_ray(ray);
        uint8_t* px = rgba + 4 * ((size_t)(H - y - 1) * W + x);
        if (h.status == 0) {
          px[0] = (uint8_t)(vp->background >> 24);
          px[1] = (uint8_t)(vp->background >> 16);
          px[2] = (uint8_t)(vp->background >> 8);
          px[3] = (uint8_t)vp->background;
        } else if (h.status == 1 && (h.entry.kind & 1u)) {
          const float strength = 1.0f - (dot(h.normal, light) / 2.0f + 0.5f);
          const uint32_t a = h.entry.rgba;
          px[0] = as_u8((float)(uint8_t)(a >> 24) * strength);
          px[1] = as_u8((float)(uint8_t)(a >> 16) * strength);
          px[2] = as_u8((float)(uint8_t)(a >> 8) * strength);
          px[3] = 255;
        } else {
          px[0] = px[1] = px[2] = px[3] = 0;
          ++local;
        }
      }
    bad += local;
  };
  if (threads <= 1 || (uint64_t)W * H < 4096) {
    work(0, W);
  } else {
    std::vector<std::thread> pool;
    const uint32_t chunk = (W + threads - 1) / threads;
    for (int k = 0; k < threads; ++k) {
      const uint32_t b = (uint32_t)k * chunk, e = std::min(W, b + chunk);
      if (b >= e) break;
      pool.emplace_back(work, b, e);
    }
    for (auto& th : pool) th.join();
  }
  if (unshaded) *unshaded = bad.load();
  return ORC_OK;
}

uint64_t orc_node_count(void* tree) { return static_cast<Octree*>(tree)->nodes.len(); }

// ---- MIP maps (octree/mipmap.rs, the StrategyUpdater of octree/mod.rs) ----
int orc_mip_switch(void* tree, int enabled) {
  return guarded([&] {
    static_cast<Octree*>(tree)->switch_albedo_mip_maps(enabled != 0);
    return ORC_OK;
  });
}
int orc_mip_set_method(void* tree, uint32_t level, uint32_t method, float thr) {
  if (method > 4) return ORC_ERR_ARGUMENT;
  Octree* t = static_cast<Octree*>(tree);
  if (method >= 3) thr = std::min(std::max(thr, 0.0f), 1.0f);  // set_method_at_internal clamps thresholds
  t->mip_methods[level] = Octree::MipSampler{(Octree::MipMethod)method, thr};
  return ORC_OK;
}
int orc_mip_set_color_threshold(void* tree, uint32_t level, float thr) {
  static_cast<Octree*>(tree)->mip_color_thr[level] = std::min(std::max(thr, 0.0f), 1.0f);
  return ORC_OK;
}
int orc_mip_recalculate(void* tree) {
  return guarded([&] {
    static_cast<Octree*>(tree)->recalculate_mips();
    return ORC_OK;
  });
}
int orc_mip_sample_root(void* tree, uint32_t octant, uint32_t x, uint32_t y, uint32_t z, uint32_t out[3]) {
  const uint32_t p[3] = {x, y, z};
  return guarded([&] {
    Entry e = static_cast<Octree*>(tree)->sample_root_mip((uint8_t)octant, p);
    out[0] = e.kind;
    out[1] = e.rgba;
    out[2] = e.user;
    return ORC_OK;
  });
}
// The MIP brick of a node: kind (0 empty, 1 solid, 2 parted, 3 no entry: past node_mips), its
// solid value or brick_dim^3 values into `values` (when not NULL).
int orc_node_mip(void* tree, uint64_t key, uint32_t* kind, uint32_t* values) {
  const Octree* t = static_cast<const Octree*>(tree);
  if (key >= t->node_mips.size()) {
    *kind = 3;
    return ORC_OK;
  }
  const BrickData& m = t->node_mips[key];
  *kind = m.kind == B_EMPTY ? 0u : (m.kind == B_SOLID ? 1u : 2u);
  if (values && m.kind == B_SOLID) values[0] = m.solid;
  if (values && m.kind == B_PARTED) std::copy(m.parted.begin(), m.parted.end(), values);
  return ORC_OK;
}

static uint64_t fnv_brick(const std::vector<uint32_t>& v) {
  uint64_t h = 1469598103934665603ull;
  for (uint32_t w : v)
    for (int b = 0; b < 4; ++b) {
      h ^= (w >> (8 * b)) & 0xFF;
      h *= 1099511628211ull;
    }
  return h ^ v.size();
}

int orc_node_record(void* tree, uint64_t key, uint64_t rec[40]) {
  Octree* t = static_cast<Octree*>(tree);
  std::memset(rec, 0, sizeof(uint64_t) * 40);
  if (key >= t->nodes.len()) return ORC_ERR_ARGUMENT;
  const PoolItem& it = t->nodes.buffer[key];
  rec[0] = it.reserved;
  rec[1] = it.item.kind;
  rec[2] = it.item.kind == C_INTERNAL ? it.item.ocbits : 0;
  if (key < t->node_children.size()) {
    const NodeChildren& c = t->node_children[key];
    rec[3] = c.kind;
    for (int i = 0; i < 8; ++i) rec[4 + i] = c.kind == CH_CHILDREN ? c.c[i] : 0;
    rec[12] = c.kind == CH_BITMAP ? c.bitmap : 0;
  } else {
    rec[3] = 0xFF;
  }
  int nb = it.item.kind == C_LEAF ? 8 : (it.item.kind == C_UNIFORM ? 1 : 0);
  for (int i = 0; i < nb; ++i) {
    const BrickData& b = it.item.bricks[i];
    rec[13 + i] = b.kind;
    rec[21 + i] = b.kind == B_SOLID ? b.solid : 0;
    rec[29 + i] = b.kind == B_PARTED ? fnv_brick(b.parted) : 0;
  }
  if (key >= t->node_mips.size()) {
    rec[37] = 3;
  } else {
    const BrickData& m = t->node_mips[key];
    rec[37] = m.kind;
    rec[38] = m.kind == B_SOLID ? m.solid : 0;
    rec[39] = m.kind == B_PARTED ? fnv_brick(m.parted) : 0;
  }
  return ORC_OK;
}

uint64_t orc_palette(void* tree, int which, uint32_t* out, uint64_t max) {
  Octree* t = static_cast<Octree*>(tree);
  const auto& p = which == 0 ? t->color_palette : t->data_palette;
  if (out)
    for (uint64_t i = 0; i < std::min<uint64_t>(max, p.size()); ++i) out[i] = p[i];
  return p.size();
}

void orc_luts(uint64_t ray_to_node[512], uint32_t octant_step[27], uint64_t octant_mask[8], uint8_t bitmap_index[64],
              float octant_offset[24]) {
  const Luts& L = luts();
  std::memcpy(ray_to_node, L.ray_to_node, sizeof(L.ray_to_node));
  std::memcpy(octant_step, L.octant_step, sizeof(L.octant_step));
  std::memcpy(octant_mask, L.octant_mask, sizeof(L.octant_mask));
  std::memcpy(bitmap_index, L.bitmap_index, sizeof(L.bitmap_index));
  for (int i = 0; i < 8; ++i) {
    octant_offset[i * 3 + 0] = OCTANT_OFFSET_REGION_LUT[i].x;
    octant_offset[i * 3 + 1] = OCTANT_OFFSET_REGION_LUT[i].y;
    octant_offset[i * 3 + 2] = OCTANT_OFFSET_REGION_LUT[i].z;
  }
}

int orc_intersect_ray(const float cube[4], const float ray[6], float* distance) {
  Cube c{V3f{cube[0], cube[1], cube[2]}, cube[3]};
  Ray r{V3f{ray[0], ray[1], ray[2]}, V3f{ray[3], ray[4], ray[5]}};
  return intersect_ray(c, r, distance);
}
void orc_cube_impact_normal(const float cube[4], const float point[3], float out[3]) {
  V3f n = cube_impact_normal(Cube{V3f{cube[0], cube[1], cube[2]}, cube[3]}, V3f{point[0], point[1], point[2]});
  out[0] = n.x;
  out[1] = n.y;
  out[2] = n.z;
}
uint32_t orc_hash_region(const float offset[3], float size_half) {
  return hash_region(V3f{offset[0], offset[1], offset[2]}, size_half);
}
uint64_t orc_position_in_bitmap(uint64_t x, uint64_t y, uint64_t z, uint64_t brick_size) {
  return position_in_bitmap_64bits(V3u{x, y, z}, brick_size);
}
uint64_t orc_set_occupancy(uint64_t x, uint64_t y, uint64_t z, uint64_t size, uint64_t brick_dim, int occupied,
                           uint64_t bitmap) {
  set_occupancy_in_bitmap_64bits(V3u{x, y, z}, size, brick_dim, occupied != 0, &bitmap);
  return bitmap;
}
int orc_plane_line_intersection(const float pp[3], const float pn[3], const float lo[3], const float ld[3], float* out) {
  return plane_line_intersection(V3f{pp[0], pp[1], pp[2]}, V3f{pn[0], pn[1], pn[2]}, V3f{lo[0], lo[1], lo[2]},
                                 V3f{ld[0], ld[1], ld[2]}, out)
             ? 1
             : 0;
}
void orc_child_bounds(const float cube[4], uint32_t octant, float out[4]) {
  Cube c = child_bounds_for(Cube{V3f{cube[0], cube[1], cube[2]}, cube[3]}, (uint8_t)octant);
  out[0] = c.min_position.x;
  out[1] = c.min_position.y;
  out[2] = c.min_position.z;
  out[3] = c.size;
}
void orc_dda_step(const float ray[6], float point[3], const float cube[4], float step_out[3]) {
  Ray r{V3f{ray[0], ray[1], ray[2]}, V3f{ray[3], ray[4], ray[5]}};
  V3f p{point[0], point[1], point[2]};
  V3f s = Octree::dda_step_to_next_sibling(r, p, Cube{V3f{cube[0], cube[1], cube[2]}, cube[3]},
                                           Octree::get_dda_scale_factors(r));
  point[0] = p.x;
  point[1] = p.y;
  point[2] = p.z;
  step_out[0] = s.x;
  step_out[1] = s.y;
  step_out[2] = s.z;
}
uint64_t orc_flat_projection(uint64_t x, uint64_t y, uint64_t z, uint64_t size) { return flat_projection(x, y, z, size); }

// BrickData::is_empty_throughout / is_part_empty_throughout (node.rs:75-209) on a brick of kind 0
// (Empty), 1 (Solid: pix[0]) or 2 (Parted: dim^3 values) against the given palettes: 1 empty, 0 not,
// ORC_ERR_REFERENCE_PANIC where the reference panics.  part < 0: the whole octant; else part is the octant of
// the part inside it (the brick tests of src/octree/tests.rs:8-158).
int orc_brick_empty_throughout(const uint32_t* pix, uint32_t dim, uint32_t kind, uint32_t octant, int32_t part,
                               const uint32_t* colors, uint32_t n_colors, const uint32_t* datas, uint32_t n_datas) {
  Octree t;
  t.color_palette.assign(colors, colors + n_colors);
  t.data_palette.assign(datas, datas + n_datas);
  BrickData b;
  if (kind == 1) {
    b.kind = B_SOLID;
    b.solid = pix[0];
  } else if (kind == 2) {
    b.kind = B_PARTED;
    b.parted.assign(pix, pix + (size_t)dim * dim * dim);
  }
  return guarded([&] {
    const bool e = part < 0 ? t.is_empty_throughout(b, (uint8_t)octant, dim)
                            : t.is_part_empty_throughout(b, (uint8_t)octant, (uint8_t)part, dim);
    return e ? 1 : 0;
  });
}

// NodeStack<T, SIZE> (raytracing_on_cpu.rs:20-82) with a runtime SIZE for the ring-stack tests
struct StackHarness {
  std::vector<int32_t> data;
  size_t head = 0;
  uint8_t count = 0;
};
void* orc_stack_new(uint32_t size) {
  if (size < 1 || size > 8) return nullptr;
  StackHarness* s = new StackHarness();
  s->data.assign(size, 0);
  return s;
}
void orc_stack_free(void* s) { delete static_cast<StackHarness*>(s); }
void orc_stack_push(void* sp, int32_t v) {
  StackHarness* s = static_cast<StackHarness*>(sp);
  size_t SIZE = s->data.size();
  s->head = (s->head + 1) % SIZE;
  s->count = (uint8_t)std::min<size_t>(s->count + 1, SIZE);
  s->data[s->head] = v;
}
int orc_stack_pop(void* sp, int32_t* out) {
  StackHarness* s = static_cast<StackHarness*>(sp);
  if (s->count == 0) return 0;
  s->count -= 1;
  *out = s->data[s->head];
  s->head = s->head == 0 ? s->data.size() - 1 : s->head - 1;
  return 1;
}
int orc_stack_last(void* sp, int32_t* out) {
  StackHarness* s = static_cast<StackHarness*>(sp);
  if (s->count == 0) return 0;
  *out = s->data[s->head];
  return 1;
}
int orc_stack_add_last(void* sp, int32_t delta) {
  StackHarness* s = static_cast<StackHarness*>(sp);
  if (s->count == 0) return 0;
  s->data[s->head] += delta;
  return 1;
}
int orc_stack_is_empty(void* sp) { return static_cast<StackHarness*>(sp)->count == 0; }

}  // extern "C"
