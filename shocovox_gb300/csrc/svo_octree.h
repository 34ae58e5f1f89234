// svo_octree.h -- host side of libsvo: the octree that construction and
// update operate on, stored as flat pools that map one-to-one onto the
// device image.
//
// Node numbering, pool reuse and every structural decision follow the
// reference octree (shocovox-rs v0.11.1, src/octree/**, src/object_pool.rs)
// so that node keys and brick contents match it exactly; only the storage
// differs: node content, children and bricks live in flat arrays and a
// brick arena instead of per-node enums and heap vectors.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace svo {

constexpr uint32_t kEmpty32 = 0xFFFFFFFFu;
constexpr uint32_t kEmpty16 = 0xFFFFu;
constexpr uint32_t kNoSlot = 0xFFFFFFFFu;

enum ContentKind : uint8_t { kNothing = 0, kInternal = 1, kLeaf = 2, kUniform = 3 };
enum BrickKind : uint8_t { kBrickEmpty = 0, kBrickSolid = 1, kBrickParted = 2 };
enum ChildrenKind : uint8_t { kNoChildren = 0, kChildren = 1, kBitmap = 2 };

// The reference would panic (slice index out of bounds, unbounded recursion).
struct ReferencePanic : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct BrickRef {
  uint8_t kind = kBrickEmpty;
  uint32_t v = 0;  // Solid: PaletteIndexValues; Parted: arena slot
};

// Node content held by value while it is moved between nodes.  Parted bricks
// are owned arena slots; whoever holds a Content must release or store it.
struct Content {
  uint8_t kind = kNothing;
  uint64_t ocbits = 0;
  BrickRef b[8];
};

struct Cube {
  float x, y, z, size;
};

// Fixed-size voxel bricks (D^3 PaletteIndexValues each) in one growing array.
class BrickArena {
 public:
  void init(uint32_t dim);
  uint32_t alloc();                   // contents undefined
  uint32_t alloc_fill(uint32_t value);
  uint32_t clone(uint32_t slot);
  void release(uint32_t slot);
  uint32_t* at(uint32_t slot) { return &data_[(size_t)slot * len_]; }
  // an index whose voxel differed from voxel 0 when last looked at (a hint: checked before use)
  uint32_t& differs_at(uint32_t slot) const { return hint_[2 * (size_t)slot]; }
  // a 2x2x2 cell (at half resolution, x + y H + z H^2) that was not uniform when last looked at
  uint32_t& mixed_cell(uint32_t slot) const { return hint_[2 * (size_t)slot + 1]; }
  const uint32_t* at(uint32_t slot) const { return &data_[(size_t)slot * len_]; }
  uint32_t len() const { return len_; }
  uint32_t slots() const { return (uint32_t)live_.size(); }
  uint64_t live_count() const { return live_count_; }
  bool live(uint32_t s) const { return s < live_.size() && live_[s]; }
  void mark(uint32_t s) {
    if (s < dirty_.size()) dirty_[s] = 1;
  }
  std::vector<uint8_t>& dirty() { return dirty_; }
  const std::vector<uint32_t>& raw() const { return data_; }

 private:
  uint32_t len_ = 0;
  std::vector<uint32_t> data_;
  mutable std::vector<uint32_t> hint_;
  std::vector<uint8_t> live_, dirty_;
  std::vector<uint32_t> free_;
  uint64_t live_count_ = 0;
};

struct Entry {
  uint32_t kind = 0, rgba = 0, user = 0;
};

class HostOctree {
 public:
  // Octree::new (src/octree/mod.rs:173-206); returns an svo_status code.
  static int create(uint32_t size, uint32_t dim, HostOctree* t);

  int insert_at_lod(bool overwrite_if_empty, const uint32_t pos[3], uint32_t insert_size, const Entry& data);
  int clear_at_lod(const uint32_t pos[3], uint32_t clear_size);
  Entry get(const uint32_t pos[3]);
  void node_record(uint64_t key, uint64_t rec[40]) const;

  // --- MIP maps (src/octree/mipmap.rs) ---
  enum MipMethod : uint32_t { kMipBox = 0, kMipPoint = 1, kMipPointBD = 2, kMipPosterize = 3, kMipPosterizeBD = 4 };
  struct MipSampler {
    uint32_t method;
    float thr;
  };
  void switch_albedo_mip_maps(bool enabled);
  void set_mip_method(uint32_t level, uint32_t method, float thr);
  void set_mip_color_threshold(uint32_t level, float thr);
  void recalculate_mips();
  Entry sample_root_mip(uint8_t octant, const uint32_t pos[3]);

  // --- persistence: Octree::to_bytes / from_bytes (src/octree/mod.rs:138-168, src/convert/bytecode.rs) ---
  void encode(std::string& out) const;
  // returns an svo_status code; `t` must be default-constructed
  static int decode(const uint8_t* bytes, size_t length, HostOctree* t, std::string* error);

  // --- state (read by the device image builder) ---
  uint32_t size = 0, dim = 0;
  bool auto_simplify = true;
  std::vector<uint8_t> reserved, kind;
  std::vector<uint64_t> ocbits;
  std::vector<BrickRef> bricks;  // 8 per node
  std::vector<uint8_t> ch_kind;
  std::vector<uint32_t> ch;  // 8 per node
  std::vector<uint64_t> ch_bitmap;
  size_t first_available = 0;
  std::vector<uint32_t> colors, datas;
  BrickArena arena;
  std::vector<uint8_t> node_dirty;
  uint64_t colors_synced = 0, datas_synced = 0;
  bool structure_grew = true;
  // node_mips: one brick per node key, as long as the reference's vector (which is resized beside
  // most, not all, node pushes); Parted MIP bricks live in the arena
  bool mips_enabled = false;
  std::vector<BrickRef> mips;
  std::vector<std::pair<uint32_t, MipSampler>> mip_methods;  // level -> sampler
  std::vector<std::pair<uint32_t, float>> mip_color_thr;     // level -> colour matching threshold

  bool pix_empty(uint32_t p) const;
  uint64_t stored_occupied_bits(size_t k) const;
  size_t nodes() const { return reserved.size(); }
  bool key_valid(uint64_t k) const { return k < reserved.size() && reserved[k]; }

 private:
  int depth_ = 0;
  std::vector<uint32_t> unified_;     // scratch brick of simplify()
  std::vector<uint32_t> dilute_src_;  // scratch copy of dilute()'s source brick
  struct PathFrame {
    uint32_t key;
    Cube b;
  };
  std::vector<PathFrame> path_;       // scratch: the nodes an insert or clear walks down
  std::unordered_map<uint32_t, uint32_t> color_index_, data_index_;

  // pool (src/object_pool.rs:151-240)
  size_t pool_allocate();
  size_t push(Content&& c);
  void pool_free(size_t k);
  void pool_swap(size_t a, size_t b);
  void grow_nodes(size_t n);
  void touch(size_t k) { node_dirty[k] = 1; }

  // content handling
  Content take(size_t k);
  void store(size_t k, Content&& c);
  void release(Content& c);
  Content clone_content(size_t k);
  BrickRef clone_brick(const BrickRef& b);
  void set_children_none(size_t k);
  void set_children_bitmap(size_t k, uint64_t bits);
  uint64_t child(size_t k, uint8_t octant) const {
    return ch_kind[k] == kChildren ? (uint64_t)ch[k * 8 + octant] : (uint64_t)kEmpty32;
  }
  uint32_t* child_mut(size_t k, size_t index);
  void children_clear(size_t k, size_t index);
  void check_key(uint64_t k) const {
    if (k >= reserved.size()) throw ReferencePanic("node index out of bounds");
  }

  uint32_t add_color(uint32_t rgba);
  uint32_t add_data(uint32_t v);
  uint32_t add_to_palette(const Entry& e);
  Entry pix_entry(uint32_t p) const;

  // bricks
  bool brick_homogeneous(const BrickRef& b, uint32_t* out) const;
  bool brick_simplify(BrickRef& b);
  bool brick_equal(const BrickRef& a, const BrickRef& b) const;
  bool brick_empty_throughout(const BrickRef& b, uint8_t octant) const;
  bool brick_part_empty_throughout(const BrickRef& b, uint8_t part, uint8_t target) const;
  uint64_t brick_occupied_bits(const uint32_t* v) const;
  uint64_t brick_ref_occupied_bits(const BrickRef& b) const;
  void dilute(uint32_t src_slot, uint32_t out_slots[8]);
  size_t update_brick(bool overwrite, uint32_t slot, const Cube& bounds, const uint32_t pos[3], uint32_t size,
                      uint32_t data);

  // structure
  bool content_is_empty(size_t k) const;
  bool content_is_all(size_t k, uint32_t data) const;
  bool content_compare(size_t a, size_t b) const;
  bool should_bitmap_be_empty_at_index(size_t k, const uint64_t idx[3]);
  bool should_bitmap_be_empty_at_octants(size_t k, uint8_t oct, uint8_t child_oct);
  bool node_empty_at(size_t k, uint8_t oct);
  void subdivide_leaf_to_nodes(size_t k, size_t target_octant);
  BrickRef try_brick_from_node(uint64_t k);
  void deallocate_children_of(uint64_t k);
  void store_occupied_bits(size_t k, uint64_t bits);
  size_t leaf_update(bool overwrite, size_t k, const Cube& node_b, const Cube& target_b, size_t target_octant,
                     const uint32_t pos[3], uint32_t size, uint32_t target_content);
  bool simplify(uint64_t k);

  // MIP maps
  Entry get_internal(size_t k, Cube cb, const uint32_t pos[3]);
  void mips_resize() {
    for (size_t k = mips.size(); k < nodes(); ++k) touch(k);  // their device records gain an entry
    if (mips.size() < nodes()) mips.resize(nodes());
  }
  BrickRef& mip(size_t k) {
    if (k >= mips.size()) throw ReferencePanic("node_mips index out of bounds");
    return mips[k];
  }
  void set_mip(size_t k, BrickRef b);
  void update_mip(size_t k, const Cube& b, const uint32_t pos[3]);
  void recalculate_mip(size_t k, const Cube& b);
};

}  // namespace svo
