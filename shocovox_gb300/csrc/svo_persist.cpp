// svo_persist.cpp -- the reference's bytecode format for octrees (Octree::to_bytes / from_bytes,
// src/octree/mod.rs:138-168), a bencode list written by src/convert/bytecode.rs and
// src/object_pool.rs:25-140:
//
//   octree   = l  i<auto_simplify>e  i<octree_size>e  i<brick_dim>e  pool  children  mips
//                 colours  data  strategy  e
//   pool     = l  i<first_available>e  l (l i<reserved>e content e)* e  e
//   content  = "#" | l "##" i<occupied bits>e e | l "###" brick*8 e | l "##u#" brick e
//   brick    = "#b" | l "#b#" i<voxel>e e | l "##b#" i<len>e i<voxel>e*len "#" e
//   children = l ( l "##c##" i<child>e*8 e | "##x##" | l "##b##" i<bitmap>e e )* e
//   mips     = l brick* e;  colours = l (l i<r>e i<g>e i<b>e i<a>e e)* e;  data = l i<u32>e* e
//   strategy = l i<enabled>e i<n>e (i<level>e i<method>e)*n i<m>e (i<level>e i<thr*1000>e)*m e
//   method   = 0 BoxFilter | 1 PointFilter | 2 PointFilterBD | 3 + thr*1000 Posterize
//              | 1003 + thr*1000 PosterizeBD
//
// The strategy's maps are HashMaps in the reference, written in their per-process iteration
// order; they are written here in ascending level order (the reader accepts any order).  A node
// the pool has freed keeps its last content in the reference's buffer (ObjectPool::free does not
// clear it) and is never read again; it is written here as "#".
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "svo_octree.h"

namespace svo {
namespace {

// ---------------------------------------------------------------- writing
struct Writer {
  std::string& o;
  void i(uint64_t v) {
    o += 'i';
    o += std::to_string(v);
    o += 'e';
  }
  void s(const char* str) {
    const size_t n = std::strlen(str);
    o += std::to_string(n);
    o += ':';
    o.append(str, n);
  }
  void l() { o += 'l'; }
  void e() { o += 'e'; }
};

// ---------------------------------------------------------------- reading
struct Item {
  enum Kind { kInt, kBytes, kList } kind;
  uint64_t v = 0;
  std::string bytes;
  std::vector<Item> list;
};

struct Reader {
  const uint8_t* p;
  const uint8_t* end;
  std::string err;
  int depth = 0;

  bool fail(const std::string& what) {
    if (err.empty()) err = what;
    return false;
  }
  bool parse(Item& out) {
    if (p >= end) return fail("unexpected end of data");
    if (++depth > 64) return fail("nesting too deep");
    bool ok;
    if (*p == 'i') {
      ++p;
      out.kind = Item::kInt;
      uint64_t v = 0;
      bool any = false;
      while (p < end && *p >= '0' && *p <= '9') {
        const uint64_t d = (uint64_t)(*p - '0');
        if (v > (UINT64_MAX - d) / 10) return fail("integer out of range");
        v = v * 10 + d;
        ++p;
        any = true;
      }
      if (!any || p >= end || *p != 'e') return fail("malformed integer");
      ++p;
      out.v = v;
      ok = true;
    } else if (*p == 'l') {
      ++p;
      out.kind = Item::kList;
      ok = true;
      while (ok) {
        if (p >= end) return fail("unterminated list");
        if (*p == 'e') {
          ++p;
          break;
        }
        out.list.emplace_back();
        ok = parse(out.list.back());
      }
    } else if (*p >= '0' && *p <= '9') {
      uint64_t n = 0;
      while (p < end && *p >= '0' && *p <= '9') {
        n = n * 10 + (uint64_t)(*p - '0');
        if (n > (uint64_t)(end - p)) return fail("byte string longer than the data");
        ++p;
      }
      if (p >= end || *p != ':' || n > (uint64_t)(end - p - 1)) return fail("malformed byte string");
      ++p;
      out.kind = Item::kBytes;
      out.bytes.assign(reinterpret_cast<const char*>(p), n);
      p += n;
      ok = true;
    } else {
      return fail("unexpected byte in the bencode data");
    }
    --depth;
    return ok;
  }
};

bool is_int(const Item& it) { return it.kind == Item::kInt; }
bool is_tag(const Item& it, const char* tag) { return it.kind == Item::kBytes && it.bytes == tag; }

}  // namespace

void HostOctree::encode(std::string& out) const {
  Writer w{out};
  auto brick = [&](const BrickRef& b) {
    if (b.kind == kBrickEmpty) {
      w.s("#b");
    } else if (b.kind == kBrickSolid) {
      w.l();
      w.s("#b#");
      w.i(b.v);
      w.e();
    } else {
      w.l();
      w.s("##b#");
      w.i(arena.len());
      const uint32_t* v = arena.at(b.v);
      for (uint32_t j = 0; j < arena.len(); ++j) w.i(v[j]);
      w.s("#");
      w.e();
    }
  };
  w.l();
  w.i(auto_simplify ? 1 : 0);
  w.i(size);
  w.i(dim);
  // nodes (ObjectPool)
  w.l();
  w.i(first_available);
  w.l();
  for (size_t k = 0; k < nodes(); ++k) {
    w.l();
    w.i(reserved[k]);
    if (!reserved[k] || kind[k] == kNothing) {
      w.s("#");
    } else if (kind[k] == kInternal) {
      w.l();
      w.s("##");
      w.i(ocbits[k]);
      w.e();
    } else if (kind[k] == kLeaf) {
      w.l();
      w.s("###");
      for (int i = 0; i < 8; ++i) brick(bricks[k * 8 + i]);
      w.e();
    } else {
      w.l();
      w.s("##u#");
      brick(bricks[k * 8]);
      w.e();
    }
    w.e();
  }
  w.e();
  w.e();
  // node_children
  w.l();
  for (size_t k = 0; k < nodes(); ++k) {
    if (ch_kind[k] == kChildren) {
      w.l();
      w.s("##c##");
      for (int i = 0; i < 8; ++i) w.i(ch[k * 8 + i]);
      w.e();
    } else if (ch_kind[k] == kBitmap) {
      w.l();
      w.s("##b##");
      w.i(ch_bitmap[k]);
      w.e();
    } else {
      w.s("##x##");
    }
  }
  w.e();
  // node_mips
  w.l();
  for (const BrickRef& m : mips) brick(m);
  w.e();
  // palettes
  w.l();
  for (uint32_t c : colors) {
    w.l();
    w.i(c >> 24);
    w.i((c >> 16) & 0xFFu);
    w.i((c >> 8) & 0xFFu);
    w.i(c & 0xFFu);
    w.e();
  }
  w.e();
  w.l();
  for (uint32_t d : datas) w.i(d);
  w.e();
  // MIP strategy
  auto methods = mip_methods;
  std::sort(methods.begin(), methods.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  auto thresholds = mip_color_thr;
  std::sort(thresholds.begin(), thresholds.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  auto as_u32 = [](float v) -> uint64_t {  // `f32 as u32`
    if (!(v > 0.0f)) return 0;
    if (v >= 4294967296.0f) return 4294967295u;
    return (uint64_t)v;
  };
  w.l();
  w.i(mips_enabled ? 1 : 0);
  w.i(methods.size());
  for (const auto& m : methods) {
    w.i(m.first);
    const uint32_t kind_ = m.second.method;
    if (kind_ <= kMipPointBD)
      w.i(kind_);
    else
      w.i((kind_ == kMipPosterize ? 3u : 1003u) + as_u32(m.second.thr * 1000.0f));
  }
  w.i(thresholds.size());
  for (const auto& t : thresholds) {
    w.i(t.first);
    w.i(as_u32(t.second * 1000.0f));
  }
  w.e();
  w.e();
}

int HostOctree::decode(const uint8_t* bytes, size_t length, HostOctree* t, std::string* error) {
  Reader r{bytes, bytes + length, {}};
  Item root;
  auto bad = [&](const std::string& what) {
    if (error) *error = what;
    return 6;  // SVO_ERR_ARGUMENT
  };
  if (!r.parse(root)) return bad("bencode: " + r.err);
  if (r.p != r.end) return bad("bencode: trailing bytes after the octree");
  if (root.kind != Item::kList || root.list.size() != 9) return bad("octree: expected a list of 9 fields");
  const std::vector<Item>& f = root.list;
  for (int i = 0; i < 3; ++i)
    if (!is_int(f[i])) return bad("octree: auto_simplify, octree_size and brick_dim must be integers");
  if (f[0].v > 1) return bad("octree: auto_simplify must be 0 or 1");
  if (f[1].v > 0xFFFFFFFFu || f[2].v > 0xFFFFFFFFu) return bad("octree: size out of range");
  const int rc = create((uint32_t)f[1].v, (uint32_t)f[2].v, t);
  if (rc != 0) return rc;
  t->auto_simplify = f[0].v == 1;
  const uint32_t len = t->arena.len();
  // bricks: Empty, Solid, or a Parted brick of brick_dim^3 voxels stored in a fresh arena slot
  auto brick = [&](const Item& it, BrickRef* out) {
    if (is_tag(it, "#b")) {
      *out = BrickRef{};
      return true;
    }
    if (it.kind != Item::kList || it.list.empty()) return false;
    if (is_tag(it.list[0], "#b#") && it.list.size() == 2 && is_int(it.list[1]) && it.list[1].v <= 0xFFFFFFFFu) {
      *out = BrickRef{kBrickSolid, (uint32_t)it.list[1].v};
      return true;
    }
    if (!is_tag(it.list[0], "##b#") || it.list.size() < 3 || !is_int(it.list[1]) || it.list[1].v != len ||
        it.list.size() != (size_t)len + 3 || !is_tag(it.list.back(), "#"))
      return false;
    const uint32_t slot = t->arena.alloc();
    uint32_t* v = t->arena.at(slot);
    for (uint32_t j = 0; j < len; ++j) {
      const Item& x = it.list[2 + j];
      if (!is_int(x) || x.v > 0xFFFFFFFFu) {
        t->arena.release(slot);
        return false;
      }
      v[j] = (uint32_t)x.v;
    }
    *out = BrickRef{kBrickParted, slot};
    return true;
  };
  // nodes
  const Item& pool = f[3];
  if (pool.kind != Item::kList || pool.list.size() != 2 || !is_int(pool.list[0]) || pool.list[1].kind != Item::kList)
    return bad("nodes: expected l i<first_available>e l<items>e e");
  const std::vector<Item>& items = pool.list[1].list;
  if (items.empty()) return bad("nodes: the pool holds no root node");
  t->reserved.clear();
  t->kind.clear();
  t->ocbits.clear();
  t->bricks.clear();
  t->ch_kind.clear();
  t->ch.clear();
  t->ch_bitmap.clear();
  t->node_dirty.clear();
  t->grow_nodes(items.size());
  t->first_available = (size_t)pool.list[0].v;
  for (size_t k = 0; k < items.size(); ++k) {
    const Item& it = items[k];
    if (it.kind != Item::kList || it.list.size() != 2 || !is_int(it.list[0]) || it.list[0].v > 1)
      return bad("nodes: item " + std::to_string(k) + " is not l i<reserved>e <content> e");
    t->reserved[k] = (uint8_t)it.list[0].v;
    const Item& c = it.list[1];
    Content content;
    if (is_tag(c, "#")) {
      content.kind = kNothing;
    } else if (c.kind == Item::kList && !c.list.empty() && is_tag(c.list[0], "##") && c.list.size() == 2 &&
               is_int(c.list[1])) {
      content.kind = kInternal;
      content.ocbits = c.list[1].v;
    } else if (c.kind == Item::kList && !c.list.empty() && is_tag(c.list[0], "###") && c.list.size() == 9) {
      content.kind = kLeaf;
      for (int i = 0; i < 8; ++i)
        if (!brick(c.list[1 + i], &content.b[i])) return bad("nodes: a Leaf brick of node " + std::to_string(k));
    } else if (c.kind == Item::kList && !c.list.empty() && is_tag(c.list[0], "##u#") && c.list.size() == 2) {
      content.kind = kUniform;
      if (!brick(c.list[1], &content.b[0])) return bad("nodes: the UniformLeaf brick of node " + std::to_string(k));
    } else {
      return bad("nodes: unknown content of node " + std::to_string(k));
    }
    if (!t->reserved[k]) t->release(content);  // a freed node's content is never read again
    t->store(k, std::move(content));
  }
  // node_children: as long as the pool (the reference grows both together)
  if (f[4].kind != Item::kList || f[4].list.size() != items.size())
    return bad("node_children: expected one entry per pool item");
  for (size_t k = 0; k < items.size(); ++k) {
    const Item& c = f[4].list[k];
    if (is_tag(c, "##x##")) {
      t->ch_kind[k] = kNoChildren;
    } else if (c.kind == Item::kList && c.list.size() == 9 && is_tag(c.list[0], "##c##")) {
      t->ch_kind[k] = kChildren;
      for (int i = 0; i < 8; ++i) {
        if (!is_int(c.list[1 + i]) || c.list[1 + i].v > 0xFFFFFFFFu) return bad("node_children: bad child key");
        t->ch[k * 8 + i] = (uint32_t)c.list[1 + i].v;
      }
    } else if (c.kind == Item::kList && c.list.size() == 2 && is_tag(c.list[0], "##b##") && is_int(c.list[1])) {
      t->ch_kind[k] = kBitmap;
      t->ch_bitmap[k] = c.list[1].v;
    } else {
      return bad("node_children: unknown entry " + std::to_string(k));
    }
  }
  // node_mips
  if (f[5].kind != Item::kList || f[5].list.size() > items.size()) return bad("node_mips: expected at most one per node");
  t->mips.assign(f[5].list.size(), BrickRef{});
  for (size_t k = 0; k < f[5].list.size(); ++k)
    if (!brick(f[5].list[k], &t->mips[k])) return bad("node_mips: bad MIP brick " + std::to_string(k));
  // palettes (the lookup maps are rebuilt in order, later duplicates winning, as the reference does)
  if (f[6].kind != Item::kList || f[7].kind != Item::kList) return bad("palettes: expected lists");
  for (const Item& c : f[6].list) {
    if (c.kind != Item::kList || c.list.size() != 4) return bad("colour palette: expected l r g b a e");
    uint32_t rgba = 0;
    for (int i = 0; i < 4; ++i) {
      if (!is_int(c.list[i]) || c.list[i].v > 255) return bad("colour palette: channel out of range");
      rgba = (rgba << 8) | (uint32_t)c.list[i].v;
    }
    t->color_index_[rgba] = (uint32_t)t->colors.size();
    t->colors.push_back(rgba);
  }
  for (const Item& d : f[7].list) {
    if (!is_int(d) || d.v > 0xFFFFFFFFu) return bad("data palette: expected u32 integers");
    t->data_index_[(uint32_t)d.v] = (uint32_t)t->datas.size();
    t->datas.push_back((uint32_t)d.v);
  }
  // MIP strategy
  const Item& st = f[8];
  if (st.kind != Item::kList || st.list.size() < 2 || !is_int(st.list[0]) || st.list[0].v > 1 || !is_int(st.list[1]))
    return bad("MIP strategy: expected l i<enabled>e i<n>e ...");
  t->mips_enabled = st.list[0].v == 1;
  const size_t n = (size_t)st.list[1].v;
  if (st.list.size() < 2 + 2 * n + 1) return bad("MIP strategy: too few method entries");
  t->mip_methods.clear();
  for (size_t i = 0; i < n; ++i) {
    const Item& lv = st.list[2 + 2 * i];
    const Item& mv = st.list[3 + 2 * i];
    if (!is_int(lv) || !is_int(mv) || lv.v > 0xFFFFFFFFu) return bad("MIP strategy: bad method entry");
    MipSampler s;
    if (mv.v <= 2) {
      s = MipSampler{(uint32_t)mv.v, 0.0f};
    } else if (mv.v >= 3 && mv.v < 1002) {
      s = MipSampler{kMipPosterize, ((float)mv.v - 3.0f) / 1000.0f};
    } else if (mv.v >= 1003 && mv.v < 2001) {
      s = MipSampler{kMipPosterizeBD, ((float)mv.v - 1003.0f) / 1000.0f};
    } else {
      return bad("MIP strategy: unknown method " + std::to_string(mv.v));
    }
    t->mip_methods.erase(std::remove_if(t->mip_methods.begin(), t->mip_methods.end(),
                                        [&](const auto& e) { return e.first == (uint32_t)lv.v; }),
                         t->mip_methods.end());
    t->mip_methods.push_back({(uint32_t)lv.v, s});
  }
  const size_t at = 2 + 2 * n;
  if (!is_int(st.list[at])) return bad("MIP strategy: expected the threshold count");
  const size_t m = (size_t)st.list[at].v;
  if (st.list.size() != at + 1 + 2 * m) return bad("MIP strategy: wrong number of threshold entries");
  t->mip_color_thr.clear();
  for (size_t i = 0; i < m; ++i) {
    const Item& lv = st.list[at + 1 + 2 * i];
    const Item& tv = st.list[at + 2 + 2 * i];
    if (!is_int(lv) || !is_int(tv) || lv.v > 0xFFFFFFFFu || tv.v > 0xFFFFFFFFu) return bad("MIP strategy: bad threshold");
    t->mip_color_thr.erase(std::remove_if(t->mip_color_thr.begin(), t->mip_color_thr.end(),
                                          [&](const auto& e) { return e.first == (uint32_t)lv.v; }),
                           t->mip_color_thr.end());
    t->mip_color_thr.push_back({(uint32_t)lv.v, (float)tv.v / 1000.0f});
  }
  std::fill(t->node_dirty.begin(), t->node_dirty.end(), 1);
  t->structure_grew = true;
  return 0;
}

}  // namespace svo
