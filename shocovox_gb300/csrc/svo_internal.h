// svo_internal.h -- definitions shared by libsvo's translation units: the
// scene handle, the device image layout and the error reporting helpers.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/svo.h"
#include "svo_octree.h"

namespace svo {

// One node of the device image: 64 bytes, 64-byte aligned, so a node visit
// reads one 32-byte sector for (ocbits, meta) and one for the 8 slots.
struct alignas(64) DevNode {
  uint64_t ocbits;   // stored_occupied_bits (src/octree/detail.rs:508-528)
  uint32_t meta;     // [1:0] content kind, [2] reserved, [23:8] 2-bit brick kind per octant,
                     // [25:24] MIP brick kind (3: the key has no node_mips entry)
  uint32_t mip;      // the node's MIP brick: Solid value or arena slot
  uint32_t pad1[4];
  uint32_t slot[8];  // Internal: child key or kInvalidChild; Leaf: brick per octant; UniformLeaf: slot[0]
};
static_assert(sizeof(DevNode) == 64, "DevNode must be 64 bytes");

constexpr uint32_t kInvalidChild = 0xFFFFFFFFu;

// svo_hits is an array of kHitFields pointers; bytes per ray of each field, in declaration order.
constexpr int kHitFields = 18;
constexpr size_t kHitFieldBytes[kHitFields] = {1, 1, 1, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4};
static_assert(sizeof(svo_hits) == kHitFields * sizeof(void*), "svo_hits must hold only the field pointers");
inline bool counts_requested(const svo_hits& h) {
  return h.node_visits || h.child_reads || h.voxel_reads || h.run_visits;
}

// Everything a cast kernel needs to read one scene (all device pointers).
struct SceneView {
  const DevNode* nodes;
  const uint32_t* voxels;  // brick arena: slot * D^3 PaletteIndexValues
  const uint32_t* vbits;   // per slot: vwords words, bit f set <=> voxel f is not empty
  const uint32_t* colors;  // colour palette, 0xRRGGBBAA
  const uint32_t* datas;   // user-data palette
  uint32_t n_nodes, n_colors, n_datas;
  uint32_t dim;     // brick dimension D
  uint32_t vwords;  // max(1, D^3 / 32)
  float size;       // octree size
  float inv_size;   // 1 / size (exact: a power of two)
  float inv_dim;    // 1 / D (exact: a power of two)
  uint32_t literal; // 1: every ray takes the literal form of the cast (diagnostics)
  uint32_t mips;    // MIP maps enabled (get_by_ray_at_lod reads node MIPs)
  float mip_top;    // log2(size / D): the MIP level the LOD cast starts at (an integer)
};

// Cast form selected by svo_set_cast_mode (0 automatic, 1 literal only).
extern int g_cast_mode;

struct CastQueues;  // work counters of the queued cast (svo_device.cu)

struct DeviceImage {
  DevNode* nodes = nullptr;
  uint32_t* voxels = nullptr;
  uint32_t* vbits = nullptr;
  uint32_t* colors = nullptr;
  uint32_t* datas = nullptr;
  uint64_t node_cap = 0, brick_cap = 0, color_cap = 0, data_cap = 0;
  uint64_t n_nodes = 0, n_bricks = 0, n_colors = 0, n_datas = 0;
  bool valid = false;
  // host mirror of the node records and voxel bits (source of in-place syncs)
  std::vector<DevNode> host_nodes;
  std::vector<uint32_t> host_vbits;
  // workspace of svo_cast_host (device buffers, grown on demand)
  void* ws = nullptr;
  uint64_t ws_bytes = 0;
  // one work counter per stream that casts this scene; kept across re-uploads
  CastQueues* queues = nullptr;
};

}  // namespace svo

struct svo_scene {
  svo::HostOctree tree;
  svo::DeviceImage dev;
};

namespace svo {
struct CameraFrame {
  float fwd[3], right[3];
  float tan_half, aspect;
};
void camera_frame(const float eye[3], const float target[3], float fov_deg, uint32_t width, uint32_t height,
                  CameraFrame* out);
// device image size in bytes: as allocated (uploaded scene) or as a full upload would allocate
uint64_t device_image_bytes(const svo_scene* s);
uint64_t device_image_bytes_estimate(const svo_scene* s);
void set_error(const std::string& msg);
svo_status fail(svo_status code, const std::string& msg);
SceneView scene_view(const svo_scene* s);
}  // namespace svo
