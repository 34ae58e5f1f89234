// svo_internal.h -- definitions shared by libsvo's translation units: the
// scene handle, the device image layout and the error reporting helpers.
#pragma once

#include <cuda_runtime.h>

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
  uint16_t stage[8]; // Internal: the child's index in the scene's top table, kNotStaged when it has none
  uint32_t slot[8];  // Internal: child key or kInvalidChild; Leaf: brick per octant; UniformLeaf: slot[0]
};
static_assert(sizeof(DevNode) == 64, "DevNode must be 64 bytes");

constexpr uint32_t kInvalidChild = 0xFFFFFFFFu;

// Top table of a scene: its Internal nodes of depth < kMaxStageDepth (the root has depth 0) in
// breadth-first order, children in octant order, so the nodes of depth < K are the table's first
// top_count[K] records.  A cast with staging depth K copies those records into shared memory and
// reads them from there; a node key with kStagedBit set is an index into that copy.
constexpr uint32_t kMaxStageDepth = 4;
constexpr uint32_t kMaxStaged = 1 + 8 + 64 + 512;  // records of depth < 4
constexpr uint16_t kNotStaged = 0xFFFFu;
constexpr uint32_t kStagedBit = 0x80000000u;

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
  const DevNode* top;  // the top table (breadth-first Internal nodes of depth < kMaxStageDepth)
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
  DevNode* top = nullptr;                         // kMaxStaged records
  uint32_t top_count[kMaxStageDepth + 1] = {};    // records of depth < K, K = 0..kMaxStageDepth
  std::vector<uint32_t> top_keys;                 // node key of each top-table record
  std::vector<DevNode> host_top;                  // the records as uploaded
  bool valid = false;
  bool ordered = false;    // image arrays from the stream-ordered pool (a server's residency)
  bool mirror_ok = false;  // host_nodes / host_vbits / the top table match the tree but for dirty elements
  // A server's resident image is one block of the stream-ordered pool (`block`, the arrays above point
  // into it), copied from a pinned host image laid out like it (`blob`).  While the tree is unchanged
  // the blob stays valid across evictions, so uploading the scene again is one allocation and
  // asynchronous copies, with no host work.
  void* block = nullptr;
  uint8_t* blob = nullptr;
  uint64_t blob_bytes = 0;
  uint32_t blob_top_count[kMaxStageDepth + 1] = {};
  bool blob_ok = false;
  cudaEvent_t blob_done = nullptr;  // recorded after the last copy out of the blob
  // recorded on the upload's stream after a server's upload of the image: a launch on another stream
  // waits for it before it reads the image
  cudaEvent_t ready = nullptr;
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
// A server's residency: the image allocated from the stream-ordered pool on `st` (unless the caller's
// allocator is installed), and given back the same way, so that evicting one scene and uploading
// another does not wait for the whole device.  The evicted scene must have no cast in flight.  The
// upload records DeviceImage::ready on `st`: a cast on another stream waits for it.
svo_status upload_ordered(svo_scene* s, cudaStream_t st);
svo_status evict_ordered(svo_scene* s, cudaStream_t st);
// records of the top table that a cast with staging depth `depth` copies (0 when the scene has none)
uint32_t staged_records(const svo_scene* s, uint32_t depth);
}  // namespace svo
