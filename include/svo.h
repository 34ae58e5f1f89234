/*
 * svo.h -- C ABI of libsvo, the GB300-native sparse voxel octree ray caster.
 *
 * libsvo keeps the API surface of shocovox-rs v0.11.1 for the ray-cast hot
 * path: octree construction and update (host side), a device-resident image
 * of the octree that is uploaded once and then updated in place, and the
 * first-hit ray cast `get_by_ray` run as sm_103a CUDA kernels.
 *
 * Conventions
 *  - Every entry point returns an svo_status; 0 is success.  No C++
 *    exception or panic crosses this boundary.  svo_last_error() returns a
 *    thread-local message for the last failure on the calling thread.
 *  - `stream` arguments are cudaStream_t values passed as void* (NULL is the
 *    legacy default stream).  All GPU work is stream ordered; no entry point
 *    synchronises the device except the *_host convenience calls, which
 *    synchronise their stream before returning.
 *  - An svo_scene is externally synchronised for construction/update (like
 *    `&mut Octree`); casts on an uploaded scene may run concurrently on any
 *    number of streams (like `&Octree`).
 *  - Albedo values are packed as the reference's `Albedo::from(u32)` reads
 *    them: 0xRRGGBBAA.  User data is the reference's default T = u32.
 */
#ifndef SVO_H
#define SVO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t svo_status;
enum {
  SVO_OK = 0,
  SVO_ERR_INVALID_SIZE = 1,        /* OctreeError::InvalidSize (src/octree/types.rs:11) */
  SVO_ERR_INVALID_BRICK_DIM = 2,   /* OctreeError::InvalidBrickDimension (types.rs:14) */
  SVO_ERR_INVALID_STRUCTURE = 3,   /* OctreeError::InvalidStructure (types.rs:17) */
  SVO_ERR_INVALID_POSITION = 4,    /* OctreeError::InvalidPosition (types.rs:20) */
  SVO_ERR_REFERENCE_PANIC = 5,     /* the reference panics on this input; the scene is left unusable */
  SVO_ERR_ARGUMENT = 6,            /* NULL handle/pointer or out-of-range argument */
  SVO_ERR_CUDA = 7,                /* a CUDA runtime call failed (see svo_last_error) */
  SVO_ERR_NOT_UPLOADED = 8,        /* cast on a scene without a device image */
  SVO_ERR_OUT_OF_MEMORY = 9,       /* device allocation failed */
  SVO_ERR_BUDGET = 10,             /* a server admission exceeds its device-memory budget */
  SVO_ERR_NOT_FOUND = 11,          /* unknown server scene / request id */
  SVO_ERR_BUSY = 12,               /* request queue full or a result not ready yet */
  SVO_ERR_IO = 13                  /* a file could not be opened, read or written */
};

/* Per-ray status codes written by the cast. */
enum {
  SVO_RAY_MISS = 0,
  SVO_RAY_HIT = 1,
  SVO_RAY_WORK_CAP = 2,      /* 2^22 traversal steps exceeded: the reference would loop forever */
  SVO_RAY_REFERENCE_PANIC = 3 /* the reference indexes BITMAP_INDEX_LUT out of bounds on this ray */
};

/* Operation kinds of svo_op (construction recipes shared by tests and benches). */
enum { SVO_OP_INSERT = 0, SVO_OP_UPDATE = 1, SVO_OP_INSERT_AT_LOD = 2, SVO_OP_CLEAR = 3, SVO_OP_CLEAR_AT_LOD = 4 };
/* Entry kinds (OctreeEntry, src/octree/types.rs:23-36): bit0 albedo, bit1 user data. */
enum { SVO_ENTRY_EMPTY = 0, SVO_ENTRY_VISUAL = 1, SVO_ENTRY_INFORMATIVE = 2, SVO_ENTRY_COMPLEX = 3 };

typedef struct svo_scene svo_scene;

typedef struct {
  uint16_t x, y, z;
  uint8_t op;   /* SVO_OP_* */
  uint8_t kind; /* SVO_ENTRY_* bits */
  uint32_t size;
  uint32_t rgba;
  uint32_t user;
} svo_op; /* 20 bytes */

/* Rays as six f32 arrays (struct of arrays), device or host memory per call. */
typedef struct {
  const float *ox, *oy, *oz;
  const float *dx, *dy, *dz;
} svo_rays;

/* Per-ray results (struct of arrays).  Any pointer may be NULL to skip that output. */
typedef struct {
  uint8_t* status;       /* SVO_RAY_* */
  uint8_t* brick_octant; /* octant of the hit brick inside a Leaf node, 0 for a UniformLeaf */
  uint8_t* entry_kind;   /* SVO_ENTRY_* of the hit voxel */
  uint32_t* node_key;    /* key of the leaf node that holds the hit (reference node numbering) */
  uint32_t* voxel_index; /* flat index x + y*D + z*D*D inside the brick, 0xFFFFFFFF for a Solid brick */
  uint32_t* pix;         /* PaletteIndexValues of the hit voxel */
  uint32_t* albedo;      /* 0xRRGGBBAA, 0 when the entry has no albedo */
  uint32_t* user;        /* user data, 0 when the entry has none */
  float *px, *py, *pz;   /* impact point */
  float *nx, *ny, *nz;   /* impact normal */
  uint32_t* node_visits; /* optional instrumentation counters */
  uint32_t* child_reads;
  uint32_t* voxel_reads;
  uint32_t* run_visits;  /* of node_visits, the restart visits that the cast counted without performing them one
                            by one (runs of restarts whose root test fails; no counterpart in the reference) */
} svo_hits;

typedef struct {
  uint64_t nodes;         /* node pool length (reserved or not) */
  uint64_t reserved_nodes;
  uint64_t parted_bricks; /* live Parted bricks */
  uint64_t colors, datas; /* palette sizes */
  uint64_t device_bytes;  /* bytes of the device image (0 when not uploaded) */
  uint32_t size, brick_dim;
} svo_scene_stats;

const char* svo_last_error(void);
int32_t svo_version(void);

/* ---- construction and update (host) ---------------------------------- */
/* Octree::new (src/octree/mod.rs:173-206) */
svo_status svo_scene_create(uint32_t size, uint32_t brick_dim, svo_scene** out);
void svo_scene_destroy(svo_scene* scene);
/* Octree::auto_simplify (src/octree/types.rs:203) */
svo_status svo_set_auto_simplify(svo_scene* scene, int32_t enabled);
/* Octree::insert (src/octree/update/insert.rs:47-56) */
svo_status svo_insert(svo_scene* scene, uint32_t x, uint32_t y, uint32_t z, uint32_t kind, uint32_t rgba, uint32_t user);
/* Octree::update (insert.rs:79-88) */
svo_status svo_update(svo_scene* scene, uint32_t x, uint32_t y, uint32_t z, uint32_t kind, uint32_t rgba, uint32_t user);
/* Octree::insert_at_lod (insert.rs:63-73) */
svo_status svo_insert_at_lod(svo_scene* scene, uint32_t x, uint32_t y, uint32_t z, uint32_t insert_size, uint32_t kind,
                             uint32_t rgba, uint32_t user);
/* Octree::clear / clear_at_lod (src/octree/update/clear.rs:40-60) */
svo_status svo_clear(svo_scene* scene, uint32_t x, uint32_t y, uint32_t z);
svo_status svo_clear_at_lod(svo_scene* scene, uint32_t x, uint32_t y, uint32_t z, uint32_t clear_size);
/* Applies a recipe of operations in order; *n_done receives how many succeeded. */
svo_status svo_apply_ops(svo_scene* scene, const svo_op* ops, uint64_t n, uint64_t* n_done);
/* Bulk insert of a dense w x h x d block at (x0, y0, z0): voxel (x0 + i, y0 + j, z0 + k) receives
 * rgba[i + w (j + h k)] as its albedo and user[...] as its user data (either array may be NULL, not
 * both), inserted in the nesting of the reference's fill loops (i outermost, k innermost,
 * src/raytracing/tests.rs:693-713) exactly as that many Octree::insert calls; an entry without
 * albedo (alpha 0) or user data (0) inserts nothing.  *n_done receives the number of inserts made. */
svo_status svo_insert_dense(svo_scene* scene, uint32_t x0, uint32_t y0, uint32_t z0, uint32_t w, uint32_t h, uint32_t d,
                            const uint32_t* rgba, const uint32_t* user, uint64_t* n_done);
/* Octree::get (src/octree/mod.rs:209-215) */
svo_status svo_get(svo_scene* scene, uint32_t x, uint32_t y, uint32_t z, uint32_t* kind, uint32_t* rgba, uint32_t* user);
svo_status svo_scene_stats_get(svo_scene* scene, svo_scene_stats* out);

/* ---- persistence: Octree::to_bytes / from_bytes / save / load (src/octree/mod.rs:138-168) in the
 *      reference's bencode bytecode format (src/convert/bytecode.rs) ---------------------------- */
/* Serialises the octree (node pool, children, MIPs, palettes, MIP strategy); with out NULL only
 * *length is set. */
svo_status svo_scene_to_bytes(svo_scene* scene, uint8_t* out, uint64_t capacity, uint64_t* length);
/* A new scene from serialised bytes (no device image yet). */
svo_status svo_scene_from_bytes(const uint8_t* bytes, uint64_t length, svo_scene** out);
svo_status svo_scene_save(svo_scene* scene, const char* path);
svo_status svo_scene_load(const char* path, svo_scene** out);

/* ---- MagicaVoxel .vox import (src/convert/magicavoxel.rs) -------------------------------- */
/* Octree::load_vox_file (magicavoxel.rs:266-286): a new scene of size 2^ceil(log2(extent)) holding
 * every voxel of frame 0 of the file's scene graph, inserted in file order as its palette colour. */
svo_status svo_scene_from_vox(const uint8_t* bytes, uint64_t length, uint32_t brick_dim, svo_scene** out);
svo_status svo_scene_load_vox(const char* path, uint32_t brick_dim, svo_scene** out);
/* The two halves of MIPMapStrategy::load_vox_file (magicavoxel.rs:204-241), which sets the MIP
 * strategy between them: the octree size the file asks for, and the insertion of its voxels into
 * a scene (load_vox_data_internal, magicavoxel.rs:337-385). */
svo_status svo_vox_tree_size(const uint8_t* bytes, uint64_t length, uint32_t* size);
svo_status svo_vox_insert(svo_scene* scene, const uint8_t* bytes, uint64_t length);
/* parse_rotation_matrix (magicavoxel.rs:61-90): the 3x3 row-major matrix of a rotation byte;
 * SVO_ERR_REFERENCE_PANIC where the reference indexes past the matrix. */
svo_status svo_vox_rotation(uint8_t byte, int8_t out[9]);

/* ---- MIP maps: the StrategyUpdater of Octree::albedo_mip_map_resampling_strategy()
 *      (src/octree/mipmap.rs:609-880; disabled by default) ---------------------------- */
typedef enum {
  SVO_MIP_BOX_FILTER = 0,     /* MIPResamplingMethods::BoxFilter */
  SVO_MIP_POINT_FILTER = 1,   /* PointFilter */
  SVO_MIP_POINT_FILTER_BD = 2, /* PointFilterBD */
  SVO_MIP_POSTERIZE = 3,      /* Posterize(threshold) */
  SVO_MIP_POSTERIZE_BD = 4    /* PosterizeBD(threshold) */
} svo_mip_method;
/* switch_albedo_mip_maps: enabling recalculates every MIP (when the root is not empty); while
 * enabled, insert and clear update the MIPs on their path. */
svo_status svo_mip_switch(svo_scene* scene, int32_t enabled);
/* set_method_at: the resampling method of one MIP level (threshold clamped to 0..1). */
svo_status svo_mip_set_method(svo_scene* scene, uint32_t level, uint32_t method, float threshold);
/* set_color_similarity_thr_at: colours closer than threshold * 255 reuse a palette entry. */
svo_status svo_mip_set_color_threshold(svo_scene* scene, uint32_t level, float threshold);
/* recalculate_mips */
svo_status svo_mip_recalculate(svo_scene* scene);
/* sample_root_mip: the root's MIP (octant 8) or a root child's, at a position inside the MIP. */
svo_status svo_mip_sample_root(svo_scene* scene, uint32_t octant, uint32_t x, uint32_t y, uint32_t z, uint32_t* kind,
                               uint32_t* rgba, uint32_t* user);
/* Canonical per-node record used to compare structures (key, content, children, bricks). */
svo_status svo_node_record(svo_scene* scene, uint64_t key, uint64_t rec[40]);
/* Copies palette `which` (0 colours, 1 user data); returns its length. */
uint64_t svo_palette(svo_scene* scene, int32_t which, uint32_t* out, uint64_t max);

/* ---- device image (replaces OctreeGPUHost / create_new_view / write_to_gpu,
 *      src/raytracing/bevy/data.rs:111-166, 365-773) ----------------------- */
/* Uploads the whole scene as device-resident pools (node records, bricks, voxel
 * occupancy bits, palettes).  Allocates device memory. */
svo_status svo_scene_upload(svo_scene* scene, void* stream);
/* Writes the node records, bricks and palette entries changed since the last
 * upload/sync in place (falls back to a full upload when a pool outgrew its
 * device allocation). */
svo_status svo_scene_sync(svo_scene* scene, void* stream);
svo_status svo_scene_release_device(svo_scene* scene);
/* Device memory of scene images from the caller's allocator (process-wide) instead of cudaMalloc /
 * cudaFree: for callers that pool device memory or cap it themselves.  `alloc` gets the byte count
 * and the stream of the upload and returns device memory (at least 256-byte aligned) or NULL, which
 * makes the upload return SVO_ERR_OUT_OF_MEMORY after releasing what it had taken (the scene is then
 * left without a device image); `release` frees what `alloc` returned.  Both NULL restores
 * cudaMalloc / cudaFree.  Change it only while no scene holds a device image from the other one.
 * No counterpart in the reference (the Bevy plugin's buffers belong to wgpu). */
typedef void* (*svo_alloc_fn)(size_t bytes, void* stream, void* user);
typedef void (*svo_free_fn)(void* ptr, void* user);
svo_status svo_set_device_allocator(svo_alloc_fn alloc, svo_free_fn release, void* user);

/* ---- the hot path: Octree::get_by_ray (src/raytracing/raytracing_on_cpu.rs:316-565) ---- */
/* n rays in device memory -> per-ray hits in device memory.  Allocates nothing.
 * Batches of 32768 rays and more run as a work queue: warps claim 32 rays at a time from a
 * counter that the scene keeps per stream (up to 64 streams; casts on further streams, and on
 * cudaStreamPerThread, use one thread per ray).  Casts of one scene on different streams may
 * overlap.  A CUDA graph that captured a cast reuses the counter of the stream it was captured
 * on: do not run it concurrently with casts on that stream. */
svo_status svo_cast(svo_scene* scene, const svo_rays* rays, uint64_t n, const svo_hits* hits, void* stream);
/* Octree::get_by_ray_at_lod (raytracing_on_cpu.rs:325-565): with MIP maps enabled (svo_mip_switch) a
 * node's MIP brick is read once its level is below (origin - p rounded to the level's grid).length()
 * / viewing_distance; a hit on a MIP brick reports brick_octant 8.  Without MIP maps this is
 * svo_cast.  Device buffers, the same work queue as svo_cast. */
svo_status svo_cast_lod(svo_scene* scene, const svo_rays* rays, uint64_t n, const svo_hits* hits, float viewing_distance,
                        void* stream);
/* Same cast with host ray and hit buffers, stream synchronised before return.  The batch is staged
 * in chunks through a per-scene device workspace that grows on demand, copies overlapping the casts
 * (with pinned host memory); camera images given with their row length (svo_cast_host_rows) are
 * read and written in place where the device reads host memory through the CPU's page tables
 * (Grace), see svo_set_host_transfer: a large image (four claims or more per resident warp) is cast
 * two 16 x 2 ray blocks per warp, each hit field written row by row in 32-ray pieces. */
svo_status svo_cast_host(svo_scene* scene, const svo_rays* rays, uint64_t n, const svo_hits* hits, void* stream);
/* The three casts above for rays laid out as rows of row_length rays (a camera image in raster
 * order, or several images one after the other): the work queue hands each warp 8 neighbouring rays
 * of 4 neighbouring rows instead of 32 rays of one row, so its rays stay in step longer (16 rays of
 * 2 rows where svo_cast_host_rows reads the host's arrays in place).  Hits are
 * identical to the plain calls' (rays are independent); row_length 0, or a batch of fewer than 4
 * rows, casts in plain order.  No counterpart in the reference, whose renderer casts one pixel at a
 * time (examples/cpu_render.rs:104-138). */
svo_status svo_cast_rows(svo_scene* scene, const svo_rays* rays, uint64_t n, uint32_t row_length, const svo_hits* hits,
                         void* stream);
svo_status svo_cast_lod_rows(svo_scene* scene, const svo_rays* rays, uint64_t n, uint32_t row_length,
                             const svo_hits* hits, float viewing_distance, void* stream);
svo_status svo_cast_host_rows(svo_scene* scene, const svo_rays* rays, uint64_t n, uint32_t row_length,
                              const svo_hits* hits, void* stream);

/* ---- fused viewport render: examples/cpu_render.rs:77-138 on the device ---- */
/* The example's frame: a viewport of width x height world units at distance fov in front of
 * origin along direction (unit length, as the example makes it), right = normalize(up x
 * direction); pixel (x, y) casts from origin towards bottom_left + right * x * (width / W) +
 * up * y * (height / H), bottom_left = origin + direction * fov - up * height / 2 -
 * right * width / 2.  A hit is shaded 1 - (normal . light / 2 + 0.5) times its albedo's r, g,
 * b (cast to u8), alpha 255; a miss gets background.  The example uses width = height = 4,
 * fov = 3, up = (0, 1, 0), light = normalize(0, -1, 1) and background (128, 128, 128). */
typedef struct {
  float origin[3];
  float direction[3];
  float up[3];
  float width, height, fov;
  float light[3];
  uint32_t background; /* 0xRRGGBBAA */
} svo_viewport;
/* Ray generation, cast and shading in one kernel: W x H pixels, 4 bytes (r, g, b, a) each,
 * row-major from the top row (the example's `viewport_size_height - y - 1`), into device memory
 * `rgba`.  Pixels where the example panics (a hit without albedo) or loops forever (work cap)
 * are written as (0, 0, 0, 0) and counted into the optional device counter *unshaded (added to,
 * not reset).  Allocates nothing; rays never touch memory. */
svo_status svo_render_viewport(svo_scene* scene, const svo_viewport* viewport, uint32_t width_px, uint32_t height_px,
                               uint8_t* rgba, unsigned long long* unshaded, void* stream);
/* n_views viewports of one scene, each W x H, frame k at rgba + k * W * H * 4: the same pixels as
 * n_views svo_render_viewport calls, in one launch per 16 views (a launch's last tiles no longer
 * leave the GPU idle once per frame).  Pixels whose ray misses the octree's root box are coloured
 * at once; the rays that enter are packed into full warps. */
svo_status svo_render_viewports(svo_scene* scene, const svo_viewport* viewports, uint32_t n_views, uint32_t width_px,
                                uint32_t height_px, uint8_t* rgba, unsigned long long* unshaded, void* stream);

/* ---- batched multi-scene cast (one persistent launch) ------------------ */
typedef struct {
  svo_scene* scene;
  svo_rays rays; /* device pointers */
  uint64_t n;
  svo_hits hits; /* device pointers */
  uint32_t row_length; /* rays laid out as rows of this many rays (a camera image): cast in 8 x 4 ray
                          blocks like svo_cast_rows; 0 = plain order */
  uint32_t reserved;   /* 0 */
} svo_batch_item;

typedef struct {
  uint32_t block;          /* threads per block (multiple of 32, <= 128); 0 = default 128 */
  uint32_t rays_per_chunk; /* rays a warp claims per work-queue grab; 0 = default 64 */
  uint32_t blocks_per_sm;  /* persistent CTAs per SM; 0 = default from occupancy */
  uint32_t block_shape;    /* rays of an item with a row length cast together: 0 or 3 = 8 x 4, 4 = 16 x 2,
                              5 = 32 x 1 (log2 of the width) */
  uint32_t sort_key;       /* order of the rays of the items without a row length: 0 = index order;
                              1 = sorted by (item, octant of the direction, Morton code of the point
                              where the ray enters the octree), so that a warp's rays walk much the
                              same nodes (svo_cast_batched only: needs the workspace's buffers, which
                              grow to 128 bytes per such ray) */
  uint32_t staging_depth;  /* top tree levels staged in shared memory by every block: the Internal nodes of
                              depth < staging_depth (0..4) of each scene of the call, as far as 48 KB of
                              records per block reach (scenes past that read their nodes from L1/L2) */
  uint32_t refill_below;   /* with sort_key 1: the sorted rays' cast parks a warp's rays at a node visit once
                              fewer than refill_below (1..32) are in flight, gives its idle lanes the next
                              sorted rays and resumes (see svo_set_refill); 0 = each warp's rays run to
                              their ends.  The hits are the same for every value. */
} svo_launch_config;

/* Casts every item's rays in one persistent kernel launch driven by a device
 * work counter.  The per-launch item table and counter live in a workspace
 * owned by `ws` (create it once; it grows only when the item count grows).
 * With sort_key 1 the items without a row length are cast through the ray sort
 * instead: a binning launch (misses written at once), a scan of the bucket
 * counts, a scatter into bucket order and a persistent cast of the sorted
 * entering rays, all on `stream`; the hits are the same as in index order.  The
 * sort's buffers grow only when the rays (or buckets) of a call outgrow them:
 * make the largest call once before a stream capture.  A graph that captured a
 * call reads the workspace's host-side item table and device buffers at every
 * replay: while that graph may still be replayed, make other casts through
 * another workspace (a call on this one rewrites the table the graph reads,
 * and one that outgrows the buffers frees those the graph uses). */
typedef struct svo_batch_workspace svo_batch_workspace;
svo_status svo_batch_workspace_create(svo_batch_workspace** out);
void svo_batch_workspace_destroy(svo_batch_workspace* ws);
svo_status svo_cast_batched(svo_batch_workspace* ws, const svo_batch_item* items, uint32_t n_items,
                            const svo_launch_config* cfg, void* stream);

/* Allocation-free variant of svo_cast_batched for callers that cannot allocate
 * device memory when they cast (a fixed memory budget handed over at start-up,
 * or a frame loop where a cudaMalloc would synchronise the device).  No
 * counterpart in the reference.  The item table and work counter live in one
 * scratch array compiled into the library (47,360 bytes, reserved on every GPU
 * that loads the library until the process exits), so at most 128 items are
 * accepted per call; more return SVO_ERR_ARGUMENT.  The first call on a device
 * looks up the array's device address on the current device, which must be the
 * device that owns `stream`; the address is kept for the life of the process,
 * so a cudaDeviceReset makes it stale.  The item table is copied from the
 * call's own stack frame, so a call on a stream that is being captured returns
 * SVO_ERR_ARGUMENT with nothing enqueued.  Calls that overlap on the GPU share
 * the array and race: issue them on one stream, or wait for one before
 * starting the next.  Allocates nothing and calls no allocating CUDA or
 * library routine. */
svo_status svo_cast_batched_noalloc(const svo_batch_item* items, uint32_t n_items, const svo_launch_config* cfg,
                                    void* stream);

/* ---- serving: continuous batching of camera requests over resident scenes ---- */
typedef struct svo_server svo_server;

typedef struct {
  uint64_t budget_bytes;        /* device memory for resident scene images; LRU scenes are evicted above it */
  uint32_t max_batch_requests;  /* requests admitted into one launch (1..128) */
  uint32_t max_batch_rays;      /* rays admitted into one launch (a single larger request still runs alone) */
  uint32_t max_inflight;        /* launches in flight at once (1..4), each on its own stream */
  svo_launch_config launch;     /* persistent-kernel launch configuration (0 = defaults) */
} svo_server_config;

/* A pinhole camera request: width*height rays generated on the device exactly as
 * svo_gen_camera_rays generates them, cast against the scene, results copied to
 * the caller's HOST buffers (any field may be NULL).  The buffers must stay valid
 * until the request completes. */
typedef struct {
  uint32_t scene_id;
  float eye[3], target[3], fov_deg;
  uint32_t width, height;
  svo_hits hits;
} svo_request;

typedef struct {
  int32_t status;          /* SVO_OK, or the error that failed the request */
  double submit_s, start_s, done_s; /* server clock: submitted, launched, results in host memory */
  uint32_t batch_requests; /* requests that shared its launch */
} svo_request_result;

typedef struct {
  uint64_t requests_done, rays_done, launches, uploads, evictions;
  uint64_t resident_bytes;
} svo_server_stats;

/* Starts the server and its worker thread on the current device. */
svo_status svo_server_create(const svo_server_config* cfg, svo_server** out);
/* Stops the worker after the requests submitted so far complete (or fail: a launch that fails on
 * the device fails its requests) and releases the server's device memory. */
void svo_server_destroy(svo_server* server);
/* Registers a scene (not owned; the caller keeps it alive and leaves it untouched while registered).
 * The server uploads and evicts its device image under the budget; a launch waits for the uploads of
 * its scenes made on other launches' streams.  A device image the caller uploaded must be complete
 * (its stream synchronised) before the scene is registered. */
svo_status svo_server_add_scene(svo_server* server, svo_scene* scene, uint32_t* scene_id);
/* Queues a request; returns at once with its id. */
svo_status svo_server_submit(svo_server* server, const svo_request* request, uint64_t* request_id);
/* Waits up to timeout_s seconds for a request; SVO_ERR_BUSY on timeout. */
svo_status svo_server_wait(svo_server* server, uint64_t request_id, double timeout_s, svo_request_result* out);
svo_status svo_server_stats_get(svo_server* server, svo_server_stats* out);
/* Seconds on the server clock (the clock of svo_request_result). */
double svo_server_now(svo_server* server);

/* ---- synthetic workloads (seeded, deterministic on x86_64 and aarch64) ---- */
typedef struct {
  uint32_t kind;      /* 0 heightfield+spheres, 1 terrain+caves, 2 sparse+uniform blocks, 3 noise+spheres,
                         4 boxes of insert_at_lod cubes */
  uint32_t size, brick_dim;
  uint64_t seed;
  float occupancy;    /* target fraction for kinds 2 and 3 */
  uint32_t spheres;   /* sphere count (kinds 0 and 3) */
  uint32_t octaves;
  float base_freq;
  float height_lo, height_hi;
  float cave_threshold; /* kind 1 */
} svo_scene_recipe;
/* Writes the scene's construction ops into `ops` (capacity max_ops); *n_ops gets
 * the count (also when max_ops is too small, so callers can size the buffer). */
svo_status svo_gen_scene(const svo_scene_recipe* recipe, svo_op* ops, uint64_t max_ops, uint64_t* n_ops);
/* Pinhole camera rays (host memory), direction = normalize(fwd + u*right + v*up). */
svo_status svo_gen_camera_rays(const float eye[3], const float target[3], float fov_deg, uint32_t width,
                               uint32_t height, float* ox, float* oy, float* oz, float* dx, float* dy, float* dz);
/* Rays with origins uniform on a sphere (center, radius) and uniform directions. */
svo_status svo_gen_sphere_rays(const float center[3], float radius, uint64_t n, uint64_t seed, float* ox, float* oy,
                               float* oz, float* dx, float* dy, float* dz);

/* ---- diagnostics ------------------------------------------------------ */
/* Evaluates the kernels' look-up-table arithmetic on the GPU and copies back
 * RAY_TO_NODE_OCCUPANCY_BITMASK_LUT[64][8], OCTANT_STEP_RESULT_LUT[3][3][3] and
 * BITMAP_MASK_FOR_OCTANT_LUT[8] (src/spatial/lut.rs) for comparison with the
 * reference constants.  Allocates a few bytes of device memory. */
svo_status svo_selftest_luts(uint64_t* ray_to_node, uint32_t* octant_step, uint64_t* octant_masks);
/* Selects the form of the cast kernels for casts launched afterwards (process-wide):
 * 0 (default) the fast form for rays without NaN in the direction and the literal
 * restatement otherwise; 1 the literal restatement for every ray.  Both give the
 * same results; mode 1 exists so tests can check that. */
svo_status svo_set_cast_mode(int32_t mode);
/* How svo_cast_host moves rays and hits (process-wide): 0 (default) lets the kernel read and write
 * the host buffers in place for batches with a row layout (svo_cast_host_rows, row_length >= 16)
 * when the device accesses host memory through the CPU's page tables (Grace systems), and stages
 * copies otherwise; 1 always stages copies (chunks over three streams); 2 always accesses host
 * memory directly (an error where the device cannot); 3 as 2, with each warp writing its own 16 x 2
 * ray block (pieces of 64 and 16 bytes a row) instead of two blocks' rows of 32 rays (pieces of 128
 * and 32 bytes), for comparison. */
svo_status svo_set_host_transfer(int32_t mode);
/* Staging depth of the plain casts launched afterwards (svo_cast, svo_cast_rows and the host-buffer
 * casts; process-wide): each block first copies the scene's Internal nodes of depth < depth (the
 * root has depth 0; at most 1, 9, 73 or 585 records of 64 bytes for depth 1..4) into shared memory,
 * and the traversal reads those nodes there instead of through L1/L2.  0 (default) stages nothing.
 * The results are the same at every depth; the batched cast takes its depth from
 * svo_launch_config.staging_depth.  No counterpart in the reference. */
svo_status svo_set_staging_depth(int32_t depth);
/* Lane refill of the plain casts launched afterwards (process-wide): 0 (default) casts each warp's
 * 32 rays to their ends; 1..32: a warp whose rays in flight drop below park_below stops them at their
 * next node visit, gives its idle lanes new rays and continues all of them together, so that rays of
 * very different lengths (rays in no particular order) keep the lanes busy.  The results are the same
 * for every value.  No counterpart in the reference. */
svo_status svo_set_refill(int32_t park_below);

#ifdef __cplusplus
}
#endif
#endif /* SVO_H */
