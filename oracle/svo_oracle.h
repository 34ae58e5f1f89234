/*
 * svo_oracle.h -- C interface of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain CPU restatement of the
 * reference crate shocovox-rs v0.11.1 (octree construction, update and the
 * CPU ray cast `Octree::get_by_ray`).  It exists to check the GB300 product
 * library (libsvo) and to time the CPU baseline.  Only the test suite,
 * `__graft_entry__.smoke()` and the `cpu_baseline` / `--impl reference`
 * legs of bench.py load it.  Nothing in the product links against it.
 *
 * Parity anchor: the reference is Rust and cannot be compiled in this
 * environment (no cargo/rustc), so the restatement is pinned by the
 * reference's own known-answer tests (src/raytracing/tests.rs,
 * src/spatial/raytracing/tests.rs, src/spatial/math/tests.rs, src/octree/update/tests.rs)
 * and by the look-up
 * tables extracted from src/spatial/lut.rs (tests/golden/).
 */
#ifndef SVO_ORACLE_H
#define SVO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes; 1..4 mirror OctreeError (src/octree/types.rs:8-21). */
enum {
  ORC_OK = 0,
  ORC_ERR_INVALID_SIZE = 1,
  ORC_ERR_INVALID_BRICK_DIM = 2,
  ORC_ERR_INVALID_STRUCTURE = 3,
  ORC_ERR_INVALID_POSITION = 4,
  ORC_ERR_REFERENCE_PANIC = 5, /* the reference would panic / overflow its stack here */
  ORC_ERR_ARGUMENT = 6
};

/* One scene-construction operation; identical layout to svo_op in include/svo.h. */
typedef struct {
  uint16_t x, y, z;
  uint8_t op;   /* 0 insert, 1 update, 2 insert_at_lod, 3 clear, 4 clear_at_lod */
  uint8_t kind; /* bit0: albedo present, bit1: user data present */
  uint32_t size;
  uint32_t rgba; /* Albedo packed as Albedo::from(u32): 0xRRGGBBAA */
  uint32_t user;
} orc_op;

/* Per-ray outputs of orc_cast (struct of arrays; any pointer may be NULL). */
typedef struct {
  uint8_t* status;       /* 0 miss, 1 hit, 2 work cap exceeded, 3 reference would panic */
  uint8_t* brick_octant; /* octant of the hit brick inside a Leaf, 0 for UniformLeaf */
  uint8_t* entry_kind;   /* 0 Empty, 1 Visual, 2 Informative, 3 Complex */
  uint32_t* node_key;
  uint32_t* voxel_index; /* flat index inside the brick, 0xFFFFFFFF for a Solid brick */
  uint32_t* pix;         /* PaletteIndexValues of the hit voxel */
  uint32_t* albedo;      /* 0xRRGGBBAA, 0 when the entry has no albedo */
  uint32_t* user;        /* user data, 0 when the entry has none */
  float *px, *py, *pz;   /* impact point */
  float *nx, *ny, *nz;   /* impact normal */
  uint32_t* node_visits; /* instrumentation: inner traversal-loop iterations */
  uint32_t* child_reads; /* instrumentation: child-key reads */
  uint32_t* voxel_reads; /* instrumentation: brick voxel reads */
} orc_hits;

int orc_new(uint32_t size, uint32_t brick_dim, void** out);
void orc_free(void* tree);
void orc_set_auto_simplify(void* tree, int enabled);
int orc_insert(void* tree, uint32_t x, uint32_t y, uint32_t z, uint32_t kind, uint32_t rgba, uint32_t user);
int orc_update(void* tree, uint32_t x, uint32_t y, uint32_t z, uint32_t kind, uint32_t rgba, uint32_t user);
int orc_insert_at_lod(void* tree, uint32_t x, uint32_t y, uint32_t z, uint32_t size, uint32_t kind,
                      uint32_t rgba, uint32_t user);
int orc_clear(void* tree, uint32_t x, uint32_t y, uint32_t z);
int orc_clear_at_lod(void* tree, uint32_t x, uint32_t y, uint32_t z, uint32_t size);
int orc_apply_ops(void* tree, const orc_op* ops, uint64_t n, uint64_t* n_done);
int orc_get(void* tree, uint32_t x, uint32_t y, uint32_t z, uint32_t out_kind_rgba_user[3]);

/* Casts n rays (SoA f32 origin / direction) with `threads` host threads. */
int orc_cast(void* tree, uint64_t n, const float* ox, const float* oy, const float* oz, const float* dx,
             const float* dy, const float* dz, const orc_hits* out, int threads);

/* Structure inspection (canonical per-node records, palettes). */
/* One frame of examples/cpu_render.rs: a viewport of width x height world units at distance fov
   in front of origin along direction, pixels spread from its bottom-left corner along right =
   normalize(up x direction) and up, one ray per pixel from origin, diffuse shading against light. */
typedef struct {
  float origin[3], direction[3], up[3];
  float width, height, fov;
  float light[3];
  uint32_t background; /* 0xRRGGBBAA of a pixel whose ray hits nothing */
} orc_viewport;
/* rgba: 4 bytes (r, g, b, a) per pixel, row-major from the top row.  A hit whose entry has no
   albedo (where the example's unwrap() panics) or a ray that reaches the work cap is stored as
   (0, 0, 0, 0) and counted in *unshaded (may be NULL). */
int orc_render_viewport(void* tree, const orc_viewport* vp, uint32_t width_px, uint32_t height_px, uint8_t* rgba,
                        uint64_t* unshaded, int threads);

/* get_by_ray_at_lod (raytracing_on_cpu.rs:325-565): the cast with a viewing distance; orc_cast is
   this with f32::MAX.  A hit on a node's MIP brick reports brick_octant 8. */
int orc_cast_lod(void* tree, uint64_t n, const float* ox, const float* oy, const float* oz, const float* dx,
                 const float* dy, const float* dz, float viewing_distance, const orc_hits* out, int threads);
/* MIP maps (octree/mipmap.rs).  method: 0 BoxFilter, 1 PointFilter, 2 PointFilterBD, 3 Posterize(thr),
   4 PosterizeBD(thr). */
int orc_mip_switch(void* tree, int enabled);
int orc_mip_set_method(void* tree, uint32_t level, uint32_t method, float thr);
int orc_mip_set_color_threshold(void* tree, uint32_t level, float thr);
int orc_mip_recalculate(void* tree);
int orc_mip_sample_root(void* tree, uint32_t octant, uint32_t x, uint32_t y, uint32_t z, uint32_t out_kind_rgba_user[3]);
int orc_node_mip(void* tree, uint64_t key, uint32_t* kind, uint32_t* values);

uint64_t orc_node_count(void* tree);
int orc_node_record(void* tree, uint64_t key, uint64_t rec[40]);
uint64_t orc_palette(void* tree, int which, uint32_t* out, uint64_t max);

/* Look-up tables generated with the reference's generator functions. */
void orc_luts(uint64_t ray_to_node[512], uint32_t octant_step[27], uint64_t octant_mask[8],
              uint8_t bitmap_index[64], float octant_offset[24]);

/* Spatial helpers exposed for the ported spatial tests. */
int orc_intersect_ray(const float cube[4], const float ray[6], float* distance); /* 0 none, 1 inside, 2 dist */
void orc_cube_impact_normal(const float cube[4], const float point[3], float out[3]);
uint32_t orc_hash_region(const float offset[3], float size_half);
uint64_t orc_position_in_bitmap(uint64_t x, uint64_t y, uint64_t z, uint64_t brick_size);
uint64_t orc_set_occupancy(uint64_t x, uint64_t y, uint64_t z, uint64_t size, uint64_t brick_dim, int occupied,
                           uint64_t bitmap);
int orc_plane_line_intersection(const float plane_point[3], const float plane_normal[3], const float line_origin[3],
                                const float line_direction[3], float* out);
void orc_child_bounds(const float cube[4], uint32_t octant, float out[4]);
void orc_dda_step(const float ray[6], float point[3], const float cube[4], float step_out[3]);
uint64_t orc_flat_projection(uint64_t x, uint64_t y, uint64_t z, uint64_t size);
int orc_brick_empty_throughout(const uint32_t* pix, uint32_t dim, uint32_t kind, uint32_t octant, int32_t part,
                               const uint32_t* colors, uint32_t n_colors, const uint32_t* datas, uint32_t n_datas);

/* Seeded synthetic workloads of the benchmark (oracle/workloads.cpp): the same op lists and rays as
   the product's svo_gen_scene / svo_gen_camera_rays / svo_gen_sphere_rays, so that the CPU baseline
   needs no product code.  The recipe has the layout of svo_scene_recipe. */
typedef struct {
  uint32_t kind; /* 0 heightfield+spheres, 1 terrain+caves, 2 sparse+uniform blocks, 3 noise+spheres, 4 boxes */
  uint32_t size, brick_dim;
  uint64_t seed;
  float occupancy;
  uint32_t spheres;
  uint32_t octaves;
  float base_freq;
  float height_lo, height_hi;
  float cave_threshold;
} orc_recipe;
int orc_gen_scene(const orc_recipe* recipe, orc_op* ops, uint64_t max_ops, uint64_t* n_ops);
int orc_gen_camera_rays(const float eye[3], const float target[3], float fov_deg, uint32_t width, uint32_t height,
                        float* ox, float* oy, float* oz, float* dx, float* dy, float* dz);
/* The camera rays of pixels first, first + stride, ... (n of them) of the width x height image. */
int orc_gen_camera_rays_strided(const float eye[3], const float target[3], float fov_deg, uint32_t width,
                                uint32_t height, uint64_t first, uint64_t stride, uint64_t n, float* ox, float* oy,
                                float* oz, float* dx, float* dy, float* dz);
int orc_gen_sphere_rays(const float center[3], float radius, uint64_t n, uint64_t seed, float* ox, float* oy, float* oz,
                        float* dx, float* dy, float* dz);

/* NodeStack<i32, size> harness for the ported ring-stack tests (size 1..8). */
void* orc_stack_new(uint32_t size);
void orc_stack_free(void* s);
void orc_stack_push(void* s, int32_t v);
int orc_stack_pop(void* s, int32_t* out);      /* 1 = Some, 0 = None */
int orc_stack_last(void* s, int32_t* out);     /* 1 = Some, 0 = None */
int orc_stack_add_last(void* s, int32_t delta); /* last_mut += delta; 1 = Some */
int orc_stack_is_empty(void* s);

#ifdef __cplusplus
}
#endif
#endif
