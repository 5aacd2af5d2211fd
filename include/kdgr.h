/* kdgr.h -- C ABI of libkdgr, a GB300-native (sm_103a) implementation of the
 * hybrid kd-tree Gaussian ray tracer of hydarlisk/3dgrt_kdtree.
 *
 * Paths below are relative to the reference's Kd-treeConverter_v0.9/
 * Kd-treeConverter/ directory.  Every entry point names the reference
 * interface it replaces.
 *
 * Conventions (all entry points):
 *   - return a kdgr_status; KDGR_OK is 0, errors are positive and never exit
 *     the process (the reference's CUDA_CHECK calls exit(), cudaRenderer.cu:25-31);
 *     kdgr_last_error() gives the message of the calling thread's last error;
 *   - plain pointers and sizes; device buffers are raw CUDA device pointers,
 *     streams are cudaStream_t passed as void*; the caller owns every buffer;
 *     render outputs may also be page-locked host memory (cudaHostAlloc /
 *     cudaMallocHost), which the kernels then write directly -- on GB300 over
 *     NVLink-C2C while the frame renders, with no separate copy;
 *   - a scene handle may be used from several threads; calls on one handle
 *     that write the same output buffers must be ordered by the caller;
 *   - every call on a scene runs on the device the scene was created on
 *     (the call makes it current and restores the caller's device after), so
 *     output buffers and streams must belong to that device.
 */
#ifndef KDGR_H_
#define KDGR_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  KDGR_OK = 0,
  KDGR_ERR_INVALID_ARG = 1,
  KDGR_ERR_CUDA = 2,
  KDGR_ERR_OUT_OF_MEMORY = 3,
  KDGR_ERR_IO = 4,
  KDGR_ERR_FORMAT = 5,    /* malformed tree or file */
  KDGR_ERR_BUDGET = 6,    /* serving admission refused by the HBM budget */
  KDGR_ERR_TIMEOUT = 7,   /* a bounded wait expired */
  KDGR_ERR_NOT_INITIALIZED = 8,
  KDGR_ERR_CANCELLED = 9,
  KDGR_ERR_LIMIT = 10     /* a size beyond a fixed maximum */
} kdgr_status;

/* ---------------------------------------------------------------- camera */

/* The fields of the reference's Camera (OpenGLStuffs.h:21-28) that the
 * renderer reads: position, right (u), up (v) and back (n) axes, and the
 * double-precision vertical field of view in degrees, aspect ratio and near
 * plane.  The camera looks along -naxis. */
typedef struct {
  float pos[3];
  float uaxis[3];
  float vaxis[3];
  float naxis[3];
  double fovy;
  double aspect;
  double near_c;
} kdgr_camera;

/* ------------------------------------------------------------------ tree */

/* Build parameters of the reference kd-tree builder (CLI -m/-f/-i/-s/-sc,
 * Kd-treeConverterMain.cpp:3679-3733; defaults of the render benchmark). */
typedef struct {
  int32_t max_level;    /* MAX_LEVEL (24) */
  int32_t force_split;  /* FORCE_SPLIT_THRESHOLD in triangles (16); 0 = off */
  float isect_cost;     /* ISCET_COST (5.0) */
  int32_t sah_mode;     /* SAH_MODE: 0, 1 (default), 4 or 7 */
  float sort_cost;      /* SORT_COST (0.5), used by SAH_MODE 7 */
  int32_t threads;      /* host threads; 0 = all */
} kdgr_build_params;

/* A kd-tree in the reference's flat layout (KdTreeNode, Kd-treeConverter.h:
 * 282-296,402-410): nodes[2*i] = x, nodes[2*i+1] = y.  Inner: x = child<<3 |
 * axis, y = split bits; children at child and child+1.  Leaf: x = count<<3 |
 * 3, y = offset into offsets[].  aabb is in .kdt order (xmin, ymin, zmin,
 * xmax, ymax, zmax).  Arrays are malloc'd by the library: kdgr_tree_free. */
typedef struct {
  uint32_t* nodes;
  uint32_t n_nodes;
  uint32_t* offsets;
  uint32_t n_offsets;
  float aabb[6];
  uint32_t depth;
  uint32_t n_leaves;
  uint32_t max_leaf;
  uint8_t* valid;        /* per Gaussian: 1 if it has proxy triangles (built trees) */
  uint32_t n_gaussians;  /* 0 for trees read from a file */
} kdgr_tree;

typedef struct {
  double proxy_s;
  double build_s;      /* split search and partition, including serialize_s */
  uint64_t n_triangles;
  uint32_t n_valid;
  double serialize_s;  /* numbering the nodes in the reference's order and copying the leaf lists out */
} kdgr_build_stats;

void kdgr_build_params_default(kdgr_build_params* params);

/* Proxy-mesh + SAH kd-tree build over activated Gaussians (64-float records,
 * the reference's Gaussian layout, scales NOT inverted).  Same tree, bit for
 * bit, as build_kd_tree_for_composite_object (Kd-treeConverter.cpp:22) after
 * create_composite_object_from_gaussians (Kd-treeConverterMain.cpp:1925). */
int kdgr_build_tree(const float* gaussians, uint32_t n_gaussians, const kdgr_build_params* params,
                    kdgr_tree* out, kdgr_build_stats* stats);

/* The same build on the current CUDA device (breadth first, one level per
 * step, sorts and scans on the device); the tree is the one kdgr_build_tree
 * returns, bit for bit.  Uses params->threads for nothing. */
int kdgr_build_tree_gpu(const float* gaussians, uint32_t n_gaussians, const kdgr_build_params* params,
                        kdgr_tree* out, kdgr_build_stats* stats);

/* read_kd_tree_from_file(obj, path, KD_TREE_DUMP_IN_BINARY)
 * (Kd-treeConverter.cpp:444-495), with structural validation. */
int kdgr_read_kdt(const char* path, kdgr_tree* out);

/* dump_kd_tree_for_composite_object(obj, KD_TREE_DUMP_IN_BINARY, path, ...)
 * (Kd-treeConverter.cpp:297-342). */
int kdgr_write_kdt(const kdgr_tree* tree, const char* path);

/* The ASCII forms of the same two calls (KD_TREE_DUMP_IN_ASCII,
 * Kd-treeConverter.cpp:345-380, 496-541).  The format has no scene box (aabb
 * reads back as zeros: pass the box to kdgr_scene_create yourself) and prints
 * splits with six decimals, so a round trip moves split planes, as in the
 * reference. */
int kdgr_read_kdt_ascii(const char* path, kdgr_tree* out);
int kdgr_write_kdt_ascii(const kdgr_tree* tree, const char* path);

/* Gaussians in the reference's 64-float record (Kd-treeConverter.h:319-335),
 * activated; malloc'd by the library: kdgr_gaussians_free. */
typedef struct {
  float* records;
  uint32_t n;
} kdgr_gaussians;

/* loadGaussiansFromPly (Kd-treeConverterMain.cpp:1652-1769): a binary
 * little-endian 3DGS .ply, fields found by property name, activated (sigmoid
 * opacity, exp scale, normalised quaternion, k_scale).  Scales come back
 * activated, not inverted. */
int kdgr_read_ply(const char* path, kdgr_gaussians* out);
void kdgr_gaussians_free(kdgr_gaussians* g);

/* Child/leaf ranges in bounds, IDs < n_gaussians, no node reached twice. */
int kdgr_validate_tree(const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets, uint32_t n_offsets,
                       uint32_t n_gaussians);

void kdgr_tree_free(kdgr_tree* tree);

const char* kdgr_last_error(void);

/* ------------------------------------------------------------ scenes */

typedef struct kdgr_scene_s* kdgr_scene_t;

/* kdgr_scene_create flags */
#define KDGR_SCALES_INVERTED 0x1u /* scale[] holds 1/s already, as the reference's
                                     caller leaves it (Kd-treeConverterMain.cpp:3636-3650) */
#define KDGR_FORM_EXACT 0x10u     /* oracle-matching arrays (kdgr_render) */
#define KDGR_FORM_FAST 0x20u      /* FP32 fast arrays (kdgr_render_fast, batches) */
#define KDGR_FORM_PACKED 0x40u    /* BF16 SH + FP16 shape arrays (precision form) */
/* flags without any KDGR_FORM_* bit materialise EXACT | FAST */

typedef struct {
  uint32_t n_nodes, n_offsets, n_gaussians;
  uint32_t depth, n_leaves, max_leaf;
  uint32_t forms;         /* KDGR_FORM_* present */
  uint32_t top_nodes;     /* fast form: nodes of the breadth-first top (10 levels) of the relaid tree */
  uint32_t n_aniso;       /* packed form: Gaussians with FP64-precomputed factors */
  uint64_t device_bytes;  /* HBM held by the scene */
} kdgr_scene_info;

/* Select the device the calling thread uses (initCuda, cudaRenderer.cu:2445). */
int kdgr_init(int device);
/* Synchronise the device; scenes must be destroyed by the caller. */
int kdgr_shutdown(void);

/* renderGaussianWithCudaSetup (cudaRenderer.cu:2557-2703): upload a tree in
 * the reference layout and activated Gaussians (64-float records, the
 * reference's Gaussian struct).  Validates the tree first (KDGR_ERR_FORMAT). */
int kdgr_scene_create(const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets, uint32_t n_offsets,
                      const float aabb[6], const float* gaussians, uint32_t n_gaussians, uint32_t flags,
                      kdgr_scene_t* out);
/* kdgr_scene_create with the Gaussian records already in device memory
 * (d_gaussians: n_gaussians 64-float records on the current device, e.g.
 * from kdgr_read_ply_device); the tree arrays are host arrays, validated
 * first.  kdgr_scene_create itself copies the host records to the device and
 * continues here: every form's per-Gaussian arrays are packed by device
 * kernels (renderGaussianWithCudaSetup, cudaRenderer.cu:2557-2703). */
int kdgr_scene_create_device(const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets, uint32_t n_offsets,
                             const float aabb[6], const float* d_gaussians, uint32_t n_gaussians, uint32_t flags,
                             kdgr_scene_t* out);

/* loadGaussiansFromPly (Kd-treeConverterMain.cpp:1652-1769) on the device:
 * the header is parsed on the host, the vertex block streams to the device
 * in chunks through pinned buffers and is activated there (sigmoid opacity,
 * exp scale, normalised quaternion, k_scale) into 64-float records at
 * d_records, the same records as kdgr_read_ply.  With d_records null only
 * *n_out is set (the vertex count, for sizing the buffer); a file with more
 * than `capacity` vertices is KDGR_ERR_LIMIT.  Synchronises `stream`. */
int kdgr_read_ply_device(const char* path, float* d_records, uint32_t capacity, uint32_t* n_out, void* stream);

/* A scene straight from the reference's two files: the .ply activated on the
 * device (kdgr_read_ply_device) and the binary .kdt (read_kd_tree_from_file,
 * Kd-treeConverter.cpp:444-495) validated and uploaded into the device tree
 * arrays; the per-Gaussian arrays are packed on the device.  flags as
 * kdgr_scene_create without KDGR_SCALES_INVERTED (PLY records are
 * activated). */
int kdgr_scene_create_from_files(const char* ply_path, const char* kdt_path, uint32_t flags, kdgr_scene_t* out);

/* cleanupCudaResources (cudaRenderer.cu) for one scene. */
int kdgr_scene_destroy(kdgr_scene_t scene);
int kdgr_scene_info_get(kdgr_scene_t scene, kdgr_scene_info* out);
/* Error bits the kernels raised for this scene since the last clear
 * (bounds violations; a bounded wait that expired).  Synchronises. */
int kdgr_scene_status(kdgr_scene_t scene, uint32_t* bits, int clear);

/* ------------------------------------------------------------ rendering */

/* renderGaussianWithCudaFrame (cudaRenderer.cu:3099-3484), plain drop-in
 * form: oracle-matching arithmetic, one launch per view.  Writes
 * d_rgb[3*((H-1-y)*W + x) + c] (rows flipped, as the reference) and, when
 * non-null, alpha and depth at the same pixel index.  With ms_out non-null
 * the call waits for the kernel and returns its time (the reference returns
 * FPS after an event sync); otherwise it is asynchronous on `stream`. */
int kdgr_render(kdgr_scene_t scene, const kdgr_camera* cam, int width, int height, float* d_rgb, float* d_alpha,
                float* d_depth, void* stream, float* ms_out);

/* ------------------------------------------------------- batched rendering
 * The batching, precision and serving forms.  One persistent launch draws
 * 32-ray pixel tiles of every queued view from an atomic work queue.  These
 * forms use fast FP32 arithmetic (FMA, rsqrt, exp2 approximation) and accept
 * hits with t* in the half-open leaf interval [t_near, t_far); they agree
 * with the FP64 oracle to <= 1e-3 RMSE.  No reference counterpart: the
 * reference renders one view per launch (cudaRenderer.cu:3406). */
typedef struct {
  kdgr_camera cam;
  int32_t width;
  int32_t height;
  uint64_t out_offset; /* first pixel of this view in the output buffers */
} kdgr_view;

/* How the persistent kernel hands out pixels. */
#define KDGR_SCHED_WARP_TILES 0  /* each warp takes 8x4-pixel tiles */
#define KDGR_SCHED_CTA_BLOCKS 1  /* each CTA takes 16x8 blocks; its 4 warps render the quarters */
#define KDGR_SCHED_SM_STRIPS 2   /* as CTA_BLOCKS, but the blocks are cut into one contiguous strip per
                                    SM; a CTA takes the next block of its SM's strip (neighbours share
                                    the SM's L1) and steals from the following strips when it is done */
#define KDGR_SCHED_WARP_STRIPS 3 /* as SM_STRIPS, but each warp claims the next quarter of a block on its
                                    own: no CTA barrier between work items */

/* Tree walk of the batch kernel.  Both give every ray its own leaves, in its
 * own front-to-back order, with its own leaf intervals. */
#define KDGR_TRAV_PACKET 0 /* the 32 rays of a warp's tile walk the tree together (a child is entered
                              when any ray needs it); leaf records become warp-uniform loads */
#define KDGR_TRAV_RAY 1    /* each lane walks its own ray independently */

/* Pixel tile of one warp (32 rays) inside a 16x8 block; the warp-tile
 * schedule renders 8x4 tiles only. */
#define KDGR_TILE_8X4 0
#define KDGR_TILE_4X8 1
#define KDGR_TILE_16X2 2

typedef struct {
  int32_t schedule;      /* KDGR_SCHED_* */
  int32_t min_blocks;    /* register cap: 0 (compiler), 6 or 8 resident 128-thread CTAs per SM */
  int32_t blocks_per_sm; /* persistent CTAs per SM; 0 = occupancy maximum */
  int32_t chunk;         /* work items taken per queue operation (1..64) */
  int32_t precision;     /* 0: FP32 arrays (KDGR_FORM_FAST); 1: BF16/FP16 arrays (KDGR_FORM_PACKED) */
  int32_t hit_buffer;    /* per-leaf register hit buffer: 4 or 8 entries (0 = 4); a leaf with more
                            accepted hits is re-scanned for the next ones */
  int32_t traversal;     /* KDGR_TRAV_*: how the rays of a warp walk the tree */
  int32_t tile_shape;    /* KDGR_TILE_*: the warp's pixel tile inside each 16x8 block */
  int32_t rays_per_warp; /* 32 (0 = 32), 16 or 8: with fewer rays per warp, 2 or 4 lanes share each ray and
                            split its leaves' candidate tests (more warps in flight and shorter rays for
                            small batches); needs KDGR_SCHED_WARP_STRIPS, warp packets and 8x4 tiles */
} kdgr_batch_config;

void kdgr_batch_config_default(kdgr_batch_config* cfg);

/* Render all views in one persistent launch.  Output pixel p of view v is at
 * views[v].out_offset + (H-1-y)*W + x (rows flipped per view); rgb holds 3
 * floats per pixel.  Scratch (view table, queue counter) is stream-ordered
 * device memory taken and returned on `stream`.  ms_out as kdgr_render. */
int kdgr_render_batch(kdgr_scene_t scene, const kdgr_view* views, int n_views, float* d_rgb, float* d_alpha,
                      float* d_depth, const kdgr_batch_config* cfg, void* stream, float* ms_out);

/* kdgr_render_batch for callers that cannot allocate device memory (a host
 * that owns the whole device-memory budget, or a frame loop that must never
 * enter the allocator).  No counterpart in the reference.  Same kernel and
 * results as kdgr_render_batch, but the scratch (view table + work-queue
 * counter) is a fixed 32 KiB file-scope device array, so at most 256 views
 * per call (KDGR_ERR_LIMIT beyond); it calls no device allocator.  The view
 * table reaches the array inside the parameters of a small staging kernel,
 * so nothing enqueued refers to host memory after the call returns.  The
 * first call on a device looks up the array's device address -- make it
 * before any stream capture.  Calls share the array: calls that overlap on
 * the GPU race; issue them on one stream.  Asynchronous on `stream`. */
int kdgr_render_batch_noalloc(kdgr_scene_t scene, const kdgr_view* views, int n_views, float* d_rgb,
                              float* d_alpha, float* d_depth, const kdgr_batch_config* cfg, void* stream);

/* One view through the batch kernel with the default configuration;
 * precision 0 = FP32 arrays, 1 = packed BF16/FP16 arrays. */
int kdgr_render_fast(kdgr_scene_t scene, const kdgr_camera* cam, int width, int height, float* d_rgb,
                     float* d_alpha, float* d_depth, int precision, void* stream, float* ms_out);

/* A fixed batch captured once as a CUDA graph (queue reset + persistent
 * launch) and replayed by kdgr_batch_run. */
typedef struct kdgr_batch_s* kdgr_batch_t;
int kdgr_batch_create(kdgr_scene_t scene, const kdgr_view* views, int n_views, float* d_rgb, float* d_alpha,
                      float* d_depth, const kdgr_batch_config* cfg, kdgr_batch_t* out);
int kdgr_batch_run(kdgr_batch_t batch, void* stream);
int kdgr_batch_destroy(kdgr_batch_t batch);

/* Time the kernel variants on the given views and return the fastest
 * configuration (pixel schedule, register cap, work items per queue
 * operation).
 * d_rgb must hold the views' pixels.  report (may be null) receives a JSON
 * line per variant. */
int kdgr_autotune(kdgr_scene_t scene, const kdgr_view* views, int n_views, int precision, float* d_rgb,
                  kdgr_batch_config* best, char* report, int report_len);

/* ------------------------------------------------------------ serving
 * Serving form: scenes resident in HBM under an admission budget; render
 * requests (a scene and 1..N views) are batched continuously -- everything
 * queued when a lane (stream) frees up goes into one persistent multi-scene
 * launch, so requests arriving while others are on the GPU overlap with them.
 * Each ray depends only on its own view: a request's frames are identical
 * alone and in any mix.  No reference counterpart. */
typedef struct kdgr_server_s* kdgr_server_t;

typedef struct {
  uint64_t hbm_budget_bytes;     /* resident scenes + output arena may not exceed this */
  uint64_t arena_bytes;          /* device output arena shared by in-flight requests */
  int32_t max_views_per_launch;  /* views per persistent launch (and per request) */
  int32_t lanes;                 /* launches in flight at once (streams), 1..8 */
  int32_t precision;             /* 0: FP32 fast arrays; 1: BF16/FP16 arrays */
} kdgr_server_config;

typedef struct {
  double latency_ms;  /* submit -> frames in the host buffer */
  double queue_ms;    /* submit -> launch */
  uint64_t rays;
} kdgr_request_stats;

typedef struct {
  uint64_t completed, cancelled, queued;
  double p50_ms, p99_ms, mean_ms, max_ms;
  double mrays_per_s; /* rays completed / (last completion - first submit) */
  uint64_t rays, launches, views_launched, max_views_per_launch;
  uint64_t resident_bytes;
} kdgr_server_stats;

void kdgr_server_config_default(kdgr_server_config* cfg);
int kdgr_server_create(const kdgr_server_config* cfg, kdgr_server_t* out);
/* Upload a scene into a free slot; KDGR_ERR_BUDGET when it does not fit. */
int kdgr_server_add_scene(kdgr_server_t server, const uint32_t* nodes, uint32_t n_nodes, const uint32_t* offsets,
                          uint32_t n_offsets, const float aabb[6], const float* gaussians, uint32_t n_gaussians,
                          uint32_t flags, int* slot);
/* Evict a scene: its queued requests finish with KDGR_ERR_CANCELLED; waits
 * (at most 60 s) for launches that use it. */
int kdgr_server_remove_scene(kdgr_server_t server, int slot);
/* Queue a request.  host_rgb receives 3 floats per pixel at each view's
 * out_offset (rows flipped per view).  Page-locked host_rgb (cudaMallocHost,
 * cudaHostRegister) is written by the render kernel itself and takes no
 * arena space; pageable host_rgb is rendered into the arena and copied out
 * when the launch completes.  Returns KDGR_ERR_BUDGET when a pageable
 * request's output can never fit the arena. */
int kdgr_server_submit(kdgr_server_t server, int slot, const kdgr_view* views, int n_views, float* host_rgb,
                       uint64_t* ticket);
/* Wait (at most timeout_ms) for a request; returns its status (KDGR_OK,
 * KDGR_ERR_CANCELLED) or KDGR_ERR_TIMEOUT.  A finished ticket is released. */
int kdgr_server_wait(kdgr_server_t server, uint64_t ticket, int timeout_ms, kdgr_request_stats* stats);
/* Cancel a request that has not been launched yet. */
int kdgr_server_cancel(kdgr_server_t server, uint64_t ticket);
int kdgr_server_stats_get(kdgr_server_t server, kdgr_server_stats* out);
int kdgr_server_reset_stats(kdgr_server_t server);
/* Stop the loop (queued requests are cancelled, launches drain) and free everything. */
int kdgr_server_destroy(kdgr_server_t server);

/* ------------------------------------------------------------ per-ray trace
 * Written by the oracle-matching render path in trace mode (and by the CPU
 * oracle) so the two can be compared ray by ray.  The counters are the
 * reference's HIT_AND_NODE_COUNT_DEBUG quantities (cudaRenderer.cu:1504-1510,
 * 1569-1606, 1679-1681); the hashes are 64-bit FNV-1a over the sequences. */
typedef struct {
  uint32_t n_inner;    /* inner-node descent steps */
  uint32_t n_leaf;     /* leaves visited */
  uint32_t n_cand;     /* candidates tested (sum of visited leaf sizes) */
  uint32_t n_hit;      /* accepted hits the compositing loop reached */
  uint32_t n_blend;    /* hits composited */
  uint32_t n_restart;  /* restarts from the root after the short stack ran dry */
  uint32_t n_found;    /* hits accepted in all visited leaves (hits_found, :1604) */
  uint32_t max_sort;   /* most hits accepted in one leaf (max_sort_size, :1605) */
  uint64_t h_leaf;     /* visited leaf node indices, in visit order */
  uint64_t h_hit;      /* Gaussian IDs of reached hits, in compositing order */
  uint64_t h_blend;    /* Gaussian IDs of composited hits, in order */
} kdgr_ray_trace;

/* kdgr_render plus one kdgr_ray_trace per pixel at d_trace[y*W + x] (kernel
 * row order, not flipped).  Asynchronous on `stream`. */
int kdgr_render_trace(kdgr_scene_t scene, const kdgr_camera* cam, int width, int height, float* d_rgb,
                      float* d_alpha, float* d_depth, kdgr_ray_trace* d_trace, void* stream);

/* ------------------------------------------------------------ secondary rays
 * The reference's SECONDARY_RAY renderer (renderKernelGaussian_Mesh_Hybrid,
 * cudaRenderer.cu:2217-2311): up to five bounces; per bounce the closest
 * secondary primitive clips the Gaussian pass (max_t), then a mirror
 * reflects, glass refracts (or totally reflects) and an opaque surface ends
 * the ray.  Oracle-matching arithmetic, like kdgr_render.  Output: RGB, rows
 * flipped, each channel clamped to <= 1. */
typedef struct {
  int32_t material;  /* 0 opaque, 1 mirror, 2 glass */
  float reflectivity;
  float ior;
  float color[3];
} kdgr_material;

typedef struct {
  float center[3];
  float radius;
  kdgr_material material;
} kdgr_sphere;

typedef struct kdgr_secondary_s* kdgr_secondary_t;

/* The reference's two demo spheres (cudaRenderer.cu:2158-2168). */
int kdgr_demo_spheres(kdgr_sphere out[2]);
/* SecondaryMesh defaults with the caller's mirror material
 * (cudaRenderer.h:12-19, Kd-treeConverterMain.cpp:3054). */
void kdgr_secondary_mesh_material_default(kdgr_material* m);
/* loadSecondaryMesh (Kd-treeConverterMain.cpp:179-221): triangles of an
 * .obj file (polygons fan-triangulated), each vertex mapped (x, y, z) ->
 * (x, -z, y); *verts holds 9 floats per triangle, free with kdgr_free. */
int kdgr_read_obj(const char* path, float** verts, uint32_t* n_tris);
void kdgr_free(void* p);
/* Upload secondary primitives: spheres, and/or one triangle mesh with one
 * material (the reference uses one kind at a time; with both, the closest
 * hit of either wins). */
int kdgr_secondary_create(const kdgr_sphere* spheres, int n_spheres, const float* tri_verts, uint32_t n_tris,
                          const kdgr_material* tri_material, kdgr_secondary_t* out);
int kdgr_secondary_destroy(kdgr_secondary_t sec);
int kdgr_render_hybrid(kdgr_scene_t scene, const kdgr_camera* cam, int width, int height, kdgr_secondary_t sec,
                       float* d_rgb, void* stream, float* ms_out);

/* ------------------------------------------------------------ debug report
 * Headless form of the reference's HIT_AND_NODE_COUNT_DEBUG report
 * (cudaRenderer.cu:3173-3400).  Counters, in this order: node visits, leaf
 * visits, intersection tests, hits found, blend ops, max sort size
 * (kdgr_ray_trace n_inner, n_leaf, n_cand, n_found, n_blend, max_sort).
 * Averages and totals are over pixels with at least one blend, accumulated
 * in FP32 in pixel order as the reference does; maxima over all pixels. */
typedef struct {
  float avg[6];
  float total[6];
  int32_t max[6];
  uint32_t n_pixels; /* pixels that blended at least one Gaussian */
} kdgr_debug_stats;

/* Reduce host-resident traces (d_trace of kdgr_render_trace copied back,
 * y*W + x order) to `out` (nullable) and, when out_dir is non-null, write the
 * reference's report files there: renderStats.txt, render_stats.csv,
 * heatmap_{node_visits,leaf_visits,intersection,hits_found,blend_ops,
 * max_sort_size}.{png,csv}, isectCnt_kd.bin and blendCnt_kd.bin.  Heatmaps
 * use the Turbo colormap over [0, heat_max] (the reference fixes 120).  Host
 * only; needs no GPU. */
int kdgr_debug_report(const kdgr_ray_trace* trace, int width, int height, const char* out_dir, float heat_max,
                      kdgr_debug_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* KDGR_H_ */
