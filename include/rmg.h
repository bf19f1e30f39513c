/*
 * rmg.h -- C ABI of the GB300 range-sensor ray-casting library.
 *
 * Every entry point is plain C: POD structs, raw pointers, sizes, an int
 * status.  No exception crosses this boundary and no torch type appears in it.
 * Device pointers are CUDA device (or managed) addresses; host pointers are
 * ordinary process memory.  `stream` is a cudaStream_t passed as void*
 * (NULL = the legacy default stream).  All GPU work is enqueued
 * asynchronously on that stream unless a function says it synchronises.
 *
 * Each declaration names the rmagine (uos/rmagine v2.4.2) interface it
 * replaces, as path:line inside that project.
 */
#ifndef RMG_H
#define RMG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RMG_ABI_VERSION 1

/* ---------------------------------------------------------------------------
 * Status codes.  The C++ wrapper turns a non-zero status into an exception,
 * mirroring RM_THROW / CudaException (src/rmagine_core/include/rmagine/util/
 * exceptions.h:48,78-85).
 * ------------------------------------------------------------------------- */
typedef enum rmg_status {
  RMG_OK = 0,
  RMG_ERR_INVALID_ARG = 1,       /* NULL handle, size out of range, bad model */
  RMG_ERR_CUDA = 2,              /* a CUDA runtime call failed */
  RMG_ERR_OOM = 3,               /* device allocation failed */
  RMG_ERR_TIMEOUT = 4,           /* rmg_stream_wait ran out of time */
  RMG_ERR_TRAVERSAL_BUDGET = 5,  /* a ray exceeded its node-visit budget (corrupt BVH) */
  RMG_ERR_NO_DEVICE = 6,         /* no CUDA device, or not an sm_103 part */
  RMG_ERR_UNSUPPORTED = 7        /* option value outside the compiled variants */
} rmg_status;

/* ---------------------------------------------------------------------------
 * Plain data types, byte-compatible with rmagine's.
 * ------------------------------------------------------------------------- */

/* rmagine::Vector3 (math/types/Vector3.hpp:52-56): 12 B. */
typedef struct rmg_vec3 { float x, y, z; } rmg_vec3;

/* rmagine::Quaternion (math/types/Quaternion.hpp:58-64): x, y, z, w. */
typedef struct rmg_quat { float x, y, z, w; } rmg_quat;

/* rmagine::Transform (math/types/Transform.hpp:63-68): 32 B, same field order. */
typedef struct rmg_transform { rmg_quat R; rmg_vec3 t; uint32_t stamp; } rmg_transform;

/* rmagine::Face (types/mesh_types.h:54-73): three vertex indices. */
typedef struct rmg_face { uint32_t v0, v1, v2; } rmg_face;

/* rmagine::Matrix3x3 storage is column-major: data[col*3 + row]
 * (math/types/Matrix.tcc:81-84). */
typedef struct rmg_mat3 { float data[9]; } rmg_mat3;

/* rmagine::CrossStatistics (math/types/CrossStatistics.hpp:51-57): 64 B. */
typedef struct rmg_cross_stats {
  rmg_vec3 dataset_mean;
  rmg_vec3 model_mean;
  rmg_mat3 covariance;   /* (1/n) sum (m_i - m_mean)(d_i - d_mean)^T, column-major */
  uint32_t n_meas;
} rmg_cross_stats;

/* rmagine::Interval / DiscreteInterval (types/sensor_models.h:54-105). */
typedef struct rmg_interval { float min, max; } rmg_interval;
typedef struct rmg_discrete_interval { float min, inc; uint32_t size; } rmg_discrete_interval;

typedef enum rmg_model_kind {
  RMG_MODEL_SPHERICAL = 0,  /* SphericalModel  sensor_models.h:118-215 */
  RMG_MODEL_PINHOLE = 1,    /* PinholeModel    sensor_models.h:217-315 */
  RMG_MODEL_O1DN = 2,       /* O1DnModel_      sensor_models.h:338-417 */
  RMG_MODEL_ONDN = 3        /* OnDnModel_      sensor_models.h:422-502 */
} rmg_model_kind;

/* One sensor model.  Fields a kind does not use are ignored.
 *  spherical: phi (vertical, rows), theta (horizontal, cols), range
 *  pinhole:   width, height, range, f[2] = (fx, fy), c[2] = (cx, cy)
 *  O1Dn:      width, height, range, orig, dirs[width*height]
 *  OnDn:      width, height, range, origs[width*height], dirs[width*height]
 * dirs / origs are HOST pointers; rmg_sensor_create copies them. */
typedef struct rmg_model {
  uint32_t kind;
  uint32_t width;
  uint32_t height;
  rmg_interval range;
  rmg_discrete_interval phi;
  rmg_discrete_interval theta;
  float f[2];
  float c[2];
  rmg_vec3 orig;
  const rmg_vec3* dirs;
  const rmg_vec3* origs;
} rmg_model;

/* Result buffers of one simulate call: the attribute set of rmagine's
 * IntAttrAll bundle (simulation/SimulationResults.hpp:56-159).  DEVICE
 * pointers, each sized n_poses*width*height, indexed
 * pose*width*height + row*width + col (SphereSimulatorEmbree.tcc:75-82).
 * A NULL pointer means "not requested", like a zero-sized Memory in the
 * reference's set_simulation_flags_ (embree_common.h:79-139). */
typedef struct rmg_outputs {
  uint8_t* hits;
  float* ranges;
  rmg_vec3* points;
  rmg_vec3* normals;
  uint32_t* face_ids;
  uint32_t* geom_ids;
  uint32_t* object_ids;
} rmg_outputs;

/* Traversal launch options (the knobs the autotuner searches). */
typedef struct rmg_launch_config {
  uint32_t stack_depth;   /* short-stack entries per ray: 0 (stackless, parent pointers), 8 or 16 */
  uint32_t block_warps;   /* warps per CTA */
  uint32_t tile_w;        /* a warp covers tile_h x tile_w rays of one pose */
  uint32_t tile_h;        /* tile_w * tile_h must be 32 */
  uint32_t refill;        /* 0: one tile per warp.  1..32: persistent warps that hand new rays to
                             idle lanes whenever fewer than `refill` lanes are busy (stack_depth 8 or 16) */
  uint32_t chunk;         /* refill mode: tiles a warp takes from the work counter at a time (>= 1) */
  uint32_t bvh_width;     /* 2: walk the binary tree; 4: the 4-wide tree collapsed from it; 8: the 8-wide
                             tree with quantized boxes collapsed from it (4 and 8 when the map has the tree
                             and refill == 0); 0: the default.  Results are identical. */
  uint32_t packet;        /* 1: the warp walks the binary tree together (a node is visited when any of
                             its 32 rays needs it; refill == 0, bvh_width != 4); 0: each ray walks alone;
                             2: the default.  Results are identical. */
} rmg_launch_config;

typedef struct rmg_map_info {
  uint32_t n_vertices;
  uint32_t n_faces;
  uint32_t n_nodes;       /* internal BVH nodes */
  uint32_t depth;         /* longest root-to-leaf path (edges) */
  uint64_t device_bytes;  /* BVH nodes (binary, 4-wide, 8-wide) + packed triangles (and their 8-wide copy)
                             + vertices + faces */
  float bounds_lo[3];
  float bounds_hi[3];
} rmg_map_info;

typedef struct rmg_map rmg_map;        /* opaque: triangle mesh + LBVH on one GPU */
typedef struct rmg_sensor rmg_sensor;  /* opaque: model + its device ray-direction table */

/* ---------------------------------------------------------------------------
 * Library / device.
 * ------------------------------------------------------------------------- */
const char* rmg_status_string(int status);
/* Last error message of the calling thread ("" when none). */
const char* rmg_last_error(void);
int rmg_abi_version(void);
/* Number of SMs and compute capability of the current device. */
int rmg_device_info(int* sm_count, int* cc_major, int* cc_minor);
/* Polls the stream until its work is done or timeout_ms elapses
 * (RMG_ERR_TIMEOUT).  Never blocks longer than the timeout. */
int rmg_stream_wait(void* stream, uint32_t timeout_ms);

/* ---------------------------------------------------------------------------
 * Map: triangle mesh + BVH.
 * Replaces EmbreeMesh::init/computeFaceNormals/apply + EmbreeScene::commit
 * (src/rmagine_embree/src/map/embree/EmbreeMesh.cpp:162-335,
 *  EmbreeScene.cpp:187-191) and OptixScene::commit (OptixScene.cpp:242-481).
 * vertices / faces are HOST arrays, copied before the call returns.  The
 * build runs on `stream` and the call synchronises with it.  n_faces == 0 is
 * allowed: every ray of such a map misses.
 * ------------------------------------------------------------------------- */
int rmg_map_build(const rmg_vec3* vertices, uint32_t n_vertices,
                  const rmg_face* faces, uint32_t n_faces,
                  void* stream, rmg_map** out);

/* Tree builders.  Results of every query are the same for both (the closest
 * hit does not depend on the tree); they differ in build time and in how many
 * nodes a ray visits. */
typedef enum rmg_builder {
  RMG_BUILD_SAH = 0,   /* top-down binned surface area heuristic, one triangle per leaf, depth <= 32
                          (the quality class of Embree's default build, EmbreeScene.hpp:61-83); the
                          default of rmg_map_build */
  RMG_BUILD_LBVH = 1   /* linear BVH over 63-bit Morton codes (Karras 2012): fastest build */
} rmg_builder;
/* rmg_map_build with an explicit builder. */
int rmg_map_build_ex(const rmg_vec3* vertices, uint32_t n_vertices,
                     const rmg_face* faces, uint32_t n_faces, uint32_t builder,
                     void* stream, rmg_map** out);
/* Moves the vertices (same count, same faces) and refits every box of the
 * existing tree bottom-up without re-sorting.  Needs exclusive use of the
 * map (no simulate in flight).  Synchronises with `stream`. */
int rmg_map_refit(rmg_map* map, const rmg_vec3* vertices, uint32_t n_vertices, void* stream);

/* Adds the 8-wide tree with quantized child boxes (80-byte nodes after Ylitie,
 * Karras and Laine, HPG 2017) collapsed from the map's binary tree, for
 * rmg_launch_config.bvh_width = 8; refits refresh it.  Opt-in, as Embree's
 * scene build options choose its BVH (EmbreeScene.hpp:61-83): on the
 * workloads measured here the binary walk is faster, so maps do not build it
 * by default.  Not concurrent with simulate calls on the same map; synchronises
 * with `stream`.  A map whose boxes cannot be quantized (extents beyond
 * 255 * 2^60) keeps no 8-wide tree. */
int rmg_map_build_wide8(rmg_map* map, void* stream);
int rmg_map_destroy(rmg_map* map);
int rmg_map_info_get(const rmg_map* map, rmg_map_info* out);
/* Copies the tree to host memory (tests): nodes = n_nodes*16 floats/ints
 * (the 64-byte node records), tris = n_faces*12 floats (48-byte records),
 * leaf_order = n_faces sorted face ids.  Any pointer may be NULL. */
int rmg_map_export(const rmg_map* map, void* nodes, void* tris, uint32_t* leaf_order);
/* Reads the map's device error word (synchronous).  Returns RMG_OK or the
 * recorded error (e.g. RMG_ERR_TRAVERSAL_BUDGET); `clear` != 0 resets it. */
int rmg_map_status(rmg_map* map, int clear);
/* Test hook: overwrite one child link of one BVH node (synchronous).  Used
 * to check that a corrupt tree ends in RMG_ERR_TRAVERSAL_BUDGET, not a
 * fault; values are range-checked so every link stays inside the arrays.
 * which 0 / 1: left / right link of binary node `node` (the map then drops
 * its 4-wide tree, so the damaged binary tree is the one walked);
 * which 2..5: slot which-2 of 4-wide node `node`. */
int rmg_map_debug_set_child(rmg_map* map, uint32_t node, uint32_t which, int32_t child);

/* ---------------------------------------------------------------------------
 * Sensor model.
 * Replaces XSimulator::setModel (SphereSimulatorEmbree.hpp:115-116,
 * SphereSimulatorOptix.hpp:130-131).  The model's per-ray sensor-frame
 * directions (and OnDn origins) are materialised once in device memory:
 * SphericalModel::getDirection (sensor_models.h:169-174) and
 * PinholeModel::getDirection (:256-276) are evaluated on the GPU; O1Dn/OnDn
 * tables (:375-384, :460-468) are copied from the host arrays.  An O1Dn/OnDn
 * table whose directions are scattered (its neighbours far apart, as in a
 * table of random directions) gets a visiting order sorted by elevation band
 * and azimuth, so that the rays a warp walks together share their paths;
 * outputs, observations and every other per-ray array keep the table's own
 * order, and the results are the same.
 * ------------------------------------------------------------------------- */
int rmg_sensor_create(const rmg_model* model, void* stream, rmg_sensor** out);
int rmg_sensor_destroy(rmg_sensor* sensor);
/* Copies the sensor-frame direction table (width*height) to host memory. */
int rmg_sensor_directions(const rmg_sensor* sensor, rmg_vec3* host_out);
int rmg_sensor_size(const rmg_sensor* sensor, uint32_t* width, uint32_t* height);
/* No counterpart in the reference (Embree casts each ray on its own).
 * *sorted = 1 when the sensor visits its rays in a sorted order (and, when
 * host_out is not NULL, copies that order: width*height table indices),
 * *sorted = 0 when it visits them in the table's order. */
int rmg_sensor_visit_order(const rmg_sensor* sensor, uint32_t* host_out, int* sorted);

/* ---------------------------------------------------------------------------
 * Simulate.
 * Replaces {Sphere,Pinhole,O1Dn,OnDn}Simulator{Embree,Optix}::simulate
 * (SphereSimulatorEmbree.tcc:51-254, PinholeSimulatorEmbree.tcc:51-254,
 *  O1DnSimulatorEmbree.tcc:50-254, OnDnSimulatorEmbree.tcc:51-257;
 *  SphereSimulatorOptix.tcc:44-90 for the device-buffer form).
 * Tsb: HOST pointer to one sensor-to-base transform (setTsb,
 *      SimulatorEmbree.hpp:60-61).
 * Tbm: DEVICE array of n_poses base-to-map transforms.
 * Semantics follow the Embree path: closest hit in (0, range.max]; hits =
 * (t >= range.min); ranges = t; points = dir_s*t (+ orig_s); normals =
 * geometric normal in the sensor frame facing the ray; face_ids = primitive
 * id; geom_ids = object_ids = 0 (single mesh).  Misses: hits 0, ranges =
 * range.max + 1, points/normals NaN, ids UINT32_MAX.
 * Asynchronous on `stream`.
 * ------------------------------------------------------------------------- */
int rmg_simulate(const rmg_map* map, const rmg_sensor* sensor,
                 const rmg_transform* Tsb, const rmg_transform* Tbm, uint32_t n_poses,
                 const rmg_outputs* out, void* stream);
/* Same with explicit launch options (NULL = library default). */
int rmg_simulate_ex(const rmg_map* map, const rmg_sensor* sensor,
                    const rmg_transform* Tsb, const rmg_transform* Tbm, uint32_t n_poses,
                    const rmg_outputs* out, const rmg_launch_config* cfg, void* stream);
/* Fills *cfg with the library default for this sensor/map. */
int rmg_default_launch_config(const rmg_map* map, const rmg_sensor* sensor, rmg_launch_config* cfg);

/* Host form of rmg_simulate: the RAM-bundle overload of the Embree simulators
 * (SphereSimulatorEmbree.hpp:130-155, simulate(Memory<Transform,RAM>, Bundle
 * of RAM buffers)).  Tbm and every non-NULL output are HOST pointers (pinned
 * or pageable; device pointers also work).  The poses are uploaded once and
 * the rays cast in pose chunks into device staging memory on `stream`; each
 * chunk's outputs are copied to the host on a second stream while the next
 * chunks are cast.  Results are bit-identical to rmg_simulate.  Synchronous:
 * returns when `out` holds every result.  cfg may be NULL (library default).
 * Staging comes from a per-device stream-ordered pool that keeps its memory
 * between calls (rmg_host_staging_trim releases it). */
int rmg_simulate_host(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                      const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                      const rmg_launch_config* cfg, void* stream);
/* Pipeline shape of the host forms (process-wide): output bytes per pose
 * chunk (0 = the default, 128 MiB; at least one pose per chunk) and compute
 * streams the chunks alternate over (0 = the default, 2; at most 3), so that
 * one chunk's last warps overlap the next chunk's first ones.  Results do not
 * depend on either. */
int rmg_host_set_pipeline(uint64_t chunk_bytes, uint32_t compute_streams);
/* Points in the host forms of simulate (process-wide; no counterpart in the
 * reference).  A point is dir_s * range (+ orig_s) for a hit and NaN for a
 * miss, so when Ranges and at least 64 MB of Points are wanted, host threads
 * form the points from the copied ranges instead of moving 12 bytes per ray
 * over the host link (policy 0, the default); policy 1 copies them like the
 * other attributes and keeps the host threads free.  The results are the same
 * bytes under both. */
int rmg_host_set_points_policy(uint32_t policy);
/* Returns the host forms' cached staging memory to the driver. */
int rmg_host_staging_trim(void);

/* Times a fixed set of launch configurations (per-ray binary walk, warp
 * packet walk, 4-wide walk; tiles 8x4, 16x2, 4x8; 4 or 2 warps per CTA) on
 * the caller's poses and output buffers -- all write the same results -- and
 * returns the fastest (median of `reps` runs after a warm-up).  Same pointer
 * rules as rmg_simulate; synchronises.  No counterpart in the reference. */
int rmg_autotune_launch_config(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                               const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out,
                               uint32_t reps, rmg_launch_config* best, void* stream);

/* ---------------------------------------------------------------------------
 * Batched heterogeneous sensors (no counterpart in the reference, where each
 * simulator call launches once per sensor: SphereSimulatorOptix.cpp:64-81).
 * A plan binds many (sensor, Tsb, Tbm, n_poses, outputs) jobs on one map; a
 * launch runs ALL their rays in one persistent kernel replayed from a CUDA
 * graph.  Outputs are bit-identical to one rmg_simulate per job.  The plan
 * keeps the DEVICE pointers given at creation (update poses in place).
 * ------------------------------------------------------------------------- */
typedef struct rmg_batch_entry {
  const rmg_sensor* sensor;
  rmg_transform Tsb;           /* by value */
  const rmg_transform* Tbm;    /* DEVICE, n_poses records */
  uint32_t n_poses;
  rmg_outputs out;             /* DEVICE buffers, as for rmg_simulate */
} rmg_batch_entry;

typedef struct rmg_batch_config {
  uint32_t stack_depth;  /* 0, 8 or 16 */
  uint32_t block_warps;  /* 1..8 */
  uint32_t tile_w;       /* tile of a 2-D sensor, tile_w * tile_h == 32; 1-row sensors use 32 x 1 */
  uint32_t tile_h;
  uint32_t grab;         /* tiles a warp takes from the work counter at a time, 1..64 */
  uint32_t ctas_per_sm;  /* 0 = as many as fit */
  uint32_t use_graph;    /* 1 = replay a captured CUDA graph, 0 = direct launch */
} rmg_batch_config;

typedef struct rmg_batch rmg_batch;

int rmg_batch_default_config(rmg_batch_config* cfg);
int rmg_batch_create(const rmg_map* map, const rmg_batch_entry* entries, uint32_t n_entries, rmg_batch** out);
int rmg_batch_set_config(rmg_batch* batch, const rmg_batch_config* cfg);
int rmg_batch_get_config(const rmg_batch* batch, rmg_batch_config* cfg);
int rmg_batch_info(const rmg_batch* batch, uint64_t* total_rays, uint64_t* total_tiles);
/* Asynchronous on `stream`.  The first launch after creation or a config
 * change captures the graph (do not call it while `stream` is capturing). */
int rmg_batch_launch(rmg_batch* batch, void* stream);
/* Times candidate configs on the plan itself (reps timed launches each, after
 * a warm-up), keeps the fastest and returns it in *best (may be NULL).
 * Runs the plan's work several times: outputs hold the last run's results. */
int rmg_batch_autotune(rmg_batch* batch, void* stream, uint32_t reps, rmg_batch_config* best);
int rmg_batch_destroy(rmg_batch* batch);

/* ---------------------------------------------------------------------------
 * Range adjoint (no counterpart in the reference: rmagine has no
 * differentiable simulator).  Casts the rays of every pose exactly as
 * rmg_simulate does and, in the same kernel, accumulates per pose
 *   loss = sum Huber_delta(r_sim - r_obs),  grad = dloss/dxi (6 floats)
 * over rays with a simulated hit (range.min <= t) and an observation in
 * [range.min, range.max].  xi = (rho, omega) is the right perturbation
 * T_bm * exp(xi^) (lie.h:57-114 conventions), translation first.
 * ranges_obs: DEVICE n_poses*W*H.  grad: DEVICE n_poses*6, loss: DEVICE
 * n_poses (either may be NULL, not both); ranges_sim / face_ids: optional
 * DEVICE copies of the simulated ranges and face ids.  At most 65535 poses
 * per call.  Deterministic (fixed reduction order).  Asynchronous. */
int rmg_range_pose_grad(const rmg_map* map, const rmg_sensor* sensor,
                        const rmg_transform* Tsb, const rmg_transform* Tbm, uint32_t n_poses,
                        const float* ranges_obs, float huber_delta,
                        float* grad, float* loss, float* ranges_sim, uint32_t* face_ids, void* stream);

/* Host form of rmg_range_pose_grad: Tbm, ranges_obs and every output are HOST
 * pointers (pinned or pageable).  Observations are uploaded and results
 * downloaded in pose chunks that overlap the launches; any number of poses.
 * Results are bit-identical to rmg_range_pose_grad.  Synchronous. */
int rmg_range_pose_grad_host(const rmg_map* map, const rmg_sensor* sensor,
                             const rmg_transform* Tsb, const rmg_transform* Tbm, uint32_t n_poses,
                             const float* ranges_obs, float huber_delta,
                             float* grad, float* loss, float* ranges_sim, uint32_t* face_ids, void* stream);

/* ---------------------------------------------------------------------------
 * Correspondence statistics and Umeyama.
 *
 * rmagine::UmeyamaReductionConstraints (types/UmeyamaReductionConstraints.hpp:46-59). */
typedef struct rmg_umeyama_constraints {
  float max_dist;        /* ignore correspondences at or beyond this distance */
  uint32_t dataset_id;   /* with dataset_ids: keep only this id */
  uint32_t model_id;     /* with model_ids: keep only this id */
} rmg_umeyama_constraints;

/* Batched statistics_p2p (statistics.cpp:19-57, statistics.cu:58-160):
 * batch b reduces correspondences [b*n_per_batch, (b+1)*n_per_batch) of the
 * DEVICE arrays dataset_points / model_points (+ optional masks and ids,
 * NULL = unused) to one CrossStatistics.  Dataset points are first mapped by
 * pre_transforms (DEVICE; NULL = identity; stride 0 = one transform for all
 * batches, 1 = one per batch).  Filter: masks > 0, ids == params ids,
 * ||M - D||^2 < max_dist^2.  Accumulation in binary64.  Outputs (DEVICE, NULL
 * = not wanted): stats[n_batches] and transforms[n_batches] = the Umeyama
 * transform of each batch (optimization.cpp:12-49, memory_math.cu:1627-1708)
 * solved in binary64.  params is a HOST pointer.  Asynchronous. */
int rmg_statistics_p2p(const rmg_transform* pre_transforms, uint32_t pre_transform_stride,
                       const rmg_vec3* dataset_points, const uint8_t* dataset_mask, const uint32_t* dataset_ids,
                       const rmg_vec3* model_points, const uint8_t* model_mask, const uint32_t* model_ids,
                       const rmg_umeyama_constraints* params, uint32_t n_batches, uint32_t n_per_batch,
                       rmg_cross_stats* stats, rmg_transform* transforms, void* stream);

/* Batched statistics_p2l (statistics.cpp:84-126, statistics.cu:190-276):
 * model points are plane points with model_normals; the model correspondence is
 * the projection M = D + N ((I - D) . N), kept when |(I - D) . N| < max_dist. */
int rmg_statistics_p2l(const rmg_transform* pre_transforms, uint32_t pre_transform_stride,
                       const rmg_vec3* dataset_points, const uint8_t* dataset_mask, const uint32_t* dataset_ids,
                       const rmg_vec3* model_points, const rmg_vec3* model_normals,
                       const uint8_t* model_mask, const uint32_t* model_ids,
                       const rmg_umeyama_constraints* params, uint32_t n_batches, uint32_t n_per_batch,
                       rmg_cross_stats* stats, rmg_transform* transforms, void* stream);

/* Batched umeyama_transform(CrossStatistics) (memory_math.cu:1646-1656,
 * optimization.cpp:51-55): DEVICE stats[n] -> DEVICE out[n]. */
int rmg_umeyama_transform(const rmg_cross_stats* stats, uint32_t n, rmg_transform* out, void* stream);

/* Batched 3x3 singular value decomposition A = U W V^T.  Replaces rmagine's
 * svd(MemoryView<Matrix3x3,VRAM_CUDA> As, Us, Ws, Vs) and the ws-vector form
 * (src/rmagine_cuda/include/rmagine/math/memory_math.cuh:561-578, kernels
 * memory_math.cu:1564-1622) and the per-matrix svd (math/linalg.h:164-175,
 * linalg.cpp:101, 645).  A, U, W, V: n column-major 3x3 float matrices
 * (rmagine::Matrix3x3) in DEVICE memory; w: n Vector3 (the diagonal of W);
 * any output may be NULL.  Computed in binary64 (Jacobi on A^T A), returned in
 * binary32.  rotations == 0: the usual form, W >= 0 sorted descending, U and V
 * orthogonal.  rotations != 0: U and V both
 * rotations and the last singular value signed (sign det A), the form of the
 * Kabsch/Umeyama step (R = U V^T).  Singular values are unique; U and V are
 * unique only up to the usual sign and subspace freedom, so parity with
 * rmagine's Numerical-Recipes svdcmp is on the reconstruction, the
 * orthonormality and the singular values, as in its own tests
 * (tests/core/math_svd.cpp:161-237, tests/cuda/math_svd.cpp:38-109). */
int rmg_svd3(const float* A, float* U, float* W, float* w, float* V, uint32_t n, int rotations, void* stream);

/* Backward of statistics_p2p + Umeyama (no counterpart in the reference):
 * given the forward's stats and upstream gradients grad_R (DEVICE, 9 floats
 * per batch, row-major dL/dR of the rotation matrix; NULL = 0) and grad_t
 * (DEVICE, 3 per batch; NULL = 0), writes dL/d(dataset point) and dL/d(model
 * point) for every correspondence (DEVICE float3 arrays; NULL = skip;
 * filtered-out correspondences get 0).  Same inputs and filter as the forward. */
int rmg_umeyama_backward(const rmg_transform* pre_transforms, uint32_t pre_transform_stride,
                         const rmg_vec3* dataset_points, const uint8_t* dataset_mask, const uint32_t* dataset_ids,
                         const rmg_vec3* model_points, const uint8_t* model_mask, const uint32_t* model_ids,
                         const rmg_umeyama_constraints* params, uint32_t n_batches, uint32_t n_per_batch,
                         const rmg_cross_stats* stats, const float* grad_R, const float* grad_t,
                         rmg_vec3* grad_dataset, rmg_vec3* grad_model, void* stream);

/* ---------------------------------------------------------------------------
 * Mesh files and map files.
 *
 * rmg_mesh_read stands in for AssimpIO::ReadFile (map/AssimpIO.hpp:50-66) as
 * used by import_embree_map / import_optix_map (EmbreeMap.hpp:94-117) for
 * the mesh formats maps come in: PLY (ascii, binary little / big endian),
 * Wavefront OBJ and STL (binary, ascii), chosen by the file extension.
 * Polygons are split into triangle fans; OBJ objects / groups become groups
 * (face_group), the separate meshes Assimp makes of them; STL triangles keep
 * their own three vertices.  The arrays are HOST memory owned by the library:
 * release them with rmg_mesh_free.  Malformed files: RMG_ERR_INVALID_ARG. */
typedef struct rmg_mesh {
  rmg_vec3* vertices;
  uint32_t n_vertices;
  rmg_face* faces;
  uint32_t n_faces;
  uint32_t* face_group;  /* group of each face (0 for PLY / STL) */
  uint32_t n_groups;
} rmg_mesh;

int rmg_mesh_read(const char* path, rmg_mesh* out);
void rmg_mesh_free(rmg_mesh* mesh);
/* Binary PLY (host byte order) of HOST arrays, readable by rmg_mesh_read. */
int rmg_mesh_write_ply(const char* path, const rmg_vec3* vertices, uint32_t n_vertices,
                       const rmg_face* faces, uint32_t n_faces);

/* The built map (mesh + tree) to a file and back, without a rebuild.  No
 * counterpart in the reference (it rebuilds on every import).  A load checks
 * sizes, a checksum and every index the kernels follow before uploading;
 * a damaged file gives RMG_ERR_INVALID_ARG.  Both synchronise. */
int rmg_map_save(const rmg_map* map, const char* path);
int rmg_map_load(const char* path, void* stream, rmg_map** out);

/* ---------------------------------------------------------------------------
 * Range noise, applied in place to a DEVICE Ranges buffer.
 *
 * Replaces GaussianNoiseCuda / RelGaussianNoiseCuda / UniformDustNoiseCuda
 * ::apply (src/rmagine_cuda/src/noise/GaussianNoiseCuda.cu:9-52,
 * RelGaussianNoiseCuda.cu:9-58, UniformDustNoiseCuda.cu:8-73) with the same
 * per-element arithmetic and Noise::Options (seed, max_range;
 * noise/Noise.hpp:52-55).  Random numbers come from the counter-based
 * Philox4x32-10 generator keyed by `seed`, with `call` as the upper counter
 * words: a pure function of (seed, call, element), no per-element state.
 * Increment `call` for each apply to draw fresh noise (the reference's
 * curand states advance instead).  Asynchronous. */
typedef enum rmg_noise_kind {
  RMG_NOISE_GAUSSIAN = 0,      /* r <= max_range: r += z * stddev + mean */
  RMG_NOISE_REL_GAUSSIAN = 1,  /* r <= max_range: r += z * (stddev * r^range_exp) + mean */
  RMG_NOISE_UNIFORM_DUST = 2   /* early returns with probability 1 - (1 - hit_probability)^r ... */
} rmg_noise_kind;

typedef struct rmg_noise {
  uint32_t kind;
  float mean;
  float stddev;
  float range_exp;
  float hit_probability;      /* dust: hit probability per metre */
  float return_probability;   /* dust: return probability per metre */
  float max_range;            /* Noise::Options::max_range (10000 by default) */
  uint64_t seed;              /* Noise::Options::seed (42 by default) */
  uint64_t call;              /* apply-call counter */
} rmg_noise;

int rmg_noise_apply(const rmg_noise* noise, float* ranges, uint64_t n, void* stream);
/* Device error word of the noise kernels on the current device: 0, or
 * RMG_ERR_TIMEOUT when a bulk copy into a kernel's shared-memory ring did not
 * land within the kernel's wait limit (that chunk and the rest of its CTA's
 * chunks were left unchanged).  Synchronises; `clear` != 0 resets it.  No
 * counterpart in rmagine, whose noise kernels have no waits. */
int rmg_noise_status(uint32_t* status, int clear);
/* The generator itself (for tests): out[4*i .. 4*i+3] = Philox4x32-10 of
 * counter (i, call) and key seed, i < n_blocks; DEVICE out. */
int rmg_noise_philox(const rmg_noise* noise, uint32_t* out, uint64_t n_blocks, void* stream);

/* ---------------------------------------------------------------------------
 * Scenes: several meshes and instances of them (two-level BVH).
 *
 * Replaces EmbreeScene::add / commit with EmbreeInstance::set / setTransform /
 * setScale / apply (EmbreeScene.cpp:246-406, EmbreeInstance.cpp:33-60,
 * EmbreeGeometry.cpp) and OptixScene's instance hierarchy (OptixScene.cpp:
 * 396-481).  Each instance places one geometry (an rmg_map, the bottom-level
 * tree, which the scene references and does not own) in the map frame with
 * x_map = T * (scale (.) x_mesh), EmbreeInstance::apply's M = T * diag(scale).
 * The scene builds a top-level LBVH over the instances' map-frame boxes.
 *
 * Hits report, as the reference's IntAttrAll does for instanced scenes
 * (SphereSimulatorEmbree.tcc:160-186, SensorProgramHit.cu:220-262):
 * face_ids = the triangle's index in its own mesh, geom_ids / object_ids =
 * the instance's geom_id / object_id fields.  A binding that mirrors rmagine
 * sets object_id = the instance's id in the top-level scene and geom_id = the
 * mesh's id inside the instanced scene; for a mesh added to the scene without
 * an instance both are the mesh's id (and T = identity, scale = 1).
 * Normals are the hit triangle's normal taken to the map frame by the
 * instance (R * scale^-1 (.) n, the OptiX path's
 * optixTransformNormalFromObjectToWorldSpace, SensorProgramHit.cu:120-136),
 * then to the sensor frame as for a single mesh.
 * The closest hit over all instances wins; equal ranges go to the smaller
 * instance index, then the smaller face index. */
typedef struct rmg_scene rmg_scene;  /* opaque */

typedef struct rmg_instance_desc {
  uint32_t geometry;   /* index into the scene's geometry list */
  uint32_t geom_id;    /* reported in GeomIds for hits on this instance */
  uint32_t object_id;  /* reported in ObjectIds */
  rmg_transform T;     /* instance pose in the map frame */
  rmg_vec3 scale;      /* per-axis scale applied before T; no component may be 0 */
} rmg_instance_desc;

/* geometries: HOST array of n_geometries map handles (each built with
 * rmg_map_build, tree depth <= 32, alive as long as the scene);
 * instances: HOST array.  Builds the top-level tree on `stream` and
 * synchronises with it.  n_instances == 0 gives a scene where every ray misses.
 * The tree of a geometry of 32,768 triangles or more is opened into pieces
 * that enter the top-level tree separately (same results, faster walks). */
int rmg_scene_create(const rmg_map* const* geometries, uint32_t n_geometries,
                     const rmg_instance_desc* instances, uint32_t n_instances, void* stream, rmg_scene** out);
/* New instance poses, scales or ids (same count).  rebuild == 0 refits the
 * top-level tree in place (rmg_map_refit's semantics: fast, topology kept);
 * rebuild != 0 builds it anew.  Call it too after rmg_map_refit of a geometry
 * (its bounds changed).  Needs exclusive use of the scene; synchronises. */
int rmg_scene_update(rmg_scene* scene, const rmg_instance_desc* instances, uint32_t n_instances, int rebuild,
                     void* stream);
int rmg_scene_destroy(rmg_scene* scene);
/* Device error word of the scene (RMG_ERR_TRAVERSAL_BUDGET after a corrupt
 * tree), like rmg_map_status; synchronises. */
int rmg_scene_status(rmg_scene* scene, int clear);
/* rmg_simulate on a scene: same sensors, poses, outputs and semantics. */
int rmg_simulate_scene(const rmg_scene* scene, const rmg_sensor* sensor, const rmg_transform* Tsb,
                       const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out, void* stream);
/* Host form of rmg_simulate_scene (host poses and outputs), pipelined and
 * synchronous like rmg_simulate_host. */
int rmg_simulate_scene_host(const rmg_scene* scene, const rmg_sensor* sensor, const rmg_transform* Tsb,
                            const rmg_transform* Tbm, uint32_t n_poses, const rmg_outputs* out, void* stream);

/* ---------------------------------------------------------------------------
 * Fused simulate -> statistics (the inner step of the RCC / MICP-L correction
 * loop, tests/embree/correction_rcc.cpp:139-160).
 *
 * Replaces, per pose p, the sequence
 *     simulate(Tbm[p], model bundle: Points, Normals, Hits)
 *         (SphereSimulatorEmbree.tcc:42-253 and the other three models)
 *     stats[p] = statistics_p2l(pre, dataset, model, params)   (statistics.cpp:84-126)
 *          (or statistics_p2p, statistics.cpp:19-57, when point_to_plane == 0)
 *     transforms[p] = umeyama_transform(stats[p])              (optimization.cpp:12-49)
 * in one ray-casting launch that never writes the model bundle: ray i of pose
 * p is paired with dataset point i of the pose's scan.  The model side of ray i
 * is valid when it hits with range >= range.min (the Hits attribute); its point
 * and normal equal the Points / Normals attributes of rmg_simulate bit for bit.
 * The filter and pairing follow rmg_statistics_p2p / _p2l; the model ids filter
 * is not applied (a simulated model cloud carries no ids in that loop:
 * correction_rcc.cpp:143-147 builds it from points, hits and normals).
 * Dataset rays that are masked out are not cast.  The sums may be added in a
 * different order from rmg_simulate + rmg_statistics_p2l (binary32 partial
 * sums folded into binary64), so the statistics agree with that pair to
 * binary32 rounding and n_meas agrees exactly. */
typedef struct rmg_scan {
  const rmg_vec3* points;  /* DEVICE [n_scans][width*height], sensor frame, ray order of rmg_simulate */
  const uint8_t* mask;     /* DEVICE, > 0 = valid (e.g. the scan's Hits), or NULL */
  const uint32_t* ids;     /* DEVICE, compared with params->dataset_id, or NULL */
  uint32_t per_pose;       /* 1: scan p belongs to pose p; 0: one scan for every pose */
} rmg_scan;

/* Tsb, dataset and params are HOST pointers; Tbm[n_poses], pre_transforms
 * (NULL = identity; stride 0 = one for all poses, 1 = one per pose) and the
 * outputs stats[n_poses] / transforms[n_poses] (NULL = not wanted, not both)
 * are DEVICE pointers.  Asynchronous on `stream`.  No counterpart in the
 * reference (it always materialises the model bundle). */
int rmg_simulate_statistics(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                            const rmg_transform* Tbm, uint32_t n_poses, const rmg_scan* dataset,
                            const rmg_transform* pre_transforms, uint32_t pre_transform_stride,
                            const rmg_umeyama_constraints* params, int point_to_plane,
                            rmg_cross_stats* stats, rmg_transform* transforms, void* stream);

/* Host form of rmg_simulate_statistics: Tbm, the dataset's arrays,
 * pre_transforms and the outputs are HOST pointers (pinned or pageable).
 * Per-pose scans are uploaded in pose chunks while earlier chunks are
 * reduced; results are bit-identical to rmg_simulate_statistics on the same
 * data.  Synchronous.  rmg_host_set_pipeline shapes the chunks (input bytes
 * per chunk) and the compute streams. */
int rmg_simulate_statistics_host(const rmg_map* map, const rmg_sensor* sensor, const rmg_transform* Tsb,
                                 const rmg_transform* Tbm, uint32_t n_poses, const rmg_scan* dataset,
                                 const rmg_transform* pre_transforms, uint32_t pre_transform_stride,
                                 const rmg_umeyama_constraints* params, int point_to_plane,
                                 rmg_cross_stats* stats, rmg_transform* transforms, void* stream);

/* Batched Transform::mult (Transform.tcc:34-42; multInplace :44-56 when out
 * aliases a): out[i] = a[i] * b[i] for i < n, all DEVICE arrays; stride 0
 * repeats element 0 of that operand.  Lets a correction loop keep its pose
 * estimates on the device (Tpre = Tpre * T, Tbm = Tbm * Tpre). */
int rmg_transforms_compose(const rmg_transform* a, uint32_t a_stride, const rmg_transform* b, uint32_t b_stride,
                           rmg_transform* out, uint32_t n, void* stream);

/* ---------------------------------------------------------------------------
 * LBVH build without device allocation.
 * No counterpart in the reference: rmagine's maps always allocate their own
 * memory.  This is for callers that cannot call cudaMalloc -- real-time loops
 * that forbid allocator calls once they run, and hosts that hand the library
 * one fixed device arena and own every other byte of device memory.  The
 * caller passes the mesh in DEVICE
 * memory and receives the tree in its own DEVICE buffers, in the same record
 * layouts rmg_map_export returns; the build's temporary data (Morton keys,
 * sort buffers, bounds) lives in a fixed 4 MiB device array inside the
 * library, which limits the mesh to RMG_NOALLOC_MAX_FACES faces (larger
 * meshes return RMG_ERR_INVALID_ARG).  The first call on a device looks up
 * that array's address.  Calls share the
 * array and it keeps the last call's contents (each call clears what must
 * start at zero): calls that overlap on the GPU race.  Synchronises with
 * `stream` once (face-index check).
 * ------------------------------------------------------------------------- */
#define RMG_NOALLOC_MAX_FACES 65536u

typedef struct rmg_lbvh_buffers {
  void* nodes;            /* max(n_faces - 1, 1) 64-byte node records, 16-byte aligned */
  void* tris;             /* n_faces 48-byte triangle records, 16-byte aligned */
  uint32_t* leaf_order;   /* n_faces: face id of each leaf */
  int32_t* leaf_parent;   /* n_faces: parent node of each leaf */
  uint32_t* flags;        /* max(n_faces - 1, 1) refit counters (cleared by the call) */
} rmg_lbvh_buffers;

int rmg_lbvh_build_noalloc(const rmg_vec3* vertices, uint32_t n_vertices,
                           const rmg_face* faces, uint32_t n_faces,
                           const rmg_lbvh_buffers* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* RMG_H */
