/*
 * bonxai_gb300 -- C ABI of the GB300 (sm_103a) sparse voxel grid.
 *
 * This is the drop-in boundary: the C++ headers include/bonxai/bonxai.hpp and
 * include/bonxai_map/probabilistic_map.hpp re-create the reference's classes
 * on top of these functions, and any other language binds them through its FFI
 * (plain pointers and sizes, no C++ or torch types).
 *
 * Every entry point is named after the reference interface it replaces, cited
 * as path:line in the reference repository (bonxai_core/include/bonxai/ and
 * bonxai_map/). The reference is a header-only C++ library with no C ABI of its
 * own; each batch function here performs, in one GPU pass, what a loop of the
 * cited scalar C++ calls does, with the same results.
 *
 * Pointers: every input/output array may be host memory (pageable or pinned)
 * or device memory; the library checks with cudaPointerGetAttributes and
 * stages host arrays through the handle's device scratch. Coordinates are
 * packed int32 x,y,z triples. Points are packed x,y,z of float or double with
 * an optional byte stride (e.g. 16 for pcl::PointXYZ).
 *
 * Errors: every function returns a bxg_status. The reference throws
 * std::runtime_error or returns nullptr (bonxai.hpp:399-401,
 * serialization.hpp:128-130); here the text of the last error of a handle is
 * kept and returned by bxg_last_error(). A failed call leaves the map usable.
 *
 * Threading: calls on one handle are serialised by the caller (the reference's
 * writers are not thread-safe either, README.md:128-133); different handles
 * may be used from different host threads. Each handle runs on its own CUDA
 * stream (or the one given in bxg_config). Synchronous calls return after the
 * GPU work completes, like the reference's calls.
 */
#ifndef BONXAI_GB300_H
#define BONXAI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  BXG_OK = 0,
  BXG_ERR_INVALID_ARG = 1,
  BXG_ERR_OUT_OF_POOL = 2,    /* node pools reached the configured HBM budget */
  BXG_ERR_HASH_FULL = 3,      /* root hash could not grow within the budget */
  BXG_ERR_WAIT_TIMEOUT = 4,   /* a bounded device-side wait gave up */
  BXG_ERR_CUDA = 5,           /* a CUDA runtime call failed */
  BXG_ERR_NO_DEVICE = 6,      /* no usable CUDA device */
  BXG_ERR_CAPACITY = 7        /* caller's output buffer too small (size returned) */
} bxg_status;

/* Pool/stream configuration; zero-initialise and set what you need. */
typedef struct {
  size_t pool_budget_bytes; /* max device bytes for hash+inner+leaf pools; 0 = 16 GiB */
  uint32_t initial_leaves;  /* leaf slots allocated up front; 0 = 4096 */
  uint32_t initial_inners;  /* inner slots allocated up front; 0 = 1024 */
  uint32_t hash_buckets;    /* root hash buckets (power of two); 0 = 4096 */
  float hash_load_factor;   /* grow the root hash above this load; 0 = 0.5 */
  int device;               /* CUDA device ordinal; -1 = current */
  void* stream;             /* cudaStream_t to run on; NULL = a stream of its own */
  uint32_t rays_per_warp;   /* ray kernel: rays per warp 1, 2 or 4; 0 = 1 */
  uint32_t block_size;      /* ray kernel threads per block, 64..1024 (256 at most with
                               ray_unroll 2); 0 = 1024 for scans of at least
                               2 x SMs x 32 x rays_per_warp points, else 256 */
  uint32_t flags;           /* BXG_FLAG_* */
  uint32_t ray_unroll;      /* ray kernel: cells per lane per step, 1 or 2; 0 = 1 */
  /* (the defaults are what python -m bonxai_gb300.autotune picks on a GB300) */
} bxg_config;

/* Drop points with a NaN or infinite coordinate before insertion, as the
 * reference's ROS node does before calling insertPointCloud
 * (bonxai_ros/src/bonxai_server.cpp:147-154). Default on. */
#define BXG_FLAG_KEEP_NONFINITE 1u
/* Record CUDA events around each kernel (see bxg_pmap_kernel_times). */
#define BXG_FLAG_TIMING 2u
/* Batched ticks: launch directly instead of replaying a captured CUDA graph. */
#define BXG_FLAG_NO_GRAPH 4u
/* The ray phase of a scan walks each ray once and updates its cells on the
 * way (one pass), instead of marking the scan's ray cells in a bitmap and
 * then updating each marked leaf once (two phases, the default). Same
 * results; which is faster depends on the scan (the autotuner times both). A
 * batched tick uses one pass when any of its maps has this flag. */
#define BXG_FLAG_RAYS_SINGLE_PASS 8u

void bxg_config_default(bxg_config* cfg);
const char* bxg_status_string(int status);
/* Version of this library as major*10000 + minor*100 + patch. */
int bxg_version(void);

/* ========================================================================
 * VoxelGrid<T>  (bonxai_core/include/bonxai/bonxai.hpp:114-333)
 * ======================================================================== */
typedef struct bxg_grid_s* bxg_grid;

/* VoxelGrid(double voxel_size, uint8_t inner_bits=2, uint8_t leaf_bits=3)
 * (bonxai.hpp:138,389-402). value_bytes = sizeof(T): 1, 2, 4, 8 or 0 for
 * BinaryVoxelGrid = VoxelGrid<EmptyVoxel> (bonxai.hpp:335). inner_bits in
 * [1,4], leaf_bits in [1,5]; the reference rejects bits < 1 the same way. */
int bxg_grid_create(bxg_grid* out, double voxel_size, int inner_bits, int leaf_bits,
                    size_t value_bytes, const bxg_config* cfg);
int bxg_grid_destroy(bxg_grid g);
const char* bxg_last_error(const void* handle);

/* posToCoord(x,y,z) = floor(x * (1.0/voxel_size)) per axis in double
 * (bonxai.hpp:404-410) for n double points. */
int bxg_grid_pos_to_coord(bxg_grid g, const double* xyz, size_t n, int32_t* out_xyz);

/* Accessor::setValue(coord, value) for items 0..n-1 in order
 * (bonxai.hpp:449-466): a cell written several times keeps the value of the
 * highest index. was_on (optional) gets each call's return value: the cell's
 * state before that call. */
int bxg_grid_set_values(bxg_grid g, const int32_t* xyz, const void* values, size_t n,
                        uint8_t* was_on);
/* setValue batch that allocates no GPU memory (this entry point has no
 * counterpart in the reference). For callers that cannot call cudaMalloc while
 * they run -- a real-time thread, where an allocation can block for
 * milliseconds and a free synchronises the device, or a process that reserves
 * its device memory up front. Inputs must be device memory of the grid's own
 * GPU (BXG_ERR_INVALID_ARG otherwise); at most 131072 items per call (split
 * larger batches: consecutive batches give the same cells).
 * Nothing is grown: the node pools and the root hash keep the sizes they have.
 * A full leaf or inner pool returns BXG_ERR_OUT_OF_POOL; a root hash past its
 * capacity returns BXG_ERR_HASH_FULL (create the grid with hash_buckets of at
 * least twice the roots it will hold, and initial_leaves / initial_inners for
 * its leaves, or let bxg_grid_set_values grow them first). A call that fails
 * may have written part of its batch; running the same batch again (here or
 * through bxg_grid_set_values, after room is made) gives the same grid as one
 * successful call.
 * Its scratch table is a fixed 4 MiB array that each GPU loading this library
 * holds until exit and that all calls share: calls that overlap on the GPU
 * race. The first call on each device looks up that array's device address;
 * make it before any stream capture. */
int bxg_grid_set_values_noalloc(bxg_grid g, const int32_t* d_xyz, const void* d_values,
                                size_t n);
/* setValue(posToCoord(p), value) with float/double points (stride in bytes, 0 =
 * packed); the grid computes posToCoord in double. */
int bxg_grid_set_values_at_points_f32(bxg_grid g, const float* xyz, size_t stride, size_t n,
                                      const void* values);
int bxg_grid_set_values_at_points_f64(bxg_grid g, const double* xyz, size_t stride, size_t n,
                                      const void* values);

/* Accessor::value(coord, create_if_missing) (bonxai.hpp:469-494) and
 * ConstAccessor::value (bonxai.hpp:496-516): found[i] = 1 when the cell exists
 * (or was created, which sets it to T{}); out receives the value (T{} when not
 * found). Either output may be NULL. */
int bxg_grid_get_values(bxg_grid g, const int32_t* xyz, size_t n, void* out_values,
                        uint8_t* found, int create_if_missing);
/* setCellOn(coord, default_value) (bonxai.hpp:537-553). */
int bxg_grid_set_cells_on(bxg_grid g, const int32_t* xyz, size_t n, const void* default_value,
                          uint8_t* was_on);
/* setCellOff(coord) (bonxai.hpp:556-569). */
int bxg_grid_set_cells_off(bxg_grid g, const int32_t* xyz, size_t n, uint8_t* was_on);
/* The write-back half of a mutable forEachCell visitor (bonxai.hpp:194-207):
 * stores values[i] into cells that are on and leaves cells that are off (or
 * missing) untouched. */
int bxg_grid_store_if_on(bxg_grid g, const int32_t* xyz, const void* values, size_t n);
/* ConstAccessor::isCellOn(coord) (bonxai.hpp:518-534). */
int bxg_grid_is_cell_on(bxg_grid g, const int32_t* xyz, size_t n, uint8_t* out);

/* activeCellsCount() (bonxai.hpp:689-701). */
int bxg_grid_active_cells(bxg_grid g, size_t* out);
/* Node counts: roots (root map entries), inner nodes, leaves in use. */
int bxg_grid_node_counts(bxg_grid g, size_t* roots, size_t* leaves);
/* memUsage() (bonxai.hpp:649-676): device bytes held by this grid's pools. */
int bxg_grid_mem_usage(bxg_grid g, size_t* out);
/* forEachCell (bonxai.hpp:703-743) as a dump: every active cell's coordinate
 * and value, in an unspecified order (the reference's order is that of an
 * unordered_map). Writes at most cap items, *n_out = active count; returns
 * BXG_ERR_CAPACITY if cap was too small. */
int bxg_grid_dump(bxg_grid g, int32_t* out_xyz, void* out_values, size_t cap, size_t* n_out);
/* clear(CLEAR_MEMORY = 0 | SET_ALL_CELLS_OFF = 1) (bonxai.hpp:678-687). */
int bxg_grid_clear(bxg_grid g, int option);
/* releaseUnusedMemory() (bonxai.hpp:367-387): leaves with every cell off go
 * back to the pool, and roots with no leaf leave the root map. */
int bxg_grid_release_unused(bxg_grid g);
int bxg_grid_synchronize(bxg_grid g);
/* The grid's leaf pool as raw device pointers, for device-side visitors
 * (include/bonxai/device_visit.cuh): leaf l holds mask words
 * leaf_mask[l * words .. + words) (words = max(8^leaf_bits / 64, 1)), cell
 * values leaf_data[(l * 8^leaf_bits + i) * value_bytes] with i = x | y << lb |
 * z << 2lb (bonxai.hpp:441-447), and its corner coordinate
 * leaf_key[4l .. 4l+2] (leaf_key[4l+3] == -1: a free slot). Valid until the
 * next call that can grow the pools. Synchronises the grid's stream. */
typedef struct {
  unsigned long long* leaf_mask;
  unsigned char* leaf_data;
  const int32_t* leaf_key;
  uint32_t n_leaves;
  int inner_bits, leaf_bits;
  int value_bytes;
  double resolution;
  void* stream; /* cudaStream_t the grid runs on */
} bxg_device_view;
int bxg_grid_device_view(bxg_grid g, bxg_device_view* out);

/* Accessor::getLeafGrid / ConstAccessor::getLeafGrid
 * (bonxai_core/include/bonxai/bonxai.hpp:588-647) for host code: one leaf and
 * the mask of its inner node, copied to host buffers (each may be NULL).
 * inner_mask: max(2^(3*inner_bits)/64, 1) words; leaf_mask: max(2^(3*leaf_bits)/64,
 * 1) words; cells: 2^(3*leaf_bits) values of value_bytes each, x fastest (cells
 * whose mask bit is off read as zero bytes). *found: bit 0 set when the root
 * (inner node) exists, bit 1 when the leaf exists; missing parts read as zero. */
int bxg_grid_read_leaf(bxg_grid g, const int32_t xyz[3], uint64_t* inner_mask,
                       uint64_t* leaf_mask, void* cells, int* found);

/* Test hook (no counterpart in the reference): marks the leaf that would hold
 * xyz as being created by a creator that never finishes. Any later access to
 * that leaf waits out the device-side spin limit (about a second) and the call
 * returns BXG_ERR_WAIT_TIMEOUT with the handle still usable; clear() releases
 * the mark. For tests of the bounded waits only. BXG_ERR_INVALID_ARG if that
 * leaf already exists. */
int bxg_debug_hold_leaf(bxg_grid g, const int32_t xyz[3]);

/* Serialize(out, grid) (bonxai_core/include/bonxai/serialization.hpp:77-116):
 * the reference's byte format -- header line
 * "Bonxai::VoxelGrid<type_name,inner_bits,leaf_bits>(resolution)\n", uint32
 * root count, per root its key, inner mask words, and per leaf its mask words
 * and on-cell values -- with roots in ascending key order. type_name is the
 * demangled C++ type (e.g. "float"). Two-call pattern: *n_out = bytes needed;
 * BXG_ERR_CAPACITY if cap was too small. */
int bxg_grid_serialize(bxg_grid g, const char* type_name, void* out, size_t cap, size_t* n_out);
/* Deserialize (serialization.hpp:126-199) into this grid (its bits must match
 * the header's; values are set like setValue). */
int bxg_grid_deserialize(bxg_grid g, const void* data, size_t n);

/* ========================================================================
 * ProbabilisticMap  (bonxai_map/include/bonxai_map/probabilistic_map.hpp:27-137)
 * ======================================================================== */
typedef struct bxg_pmap_s* bxg_pmap;

/* Options (probabilistic_map.hpp:56-64), int32 fixed-point log-odds x 1e6. */
typedef struct {
  int32_t prob_miss_log;           /* logods(0.4f)  = -405465 */
  int32_t prob_hit_log;            /* logods(0.7f)  =  847297 */
  int32_t clamp_min_log;           /* logods(0.12f) = -1992430 */
  int32_t clamp_max_log;           /* logods(0.97f) = 3476099 */
  int32_t occupancy_threshold_log; /* logods(0.5)   = 0 */
} bxg_pmap_options;

/* ProbabilisticMap(double resolution) (probabilistic_map.hpp:68,
 * probabilistic_map.cpp:12-14), default Options, scan counter 1. */
int bxg_pmap_create(bxg_pmap* out, double resolution, const bxg_config* cfg);
int bxg_pmap_destroy(bxg_pmap m);
/* options() / setOptions() (probabilistic_map.cpp:20-28). */
int bxg_pmap_get_options(bxg_pmap m, bxg_pmap_options* out);
int bxg_pmap_set_options(bxg_pmap m, const bxg_pmap_options* opt);

/* insertPointCloud(points, origin, max_range) (probabilistic_map.hpp:141-160):
 * n points of float (or double) x,y,z with the given byte stride (0 = packed),
 * origin of the same type. Bit-exact with the reference: endpoint math in
 * double without contraction, the per-scan update_id gate, Bresenham rays that
 * include the origin cell and exclude the endpoint, one miss update per ray
 * cell per scan. Synchronous. ray_cells (optional) receives
 * V = points + sum of cast ray lengths. */
int bxg_pmap_insert_point_cloud_f32(bxg_pmap m, const float* xyz, size_t stride, size_t n,
                                    const float origin[3], double max_range,
                                    uint64_t* ray_cells);
int bxg_pmap_insert_point_cloud_f64(bxg_pmap m, const double* xyz, size_t stride, size_t n,
                                    const double origin[3], double max_range,
                                    uint64_t* ray_cells);
/* A mixed, ordered batch of addHitPoint (kinds[i] = 0) and addMissPoint
 * (kinds[i] = 1) calls: the lowest index among the points of one cell decides,
 * exactly as the calls in this order would (probabilistic_map.cpp:30-54). */
int bxg_pmap_add_points(bxg_pmap m, const double* xyz, const uint8_t* kinds, size_t n);
/* Same, asynchronous on the handle's stream: returns after enqueueing. Errors
 * of the device phases are reported by the next synchronous call or by
 * bxg_pmap_synchronize. */
int bxg_pmap_insert_point_cloud_f32_async(bxg_pmap m, const float* xyz, size_t stride,
                                          size_t n, const float origin[3], double max_range);

/* The ROS node's cloud callback (bonxai_ros/src/bonxai_server.cpp:140-182)
 * fused into one scan: n float x,y,z points in the SENSOR frame (byte stride,
 * 0 = packed), sensor_to_world a row-major 3x4 float transform [R | t].
 * Points with a non-finite coordinate are dropped (:147-154); the others are
 * transformed in float, ((r0*x + r1*y) + r2*z) + t per axis without
 * contraction (pcl::transformPointCloud, :166-168), and inserted from the
 * origin t (:171-173) as bxg_pmap_insert_point_cloud_f32 would; max_range < 0
 * means no limit (:174-179). */
int bxg_pmap_insert_sensor_cloud_f32(bxg_pmap m, const float* xyz, size_t stride, size_t n,
                                     const float sensor_to_world[12], double max_range,
                                     uint64_t* ray_cells);

/* addHitPoint / addMissPoint for n double points, in order
 * (probabilistic_map.hpp:98,103, probabilistic_map.cpp:30-54). The cells are
 * updated immediately; their rays are cast by bxg_pmap_update_free_cells. */
int bxg_pmap_add_hit_points(bxg_pmap m, const double* xyz, size_t n);
int bxg_pmap_add_miss_points(bxg_pmap m, const double* xyz, size_t n);
/* updateFreeCells(origin) (probabilistic_map.hpp:136, probabilistic_map.cpp:77-106;
 * private in the reference, public here): casts the queued rays, then
 * advances the scan counter 1 -> 2 -> 3 -> 1. ray_cells optional. */
int bxg_pmap_update_free_cells(bxg_pmap m, const double origin[3], uint64_t* ray_cells);

/* isOccupied / isUnknown / isFree (probabilistic_map.cpp:56-75) for n
 * coordinates; out[i] = 0/1. */
int bxg_pmap_is_occupied(bxg_pmap m, const int32_t* xyz, size_t n, uint8_t* out);
int bxg_pmap_is_unknown(bxg_pmap m, const int32_t* xyz, size_t n, uint8_t* out);
int bxg_pmap_is_free(bxg_pmap m, const int32_t* xyz, size_t n, uint8_t* out);
/* getOccupiedVoxels / getFreeVoxels (probabilistic_map.cpp:108-126), unordered. */
int bxg_pmap_get_occupied(bxg_pmap m, int32_t* out_xyz, size_t cap, size_t* n_out);
int bxg_pmap_get_free(bxg_pmap m, int32_t* out_xyz, size_t cap, size_t* n_out);
/* The occupied-voxel export of the ROS node (bonxai_server.cpp:217-243): the
 * PointT overload of getOccupiedVoxels (probabilistic_map.hpp:115-124), i.e.
 * corner positions double(c) * resolution, kept where min_z <= z <= max_z,
 * written as float x,y,z. out_xyz may be device memory (a headless buffer
 * that stays on the GPU) or host memory. Unordered; BXG_ERR_CAPACITY with
 * *n_out set when cap is too small. */
int bxg_pmap_export_occupied_f32(bxg_pmap m, float* out_xyz, size_t cap, size_t* n_out,
                                 double min_z, double max_z);
/* grid().forEachCell over the map (bonxai.hpp:703-743): coordinates and the
 * packed 4-byte CellT words (update_id in bits 0-3, probability_log in bits
 * 4-31, the layout GCC gives probabilistic_map.hpp:44-53). */
int bxg_pmap_dump(bxg_pmap m, int32_t* out_xyz, int32_t* out_cells, size_t cap,
                  size_t* n_out);
int bxg_pmap_active_cells(bxg_pmap m, size_t* out);
int bxg_pmap_node_counts(bxg_pmap m, size_t* roots, size_t* leaves);
int bxg_pmap_mem_usage(bxg_pmap m, size_t* out);
/* The scan counter (_update_count, probabilistic_map.hpp:129): 1, 2 or 3. */
int bxg_pmap_update_count(bxg_pmap m, int* out);
/* grid().clear(CLEAR_MEMORY): drops every cell; options and counter kept. */
int bxg_pmap_clear(bxg_pmap m);
int bxg_pmap_synchronize(bxg_pmap m);
/* Statistics of the last scan: [0] points, [1] cast rays, [2] ray cells
 * visited, [3] cells updated by rays, [4] new leaves, [5] kernel launches. */
int bxg_pmap_last_stats(bxg_pmap m, uint64_t out[8]);
/* Device time (ms) of the last isOccupied / isUnknown / isFree kernel, with
 * BXG_FLAG_TIMING (CUDA events around the kernel on the handle's stream). */
int bxg_pmap_last_query_ms(bxg_pmap m, float* ms);
/* With BXG_FLAG_TIMING: device milliseconds of each phase of the last scan,
 * measured with CUDA events on the handle's stream: [0] endpoints,
 * [1] endpoint winners, [2] endpoint update, [3] rays. */
int bxg_pmap_kernel_times(bxg_pmap m, float out[4]);
/* The CUDA stream the handle runs on (a cudaStream_t). */
void* bxg_pmap_stream(bxg_pmap m);
/* grid() (probabilistic_map.hpp:70-72): a borrowed VoxelGrid<CellT> handle
 * (value_bytes 4, the packed CellT word) over the map's own pools. Valid while
 * the map lives; never pass it to bxg_grid_destroy. */
bxg_grid bxg_pmap_grid(bxg_pmap m);

/* ========================================================================
 * Batched scans: insertPointCloud (probabilistic_map.hpp:141-160) on many
 * independent maps at once -- one scan per map per call, all maps' phases in
 * one persistent launch replayed from a CUDA graph. Each map ends bit-identical
 * to inserting its scan alone; the maps must live on the batch's device and
 * have no rays queued by bxg_pmap_add_*_points.
 * ======================================================================== */
typedef struct bxg_batch_s* bxg_batch;

/* cfg: device, rays_per_warp (1, 2 or 4) and flags (BXG_FLAG_NO_GRAPH). */
int bxg_batch_create(bxg_batch* out, const bxg_config* cfg);
int bxg_batch_destroy(bxg_batch b);
const char* bxg_batch_last_error(bxg_batch b);
/* One tick: scan s (s < n_scans <= 128) inserts points
 * xyz[3*offsets[s] .. 3*offsets[s+1]) (packed float, host or device memory)
 * into maps[s] from origins[3*s..3*s+2] with max_ranges[s]. ray_cells
 * (optional, n_scans) receives each scan's ray-cell updates. A map whose pool
 * runs out during the tick is completed by the per-map path after it grows. */
int bxg_batch_insert_f32(bxg_batch b, const bxg_pmap* maps, size_t n_scans, const float* xyz,
                         const uint64_t* offsets, const float* origins, const double* max_ranges,
                         uint64_t* ray_cells);
/* Last tick: [0] device ms, [1] ran as a CUDA graph, [2] maps completed after
 * a pool ran out, [3] ticks so far, [4] persistent grid (blocks), [5] tick
 * launches so far, [6] endpoint phase ms, [7] winner + ray phases ms. */
int bxg_batch_stats(bxg_batch b, double out[8]);
/* Last tick's phases in ms (device global timer): [0] clear, [1] endpoints,
 * [2] winners, [3] ray-list prefix, [4] rays, [5] the marking part of [4]
 * (two-phase form; 0 otherwise). */
int bxg_batch_phase_ms(bxg_batch b, double out[6]);

/* ========================================================================
 * Serving: many clients, each with a persistent map on the device, sending
 * insertPointCloud / isOccupied / getOccupiedVoxels requests
 * (probabilistic_map.hpp:91-124). A worker thread batches whatever is queued
 * into ticks (continuous batching); requests on one map run in submission
 * order and see exactly the state they would see alone. Admission: insert
 * slots and points per tick, and an HBM budget across all maps' node pools;
 * an insert that does not fit the budget waits at the head of its map's queue
 * until memory frees up (a clear of another map), and completes with
 * BXG_ERR_OUT_OF_POOL only after admission_timeout_s.
 * ======================================================================== */
typedef struct bxg_server_s* bxg_server;

typedef struct {
  size_t pool_budget_bytes;      /* across all maps' node pools; 0 = 40 GiB */
  uint32_t max_scans_per_tick;   /* insert slots per tick (<= 128); 0 = 128 */
  uint64_t max_points_per_tick;  /* 0 = 64 Mi points */
  uint64_t max_lookups_per_tick; /* 0 = 64 Mi coordinates */
  int device;                    /* -1 = current */
  uint32_t rays_per_warp;        /* batched ray kernel, 1/2/4 */
  uint32_t ray_unroll;           /* batched ray kernel, 1/2 */
  uint32_t flags;                /* BXG_FLAG_* for the maps and the batch */
  uint32_t initial_leaves;       /* per map; 0 = 4096 */
  double admission_timeout_s;    /* an insert waits this long for budget; 0 = 10 s */
} bxg_server_config;

typedef struct {
  int status;        /* bxg_status of the request */
  int kind;          /* 0 insert, 1 lookup, 2 getOccupiedVoxels, 3 clear */
  uint32_t map;
  uint64_t ray_cells;/* inserts: ray-cell updates */
  size_t n_out;      /* lookups: answers; getOccupiedVoxels: coordinates */
  double latency_ms; /* submission to completion */
  double queue_ms;   /* submission to the start of its tick */
  uint64_t tick;
} bxg_server_result;

void bxg_server_config_default(bxg_server_config* cfg);
/* One map per client, resolutions[i] for map i; starts the worker thread. */
int bxg_server_create(bxg_server* out, const double* resolutions, size_t n_maps,
                      const bxg_server_config* cfg);
/* Stops the worker after the queued requests (waits for them). */
int bxg_server_destroy(bxg_server s);
const char* bxg_server_last_error(bxg_server s);
/* Submissions copy their inputs and return a ticket. With discard != 0 the
 * result is dropped on completion (only its latency is recorded) and the
 * ticket cannot be waited for. */
int bxg_server_insert(bxg_server s, uint32_t map, const float* xyz, size_t n,
                      const float origin[3], double max_range, int discard, uint64_t* ticket);
/* mode 0 isOccupied, 1 isUnknown, 2 isFree. */
int bxg_server_query(bxg_server s, uint32_t map, const int32_t* xyz, size_t n, int mode,
                     int discard, uint64_t* ticket);
int bxg_server_get_occupied(bxg_server s, uint32_t map, int discard, uint64_t* ticket);
/* clear(CLEAR_MEMORY) of a map (bonxai_core/include/bonxai/bonxai.hpp:678-684)
 * in its request order; with release_memory the map's node pools shrink back
 * to their sizes at creation, which frees budget for waiting inserts. The
 * result's kind is 3. */
int bxg_server_clear(bxg_server s, uint32_t map, int release_memory, int discard,
                     uint64_t* ticket);
/* Waits for a ticket; copies lookup answers (cap bytes) or occupied
 * coordinates (cap coordinates) to out and releases the ticket. With
 * out == NULL a lookup or getOccupiedVoxels ticket is kept: res->n_out tells
 * the size to allocate for a second call. */
int bxg_server_wait(bxg_server s, uint64_t ticket, double timeout_s, bxg_server_result* res,
                    void* out, size_t cap);
/* Waits until every submitted request has completed. */
int bxg_server_drain(bxg_server s, double timeout_s);
/* [0] completed [1] inserts [2] lookups [3] occupied [4] ticks [5] p50 ms
 * [6] p99 ms [7] insert p50 [8] insert p99 [9] lookup p50 [10] lookup p99
 * [11] ray-cell updates [12] lookup coordinates [13] rejected [14] busy s
 * [15] first submission to last completion s [16] occupied p50 [17] occupied
 * p99 [18] pool bytes of all maps [19] insert admissions postponed for budget. */
int bxg_server_stats(bxg_server s, double out[20]);
/* The map of one client (for inspection after bxg_server_drain). */
bxg_pmap bxg_server_map(bxg_server s, uint32_t map);

/* ComputeRay(origin, end) (probabilistic_map.hpp:13-19,162-203) on the GPU for
 * n rays: out_len[i] = ray length; cells of ray i are written at
 * out_xyz[3*(offsets[i] + k)] when out_xyz != NULL, offsets = exclusive
 * prefix sum of the lengths (computed by the caller from out_len). */
int bxg_compute_rays(const int32_t* origin_xyz, const int32_t* end_xyz, size_t n,
                     uint32_t* out_len, const uint64_t* offsets, int32_t* out_xyz);

#ifdef __cplusplus
}
#endif
#endif /* BONXAI_GB300_H */
