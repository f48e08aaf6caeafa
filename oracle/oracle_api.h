/*
 * C API of the CPU oracle (test infrastructure only; never shipped).
 *
 * Two libraries implement it with the same symbols:
 *   - oracle/_build/liboracle_port.so: this project's own C++ restatement of the
 *     reference algorithm (oracle/bonxai_oracle.cpp). It builds anywhere gcc
 *     exists and is the checker used by the GPU parity tests, smoke() and the
 *     CPU-baseline leg of bench.py.
 *   - oracle/_ref/liboracle_ref.so: the reference's own headers and
 *     probabilistic_map.cpp compiled unmodified behind this API
 *     (oracle/ref_harness.cpp). It only builds where the reference sources are
 *     mounted; it pins the restatement and generates tests/golden/ fixtures.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may load these.
 */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Grid value types accepted by orc_grid_create. */
enum { ORC_F32 = 0, ORC_I32 = 1, ORC_U32 = 2, ORC_F64 = 3, ORC_I64 = 4 };

/* ---------------- ProbabilisticMap ---------------- */
void* orc_pmap_create(double resolution);
void orc_pmap_destroy(void* m);
/* options[5] = {prob_miss_log, prob_hit_log, clamp_min_log, clamp_max_log,
 *               occupancy_threshold_log} */
void orc_pmap_get_options(void* m, int32_t* options);
void orc_pmap_set_options(void* m, const int32_t* options);
int orc_pmap_update_count(void* m);
/* insertPointCloud over n packed xyz points with an origin of the same type.
 * Returns the ray-cell update count V = n + sum of cast ray lengths. */
uint64_t orc_pmap_insert_f32(void* m, const float* xyz, size_t n, const float* origin,
                             double max_range);
uint64_t orc_pmap_insert_f64(void* m, const double* xyz, size_t n, const double* origin,
                             double max_range);
void orc_pmap_add_hit(void* m, const double* xyz, size_t n);
void orc_pmap_add_miss(void* m, const double* xyz, size_t n);
/* Returns the number of ray cells visited. */
uint64_t orc_pmap_update_free_cells(void* m, const double* origin);
size_t orc_pmap_cell_count(void* m);
/* Writes every active cell (any order) as xyz and the packed 4-byte cell word:
 * bits 0-3 update_id, bits 4-31 probability_log. Returns the count written. */
size_t orc_pmap_dump(void* m, int32_t* xyz, int32_t* packed, size_t cap);
/* occupied/unknown/free per coordinate (any pointer may be NULL). */
void orc_pmap_query(void* m, const int32_t* xyz, size_t n, uint8_t* occ, uint8_t* unk,
                    uint8_t* fre);
size_t orc_pmap_get_occupied(void* m, int32_t* xyz, size_t cap);
size_t orc_pmap_get_free(void* m, int32_t* xyz, size_t cap);
/* getOccupiedVoxels(std::vector<PointT>&) (probabilistic_map.hpp:115-124)
 * filtered to min_z <= z <= max_z and narrowed to float, as the ROS node
 * publishes it (bonxai_server.cpp:217-243). Any order; returns the count. */
size_t orc_pmap_export_occupied_f32(void* m, double min_z, double max_z, float* xyz,
                                    size_t cap);
/* Restatement of the ROS node's ingest (bonxai_server.cpp:147-168): drops
 * non-finite points and applies a row-major 3x4 float transform. Port
 * library only (the node and PCL are not part of the compiled reference). */
size_t orc_sensor_to_world_f32(const float* m12, const float* xyz, size_t n, float* out);

/* ---------------- VoxelGrid<T> ---------------- */
void* orc_grid_create(double voxel_size, int inner_bits, int leaf_bits, int dtype);
void orc_grid_destroy(void* g);
void orc_grid_pos_to_coord(void* g, const double* xyz, size_t n, int32_t* out);
/* setValue for each item in order; was_on may be NULL. */
void orc_grid_set_values(void* g, const int32_t* xyz, const void* values, size_t n,
                         uint8_t* was_on);
/* Accessor::value(coord, create) for each item in order. */
void orc_grid_get_values(void* g, const int32_t* xyz, size_t n, void* out, uint8_t* found,
                         int create);
void orc_grid_set_cells_on(void* g, const int32_t* xyz, size_t n, const void* default_value,
                           uint8_t* was_on);
void orc_grid_set_cells_off(void* g, const int32_t* xyz, size_t n, uint8_t* was_on);
void orc_grid_is_cell_on(void* g, const int32_t* xyz, size_t n, uint8_t* out);
size_t orc_grid_active_cells(void* g);
size_t orc_grid_leaf_count(void* g);
size_t orc_grid_root_count(void* g);
size_t orc_grid_dump(void* g, int32_t* xyz, void* values, size_t cap);
void orc_grid_clear(void* g, int option);
void orc_grid_release_unused(void* g);

/* ---------------- rays ---------------- */
/* ComputeRay(origin, end): writes up to cap cells, returns the ray length. */
size_t orc_compute_ray(const int32_t* origin, const int32_t* end, int32_t* out, size_t cap);

#ifdef __cplusplus
}
#endif
