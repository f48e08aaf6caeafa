// ProbabilisticMap on one GB300, with the interface of the reference's
// bonxai_map/include/bonxai_map/probabilistic_map.hpp so that caller code
// (e.g. a ROS node calling insertPointCloud with a pcl cloud, or a KITTI
// driver with Eigen points) compiles unchanged and gets bit-identical maps.
//
// Differences a caller can see:
//  * updateFreeCells is public (the reference declares it private yet asks
//    callers of addHitPoint/addMissPoint to call it).
//  * addHitPoint/addMissPoint calls are buffered on the host in call order and
//    sent as one ordered batch before the next operation that could observe
//    them, which gives the same cells as immediate updates.
//  * Points with a NaN or infinite coordinate are dropped by insertPointCloud
//    (the reference's own ROS node filters them before calling it); a config
//    flag keeps them.
//  * grid() is a VoxelGrid<CellT> view of the map's device pools.
//  * Vector3D is Eigen::Vector3d when Eigen is available, else Point3D; every
//    entry point accepts any xyz type.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <type_traits>
#include <vector>

#include "bonxai/bonxai.hpp"

#if defined(__has_include)
#if __has_include(<eigen3/Eigen/Geometry>) && !defined(BONXAI_GB300_NO_EIGEN)
#include <eigen3/Eigen/Geometry>
#define BONXAI_GB300_HAVE_EIGEN 1
#endif
#endif

namespace Bonxai {

template <class Functor>
void RayIterator(const CoordT& key_origin, const CoordT& key_end, const Functor& func);

inline void ComputeRay(const CoordT& key_origin, const CoordT& key_end, std::vector<CoordT>& ray) {
  ray.clear();
  RayIterator(key_origin, key_end, [&ray](const CoordT& coord) {
    ray.push_back(coord);
    return true;
  });
}

class ProbabilisticMap {
 public:
#ifdef BONXAI_GB300_HAVE_EIGEN
  using Vector3D = Eigen::Vector3d;
#else
  using Vector3D = Point3D;
#endif

  /// log-odds as int32 fixed point x 1e6 (probabilistic_map.hpp:31-36)
  [[nodiscard]] static int32_t logods(float prob) {
    return int32_t(1e6 * std::log(prob / (1.0 - prob)));
  }
  /// inverse of logods (probabilistic_map.hpp:38-42)
  [[nodiscard]] static float prob(int32_t logods_fixed) {
    float l = float(logods_fixed) * 1e-6;
    return (1.0 - 1.0 / (1.0 + std::exp(l)));
  }

  /// The packed 4-byte cell (probabilistic_map.hpp:44-53); the device stores
  /// exactly this layout.
  struct CellT {
    int32_t update_id : 4;
    int32_t probability_log : 28;
    CellT() : update_id(0), probability_log(0) {}
  };
  static_assert(sizeof(int32_t) == 4, "");

  /// OctoMap defaults (probabilistic_map.hpp:55-64).
  struct Options {
    int32_t prob_miss_log = logods(0.4f);
    int32_t prob_hit_log = logods(0.7f);
    int32_t clamp_min_log = logods(0.12f);
    int32_t clamp_max_log = logods(0.97f);
    int32_t occupancy_threshold_log = logods(0.5);
  };

  static inline const int32_t UnknownProbability = 0;

  explicit ProbabilisticMap(double resolution, const bxg_config* cfg = nullptr)
      : resolution_(resolution) {
    detail::check(bxg_pmap_create(&h_, resolution, cfg), nullptr);
    grid_ = VoxelGrid<CellT>(bxg_pmap_grid(h_), resolution);
  }
  ProbabilisticMap(const ProbabilisticMap&) = delete;
  ProbabilisticMap& operator=(const ProbabilisticMap&) = delete;
  ~ProbabilisticMap() {
    if (h_) bxg_pmap_destroy(h_);
  }

  [[nodiscard]] VoxelGrid<CellT>& grid() {
    flush();
    return grid_;
  }
  [[nodiscard]] const VoxelGrid<CellT>& grid() const {
    const_cast<ProbabilisticMap*>(this)->flush();
    return grid_;
  }
  bxg_pmap handle() const { return h_; }

  [[nodiscard]] const Options& options() const { return options_; }
  void setOptions(const Options& o) {
    flush();
    options_ = o;
    bxg_pmap_options d{o.prob_miss_log, o.prob_hit_log, o.clamp_min_log, o.clamp_max_log,
                       o.occupancy_threshold_log};
    detail::check(bxg_pmap_set_options(h_, &d), h_);
  }

  /// insertPointCloud (probabilistic_map.hpp:91-93,141-160).
  template <typename PointT, typename Allocator>
  void insertPointCloud(const std::vector<PointT, Allocator>& points, const PointT& origin,
                        double max_range) {
    flush();
    using S = detail::scalar_t<PointT>;
    if constexpr (std::is_same_v<S, float>) {
      std::vector<float> xyz(points.size() * 3);
      for (size_t i = 0; i < points.size(); i++) {
        const auto p = ConvertPoint<Point3D>(points[i]);  // exact: float -> double
        xyz[3 * i] = float(p.x);
        xyz[3 * i + 1] = float(p.y);
        xyz[3 * i + 2] = float(p.z);
      }
      const auto o = ConvertPoint<Point3D>(origin);
      const float of[3] = {float(o.x), float(o.y), float(o.z)};
      detail::check(bxg_pmap_insert_point_cloud_f32(h_, xyz.data(), 0, points.size(), of,
                                                    max_range, &last_ray_cells_),
                    h_);
    } else {
      std::vector<double> xyz(points.size() * 3);
      for (size_t i = 0; i < points.size(); i++) {
        const auto p = ConvertPoint<Point3D>(points[i]);
        xyz[3 * i] = p.x;
        xyz[3 * i + 1] = p.y;
        xyz[3 * i + 2] = p.z;
      }
      const auto o = ConvertPoint<Point3D>(origin);
      const double od[3] = {o.x, o.y, o.z};
      detail::check(bxg_pmap_insert_point_cloud_f64(h_, xyz.data(), 0, points.size(), od,
                                                    max_range, &last_ray_cells_),
                    h_);
    }
  }

  /// Batch form: n packed float xyz points (host or device memory).
  void insertPointCloud(const float* xyz, size_t n, const float origin[3], double max_range) {
    flush();
    detail::check(
        bxg_pmap_insert_point_cloud_f32(h_, xyz, 0, n, origin, max_range, &last_ray_cells_), h_);
  }

  /// The ROS node's cloud callback (bonxai_server.cpp:140-182) as one scan:
  /// float points in the sensor frame and the sensor-to-world transform as
  /// any 4x4 or 3x4 matrix type with operator()(row, col) (Eigen::Matrix4f
  /// works). Non-finite points are dropped, the rest transformed in float on
  /// the GPU, the origin is the translation, max_range < 0 means no limit.
  template <typename PointT, typename Allocator, typename Matrix>
  void insertSensorCloud(const std::vector<PointT, Allocator>& sensor_points,
                         const Matrix& sensor_to_world, double max_range) {
    std::vector<float> xyz(sensor_points.size() * 3);
    for (size_t i = 0; i < sensor_points.size(); i++) {
      const auto p = ConvertPoint<Point3D>(sensor_points[i]);
      xyz[3 * i] = float(p.x);
      xyz[3 * i + 1] = float(p.y);
      xyz[3 * i + 2] = float(p.z);
    }
    float m[12];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 4; c++) m[4 * r + c] = float(sensor_to_world(r, c));
    insertSensorCloud(xyz.data(), sensor_points.size(), m, max_range);
  }
  /// Batch form: n packed float xyz points (host or device memory) and a
  /// row-major 3x4 transform.
  void insertSensorCloud(const float* xyz, size_t n, const float sensor_to_world[12],
                         double max_range) {
    flush();
    detail::check(bxg_pmap_insert_sensor_cloud_f32(h_, xyz, 0, n, sensor_to_world, max_range,
                                                   &last_ray_cells_),
                  h_);
  }

  /// addHitPoint / addMissPoint (probabilistic_map.hpp:95-103).
  template <typename V>
  void addHitPoint(const V& point) {
    push(ConvertPoint<Point3D>(point), 0);
  }
  template <typename V>
  void addMissPoint(const V& point) {
    push(ConvertPoint<Point3D>(point), 1);
  }

  /// updateFreeCells (probabilistic_map.hpp:136; private in the reference).
  template <typename V>
  void updateFreeCells(const V& origin) {
    flush();
    const auto o = ConvertPoint<Point3D>(origin);
    const double od[3] = {o.x, o.y, o.z};
    detail::check(bxg_pmap_update_free_cells(h_, od, &last_ray_cells_), h_);
  }

  [[nodiscard]] bool isOccupied(const CoordT& coord) const { return query1(coord, 0); }
  [[nodiscard]] bool isUnknown(const CoordT& coord) const { return query1(coord, 1); }
  [[nodiscard]] bool isFree(const CoordT& coord) const { return query1(coord, 2); }

  /// Batch forms: out[i] = 0/1.
  void isOccupied(const std::vector<CoordT>& c, std::vector<uint8_t>& out) const {
    queryN(c, out, 0);
  }
  void isUnknown(const std::vector<CoordT>& c, std::vector<uint8_t>& out) const {
    queryN(c, out, 1);
  }
  void isFree(const std::vector<CoordT>& c, std::vector<uint8_t>& out) const {
    queryN(c, out, 2);
  }

  void getOccupiedVoxels(std::vector<CoordT>& coords) { collect(coords, true); }
  void getFreeVoxels(std::vector<CoordT>& coords) { collect(coords, false); }

  template <typename PointT>
  void getOccupiedVoxels(std::vector<PointT>& points) {
    std::vector<CoordT> coords;
    getOccupiedVoxels(coords);
    for (const auto& c : coords) {
      const auto p = grid_.coordToPos(c);
      points.emplace_back(p.x, p.y, p.z);
    }
  }

  /// The ROS node's occupied-voxel export (bonxai_server.cpp:217-243) on the
  /// GPU: corner positions of occupied cells with min_z <= z <= max_z as
  /// float xyz into out_xyz (host or device memory, cap points). Returns the
  /// number of such cells; throws if it exceeds cap.
  size_t exportOccupied(float* out_xyz, size_t cap, double min_z, double max_z) {
    flush();
    size_t n = 0;
    detail::check(bxg_pmap_export_occupied_f32(h_, out_xyz, cap, &n, min_z, max_z), h_);
    return n;
  }
  /// Number of occupied cells in the z band (no output written).
  size_t countOccupied(double min_z, double max_z) {
    flush();
    size_t n = 0;
    const int st = bxg_pmap_export_occupied_f32(h_, nullptr, 0, &n, min_z, max_z);
    if (st != BXG_OK && st != BXG_ERR_CAPACITY) detail::check(st, h_);
    return n;
  }

  /// Ray-cell updates of the last insertPointCloud (points + ray cells) or
  /// updateFreeCells (ray cells).
  uint64_t lastRayCells() const { return last_ray_cells_; }

 private:
  void push(const Point3D& p, uint8_t kind) {
    pend_xyz_.push_back(p.x);
    pend_xyz_.push_back(p.y);
    pend_xyz_.push_back(p.z);
    pend_kind_.push_back(kind);
  }
  void flush() {
    if (pend_kind_.empty()) return;
    const int st = bxg_pmap_add_points(h_, pend_xyz_.data(), pend_kind_.data(), pend_kind_.size());
    pend_xyz_.clear();
    pend_kind_.clear();
    detail::check(st, h_);
  }
  bool query1(const CoordT& c, int mode) const {
    const_cast<ProbabilisticMap*>(this)->flush();
    uint8_t r = 0;
    int st = mode == 0   ? bxg_pmap_is_occupied(h_, &c.x, 1, &r)
             : mode == 1 ? bxg_pmap_is_unknown(h_, &c.x, 1, &r)
                         : bxg_pmap_is_free(h_, &c.x, 1, &r);
    detail::check(st, h_);
    return r != 0;
  }
  void queryN(const std::vector<CoordT>& c, std::vector<uint8_t>& out, int mode) const {
    const_cast<ProbabilisticMap*>(this)->flush();
    out.assign(c.size(), 0);
    if (c.empty()) return;
    int st = mode == 0   ? bxg_pmap_is_occupied(h_, &c[0].x, c.size(), out.data())
             : mode == 1 ? bxg_pmap_is_unknown(h_, &c[0].x, c.size(), out.data())
                         : bxg_pmap_is_free(h_, &c[0].x, c.size(), out.data());
    detail::check(st, h_);
  }
  void collect(std::vector<CoordT>& coords, bool occupied) {
    flush();
    coords.clear();
    size_t n = 0;
    int st = occupied ? bxg_pmap_get_occupied(h_, nullptr, 0, &n)
                      : bxg_pmap_get_free(h_, nullptr, 0, &n);
    if (st != BXG_OK && st != BXG_ERR_CAPACITY) detail::check(st, h_);
    coords.resize(n);
    if (n == 0) return;
    size_t got = 0;
    st = occupied ? bxg_pmap_get_occupied(h_, &coords[0].x, n, &got)
                  : bxg_pmap_get_free(h_, &coords[0].x, n, &got);
    detail::check(st, h_);
    coords.resize(got);
  }

  bxg_pmap h_ = nullptr;
  double resolution_;
  Options options_;
  VoxelGrid<CellT> grid_{nullptr, 1.0};
  std::vector<double> pend_xyz_;
  std::vector<uint8_t> pend_kind_;
  uint64_t last_ray_cells_ = 0;
};

/// RayIterator (probabilistic_map.hpp:162-203) on the host, for callers that
/// walk single rays: visits the origin and the next max-1 Bresenham cells
/// (the end cell is excluded; nothing when origin == end). The device kernels
/// walk the same cells in closed form.
template <class Functor>
inline void RayIterator(const CoordT& key_origin, const CoordT& key_end, const Functor& func) {
  if (key_origin == key_end) return;
  if (!func(key_origin)) return;
  const CoordT d0 = key_end - key_origin;
  const int32_t ax = d0.x < 0 ? -d0.x : d0.x, ay = d0.y < 0 ? -d0.y : d0.y,
                az = d0.z < 0 ? -d0.z : d0.z;
  const int32_t m = std::max(std::max(ax, ay), az);
  const int64_t two_m = 2 * int64_t(m);
  for (int32_t k = 1; k < m; ++k) {
    const CoordT c{
        key_origin.x + (d0.x < 0 ? -1 : 1) * int32_t((2 * int64_t(k) * ax + m) / two_m),
        key_origin.y + (d0.y < 0 ? -1 : 1) * int32_t((2 * int64_t(k) * ay + m) / two_m),
        key_origin.z + (d0.z < 0 ? -1 : 1) * int32_t((2 * int64_t(k) * az + m) / two_m)};
    if (!func(c)) return;
  }
}

}  // namespace Bonxai
