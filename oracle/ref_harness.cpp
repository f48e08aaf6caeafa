/*
 * Harness that exposes the reference's own code behind oracle_api.h
 * (test infrastructure only; never shipped).
 *
 * Built by oracle/build_ref.sh from the unmodified reference headers
 * (bonxai_core/include/bonxai/*.hpp, bonxai_map/include/bonxai_map/
 * probabilistic_map.hpp) and bonxai_map/src/probabilistic_map.cpp, plus the
 * repo-authored Eigen shim. Output goes to oracle/_ref/ only.
 *
 * Two deliberate choices:
 *  - Queries use a ConstAccessor over grid() and the predicates of
 *    probabilistic_map.cpp:56-75, not ProbabilisticMap::isOccupied, because the
 *    latter caches a null leaf pointer in the accessor that addHitPoint shares
 *    (bonxai.hpp:478-481, probabilistic_map.cpp:32-34) and a later insert into
 *    that leaf dereferences it.
 *  - updateFreeCells and the hit/miss lists are private; the harness opens them
 *    with an access macro so that it can count the ray cells of each scan. The
 *    scan itself is always the reference's insertPointCloud
 *    (probabilistic_map.hpp:141-160); the count is taken from a second path
 *    that calls the reference's addHitPoint/addMissPoint/updateFreeCells in the
 *    same order, and tests check both paths leave identical maps.
 */
#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <iostream>
#include <limits>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

#define private public
#include "bonxai/bonxai.hpp"
#include "bonxai/serialization.hpp"
#include "bonxai_map/probabilistic_map.hpp"
#undef private

#include "oracle_api.h"

using Bonxai::CoordT;
using Bonxai::ProbabilisticMap;

namespace {

struct F3 {
  float x, y, z;
};
struct D3 {
  double x, y, z;
};

struct RefPMap {
  explicit RefPMap(double res) : map(res) {}
  ProbabilisticMap map;
};

inline int32_t pack_cell(const ProbabilisticMap::CellT& c) {
  int32_t w;
  static_assert(sizeof(c) == 4, "CellT must be 4 bytes");
  std::memcpy(&w, &c, 4);
  return w;
}

template <typename PT>
uint64_t count_and_insert(ProbabilisticMap& map, const std::vector<PT>& pts, const PT& origin,
                          double max_range) {
  // Same order of operations as probabilistic_map.hpp:141-160, calling the
  // reference's addHitPoint / addMissPoint / updateFreeCells.
  using V3 = ProbabilisticMap::Vector3D;
  const auto from = Bonxai::ConvertPoint<V3>(origin);
  const double max_range_sqr = max_range * max_range;
  for (const auto& point : pts) {
    const auto to = Bonxai::ConvertPoint<V3>(point);
    V3 vect(to - from);
    const double squared_norm = vect.squaredNorm();
    if (squared_norm >= max_range_sqr) {
      const V3 new_point = from + ((vect / std::sqrt(squared_norm)) * max_range);
      map.addMissPoint(new_point);
    } else {
      map.addHitPoint(to);
    }
  }
  uint64_t v = pts.size();
  const CoordT o = map._grid.posToCoord(from);
  for (const auto* list : {&map._hit_coords, &map._miss_coords}) {
    for (const auto& e : *list) {
      if (e == o) continue;
      const int64_t dx = std::abs(int64_t(e.x) - o.x), dy = std::abs(int64_t(e.y) - o.y),
                    dz = std::abs(int64_t(e.z) - o.z);
      v += uint64_t(std::max(dx, std::max(dy, dz)));
    }
  }
  map.updateFreeCells(from);
  return v;
}

// ---------------- VoxelGrid<T> behind a type-erased interface ----------------
struct GridBase {
  virtual ~GridBase() = default;
  virtual void pos_to_coord(const double* xyz, size_t n, int32_t* out) = 0;
  virtual void set_values(const int32_t* xyz, const void* v, size_t n, uint8_t* was_on) = 0;
  virtual void get_values(const int32_t* xyz, size_t n, void* out, uint8_t* found,
                          int create) = 0;
  virtual void set_on(const int32_t* xyz, size_t n, const void* dflt, uint8_t* was_on) = 0;
  virtual void set_off(const int32_t* xyz, size_t n, uint8_t* was_on) = 0;
  virtual void is_on(const int32_t* xyz, size_t n, uint8_t* out) = 0;
  virtual size_t active() = 0;
  virtual size_t leaves() = 0;
  virtual size_t roots() = 0;
  virtual size_t dump(int32_t* xyz, void* v, size_t cap) = 0;
  virtual void clear(int opt) = 0;
  virtual void release() = 0;
  virtual std::string serialize() = 0;
};

template <typename T>
struct RefGrid : GridBase {
  using Acc = typename Bonxai::VoxelGrid<T>::Accessor;
  RefGrid(double res, int ib, int lb)
      : grid(res, uint8_t(ib), uint8_t(lb)), accp(new Acc(grid.createAccessor())) {}
  Bonxai::VoxelGrid<T> grid;
  std::unique_ptr<Acc> accp;
  Acc& acc_() { return *accp; }

  static CoordT C(const int32_t* p) { return CoordT{p[0], p[1], p[2]}; }

  void pos_to_coord(const double* xyz, size_t n, int32_t* out) override {
    for (size_t i = 0; i < n; i++) {
      const CoordT c = grid.posToCoord(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
      out[3 * i] = c.x;
      out[3 * i + 1] = c.y;
      out[3 * i + 2] = c.z;
    }
  }
  void set_values(const int32_t* xyz, const void* v, size_t n, uint8_t* was_on) override {
    const T* vals = static_cast<const T*>(v);
    for (size_t i = 0; i < n; i++) {
      const bool w = acc_().setValue(C(xyz + 3 * i), vals[i]);
      if (was_on) was_on[i] = w;
    }
  }
  void get_values(const int32_t* xyz, size_t n, void* out, uint8_t* found, int create) override {
    T* o = static_cast<T*>(out);
    for (size_t i = 0; i < n; i++) {
      T* p = acc_().value(C(xyz + 3 * i), create != 0);
      if (found) found[i] = p != nullptr;
      if (o) o[i] = p ? *p : T{};
    }
  }
  void set_on(const int32_t* xyz, size_t n, const void* dflt, uint8_t* was_on) override {
    const T d = *static_cast<const T*>(dflt);
    for (size_t i = 0; i < n; i++) {
      const bool w = acc_().setCellOn(C(xyz + 3 * i), d);
      if (was_on) was_on[i] = w;
    }
  }
  void set_off(const int32_t* xyz, size_t n, uint8_t* was_on) override {
    for (size_t i = 0; i < n; i++) {
      const bool w = acc_().setCellOff(C(xyz + 3 * i));
      if (was_on) was_on[i] = w;
    }
  }
  void is_on(const int32_t* xyz, size_t n, uint8_t* out) override {
    auto ca = grid.createConstAccessor();
    for (size_t i = 0; i < n; i++) out[i] = ca.isCellOn(C(xyz + 3 * i));
  }
  size_t active() override { return grid.activeCellsCount(); }
  size_t leaves() override {
    size_t n = 0;
    for (const auto& kv : grid.rootMap()) n += kv.second.mask().countOn();
    return n;
  }
  size_t roots() override { return grid.rootMap().size(); }
  size_t dump(int32_t* xyz, void* v, size_t cap) override {
    T* vals = static_cast<T*>(v);
    size_t k = 0;
    grid.forEachCell([&](const T& val, const CoordT& c) {
      if (k < cap) {
        xyz[3 * k] = c.x;
        xyz[3 * k + 1] = c.y;
        xyz[3 * k + 2] = c.z;
        if (vals) vals[k] = val;
      }
      k++;
    });
    return k;
  }
  void clear(int opt) override {
    grid.clear(opt == 0 ? Bonxai::CLEAR_MEMORY : Bonxai::SET_ALL_CELLS_OFF);
    accp.reset(new Acc(grid.createAccessor()));
  }
  void release() override {
    grid.releaseUnusedMemory();
    accp.reset(new Acc(grid.createAccessor()));
  }
  std::string serialize() override {
    std::ostringstream os(std::ios::binary);
    Bonxai::Serialize(os, grid);
    return os.str();
  }
};

}  // namespace

extern "C" {

void* orc_pmap_create(double resolution) { return new RefPMap(resolution); }
void orc_pmap_destroy(void* m) { delete static_cast<RefPMap*>(m); }

void orc_pmap_get_options(void* m, int32_t* o) {
  const auto& op = static_cast<RefPMap*>(m)->map.options();
  o[0] = op.prob_miss_log;
  o[1] = op.prob_hit_log;
  o[2] = op.clamp_min_log;
  o[3] = op.clamp_max_log;
  o[4] = op.occupancy_threshold_log;
}

void orc_pmap_set_options(void* m, const int32_t* o) {
  ProbabilisticMap::Options op;
  op.prob_miss_log = o[0];
  op.prob_hit_log = o[1];
  op.clamp_min_log = o[2];
  op.clamp_max_log = o[3];
  op.occupancy_threshold_log = o[4];
  static_cast<RefPMap*>(m)->map.setOptions(op);
}

int orc_pmap_update_count(void* m) { return static_cast<RefPMap*>(m)->map._update_count; }

uint64_t orc_pmap_insert_f32(void* m, const float* xyz, size_t n, const float* origin,
                             double max_range) {
  std::vector<F3> pts(n);
  std::memcpy(pts.data(), xyz, n * sizeof(F3));
  const F3 o{origin[0], origin[1], origin[2]};
  return count_and_insert(static_cast<RefPMap*>(m)->map, pts, o, max_range);
}

uint64_t orc_pmap_insert_f64(void* m, const double* xyz, size_t n, const double* origin,
                             double max_range) {
  std::vector<D3> pts(n);
  std::memcpy(pts.data(), xyz, n * sizeof(D3));
  const D3 o{origin[0], origin[1], origin[2]};
  return count_and_insert(static_cast<RefPMap*>(m)->map, pts, o, max_range);
}

/* The reference's own insertPointCloud, unchanged (no count). */
void orc_ref_insert_point_cloud_f32(void* m, const float* xyz, size_t n, const float* origin,
                                    double max_range) {
  std::vector<F3> pts(n);
  std::memcpy(pts.data(), xyz, n * sizeof(F3));
  const F3 o{origin[0], origin[1], origin[2]};
  static_cast<RefPMap*>(m)->map.insertPointCloud(pts, o, max_range);
}

void orc_pmap_add_hit(void* m, const double* xyz, size_t n) {
  for (size_t i = 0; i < n; i++) {
    static_cast<RefPMap*>(m)->map.addHitPoint({xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
  }
}

void orc_pmap_add_miss(void* m, const double* xyz, size_t n) {
  for (size_t i = 0; i < n; i++) {
    static_cast<RefPMap*>(m)->map.addMissPoint({xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
  }
}

uint64_t orc_pmap_update_free_cells(void* m, const double* origin) {
  auto& map = static_cast<RefPMap*>(m)->map;
  const ProbabilisticMap::Vector3D from(origin[0], origin[1], origin[2]);
  const CoordT o = map._grid.posToCoord(from);
  uint64_t v = 0;
  for (const auto* list : {&map._hit_coords, &map._miss_coords}) {
    for (const auto& e : *list) {
      if (e == o) continue;
      const int64_t dx = std::abs(int64_t(e.x) - o.x), dy = std::abs(int64_t(e.y) - o.y),
                    dz = std::abs(int64_t(e.z) - o.z);
      v += uint64_t(std::max(dx, std::max(dy, dz)));
    }
  }
  map.updateFreeCells(from);
  return v;
}

size_t orc_pmap_cell_count(void* m) {
  return static_cast<RefPMap*>(m)->map.grid().activeCellsCount();
}

size_t orc_pmap_dump(void* m, int32_t* xyz, int32_t* packed, size_t cap) {
  size_t k = 0;
  static_cast<RefPMap*>(m)->map.grid().forEachCell(
      [&](const ProbabilisticMap::CellT& c, const CoordT& p) {
        if (k < cap) {
          xyz[3 * k] = p.x;
          xyz[3 * k + 1] = p.y;
          xyz[3 * k + 2] = p.z;
          packed[k] = pack_cell(c);
        }
        k++;
      });
  return k;
}

void orc_pmap_query(void* m, const int32_t* xyz, size_t n, uint8_t* occ, uint8_t* unk,
                    uint8_t* fre) {
  auto& map = static_cast<RefPMap*>(m)->map;
  const int32_t thr = map.options().occupancy_threshold_log;
  auto ca = map.grid().createConstAccessor();
  for (size_t i = 0; i < n; i++) {
    const auto* c = ca.value(CoordT{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
    if (occ) occ[i] = c ? (c->probability_log > thr) : 0;
    if (unk) unk[i] = c ? (c->probability_log == thr) : 1;
    if (fre) fre[i] = c ? (c->probability_log < thr) : 0;
  }
}

static size_t copy_coords(const std::vector<CoordT>& v, int32_t* xyz, size_t cap) {
  for (size_t k = 0; k < v.size() && k < cap; k++) {
    xyz[3 * k] = v[k].x;
    xyz[3 * k + 1] = v[k].y;
    xyz[3 * k + 2] = v[k].z;
  }
  return v.size();
}

size_t orc_pmap_get_occupied(void* m, int32_t* xyz, size_t cap) {
  std::vector<CoordT> v;
  static_cast<RefPMap*>(m)->map.getOccupiedVoxels(v);
  return copy_coords(v, xyz, cap);
}

size_t orc_pmap_export_occupied_f32(void* m, double min_z, double max_z, float* xyz,
                                    size_t cap) {
  // the reference's PointT overload (coordToPos), then the node's z band
  std::vector<ProbabilisticMap::Vector3D> v;
  static_cast<RefPMap*>(m)->map.getOccupiedVoxels(v);
  size_t k = 0;
  for (const auto& p : v) {
    if (!(p.z() >= min_z && p.z() <= max_z)) continue;
    if (k < cap) {
      xyz[3 * k] = float(p.x());
      xyz[3 * k + 1] = float(p.y());
      xyz[3 * k + 2] = float(p.z());
    }
    k++;
  }
  return k;
}

size_t orc_pmap_get_free(void* m, int32_t* xyz, size_t cap) {
  std::vector<CoordT> v;
  static_cast<RefPMap*>(m)->map.getFreeVoxels(v);
  return copy_coords(v, xyz, cap);
}

void* orc_grid_create(double voxel_size, int ib, int lb, int dtype) {
  switch (dtype) {
    case ORC_F32: return static_cast<GridBase*>(new RefGrid<float>(voxel_size, ib, lb));
    case ORC_I32: return static_cast<GridBase*>(new RefGrid<int32_t>(voxel_size, ib, lb));
    case ORC_U32: return static_cast<GridBase*>(new RefGrid<uint32_t>(voxel_size, ib, lb));
    case ORC_F64: return static_cast<GridBase*>(new RefGrid<double>(voxel_size, ib, lb));
    case ORC_I64: return static_cast<GridBase*>(new RefGrid<int64_t>(voxel_size, ib, lb));
    default: return nullptr;
  }
}
void orc_grid_destroy(void* g) { delete static_cast<GridBase*>(g); }
void orc_grid_pos_to_coord(void* g, const double* xyz, size_t n, int32_t* out) {
  static_cast<GridBase*>(g)->pos_to_coord(xyz, n, out);
}
void orc_grid_set_values(void* g, const int32_t* xyz, const void* v, size_t n, uint8_t* w) {
  static_cast<GridBase*>(g)->set_values(xyz, v, n, w);
}
void orc_grid_get_values(void* g, const int32_t* xyz, size_t n, void* out, uint8_t* found,
                         int create) {
  static_cast<GridBase*>(g)->get_values(xyz, n, out, found, create);
}
void orc_grid_set_cells_on(void* g, const int32_t* xyz, size_t n, const void* d, uint8_t* w) {
  static_cast<GridBase*>(g)->set_on(xyz, n, d, w);
}
void orc_grid_set_cells_off(void* g, const int32_t* xyz, size_t n, uint8_t* w) {
  static_cast<GridBase*>(g)->set_off(xyz, n, w);
}
void orc_grid_is_cell_on(void* g, const int32_t* xyz, size_t n, uint8_t* out) {
  static_cast<GridBase*>(g)->is_on(xyz, n, out);
}
size_t orc_grid_active_cells(void* g) { return static_cast<GridBase*>(g)->active(); }
size_t orc_grid_leaf_count(void* g) { return static_cast<GridBase*>(g)->leaves(); }
size_t orc_grid_root_count(void* g) { return static_cast<GridBase*>(g)->roots(); }
size_t orc_grid_dump(void* g, int32_t* xyz, void* v, size_t cap) {
  return static_cast<GridBase*>(g)->dump(xyz, v, cap);
}
void orc_grid_clear(void* g, int opt) { static_cast<GridBase*>(g)->clear(opt); }
void orc_grid_release_unused(void* g) { static_cast<GridBase*>(g)->release(); }

/* Reference-only: Bonxai::Serialize of a grid or of a map's grid
 * (serialization.hpp:77-116). Returns the byte count; writes up to cap. */
size_t orc_ref_grid_serialize(void* g, char* out, size_t cap) {
  const std::string s = static_cast<GridBase*>(g)->serialize();
  if (out) std::memcpy(out, s.data(), std::min(cap, s.size()));
  return s.size();
}
size_t orc_ref_pmap_serialize(void* m, char* out, size_t cap) {
  std::ostringstream os(std::ios::binary);
  Bonxai::Serialize(os, static_cast<RefPMap*>(m)->map.grid());
  const std::string s = os.str();
  if (out) std::memcpy(out, s.data(), std::min(cap, s.size()));
  return s.size();
}

size_t orc_compute_ray(const int32_t* o, const int32_t* e, int32_t* out, size_t cap) {
  std::vector<CoordT> ray;
  Bonxai::ComputeRay(CoordT{o[0], o[1], o[2]}, CoordT{e[0], e[1], e[2]}, ray);
  return copy_coords(ray, out, cap);
}

}  // extern "C"
