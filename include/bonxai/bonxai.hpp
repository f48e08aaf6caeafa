// VoxelGrid<T> on one GB300, with the interface of the reference's
// bonxai_core/include/bonxai/bonxai.hpp (VoxelGrid, Accessor, ConstAccessor,
// BinaryVoxelGrid, ClearOption) so that caller code compiles unchanged.
//
// The grid lives in GPU memory (see include/bonxai_gb300.h). Two ways in:
//  * the reference's scalar calls -- Accessor::setValue / value / setCellOn /
//    setCellOff, ConstAccessor::value / isCellOn -- each one GPU round trip,
//    correct but slow;
//  * batch calls (setValues, values, setCellsOn, ...) that do a whole vector in
//    one pass: the fast path.
//
// Pointers returned by value(): the cell lives on the device, so value()
// returns a pointer to a host copy held by the accessor. Writes through it are
// stored back to the device at the accessor's next call, at flush(), or when
// the accessor is destroyed. The accessor keeps the last kSlots copies, so up
// to kSlots pointers from value() stay usable at a time (the reference's stay
// valid until the leaf is freed).
//
// forEachCell(func) copies every active cell to the host, calls func on each
// (in an unspecified order, as the reference's unordered_map gives), and
// stores back the values a mutable visitor changed (cells the visitor turned
// off through an accessor stay off).
#pragma once

#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "bonxai/grid_coord.hpp"
#include "bonxai_gb300.h"

namespace Bonxai {

// empty data structure used exclusively in BinaryVoxelGrid (bonxai.hpp:29-30)
struct EmptyVoxel {};

enum ClearOption {
  // reset the entire grid, freeing all the memory allocated so far
  CLEAR_MEMORY,
  // keep the memory allocated, but set all the cells to OFF
  SET_ALL_CELLS_OFF
};

namespace detail {
inline void check(int st, const void* h) {
  if (st != BXG_OK) {
    std::string msg = bxg_status_string(st);
    const char* e = bxg_last_error(h);
    if (e && *e) msg += std::string(": ") + e;
    throw std::runtime_error(msg);
  }
}
template <class T>
constexpr size_t value_bytes() {
  if constexpr (std::is_same_v<T, EmptyVoxel>) {
    return 0;
  } else {
    static_assert(std::is_trivially_copyable_v<T>, "DataT must be trivially copyable");
    static_assert(sizeof(T) == 1 || sizeof(T) == 2 || sizeof(T) == 4 || sizeof(T) == 8,
                  "DataT must be 1, 2, 4 or 8 bytes");
    return sizeof(T);
  }
}
}  // namespace detail

template <typename DataT>
class VoxelGrid {
 public:
  static constexpr size_t kSlots = 16;

  explicit VoxelGrid(double voxel_size, uint8_t inner_bits = 2, uint8_t leaf_bits = 3,
                     const bxg_config* cfg = nullptr)
      : inner_bits_(inner_bits),
        leaf_bits_(leaf_bits),
        resolution_(voxel_size),
        inv_resolution_(1.0 / voxel_size) {
    if (leaf_bits < 1 || inner_bits < 1) {
      throw std::runtime_error("The minimum value of the inner_bits and leaf_bits should be 1");
    }
    detail::check(bxg_grid_create(&h_, voxel_size, inner_bits, leaf_bits,
                                  detail::value_bytes<DataT>(), cfg),
                  nullptr);
  }

  // A non-owning view over an existing device grid (ProbabilisticMap::grid()).
  VoxelGrid(bxg_grid borrowed, double voxel_size)
      : h_(borrowed),
        owned_(false),
        inner_bits_(2),
        leaf_bits_(3),
        resolution_(voxel_size),
        inv_resolution_(1.0 / voxel_size) {}

  VoxelGrid(const VoxelGrid&) = delete;
  VoxelGrid& operator=(const VoxelGrid&) = delete;
  VoxelGrid(VoxelGrid&& o) noexcept { *this = std::move(o); }
  VoxelGrid& operator=(VoxelGrid&& o) noexcept {
    std::swap(h_, o.h_);
    std::swap(owned_, o.owned_);
    inner_bits_ = o.inner_bits_;
    leaf_bits_ = o.leaf_bits_;
    resolution_ = o.resolution_;
    inv_resolution_ = o.inv_resolution_;
    return *this;
  }
  ~VoxelGrid() {
    if (h_ && owned_) bxg_grid_destroy(h_);
  }

  uint32_t innetBits() const { return inner_bits_; }
  uint32_t leafBits() const { return leaf_bits_; }
  double voxelSize() const { return resolution_; }
  bxg_grid handle() const { return h_; }

  /// memUsage: device bytes held by the pools.
  size_t memUsage() const {
    size_t n = 0;
    detail::check(bxg_grid_mem_usage(h_, &n), h_);
    return n;
  }
  void releaseUnusedMemory() { detail::check(bxg_grid_release_unused(h_), h_); }
  size_t activeCellsCount() const {
    size_t n = 0;
    detail::check(bxg_grid_active_cells(h_, &n), h_);
    return n;
  }

  // bonxai.hpp:404-417
  CoordT posToCoord(double x, double y, double z) const {
    return {static_cast<int32_t>(std::floor(x * inv_resolution_)),
            static_cast<int32_t>(std::floor(y * inv_resolution_)),
            static_cast<int32_t>(std::floor(z * inv_resolution_))};
  }
  CoordT posToCoord(const Point3D& p) const { return posToCoord(p.x, p.y, p.z); }
  Point3D coordToPos(const CoordT& c) const {
    return {static_cast<double>(c.x) * resolution_, static_cast<double>(c.y) * resolution_,
            static_cast<double>(c.z) * resolution_};
  }

  // bonxai.hpp:419-447
  CoordT getRootKey(const CoordT& c) const {
    const int32_t m = ~((1 << (inner_bits_ + leaf_bits_)) - 1);
    return {c.x & m, c.y & m, c.z & m};
  }
  CoordT getInnerKey(const CoordT& c) const {
    const int32_t m = ~((1 << leaf_bits_) - 1);
    return {c.x & m, c.y & m, c.z & m};
  }
  uint32_t getInnerIndex(const CoordT& c) const {
    const int32_t im = (1 << inner_bits_) - 1;
    return uint32_t(((c.x >> leaf_bits_) & im) | (((c.y >> leaf_bits_) & im) << inner_bits_) |
                    (((c.z >> leaf_bits_) & im) << (2 * inner_bits_)));
  }
  uint32_t getLeafIndex(const CoordT& c) const {
    const int32_t lm = (1 << leaf_bits_) - 1;
    return uint32_t((c.x & lm) | ((c.y & lm) << leaf_bits_) | ((c.z & lm) << (2 * leaf_bits_)));
  }

  // ------------------------------------------------------------------ batches
  /// setValue for every item, in order (highest index wins per cell).
  void setValues(const std::vector<CoordT>& coords, const std::vector<DataT>& values,
                 std::vector<uint8_t>* was_on = nullptr) {
    static_assert(!std::is_same_v<DataT, EmptyVoxel>, "use setCellsOn");
    if (coords.size() != values.size()) throw std::runtime_error("size mismatch");
    if (was_on) was_on->assign(coords.size(), 0);
    detail::check(bxg_grid_set_values(h_, &coords[0].x, values.data(), coords.size(),
                                      was_on ? was_on->data() : nullptr),
                  h_);
  }
  /// value(coord, create) for every item.
  void values(const std::vector<CoordT>& coords, std::vector<DataT>& out,
              std::vector<uint8_t>& found, bool create_if_missing = false) {
    out.assign(coords.size(), DataT{});
    found.assign(coords.size(), 0);
    if (coords.empty()) return;
    detail::check(bxg_grid_get_values(h_, &coords[0].x, coords.size(), out.data(),
                                      found.data(), create_if_missing ? 1 : 0),
                  h_);
  }
  void setCellsOn(const std::vector<CoordT>& coords, const DataT& dflt = DataT(),
                  std::vector<uint8_t>* was_on = nullptr) {
    if (was_on) was_on->assign(coords.size(), 0);
    if (coords.empty()) return;
    detail::check(bxg_grid_set_cells_on(h_, &coords[0].x, coords.size(), &dflt,
                                        was_on ? was_on->data() : nullptr),
                  h_);
  }
  void setCellsOff(const std::vector<CoordT>& coords, std::vector<uint8_t>* was_on = nullptr) {
    if (was_on) was_on->assign(coords.size(), 0);
    if (coords.empty()) return;
    detail::check(
        bxg_grid_set_cells_off(h_, &coords[0].x, coords.size(), was_on ? was_on->data() : nullptr),
        h_);
  }
  /// Every active cell (coordinates and values), unordered.
  void dump(std::vector<CoordT>& coords, std::vector<DataT>* values = nullptr) const {
    size_t n = activeCellsCount(), got = 0;
    coords.resize(n);
    if (values) values->resize(n);
    if (n == 0) return;
    detail::check(bxg_grid_dump(h_, &coords[0].x, values ? values->data() : nullptr, n, &got),
                  h_);
    coords.resize(got);
    if (values) values->resize(got);
  }

  /// forEachCell with func(DataT&, const CoordT&) (bonxai.hpp:194-207).
  template <class VisitorFunction>
  void forEachCell(VisitorFunction func) {
    std::vector<CoordT> coords;
    if constexpr (std::is_same_v<DataT, EmptyVoxel>) {
      dump(coords);
      EmptyVoxel dummy{};
      for (const auto& c : coords) func(dummy, c);
    } else {
      std::vector<DataT> vals;
      dump(coords, &vals);
      std::vector<DataT> before = vals;
      for (size_t i = 0; i < coords.size(); i++) func(vals[i], coords[i]);
      std::vector<CoordT> wc;
      std::vector<DataT> wv;
      for (size_t i = 0; i < coords.size(); i++) {
        if (std::memcmp(&vals[i], &before[i], sizeof(DataT)) != 0) {
          wc.push_back(coords[i]);
          wv.push_back(vals[i]);
        }
      }
      if (!wc.empty())
        detail::check(bxg_grid_store_if_on(h_, &wc[0].x, wv.data(), wc.size()), h_);
    }
  }
  /// forEachCell with func(const DataT&, const CoordT&).
  template <class VisitorFunction>
  void forEachCell(VisitorFunction func) const {
    std::vector<CoordT> coords;
    if constexpr (std::is_same_v<DataT, EmptyVoxel>) {
      dump(coords);
      const EmptyVoxel dummy{};
      for (const auto& c : coords) func(dummy, c);
    } else {
      std::vector<DataT> vals;
      dump(coords, &vals);
      for (size_t i = 0; i < coords.size(); i++) func(static_cast<const DataT&>(vals[i]), coords[i]);
    }
  }

  void clear(ClearOption opt) {
    detail::check(bxg_grid_clear(h_, opt == CLEAR_MEMORY ? 0 : 1), h_);
  }

  // ---------------------------------------------------------------- accessors
  class ConstAccessor {
   public:
    ConstAccessor(const VoxelGrid& grid) : grid_(grid) {}
    ConstAccessor(const ConstAccessor&) = default;
    virtual ~ConstAccessor() = default;

    /// value(coord): pointer to a host copy of the cell, or nullptr.
    const DataT* value(const CoordT& coord) const {
      static_assert(!std::is_same_v<DataT, EmptyVoxel>,
                    "You can not access a value when using type EmptyVoxel. Use isCellOn");
      uint8_t found = 0;
      Slot& s = next_slot();
      detail::check(bxg_grid_get_values(grid_.h_, &coord.x, 1, &s.value, &found, 0), grid_.h_);
      s.coord = coord;
      s.orig = s.value;
      s.live = found != 0;
      return found ? &s.value : nullptr;
    }
    bool isCellOn(const CoordT& coord) const {
      uint8_t on = 0;
      detail::check(bxg_grid_is_cell_on(grid_.h_, &coord.x, 1, &on), grid_.h_);
      return on != 0;
    }

   protected:
    struct Slot {
      CoordT coord{0, 0, 0};
      std::conditional_t<std::is_same_v<DataT, EmptyVoxel>, int, DataT> value{};
      std::conditional_t<std::is_same_v<DataT, EmptyVoxel>, int, DataT> orig{};
      bool live = false;
    };
    Slot& next_slot() const {
      Slot& s = slots_[next_ % kSlots];
      next_++;
      return s;
    }
    const VoxelGrid& grid_;
    mutable Slot slots_[kSlots];
    mutable size_t next_ = 0;
  };

  class Accessor : public ConstAccessor {
   public:
    Accessor(VoxelGrid& grid) : ConstAccessor(grid), mgrid_(grid) {}
    Accessor(const Accessor& o) : ConstAccessor(o), mgrid_(o.mgrid_) {
      for (auto& s : this->slots_) s.live = false;
    }
    ~Accessor() override {
      try {
        flush();
      } catch (...) {
      }
    }

    /// Stores back every value changed through a pointer from value().
    void flush() {
      if constexpr (!std::is_same_v<DataT, EmptyVoxel>) {
        for (auto& s : this->slots_) {
          if (s.live && std::memcmp(&s.value, &s.orig, sizeof(DataT)) != 0) {
            detail::check(bxg_grid_store_if_on(mgrid_.h_, &s.coord.x, &s.value, 1), mgrid_.h_);
            s.orig = s.value;
          }
        }
      }
    }

    /// setValue (bonxai.hpp:449-466): returns the previous state of the cell.
    bool setValue(const CoordT& coord, const DataT& value) {
      static_assert(!std::is_same_v<DataT, EmptyVoxel>,
                    "You can not access a value when using type EmptyVoxel. Use "
                    "setCellOn / setCellOff");
      flush();
      forget(coord);
      uint8_t was = 0;
      detail::check(bxg_grid_set_values(mgrid_.h_, &coord.x, &value, 1, &was), mgrid_.h_);
      return was != 0;
    }

    /// value(coord, create_if_missing) (bonxai.hpp:469-494).
    DataT* value(const CoordT& coord, bool create_if_missing = false) {
      static_assert(!std::is_same_v<DataT, EmptyVoxel>,
                    "You can not access a value when using type EmptyVoxel. Use "
                    "isCellOn / setCellOn / setCellOff");
      flush();
      uint8_t found = 0;
      auto& s = this->next_slot();
      detail::check(bxg_grid_get_values(mgrid_.h_, &coord.x, 1, &s.value, &found,
                                        create_if_missing ? 1 : 0),
                    mgrid_.h_);
      s.coord = coord;
      s.orig = s.value;
      s.live = found != 0;
      return found ? &s.value : nullptr;
    }

    /// setCellOn (bonxai.hpp:537-553).
    bool setCellOn(const CoordT& coord, const DataT& default_value = DataT()) {
      flush();
      forget(coord);
      uint8_t was = 0;
      const void* d = nullptr;
      if constexpr (!std::is_same_v<DataT, EmptyVoxel>) d = &default_value;
      detail::check(bxg_grid_set_cells_on(mgrid_.h_, &coord.x, 1, d, &was), mgrid_.h_);
      return was != 0;
    }

    /// setCellOff (bonxai.hpp:556-569).
    bool setCellOff(const CoordT& coord) {
      flush();
      forget(coord);
      uint8_t was = 0;
      detail::check(bxg_grid_set_cells_off(mgrid_.h_, &coord.x, 1, &was), mgrid_.h_);
      return was != 0;
    }

   private:
    void forget(const CoordT& c) {
      for (auto& s : this->slots_)
        if (s.live && s.coord == c) s.live = false;
    }
    VoxelGrid& mgrid_;
  };

  Accessor createAccessor() { return Accessor(*this); }
  ConstAccessor createConstAccessor() const { return ConstAccessor(*this); }

 private:
  bxg_grid h_ = nullptr;
  bool owned_ = true;
  uint32_t inner_bits_ = 2, leaf_bits_ = 3;
  double resolution_ = 0, inv_resolution_ = 0;
};

using BinaryVoxelGrid = VoxelGrid<EmptyVoxel>;

}  // namespace Bonxai
