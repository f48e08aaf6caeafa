// VoxelGrid<T> on one GB300, with the interface of the reference's
// bonxai_core/include/bonxai/bonxai.hpp (VoxelGrid, Grid, Accessor,
// ConstAccessor, BinaryVoxelGrid, ClearOption) so that caller code compiles
// unchanged.
//
// The grid lives in GPU memory (see include/bonxai_gb300.h). Two ways in:
//  * the reference's scalar calls -- Accessor::setValue / value / setCellOn /
//    setCellOff / getLeafGrid, ConstAccessor::value / isCellOn / getLeafGrid --
//    each one GPU round trip, correct but slow;
//  * batch calls (setValues, values, setCellsOn, ...) that do a whole vector in
//    one pass: the fast path.
//
// Pointers returned by value() and getLeafGrid(): the cells live on the
// device, so an accessor hands out pointers to host copies it owns. Each
// coordinate (each leaf, for getLeafGrid) gets one copy at a fixed address, so
// the same cell always yields the same pointer, as in the reference, and the
// pointer stays valid until the accessor's releasePointers() or its end.
// Writes through a mutable pointer are stored back to the device at the
// accessor's next call, at flush(), or when the accessor ends; a call of the
// accessor re-reads the cells it returns. At most kMaxLivePointers cell copies
// and kMaxLiveLeaves leaf copies are held: a call that would need one more
// throws std::length_error (call releasePointers() to end the old ones, or use
// the batch calls); copies are never recycled behind the caller's back.
//
// rootMap() is a host snapshot of the whole tree (one download), valid until
// the next rootMap() call of this grid; it is read-only.
//
// forEachCell(func) copies every active cell to the host, calls func on each
// (in an unspecified order, as the reference's unordered_map gives), and
// stores back the values a mutable visitor changed (cells the visitor turned
// off through an accessor stay off).
#pragma once

#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#include "bonxai/grid_coord.hpp"
#include "bonxai/mask.hpp"
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

/// One node of the tree (bonxai.hpp:39-103), as a host snapshot: a mask and
/// 2^(3*log2dim) cells. InnerGrid = Grid<std::shared_ptr<LeafGrid>> holds its
/// leaves; LeafGrid = Grid<DataT> holds cell values (none for EmptyVoxel).
template <typename DataT>
class Grid {
 public:
  explicit Grid(size_t log2dim)
      : dim_(uint8_t(1u << log2dim)), mask_(log2dim) {
    if constexpr (!std::is_same_v<DataT, EmptyVoxel>) {
      size_ = uint32_t(dim_) * dim_ * dim_;
      data_.resize(size_);
    }
  }
  Grid(const Grid&) = delete;
  Grid& operator=(const Grid&) = delete;
  Grid(Grid&&) = default;
  Grid& operator=(Grid&&) = default;

  size_t memUsage() const { return sizeof(Grid) + mask_.memUsage() + data_.size() * sizeof(DataT); }
  size_t size() const { return size_; }
  Mask& mask() { return mask_; }
  const Mask& mask() const { return mask_; }
  DataT& cell(size_t index) {
    static_assert(!std::is_same_v<DataT, EmptyVoxel>,
                  "Cells have no value, when DataT == EmptyVoxel");
    return data_[index];
  }
  const DataT& cell(size_t index) const {
    static_assert(!std::is_same_v<DataT, EmptyVoxel>,
                  "Cells have no value, when DataT == EmptyVoxel");
    return data_[index];
  }

 private:
  uint8_t dim_ = 0;
  uint32_t size_ = 0;
  Mask mask_;
  std::vector<DataT> data_;
};

template <typename DataT>
class VoxelGrid {
 public:
  using LeafGrid = Grid<DataT>;
  using InnerGrid = Grid<std::shared_ptr<LeafGrid>>;
  using RootMap = std::unordered_map<CoordT, InnerGrid>;
  /// Host copies an accessor may hold at once (see the header comment).
  static constexpr size_t kMaxLivePointers = size_t(1) << 16;
  static constexpr size_t kMaxLiveLeaves = 256;

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

  /// rootMap() (bonxai.hpp:156-161): a read-only host snapshot of every root,
  /// inner node and leaf, taken by this call from one download of the pools;
  /// valid until the next rootMap() call on this grid. Callers that walk the
  /// tree (as the reference's Serialize does) use it unchanged.
  const RootMap& rootMap() const {
    size_t n = 0;
    const int st0 = bxg_grid_serialize(h_, "T", nullptr, 0, &n);  // size query
    if (st0 != BXG_OK && st0 != BXG_ERR_CAPACITY) detail::check(st0, h_);
    std::vector<char> buf(n);
    size_t got = 0;
    detail::check(bxg_grid_serialize(h_, "T", buf.data(), n, &got), h_);
    snapshot_ = std::make_shared<RootMap>();
    const char* p = static_cast<const char*>(std::memchr(buf.data(), '\n', got));
    if (!p) throw std::runtime_error("rootMap: malformed snapshot");
    ++p;
    auto take = [&](void* dst, size_t k) {
      if (p + k > buf.data() + got) throw std::runtime_error("rootMap: truncated snapshot");
      std::memcpy(dst, p, k);
      p += k;
    };
    uint32_t roots = 0;
    take(&roots, 4);
    constexpr size_t vb = detail::value_bytes<DataT>();
    for (uint32_t r = 0; r < roots; r++) {
      CoordT key{0, 0, 0};
      take(&key.x, 4);
      take(&key.y, 4);
      take(&key.z, 4);
      InnerGrid inner(inner_bits_);
      for (uint32_t w = 0; w < inner.mask().wordCount(); w++) {
        uint64_t v = 0;
        take(&v, 8);
        inner.mask().setWord(w, v);
      }
      for (auto ii = inner.mask().beginOn(); ii; ++ii) {
        auto leaf = std::make_shared<LeafGrid>(leaf_bits_);
        for (uint32_t w = 0; w < leaf->mask().wordCount(); w++) {
          uint64_t v = 0;
          take(&v, 8);
          leaf->mask().setWord(w, v);
        }
        if constexpr (vb > 0) {
          for (auto li = leaf->mask().beginOn(); li; ++li) take(&leaf->cell(*li), vb);
        }
        inner.cell(*ii) = std::move(leaf);
      }
      snapshot_->emplace(key, std::move(inner));
    }
    return *snapshot_;
  }

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
    ConstAccessor(const ConstAccessor& o) : grid_(o.grid_) {}
    virtual ~ConstAccessor() = default;

    /// value(coord) (bonxai.hpp:496-516): pointer to this accessor's host copy
    /// of the cell, or nullptr when the cell is off.
    const DataT* value(const CoordT& coord) const {
      static_assert(!std::is_same_v<DataT, EmptyVoxel>,
                    "You can not access a value when using type EmptyVoxel. Use isCellOn");
      return fetch(coord, false);
    }
    bool isCellOn(const CoordT& coord) const {
      uint8_t on = 0;
      detail::check(bxg_grid_is_cell_on(grid_.h_, &coord.x, 1, &on), grid_.h_);
      return on != 0;
    }
    /// getLeafGrid(coord) (bonxai.hpp:623-647): this accessor's host copy of
    /// the leaf holding coord, or nullptr when that leaf does not exist.
    const LeafGrid* getLeafGrid(const CoordT& coord) const { return leaf_copy(coord); }
    /// The inner node and leaf of the last getLeafGrid call (bonxai.hpp:233-243).
    /// The inner node copy holds the node's mask and the leaf last read.
    const InnerGrid* lastInnerGrid() const { return last_inner_.get(); }
    const LeafGrid* lastLeafGrid() const { return last_leaf_; }

    /// Ends every pointer this accessor handed out (and frees the copies).
    virtual void releasePointers() {
      cells_.clear();
      index_.clear();
      leaves_.clear();
      leaf_index_.clear();
      last_inner_.reset();
      last_leaf_ = nullptr;
    }

   protected:
    using V = std::conditional_t<std::is_same_v<DataT, EmptyVoxel>, int, DataT>;
    struct CellCopy {
      CoordT coord;
      V value;
      V orig;
      bool on;
    };
    struct LeafCopy {
      CoordT key;  // coordinate of the leaf's first cell
      LeafGrid now;
      LeafGrid orig;
      LeafCopy(const CoordT& k, int lb) : key(k), now(lb), orig(lb) {}
    };

    // The host copy of coord's cell, refreshed from the device; nullptr when
    // the cell is off (or was created off, see Accessor::value).
    V* fetch(const CoordT& coord, bool create) const {
      V v{};
      uint8_t found = 0;
      detail::check(bxg_grid_get_values(grid_.h_, &coord.x, 1, &v, &found, create ? 1 : 0),
                    grid_.h_);
      auto it = index_.find(coord);
      if (!found) {
        if (it != index_.end()) cells_[it->second].on = false;
        return nullptr;
      }
      CellCopy* c;
      if (it != index_.end()) {
        c = &cells_[it->second];
      } else {
        if (cells_.size() >= kMaxLivePointers)
          throw std::length_error(
              "Bonxai accessor: more than kMaxLivePointers cell pointers from value() are live; "
              "call releasePointers() or use the batch calls");
        index_.emplace(coord, cells_.size());
        cells_.push_back(CellCopy{coord, V{}, V{}, false});
        c = &cells_.back();
      }
      c->value = c->orig = v;
      c->on = true;
      return &c->value;
    }

    LeafGrid* leaf_copy(const CoordT& coord) const {
      const int lb = int(grid_.leaf_bits_), ib = int(grid_.inner_bits_);
      const CoordT key = grid_.getInnerKey(coord);
      auto inner = std::make_shared<InnerGrid>(ib);
      std::vector<uint64_t> im(inner->mask().wordCount());
      LeafGrid tmp(lb);
      std::vector<uint64_t> lm(tmp.mask().wordCount());
      constexpr size_t vb = detail::value_bytes<DataT>();
      std::vector<uint8_t> vals((size_t(1) << (3 * lb)) * (vb ? vb : 1));
      int found = 0;
      detail::check(bxg_grid_read_leaf(grid_.h_, &coord.x, im.data(), lm.data(),
                                       vb ? vals.data() : nullptr, &found),
                    grid_.h_);
      for (size_t w = 0; w < im.size(); w++) inner->mask().setWord(w, im[w]);
      last_inner_ = (found & 1) ? inner : nullptr;
      auto it = leaf_index_.find(key);
      if (!(found & 2)) {
        if (it != leaf_index_.end()) leaves_[it->second].reset();
        last_leaf_ = nullptr;
        return nullptr;
      }
      size_t slot;
      if (it != leaf_index_.end() && leaves_[it->second]) {
        slot = it->second;
      } else if (it != leaf_index_.end()) {
        slot = it->second;
        leaves_[slot] = std::make_unique<LeafCopy>(key, lb);
      } else {
        if (leaves_.size() >= kMaxLiveLeaves)
          throw std::length_error(
              "Bonxai accessor: more than kMaxLiveLeaves leaf pointers from getLeafGrid() are "
              "live; call releasePointers()");
        slot = leaves_.size();
        leaf_index_.emplace(key, slot);
        leaves_.push_back(std::make_unique<LeafCopy>(key, lb));
      }
      LeafCopy& lc = *leaves_[slot];
      for (size_t w = 0; w < lm.size(); w++) {
        lc.now.mask().setWord(w, lm[w]);
        lc.orig.mask().setWord(w, lm[w]);
      }
      if constexpr (vb > 0) {
        for (size_t i = 0; i < lc.now.size(); i++) {
          std::memcpy(&lc.now.cell(i), vals.data() + i * vb, vb);
          std::memcpy(&lc.orig.cell(i), vals.data() + i * vb, vb);
        }
      }
      last_leaf_ = &lc.now;
      return &lc.now;
    }

    const VoxelGrid& grid_;
    mutable std::deque<CellCopy> cells_;
    mutable std::unordered_map<CoordT, size_t> index_;
    mutable std::vector<std::unique_ptr<LeafCopy>> leaves_;
    mutable std::unordered_map<CoordT, size_t> leaf_index_;
    mutable std::shared_ptr<InnerGrid> last_inner_;
    mutable const LeafGrid* last_leaf_ = nullptr;
  };

  class Accessor : public ConstAccessor {
   public:
    Accessor(VoxelGrid& grid) : ConstAccessor(grid), mgrid_(grid) {}
    Accessor(const Accessor& o) : ConstAccessor(o), mgrid_(o.mgrid_) {}
    ~Accessor() override {
      try {
        flush();
      } catch (...) {
      }
    }

    /// Stores back every value changed through a pointer from value() or
    /// getLeafGrid(); the pointers stay valid.
    void flush() {
      if constexpr (!std::is_same_v<DataT, EmptyVoxel>) {
        std::vector<CoordT> wc;
        std::vector<DataT> wv;
        for (auto& c : this->cells_) {
          if (c.on && std::memcmp(&c.value, &c.orig, sizeof(DataT)) != 0) {
            wc.push_back(c.coord);
            wv.push_back(c.value);
            c.orig = c.value;
          }
        }
        if (!wc.empty())
          detail::check(bxg_grid_store_if_on(mgrid_.h_, &wc[0].x, wv.data(), wc.size()),
                        mgrid_.h_);
      }
      flush_leaves();
    }
    void releasePointers() override {
      flush();
      ConstAccessor::releasePointers();
    }

    /// setValue (bonxai.hpp:449-466): returns the previous state of the cell.
    bool setValue(const CoordT& coord, const DataT& value) {
      static_assert(!std::is_same_v<DataT, EmptyVoxel>,
                    "You can not access a value when using type EmptyVoxel. Use "
                    "setCellOn / setCellOff");
      flush();
      uint8_t was = 0;
      detail::check(bxg_grid_set_values(mgrid_.h_, &coord.x, &value, 1, &was), mgrid_.h_);
      refresh(coord);
      return was != 0;
    }

    /// value(coord, create_if_missing) (bonxai.hpp:469-494).
    DataT* value(const CoordT& coord, bool create_if_missing = false) {
      static_assert(!std::is_same_v<DataT, EmptyVoxel>,
                    "You can not access a value when using type EmptyVoxel. Use "
                    "isCellOn / setCellOn / setCellOff");
      flush();
      return this->fetch(coord, create_if_missing);
    }

    /// setCellOn (bonxai.hpp:537-553).
    bool setCellOn(const CoordT& coord, const DataT& default_value = DataT()) {
      flush();
      uint8_t was = 0;
      const void* d = nullptr;
      if constexpr (!std::is_same_v<DataT, EmptyVoxel>) d = &default_value;
      detail::check(bxg_grid_set_cells_on(mgrid_.h_, &coord.x, 1, d, &was), mgrid_.h_);
      refresh(coord);
      return was != 0;
    }

    /// setCellOff (bonxai.hpp:556-569).
    bool setCellOff(const CoordT& coord) {
      flush();
      uint8_t was = 0;
      detail::check(bxg_grid_set_cells_off(mgrid_.h_, &coord.x, 1, &was), mgrid_.h_);
      refresh(coord);
      return was != 0;
    }

    /// getLeafGrid(coord, create_if_missing) (bonxai.hpp:588-621): this
    /// accessor's host copy of the leaf; mask and cell changes made through it
    /// are stored back like value() writes. With create_if_missing a missing
    /// leaf is created with every cell off.
    LeafGrid* getLeafGrid(const CoordT& coord, bool create_if_missing = false) {
      flush();
      if (create_if_missing) {
        uint8_t was = 0;
        DataT zero{};
        const void* d = nullptr;
        if constexpr (!std::is_same_v<DataT, EmptyVoxel>) d = &zero;
        detail::check(bxg_grid_set_cells_on(mgrid_.h_, &coord.x, 1, d, &was), mgrid_.h_);
        if (!was) detail::check(bxg_grid_set_cells_off(mgrid_.h_, &coord.x, 1, nullptr), mgrid_.h_);
        refresh(coord);
      }
      return this->leaf_copy(coord);
    }

   private:
    // After a write that bypassed the copies, the copies of that cell (and of
    // its leaf) are read again so that they show the device state.
    void refresh(const CoordT& coord) {
      if constexpr (!std::is_same_v<DataT, EmptyVoxel>) {
        if (this->index_.count(coord)) this->fetch(coord, false);
      }
      const CoordT key = mgrid_.getInnerKey(coord);
      auto it = this->leaf_index_.find(key);
      if (it != this->leaf_index_.end() && this->leaves_[it->second]) this->leaf_copy(coord);
    }

    void flush_leaves() {
      constexpr size_t vb = detail::value_bytes<DataT>();
      for (auto& lp : this->leaves_) {
        if (!lp) continue;
        auto& lc = *lp;
        const int lb = int(mgrid_.leaf_bits_);
        const int32_t lmask = (1 << lb) - 1;
        std::vector<CoordT> on_c, off_c, st_c;
        std::vector<DataT> on_v, st_v;
        const uint32_t n = lc.now.mask().size();
        for (uint32_t i = 0; i < n; i++) {
          const bool a = lc.orig.mask().isOn(i), b = lc.now.mask().isOn(i);
          bool changed = false;
          if constexpr (vb > 0) changed = std::memcmp(&lc.now.cell(i), &lc.orig.cell(i), vb) != 0;
          if (a == b && !(b && changed)) continue;
          const CoordT c{lc.key.x | int32_t(i & lmask), lc.key.y | int32_t((i >> lb) & lmask),
                         lc.key.z | int32_t((i >> (2 * lb)) & lmask)};
          if (b && !a) {
            on_c.push_back(c);
            if constexpr (vb > 0) on_v.push_back(lc.now.cell(i));
          } else if (!b && a) {
            off_c.push_back(c);
          } else {
            st_c.push_back(c);
            if constexpr (vb > 0) st_v.push_back(lc.now.cell(i));
          }
        }
        for (size_t k = 0; k < on_c.size(); k++) {
          const void* d = nullptr;
          if constexpr (vb > 0) d = &on_v[k];
          detail::check(bxg_grid_set_cells_on(mgrid_.h_, &on_c[k].x, 1, d, nullptr), mgrid_.h_);
          if constexpr (vb > 0)
            detail::check(bxg_grid_store_if_on(mgrid_.h_, &on_c[k].x, &on_v[k], 1), mgrid_.h_);
        }
        if (!off_c.empty())
          detail::check(bxg_grid_set_cells_off(mgrid_.h_, &off_c[0].x, off_c.size(), nullptr),
                        mgrid_.h_);
        if constexpr (vb > 0) {
          if (!st_c.empty())
            detail::check(bxg_grid_store_if_on(mgrid_.h_, &st_c[0].x, st_v.data(), st_c.size()),
                          mgrid_.h_);
        }
        for (uint32_t w = 0; w < lc.now.mask().wordCount(); w++)
          lc.orig.mask().setWord(w, lc.now.mask().getWord(w));
        if constexpr (vb > 0)
          for (size_t i = 0; i < lc.now.size(); i++) lc.orig.cell(i) = lc.now.cell(i);
      }
    }
    VoxelGrid& mgrid_;
  };

  Accessor createAccessor() { return Accessor(*this); }
  ConstAccessor createConstAccessor() const { return ConstAccessor(*this); }

 private:
  mutable std::shared_ptr<RootMap> snapshot_;
  bxg_grid h_ = nullptr;
  bool owned_ = true;
  uint32_t inner_bits_ = 2, leaf_bits_ = 3;
  double resolution_ = 0, inv_resolution_ = 0;
};

using BinaryVoxelGrid = VoxelGrid<EmptyVoxel>;

}  // namespace Bonxai
