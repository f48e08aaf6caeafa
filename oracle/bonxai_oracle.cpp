/*
 * CPU oracle: a restatement of the reference's sparse voxel grid and
 * probabilistic-map scan, written for this project (test infrastructure only).
 *
 * It is the checker for the CUDA path (tests/, __graft_entry__.smoke()) and
 * the CPU baseline timed by bench.py. Nothing shipped links it. It is pinned
 * against the reference's own code in two ways: tests/golden/ fixtures made by
 * the reference compiled unmodified (oracle/_ref), and, where the reference
 * sources are mounted, direct comparison on random cases.
 *
 * The data structure follows the reference one-to-one so that the CPU timing
 * is representative: a hash map from root key to an inner node, inner nodes of
 * (2^inner_bits)^3 leaf pointers with a bit mask, leaves of (2^leaf_bits)^3
 * cells with a bit mask, and an accessor with a one-entry leaf cache.
 * Citations are reference paths relative to the reference repository root.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <unordered_map>
#include <vector>

#include "oracle_api.h"

namespace orc {

struct Coord {
  int32_t x, y, z;
  bool operator==(const Coord& o) const { return x == o.x && y == o.y && z == o.z; }
  bool operator!=(const Coord& o) const { return !(*this == o); }
};

struct CoordHash {
  // Any hash gives the same map contents; iteration order is never compared.
  size_t operator()(const Coord& c) const {
    uint64_t h = uint64_t(uint32_t(c.x)) * 0x9E3779B97F4A7C15ull;
    h ^= uint64_t(uint32_t(c.y)) * 0xC2B2AE3D27D4EB4Full + (h >> 29);
    h ^= uint64_t(uint32_t(c.z)) * 0x165667B19E3779F9ull + (h >> 31);
    return size_t(h ^ (h >> 32));
  }
};

// Bit set of 2^(3*log2dim) bits in 64-bit words (mask.hpp:19-140,255-263).
// Up to eight words (leaf_bits <= 3, every inner node of inner_bits <= 3) live
// inside the object, as the reference's Mask keeps them, so a mask test costs
// no pointer chase; larger masks live on the heap.
class Bits {
 public:
  explicit Bits(int log2dim)
      : nbits_(1u << (3 * log2dim)), nw_(std::max<uint32_t>(nbits_ >> 6, 1u)) {
    if (nw_ > kInline) big_.assign(nw_, 0);
  }
  bool on(uint32_t i) const { return (w()[i >> 6] >> (i & 63)) & 1u; }
  // setOn / setOff return the previous state (mask.hpp:351-365).
  bool set_on(uint32_t i) {
    uint64_t& x = w()[i >> 6];
    const uint64_t b = uint64_t(1) << (i & 63);
    const bool was = x & b;
    x |= b;
    return was;
  }
  bool set_off(uint32_t i) {
    uint64_t& x = w()[i >> 6];
    const uint64_t b = uint64_t(1) << (i & 63);
    const bool was = x & b;
    x &= ~b;
    return was;
  }
  uint32_t count() const {
    uint32_t n = 0;
    for (uint32_t k = 0; k < nw_; k++) n += uint32_t(__builtin_popcountll(w()[k]));
    return n;
  }
  bool none() const {
    for (uint32_t k = 0; k < nw_; k++)
      if (w()[k]) return false;
    return true;
  }
  // Calls f(i) for every set bit, lowest first (mask.hpp:154-253).
  template <class F>
  void for_each(F&& f) const {
    for (uint32_t k = 0; k < nw_; k++) {
      uint64_t x = w()[k];
      while (x) {
        const uint32_t b = uint32_t(__builtin_ctzll(x));
        f((k << 6) + b);
        x &= x - 1;
      }
    }
  }
  void clear() { std::fill(w(), w() + nw_, uint64_t(0)); }

 private:
  static constexpr uint32_t kInline = 8;
  uint64_t* w() { return nw_ <= kInline ? inl_ : big_.data(); }
  const uint64_t* w() const { return nw_ <= kInline ? inl_ : big_.data(); }
  uint32_t nbits_, nw_;
  uint64_t inl_[kInline] = {0, 0, 0, 0, 0, 0, 0, 0};
  std::vector<uint64_t> big_;
};

template <class T>
struct Leaf {
  explicit Leaf(int lb) : bits(lb), cells(size_t(1) << (3 * lb)) {}
  Bits bits;
  std::vector<T> cells;
};

template <class T>
struct Inner {
  explicit Inner(int ib) : bits(ib), child(size_t(1) << (3 * ib)) {}
  Bits bits;
  std::vector<std::unique_ptr<Leaf<T>>> child;
};

// VoxelGrid<T> (bonxai.hpp:114-333).
template <class T>
class Grid {
 public:
  Grid(double res, int ib, int lb)
      : ib_(ib), lb_(lb), res_(res), inv_res_(1.0 / res),  // bonxai.hpp:390-398
        inner_mask_((1 << ib) - 1), leaf_mask_((1 << lb) - 1) {}

  double resolution() const { return res_; }

  // posToCoord: floor(x * inv_resolution) in double (bonxai.hpp:404-410).
  Coord pos_to_coord(double x, double y, double z) const {
    return {int32_t(std::floor(x * inv_res_)), int32_t(std::floor(y * inv_res_)),
            int32_t(std::floor(z * inv_res_))};
  }
  // getRootKey / getInnerKey / getInnerIndex / getLeafIndex (bonxai.hpp:419-447).
  Coord root_key(const Coord& c) const {
    const int32_t m = ~((1 << (ib_ + lb_)) - 1);
    return {c.x & m, c.y & m, c.z & m};
  }
  Coord leaf_key(const Coord& c) const {
    const int32_t m = ~((1 << lb_) - 1);
    return {c.x & m, c.y & m, c.z & m};
  }
  uint32_t inner_index(const Coord& c) const {
    return uint32_t(((c.x >> lb_) & inner_mask_) | (((c.y >> lb_) & inner_mask_) << ib_) |
                    (((c.z >> lb_) & inner_mask_) << (2 * ib_)));
  }
  uint32_t leaf_index(const Coord& c) const {
    return uint32_t((c.x & leaf_mask_) | ((c.y & leaf_mask_) << lb_) |
                    ((c.z & leaf_mask_) << (2 * lb_)));
  }

  // Accessor::getLeafGrid (bonxai.hpp:588-621). The caller's one-entry root
  // cache (*rk_cache, *in_cache) skips the hash lookup while consecutive
  // leaves share a root; node addresses of the unordered_map are stable until
  // an erase, and every erase path resets the accessors.
  Leaf<T>* leaf(const Coord& c, bool create, Coord* rk_cache = nullptr,
                Inner<T>** in_cache = nullptr) {
    const Coord rk = root_key(c);
    Inner<T>* inp = nullptr;
    if (in_cache && *in_cache && *rk_cache == rk) {
      inp = *in_cache;
    } else {
      auto it = roots_.find(rk);
      if (it == roots_.end()) {
        if (!create) return nullptr;
        it = roots_.emplace(rk, Inner<T>(ib_)).first;
      }
      inp = &it->second;
      if (in_cache) {
        *in_cache = inp;
        *rk_cache = rk;
      }
    }
    Inner<T>& in = *inp;
    const uint32_t ii = inner_index(c);
    if (create) {
      if (!in.bits.set_on(ii)) in.child[ii].reset(new Leaf<T>(lb_));
    } else if (!in.bits.on(ii)) {
      return nullptr;
    }
    return in.child[ii].get();
  }

  // forEachCell (bonxai.hpp:703-743): coordinate rebuilt from root, inner and
  // leaf indices.
  template <class F>
  void for_each(F&& f) {
    for (auto& kv : roots_) {
      const Coord& r = kv.first;
      Inner<T>& in = kv.second;
      in.bits.for_each([&](uint32_t ii) {
        const int32_t xb = r.x | int32_t((ii & inner_mask_) << lb_);
        const int32_t yb = r.y | int32_t(((ii >> ib_) & inner_mask_) << lb_);
        const int32_t zb = r.z | int32_t(((ii >> (2 * ib_)) & inner_mask_) << lb_);
        Leaf<T>& lf = *in.child[ii];
        lf.bits.for_each([&](uint32_t li) {
          const Coord c{xb | int32_t(li & leaf_mask_), yb | int32_t((li >> lb_) & leaf_mask_),
                        zb | int32_t((li >> (2 * lb_)) & leaf_mask_)};
          f(lf.cells[li], c);
        });
      });
    }
  }

  size_t active() {
    size_t n = 0;
    for (auto& kv : roots_)
      kv.second.bits.for_each([&](uint32_t ii) { n += kv.second.child[ii]->bits.count(); });
    return n;
  }
  size_t leaves() {
    size_t n = 0;
    for (auto& kv : roots_) n += kv.second.bits.count();
    return n;
  }
  size_t roots() const { return roots_.size(); }
  void clear_memory() { roots_.clear(); }  // clear(CLEAR_MEMORY), bonxai.hpp:678-684
  // releaseUnusedMemory (bonxai.hpp:367-387).
  void release_unused() {
    for (auto it = roots_.begin(); it != roots_.end();) {
      Inner<T>& in = it->second;
      std::vector<uint32_t> drop;
      in.bits.for_each([&](uint32_t ii) {
        if (in.child[ii]->bits.none()) drop.push_back(ii);
      });
      for (uint32_t ii : drop) {
        in.bits.set_off(ii);
        in.child[ii].reset();
      }
      if (in.bits.none()) {
        it = roots_.erase(it);
      } else {
        ++it;
      }
    }
  }

 private:
  int ib_, lb_;
  double res_, inv_res_;
  int32_t inner_mask_, leaf_mask_;
  std::unordered_map<Coord, Inner<T>, CoordHash> roots_;
};

// Accessor with the one-entry leaf cache of bonxai.hpp:449-569.
template <class T>
class Access {
 public:
  explicit Access(Grid<T>& g) : g_(g) {}
  void reset() {
    has_ = false;
    leaf_ = nullptr;
    inner_ = nullptr;
  }
  // The cache test is inline; the lookup behind it is out of line, as the
  // reference keeps getLeafGrid behind its inline key comparison
  // (bonxai.hpp:476-481).
  Leaf<T>* leaf_for(const Coord& c, bool create) {
    const Coord k = g_.leaf_key(c);
    if (has_ && k == key_ && !(create && leaf_ == nullptr)) return leaf_;
    return refill(c, k, create);
  }
  // setValue (bonxai.hpp:449-466): returns the previous on-state.
  bool set_value(const Coord& c, const T& v) {
    Leaf<T>* lf = leaf_for(c, true);
    const uint32_t i = g_.leaf_index(c);
    const bool was = lf->bits.set_on(i);
    lf->cells[i] = v;
    return was;
  }
  // value(coord, create) (bonxai.hpp:469-494): a created cell holds T{}.
  T* value(const Coord& c, bool create) {
    Leaf<T>* lf = leaf_for(c, create);
    if (!lf) return nullptr;
    const uint32_t i = g_.leaf_index(c);
    if (lf->bits.on(i)) return &lf->cells[i];
    if (!create) return nullptr;
    lf->bits.set_on(i);
    lf->cells[i] = T{};
    return &lf->cells[i];
  }
  // setCellOn (bonxai.hpp:537-553): the default is written only when created.
  bool set_on(const Coord& c, const T& dflt) {
    Leaf<T>* lf = leaf_for(c, true);
    const uint32_t i = g_.leaf_index(c);
    const bool was = lf->bits.set_on(i);
    if (!was) lf->cells[i] = dflt;
    return was;
  }
  // setCellOff (bonxai.hpp:556-569): the content is kept.
  bool set_off(const Coord& c) {
    Leaf<T>* lf = leaf_for(c, false);
    if (!lf) return false;
    return lf->bits.set_off(g_.leaf_index(c));
  }

 private:
  __attribute__((noinline)) Leaf<T>* refill(const Coord& c, const Coord& k, bool create) {
    leaf_ = g_.leaf(c, create, &root_, &inner_);
    key_ = k;
    has_ = true;
    return leaf_;
  }

  Grid<T>& g_;
  bool has_ = false;
  Coord key_{0, 0, 0};
  Leaf<T>* leaf_ = nullptr;
  Coord root_{0, 0, 0};
  Inner<T>* inner_ = nullptr;
};

// RayIterator (probabilistic_map.hpp:162-203): integer 3D Bresenham that visits
// the origin and then max-1 further cells; the end cell is never visited and
// no cell is visited when origin == end. Per step the x, y, z errors are
// tested in that order with (error << 1) >= max.
template <class F>
void walk_ray(const Coord& o, const Coord& e, F&& f) {
  if (o == e) return;
  f(o);
  const int32_t dx0 = e.x - o.x, dy0 = e.y - o.y, dz0 = e.z - o.z;
  const int32_t sx = dx0 < 0 ? -1 : 1, sy = dy0 < 0 ? -1 : 1, sz = dz0 < 0 ? -1 : 1;
  const int32_t dx = dx0 < 0 ? -dx0 : dx0, dy = dy0 < 0 ? -dy0 : dy0,
                dz = dz0 < 0 ? -dz0 : dz0;
  const int32_t m = std::max(std::max(dx, dy), dz);
  int32_t ex = 0, ey = 0, ez = 0;
  Coord c = o;
  for (int32_t i = 0; i < m - 1; ++i) {
    ex += dx;
    ey += dy;
    ez += dz;
    if ((ex << 1) >= m) {
      c.x += sx;
      ex -= m;
    }
    if ((ey << 1) >= m) {
      c.y += sy;
      ey -= m;
    }
    if ((ez << 1) >= m) {
      c.z += sz;
      ez -= m;
    }
    f(c);
  }
}

inline int64_t chebyshev(const Coord& a, const Coord& b) {
  const int64_t dx = std::llabs(int64_t(b.x) - a.x), dy = std::llabs(int64_t(b.y) - a.y),
                dz = std::llabs(int64_t(b.z) - a.z);
  return std::max(dx, std::max(dy, dz));
}

// Packed cell word, laid out as GCC lays out ProbabilisticMap::CellT
// {int32_t update_id : 4; int32_t probability_log : 28;}
// (probabilistic_map.hpp:44-53): update_id in bits 0-3, probability_log in
// bits 4-31, both signed.
inline int32_t cell_id(int32_t w) { return int32_t(uint32_t(w) << 28) >> 28; }
inline int32_t cell_prob(int32_t w) { return w >> 4; }
inline int32_t cell_pack(int32_t prob, int32_t id) {
  return int32_t((uint32_t(prob) << 4) | (uint32_t(id) & 0xFu));
}
inline int32_t wrap_add(int32_t a, int32_t b) { return int32_t(uint32_t(a) + uint32_t(b)); }

// ProbabilisticMap (probabilistic_map.hpp:27-137, probabilistic_map.cpp).
class PMap {
 public:
  explicit PMap(double res) : grid_(res, 2, 3), acc_(grid_) {}

  // Default options: logods(0.4f), logods(0.7f), logods(0.12f), logods(0.97f),
  // logods(0.5) with logods(p) = int32_t(1e6 * log(p / (1.0 - p)))
  // (probabilistic_map.hpp:34-36,56-64).
  static int32_t logods(float p) { return int32_t(1e6 * std::log(p / (1.0 - p))); }
  int32_t miss = logods(0.4f), hit = logods(0.7f), cmin = logods(0.12f),
          cmax = logods(0.97f), thr = logods(0.5f);
  int update_count = 1;

  // addHitPoint / addMissPoint (probabilistic_map.cpp:30-54): the endpoint is
  // updated and queued for a ray only if it was not already updated in this
  // scan.
  void add_point(double x, double y, double z, bool is_hit) {
    const Coord c = grid_.pos_to_coord(x, y, z);
    int32_t* w = acc_.value(c, true);
    if (cell_id(*w) != update_count) {
      const int32_t p = cell_prob(*w);
      const int32_t np = is_hit ? std::min(wrap_add(p, hit), cmax)
                                : std::max(wrap_add(p, miss), cmin);
      *w = cell_pack(np, update_count);
      (is_hit ? hits_ : misses_).push_back(c);
    }
  }

  // updateFreeCells (probabilistic_map.cpp:77-106): rays from the origin cell
  // to every queued endpoint, hits then misses; each ray cell is created and
  // gets one miss update per scan; then the scan counter cycles 1 -> 2 -> 3 -> 1.
  uint64_t update_free_cells(double ox, double oy, double oz) {
    Access<int32_t> acc(grid_);
    const Coord o = grid_.pos_to_coord(ox, oy, oz);
    // a ray visits chebyshev(o, e) cells (none when e == o), so the count of
    // visited cells is summed per ray rather than per cell
    uint64_t visited = 0;
    auto clear_point = [&](const Coord& c) {
      int32_t* w = acc.value(c, true);
      if (cell_id(*w) != update_count) {
        *w = cell_pack(std::max(wrap_add(cell_prob(*w), miss), cmin), update_count);
      }
    };
    for (const Coord& e : hits_) {
      visited += uint64_t(chebyshev(o, e));
      walk_ray(o, e, clear_point);
    }
    hits_.clear();
    for (const Coord& e : misses_) {
      visited += uint64_t(chebyshev(o, e));
      walk_ray(o, e, clear_point);
    }
    misses_.clear();
    if (++update_count == 4) update_count = 1;
    return visited;
  }

  // insertPointCloud (probabilistic_map.hpp:141-160), all in double:
  // vect = to - from; |vect|^2 = (x*x + y*y) + z*z; a point at or beyond
  // max_range becomes a miss at from + (vect / sqrt(|vect|^2)) * max_range.
  template <class P>
  uint64_t insert(const P* pts, size_t n, const P* origin, double max_range) {
    const double fx = double(origin[0]), fy = double(origin[1]), fz = double(origin[2]);
    const double mr2 = max_range * max_range;
    for (size_t i = 0; i < n; i++) {
      const double tx = double(pts[3 * i]), ty = double(pts[3 * i + 1]),
                   tz = double(pts[3 * i + 2]);
      const double vx = tx - fx, vy = ty - fy, vz = tz - fz;
      const double xy = vx * vx + vy * vy;
      const double sq = xy + vz * vz;
      if (sq >= mr2) {
        const double s = std::sqrt(sq);
        add_point(fx + ((vx / s) * max_range), fy + ((vy / s) * max_range),
                  fz + ((vz / s) * max_range), false);
      } else {
        add_point(tx, ty, tz, true);
      }
    }
    return uint64_t(n) + update_free_cells(fx, fy, fz);
  }

  Grid<int32_t>& grid() { return grid_; }
  void invalidate_cache() { acc_.reset(); }

 private:
  Grid<int32_t> grid_;
  Access<int32_t> acc_;
  std::vector<Coord> hits_, misses_;
};

// Type-erased grid for the C API.
struct GridIf {
  virtual ~GridIf() = default;
  virtual void pos_to_coord(const double* xyz, size_t n, int32_t* out) = 0;
  virtual void set_values(const int32_t* xyz, const void* v, size_t n, uint8_t* w) = 0;
  virtual void get_values(const int32_t* xyz, size_t n, void* out, uint8_t* f, int cr) = 0;
  virtual void set_on(const int32_t* xyz, size_t n, const void* d, uint8_t* w) = 0;
  virtual void set_off(const int32_t* xyz, size_t n, uint8_t* w) = 0;
  virtual void is_on(const int32_t* xyz, size_t n, uint8_t* out) = 0;
  virtual size_t active() = 0;
  virtual size_t leaves() = 0;
  virtual size_t roots() = 0;
  virtual size_t dump(int32_t* xyz, void* v, size_t cap) = 0;
  virtual void clear(int opt) = 0;
  virtual void release() = 0;
};

template <class T>
struct GridImpl : GridIf {
  GridImpl(double r, int ib, int lb) : g(r, ib, lb), a(g) {}
  Grid<T> g;
  Access<T> a;
  static Coord C(const int32_t* p) { return {p[0], p[1], p[2]}; }
  void pos_to_coord(const double* xyz, size_t n, int32_t* out) override {
    for (size_t i = 0; i < n; i++) {
      const Coord c = g.pos_to_coord(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
      out[3 * i] = c.x;
      out[3 * i + 1] = c.y;
      out[3 * i + 2] = c.z;
    }
  }
  void set_values(const int32_t* xyz, const void* v, size_t n, uint8_t* w) override {
    const T* vals = static_cast<const T*>(v);
    for (size_t i = 0; i < n; i++) {
      const bool was = a.set_value(C(xyz + 3 * i), vals[i]);
      if (w) w[i] = was;
    }
  }
  void get_values(const int32_t* xyz, size_t n, void* out, uint8_t* f, int cr) override {
    T* o = static_cast<T*>(out);
    for (size_t i = 0; i < n; i++) {
      T* p = a.value(C(xyz + 3 * i), cr != 0);
      if (f) f[i] = p != nullptr;
      if (o) o[i] = p ? *p : T{};
    }
  }
  void set_on(const int32_t* xyz, size_t n, const void* d, uint8_t* w) override {
    const T dv = *static_cast<const T*>(d);
    for (size_t i = 0; i < n; i++) {
      const bool was = a.set_on(C(xyz + 3 * i), dv);
      if (w) w[i] = was;
    }
  }
  void set_off(const int32_t* xyz, size_t n, uint8_t* w) override {
    for (size_t i = 0; i < n; i++) {
      const bool was = a.set_off(C(xyz + 3 * i));
      if (w) w[i] = was;
    }
  }
  void is_on(const int32_t* xyz, size_t n, uint8_t* out) override {
    for (size_t i = 0; i < n; i++) {
      Leaf<T>* lf = g.leaf(C(xyz + 3 * i), false);
      out[i] = lf ? lf->bits.on(g.leaf_index(C(xyz + 3 * i))) : 0;
    }
  }
  size_t active() override { return g.active(); }
  size_t leaves() override { return g.leaves(); }
  size_t roots() override { return g.roots(); }
  size_t dump(int32_t* xyz, void* v, size_t cap) override {
    T* vals = static_cast<T*>(v);
    size_t k = 0;
    g.for_each([&](const T& val, const Coord& c) {
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
  // clear(SET_ALL_CELLS_OFF) turns every cell off and keeps the nodes
  // (bonxai.hpp:685-686).
  void clear(int opt) override {
    if (opt == 0) {
      g.clear_memory();
    } else {
      std::vector<Coord> on;
      g.for_each([&](const T&, const Coord& c) { on.push_back(c); });
      for (const Coord& c : on) a.set_off(c);
    }
    a.reset();
  }
  void release() override {
    g.release_unused();
    a.reset();
  }
};

}  // namespace orc

using orc::Coord;

extern "C" {

void* orc_pmap_create(double resolution) { return new orc::PMap(resolution); }
void orc_pmap_destroy(void* m) { delete static_cast<orc::PMap*>(m); }
void orc_pmap_get_options(void* m, int32_t* o) {
  auto* p = static_cast<orc::PMap*>(m);
  o[0] = p->miss;
  o[1] = p->hit;
  o[2] = p->cmin;
  o[3] = p->cmax;
  o[4] = p->thr;
}
void orc_pmap_set_options(void* m, const int32_t* o) {
  auto* p = static_cast<orc::PMap*>(m);
  p->miss = o[0];
  p->hit = o[1];
  p->cmin = o[2];
  p->cmax = o[3];
  p->thr = o[4];
}
int orc_pmap_update_count(void* m) { return static_cast<orc::PMap*>(m)->update_count; }
uint64_t orc_pmap_insert_f32(void* m, const float* xyz, size_t n, const float* origin,
                             double max_range) {
  return static_cast<orc::PMap*>(m)->insert(xyz, n, origin, max_range);
}
uint64_t orc_pmap_insert_f64(void* m, const double* xyz, size_t n, const double* origin,
                             double max_range) {
  return static_cast<orc::PMap*>(m)->insert(xyz, n, origin, max_range);
}
void orc_pmap_add_hit(void* m, const double* xyz, size_t n) {
  for (size_t i = 0; i < n; i++)
    static_cast<orc::PMap*>(m)->add_point(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], true);
}
void orc_pmap_add_miss(void* m, const double* xyz, size_t n) {
  for (size_t i = 0; i < n; i++)
    static_cast<orc::PMap*>(m)->add_point(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], false);
}
uint64_t orc_pmap_update_free_cells(void* m, const double* o) {
  return static_cast<orc::PMap*>(m)->update_free_cells(o[0], o[1], o[2]);
}
size_t orc_pmap_cell_count(void* m) { return static_cast<orc::PMap*>(m)->grid().active(); }
size_t orc_pmap_dump(void* m, int32_t* xyz, int32_t* packed, size_t cap) {
  size_t k = 0;
  static_cast<orc::PMap*>(m)->grid().for_each([&](const int32_t& w, const Coord& c) {
    if (k < cap) {
      xyz[3 * k] = c.x;
      xyz[3 * k + 1] = c.y;
      xyz[3 * k + 2] = c.z;
      packed[k] = w;
    }
    k++;
  });
  return k;
}
// isOccupied / isUnknown / isFree (probabilistic_map.cpp:56-75): a missing cell
// is unknown.
void orc_pmap_query(void* m, const int32_t* xyz, size_t n, uint8_t* occ, uint8_t* unk,
                    uint8_t* fre) {
  auto* p = static_cast<orc::PMap*>(m);
  auto& g = p->grid();
  for (size_t i = 0; i < n; i++) {
    const Coord c{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    orc::Leaf<int32_t>* lf = g.leaf(c, false);
    const uint32_t li = g.leaf_index(c);
    const bool have = lf && lf->bits.on(li);
    const int32_t pr = have ? orc::cell_prob(lf->cells[li]) : 0;
    if (occ) occ[i] = have && pr > p->thr;
    if (unk) unk[i] = have ? pr == p->thr : 1;
    if (fre) fre[i] = have && pr < p->thr;
  }
}
// getOccupiedVoxels / getFreeVoxels (probabilistic_map.cpp:108-126).
static size_t pmap_filter(void* m, int32_t* xyz, size_t cap, int sign) {
  auto* p = static_cast<orc::PMap*>(m);
  size_t k = 0;
  p->grid().for_each([&](const int32_t& w, const Coord& c) {
    const int32_t pr = orc::cell_prob(w);
    const bool keep = sign > 0 ? pr > p->thr : pr < p->thr;
    if (!keep) return;
    if (k < cap) {
      xyz[3 * k] = c.x;
      xyz[3 * k + 1] = c.y;
      xyz[3 * k + 2] = c.z;
    }
    k++;
  });
  return k;
}
size_t orc_pmap_get_occupied(void* m, int32_t* xyz, size_t cap) {
  return pmap_filter(m, xyz, cap, 1);
}
// The ROS node's occupied-voxel export (bonxai_server.cpp:217-243): the
// PointT getOccupiedVoxels (probabilistic_map.hpp:115-124) gives corner
// positions double(c) * resolution (bonxai.hpp:413-417); z in [min_z, max_z]
// is kept and narrowed to float.
size_t orc_pmap_export_occupied_f32(void* m, double min_z, double max_z, float* xyz,
                                    size_t cap) {
  auto* p = static_cast<orc::PMap*>(m);
  const double res = p->grid().resolution();
  size_t k = 0;
  p->grid().for_each([&](const int32_t& w, const Coord& c) {
    if (!(orc::cell_prob(w) > p->thr)) return;
    const double x = double(c.x) * res, y = double(c.y) * res, z = double(c.z) * res;
    if (!(z >= min_z && z <= max_z)) return;
    if (k < cap) {
      xyz[3 * k] = float(x);
      xyz[3 * k + 1] = float(y);
      xyz[3 * k + 2] = float(z);
    }
    k++;
  });
  return k;
}
size_t orc_pmap_get_free(void* m, int32_t* xyz, size_t cap) {
  return pmap_filter(m, xyz, cap, -1);
}

void* orc_grid_create(double r, int ib, int lb, int dtype) {
  switch (dtype) {
    case ORC_F32: return static_cast<orc::GridIf*>(new orc::GridImpl<float>(r, ib, lb));
    case ORC_I32: return static_cast<orc::GridIf*>(new orc::GridImpl<int32_t>(r, ib, lb));
    case ORC_U32: return static_cast<orc::GridIf*>(new orc::GridImpl<uint32_t>(r, ib, lb));
    case ORC_F64: return static_cast<orc::GridIf*>(new orc::GridImpl<double>(r, ib, lb));
    case ORC_I64: return static_cast<orc::GridIf*>(new orc::GridImpl<int64_t>(r, ib, lb));
    default: return nullptr;
  }
}
void orc_grid_destroy(void* g) { delete static_cast<orc::GridIf*>(g); }
void orc_grid_pos_to_coord(void* g, const double* xyz, size_t n, int32_t* out) {
  static_cast<orc::GridIf*>(g)->pos_to_coord(xyz, n, out);
}
void orc_grid_set_values(void* g, const int32_t* xyz, const void* v, size_t n, uint8_t* w) {
  static_cast<orc::GridIf*>(g)->set_values(xyz, v, n, w);
}
void orc_grid_get_values(void* g, const int32_t* xyz, size_t n, void* out, uint8_t* f, int c) {
  static_cast<orc::GridIf*>(g)->get_values(xyz, n, out, f, c);
}
void orc_grid_set_cells_on(void* g, const int32_t* xyz, size_t n, const void* d, uint8_t* w) {
  static_cast<orc::GridIf*>(g)->set_on(xyz, n, d, w);
}
void orc_grid_set_cells_off(void* g, const int32_t* xyz, size_t n, uint8_t* w) {
  static_cast<orc::GridIf*>(g)->set_off(xyz, n, w);
}
void orc_grid_is_cell_on(void* g, const int32_t* xyz, size_t n, uint8_t* out) {
  static_cast<orc::GridIf*>(g)->is_on(xyz, n, out);
}
size_t orc_grid_active_cells(void* g) { return static_cast<orc::GridIf*>(g)->active(); }
size_t orc_grid_leaf_count(void* g) { return static_cast<orc::GridIf*>(g)->leaves(); }
size_t orc_grid_root_count(void* g) { return static_cast<orc::GridIf*>(g)->roots(); }
size_t orc_grid_dump(void* g, int32_t* xyz, void* v, size_t cap) {
  return static_cast<orc::GridIf*>(g)->dump(xyz, v, cap);
}
void orc_grid_clear(void* g, int opt) { static_cast<orc::GridIf*>(g)->clear(opt); }
void orc_grid_release_unused(void* g) { static_cast<orc::GridIf*>(g)->release(); }

// The ROS node's cloud ingest (bonxai_server.cpp:147-168): drop points with a
// non-finite coordinate, then transform by a row-major 3x4 float [R | t] in
// float, ((r0*x + r1*y) + r2*z) + t per axis (built without contraction).
// PCL is not part of the reference's repository; this operation order is the
// stated assumption the GPU path shares. Returns the points kept.
size_t orc_sensor_to_world_f32(const float* m12, const float* xyz, size_t n, float* out) {
  size_t k = 0;
  for (size_t i = 0; i < n; i++) {
    const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    if (!(std::isfinite(x) && std::isfinite(y) && std::isfinite(z))) continue;
    for (int r = 0; r < 3; r++) {
      float v = m12[4 * r] * x;
      v = v + m12[4 * r + 1] * y;
      v = v + m12[4 * r + 2] * z;
      out[3 * k + r] = v + m12[4 * r + 3];
    }
    k++;
  }
  return k;
}

size_t orc_compute_ray(const int32_t* o, const int32_t* e, int32_t* out, size_t cap) {
  size_t k = 0;
  orc::walk_ray(Coord{o[0], o[1], o[2]}, Coord{e[0], e[1], e[2]}, [&](const Coord& c) {
    if (k < cap) {
      out[3 * k] = c.x;
      out[3 * k + 1] = c.y;
      out[3 * k + 2] = c.z;
    }
    k++;
  });
  return k;
}

}  // extern "C"
