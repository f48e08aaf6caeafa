// Per-point and per-ray device logic of the ProbabilisticMap scan, shared by
// the single-map kernels (bxg_pmap.cu) and the batched multi-map kernel
// (bxg_batch.cu), so both run identical arithmetic.
//
// Why a scan parallelises without changing its result. Let u be the scan
// counter (1, 2, 3, cycling; probabilistic_map.cpp:103-105).
//  * Endpoint phase (insertPointCloud loop + addHit/MissPoint, hpp:146-158,
//    cpp:30-54). Only endpoint cells change, and each changes at most once:
//    the first point (lowest input index) that lands in a cell whose
//    update_id != u updates it and queues one ray; every later point in that
//    cell sees update_id == u and does nothing. A cell that already had
//    update_id == u before the scan is neither updated nor ray-cast. So the
//    outcome per cell depends only on its pre-scan word and the lowest index
//    landing in it.
//  * Ray phase (updateFreeCells, cpp:77-106). Every queued ray visits the
//    origin cell and the next max-1 Bresenham cells; each visited cell is
//    created (T{} = {0, 0}) and, if its update_id != u, becomes
//    {max(p + miss, clamp_min), u}. After the endpoint phase the only writes
//    are this one function of the word, so the order of rays and cells is
//    irrelevant and racing writers store the same value: a plain load and a
//    conditional store suffice.
#pragma once

#include <cmath>

#include "bxg_device.cuh"

namespace bxg {

struct Opts {
  int32_t miss, hit, cmin, cmax;
};

__device__ __forceinline__ bool finite3(double a, double b, double c) {
  return isfinite(a) && isfinite(b) && isfinite(c);
}

// Lowest index per endpoint cell (scratch table, all-ones = empty).
__device__ __forceinline__ void dedup_min_insert(uint4* tab, uint32_t tmask, int x, int y, int z,
                                                 uint32_t i, const DMap& M) {
  const uint4 kEmpty = make_uint4(kNone, kNone, kNone, kNone);
  const uint4 mine = make_uint4(uint32_t(x), uint32_t(y), uint32_t(z), i);
  uint32_t h = cell_hash(x, y, z) & tmask;
  for (uint32_t p = 0; p <= tmask; ++p, h = (h + 1) & tmask) {
    const uint4 old = cas128(tab + h, kEmpty, mine);
    if (eq4(old, kEmpty)) return;
    if (key_eq(old, x, y, z)) {
      atomicMin(&tab[h].w, i);
      return;
    }
  }
  set_err(M, ERR_SCRATCH);
}

__device__ __forceinline__ uint32_t dedup_lookup(const uint4* tab, uint32_t tmask, int x, int y,
                                                 int z) {
  uint32_t h = cell_hash(x, y, z) & tmask;
  for (uint32_t p = 0; p <= tmask; ++p, h = (h + 1) & tmask) {
    const uint4 b = tab[h];
    if (b.w == kNone) return kNone;
    if (key_eq(b, x, y, z)) return b.w;
  }
  return kNone;
}

// float32 filter for the endpoint math of float clouds. GB300 runs double
// precision at a small fraction of its float rate, and the double math was the
// bound of the endpoint kernel (fp64 pipe 60 % busy). Each point is first
// computed in float with a bound on its distance from the double result; a
// result that no error within the bound can change -- the hit/miss test
// decided with margin, every floor() at least the bound away from an integer
// -- is exact, and any other point goes through the double path unchanged
// (an adaptive-precision filter in the manner of Shewchuk's predicates).
//
// Bounds, with u = 2^-24 and all float operations rounded to nearest:
//   sq:  |sq_f - sq| <= 5u sq               (vx, vy, vz exact in double or
//                                           within u; three products, two sums)
//   hit: |y_f - y_d| <= 2u |y|              (inv_res rounded to float, one product)
//   miss: |y_f - y_d| <= ((7.5 mr + |e|) inv_res + 2 |y|) u
//        (sqrt 3.5u, quotient 5.5u, times max_range 7.5u, plus origin, times inv_res)
// The filter uses margins four times these bounds.
struct EpFast {
  float ox, oy, oz;    // origin (exactly the double origin)
  float inv_res;       // 1 / resolution rounded to float
  float mr;            // max_range rounded to float
  float sq_hi, sq_lo;  // sq_f above sq_hi: miss; below sq_lo: hit; else double path
  int on;              // the filter applies (float origin, finite parameters)
};

inline EpFast make_ep_fast(double fx, double fy, double fz, double max_range, double inv_res) {
  EpFast F{};
  F.ox = static_cast<float>(fx);
  F.oy = static_cast<float>(fy);
  F.oz = static_cast<float>(fz);
  F.inv_res = static_cast<float>(inv_res);
  F.mr = static_cast<float>(max_range);
  const double mr2 = max_range * max_range;
  const double hi = mr2 * (1.0 + 0x1p-19), lo = mr2 * (1.0 - 0x1p-19);
  F.sq_hi = std::nextafter(static_cast<float>(hi), HUGE_VALF);
  F.sq_lo = std::nextafter(static_cast<float>(lo), 0.0f);
  F.on = static_cast<double>(F.ox) == fx && static_cast<double>(F.oy) == fy &&
         static_cast<double>(F.oz) == fz && std::isfinite(F.inv_res) && F.inv_res > 0.0f &&
         !std::isnan(max_range) && max_range >= 0.0 &&
         (std::isinf(max_range) || max_range < 1e30);
  if (std::isinf(max_range)) F.sq_hi = F.sq_lo = HUGE_VALF;
  return F;
}

// floor(y) when y is more than tol from an integer (and |y| < 2^23, where the
// fractional part of a float is exact).
__device__ __forceinline__ bool floor_filtered(float y, float tol, int& c) {
  if (!(fabsf(y) < 8388608.0f)) return false;
  const float fl = floorf(y);
  if (__fsub_rn(y, fl) <= tol || __fsub_rn(__fadd_rn(fl, 1.0f), y) <= tol) return false;
  c = static_cast<int>(fl);
  return true;
}

// The float filter for one finite point; false = use the double path.
__device__ __forceinline__ bool endpoint_fast(float px, float py, float pz, const EpFast& F,
                                              int4& out) {
  const float vx = __fsub_rn(px, F.ox), vy = __fsub_rn(py, F.oy), vz = __fsub_rn(pz, F.oz);
  const float sq = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
  if (!(sq < 1e30f)) return false;
  float ex, ey, ez, tx, ty, tz;
  int kind;
  if (sq < F.sq_lo) {
    ex = px;
    ey = py;
    ez = pz;
    kind = EP_HIT;
  } else if (sq > F.sq_hi) {
    const float s = __fsqrt_rn(sq);
    ex = __fadd_rn(F.ox, __fmul_rn(__fdiv_rn(vx, s), F.mr));
    ey = __fadd_rn(F.oy, __fmul_rn(__fdiv_rn(vy, s), F.mr));
    ez = __fadd_rn(F.oz, __fmul_rn(__fdiv_rn(vz, s), F.mr));
    kind = EP_MISS;
  } else {
    return false;
  }
  const float yx = __fmul_rn(ex, F.inv_res), yy = __fmul_rn(ey, F.inv_res),
              yz = __fmul_rn(ez, F.inv_res);
  if (kind == EP_HIT) {  // 4 x 2u |y|
    tx = fabsf(yx) * 4.76837158e-7f;
    ty = fabsf(yy) * 4.76837158e-7f;
    tz = fabsf(yz) * 4.76837158e-7f;
  } else {  // 4 x ((7.5 mr + |e|) inv_res + 2 |y|) u, with 8 for 7.5
    const float m8 = 8.0f * F.mr;
    tx = ((m8 + fabsf(ex)) * F.inv_res + 2.0f * fabsf(yx)) * 2.38418579e-7f;
    ty = ((m8 + fabsf(ey)) * F.inv_res + 2.0f * fabsf(yy)) * 2.38418579e-7f;
    tz = ((m8 + fabsf(ez)) * F.inv_res + 2.0f * fabsf(yz)) * 2.38418579e-7f;
  }
  int cx, cy, cz;
  // a hit coordinate that is exactly zero gives cell 0 in double as well (a
  // miss coordinate rounded to zero in float need not be zero in double)
  const bool hit = kind == EP_HIT;
  if (hit && ex == 0.0f) cx = 0; else if (!floor_filtered(yx, tx, cx)) return false;
  if (hit && ey == 0.0f) cy = 0; else if (!floor_filtered(yy, ty, cy)) return false;
  if (hit && ez == 0.0f) cz = 0; else if (!floor_filtered(yz, tz, cz)) return false;
  out = make_int4(cx, cy, cz, kind);
  return true;
}

// insertPointCloud's per-point math (probabilistic_map.hpp:144-156) in double
// with one IEEE rounding per operation and no contraction:
//   v = to - from; sq = (vx*vx + vy*vy) + vz*vz;
//   sq >= max_range^2 ? miss at from + (v / sqrt(sq)) * max_range : hit at to
// then posToCoord = floor(p * inv_resolution) (bonxai.hpp:404-410).
// Float clouds go through the float filter first when F is on.
// Returns {cell, EP_HIT | EP_MISS | EP_SKIP}.
template <typename PT>
__device__ __forceinline__ int4 compute_endpoint(const PT* p, double fx, double fy, double fz,
                                                 double max_range, double mr2, double inv_res,
                                                 bool keep_nonfinite,
                                                 const EpFast* F = nullptr) {
  if (sizeof(PT) == 4 && F && F->on) {
    const float px = static_cast<float>(p[0]), py = static_cast<float>(p[1]),
                pz = static_cast<float>(p[2]);
    if (isfinite(px) && isfinite(py) && isfinite(pz)) {
      int4 r;
      if (endpoint_fast(px, py, pz, *F, r)) return r;
    } else if (!keep_nonfinite) {
      return make_int4(0, 0, 0, EP_SKIP);
    }
  }
  const double tx = static_cast<double>(p[0]), ty = static_cast<double>(p[1]),
               tz = static_cast<double>(p[2]);
  if (!keep_nonfinite && !finite3(tx, ty, tz)) return make_int4(0, 0, 0, EP_SKIP);
  const double vx = __dsub_rn(tx, fx), vy = __dsub_rn(ty, fy), vz = __dsub_rn(tz, fz);
  const double sq = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
  double ex, ey, ez;
  int kind;
  if (sq >= mr2) {
    const double s = __dsqrt_rn(sq);
    ex = __dadd_rn(fx, __dmul_rn(__ddiv_rn(vx, s), max_range));
    ey = __dadd_rn(fy, __dmul_rn(__ddiv_rn(vy, s), max_range));
    ez = __dadd_rn(fz, __dmul_rn(__ddiv_rn(vz, s), max_range));
    kind = EP_MISS;
  } else {
    ex = tx;
    ey = ty;
    ez = tz;
    kind = EP_HIT;
  }
  return make_int4(__double2int_rd(__dmul_rn(ex, inv_res)), __double2int_rd(__dmul_rn(ey, inv_res)),
                   __double2int_rd(__dmul_rn(ez, inv_res)), kind);
}

__device__ __forceinline__ uint32_t chebyshev(int ox, int oy, int oz, int x, int y, int z) {
  const uint32_t dx = static_cast<uint32_t>(abs(x - ox)), dy = static_cast<uint32_t>(abs(y - oy)),
                 dz = static_cast<uint32_t>(abs(z - oz));
  return max(dx, max(dy, dz));
}

// The lowest-index point of an endpoint cell decides: no update and no ray
// if the cell exists with update_id == u; otherwise it applies its hit or miss
// (probabilistic_map.cpp:35-41,49-54) and its ray is cast (returns true). The
// winner owns its cell -- no other thread writes it in this phase -- so the
// word it reads is the pre-scan word. If the pool is full the ray is still
// listed and the endpoint is completed after the pool grows.
__device__ __forceinline__ bool winner_apply(const DMap& M, int4 e, int32_t u, const Opts& o) {
  const uint32_t lf = leaf_of(M, e.x, e.y, e.z, true);
  if (lf == kNone) return true;
  const uint32_t ci = leaf_index(M, e.x, e.y, e.z);
  int32_t* cp = reinterpret_cast<int32_t*>(M.ldata) + size_t(lf) * M.lsize + ci;
  const bool on = cell_is_on(M, lf, ci);
  const int32_t w = *cp;
  if (on && cell_id(w) == u) return false;
  const int32_t p = cell_prob(w);
  const int32_t np =
      e.w == EP_HIT ? min(wrap_add(p, o.hit), o.cmax) : max(wrap_add(p, o.miss), o.cmin);
  *cp = cell_pack(np, u);
  if (!on) cell_or_on(M, lf, ci);
  return true;
}

// Walks one ray (origin -> end, end excluded) with a group of W lanes; lane sl
// handles k = sl, sl+W, ... Consecutive lanes hold consecutive cells, so the
// lanes of one step touch a few leaves: the first lane of each leaf run (a
// "head") looks the leaf up -- inline fast path first, the bounded-wait
// creation path only on a miss -- and the others take its slot by shuffle.
// The group carries the last leaf between steps. Heads probe the root hash
// directly: neighbouring heads hit the same buckets in L1, and carrying the
// last root through the group cost more shuffles than the probes it saved.
//
// Leaf runs are found by comparing a 30-bit packed leaf index (10 low bits per
// axis): two cells at most W+1 steps apart on one ray are at most a few
// leaves apart, so equal low bits mean the same leaf.
//
// A cell word is read once: a ProbabilisticMap cell that is on always has
// update_id in {1,2,3} (every path that turns a cell on updates it in the same
// scan), so a nonzero word is on, and only a zero word (new, or on with a
// user-written zero) needs the mask bit -- set with a fire-and-forget OR.
//
// walk_ray_op is the walk itself; per step every lane calls
// op(act, leaf, ci, k): act = the lane has a cell (k < m), leaf = its leaf
// slot (kNone if the pool ran out), ci = its index in the leaf, k = its
// position on the ray.
// Leaf directory: a dense cube of `side`^3 words over the leaves around the
// scan's origin, covering every leaf within max_range (x0/y0/z0: leaf
// coordinate of its corner). A word holds (epoch << 28) | leaf slot; a word of
// another epoch is empty, so the cube is cleared only when the 4-bit epoch
// wraps. The host keeps a cube and its words across scans until the origin
// leaves it or a leaf slot is released. A head inside the cube reads one word
// instead of probing the root hash and the inner node, and writes the slot it
// resolved otherwise (racing writers store the same word).
struct LeafDir {
  uint32_t* words;  // nullptr: no directory
  int x0, y0, z0;
  uint32_t side;
  uint32_t epoch;  // 1..15, in bits 28-31 of a valid word
};

// DIR: the walk reads the leaf directory D (compiled out otherwise: the code
// costs registers in kernels that never have one).
template <int W, bool DIR, class Op>
__device__ __forceinline__ void walk_ray_op(const DMap& M, int4 e, int ox, int oy, int oz,
                                            unsigned sl, unsigned gbase, unsigned gmask,
                                            Op&& op, const LeafDir* D) {
  const int dx = e.x - ox, dy = e.y - oy, dz = e.z - oz;
  const uint32_t ax = static_cast<uint32_t>(abs(dx)), ay = static_cast<uint32_t>(abs(dy)),
                 az = static_cast<uint32_t>(abs(dz));
  const uint32_t m = max(ax, max(ay, az));
  if (m == 0) return;  // origin == end: no ray (probabilistic_map.hpp:164-166)
  if (m >= kMaxRayCells) {
    if (sl == 0) set_err(M, ERR_RAY_TOO_LONG);
    return;
  }
  const int lb = M.lb;
  const int32_t rm = root_mask(M);
  const int sx = dx < 0 ? -1 : 1, sy = dy < 0 ? -1 : 1, sz = dz < 0 ? -1 : 1;
  const uint32_t two_m = 2u * m;
  const float rtm = __frcp_rn(static_cast<float>(two_m));
  AxisStep X, Y, Z;
  axis_init(X, ax, m, two_m, rtm, sl, W);
  axis_init(Y, ay, m, two_m, rtm, sl, W);
  axis_init(Z, az, m, two_m, rtm, sl, W);
  uint32_t pkey = kNone;  // packed leaf index of the previous step's last lane
  uint32_t pleaf = kNone;

  for (uint32_t base = 0; base < m; base += W) {
    const bool act = base + sl < m;
    const int cx = ox + sx * static_cast<int>(X.n);
    const int cy = oy + sy * static_cast<int>(Y.n);
    const int cz = oz + sz * static_cast<int>(Z.n);
    const uint32_t key = (static_cast<uint32_t>(cx >> lb) & 1023u) |
                         ((static_cast<uint32_t>(cy >> lb) & 1023u) << 10) |
                         ((static_cast<uint32_t>(cz >> lb) & 1023u) << 20);
    uint32_t q = __shfl_up_sync(gmask, key, 1, W);
    if (sl == 0) q = pkey;
    const bool head = act && key != q;
    uint32_t leaf = kNone;
    if (head) {
      uint32_t* dw = nullptr;
      if (DIR && D) {
        const uint32_t qx = static_cast<uint32_t>((cx >> lb) - D->x0),
                       qy = static_cast<uint32_t>((cy >> lb) - D->y0),
                       qz = static_cast<uint32_t>((cz >> lb) - D->z0);
        if (qx < D->side && qy < D->side && qz < D->side) {
          dw = D->words + (static_cast<size_t>(qx) * D->side + qy) * D->side + qz;
          const uint32_t w = *dw;
          if ((w >> 28) == D->epoch) leaf = w & 0x0FFFFFFFu;
        }
      }
      if (leaf == kNone) {
        const int rx = cx & rm, ry = cy & rm, rz = cz & rm;
        uint32_t in = root_probe_fast(M, rx, ry, rz);
        if (in == kPending) in = root_get_or_create(M, rx, ry, rz);
        if (in != kNone) {
          const uint32_t ii = inner_index(M, cx, cy, cz);
          leaf = M.ichild[static_cast<size_t>(in) * M.isize + ii];
          if (leaf >= kPending) {
            const int32_t lm = leaf_mask(M);
            leaf = leaf_get_or_create(M, in, ii, cx & lm, cy & lm, cz & lm);
          }
        }
        if (DIR && dw && leaf != kNone) *dw = (D->epoch << 28) | leaf;
      }
    }
    const unsigned hm = (__ballot_sync(gmask, head) & gmask) >> gbase;
    const unsigned below = hm & ((2u << sl) - 1u);
    const uint32_t got = __shfl_sync(gmask, leaf, below ? 31 - __clz(below) : 0, W);
    leaf = below ? got : pleaf;
    op(act, leaf, leaf_index(M, cx, cy, cz), base + sl);
    const uint32_t rem = m - base;
    const int last = static_cast<int>(rem < W ? rem : W) - 1;
    pkey = __shfl_sync(gmask, key, last, W);
    pleaf = __shfl_sync(gmask, leaf, last, W);
    axis_advance(X, two_m);
    axis_advance(Y, two_m);
    axis_advance(Z, two_m);
  }
}

// The ray walk with the miss update applied in place (the single-pass form).
template <int W, bool DIR = false>
__device__ __forceinline__ void walk_ray(const DMap& M, int4 e, int ox, int oy, int oz,
                                         int32_t u, int32_t miss, int32_t cmin, unsigned sl,
                                         unsigned gbase, unsigned gmask, uint32_t& visited,
                                         uint32_t& updated, const LeafDir* D = nullptr) {
  int32_t* const cells = reinterpret_cast<int32_t*>(M.ldata);
  walk_ray_op<W, DIR>(M, e, ox, oy, oz, sl, gbase, gmask,
                 [&](bool act, uint32_t leaf, uint32_t ci, uint32_t) {
                   if (act && leaf != kNone) {
                     int32_t* cp = cells + static_cast<size_t>(leaf) * M.lsize + ci;
                     const int32_t w = *cp;
                     if (cell_id(w) != u) {
                       *cp = cell_pack(max(wrap_add(cell_prob(w), miss), cmin), u);
                       if (w == 0) cell_or_on(M, leaf, ci);
                       updated++;
                     }
                     visited++;
                   }
                 },
                 D);
}

// Leaf slot of a head cell: the inline hash probe, else the bounded-wait
// creation path.
__device__ __forceinline__ uint32_t head_leaf(const DMap& M, int cx, int cy, int cz,
                                              int32_t rm) {
  const int rx = cx & rm, ry = cy & rm, rz = cz & rm;
  uint32_t in = root_probe_fast(M, rx, ry, rz);
  if (in == kPending) in = root_get_or_create(M, rx, ry, rz);
  if (in == kNone) return kNone;
  const uint32_t ii = inner_index(M, cx, cy, cz);
  uint32_t leaf = M.ichild[static_cast<size_t>(in) * M.isize + ii];
  if (leaf >= kPending) {
    const int32_t lm = leaf_mask(M);
    leaf = leaf_get_or_create(M, in, ii, cx & lm, cy & lm, cz & lm);
  }
  return leaf;
}

// One W-step of a lane's (n, r) state: returns the state W cells further on.
__device__ __forceinline__ void axis_peek(const AxisStep& a, uint32_t two_m, uint32_t& n,
                                          uint32_t& r) {
  r = a.r + a.R;
  n = a.n + a.Q;
  if (r >= two_m) {
    n += 1;
    r -= two_m;
  }
}

// walk_ray with two cells per lane per step (k and k + W): the two cells'
// leaf lookups and word loads are independent, which doubles the memory-level
// parallelism of a lane on this latency-bound walk. Same cells, same updates.
template <int W>
__device__ __forceinline__ void walk_ray2(const DMap& M, int4 e, int ox, int oy, int oz,
                                          int32_t u, int32_t miss, int32_t cmin, unsigned sl,
                                          unsigned gbase, unsigned gmask, uint32_t& visited,
                                          uint32_t& updated) {
  const int dx = e.x - ox, dy = e.y - oy, dz = e.z - oz;
  const uint32_t ax = static_cast<uint32_t>(abs(dx)), ay = static_cast<uint32_t>(abs(dy)),
                 az = static_cast<uint32_t>(abs(dz));
  const uint32_t m = max(ax, max(ay, az));
  if (m == 0) return;
  if (m >= kMaxRayCells) {
    if (sl == 0) set_err(M, ERR_RAY_TOO_LONG);
    return;
  }
  const int lb = M.lb;
  const int32_t rm = root_mask(M);
  int32_t* const cells = reinterpret_cast<int32_t*>(M.ldata);
  const int sx = dx < 0 ? -1 : 1, sy = dy < 0 ? -1 : 1, sz = dz < 0 ? -1 : 1;
  const uint32_t two_m = 2u * m;
  const float rtm = __frcp_rn(static_cast<float>(two_m));
  AxisStep X, Y, Z;  // state of k = base + sl; Q/R advance by W
  axis_init(X, ax, m, two_m, rtm, sl, W);
  axis_init(Y, ay, m, two_m, rtm, sl, W);
  axis_init(Z, az, m, two_m, rtm, sl, W);
  uint32_t pkey = kNone, pleaf = kNone;

  for (uint32_t base = 0; base < m; base += 2 * W) {
    uint32_t nx2, rx2, ny2, ry2, nz2, rz2;
    axis_peek(X, two_m, nx2, rx2);
    axis_peek(Y, two_m, ny2, ry2);
    axis_peek(Z, two_m, nz2, rz2);
    const bool act1 = base + sl < m, act2 = base + W + sl < m;
    const int c1x = ox + sx * static_cast<int>(X.n), c1y = oy + sy * static_cast<int>(Y.n),
              c1z = oz + sz * static_cast<int>(Z.n);
    const int c2x = ox + sx * static_cast<int>(nx2), c2y = oy + sy * static_cast<int>(ny2),
              c2z = oz + sz * static_cast<int>(nz2);
    const uint32_t key1 = (static_cast<uint32_t>(c1x >> lb) & 1023u) |
                          ((static_cast<uint32_t>(c1y >> lb) & 1023u) << 10) |
                          ((static_cast<uint32_t>(c1z >> lb) & 1023u) << 20);
    const uint32_t key2 = (static_cast<uint32_t>(c2x >> lb) & 1023u) |
                          ((static_cast<uint32_t>(c2y >> lb) & 1023u) << 10) |
                          ((static_cast<uint32_t>(c2z >> lb) & 1023u) << 20);
    uint32_t q1 = __shfl_up_sync(gmask, key1, 1, W);
    uint32_t q2 = __shfl_up_sync(gmask, key2, 1, W);
    const uint32_t last1 = __shfl_sync(gmask, key1, W - 1, W);
    if (sl == 0) {
      q1 = pkey;
      q2 = last1;
    }
    const bool head1 = act1 && key1 != q1, head2 = act2 && key2 != q2;
    uint32_t leaf1 = kNone, leaf2 = kNone;
    if (head1) leaf1 = head_leaf(M, c1x, c1y, c1z, rm);
    if (head2) leaf2 = head_leaf(M, c2x, c2y, c2z, rm);
    const unsigned hm1 = (__ballot_sync(gmask, head1) & gmask) >> gbase;
    const unsigned hm2 = (__ballot_sync(gmask, head2) & gmask) >> gbase;
    const unsigned below1 = hm1 & ((2u << sl) - 1u), below2 = hm2 & ((2u << sl) - 1u);
    const uint32_t g1 = __shfl_sync(gmask, leaf1, below1 ? 31 - __clz(below1) : 0, W);
    leaf1 = below1 ? g1 : pleaf;
    const uint32_t end1 = __shfl_sync(gmask, leaf1, W - 1, W);
    const uint32_t g2 = __shfl_sync(gmask, leaf2, below2 ? 31 - __clz(below2) : 0, W);
    leaf2 = below2 ? g2 : end1;
    const bool do1 = act1 && leaf1 != kNone, do2 = act2 && leaf2 != kNone;
    int32_t* cp1 = cells + static_cast<size_t>(do1 ? leaf1 : 0) * M.lsize +
                   leaf_index(M, c1x, c1y, c1z);
    int32_t* cp2 = cells + static_cast<size_t>(do2 ? leaf2 : 0) * M.lsize +
                   leaf_index(M, c2x, c2y, c2z);
    const int32_t w1 = do1 ? *cp1 : 0;
    const int32_t w2 = do2 ? *cp2 : 0;
    if (do1 && cell_id(w1) != u) {
      *cp1 = cell_pack(max(wrap_add(cell_prob(w1), miss), cmin), u);
      if (w1 == 0) cell_or_on(M, leaf1, leaf_index(M, c1x, c1y, c1z));
      updated++;
    }
    if (do2 && cell_id(w2) != u) {
      *cp2 = cell_pack(max(wrap_add(cell_prob(w2), miss), cmin), u);
      if (w2 == 0) cell_or_on(M, leaf2, leaf_index(M, c2x, c2y, c2z));
      updated++;
    }
    visited += (do1 ? 1u : 0u) + (do2 ? 1u : 0u);
    // carry the last active cell's leaf key and slot to the next step
    const uint32_t rem = m - base;
    if (rem > W) {
      const int last = static_cast<int>(rem - W < W ? rem - W : W) - 1;
      pkey = __shfl_sync(gmask, key2, last, W);
      pleaf = __shfl_sync(gmask, leaf2, last, W);
    } else {
      const int last = static_cast<int>(rem) - 1;
      pkey = __shfl_sync(gmask, key1, last, W);
      pleaf = __shfl_sync(gmask, leaf1, last, W);
    }
    // two W-steps
    X.n = nx2; X.r = rx2;
    Y.n = ny2; Y.r = ry2;
    Z.n = nz2; Z.r = rz2;
    axis_advance(X, two_m);
    axis_advance(Y, two_m);
    axis_advance(Z, two_m);
  }
}

}  // namespace bxg
