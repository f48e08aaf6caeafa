// ProbabilisticMap on the GPU: insertPointCloud / addHitPoint / addMissPoint /
// updateFreeCells / isOccupied / getOccupiedVoxels, bit-exact with
// bonxai_map/include/bonxai_map/probabilistic_map.hpp and
// bonxai_map/src/probabilistic_map.cpp.
//
// Why a scan parallelises without changing its result: see bxg_scan.cuh.
//
// Kernels per scan (all on the handle's stream):
//   k_endpoints   fp64 endpoint of each point, exactly as hpp:147-156 rounds
//                 it; lowest index per endpoint cell via a scratch hash table.
//   k_winners     the lowest-index point of each cell reads the pre-scan word;
//                 unless update_id == u it applies its hit/miss and appends
//                 {cell, hit/miss} to the ray list (and counts the ray length
//                 for the ray-cell total).
//   k_apply       only after a pool ran out: completes the listed endpoints.
//   k_mark        the ray phase's first part: every listed ray's cells set
//                 their bits in the scan's cube bitmap (bxg_mark.cuh).
//   k_list_touched  the marked leaf blocks onto a list, in cube order.
//   k_apply_rays  per listed leaf block, get-or-create the leaf and apply the
//                 miss update to its marked cells.
//   k_rays        the single-pass form of the ray phase, for scans the cube
//                 does not cover (rays queued by addHitPoint/addMissPoint,
//                 kept non-finite points, cubes above the size limit): a group
//                 of W lanes walks one ray, W consecutive cells per step,
//                 creating leaves on the way and applying the miss update.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bxg_internal.h"
#include "bxg_mark.cuh"
#include "bxg_scan.cuh"

namespace bxg {

// Endpoint of each point; lowest index per endpoint cell in the scratch table.
// zero: bit 0 -- the scan's statistics start at zero; bit 1 -- the ray list
// starts empty (no rays queued by earlier addHitPoint/addMissPoint batches).
// Done by the first kernel of a scan instead of memsets.
enum : int { ZERO_STATS = 1, ZERO_CAST = 2 };
__device__ __forceinline__ void zero_scan_stats(const DMap& M, int zero) {
  if (blockIdx.x != 0) return;
  if ((zero & ZERO_STATS) && threadIdx.x < S_COUNT)
    reinterpret_cast<unsigned long long*>(M.ctr + C_STATS)[threadIdx.x] = 0ull;
  if ((zero & ZERO_CAST) && threadIdx.x == 32) M.ctr[C_CAST] = 0u;
}

template <typename PT>
__global__ void k_endpoints(const __grid_constant__ DMap M, const uint8_t* __restrict__ pts, size_t stride, uint32_t n,
                            double fx, double fy, double fz, double max_range, double mr2,
                            double inv_res, int keep_nonfinite, int4* __restrict__ ep,
                            uint4* tab, uint32_t tmask, int zero_stats, EpFast F) {
  zero_scan_stats(M, zero_stats);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  int4 e = make_int4(0, 0, 0, EP_SKIP);
  if (i < n) {
    const PT* p = reinterpret_cast<const PT*>(pts + size_t(i) * stride);
    e = compute_endpoint<PT>(p, fx, fy, fz, max_range, mr2, inv_res, keep_nonfinite != 0, &F);
  }
  // Neighbouring points often share an endpoint cell: within a warp only the
  // lowest lane (lowest index) of each cell enters the table; the others can
  // never be the cell's lowest index and are marked EP_DUP.
  const unsigned vm = __ballot_sync(0xffffffffu, e.w != EP_SKIP);
  if (e.w != EP_SKIP) {
    const unsigned same = __match_any_sync(vm, e.x) & __match_any_sync(vm, e.y) &
                          __match_any_sync(vm, e.z);
    if (same & ((1u << (threadIdx.x & 31)) - 1u)) e.w = EP_DUP;
    else dedup_min_insert(tab, tmask, e.x, e.y, e.z, i, M);
  }
  if (i < n) ep[i] = e;
}

// A sensor-frame cloud with its sensor-to-world transform (row-major 3x4),
// the ingest of bonxai_ros/src/bonxai_server.cpp:147-171 fused into the
// endpoint kernel: points with a non-finite coordinate are dropped (:147-154),
// the rest are transformed in float (:166-168), then handled as k_endpoints
// does. A dropped point keeps its index, so the lowest-index rule gives the
// same winners as the host's compaction. Transform order per axis, in float
// without contraction: ((m[r][0]*x + m[r][1]*y) + m[r][2]*z) + m[r][3].
struct Xf {
  float m[12];
};

__device__ __forceinline__ float xf_row(const Xf& t, int r, float x, float y, float z) {
  return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(t.m[4 * r], x), __fmul_rn(t.m[4 * r + 1], y)),
                             __fmul_rn(t.m[4 * r + 2], z)),
                   t.m[4 * r + 3]);
}

__global__ void k_endpoints_sensor(const __grid_constant__ DMap M, const uint8_t* __restrict__ pts, size_t stride,
                                   uint32_t n, Xf xf, double fx, double fy, double fz,
                                   double max_range, double mr2, double inv_res,
                                   int4* __restrict__ ep, uint4* tab, uint32_t tmask,
                                   int zero_stats, EpFast F) {
  zero_scan_stats(M, zero_stats);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* p = reinterpret_cast<const float*>(pts + size_t(i) * stride);
  const float x = p[0], y = p[1], z = p[2];
  if (!(isfinite(x) && isfinite(y) && isfinite(z))) {
    ep[i] = make_int4(0, 0, 0, EP_SKIP);
    return;
  }
  const float w[3] = {xf_row(xf, 0, x, y, z), xf_row(xf, 1, x, y, z), xf_row(xf, 2, x, y, z)};
  const int4 e = compute_endpoint<float>(w, fx, fy, fz, max_range, mr2, inv_res, true, &F);
  ep[i] = e;
  if (e.w != EP_SKIP) dedup_min_insert(tab, tmask, e.x, e.y, e.z, i, M);
}

// addHitPoint / addMissPoint batches: double points with a given kind, or a
// per-point kind (0 hit, 1 miss) when kinds != nullptr.
__global__ void k_endpoints_kind(const __grid_constant__ DMap M, const double* __restrict__ pts, uint32_t n, int kind,
                                 const uint8_t* __restrict__ kinds, double inv_res,
                                 int4* __restrict__ ep, uint4* tab, uint32_t tmask, int zero) {
  zero_scan_stats(M, zero);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (kinds) kind = kinds[i] ? EP_MISS : EP_HIT;
  const int cx = __double2int_rd(__dmul_rn(pts[3 * i + 0], inv_res));
  const int cy = __double2int_rd(__dmul_rn(pts[3 * i + 1], inv_res));
  const int cz = __double2int_rd(__dmul_rn(pts[3 * i + 2], inv_res));
  ep[i] = make_int4(cx, cy, cz, kind);
  dedup_min_insert(tab, tmask, cx, cy, cz, i, M);
}

// The lowest-index point of each endpoint cell decides and applies
// (winner_apply) and, if its ray is cast, joins the ray list.
// One block-wide atomic each for the ray list, the point count and the ray
// lengths (a per-warp atomic on three shared counters serialised in L2).
__global__ void __launch_bounds__(256) k_winners(const __grid_constant__ DMap M, const int4* __restrict__ ep, uint32_t n,
                          const uint4* __restrict__ tab, uint32_t tmask, int ox, int oy, int oz,
                          int32_t u, Opts o, int4* __restrict__ cast, uint32_t cast_cap) {
  __shared__ uint32_t s_cnt[8], s_pts[8], s_base;
  __shared__ unsigned long long s_len[8];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool add = false;
  int4 e = make_int4(0, 0, 0, EP_SKIP);
  if (i < n) {
    e = ep[i];
    if (e.w == EP_HIT || e.w == EP_MISS) {
      if (dedup_lookup(tab, tmask, e.x, e.y, e.z) == i) add = winner_apply(M, e, u, o);
    }
  }
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned valid = __ballot_sync(0xffffffffu, i < n && e.w != EP_SKIP);
  const unsigned am = __ballot_sync(0xffffffffu, add);
  const uint32_t len = add ? chebyshev(ox, oy, oz, e.x, e.y, e.z) : 0u;
  const unsigned long long wlen = __reduce_add_sync(0xffffffffu, len >> 16) * 65536ull +
                                  __reduce_add_sync(0xffffffffu, len & 0xFFFFu);
  if (lane == 0) {
    s_cnt[wid] = __popc(am);
    s_pts[wid] = __popc(valid);
    s_len[wid] = wlen;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0, pts = 0;
    unsigned long long tl = 0;
    for (unsigned w = 0; w < blockDim.x / 32; w++) {
      const uint32_t c = s_cnt[w];
      s_cnt[w] = tot;
      tot += c;
      pts += s_pts[w];
      tl += s_len[w];
    }
    unsigned long long* st = reinterpret_cast<unsigned long long*>(M.ctr + C_STATS);
    if (pts) atomicAdd(st + S_POINTS, static_cast<unsigned long long>(pts));
    if (tl) atomicAdd(st + S_RAY_LEN, tl);
    s_base = tot ? atomicAdd(M.ctr + C_CAST, tot) : 0u;
  }
  __syncthreads();
  if (add) {
    const uint32_t k = s_base + s_cnt[wid] + __popc(am & ((1u << lane) - 1));
    if (k < cast_cap)
      cast[k] = e;
    else
      set_err(M, ERR_SCRATCH);
  }
}

// Completes listed endpoints after a pool ran out: creates each cell and
// applies its hit or miss (probabilistic_map.cpp:35-41,49-54). Idempotent --
// a cell already at u is left alone -- so it may run over the whole list.
__global__ void k_apply(const __grid_constant__ DMap M, const int4* __restrict__ cast, uint32_t cast_cap, int32_t u,
                        Opts o) {
  const uint32_t n = min(ld_volatile(M.ctr + C_CAST), cast_cap);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int4 e = cast[k];
    const uint32_t lf = leaf_of(M, e.x, e.y, e.z, true);
    if (lf == kNone) continue;
    const uint32_t ci = leaf_index(M, e.x, e.y, e.z);
    cell_mark_on(M, lf, ci);
    int32_t* cp = reinterpret_cast<int32_t*>(M.ldata) + size_t(lf) * M.lsize + ci;
    const int32_t w = *cp;
    if (cell_id(w) != u) {
      const int32_t p = cell_prob(w);
      const int32_t np = e.w == EP_HIT ? min(wrap_add(p, o.hit), o.cmax)
                                       : max(wrap_add(p, o.miss), o.cmin);
      *cp = cell_pack(np, u);
    }
  }
}

// Ray phase: one group of W lanes per listed ray (walk_ray, or walk_ray2 with
// two cells per lane per step when U == 2).
// Also clears tab[0, tab_n), the endpoint dedup table of the scan, so that
// the next scan's endpoint phase starts from an empty table without a memset.
template <int W, int U>
__global__ void __launch_bounds__(U == 2 ? 256 : 1024, U == 2 ? 3 : 1) k_rays(const __grid_constant__ DMap M, const int4* __restrict__ cast,
                                                 uint32_t cast_cap, int ox, int oy, int oz,
                                                 int32_t u, int32_t miss, int32_t cmin,
                                                 uint4* __restrict__ tab, uint32_t tab_n,
                                                 LeafDir D) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < tab_n; t += gridDim.x * blockDim.x)
    tab[t] = make_uint4(kNone, kNone, kNone, kNone);
  const uint32_t n_cast = min(ld_volatile(M.ctr + C_CAST), cast_cap);
  const unsigned lane = threadIdx.x & 31;
  const unsigned sl = lane & (W - 1);
  const unsigned gbase = lane & ~(W - 1);
  const unsigned gmask = (W == 32) ? 0xffffffffu : (((1u << W) - 1u) << gbase);
  const uint32_t gid = (blockIdx.x * blockDim.x + threadIdx.x) / W;
  const uint32_t ngroups = (gridDim.x * blockDim.x) / W;
  uint32_t visited = 0, updated = 0;
  for (uint32_t r = gid; r < n_cast; r += ngroups) {
    if (U == 2)
      walk_ray2<W>(M, cast[r], ox, oy, oz, u, miss, cmin, sl, gbase, gmask, visited, updated);
    else
      walk_ray<W, true>(M, cast[r], ox, oy, oz, u, miss, cmin, sl, gbase, gmask, visited,
                        updated, D.words ? &D : nullptr);
  }
  visited = __reduce_add_sync(0xffffffffu, visited);
  updated = __reduce_add_sync(0xffffffffu, updated);
  if (lane == 0 && visited) {
    unsigned long long* st = reinterpret_cast<unsigned long long*>(M.ctr + C_STATS);
    atomicAdd(st + S_VISITED, static_cast<unsigned long long>(visited));
    atomicAdd(st + S_UPDATED, static_cast<unsigned long long>(updated));
  }
}

// Mark phase: block tasks of consecutive rays of the list (taken from the
// counter *task, zero at launch), marked by mark_rays_block. Also clears
// tab[0, tab_n), the scan's endpoint dedup table, for the next scan.
__global__ void __launch_bounds__(1024) k_mark(const __grid_constant__ DMap M, RayCube Q,
                                               const int4* __restrict__ cast, uint32_t cast_cap,
                                               int ox, int oy, int oz,
                                               uint4* __restrict__ tab, uint32_t tab_n,
                                               uint32_t* task) {
  __shared__ uint32_t sm[kMarkSmemWords];
  __shared__ MarkRays<1024> rays;
  __shared__ uint32_t s_task;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < tab_n; t += gridDim.x * blockDim.x)
    tab[t] = make_uint4(kNone, kNone, kNone, kNone);
  for (int t = threadIdx.x; t < kMarkSmemWords; t += blockDim.x) sm[t] = 0u;
  const uint32_t n_cast = min(ld_volatile(M.ctr + C_CAST), cast_cap);
  // one task per block (a task ends with the block's shared-memory flush)
  const uint32_t chunk = max(1u, (n_cast + gridDim.x - 1) / gridDim.x);
  const uint32_t n_tasks = (n_cast + chunk - 1) / chunk;
  uint32_t visited = 0;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_task = atomicAdd(task, 1u);
    __syncthreads();
    const uint32_t t = s_task;
    if (t >= n_tasks) break;
    const uint32_t r0 = t * chunk;
    mark_rays_block<kMarkNB, 1024>(M, Q, cast, r0, min(n_cast, r0 + chunk), ox, oy, oz, sm,
                                   rays, visited);
  }
  visited = __reduce_add_sync(0xffffffffu, visited);
  if ((threadIdx.x & 31) == 0 && visited)
    atomicAdd(reinterpret_cast<unsigned long long*>(M.ctr + C_STATS) + S_VISITED,
              static_cast<unsigned long long>(visited));
}

// List phase: the marked blocks onto the scan's list (one warp per 32 words
// of the touched bitmap).
__global__ void __launch_bounds__(256) k_list_touched(const __grid_constant__ DMap M, RayCube Q) {
  const uint32_t chunks = (cube_touched_words(Q) + 31u) / 32u;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = wid; c < chunks; c += nw) list_touched(M, Q, c);
}


// Apply phase: a group of kApplyGroup lanes per listed leaf block; D: the
// map's leaf directory (D.words == nullptr: none).
__global__ void __launch_bounds__(256) k_apply_rays(const __grid_constant__ DMap M, RayCube Q, int32_t u, int32_t miss,
                                                    int32_t cmin, LeafDir D) {
  const uint32_t n = min(ld_volatile(Q.count), Q.cap);
  const unsigned lane = threadIdx.x & 31;
  const unsigned sl = lane & (kApplyGroup - 1), gbase = lane & ~unsigned(kApplyGroup - 1);
  const unsigned gmask = ((1u << kApplyGroup) - 1u) << gbase;
  const uint32_t gid = (blockIdx.x * blockDim.x + threadIdx.x) / kApplyGroup;
  const uint32_t ng = (gridDim.x * blockDim.x) / kApplyGroup;
  uint32_t updated = 0;
  for (uint32_t i = gid; i < n; i += ng)
    apply_block(M, Q, Q.list[i], u, miss, cmin, sl, gbase, gmask, updated,
                D.words ? &D : nullptr);
  updated = __reduce_add_sync(0xffffffffu, updated);
  if (lane == 0 && updated)
    atomicAdd(reinterpret_cast<unsigned long long*>(M.ctr + C_STATS) + S_UPDATED,
              static_cast<unsigned long long>(updated));
}

// isOccupied / isUnknown / isFree (probabilistic_map.cpp:56-75).
__global__ void k_query(const __grid_constant__ DMap M, const int32_t* __restrict__ xyz, uint32_t n, int mode,
                        int32_t thr, uint8_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  const uint32_t lf = leaf_of(M, x, y, z, false);
  bool have = false;
  int32_t p = 0;
  if (lf != kNone) {
    // The cell word first: an on cell of a ProbabilisticMap has update_id in
    // 1..3 (a nonzero word), an off cell holds zero, so only a zero word
    // needs the mask bit (it may be an on cell written through the grid).
    const uint32_t ci = leaf_index(M, x, y, z);
    const int32_t w = reinterpret_cast<const int32_t*>(M.ldata)[size_t(lf) * M.lsize + ci];
    have = w != 0 || cell_is_on(M, lf, ci);
    p = cell_prob(w);
  }
  uint8_t r;
  if (mode == 0)
    r = have && p > thr;
  else if (mode == 1)
    r = have ? p == thr : 1;
  else
    r = have && p < thr;
  out[i] = r;
}

// ComputeRay for a batch of rays (probabilistic_map.hpp:13-19), thread per ray.
__global__ void k_compute_rays(const int32_t* __restrict__ o, const int32_t* __restrict__ e,
                               uint32_t n, uint32_t* __restrict__ len,
                               const unsigned long long* __restrict__ off,
                               int32_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ox = o[3 * i], oy = o[3 * i + 1], oz = o[3 * i + 2];
  const int dx = e[3 * i] - ox, dy = e[3 * i + 1] - oy, dz = e[3 * i + 2] - oz;
  const uint32_t ax = abs(dx), ay = abs(dy), az = abs(dz);
  const uint32_t m = max(ax, max(ay, az));
  if (len) len[i] = m;
  if (!out || m == 0 || m >= kMaxRayCells) return;
  const uint32_t two_m = 2u * m;
  const float rtm = __frcp_rn(static_cast<float>(two_m));
  AxisStep X, Y, Z;
  axis_init(X, ax, m, two_m, rtm, 0, 1);
  axis_init(Y, ay, m, two_m, rtm, 0, 1);
  axis_init(Z, az, m, two_m, rtm, 0, 1);
  int32_t* dst = out + 3 * off[i];
  for (uint32_t k = 0; k < m; k++) {
    dst[3 * k + 0] = ox + (dx < 0 ? -int(X.n) : int(X.n));
    dst[3 * k + 1] = oy + (dy < 0 ? -int(Y.n) : int(Y.n));
    dst[3 * k + 2] = oz + (dz < 0 ? -int(Z.n) : int(Z.n));
    axis_advance(X, two_m);
    axis_advance(Y, two_m);
    axis_advance(Z, two_m);
  }
}

}  // namespace bxg

using namespace bxg;

namespace {

uint32_t next_pow2(uint64_t v) {
  uint32_t p = 64;
  while (p < v) p <<= 1;
  return p;
}

Opts opts_of(const bxg_pmap_s* pm) {
  return Opts{pm->opt.prob_miss_log, pm->opt.prob_hit_log, pm->opt.clamp_min_log,
              pm->opt.clamp_max_log};
}

// logods(p) = int32_t(1e6 * log(p / (1.0 - p))) (probabilistic_map.hpp:34-36).
int32_t logods(float p) {
  return static_cast<int32_t>(1e6 * std::log(p / (1.0 - p)));
}

void record(bxg_pmap_s* pm, int k) {
  if ((pm->core.flags & BXG_FLAG_TIMING) && pm->ev[k]) cudaEventRecord(pm->ev[k], pm->core.stream);
}

int reset_scan_stats(MapCore* m) {
  BXG_CUDA(m, cudaMemsetAsync(m->ctr.as<uint32_t>() + C_STATS, 0, S_COUNT * 8, m->stream));
  return BXG_OK;
}

// Endpoint phase for n staged points (k_endpoints or k_endpoints_kind), then
// the winners that join the ray list, then the endpoint updates.
template <class Launch>
int endpoint_phase(bxg_pmap_s* pm, uint32_t n, int ox, int oy, int oz, Launch&& launch_ep) {
  MapCore* m = &pm->core;
  const uint32_t tcap = next_pow2(uint64_t(n) * 2);
  BXG_CUDA(m, m->s_ep.ensure(size_t(n) * 16));
  const void* old_tab = m->s_dedup.p;
  BXG_CUDA(m, m->s_dedup.ensure(size_t(tcap) * 16));
  if (m->s_dedup.p != old_tab) m->dedup_clean = 0;
  // the ray list persists across add-batches until updateFreeCells
  const uint64_t need = pm->cast_ub + n;
  BXG_CUDA(m, m->s_cast.ensure_keep(need * 16, pm->cast_ub * 16, m->stream));
  if (m->dedup_clean < tcap) launch_dedup_clear(m, m->s_dedup.as<uint4>(), tcap);
  m->dedup_clean = 0;
  m->dedup_used = std::max(m->dedup_used, tcap);
  const unsigned blocks = (n + 255) / 256;
  launch_ep(blocks, m->s_ep.as<int4>(), m->s_dedup.as<uint4>(), tcap - 1);
  BXG_LAUNCHED(m);
  record(pm, 1);
  k_winners<<<blocks, 256, 0, m->stream>>>(m->dm, m->s_ep.as<int4>(), n, m->s_dedup.as<uint4>(),
                                           tcap - 1, ox, oy, oz, pm->update_count, opts_of(pm),
                                           m->s_cast.as<int4>(), uint32_t(m->s_cast.cap / 16));
  BXG_LAUNCHED(m);
  record(pm, 2);
  pm->cast_ub = need;
  return BXG_OK;
}

int launch_apply(bxg_pmap_s* pm) {
  MapCore* m = &pm->core;
  const unsigned blocks =
      unsigned(std::min<uint64_t>((pm->cast_ub + 255) / 256, uint64_t(m->sm_count) * 8));
  if (blocks) {
    k_apply<<<std::max(blocks, 1u), 256, 0, m->stream>>>(
        m->dm, m->s_cast.as<int4>(), uint32_t(m->s_cast.cap / 16), pm->update_count,
        opts_of(pm));
    BXG_LAUNCHED(m);
  }
  return BXG_OK;
}

}  // namespace

namespace bxg {
// The leaf directory for a scan from (ox, oy, oz) whose ray cells lie within
// pm->dir_reach of the origin: a cube of words over leaf coordinates, each
// (epoch << 28) | leaf slot. The cube and its words are kept across scans: a
// scan reuses them while its own cube of leaves lies inside and no leaf slot
// was released since they were written (MapCore::leaf_gen). Otherwise a new
// cube, centred on this origin with a margin so that a moving sensor keeps it
// for several scans, takes the next epoch. The whole buffer is cleared when
// the 4-bit epoch wraps, so a word of another epoch is always empty. *D stays
// empty (the walk probes the root hash for every leaf run) when the cube would
// exceed max_words words or leaf slots do not fit in 28 bits.
int leaf_dir_for_scan(bxg_pmap_s* pm, int ox, int oy, int oz, LeafDir* D, size_t max_words,
                      cudaStream_t stream) {
  MapCore* m = &pm->core;
  if (!stream) stream = m->stream;
  *D = LeafDir{};
  if (!(pm->dir_reach > 0) || m->dm.lcap >= (1u << 28)) return BXG_OK;
  const double cells = std::ceil(pm->dir_reach * m->inv_res) + 2;
  const double halfd = std::ceil(cells / double(1 << m->dm.lb)) + 1;
  if (!(halfd < 128)) return BXG_OK;
  const int half = int(halfd);
  const int cx = ox >> m->dm.lb, cy = oy >> m->dm.lb, cz = oz >> m->dm.lb;
  const int side_now = int(pm->dir_side);
  auto inside = [&](int c, int lo) { return c - half >= lo && c + half < lo + side_now; };
  const bool reuse = pm->dir_live && pm->dir_gen == m->leaf_gen && inside(cx, pm->dir_x0) &&
                     inside(cy, pm->dir_y0) && inside(cz, pm->dir_z0);
  if (!reuse) {
    auto words_of = [](int h) { return size_t(2 * h + 1) * (2 * h + 1) * (2 * h + 1); };
    int h = half + std::max(2, half / 4);
    if (words_of(h) > max_words) h = half;
    if (words_of(h) > max_words) return BXG_OK;
    const size_t words = words_of(h);
    if (m->s_dir.cap < words * 4) {
      BXG_CUDA(m, m->s_dir.ensure(words * 4));
      BXG_CUDA(m, cudaMemsetAsync(m->s_dir.p, 0, m->s_dir.cap, stream));
      pm->dir_epoch = 0;
    }
    if (++pm->dir_epoch == 16) {  // the epoch wraps: clear every word ever written
      BXG_CUDA(m, cudaMemsetAsync(m->s_dir.p, 0, m->s_dir.cap, stream));
      pm->dir_epoch = 1;
    }
    pm->dir_x0 = cx - h;
    pm->dir_y0 = cy - h;
    pm->dir_z0 = cz - h;
    pm->dir_side = uint32_t(2 * h + 1);
    pm->dir_gen = m->leaf_gen;
    pm->dir_live = true;
  }
  D->words = m->s_dir.as<uint32_t>();
  D->side = pm->dir_side;
  D->x0 = pm->dir_x0;
  D->y0 = pm->dir_y0;
  D->z0 = pm->dir_z0;
  D->epoch = pm->dir_epoch;
  return BXG_OK;
}
}  // namespace bxg

namespace bxg {
// Largest cube side (leaves): 200^3 blocks of 64 B = 512 MB of bits. Scans
// whose cube would be larger (very fine resolutions with long ranges) walk
// their rays with k_rays instead.
constexpr uint32_t kMaxCubeSide = 200;

int cube_for_scan(bxg_pmap_s* pm, int ox, int oy, int oz, double reach, RayCube* Q, bool* ok) {
  MapCore* m = &pm->core;
  *ok = false;
  if (m->dm.lb != 3 || m->dm.esz != 4 ||
      (m->flags & (BXG_FLAG_KEEP_NONFINITE | BXG_FLAG_RAYS_SINGLE_PASS)))
    return BXG_OK;
  if (!(reach > 0) || !std::isfinite(reach)) return BXG_OK;
  // Ray ends lie within ceil(reach / res) + 2 cells of the origin cell (the
  // floor of the origin and of the end each move a cell by less than one), so
  // every ray cell lies within HL leaves of the origin's leaf.
  const double cells = std::ceil(reach * m->inv_res) + 2.0;
  if (!(cells < 8.0 * kMaxCubeSide)) return BXG_OK;
  const int R = int(cells);
  const int HL = std::max((R + 7) / 8 + 1, kMarkNB + 1);
  const uint32_t S = uint32_t(2 * HL + 1);
  if (S > kMaxCubeSide) return BXG_OK;
  const size_t blocks = size_t(S) * S * S;
  const uint32_t tmask = cube_touched_mask(S);
  if (blocks > pm->cube_blocks) {
    BXG_CUDA(m, pm->cube_bits.ensure(blocks * 64));
    BXG_CUDA(m, pm->cube_touch.ensure((size_t(tmask) + 1) / 8));
    BXG_CUDA(m, pm->cube_list.ensure(blocks * 4));
    BXG_CUDA(m, cudaMemsetAsync(pm->cube_bits.p, 0, pm->cube_bits.cap, m->stream));
    BXG_CUDA(m, cudaMemsetAsync(pm->cube_touch.p, 0, pm->cube_touch.cap, m->stream));
    // the batched tick uses the buffers from another stream
    BXG_CUDA(m, cudaStreamSynchronize(m->stream));
    pm->cube_blocks = blocks;
  }
  Q->bits = pm->cube_bits.as<uint32_t>();
  Q->touched = pm->cube_touch.as<uint32_t>();
  Q->list = pm->cube_list.as<uint32_t>();
  Q->count = m->ctr.as<uint32_t>() + C_LIST;
  Q->x0 = ((ox >> 3) - HL) * 8;
  Q->y0 = ((oy >> 3) - HL) * 8;
  Q->z0 = ((oz >> 3) - HL) * 8;
  Q->S = S;
  Q->cap = uint32_t(blocks);
  Q->tmask = tmask;
  *ok = true;
  return BXG_OK;
}
}  // namespace bxg

namespace {

using RayKernel = void (*)(DMap, const int4*, uint32_t, int, int, int, int32_t, int32_t, int32_t,
                           uint4*, uint32_t, LeafDir);

RayKernel ray_kernel(uint32_t rpw, bool u2) {
  if (rpw == 4) return u2 ? k_rays<8, 2> : k_rays<8, 1>;
  if (rpw == 2) return u2 ? k_rays<16, 2> : k_rays<16, 1>;
  return u2 ? k_rays<32, 2> : k_rays<32, 1>;
}

// Launch shape of the ray kernel: one resident wave (SM count x blocks per
// SM), each warp walking every (grid warps)-th ray of the list. Blocks of 1024
// threads (one per SM) let 32 warps walk 32 neighbouring rays of the list at
// once, which share cells and leaves in the SM's L1; scans with fewer ray
// slots than two such waves (the point count bounds the ray count) launch
// 256-thread blocks instead, so that their few rays still reach every SM
// (LiDAR scans: 256 threads faster at 4 k points, 1024 from 16 k points).
// U = 2 kernels hold 80 registers and launch 256 threads.
int launch_rays(bxg_pmap_s* pm, int ox, int oy, int oz) {
  MapCore* m = &pm->core;
  if (!pm->cast_ub) return BXG_OK;
  {
    // two-phase form: mark the rays' cells, then apply per leaf
    RayCube Q{};
    bool ok = false;
    int st = cube_for_scan(pm, ox, oy, oz, pm->dir_reach, &Q, &ok);
    if (st) return st;
    if (ok) {
      const Opts o = opts_of(pm);
      const uint32_t ccap = uint32_t(m->s_cast.cap / 16);
      const uint32_t tab_n = m->dedup_used;
      BXG_CUDA(m, cudaMemsetAsync(m->ctr.as<uint32_t>() + C_LIST, 0, 8, m->stream));
      const unsigned mblocks =
          unsigned(std::min<uint64_t>(m->sm_count, std::max<uint64_t>(1, pm->cast_ub / 64)));
      k_mark<<<mblocks, 1024, 0, m->stream>>>(m->dm, Q, m->s_cast.as<int4>(), ccap, ox, oy, oz,
                                             m->s_dedup.as<uint4>(), tab_n,
                                             m->ctr.as<uint32_t>() + C_TASK);
      BXG_LAUNCHED(m);
      const uint64_t chunks = (cube_touched_words(Q) + 31u) / 32u;
      const unsigned lblocks =
          unsigned(std::min<uint64_t>(uint64_t(m->sm_count) * 8, (chunks + 7) / 8));
      k_list_touched<<<std::max(lblocks, 1u), 256, 0, m->stream>>>(m->dm, Q);
      BXG_LAUNCHED(m);
      // 256 / kApplyGroup groups per block; the list holds at most
      // min(cube, 64 x rays) blocks
      const uint64_t groups = std::min<uint64_t>(Q.cap, pm->cast_ub * 64);
      const uint64_t per_block = 256 / kApplyGroup;
      const unsigned ablocks = unsigned(std::min<uint64_t>(
          uint64_t(m->sm_count) * 8, std::max<uint64_t>(1, (groups + per_block - 1) / per_block)));
      LeafDir dir{};
      st = leaf_dir_for_scan(pm, ox, oy, oz, &dir, size_t(1) << 24, m->stream);
      if (st) return st;
      k_apply_rays<<<ablocks, 256, 0, m->stream>>>(m->dm, Q, pm->update_count, o.miss, o.cmin,
                                                   dir);
      BXG_LAUNCHED(m);
      m->dedup_clean = std::max(m->dedup_clean, tab_n);
      m->dedup_used = 0;
      return BXG_OK;
    }
  }
  const uint32_t rpw = m->rays_per_warp ? m->rays_per_warp : 1;
  const bool u2 = m->ray_unroll == 2;
  const int bs_max = u2 ? 256 : 1024;
  const bool wide = pm->cast_ub >= uint64_t(2) * m->sm_count * 32 * rpw;
  const int bs = m->block_size ? std::min(bs_max, std::max(64, int(m->block_size) & ~31))
                               : (wide ? bs_max : 256);
  const RayKernel kern = ray_kernel(rpw, u2);
  const int wi = bs == 1024 ? 1 : 0;  // cached residency of the two default shapes
  if (m->ray_wave_bs[wi] != bs) {
    int per_sm = 0;
    BXG_CUDA(m, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &per_sm, reinterpret_cast<const void*>(kern), bs, 0));
    m->ray_wave_blocks[wi] = uint32_t(std::max(per_sm, 1)) * uint32_t(m->sm_count);
    m->ray_wave_bs[wi] = bs;
  }
  const uint64_t groups_per_block = uint64_t(bs) / (32 / rpw);
  uint64_t blocks = (pm->cast_ub + groups_per_block - 1) / groups_per_block;
  blocks = std::min<uint64_t>(blocks, m->ray_wave_blocks[wi]);
  if (!blocks) return BXG_OK;
  const Opts o = opts_of(pm);
  const uint32_t ccap = uint32_t(m->s_cast.cap / 16);
  const dim3 g{unsigned(blocks)}, b{unsigned(bs)};
  const uint32_t tab_n = m->dedup_used;
  LeafDir dir{};
  int st = leaf_dir_for_scan(pm, ox, oy, oz, &dir, size_t(1) << 24, m->stream);
  if (st) return st;
  kern<<<g, b, 0, m->stream>>>(m->dm, m->s_cast.as<int4>(), ccap, ox, oy, oz, pm->update_count,
                               o.miss, o.cmin, m->s_dedup.as<uint4>(), tab_n, dir);
  BXG_LAUNCHED(m);
  m->dedup_clean = std::max(m->dedup_clean, tab_n);
  m->dedup_used = 0;
  return BXG_OK;
}

// Applies the queued endpoints (if not yet applied) and casts the rays,
// growing pools and retrying on exhaustion; then ends the scan.
int finish_scan(bxg_pmap_s* pm, int ox, int oy, int oz, bool cast_rays, uint64_t* ray_cells,
                bool include_points) {
  MapCore* m = &pm->core;
  int st = BXG_OK;
  for (int attempt = 0; attempt < 12; attempt++) {
    if (attempt) {
      // a retry walks every ray again (recount the visits) but updates only
      // the cells the failed attempt could not reach: the updated-cell count
      // adds up over the attempts
      unsigned long long* s = stats_of(m);
      BXG_CUDA(m, cudaMemsetAsync(s + S_VISITED, 0, 8, m->stream));
    }
    if (attempt) {  // the winners applied the endpoints; complete them after growth
      st = launch_apply(pm);
      if (st) return st;
    }
    record(pm, 3);
    if (cast_rays) {
      st = launch_rays(pm, ox, oy, oz);
      if (st) return st;
    }
    record(pm, 4);
    uint32_t err = 0;
    st = core_sync(m, &err);
    if (st == BXG_OK) break;
    if (!(err & (ERR_POOL_INNER | ERR_POOL_LEAF | ERR_HASH_FULL)) ||
        (err & (ERR_WAIT | ERR_RAY_TOO_LONG | ERR_SCRATCH)))
      return st;
    const int g = core_grow_for(m, err);
    if (g) return g;
  }
  if (st) return st;
  const unsigned long long* hs = reinterpret_cast<const unsigned long long*>(m->h_ctr + C_STATS);
  pm->last_stats[0] = hs[S_POINTS];
  pm->last_stats[1] = pm->cast_ub ? m->h_ctr[C_CAST] : 0;
  pm->last_stats[2] = hs[S_VISITED];
  pm->last_stats[3] = hs[S_UPDATED];
  pm->last_stats[4] = m->h_ctr[C_LEAF];
  pm->last_stats[5] = m->launches;
  if (ray_cells) *ray_cells = (include_points ? hs[S_POINTS] : 0) + hs[S_RAY_LEN];
  if (m->flags & BXG_FLAG_TIMING) {
    for (int k = 0; k < 4; k++) {
      float ms = 0;
      if (pm->ev[k] && pm->ev[k + 1]) cudaEventElapsedTime(&ms, pm->ev[k], pm->ev[k + 1]);
      pm->last_times[k] = ms;
    }
  }
  if (cast_rays) {
    // end of scan: empty the ray list (the next scan's first kernel zeroes
    // the device count), advance the counter (cpp:301-310)
    pm->cast_ub = 0;
    pm->dir_reach = 0.0;
    if (++pm->update_count == 4) pm->update_count = 1;
  }
  return core_maintain(m);
}

// Σ Chebyshev length from origin cell o of the rays queued by addHitPoint /
// addMissPoint batches (their add-time lengths were measured from (0,0,0)):
// read back and summed on the host; this path is not the streaming one.
int queued_ray_cells(bxg_pmap_s* pm, const int* o, uint64_t* len) {
  MapCore* m = &pm->core;
  *len = 0;
  if (!pm->cast_ub) return BXG_OK;
  int st = core_sync(m);
  if (st) return st;
  const uint32_t n_cast = m->h_ctr[C_CAST];
  if (!n_cast) return BXG_OK;
  std::vector<int4> h(n_cast);
  BXG_CUDA(m, cudaMemcpy(h.data(), m->s_cast.p, size_t(n_cast) * 16, cudaMemcpyDeviceToHost));
  for (const int4& e : h) {
    const int64_t dx = std::llabs(int64_t(e.x) - o[0]), dy = std::llabs(int64_t(e.y) - o[1]),
                  dz = std::llabs(int64_t(e.z) - o[2]);
    *len += uint64_t(std::max(dx, std::max(dy, dz)));
  }
  return BXG_OK;
}

int origin_coord(const MapCore* m, double x, double y, double z, int* c) {
  c[0] = static_cast<int>(std::floor(x * m->inv_res));
  c[1] = static_cast<int>(std::floor(y * m->inv_res));
  c[2] = static_cast<int>(std::floor(z * m->inv_res));
  return BXG_OK;
}

template <typename PT>
int insert_impl(bxg_pmap m_, const PT* xyz, size_t stride, size_t n, const PT* origin,
                double max_range, uint64_t* ray_cells, bool sync, const Xf* xf = nullptr) {
  if (!m_) return BXG_ERR_INVALID_ARG;
  bxg_pmap_s* pm = m_;
  MapCore* m = &pm->core;
  if (!origin || (n && !xyz) || n >= 0x7FFFFFFFu)
    return set_error(m, BXG_ERR_INVALID_ARG, "null input or batch too large");
  if (!stride) stride = 3 * sizeof(PT);
  cudaSetDevice(m->device);
  // from = ConvertPoint<Vector3d>(origin): the origin widened to double.
  const double fx = static_cast<double>(origin[0]), fy = static_cast<double>(origin[1]),
               fz = static_cast<double>(origin[2]);
  int o[3];
  origin_coord(m, fx, fy, fz, o);
  // rays queued by earlier addHitPoint/addMissPoint batches are cast by this
  // scan too (updateFreeCells, probabilistic_map.hpp:159): count their cells
  uint64_t queued = 0;
  if (ray_cells && pm->cast_ub) {
    const int qs = queued_ray_cells(pm, o, &queued);
    if (qs) return qs;
  }
  // Headroom for this scan's new leaves (twice the last scan's, at least a
  // quarter of the points), so that the scan rarely has to grow and re-run.
  const uint32_t leaves_before = m->h_ctr[C_LEAF];
  int st = core_reserve(m, std::max<size_t>({size_t(2) * pm->last_new_leaves, n / 4, 1024}),
                        std::max<size_t>(n / 64, 256));
  if (st) return st;
  record(pm, 0);  // the scan's device time starts here
  if (!n) {  // otherwise the endpoint kernel zeroes the statistics
    st = reset_scan_stats(m);
    if (st) return st;
  }
  if (n) {
    const void* dpts = nullptr;
    st = stage_in(m, m->s_in, xyz, stride * (n - 1) + 3 * sizeof(PT), &dpts);
    if (st) return st;
    const double mr2 = max_range * max_range;
    const int keep = (m->flags & BXG_FLAG_KEEP_NONFINITE) ? 1 : 0;
    // rays of this scan end within max_range of the origin (hits are closer);
    // rays queued by earlier add batches may not: no directory then
    pm->dir_reach = pm->cast_ub == 0 ? max_range : 0.0;
    const int zero = ZERO_STATS | (pm->cast_ub == 0 ? ZERO_CAST : 0);
    EpFast fast = make_ep_fast(fx, fy, fz, max_range, m->inv_res);
    if (sizeof(PT) != 4) fast.on = 0;
    st = endpoint_phase(pm, uint32_t(n), o[0], o[1], o[2],
                        [&](unsigned blocks, int4* ep, uint4* tab, uint32_t tmask) {
                          if (xf)
                            k_endpoints_sensor<<<blocks, 256, 0, m->stream>>>(
                                m->dm, static_cast<const uint8_t*>(dpts), stride, uint32_t(n),
                                *xf, fx, fy, fz, max_range, mr2, m->inv_res, ep, tab, tmask, zero,
                                fast);
                          else
                            k_endpoints<PT><<<blocks, 256, 0, m->stream>>>(
                                m->dm, static_cast<const uint8_t*>(dpts), stride, uint32_t(n), fx,
                                fy, fz, max_range, mr2, m->inv_res, keep, ep, tab, tmask, zero,
                                fast);
                        });
    if (st) return st;
  }
  if (!sync) {
    // asynchronous form: no retry; pools must have room (see core_maintain)
    st = launch_rays(pm, o[0], o[1], o[2]);
    if (st) return st;
    BXG_CUDA(m, cudaMemsetAsync(m->ctr.as<uint32_t>() + C_CAST, 0, 4, m->stream));
    pm->cast_ub = 0;
    if (++pm->update_count == 4) pm->update_count = 1;
    return BXG_OK;
  }
  st = finish_scan(pm, o[0], o[1], o[2], true, ray_cells, true);
  if (!st) {
    pm->last_new_leaves = m->h_ctr[C_LEAF] > leaves_before ? m->h_ctr[C_LEAF] - leaves_before : 0;
    if (ray_cells) *ray_cells += queued;
  }
  return st;
}

int add_points(bxg_pmap m_, const double* xyz, size_t n, int kind,
               const uint8_t* kinds = nullptr) {
  if (!m_) return BXG_ERR_INVALID_ARG;
  bxg_pmap_s* pm = m_;
  MapCore* m = &pm->core;
  if (!n) return BXG_OK;
  if (!xyz || n >= 0x7FFFFFFFu) return set_error(m, BXG_ERR_INVALID_ARG, "null input");
  cudaSetDevice(m->device);
  record(pm, 0);
  // rays queued here may end anywhere: the coming ray phase has no bound
  pm->dir_reach = 0.0;
  // the first batch after a scan starts the statistics and the ray list
  const int zero = pm->cast_ub == 0 ? (ZERO_STATS | ZERO_CAST) : 0;
  const void* dpts = nullptr;
  const void* dkinds = nullptr;
  int st = stage_in(m, m->s_in, xyz, n * 24, &dpts);
  if (st) return st;
  if (kinds) {
    st = stage_in(m, m->s_in2, kinds, n, &dkinds);
    if (st) return st;
  }
  st = endpoint_phase(pm, uint32_t(n), 0, 0, 0,
                      [&](unsigned blocks, int4* ep, uint4* tab, uint32_t tmask) {
                        k_endpoints_kind<<<blocks, 256, 0, m->stream>>>(
                            m->dm, static_cast<const double*>(dpts), uint32_t(n), kind,
                            static_cast<const uint8_t*>(dkinds), m->inv_res, ep, tab, tmask,
                            zero);
                      });
  if (st) return st;
  // apply now so that queries see the endpoint updates, as in the reference
  return finish_scan(pm, 0, 0, 0, false, nullptr, false);
}

// The occupied-voxel export of bonxai_server.cpp:217-243 as one compaction:
// each occupied cell (probability_log > thr, probabilistic_map.cpp:108-116)
// becomes its corner position coordToPos(c) = double(c) * res
// (bonxai.hpp:413-417), kept when min_z <= z <= max_z, narrowed to float
// xyz (the PCLPoint the node publishes). One thread per leaf mask word; a
// warp reserves its output range with one atomic. Order is unspecified, as
// the reference's unordered_map order is.
__global__ void k_export_occupied(const __grid_constant__ DMap M, uint32_t n_leaves, float* __restrict__ out, size_t cap,
                                  unsigned long long* __restrict__ counter, int32_t thr,
                                  double res, double min_z, double max_z) {
  const size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  const uint32_t leaf = static_cast<uint32_t>(t / M.lwords);
  const uint32_t wi = static_cast<uint32_t>(t % M.lwords);
  const int lm = (1 << M.lb) - 1;
  unsigned long long w = 0;
  int4 key = make_int4(0, 0, 0, -1);
  if (leaf < n_leaves) {
    key = M.lkey[leaf];
    if (key.w != -1) w = M.lmask[static_cast<size_t>(leaf) * M.lwords + wi];
  }
  if (w) {
    const int32_t* cells = reinterpret_cast<const int32_t*>(M.ldata) +
                           static_cast<size_t>(leaf) * M.lsize + wi * 64;
    unsigned long long f = 0, rest = w;
    while (rest) {
      const int b = __ffsll(static_cast<long long>(rest)) - 1;
      rest &= rest - 1;
      const uint32_t ci = wi * 64 + b;
      const double pz = __dmul_rn(double(key.z | int((ci >> (2 * M.lb)) & lm)), res);
      if (cell_prob(cells[b]) > thr && pz >= min_z && pz <= max_z) f |= 1ull << b;
    }
    w = f;
  }
  const unsigned cnt = __popcll(w);
  const unsigned lane = threadIdx.x & 31;
  unsigned incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= static_cast<unsigned>(o)) incl += v;
  }
  const unsigned total = __shfl_sync(0xffffffffu, incl, 31);
  unsigned long long base = 0;
  if (lane == 31 && total) base = atomicAdd(counter, static_cast<unsigned long long>(total));
  base = __shfl_sync(0xffffffffu, base, 31);
  unsigned long long pos = base + incl - cnt;
  while (w) {
    const int b = __ffsll(static_cast<long long>(w)) - 1;
    w &= w - 1;
    const uint32_t ci = wi * 64 + b;
    if (pos < cap) {
      out[3 * pos + 0] = float(__dmul_rn(double(key.x | int(ci & lm)), res));
      out[3 * pos + 1] = float(__dmul_rn(double(key.y | int((ci >> M.lb) & lm)), res));
      out[3 * pos + 2] = float(__dmul_rn(double(key.z | int((ci >> (2 * M.lb)) & lm)), res));
    }
    pos++;
  }
}

int export_occupied(bxg_pmap m_, float* out_xyz, size_t cap, size_t* n_out, double min_z,
                    double max_z) {
  MapCore* m = &m_->core;
  int st = core_sync(m);
  if (st) return st;
  const uint32_t n_leaves = m->h_ctr[C_LEAF];
  void* dout = nullptr;
  if (cap && out_xyz) {
    st = stage_out(m, m->s_out, out_xyz, cap * 12, &dout);
    if (st) return st;
  }
  BXG_CUDA(m, m->s_tmp.ensure(8));
  BXG_CUDA(m, cudaMemsetAsync(m->s_tmp.p, 0, 8, m->stream));
  const size_t threads = size_t(n_leaves) * m->dm.lwords;
  const size_t wcap = dout ? cap : 0;
  if (threads) {
    k_export_occupied<<<unsigned((threads + 255) / 256), 256, 0, m->stream>>>(
        m->dm, n_leaves, static_cast<float*>(dout), wcap, m->s_tmp.as<unsigned long long>(),
        m_->opt.occupancy_threshold_log, m->res, min_z, max_z);
    BXG_LAUNCHED(m);
  }
  unsigned long long n = 0;
  BXG_CUDA(m, cudaMemcpyAsync(&n, m->s_tmp.p, 8, cudaMemcpyDeviceToHost, m->stream));
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  if (dout) {
    st = stage_out_finish(m, out_xyz, dout, std::min<size_t>(size_t(n), wcap) * 12);
    if (st) return st;
  }
  if (n_out) *n_out = size_t(n);
  if (size_t(n) > cap) return set_error(m, BXG_ERR_CAPACITY, "output buffer too small");
  return BXG_OK;
}

int query(bxg_pmap m_, const int32_t* xyz, size_t n, uint8_t* out, int mode) {
  if (!m_) return BXG_ERR_INVALID_ARG;
  MapCore* m = &m_->core;
  if (!n) return BXG_OK;
  if (!xyz || !out || n >= 0x7FFFFFFFu) return set_error(m, BXG_ERR_INVALID_ARG, "null pointer");
  cudaSetDevice(m->device);
  const void* dxyz = nullptr;
  void* dout = nullptr;
  int st = stage_in(m, m->s_in, xyz, n * 12, &dxyz);
  if (st) return st;
  st = stage_out(m, m->s_out, out, n, &dout);
  if (st) return st;
  record(m_, 0);
  k_query<<<unsigned((n + 255) / 256), 256, 0, m->stream>>>(
      m->dm, static_cast<const int32_t*>(dxyz), uint32_t(n), mode,
      m_->opt.occupancy_threshold_log, static_cast<uint8_t*>(dout));
  BXG_LAUNCHED(m);
  record(m_, 1);
  st = stage_out_finish(m, out, dout, n);
  if (st) return st;
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  if ((m->flags & BXG_FLAG_TIMING) && m_->ev[0] && m_->ev[1])
    cudaEventElapsedTime(&m_->last_query_ms, m_->ev[0], m_->ev[1]);
  return BXG_OK;
}

}  // namespace

namespace bxg {
int pmap_complete_scan(bxg_pmap_s* pm, const int4* d_cast, const uint32_t* d_count, uint32_t cap,
                       int ox, int oy, int oz, int32_t u) {
  MapCore* m = &pm->core;
  cudaSetDevice(m->device);
  const Opts o = opts_of(pm);
  uint32_t err = 0;
  int st = core_sync(m, &err);  // reads and clears what the tick left
  if (st && (!(err & (ERR_POOL_INNER | ERR_POOL_LEAF | ERR_HASH_FULL)) ||
              (err & (ERR_WAIT | ERR_RAY_TOO_LONG | ERR_SCRATCH))))
    return st;
  BXG_CUDA(m, cudaMemcpyAsync(m->ctr.as<uint32_t>() + C_CAST, d_count, 4,
                              cudaMemcpyDeviceToDevice, m->stream));
  for (int attempt = 0; attempt < 12 && err; attempt++) {
    st = core_grow_for(m, err);
    if (st) return st;
    const unsigned ablocks = unsigned(std::min<uint64_t>((cap + 255) / 256, uint64_t(m->sm_count) * 8));
    k_apply<<<std::max(ablocks, 1u), 256, 0, m->stream>>>(m->dm, d_cast, cap, u, o);
    BXG_LAUNCHED(m);
    const unsigned rblocks = unsigned(std::min<uint64_t>((cap + 7) / 8, uint64_t(m->sm_count) * 8));
    k_rays<32, 1><<<std::max(rblocks, 1u), 256, 0, m->stream>>>(m->dm, d_cast, cap, ox, oy, oz,
                                                               u, o.miss, o.cmin, nullptr, 0,
                                                               LeafDir{});
    BXG_LAUNCHED(m);
    st = core_sync(m, &err);
    if (st && (!(err & (ERR_POOL_INNER | ERR_POOL_LEAF | ERR_HASH_FULL)) ||
              (err & (ERR_WAIT | ERR_RAY_TOO_LONG | ERR_SCRATCH))))
    return st;
  }
  BXG_CUDA(m, cudaMemsetAsync(m->ctr.as<uint32_t>() + C_CAST, 0, 4, m->stream));
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  if (err) return set_error(m, BXG_ERR_OUT_OF_POOL, "pools could not grow enough");
  return BXG_OK;
}

const MapCore* core_of_handle(const void* handle) {
  // Both handle types hold their MapCore as first member.
  return reinterpret_cast<const MapCore*>(handle);
}
}  // namespace bxg

extern "C" {

int bxg_pmap_create(bxg_pmap* out, double resolution, const bxg_config* cfg) {
  if (!out) return BXG_ERR_INVALID_ARG;
  *out = nullptr;
  bxg_pmap pm = new bxg_pmap_s();
  // ProbabilisticMap's grid is VoxelGrid<CellT>(resolution) with default bits.
  int st = core_init(&pm->core, resolution, 2, 3, 4, cfg);
  if (st) {
    set_create_error(pm->core.err);
    delete pm;
    return st;
  }
  pm->opt.prob_miss_log = logods(0.4f);
  pm->opt.prob_hit_log = logods(0.7f);
  pm->opt.clamp_min_log = logods(0.12f);
  pm->opt.clamp_max_log = logods(0.97f);
  pm->opt.occupancy_threshold_log = logods(0.5f);
  if (pm->core.flags & BXG_FLAG_TIMING)
    for (auto& e : pm->ev) cudaEventCreate(&e);
  *out = pm;
  return BXG_OK;
}

int bxg_pmap_destroy(bxg_pmap m) {
  delete m;
  return BXG_OK;
}

int bxg_pmap_get_options(bxg_pmap m, bxg_pmap_options* out) {
  if (!m || !out) return BXG_ERR_INVALID_ARG;
  *out = m->opt;
  return BXG_OK;
}

int bxg_pmap_set_options(bxg_pmap m, const bxg_pmap_options* opt) {
  if (!m || !opt) return BXG_ERR_INVALID_ARG;
  m->opt = *opt;
  return BXG_OK;
}

int bxg_pmap_insert_point_cloud_f32(bxg_pmap m, const float* xyz, size_t stride, size_t n,
                                    const float origin[3], double max_range,
                                    uint64_t* ray_cells) {
  return insert_impl(m, xyz, stride, n, origin, max_range, ray_cells, true);
}

int bxg_pmap_insert_point_cloud_f64(bxg_pmap m, const double* xyz, size_t stride, size_t n,
                                    const double origin[3], double max_range,
                                    uint64_t* ray_cells) {
  return insert_impl(m, xyz, stride, n, origin, max_range, ray_cells, true);
}

int bxg_pmap_insert_point_cloud_f32_async(bxg_pmap m, const float* xyz, size_t stride,
                                          size_t n, const float origin[3], double max_range) {
  return insert_impl(m, xyz, stride, n, origin, max_range, nullptr, false);
}

int bxg_pmap_insert_sensor_cloud_f32(bxg_pmap m, const float* xyz, size_t stride, size_t n,
                                     const float sensor_to_world[12], double max_range,
                                     uint64_t* ray_cells) {
  if (!m || !sensor_to_world) return BXG_ERR_INVALID_ARG;
  Xf xf;
  std::memcpy(xf.m, sensor_to_world, sizeof(xf.m));
  // origin = the transform's translation (bonxai_server.cpp:171-173); a
  // negative max_range means no limit (:174-179)
  const float origin[3] = {xf.m[3], xf.m[7], xf.m[11]};
  if (max_range < 0) max_range = HUGE_VAL;
  return insert_impl(m, xyz, stride, n, origin, max_range, ray_cells, true, &xf);
}

int bxg_pmap_export_occupied_f32(bxg_pmap m, float* out_xyz, size_t cap, size_t* n_out,
                                 double min_z, double max_z) {
  if (!m) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(m->core.device);
  return export_occupied(m, out_xyz, cap, n_out, min_z, max_z);
}

int bxg_pmap_add_hit_points(bxg_pmap m, const double* xyz, size_t n) {
  return add_points(m, xyz, n, EP_HIT);
}

int bxg_pmap_add_miss_points(bxg_pmap m, const double* xyz, size_t n) {
  return add_points(m, xyz, n, EP_MISS);
}

int bxg_pmap_add_points(bxg_pmap m, const double* xyz, const uint8_t* kinds, size_t n) {
  if (n && !kinds) return BXG_ERR_INVALID_ARG;
  return add_points(m, xyz, n, EP_HIT, kinds);
}

bxg_grid bxg_pmap_grid(bxg_pmap m) {
  // Both handle types hold their MapCore first and the grid entry points use
  // only that, so the map itself serves as its VoxelGrid<CellT>.
  return reinterpret_cast<bxg_grid>(m);
}

int bxg_pmap_update_free_cells(bxg_pmap pm, const double origin[3], uint64_t* ray_cells) {
  if (!pm || !origin) return BXG_ERR_INVALID_ARG;
  MapCore* m = &pm->core;
  cudaSetDevice(m->device);
  int o[3];
  origin_coord(m, origin[0], origin[1], origin[2], o);
  uint64_t len = 0;
  if (ray_cells) {
    const int st = queued_ray_cells(pm, o, &len);
    if (st) return st;
  }
  const int st = finish_scan(pm, o[0], o[1], o[2], true, nullptr, false);
  if (st) return st;
  if (ray_cells) *ray_cells = len;
  return BXG_OK;
}

int bxg_pmap_is_occupied(bxg_pmap m, const int32_t* xyz, size_t n, uint8_t* out) {
  return query(m, xyz, n, out, 0);
}
int bxg_pmap_is_unknown(bxg_pmap m, const int32_t* xyz, size_t n, uint8_t* out) {
  return query(m, xyz, n, out, 1);
}
int bxg_pmap_is_free(bxg_pmap m, const int32_t* xyz, size_t n, uint8_t* out) {
  return query(m, xyz, n, out, 2);
}

int bxg_pmap_get_occupied(bxg_pmap m, int32_t* out_xyz, size_t cap, size_t* n_out) {
  if (!m) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(m->core.device);
  return core_dump(&m->core, out_xyz, nullptr, cap, n_out, 1, m->opt.occupancy_threshold_log);
}

int bxg_pmap_get_free(bxg_pmap m, int32_t* out_xyz, size_t cap, size_t* n_out) {
  if (!m) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(m->core.device);
  return core_dump(&m->core, out_xyz, nullptr, cap, n_out, 2, m->opt.occupancy_threshold_log);
}

int bxg_pmap_dump(bxg_pmap m, int32_t* out_xyz, int32_t* out_cells, size_t cap, size_t* n_out) {
  if (!m) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(m->core.device);
  return core_dump(&m->core, out_xyz, out_cells, cap, n_out, 0, 0);
}

int bxg_pmap_active_cells(bxg_pmap m, size_t* out) {
  if (!m) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(m->core.device);
  return core_active_cells(&m->core, out);
}

int bxg_pmap_node_counts(bxg_pmap m, size_t* roots, size_t* leaves) {
  if (!m) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(m->core.device);
  return core_node_counts(&m->core, roots, leaves);
}

int bxg_pmap_mem_usage(bxg_pmap m, size_t* out) {
  if (!m || !out) return BXG_ERR_INVALID_ARG;
  *out = core_mem_usage(&m->core);
  return BXG_OK;
}

int bxg_pmap_update_count(bxg_pmap m, int* out) {
  if (!m || !out) return BXG_ERR_INVALID_ARG;
  *out = m->update_count;
  return BXG_OK;
}

int bxg_pmap_clear(bxg_pmap m) {
  if (!m) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(m->core.device);
  m->cast_ub = 0;
  return core_clear(&m->core);
}

int bxg_pmap_synchronize(bxg_pmap m) {
  if (!m) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(m->core.device);
  int st = core_sync(&m->core);
  if (st) return st;
  return core_maintain(&m->core);
}

int bxg_pmap_last_stats(bxg_pmap m, uint64_t out[8]) {
  if (!m || !out) return BXG_ERR_INVALID_ARG;
  std::memcpy(out, m->last_stats, sizeof(m->last_stats));
  return BXG_OK;
}

int bxg_pmap_last_query_ms(bxg_pmap m, float* ms) {
  if (!m || !ms) return BXG_ERR_INVALID_ARG;
  *ms = m->last_query_ms;
  return BXG_OK;
}

int bxg_pmap_kernel_times(bxg_pmap m, float out[4]) {
  if (!m || !out) return BXG_ERR_INVALID_ARG;
  std::memcpy(out, m->last_times, sizeof(m->last_times));
  return BXG_OK;
}

void* bxg_pmap_stream(bxg_pmap m) { return m ? static_cast<void*>(m->core.stream) : nullptr; }

int bxg_compute_rays(const int32_t* origin_xyz, const int32_t* end_xyz, size_t n,
                     uint32_t* out_len, const uint64_t* offsets, int32_t* out_xyz) {
  if (!n) return BXG_OK;
  if (!origin_xyz || !end_xyz || n >= 0x7FFFFFFFu) return BXG_ERR_INVALID_ARG;
  if (out_xyz && !offsets) return BXG_ERR_INVALID_ARG;
  MapCore tmp;
  tmp.device = -1;
  cudaGetDevice(&tmp.device);
  cudaStream_t s = nullptr;
  BXG_CUDA(&tmp, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  tmp.stream = s;
  tmp.own_stream = true;
  const void *dO = nullptr, *dE = nullptr, *dOff = nullptr;
  void *dLen = nullptr, *dOut = nullptr;
  int st = stage_in(&tmp, tmp.s_in, origin_xyz, n * 12, &dO);
  if (!st) st = stage_in(&tmp, tmp.s_in2, end_xyz, n * 12, &dE);
  if (!st) st = stage_out(&tmp, tmp.s_out, out_len, n * 4, &dLen);
  size_t total = 0;
  if (!st && out_xyz) {
    // total cells = offsets[n-1] + length of the last ray
    uint64_t last_off = 0;
    if (is_device_ptr(offsets))
      cudaMemcpy(&last_off, offsets + (n - 1), 8, cudaMemcpyDeviceToHost);
    else
      last_off = offsets[n - 1];
    int32_t lo[3], le[3];
    if (is_device_ptr(origin_xyz)) {
      cudaMemcpy(lo, origin_xyz + 3 * (n - 1), 12, cudaMemcpyDeviceToHost);
      cudaMemcpy(le, end_xyz + 3 * (n - 1), 12, cudaMemcpyDeviceToHost);
    } else {
      std::memcpy(lo, origin_xyz + 3 * (n - 1), 12);
      std::memcpy(le, end_xyz + 3 * (n - 1), 12);
    }
    const uint64_t ml = std::max({std::llabs(int64_t(le[0]) - lo[0]),
                                  std::llabs(int64_t(le[1]) - lo[1]),
                                  std::llabs(int64_t(le[2]) - lo[2])});
    total = size_t(last_off + ml);
    st = stage_in(&tmp, tmp.s_ep, offsets, n * 8, &dOff);
    if (!st) st = stage_out(&tmp, tmp.s_out2, out_xyz, total * 12, &dOut);
  }
  if (st) return st;
  k_compute_rays<<<unsigned((n + 255) / 256), 256, 0, s>>>(
      static_cast<const int32_t*>(dO), static_cast<const int32_t*>(dE), uint32_t(n),
      static_cast<uint32_t*>(dLen), static_cast<const unsigned long long*>(dOff),
      static_cast<int32_t*>(dOut));
  BXG_LAUNCHED(&tmp);
  if (dLen) st = stage_out_finish(&tmp, out_len, dLen, n * 4);
  if (!st && dOut) st = stage_out_finish(&tmp, out_xyz, dOut, total * 12);
  if (st) return st;
  BXG_CUDA(&tmp, cudaStreamSynchronize(s));
  return BXG_OK;
}

}  // extern "C"
