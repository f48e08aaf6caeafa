// Two-phase ray update of a ProbabilisticMap scan (updateFreeCells,
// probabilistic_map.cpp:77-106): first mark, then apply.
//
// The ray update is a function of each visited cell's own word (a cell whose
// update_id != u becomes {max(p + miss, clamp_min), u}; bxg_scan.cuh), so it
// only needs the SET of cells the scan's rays visit, not the visits:
//
//   mark   Rays are walked without touching the tree. Every visited cell sets
//          its bit in a per-scan bitmap over a cube around the origin, blocked
//          by leaf (one 512-bit block of 16 words per 8^3 leaf, bit =
//          getLeafIndex, x fastest). A lane walks a segment of kMarkSeg
//          consecutive cells of one ray (closed-form Bresenham start, then the
//          RayIterator step), collects the bits that fall in one word and
//          stores them with one fire-and-forget OR. Words of the leaves next
//          to the origin, which every ray crosses, are collected in shared
//          memory first and ORed into the bitmap once per block task. The
//          first OR into a block puts the block on the scan's list
//          (test-and-set on a per-block bit).
//   apply  One group of 8 lanes per listed block: a cooperative probe of the
//          root hash (8 buckets per step), the leaf get-or-create (topology:
//          once per leaf, not once per ray crossing), then the miss update of
//          the marked cells with vector loads and stores, the mask bits of
//          cells turned on, and the block cleared for the next scan.
//
// This is the two-phase insert (topology, then values) over deduplicated
// coordinates: the bitmap is the deduplication. The result equals the per-ray
// walk's bit for bit; the cube, its bits and its list are scratch that is all
// zero between scans.
#pragma once

#include "bxg_scan.cuh"

namespace bxg {

constexpr uint32_t kMarkSeg = 16;  // cells one lane walks per segment
// Shared-memory neighbourhood of the origin: the leaves within NB of the
// origin's leaf, (2 NB + 1)^3 blocks of 16 words. NB = 3 (21.4 KiB) for the
// per-scan kernel's 1024-thread blocks, NB = 2 (7.8 KiB) in the batched tick,
// whose 256-thread blocks also hold the tick's scan table.
constexpr int kMarkNB = 3;
__host__ __device__ constexpr int mark_smem_words(int nb) {
  return (2 * nb + 1) * (2 * nb + 1) * (2 * nb + 1) * 16;
}
constexpr int kMarkSmemWords = mark_smem_words(kMarkNB);
constexpr uint32_t kMarkWarpRays = 4;  // rays a warp takes at a time
constexpr int kApplyGroup = 8;         // lanes per listed block in apply (4 blocks per warp)

// The bitmap of one scan. Block b = bx + S*(by + S*bz) covers the cells
// x0 + 8*bx .. x0 + 8*bx + 7 (likewise y, z).
struct RayCube {
  uint32_t* bits;     // S^3 * 16 words
  uint32_t* touched;  // S^3 bits: block already on the list
  uint32_t* list;     // listed blocks
  uint32_t* count;    // entries on the list (may exceed cap: then ERR_SCRATCH)
  int x0, y0, z0;     // lowest cell of the cube (multiples of 8)
  uint32_t S;         // leaves per side
  uint32_t cap;       // list capacity
};

// Fire-and-forget ORs and AND into global memory. The pointers may reach the
// code as generic addresses (the batched tick keeps its scan table, with the
// bitmap and pool pointers, in shared memory), and an atomicOr on a generic
// address compiles to an atomic that returns its old value, which the warp
// then waits for; these always issue the reduction form.
__device__ __forceinline__ void red_or(uint32_t* p, uint32_t v) {
  asm volatile("red.relaxed.gpu.global.or.b32 [%0], %1;" ::"l"(__cvta_generic_to_global(p)),
               "r"(v)
               : "memory");
}
__device__ __forceinline__ void red_or64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.or.b64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)),
               "l"(v)
               : "memory");
}
__device__ __forceinline__ void red_and(uint32_t* p, uint32_t v) {
  asm volatile("red.relaxed.gpu.global.and.b32 [%0], %1;" ::"l"(__cvta_generic_to_global(p)),
               "r"(v)
               : "memory");
}

// Puts block b on the list the first time any bit of it is set.
__device__ __forceinline__ void mark_touch(const RayCube& Q, uint32_t b, const DMap& M) {
  uint32_t* tw = Q.touched + (b >> 5);
  const uint32_t tb = 1u << (b & 31);
  // bits only go from 0 to 1 while a scan marks, so a cached 1 is never stale
  if (__ldca(tw) & tb) return;
  if (atomicOr(tw, tb) & tb) return;
  const uint32_t k = atomicAdd(Q.count, 1u);
  if (k < Q.cap)
    Q.list[k] = b;
  else
    set_err(M, ERR_SCRATCH);
}

// Shared-memory word of the cell (cx, cy, cz) (cube-relative) with bitmap
// word index wi (0..15 in its leaf) if its leaf is within NB of the origin's
// leaf (l0x..: the neighbourhood's corner, relative leaf coordinates), else -1.
template <int NB>
__device__ __forceinline__ int mark_local(int cx, int cy, int cz, uint32_t wi, int l0x, int l0y,
                                          int l0z) {
  constexpr int NS = 2 * NB + 1;
  const unsigned qx = unsigned((cx >> 3) - l0x), qy = unsigned((cy >> 3) - l0y),
                 qz = unsigned((cz >> 3) - l0z);
  if (qx < unsigned(NS) && qy < unsigned(NS) && qz < unsigned(NS))
    return int(((qz * NS + qy) * NS + qx) * 16 + wi);
  return -1;
}

// The block's warps mark rays [r0, r1) of one scan from origin cell (ox, oy,
// oz). sm (mark_smem_words(NB) words) is zero on entry and on return; every
// thread of the block calls this with the same arguments. s_next: a shared
// word. Adds the cells walked to `visited`. The cube must reach at least
// NB + 1 leaves beyond the origin's leaf on every side.
template <int NB>
__device__ __forceinline__ void mark_rays_block(const DMap& M, const RayCube& Q,
                                                const int4* __restrict__ cast, uint32_t r0,
                                                uint32_t r1, int ox, int oy, int oz,
                                                uint32_t* sm, uint32_t* s_next,
                                                uint32_t& visited) {
  constexpr int NS = 2 * NB + 1;
  const unsigned lane = threadIdx.x & 31;
  // origin's leaf relative to the cube, and the shared neighbourhood's corner
  const int l0x = ((ox - Q.x0) >> 3) - NB, l0y = ((oy - Q.y0) >> 3) - NB,
            l0z = ((oz - Q.z0) >> 3) - NB;
  const uint32_t side = Q.S * 8u;
  if (threadIdx.x == 0) *s_next = r0;
  __syncthreads();
  uint32_t last_b = kNone;  // last block this lane ORed into (touch once per run)
  // w: bitmap word; li: its shared-memory word (-1: global)
  auto flush = [&](uint32_t w, uint32_t acc, int li) {
    if (li >= 0) {
      atomicOr(sm + li, acc);
      return;
    }
    red_or(Q.bits + w, acc);
    const uint32_t b = w >> 4;
    if (b != last_b) {
      last_b = b;
      mark_touch(Q, b, M);
    }
  };
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(s_next, kMarkWarpRays);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= r1) break;
    const uint32_t ri = base + lane;
    int4 e = make_int4(ox, oy, oz, 0);
    if (lane < kMarkWarpRays && ri < r1) e = cast[ri];
    const uint32_t m0 = chebyshev(ox, oy, oz, e.x, e.y, e.z);
    const uint32_t nseg = m0 < kMaxRayCells ? (m0 + kMarkSeg - 1) / kMarkSeg : 0u;
    if (m0 >= kMaxRayCells) set_err(M, ERR_RAY_TOO_LONG);
    // segments of the warp's rays, numbered ray after ray
    uint32_t incl = nseg;
#pragma unroll
    for (int o = 1; o < int(kMarkWarpRays); o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= unsigned(o)) incl += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, kMarkWarpRays - 1);
    for (uint32_t s0 = 0; s0 < total; s0 += 32) {
      const uint32_t s = s0 + lane;
      // the ray of segment s: the first of the warp's rays whose running
      // segment total exceeds s
      uint32_t j = 0;
#pragma unroll
      for (uint32_t q = 0; q + 1 < kMarkWarpRays; ++q)
        j += __shfl_sync(0xffffffffu, incl, q) <= s ? 1u : 0u;
      const int ex = __shfl_sync(0xffffffffu, e.x, j), ey = __shfl_sync(0xffffffffu, e.y, j),
                ez = __shfl_sync(0xffffffffu, e.z, j);
      const uint32_t ij = __shfl_sync(0xffffffffu, incl, j);
      const uint32_t nj = __shfl_sync(0xffffffffu, nseg, j);
      if (s >= total) continue;
      const int dx = ex - ox, dy = ey - oy, dz = ez - oz;
      const uint32_t ax = uint32_t(abs(dx)), ay = uint32_t(abs(dy)), az = uint32_t(abs(dz));
      const uint32_t m = max(ax, max(ay, az));
      const uint32_t k0 = (s - (ij - nj)) * kMarkSeg;
      const uint32_t n = min(kMarkSeg, m - k0);
      // state at k0: n_b = floor((2 k0 d_b + m) / 2m), r_b = the remainder
      // (the closed form of bxg_device.cuh), then RayIterator's step
      const uint32_t tm = 2u * m;
      const float rtm = __frcp_rn(float(tm));
      uint32_t nx, rx, ny, ry, nz, rz;
      divmod_small(2u * k0 * ax + m, tm, rtm, nx, rx);
      divmod_small(2u * k0 * ay + m, tm, rtm, ny, ry);
      divmod_small(2u * k0 * az + m, tm, rtm, nz, rz);
      const int sx = dx < 0 ? -1 : 1, sy = dy < 0 ? -1 : 1, sz = dz < 0 ? -1 : 1;
      int cx = ox + sx * int(nx) - Q.x0, cy = oy + sy * int(ny) - Q.y0,
          cz = oz + sz * int(nz) - Q.z0;
      uint32_t cur = kNone, acc = 0;
      int cur_local = -1;
      visited += n;
      for (uint32_t i = 0; i < n; ++i) {
        if (uint32_t(cx) >= side || uint32_t(cy) >= side || uint32_t(cz) >= side) {
          set_err(M, ERR_SCRATCH);  // outside the cube: cannot happen for scan rays
          break;
        }
        const uint32_t b =
            uint32_t(cx >> 3) + Q.S * (uint32_t(cy >> 3) + Q.S * uint32_t(cz >> 3));
        const uint32_t li = uint32_t(cx & 7) | (uint32_t(cy & 7) << 3) | (uint32_t(cz & 7) << 6);
        const uint32_t w = b * 16u + (li >> 5);
        if (w != cur) {
          if (cur != kNone) flush(cur, acc, cur_local);
          cur = w;
          acc = 0;
          cur_local = mark_local<NB>(cx, cy, cz, li >> 5, l0x, l0y, l0z);
        }
        acc |= 1u << (li & 31);
        rx += 2u * ax;
        if (rx >= tm) {
          rx -= tm;
          cx += sx;
        }
        ry += 2u * ay;
        if (ry >= tm) {
          ry -= tm;
          cy += sy;
        }
        rz += 2u * az;
        if (rz >= tm) {
          rz -= tm;
          cz += sz;
        }
      }
      if (cur != kNone) flush(cur, acc, cur_local);
    }
  }
  // the neighbourhood's words into the bitmap, once per block task
  __syncthreads();
  for (int t = threadIdx.x; t < mark_smem_words(NB); t += blockDim.x) {
    const uint32_t v = sm[t];
    if (!v) continue;
    sm[t] = 0;
    const int q = t >> 4, qx = q % NS, qy = (q / NS) % NS, qz = q / (NS * NS);
    const uint32_t b = uint32_t(l0x + qx) + Q.S * (uint32_t(l0y + qy) + Q.S * uint32_t(l0z + qz));
    red_or(Q.bits + b * 16u + (t & 15), v);
    mark_touch(Q, b, M);
  }
  __syncthreads();
}

// Leaf slot of the leaf whose lowest cell is (lx, ly, lz), created if
// missing, for a group of kApplyGroup lanes (sl = lane in group, gmask = the
// group's lanes). With a leaf directory D (bxg_scan.cuh), a current word there
// gives the slot in one load; otherwise the root bucket is probed
// cooperatively, one bucket per lane, and a missing or pending root, a long
// chain or a missing leaf goes through the bounded-wait creation path on the
// group's first lane; the slot found is then written to the directory.
__device__ __forceinline__ uint32_t apply_leaf_slot(const DMap& M, int lx, int ly, int lz,
                                                    unsigned sl, unsigned gbase, unsigned gmask,
                                                    const LeafDir* D) {
  uint32_t* dw = nullptr;
  if (D) {
    const uint32_t qx = static_cast<uint32_t>((lx >> 3) - D->x0),
                   qy = static_cast<uint32_t>((ly >> 3) - D->y0),
                   qz = static_cast<uint32_t>((lz >> 3) - D->z0);
    if (qx < D->side && qy < D->side && qz < D->side) {
      dw = D->words + (static_cast<size_t>(qx) * D->side + qy) * D->side + qz;
      const uint32_t w = *dw;
      if ((w >> 28) == D->epoch) return w & 0x0FFFFFFFu;
    }
  }
  const int32_t rm = root_mask(M);
  const int rx = lx & rm, ry = ly & rm, rz = lz & rm;
  const uint32_t h0 = root_hash(M, rx, ry, rz);
  const uint4 bk = M.buckets[(h0 + sl) & M.hmask];
  const bool hit = key_eq(bk, rx, ry, rz);
  const bool empty = static_cast<int>(bk.x) == kEmptyKey;
  const unsigned hm = (__ballot_sync(gmask, hit) & gmask) >> gbase;
  const unsigned em = (__ballot_sync(gmask, empty) & gmask) >> gbase;
  uint32_t in = kPending;
  if (hm) {
    const int fh = __ffs(hm) - 1;
    const unsigned before = em & ((1u << fh) - 1u);
    const uint32_t v = __shfl_sync(gmask, bk.w, fh, kApplyGroup);
    if (!before && v < kPending) in = v;
  }
  uint32_t leaf = kNone;
  if (sl == 0) {
    if (in == kPending) in = root_get_or_create(M, rx, ry, rz);
    if (in != kNone) {
      const uint32_t ii = inner_index(M, lx, ly, lz);
      leaf = M.ichild[static_cast<size_t>(in) * M.isize + ii];
      if (leaf >= kPending) leaf = leaf_get_or_create(M, in, ii, lx, ly, lz);
    }
    if (dw && leaf != kNone) *dw = (D->epoch << 28) | leaf;
  }
  return __shfl_sync(gmask, leaf, 0, kApplyGroup);
}

// Applies the ray update to listed block b and clears it (8 lanes; lane sl
// owns bitmap words 2 sl and 2 sl + 1, i.e. the 64 cells 64 sl .. 64 sl + 63
// of the 8^3 leaf, which are mask word sl). The block's bits and list bit are
// cleared even when the leaf cannot be had (pool full, error set): the bitmap
// is clean after every apply, and a scan that is re-run after the pools grew
// marks its rays again.
__device__ __forceinline__ void apply_block(const DMap& M, const RayCube& Q, uint32_t b,
                                            int32_t u, int32_t miss, int32_t cmin, unsigned sl,
                                            unsigned gbase, unsigned gmask, uint32_t& updated,
                                            const LeafDir* D = nullptr) {
  const uint32_t SS = Q.S * Q.S;
  const uint32_t bz = b / SS, rem = b - bz * SS, by = rem / Q.S, bx = rem - by * Q.S;
  const int lx = Q.x0 + 8 * int(bx), ly = Q.y0 + 8 * int(by), lz = Q.z0 + 8 * int(bz);
  uint2* wp = reinterpret_cast<uint2*>(Q.bits + size_t(b) * 16u) + sl;
  const uint2 wv = *wp;
  const uint32_t leaf = apply_leaf_slot(M, lx, ly, lz, sl, gbase, gmask, D);
  if (sl == 0) red_and(Q.touched + (b >> 5), ~(1u << (b & 31)));
  if ((wv.x | wv.y) == 0u) return;
  *wp = make_uint2(0u, 0u);
  if (leaf == kNone) return;
  int4* cells = reinterpret_cast<int4*>(reinterpret_cast<int32_t*>(M.ldata) +
                                        static_cast<size_t>(leaf) * 512u + 64u * sl);
  unsigned long long fresh = 0;  // cells whose word was zero: turn their mask bits on
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint32_t w = h ? wv.y : wv.x;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t nib = (w >> (4 * j)) & 0xFu;
      if (!nib) continue;
      int4 v = cells[8 * h + j];
      int32_t* c = reinterpret_cast<int32_t*>(&v);
      bool changed = false;
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        if (!((nib >> t) & 1u)) continue;
        const int32_t old = c[t];
        if (cell_id(old) != u) {
          c[t] = cell_pack(max(wrap_add(cell_prob(old), miss), cmin), u);
          changed = true;
          ++updated;
        }
        if (old == 0) fresh |= 1ull << (32 * h + 4 * j + t);
      }
      if (changed) cells[8 * h + j] = v;
    }
  }
  if (fresh) red_or64(M.lmask + static_cast<size_t>(leaf) * M.lwords + sl, fresh);
}

}  // namespace bxg
