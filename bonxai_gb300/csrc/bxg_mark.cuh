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
//          getLeafIndex, x fastest). A block takes a run of rays and cuts
//          them into segments that its threads walk (closed-form Bresenham
//          start, then the RayIterator step): the cells near the origin,
//          which every ray crosses, in a neighbourhood of leaves kept in
//          shared memory and ORed into the bitmap once per block task; the
//          rest in segments of kMarkSeg cells whose bits are ORed into the
//          bitmap one word at a time, fire-and-forget. A block's first OR
//          also sets the block's bit in a per-block "touched" bitmap.
//   list   The touched bitmap is turned into the scan's list of marked blocks
//          and cleared.
//   apply  One group of 8 lanes per listed block: a cooperative probe of the
//          root hash (8 buckets per step), the leaf get-or-create (topology:
//          once per leaf, not once per ray crossing), then the miss update of
//          the marked cells with vector loads and stores, the mask bits of
//          cells turned on, and the block cleared for the next scan.
//
// This is the two-phase insert (topology, then values) over deduplicated
// coordinates: the bitmap is the deduplication. The result equals the per-ray
// walk's bit for bit; the cube, its bits and its touched bits are scratch that
// is all zero between scans.
#pragma once

#include "bxg_scan.cuh"

namespace bxg {

constexpr uint32_t kMarkSeg = 16;  // cells of a segment beyond the neighbourhood
// Shared-memory neighbourhood of the origin: the leaves within NB of the
// origin's leaf, (2 NB + 1)^3 blocks of 16 words. NB = 3 (21.4 KiB) for the
// per-scan kernel's 1024-thread blocks, NB = 2 (7.8 KiB) in the batched tick,
// whose 256-thread blocks also hold the tick's scan table. A ray's cell k
// (k cells from the origin along the major axis) lies within Chebyshev
// distance k of the origin cell, so cells k <= 8 NB are always inside the
// neighbourhood; they form each ray's first kMarkLocalParts segments.
constexpr int kMarkNB = 3;
constexpr uint32_t kMarkLocalParts = 2;
__host__ __device__ constexpr int mark_smem_words(int nb) {
  return (2 * nb + 1) * (2 * nb + 1) * (2 * nb + 1) * 16;
}
constexpr int kMarkSmemWords = mark_smem_words(kMarkNB);
constexpr int kApplyGroup = 8;  // lanes per listed block in apply (4 blocks per warp)

// The bitmap of one scan. Block b = bx + S*(by + S*bz) covers the cells
// x0 + 8*bx .. x0 + 8*bx + 7 (likewise y, z).
//
// The touched bitmap has one bit per block at a scattered position, bit
// (b * kTouchMul) mod 2^k (2^k >= S^3; odd multiplier, so a permutation whose
// inverse multiplies by kTouchInv): with bit b, one 32-byte sector held the
// flags of 256 blocks in a row, and every ray along that row set them through
// the same sector of L2 (those ORs serialised: 100 us of a 110 us LiDAR mark).
struct RayCube {
  uint32_t* bits;     // S^3 * 16 words
  uint32_t* touched;  // (tmask + 1) bits: some bit of the block is set
  uint32_t* list;     // listed blocks
  uint32_t* count;    // entries on the list
  int x0, y0, z0;     // lowest cell of the cube (multiples of 8)
  uint32_t S;         // leaves per side
  uint32_t cap;       // list capacity (S^3)
  uint32_t tmask;     // 2^k - 1 with 2^k >= max(S^3, 32)
};

constexpr uint32_t kTouchMul = 0x9E3779B1u;
constexpr uint32_t kTouchInv = 0x0E8B2F51u;  // kTouchMul * kTouchInv == 1 mod 2^32
static_assert(kTouchMul * kTouchInv == 1u, "inverse of the touched-bit permutation");

__host__ __device__ inline uint32_t cube_touched_words(const RayCube& Q) {
  return (Q.tmask + 1u) / 32u;
}
// 2^k - 1 for the smallest 2^k >= max(S^3, 32)
__host__ __device__ inline uint32_t cube_touched_mask(uint32_t S) {
  uint32_t p = 32u;
  while (p < S * S * S) p <<= 1;
  return p - 1u;
}
__device__ __forceinline__ void touch_block(const RayCube& Q, uint32_t b) {
  const uint32_t t = (b * kTouchMul) & Q.tmask;
  asm volatile("red.relaxed.gpu.global.or.b32 [%0], %1;" ::"l"(
                   __cvta_generic_to_global(Q.touched + (t >> 5))),
               "r"(1u << (t & 31))
               : "memory");
}

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

// The rays of one block task, in shared memory, T at a time: each ray's
// offset from the origin (dx, dy, dz), its length m (cells before the end
// cell), and the first of its segments beyond the neighbourhood. Also a
// direct-mapped cache of blocks whose touched bit the block task has set: a
// hit skips the OR (most blocks are crossed by many of a task's rays).
constexpr uint32_t kTouchCache = 2048;
template <int T>
struct MarkRays {
  uint2 d[T];  // (dx, dy) and (dz, m) as 16-bit halves
  uint32_t start[T];
  uint32_t wsum[32];
  uint32_t n_far;  // segments beyond the neighbourhood, all rays of the batch
  uint32_t touched[kTouchCache];
};

// Walks cells k0 .. k1 - 1 of the ray from cube cell (qx, qy, qz) with offset
// (dx, dy, dz) and length m: the closed-form state at k0 (n_b = floor((2 k0
// d_b + m) / 2m), r_b the remainder, as in bxg_device.cuh), then
// RayIterator's step. `word` maps a cell to its word and `flush` stores a
// word's collected bits.
template <class Word, class Flush>
__device__ __forceinline__ void mark_walk(int qx, int qy, int qz, int dx, int dy, int dz,
                                          uint32_t m, uint32_t k0, uint32_t k1, Word&& word,
                                          Flush&& flush) {
  const uint32_t ax = uint32_t(abs(dx)), ay = uint32_t(abs(dy)), az = uint32_t(abs(dz));
  const uint32_t tm = 2u * m;
  const float rtm = __frcp_rn(float(tm));
  uint32_t nx, rx, ny, ry, nz, rz;
  divmod_small(2u * k0 * ax + m, tm, rtm, nx, rx);
  divmod_small(2u * k0 * ay + m, tm, rtm, ny, ry);
  divmod_small(2u * k0 * az + m, tm, rtm, nz, rz);
  const int sx = dx < 0 ? -1 : 1, sy = dy < 0 ? -1 : 1, sz = dz < 0 ? -1 : 1;
  int cx = qx + sx * int(nx), cy = qy + sy * int(ny), cz = qz + sz * int(nz);
  const uint32_t ax2 = 2u * ax, ay2 = 2u * ay, az2 = 2u * az;
  uint32_t cur = word(cx, cy, cz), acc = 0;
  for (uint32_t k = k0; k < k1; ++k) {
    const uint32_t w = word(cx, cy, cz);
    if (w != cur) {
      flush(cur, acc);
      cur = w;
      acc = 0;
    }
    acc |= 1u << (uint32_t(cx & 7) | (uint32_t(cy & 3) << 3));
    rx += ax2;
    if (rx >= tm) {
      rx -= tm;
      cx += sx;
    }
    ry += ay2;
    if (ry >= tm) {
      ry -= tm;
      cy += sy;
    }
    rz += az2;
    if (rz >= tm) {
      rz -= tm;
      cz += sz;
    }
  }
  flush(cur, acc);
}

// The block marks rays [r0, r1) of one scan from origin cell (ox, oy, oz)
// (blockDim.x == T). sm (mark_smem_words(NB) words) is zero on entry and on
// return; every thread of the block calls this with the same arguments. Adds
// the cells walked to `visited`. The cube must reach at least NB + 1 leaves
// beyond the origin's leaf on every side; a ray whose end cell lies outside
// the cube sets ERR_SCRATCH and is not walked.
template <int NB, int T>
__device__ __forceinline__ void mark_rays_block(const DMap& M, const RayCube& Q,
                                                const int4* __restrict__ cast, uint32_t r0,
                                                uint32_t r1, int ox, int oy, int oz,
                                                uint32_t* sm, MarkRays<T>& R,
                                                uint32_t& visited) {
  constexpr int NS = 2 * NB + 1;
  constexpr uint32_t kNear = 8u * NB + 1u;  // cells 0 .. kNear - 1 are in the neighbourhood
  constexpr uint32_t kPart = (kNear + kMarkLocalParts - 1) / kMarkLocalParts;
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int qox = ox - Q.x0, qoy = oy - Q.y0, qoz = oz - Q.z0;  // origin, cube cells
  const int side = int(Q.S) * 8;
  // the neighbourhood's lowest cell (cube cells) and its leaf
  const int nlx = (qox >> 3) - NB, nly = (qoy >> 3) - NB, nlz = (qoz >> 3) - NB;
  const int nbx = 8 * nlx, nby = 8 * nly, nbz = 8 * nlz;
  const uint32_t S = Q.S, SS = Q.S * Q.S;
  uint32_t last_b = kNone;  // last block this thread set the touched bit of
  auto near_word = [&](int cx, int cy, int cz) -> uint32_t {
    const uint32_t ux = uint32_t(cx - nbx), uy = uint32_t(cy - nby), uz = uint32_t(cz - nbz);
    return (((uz >> 3) * NS + (uy >> 3)) * NS + (ux >> 3)) * 16u + ((uy >> 2) & 1u) +
           ((uz & 7u) << 1);
  };
  // Every ray starts at the origin, so lanes walking near segments flush the
  // same few words at once: the lanes flushing one word OR their bits
  // together and one of them issues the shared atomic (same-address shared
  // atomics are serialised).
  auto near_flush = [&](uint32_t w, uint32_t acc) {
    const unsigned grp = __match_any_sync(__activemask(), w);
    const uint32_t v = __reduce_or_sync(grp, acc);
    if (lane == unsigned(__ffs(grp) - 1)) atomicOr(sm + w, v);
  };
  auto far_word = [&](int cx, int cy, int cz) -> uint32_t {
    return ((uint32_t(cx) >> 3) + S * (uint32_t(cy) >> 3) + SS * (uint32_t(cz) >> 3)) * 16u +
           ((uint32_t(cy) >> 2) & 1u) + ((uint32_t(cz) & 7u) << 1);
  };
  auto far_flush = [&](uint32_t w, uint32_t acc) {
    red_or(Q.bits + w, acc);
    const uint32_t b = w >> 4;
    if (b != last_b) {
      last_b = b;
      uint32_t& c = R.touched[(b * kTouchMul) >> 21];
      if (c != b) {  // races between threads only repeat an OR
        c = b;
        touch_block(Q, b);
      }
    }
  };
  for (uint32_t t = threadIdx.x; t < kTouchCache; t += T) R.touched[t] = kNone;
  for (uint32_t base = r0; base < r1; base += T) {
    const uint32_t nr = min(uint32_t(T), r1 - base);
    uint32_t nfar = 0;
    if (threadIdx.x < nr) {
      const int4 e = cast[base + threadIdx.x];
      int dx = e.x - ox, dy = e.y - oy, dz = e.z - oz;
      uint32_t m = uint32_t(max(abs(dx), max(abs(dy), abs(dz))));
      if (uint32_t(e.x - Q.x0) >= uint32_t(side) || uint32_t(e.y - Q.y0) >= uint32_t(side) ||
          uint32_t(e.z - Q.z0) >= uint32_t(side)) {
        set_err(M, ERR_SCRATCH);  // outside the cube: cannot happen for scan rays
        dx = dy = dz = 0;
        m = 0;
      }
      nfar = m > kNear ? (m - kNear + kMarkSeg - 1) / kMarkSeg : 0u;
      R.d[threadIdx.x] = make_uint2((uint32_t(dx) & 0xFFFFu) | (uint32_t(dy) << 16),
                                    (uint32_t(dz) & 0xFFFFu) | (m << 16));
    }
    // exclusive prefix of the far segment counts over the batch
    uint32_t incl = nfar;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= unsigned(o)) incl += v;
    }
    if (lane == 31) R.wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const uint32_t x0 = lane < T / 32 ? R.wsum[lane] : 0u;
      uint32_t x = x0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= unsigned(o)) x += v;
      }
      if (lane < T / 32) R.wsum[lane] = x - x0;
      if (lane == 31) R.n_far = x;
    }
    __syncthreads();
    R.start[threadIdx.x] = incl - nfar + R.wsum[warp];
    __syncthreads();
    // segments: kMarkLocalParts per ray near the origin, then the far ones
    const uint32_t n_near = nr * kMarkLocalParts;
    const uint32_t total = n_near + R.n_far;
    for (uint32_t j = threadIdx.x; j < total; j += T) {
      uint32_t r, k0, k1;
      if (j < n_near) {
        r = j / kMarkLocalParts;
        k0 = (j % kMarkLocalParts) * kPart;
        k1 = min(k0 + kPart, kNear);
      } else {
        const uint32_t g = j - n_near;
        uint32_t lo = 0, hi = nr;  // last ray whose first far segment is <= g
        while (hi - lo > 1) {
          const uint32_t mid = (lo + hi) >> 1;
          if (R.start[mid] <= g) lo = mid; else hi = mid;
        }
        r = lo;
        k0 = kNear + (g - R.start[r]) * kMarkSeg;
        k1 = k0 + kMarkSeg;
      }
      const uint2 p = R.d[r];
      const uint32_t m = p.y >> 16;
      k1 = min(k1, m);
      if (k0 >= k1) continue;
      visited += k1 - k0;
      const int dx = int(p.x << 16) >> 16, dy = int(p.x) >> 16, dz = int(p.y << 16) >> 16;
      if (j < n_near)
        mark_walk(qox, qoy, qoz, dx, dy, dz, m, k0, k1, near_word, near_flush);
      else
        mark_walk(qox, qoy, qoz, dx, dy, dz, m, k0, k1, far_word, far_flush);
    }
    __syncthreads();
  }
  // the neighbourhood's words into the bitmap, once per block task; the first
  // non-zero word of each block (16 lanes) sets its touched bit
  for (int t0 = int(threadIdx.x & ~31u); t0 < mark_smem_words(NB); t0 += T) {
    const int t = t0 + int(lane);
    uint32_t v = 0;
    if (t < mark_smem_words(NB)) {
      v = sm[t];
      if (v) sm[t] = 0;
    }
    const unsigned nz = __ballot_sync(0xffffffffu, v != 0);
    if (!v) continue;
    const int q = t >> 4, qx = q % NS, qy = (q / NS) % NS, qz = q / (NS * NS);
    const uint32_t b = uint32_t(nlx + qx) + S * uint32_t(nly + qy) + SS * uint32_t(nlz + qz);
    red_or(Q.bits + b * 16u + (t & 15), v);
    const unsigned half = (nz >> (lane & 16u)) & 0xFFFFu;
    if ((lane & 15u) == unsigned(__ffs(half) - 1)) touch_block(Q, b);
  }
  __syncthreads();
}

// Moves the blocks whose touched bits are set in words [32 c, 32 c + 32) of
// the touched bitmap onto the scan's list and clears those words (one warp,
// all lanes).
__device__ __forceinline__ void list_touched(const DMap& M, const RayCube& Q, uint32_t c) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t nw = cube_touched_words(Q);
  const uint32_t wi = c * 32u + lane;
  uint32_t w = 0;
  if (wi < nw) {
    w = Q.touched[wi];
    if (w) Q.touched[wi] = 0;
  }
  const uint32_t cnt = __popc(w);
  uint32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= unsigned(o)) incl += v;
  }
  const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
  if (!tot) return;
  uint32_t base = 0;
  if (lane == 0) base = atomicAdd(Q.count, tot);
  uint32_t k = __shfl_sync(0xffffffffu, base, 0) + incl - cnt;
  while (w) {
    const uint32_t bit = uint32_t(__ffs(w) - 1);
    w &= w - 1u;
    if (k < Q.cap)
      Q.list[k] = ((wi * 32u + bit) * kTouchInv) & Q.tmask;
    else
      set_err(M, ERR_SCRATCH);
    ++k;
  }
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
// of the 8^3 leaf, which are mask word sl). The block's bits are
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
  if ((wv.x | wv.y) == 0u) return;
  *wp = make_uint2(0u, 0u);
  if (leaf == kNone) return;
  int4* cells = reinterpret_cast<int4*>(reinterpret_cast<int32_t*>(M.ldata) +
                                        static_cast<size_t>(leaf) * 512u + 64u * sl);
  unsigned long long fresh = 0;  // cells whose word was zero: turn their mask bits on
  // Per bitmap word, the marked 16-byte runs are all loaded before any is
  // stored: interleaved, each store kept the next load from issuing (the
  // compiler cannot tell the runs apart), one round trip per run.
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint32_t w = h ? wv.y : wv.x;
    if (!w) continue;
    int4 v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if ((w >> (4 * j)) & 0xFu) v[j] = cells[8 * h + j];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t nib = (w >> (4 * j)) & 0xFu;
      if (!nib) continue;
      int32_t* c = reinterpret_cast<int32_t*>(&v[j]);
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
      if (changed) cells[8 * h + j] = v[j];
    }
  }
  if (fresh) red_or64(M.lmask + static_cast<size_t>(leaf) * M.lwords + sl, fresh);
}

}  // namespace bxg
