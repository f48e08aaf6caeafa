// VoxelGrid<T> batch operations: posToCoord, setValue (last writer wins),
// value(create), setCellOn, setCellOff, isCellOn, and the grid C ABI.
//
// A batch of n calls runs as:
//   1. dedup: every item inserts its coordinate into a scratch hash table
//      (128-bit CAS per probe) keeping the highest (setValue) or lowest
//      (setCellOn/Off) item index -- that item is the one whose effect the
//      sequential reference keeps;
//   2. topology + write: the kept item of each cell gets-or-creates its root
//      and leaf (bounded-wait protocol of bxg_device.cuh), turns the cell on
//      with atomicOr and writes the value.
// Items are independent after step 1, so no two threads write one cell.
#include <algorithm>
#include <mutex>
#include <vector>

#include "bxg_internal.h"

struct bxg_grid_s {
  bxg::MapCore core;
};

namespace bxg {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// posToCoord (bonxai.hpp:404-410): floor(x * inv_resolution) in double; the
// product is rounded once (no contraction) and floor is exact.
template <typename PT>
__global__ void k_pos_to_coord(const uint8_t* __restrict__ pts, size_t stride, uint32_t n,
                               double inv_res, int32_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PT* p = reinterpret_cast<const PT*>(pts + i * stride);
  out[3 * i + 0] = __double2int_rd(__dmul_rn(static_cast<double>(p[0]), inv_res));
  out[3 * i + 1] = __double2int_rd(__dmul_rn(static_cast<double>(p[1]), inv_res));
  out[3 * i + 2] = __double2int_rd(__dmul_rn(static_cast<double>(p[2]), inv_res));
}

// Scratch dedup table: bucket {x, y, z, kept index}; all-ones = empty (a real
// entry never holds index 0xFFFFFFFF). tab_min (optional) gets the lowest index.
template <bool KEEP_MAX>
__global__ void k_dedup_insert(const __grid_constant__ DMap M, const int32_t* __restrict__ xyz, uint32_t n,
                               uint4* tab, uint32_t tmask, uint32_t* tab_min) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  const uint4 kEmpty = make_uint4(kNone, kNone, kNone, kNone);
  const uint4 mine = make_uint4(uint32_t(x), uint32_t(y), uint32_t(z), i);
  uint32_t h = cell_hash(x, y, z) & tmask;
  for (uint32_t p = 0; p <= tmask; ++p, h = (h + 1) & tmask) {
    const uint4 old = cas128(tab + h, kEmpty, mine);
    if (eq4(old, kEmpty) || key_eq(old, x, y, z)) {
      if (!eq4(old, kEmpty)) {
        if (KEEP_MAX)
          atomicMax(&tab[h].w, i);
        else
          atomicMin(&tab[h].w, i);
      }
      if (tab_min) atomicMin(tab_min + h, i);
      return;
    }
  }
  set_err(M, ERR_SCRATCH);
}

__device__ __forceinline__ uint32_t dedup_find(const uint4* tab, uint32_t tmask, int x, int y,
                                               int z) {
  uint32_t h = cell_hash(x, y, z) & tmask;
  for (uint32_t p = 0; p <= tmask; ++p, h = (h + 1) & tmask) {
    const uint4 b = tab[h];
    if (b.w == kNone) return kNone;
    if (key_eq(b, x, y, z)) return h;
  }
  return kNone;
}

// Records, for the first item of each cell, whether the cell is on before the
// batch. It runs before the (retryable) write kernel, so a retry after pool
// growth cannot change what the first call observed.
__global__ void k_pre_on(const __grid_constant__ DMap M, const int32_t* __restrict__ xyz, uint32_t n,
                         const uint4* __restrict__ tab, uint32_t tmask,
                         const uint32_t* __restrict__ tab_first, uint8_t* pre) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  const uint32_t h = dedup_find(tab, tmask, x, y, z);
  if (h == kNone) return;
  const uint32_t first = tab_first ? tab_first[h] : tab[h].w;
  if (i != first) return;
  const uint32_t lf = leaf_of(M, x, y, z, false);
  pre[h] = lf != kNone && cell_is_on(M, lf, leaf_index(M, x, y, z));
}

template <int ESZ>
__device__ __forceinline__ void copy_val(uint8_t* dst, const uint8_t* src) {
  if (ESZ == 4) {
    *reinterpret_cast<uint32_t*>(dst) = *reinterpret_cast<const uint32_t*>(src);
  } else if (ESZ == 8) {
    *reinterpret_cast<unsigned long long*>(dst) =
        *reinterpret_cast<const unsigned long long*>(src);
  } else if (ESZ == 2) {
    *reinterpret_cast<uint16_t*>(dst) = *reinterpret_cast<const uint16_t*>(src);
  } else if (ESZ == 1) {
    *dst = *src;
  }
}

// setValue for the kept (highest-index) item of each cell (bonxai.hpp:449-466).
template <int ESZ>
__global__ void k_set_values(const __grid_constant__ DMap M, const int32_t* __restrict__ xyz,
                             const uint8_t* __restrict__ vals, uint32_t n,
                             const uint4* __restrict__ tab, uint32_t tmask) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  const uint32_t h = dedup_find(tab, tmask, x, y, z);
  if (h == kNone || tab[h].w != i) return;
  const uint32_t lf = leaf_of(M, x, y, z, true);
  if (lf == kNone) return;
  const uint32_t ci = leaf_index(M, x, y, z);
  cell_set_on(M, lf, ci);
  if (ESZ > 0) copy_val<ESZ>(M.ldata + (static_cast<size_t>(lf) * M.lsize + ci) * ESZ,
                             vals + static_cast<size_t>(i) * ESZ);
}

// was_on of item i: the state before call i -- the pre-batch state for the
// first call on a cell, on for every later one.
__global__ void k_was_on_first(const int32_t* __restrict__ xyz, uint32_t n,
                               const uint4* __restrict__ tab, uint32_t tmask,
                               const uint32_t* __restrict__ tab_min,
                               const uint8_t* __restrict__ pre, uint8_t* out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t h = dedup_find(tab, tmask, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  if (h == kNone) {
    out[i] = 0;
    return;
  }
  const uint32_t first = tab_min ? tab_min[h] : tab[h].w;
  out[i] = (i == first) ? pre[h] : 1;
}

// setCellOn for the first item of each cell (bonxai.hpp:537-553): the default
// is written only if the cell was off.
template <int ESZ>
__global__ void k_set_on(const __grid_constant__ DMap M, const int32_t* __restrict__ xyz, uint32_t n,
                         const uint8_t* __restrict__ dflt, const uint4* __restrict__ tab,
                         uint32_t tmask) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  const uint32_t h = dedup_find(tab, tmask, x, y, z);
  if (h == kNone || tab[h].w != i) return;
  const uint32_t lf = leaf_of(M, x, y, z, true);
  if (lf == kNone) return;
  const uint32_t ci = leaf_index(M, x, y, z);
  const bool was = cell_set_on(M, lf, ci);
  if (ESZ > 0 && !was)
    copy_val<ESZ>(M.ldata + (static_cast<size_t>(lf) * M.lsize + ci) * ESZ, dflt);
}

// setCellOff for the first item of each cell (bonxai.hpp:556-569). The value
// is zeroed to keep the off-cells-hold-T{} invariant (not observable).
template <int ESZ>
__global__ void k_set_off(const __grid_constant__ DMap M, const int32_t* __restrict__ xyz, uint32_t n,
                          const uint4* __restrict__ tab, uint32_t tmask, uint8_t* out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  const uint32_t h = dedup_find(tab, tmask, x, y, z);
  bool was = false;
  if (h != kNone && tab[h].w == i) {
    const uint32_t lf = leaf_of(M, x, y, z, false);
    if (lf != kNone) {
      const uint32_t ci = leaf_index(M, x, y, z);
      const unsigned long long bit = 1ull << (ci & 63);
      was = (atomicAnd(mask_word(M, lf, ci), ~bit) & bit) != 0ull;
      if (was && ESZ > 0) {
        uint8_t* d = M.ldata + (static_cast<size_t>(lf) * M.lsize + ci) * ESZ;
        for (int k = 0; k < ESZ; k++) d[k] = 0;
      }
    }
  }
  if (out) out[i] = was;
}

// value(coord, create) / ConstAccessor::value / isCellOn (bonxai.hpp:469-534).
template <int ESZ>
__global__ void k_get_values(const __grid_constant__ DMap M, const int32_t* __restrict__ xyz, uint32_t n, int create,
                             uint8_t* __restrict__ out_vals, uint8_t* __restrict__ found) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  const uint32_t lf = leaf_of(M, x, y, z, create != 0);
  bool on = false;
  uint32_t ci = 0;
  if (lf != kNone) {
    ci = leaf_index(M, x, y, z);
    if (create) {
      cell_set_on(M, lf, ci);
      on = true;
    } else {
      on = cell_is_on(M, lf, ci);
    }
  }
  if (found) found[i] = on;
  if (ESZ > 0 && out_vals) {
    uint8_t* d = out_vals + static_cast<size_t>(i) * ESZ;
    if (on) {
      copy_val<ESZ>(d, M.ldata + (static_cast<size_t>(lf) * M.lsize + ci) * ESZ);
    } else {
      for (int k = 0; k < ESZ; k++) d[k] = 0;
    }
  }
}

// Write-back of a mutable visitor: only cells that are on take the value.
template <int ESZ>
__global__ void k_store_if_on(const __grid_constant__ DMap M, const int32_t* __restrict__ xyz,
                              const uint8_t* __restrict__ vals, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  const uint32_t lf = leaf_of(M, x, y, z, false);
  if (lf == kNone) return;
  const uint32_t ci = leaf_index(M, x, y, z);
  if (!cell_is_on(M, lf, ci)) return;
  copy_val<ESZ>(M.ldata + (static_cast<size_t>(lf) * M.lsize + ci) * ESZ,
                vals + static_cast<size_t>(i) * ESZ);
}

// releaseUnusedMemory (bonxai.hpp:367-387): leaves whose mask is all off are
// unlinked from their inner node and pushed on the free stack.
__global__ void k_release_leaves(const __grid_constant__ DMap M, uint32_t n_leaves) {
  const uint32_t lf = blockIdx.x * blockDim.x + threadIdx.x;
  if (lf >= n_leaves) return;
  const int4 key = M.lkey[lf];
  if (key.w == -1) return;
  for (int w = 0; w < M.lwords; w++)
    if (M.lmask[static_cast<size_t>(lf) * M.lwords + w]) return;
  const uint32_t in = static_cast<uint32_t>(key.w);
  const uint32_t ii = inner_index(M, key.x, key.y, key.z);
  M.ichild[static_cast<size_t>(in) * M.isize + ii] = kNone;
  atomicAnd(M.imask + static_cast<size_t>(in) * M.iwords + (ii >> 6), ~(1ull << (ii & 63)));
  M.lkey[lf] = make_int4(-1, -1, -1, -1);
  const uint32_t slot = atomicAdd(M.ctr + C_FREE_LEAF, 1u);
  M.lfree[slot] = lf;
}
// (the host sets has_free when it next reads the counters)

// Roots whose inner node has no leaf left are removed. Removal from an
// open-addressing table would break probe chains, so the surviving buckets
// are re-inserted into a cleared table (k_rehash) by the host afterwards.
__global__ void k_drop_empty_roots(const __grid_constant__ DMap M, uint4* out_b, uint32_t cap, uint32_t* kept) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cap) return;
  uint4 b = M.buckets[i];
  out_b[i] = make_uint4(kNone, kNone, kNone, kNone);
  if (static_cast<int>(b.x) == kEmptyKey) return;
  if (b.w < kPending) {
    bool any = false;
    for (int w = 0; w < M.iwords; w++)
      any |= M.imask[static_cast<size_t>(b.w) * M.iwords + w] != 0ull;
    if (!any) return;  // the inner slot itself is not recycled
  }
  out_b[i] = b;
  atomicAdd(kept, 1u);
}

}  // namespace bxg

using namespace bxg;

namespace {

uint32_t next_pow2(uint64_t v) {
  uint32_t p = 64;
  while (p < v) p <<= 1;
  return p;
}

int check_grid(bxg_grid g) { return g ? BXG_OK : BXG_ERR_INVALID_ARG; }

// Test hook for the bounded waits: marks the inner-node slot of the leaf
// holding (x, y, z) as being created (kPending) by a creator that never
// publishes, so every access to that leaf waits out its spin limit and sets
// ERR_WAIT. *held = 1 when the slot was empty and is now held.
__global__ void k_hold_leaf(const __grid_constant__ DMap M, int x, int y, int z, int* held) {
  *held = 0;
  const int32_t rm = root_mask(M);
  const uint32_t in = root_get_or_create(M, x & rm, y & rm, z & rm);
  if (in == kNone) return;
  uint32_t* slot = M.ichild + static_cast<size_t>(in) * M.isize + inner_index(M, x, y, z);
  if (atomicCAS(slot, kNone, kPending) == kNone) *held = 1;
}

// Accessor::getLeafGrid / ConstAccessor::getLeafGrid (bonxai.hpp:588-647)
// for the host: copies the inner-node mask of the root holding (x, y, z) and,
// when the leaf exists, its mask words and all its cell values into out:
// [int flags][pad][inner mask words][leaf mask words][cells]. flags bit 0: the
// root exists; bit 1: the leaf exists. Missing parts are written as zeros.
__global__ void k_read_leaf(const __grid_constant__ DMap M, int x, int y, int z, uint8_t* out) {
  __shared__ uint32_t s_in, s_leaf;
  if (threadIdx.x == 0) {
    const int32_t rm = root_mask(M);
    s_in = root_find(M, x & rm, y & rm, z & rm);
    s_leaf = kNone;
    if (s_in != kNone) {
      const uint32_t c = M.ichild[static_cast<size_t>(s_in) * M.isize + inner_index(M, x, y, z)];
      s_leaf = c < kPending ? c : kNone;
    }
    *reinterpret_cast<int*>(out) = (s_in != kNone ? 1 : 0) | (s_leaf != kNone ? 2 : 0);
  }
  __syncthreads();
  const uint32_t in = s_in, lf = s_leaf;
  unsigned long long* im = reinterpret_cast<unsigned long long*>(out + 8);
  unsigned long long* lm = im + M.iwords;
  uint8_t* cells = reinterpret_cast<uint8_t*>(lm + M.lwords);
  for (int t = threadIdx.x; t < M.iwords; t += blockDim.x)
    im[t] = in != kNone ? M.imask[static_cast<size_t>(in) * M.iwords + t] : 0ull;
  for (int t = threadIdx.x; t < M.lwords; t += blockDim.x)
    lm[t] = lf != kNone ? M.lmask[static_cast<size_t>(lf) * M.lwords + t] : 0ull;
  const size_t bytes = static_cast<size_t>(M.lsize) * M.esz;
  const uint8_t* src = M.ldata + static_cast<size_t>(lf) * bytes;
  for (size_t t = threadIdx.x; t < bytes; t += blockDim.x) cells[t] = lf != kNone ? src[t] : 0;
}

// Builds the dedup table for n device coordinates.
int build_dedup(MapCore* m, const int32_t* dxyz, uint32_t n, bool keep_max, bool need_min,
                uint32_t* tmask_out, uint32_t** tab_min_out) {
  const uint32_t cap = next_pow2(uint64_t(n) * 2);
  BXG_CUDA(m, m->s_dedup.ensure(size_t(cap) * 16));
  launch_dedup_clear(m, m->s_dedup.as<uint4>(), cap);
  m->dedup_clean = 0;  // a ProbabilisticMap scan on this core must clear it again
  uint32_t* tmin = nullptr;
  if (need_min) {
    BXG_CUDA(m, m->s_dedup2.ensure(size_t(cap) * 4 + size_t(cap)));
    BXG_CUDA(m, cudaMemsetAsync(m->s_dedup2.p, 0xFF, size_t(cap) * 4, m->stream));
    tmin = m->s_dedup2.as<uint32_t>();
  }
  const unsigned blocks = (n + 255) / 256;
  if (keep_max)
    k_dedup_insert<true><<<blocks, 256, 0, m->stream>>>(m->dm, dxyz, n, m->s_dedup.as<uint4>(),
                                                        cap - 1, tmin);
  else
    k_dedup_insert<false><<<blocks, 256, 0, m->stream>>>(m->dm, dxyz, n, m->s_dedup.as<uint4>(),
                                                         cap - 1, tmin);
  BXG_LAUNCHED(m);
  *tmask_out = cap - 1;
  if (tab_min_out) *tab_min_out = tmin;
  return BXG_OK;
}

// Per-slot "previous state" bytes live after the tab_min words.
uint8_t* pre_bytes(MapCore* m, uint32_t cap, bool with_min) {
  return with_min ? m->s_dedup2.as<uint8_t>() + size_t(cap) * 4 : m->s_dedup2.as<uint8_t>();
}

// Runs a batch that creates topology, retrying once pools have grown.
template <class F>
int run_with_growth(MapCore* m, F&& body) {
  for (int attempt = 0; attempt < 12; attempt++) {
    int st = body();
    if (st) return st;
    uint32_t err = 0;
    st = core_sync(m, &err);
    if (st == BXG_OK) return core_maintain(m);
    if (!(err & (ERR_POOL_INNER | ERR_POOL_LEAF | ERR_HASH_FULL)) ||
        (err & (ERR_WAIT | ERR_RAY_TOO_LONG | ERR_SCRATCH)))
      return st;
    const int g = core_grow_for(m, err);
    if (g) return g;
  }
  return set_error(m, BXG_ERR_OUT_OF_POOL, "pools could not grow enough");
}

int grid_set_values_dev(bxg_grid g, const int32_t* dxyz, const void* dvals, uint32_t n,
                        uint8_t* was_on) {
  MapCore* m = &g->core;
  const bool want_was = was_on != nullptr;
  uint32_t tmask = 0;
  uint32_t* tmin = nullptr;
  int st = build_dedup(m, dxyz, n, true, want_was, &tmask, &tmin);
  if (st) return st;
  if (!want_was) BXG_CUDA(m, m->s_dedup2.ensure(size_t(tmask) + 1));
  uint8_t* pre = pre_bytes(m, tmask + 1, want_was);
  const unsigned blocks = (n + 255) / 256;
  const uint8_t* vals = static_cast<const uint8_t*>(dvals);
  if (want_was) {
    k_pre_on<<<blocks, 256, 0, m->stream>>>(m->dm, dxyz, n, m->s_dedup.as<uint4>(), tmask, tmin,
                                            pre);
    BXG_LAUNCHED(m);
  }
  st = run_with_growth(m, [&]() -> int {
    switch (m->dm.esz) {
      case 0: k_set_values<0><<<blocks, 256, 0, m->stream>>>(m->dm, dxyz, vals, n, m->s_dedup.as<uint4>(), tmask); break;
      case 1: k_set_values<1><<<blocks, 256, 0, m->stream>>>(m->dm, dxyz, vals, n, m->s_dedup.as<uint4>(), tmask); break;
      case 2: k_set_values<2><<<blocks, 256, 0, m->stream>>>(m->dm, dxyz, vals, n, m->s_dedup.as<uint4>(), tmask); break;
      case 4: k_set_values<4><<<blocks, 256, 0, m->stream>>>(m->dm, dxyz, vals, n, m->s_dedup.as<uint4>(), tmask); break;
      default: k_set_values<8><<<blocks, 256, 0, m->stream>>>(m->dm, dxyz, vals, n, m->s_dedup.as<uint4>(), tmask); break;
    }
    BXG_LAUNCHED(m);
    return BXG_OK;
  });
  if (st) return st;
  if (want_was) {
    void* dout = nullptr;
    st = stage_out(m, m->s_out, was_on, n, &dout);
    if (st) return st;
    k_was_on_first<<<blocks, 256, 0, m->stream>>>(dxyz, n, m->s_dedup.as<uint4>(), tmask, tmin,
                                                  pre, static_cast<uint8_t*>(dout));
    BXG_LAUNCHED(m);
    st = stage_out_finish(m, was_on, dout, n);
    if (st) return st;
  }
  return BXG_OK;
}

template <typename PT>
int grid_set_at_points(bxg_grid g, const PT* xyz, size_t stride, size_t n, const void* values) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  if (!n) return BXG_OK;
  if (!xyz || (m->dm.esz && !values) || n >= 0x7FFFFFFFu)
    return set_error(m, BXG_ERR_INVALID_ARG, "null input or batch too large");
  if (!stride) stride = 3 * sizeof(PT);
  cudaSetDevice(m->device);
  const void* dpts = nullptr;
  const void* dvals = nullptr;
  int st = stage_in(m, m->s_in, xyz, stride * (n - 1) + 3 * sizeof(PT), &dpts);
  if (st) return st;
  st = stage_in(m, m->s_in2, values, n * size_t(m->dm.esz), &dvals);
  if (st) return st;
  BXG_CUDA(m, m->s_ep.ensure(n * 12));
  k_pos_to_coord<PT><<<unsigned((n + 255) / 256), 256, 0, m->stream>>>(
      static_cast<const uint8_t*>(dpts), stride, uint32_t(n), m->inv_res, m->s_ep.as<int32_t>());
  BXG_LAUNCHED(m);
  return grid_set_values_dev(g, m->s_ep.as<int32_t>(), dvals, uint32_t(n), nullptr);
}

}  // namespace

extern "C" {

int bxg_grid_create(bxg_grid* out, double voxel_size, int inner_bits, int leaf_bits,
                    size_t value_bytes, const bxg_config* cfg) {
  if (!out) return BXG_ERR_INVALID_ARG;
  *out = nullptr;
  bxg_grid g = new bxg_grid_s();
  const int st = core_init(&g->core, voxel_size, inner_bits, leaf_bits, value_bytes, cfg);
  if (st) {
    set_create_error(g->core.err);
    delete g;
    return st;
  }
  *out = g;
  return BXG_OK;
}

int bxg_grid_destroy(bxg_grid g) {
  delete g;
  return BXG_OK;
}

int bxg_grid_pos_to_coord(bxg_grid g, const double* xyz, size_t n, int32_t* out_xyz) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  if (!n) return BXG_OK;
  if (!xyz || !out_xyz) return set_error(m, BXG_ERR_INVALID_ARG, "null pointer");
  cudaSetDevice(m->device);
  const void* din = nullptr;
  void* dout = nullptr;
  int st = stage_in(m, m->s_in, xyz, n * 24, &din);
  if (st) return st;
  st = stage_out(m, m->s_out, out_xyz, n * 12, &dout);
  if (st) return st;
  k_pos_to_coord<double><<<unsigned((n + 255) / 256), 256, 0, m->stream>>>(
      static_cast<const uint8_t*>(din), 24, uint32_t(n), m->inv_res, static_cast<int32_t*>(dout));
  BXG_LAUNCHED(m);
  st = stage_out_finish(m, out_xyz, dout, n * 12);
  if (st) return st;
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  return BXG_OK;
}

int bxg_grid_set_values(bxg_grid g, const int32_t* xyz, const void* values, size_t n,
                        uint8_t* was_on) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  if (!n) return BXG_OK;
  if (!xyz || (m->dm.esz && !values) || n >= 0x7FFFFFFFu)
    return set_error(m, BXG_ERR_INVALID_ARG, "null input or batch too large");
  cudaSetDevice(m->device);
  const void* dxyz = nullptr;
  const void* dvals = nullptr;
  int st = stage_in(m, m->s_in, xyz, n * 12, &dxyz);
  if (st) return st;
  st = stage_in(m, m->s_in2, values, n * size_t(m->dm.esz), &dvals);
  if (st) return st;
  return grid_set_values_dev(g, static_cast<const int32_t*>(dxyz), dvals, uint32_t(n), was_on);
}

int bxg_grid_set_values_at_points_f32(bxg_grid g, const float* xyz, size_t stride, size_t n,
                                      const void* values) {
  return grid_set_at_points(g, xyz, stride, n, values);
}
int bxg_grid_set_values_at_points_f64(bxg_grid g, const double* xyz, size_t stride, size_t n,
                                      const void* values) {
  return grid_set_at_points(g, xyz, stride, n, values);
}

int bxg_grid_get_values(bxg_grid g, const int32_t* xyz, size_t n, void* out_values,
                        uint8_t* found, int create_if_missing) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  if (!n) return BXG_OK;
  if (!xyz || n >= 0x7FFFFFFFu) return set_error(m, BXG_ERR_INVALID_ARG, "null input");
  cudaSetDevice(m->device);
  const void* dxyz = nullptr;
  void* dvals = nullptr;
  void* dfound = nullptr;
  int st = stage_in(m, m->s_in, xyz, n * 12, &dxyz);
  if (st) return st;
  const int esz = m->dm.esz;
  if (esz) {
    st = stage_out(m, m->s_out, out_values, n * size_t(esz), &dvals);
    if (st) return st;
  }
  st = stage_out(m, m->s_out2, found, n, &dfound);
  if (st) return st;
  const unsigned blocks = unsigned((n + 255) / 256);
  auto body = [&]() -> int {
    const int32_t* c = static_cast<const int32_t*>(dxyz);
    uint8_t* v = static_cast<uint8_t*>(dvals);
    uint8_t* f = static_cast<uint8_t*>(dfound);
    switch (esz) {
      case 0: k_get_values<0><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), create_if_missing, v, f); break;
      case 1: k_get_values<1><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), create_if_missing, v, f); break;
      case 2: k_get_values<2><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), create_if_missing, v, f); break;
      case 4: k_get_values<4><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), create_if_missing, v, f); break;
      default: k_get_values<8><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), create_if_missing, v, f); break;
    }
    BXG_LAUNCHED(m);
    return BXG_OK;
  };
  st = create_if_missing ? run_with_growth(m, body) : body();
  if (st) return st;
  if (dvals) {
    st = stage_out_finish(m, out_values, dvals, n * size_t(esz));
    if (st) return st;
  }
  if (dfound) {
    st = stage_out_finish(m, found, dfound, n);
    if (st) return st;
  }
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  return BXG_OK;
}

int bxg_grid_store_if_on(bxg_grid g, const int32_t* xyz, const void* values, size_t n) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  if (!n || !m->dm.esz) return BXG_OK;
  if (!xyz || !values || n >= 0x7FFFFFFFu) return set_error(m, BXG_ERR_INVALID_ARG, "null input");
  cudaSetDevice(m->device);
  const void* dxyz = nullptr;
  const void* dvals = nullptr;
  int st = stage_in(m, m->s_in, xyz, n * 12, &dxyz);
  if (st) return st;
  st = stage_in(m, m->s_in2, values, n * size_t(m->dm.esz), &dvals);
  if (st) return st;
  const unsigned blocks = unsigned((n + 255) / 256);
  const int32_t* c = static_cast<const int32_t*>(dxyz);
  const uint8_t* v = static_cast<const uint8_t*>(dvals);
  switch (m->dm.esz) {
    case 1: k_store_if_on<1><<<blocks, 256, 0, m->stream>>>(m->dm, c, v, uint32_t(n)); break;
    case 2: k_store_if_on<2><<<blocks, 256, 0, m->stream>>>(m->dm, c, v, uint32_t(n)); break;
    case 4: k_store_if_on<4><<<blocks, 256, 0, m->stream>>>(m->dm, c, v, uint32_t(n)); break;
    default: k_store_if_on<8><<<blocks, 256, 0, m->stream>>>(m->dm, c, v, uint32_t(n)); break;
  }
  BXG_LAUNCHED(m);
  return core_sync(m);
}

int bxg_grid_is_cell_on(bxg_grid g, const int32_t* xyz, size_t n, uint8_t* out) {
  return bxg_grid_get_values(g, xyz, n, nullptr, out, 0);
}

int bxg_grid_set_cells_on(bxg_grid g, const int32_t* xyz, size_t n, const void* default_value,
                          uint8_t* was_on) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  if (!n) return BXG_OK;
  if (!xyz || n >= 0x7FFFFFFFu) return set_error(m, BXG_ERR_INVALID_ARG, "null input");
  cudaSetDevice(m->device);
  const int esz = m->dm.esz;
  const void* dxyz = nullptr;
  int st = stage_in(m, m->s_in, xyz, n * 12, &dxyz);
  if (st) return st;
  // the default value travels in s_in2
  unsigned long long zero = 0;
  const void* ddef = nullptr;
  if (esz) {
    st = stage_in(m, m->s_in2, default_value ? default_value : &zero, size_t(esz), &ddef);
    if (st) return st;
  }
  uint32_t tmask = 0;
  st = build_dedup(m, static_cast<const int32_t*>(dxyz), uint32_t(n), false, false, &tmask,
                   nullptr);
  if (st) return st;
  BXG_CUDA(m, m->s_dedup2.ensure(size_t(tmask) + 1));
  uint8_t* pre = m->s_dedup2.as<uint8_t>();
  const unsigned blocks = unsigned((n + 255) / 256);
  const int32_t* c = static_cast<const int32_t*>(dxyz);
  const uint8_t* d = static_cast<const uint8_t*>(ddef);
  if (was_on) {
    k_pre_on<<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), m->s_dedup.as<uint4>(), tmask,
                                            nullptr, pre);
    BXG_LAUNCHED(m);
  }
  st = run_with_growth(m, [&]() -> int {
    switch (esz) {
      case 0: k_set_on<0><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), d, m->s_dedup.as<uint4>(), tmask); break;
      case 1: k_set_on<1><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), d, m->s_dedup.as<uint4>(), tmask); break;
      case 2: k_set_on<2><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), d, m->s_dedup.as<uint4>(), tmask); break;
      case 4: k_set_on<4><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), d, m->s_dedup.as<uint4>(), tmask); break;
      default: k_set_on<8><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), d, m->s_dedup.as<uint4>(), tmask); break;
    }
    BXG_LAUNCHED(m);
    return BXG_OK;
  });
  if (st) return st;
  if (was_on) {
    void* dout = nullptr;
    st = stage_out(m, m->s_out, was_on, n, &dout);
    if (st) return st;
    k_was_on_first<<<blocks, 256, 0, m->stream>>>(c, uint32_t(n), m->s_dedup.as<uint4>(), tmask,
                                                  nullptr, pre, static_cast<uint8_t*>(dout));
    BXG_LAUNCHED(m);
    st = stage_out_finish(m, was_on, dout, n);
    if (st) return st;
  }
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  return BXG_OK;
}

int bxg_grid_set_cells_off(bxg_grid g, const int32_t* xyz, size_t n, uint8_t* was_on) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  if (!n) return BXG_OK;
  if (!xyz || n >= 0x7FFFFFFFu) return set_error(m, BXG_ERR_INVALID_ARG, "null input");
  cudaSetDevice(m->device);
  const void* dxyz = nullptr;
  int st = stage_in(m, m->s_in, xyz, n * 12, &dxyz);
  if (st) return st;
  uint32_t tmask = 0;
  const int32_t* c = static_cast<const int32_t*>(dxyz);
  st = build_dedup(m, c, uint32_t(n), false, false, &tmask, nullptr);
  if (st) return st;
  void* dout = nullptr;
  st = stage_out(m, m->s_out, was_on, n, &dout);
  if (st) return st;
  const unsigned blocks = unsigned((n + 255) / 256);
  uint8_t* o = static_cast<uint8_t*>(dout);
  switch (m->dm.esz) {
    case 0: k_set_off<0><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), m->s_dedup.as<uint4>(), tmask, o); break;
    case 1: k_set_off<1><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), m->s_dedup.as<uint4>(), tmask, o); break;
    case 2: k_set_off<2><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), m->s_dedup.as<uint4>(), tmask, o); break;
    case 4: k_set_off<4><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), m->s_dedup.as<uint4>(), tmask, o); break;
    default: k_set_off<8><<<blocks, 256, 0, m->stream>>>(m->dm, c, uint32_t(n), m->s_dedup.as<uint4>(), tmask, o); break;
  }
  BXG_LAUNCHED(m);
  if (dout) {
    st = stage_out_finish(m, was_on, dout, n);
    if (st) return st;
  }
  return core_sync(m);
}

int bxg_grid_active_cells(bxg_grid g, size_t* out) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(g->core.device);
  return core_active_cells(&g->core, out);
}

int bxg_grid_node_counts(bxg_grid g, size_t* roots, size_t* leaves) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(g->core.device);
  return core_node_counts(&g->core, roots, leaves);
}

int bxg_grid_mem_usage(bxg_grid g, size_t* out) {
  if (check_grid(g) || !out) return BXG_ERR_INVALID_ARG;
  *out = core_mem_usage(&g->core);
  return BXG_OK;
}

int bxg_grid_dump(bxg_grid g, int32_t* out_xyz, void* out_values, size_t cap, size_t* n_out) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(g->core.device);
  return core_dump(&g->core, out_xyz, out_values, cap, n_out, 0, 0);
}

int bxg_grid_clear(bxg_grid g, int option) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  cudaSetDevice(m->device);
  if (option == 0) return core_clear(m);
  if (option != 1) return set_error(m, BXG_ERR_INVALID_ARG, "option must be 0 or 1");
  // SET_ALL_CELLS_OFF keeps every node (bonxai.hpp:685-686).
  int st = core_sync(m);
  if (st) return st;
  const size_t nl = m->h_ctr[C_LEAF];
  BXG_CUDA(m, cudaMemsetAsync(m->lmask.p, 0, nl * m->dm.lwords * 8, m->stream));
  if (m->dm.esz)
    BXG_CUDA(m, cudaMemsetAsync(m->ldata.p, 0, nl * m->dm.lsize * m->dm.esz, m->stream));
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  return BXG_OK;
}

int bxg_grid_release_unused(bxg_grid g) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  cudaSetDevice(m->device);
  int st = core_sync(m);
  if (st) return st;
  const uint32_t nl = m->h_ctr[C_LEAF];
  m->leaf_gen++;  // released slots are handed out again at other coordinates
  if (nl) {
    k_release_leaves<<<(nl + 255) / 256, 256, 0, m->stream>>>(m->dm, nl);
    BXG_LAUNCHED(m);
  }
  // Rebuild the root table without roots that lost every leaf.
  const uint32_t cap = m->dm.hmask + 1;
  DevBuf kept_b;
  BXG_CUDA(m, kept_b.ensure(size_t(cap) * 16 + 16));
  uint32_t* kept = reinterpret_cast<uint32_t*>(kept_b.as<uint8_t>() + size_t(cap) * 16);
  BXG_CUDA(m, cudaMemsetAsync(kept, 0, 4, m->stream));
  k_drop_empty_roots<<<(cap + 255) / 256, 256, 0, m->stream>>>(m->dm, kept_b.as<uint4>(), cap,
                                                                kept);
  BXG_LAUNCHED(m);
  BXG_CUDA(m, cudaMemsetAsync(m->buckets.p, 0xFF, size_t(cap) * 16, m->stream));
  launch_rehash(m, kept_b.as<uint4>(), cap, m->dm);
  BXG_LAUNCHED(m);
  BXG_CUDA(m, cudaMemcpyAsync(m->ctr.as<uint32_t>() + C_ROOTS, kept, 4, cudaMemcpyDeviceToDevice,
                              m->stream));
  return core_sync(m);
}

int bxg_grid_synchronize(bxg_grid g) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  cudaSetDevice(g->core.device);
  return core_sync(&g->core);
}

int bxg_debug_hold_leaf(bxg_grid g, const int32_t xyz[3]) {
  if (check_grid(g) || !xyz) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  cudaSetDevice(m->device);
  BXG_CUDA(m, m->s_tmp.ensure(8));
  k_hold_leaf<<<1, 1, 0, m->stream>>>(m->dm, xyz[0], xyz[1], xyz[2], m->s_tmp.as<int>());
  BXG_LAUNCHED(m);
  int held = 0;
  BXG_CUDA(m, cudaMemcpyAsync(&held, m->s_tmp.p, 4, cudaMemcpyDeviceToHost, m->stream));
  const int st = core_sync(m);
  if (st) return st;
  if (held != 1) return set_error(m, BXG_ERR_INVALID_ARG, "the leaf exists or cannot be reached");
  return BXG_OK;
}

int bxg_grid_read_leaf(bxg_grid g, const int32_t xyz[3], uint64_t* inner_mask,
                       uint64_t* leaf_mask, void* cells, int* found) {
  if (check_grid(g) || !xyz) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  cudaSetDevice(m->device);
  const size_t iw = size_t(m->dm.iwords), lw = size_t(m->dm.lwords);
  const size_t cb = size_t(m->dm.lsize) * size_t(m->dm.esz);
  const size_t bytes = 8 + 8 * (iw + lw) + cb;
  BXG_CUDA(m, m->s_out2.ensure(bytes));
  k_read_leaf<<<1, 256, 0, m->stream>>>(m->dm, xyz[0], xyz[1], xyz[2], m->s_out2.as<uint8_t>());
  BXG_LAUNCHED(m);
  std::vector<uint8_t> h(bytes);
  BXG_CUDA(m, cudaMemcpyAsync(h.data(), m->s_out2.p, bytes, cudaMemcpyDeviceToHost, m->stream));
  const int st = core_sync(m);
  if (st) return st;
  int flags = 0;
  std::memcpy(&flags, h.data(), sizeof(int));
  if (found) *found = flags;
  if (inner_mask) std::memcpy(inner_mask, h.data() + 8, 8 * iw);
  if (leaf_mask) std::memcpy(leaf_mask, h.data() + 8 + 8 * iw, 8 * lw);
  if (cells && cb) std::memcpy(cells, h.data() + 8 + 8 * (iw + lw), cb);
  return BXG_OK;
}

int bxg_grid_device_view(bxg_grid g, bxg_device_view* out) {
  if (check_grid(g) || !out) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  cudaSetDevice(m->device);
  const int st = core_sync(m);
  if (st) return st;
  out->leaf_mask = m->dm.lmask;
  out->leaf_data = m->dm.ldata;
  out->leaf_key = reinterpret_cast<const int32_t*>(m->dm.lkey);
  out->n_leaves = m->h_ctr[C_LEAF];
  out->inner_bits = m->dm.ib;
  out->leaf_bits = m->dm.lb;
  out->value_bytes = m->dm.esz;
  out->resolution = m->res;
  out->stream = m->stream;
  return BXG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// setValue batch that allocates nothing.
//
// For callers that must not allocate GPU memory while they run: a real-time
// perception or control thread (cudaMalloc/cudaFree can block for
// milliseconds and cudaFree synchronises the whole device), or a process that
// reserves all of its device memory up front and forbids allocations later.
// bxg_grid_set_values stages host inputs and grows its scratch table and the
// node pools on demand, so it may call cudaMalloc; this variant never does.
//
// Its dedup table lives in the file-scope array below, which every GPU that
// loads this library holds until the process exits. That caps one call at
// kNoAllocMaxItems items; larger batches can be split, because consecutive
// setValue batches give the same cells as one batch. The array is shared by
// all calls on a device and keeps the last call's contents, so each call
// first resets the part it uses; two calls that overlap on the GPU (different
// streams or host threads at the same time) would race on it.
// ---------------------------------------------------------------------------
constexpr uint32_t kNoAllocMaxItems = 1u << 17;             // 131072 items per call
constexpr uint32_t kNoAllocBuckets = 2u * kNoAllocMaxItems;  // 262144 x 16 B = 4 MiB

static __device__ __align__(256) uint4 g_noalloc_dedup[kNoAllocBuckets];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
uint4* g_noalloc_dev_ptr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_dedup on the current device. In host code the
// array's name only stands in for the symbol, so the address is looked up
// once per device (with that device current) and cached.
int noalloc_table(MapCore* m, uint4** out) {
  if (m->device < 0 || m->device >= kNoAllocMaxDevices)
    return set_error(m, BXG_ERR_INVALID_ARG, "device ordinal out of range for the no-alloc path");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_dev_ptr[m->device]) {
    int cur = -1;
    BXG_CUDA(m, cudaGetDevice(&cur));
    if (cur != m->device)
      return set_error(m, BXG_ERR_CUDA, "the grid's device is not current");
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_dedup);
    if (e != cudaSuccess) return cuda_fail(m, e, "cudaGetSymbolAddress(g_noalloc_dedup)");
    g_noalloc_dev_ptr[m->device] = static_cast<uint4*>(p);
  }
  *out = g_noalloc_dev_ptr[m->device];
  return BXG_OK;
}
}  // namespace

extern "C" int bxg_grid_set_values_noalloc(bxg_grid g, const int32_t* d_xyz,
                                           const void* d_values, size_t n) {
  if (check_grid(g)) return BXG_ERR_INVALID_ARG;
  MapCore* m = &g->core;
  if (!n) return BXG_OK;
  if (n > kNoAllocMaxItems)
    return set_error(m, BXG_ERR_INVALID_ARG,
                     "bxg_grid_set_values_noalloc takes at most 131072 items per call; "
                     "split the batch");
  if (!d_xyz || (m->dm.esz && !d_values))
    return set_error(m, BXG_ERR_INVALID_ARG, "null input");
  auto on_grid_device = [m](const void* p) {
    const int d = ptr_device(p);
    return d == m->device || d == kPtrManaged;
  };
  if (!on_grid_device(d_xyz) || (m->dm.esz && !on_grid_device(d_values)))
    return set_error(m, BXG_ERR_INVALID_ARG,
                     "bxg_grid_set_values_noalloc needs device-memory inputs on the grid's "
                     "device");
  BXG_CUDA(m, cudaSetDevice(m->device));
  uint4* tab = nullptr;
  int st = noalloc_table(m, &tab);
  if (st) return st;
  const uint32_t cap = next_pow2(uint64_t(n) * 2);  // <= kNoAllocBuckets
  BXG_CUDA(m, cudaMemsetAsync(tab, 0xFF, size_t(cap) * sizeof(uint4), m->stream));
  const unsigned blocks = unsigned((n + 255) / 256);
  const uint32_t nn = uint32_t(n);
  k_dedup_insert<true><<<blocks, 256, 0, m->stream>>>(m->dm, d_xyz, nn, tab, cap - 1, nullptr);
  BXG_LAUNCHED(m);
  const uint8_t* vals = static_cast<const uint8_t*>(d_values);
  switch (m->dm.esz) {
    case 0: k_set_values<0><<<blocks, 256, 0, m->stream>>>(m->dm, d_xyz, vals, nn, tab, cap - 1); break;
    case 1: k_set_values<1><<<blocks, 256, 0, m->stream>>>(m->dm, d_xyz, vals, nn, tab, cap - 1); break;
    case 2: k_set_values<2><<<blocks, 256, 0, m->stream>>>(m->dm, d_xyz, vals, nn, tab, cap - 1); break;
    case 4: k_set_values<4><<<blocks, 256, 0, m->stream>>>(m->dm, d_xyz, vals, nn, tab, cap - 1); break;
    default: k_set_values<8><<<blocks, 256, 0, m->stream>>>(m->dm, d_xyz, vals, nn, tab, cap - 1); break;
  }
  BXG_LAUNCHED(m);
  // Reports OUT_OF_POOL when the pools were full; they are not grown here.
  return core_sync(m);
}
