// Device-side data layout and primitives of the GB300 sparse voxel grid.
//
// One map lives in HBM as flat pools indexed by 32-bit slot numbers (no
// pointers), so pools can be grown by copy and are shared by every kernel:
//
//   root hash   uint4 buckets[H]        {root.x, root.y, root.z, inner slot}
//               open addressing, linear probing, H a power of two. The key is
//               getRootKey(coord) = coord & ~((1 << (inner_bits+leaf_bits)) - 1)
//               (bonxai.hpp:419-423), so a valid key never has its low bits set
//               and the all-ones pattern marks an empty bucket.
//   inner pool  uint32 ichild[I * 2^(3*inner_bits)]   leaf slot or kNone
//               u64    imask [I * inner_words]        which children exist
//               (InnerGrid = Grid<shared_ptr<LeafGrid>>, bonxai.hpp:129)
//   leaf pool   u64    lmask [L * leaf_words]         cell on/off bits
//               T      ldata [L * 2^(3*leaf_bits)]    cell values, x fastest
//               int4   lkey  [L]                      {leaf origin xyz, inner}
//               (LeafGrid = Grid<DataT>, bonxai.hpp:128; index math
//               bonxai.hpp:431-447)
//   counters    uint32 ctr[...]                       see enum below
//
// Invariant: a cell whose mask bit is off holds T{} (all zero bytes). The
// reference never lets the content of an off cell be observed (value() returns
// nullptr, forEachCell skips it, and turning a cell on writes T{} or the given
// value, bonxai.hpp:483-491,546-551), so keeping it zero lets every creation
// path skip the write.
//
// Concurrency: creation is lock-free with bounded waits. A root is inserted by
// a 128-bit compare-and-swap of the whole bucket; the thread that inserted it
// allocates the inner slot and publishes it while other threads that need it
// wait (bounded, with backoff). Leaves use the same
// protocol on the inner node's child word (kNone -> kPending -> slot). A wait
// that runs out sets an error bit and returns kNone; no kernel waits forever.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bxg {

constexpr uint32_t kNone = 0xFFFFFFFFu;     // no slot / empty
constexpr uint32_t kPending = 0xFFFFFFFEu;  // a thread is allocating this slot
constexpr int32_t kEmptyKey = -1;           // all-ones key component
constexpr int kSpinLimit = 1 << 20;         // bounded waits (~0.1-1 s worst case)

// Error bits in ctr[C_ERR].
enum : uint32_t {
  ERR_POOL_INNER = 1u,
  ERR_POOL_LEAF = 2u,
  ERR_HASH_FULL = 4u,
  ERR_WAIT = 8u,
  ERR_RAY_TOO_LONG = 16u,
  ERR_SCRATCH = 32u,
};

// Counter words.
enum : int {
  C_ROOTS = 0,      // buckets in use
  C_INNER = 1,      // inner slots handed out (may overshoot capacity on failure)
  C_LEAF = 2,       // leaf slots handed out by the bump allocator
  C_ERR = 3,        // error bits
  C_CAST = 4,       // rays queued for the current scan
  C_FREE_LEAF = 5,  // entries on the leaf free stack
  C_LIST = 6,       // leaf blocks on the scan's marked list (bxg_mark.cuh)
  C_TASK = 7,       // next block task of the mark phase
  C_STATS = 8,      // 64-bit statistics start here (pairs of words)
  C_WORDS = 32,
};
// 64-bit statistics (indices into (unsigned long long*)(ctr + C_STATS)).
enum : int { S_POINTS = 0, S_RAY_LEN = 1, S_VISITED = 2, S_UPDATED = 3, S_COUNT = 12 };

// Kinds of endpoint.
// EP_DUP: a valid point whose endpoint cell a lower index in its warp also
// reaches (it counts as a point but cannot decide the cell).
enum : int32_t { EP_HIT = 0, EP_MISS = 1, EP_SKIP = 2, EP_DUP = 3 };

struct DMap {
  // geometry (bonxai.hpp:117-123)
  int32_t ib, lb;          // inner_bits, leaf_bits
  int32_t isize, iwords;   // children per inner node, mask words per inner node
  int32_t lsize, lwords;   // cells per leaf, mask words per leaf
  int32_t esz;             // bytes per value (0 = binary grid)
  // root hash
  uint4* buckets;
  uint32_t hmask;
  // inner pool
  uint32_t* ichild;
  unsigned long long* imask;
  uint32_t icap;
  // leaf pool
  unsigned long long* lmask;
  uint8_t* ldata;
  int4* lkey;
  uint32_t* lfree;  // stack of released leaf slots
  uint32_t lcap;
  uint32_t has_free;  // host's view: the free stack may be non-empty
  // counters
  uint32_t* ctr;
};

// ---------------------------------------------------------------------------
// memory-model helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Publication of a freshly allocated slot. What a reader needs behind the slot
// (the node's zeroed mask/cells, its kNone children) was written before the
// kernel started, so no release ordering is needed -- only visibility.
__device__ __forceinline__ void st_publish(uint32_t* p, uint32_t v) {
  *reinterpret_cast<volatile uint32_t*>(p) = v;
}
__device__ __forceinline__ uint4 ld_volatile4(const uint4* p) {
  uint4 v;
  asm volatile("ld.volatile.global.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p)
               : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
  return *reinterpret_cast<const volatile uint32_t*>(p);
}

// 128-bit compare-and-swap (atom.cas.b128, sm_90 and later): the whole bucket
// is compared and replaced atomically, and the old content is returned as one
// atomic read.
__device__ __forceinline__ uint4 cas128(uint4* addr, uint4 cmp, uint4 val) {
  const unsigned long long c0 = (static_cast<unsigned long long>(cmp.y) << 32) | cmp.x;
  const unsigned long long c1 = (static_cast<unsigned long long>(cmp.w) << 32) | cmp.z;
  const unsigned long long v0 = (static_cast<unsigned long long>(val.y) << 32) | val.x;
  const unsigned long long v1 = (static_cast<unsigned long long>(val.w) << 32) | val.z;
  unsigned long long r0, r1;
  asm volatile(
      "{\n\t.reg .b128 cc, vv, rr;\n\t"
      "mov.b128 cc, {%2, %3};\n\t"
      "mov.b128 vv, {%4, %5};\n\t"
      "atom.global.cas.b128 rr, [%6], cc, vv;\n\t"
      "mov.b128 {%0, %1}, rr;\n\t}"
      : "=l"(r0), "=l"(r1)
      : "l"(c0), "l"(c1), "l"(v0), "l"(v1), "l"(addr)
      : "memory");
  return make_uint4(static_cast<uint32_t>(r0), static_cast<uint32_t>(r0 >> 32),
                    static_cast<uint32_t>(r1), static_cast<uint32_t>(r1 >> 32));
}

__device__ __forceinline__ bool eq4(uint4 a, uint4 b) {
  return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
}
__device__ __forceinline__ bool key_eq(uint4 b, int x, int y, int z) {
  return static_cast<int>(b.x) == x && static_cast<int>(b.y) == y && static_cast<int>(b.z) == z;
}

__device__ __forceinline__ void set_err(const DMap& M, uint32_t bit) {
  atomicOr(M.ctr + C_ERR, bit);
}

// ---------------------------------------------------------------------------
// key and index math (bonxai.hpp:419-447)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t root_mask(const DMap& M) {
  return ~((1 << (M.ib + M.lb)) - 1);
}
__device__ __forceinline__ int32_t leaf_mask(const DMap& M) { return ~((1 << M.lb) - 1); }
__device__ __forceinline__ uint32_t inner_index(const DMap& M, int x, int y, int z) {
  const int im = (1 << M.ib) - 1;
  return static_cast<uint32_t>(((x >> M.lb) & im) | (((y >> M.lb) & im) << M.ib) |
                               (((z >> M.lb) & im) << (2 * M.ib)));
}
__device__ __forceinline__ uint32_t leaf_index(const DMap& M, int x, int y, int z) {
  const int lm = (1 << M.lb) - 1;
  return static_cast<uint32_t>((x & lm) | ((y & lm) << M.lb) | ((z & lm) << (2 * M.lb)));
}

__device__ __forceinline__ uint32_t mix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x7feb352du;
  h ^= h >> 15;
  h *= 0x846ca68bu;
  h ^= h >> 16;
  return h;
}
// Hash of a root key; the key is shifted down by its zero low bits first.
__device__ __forceinline__ uint32_t root_hash(const DMap& M, int x, int y, int z) {
  const int s = M.ib + M.lb;
  const uint32_t a = static_cast<uint32_t>(x >> s), b = static_cast<uint32_t>(y >> s),
                 c = static_cast<uint32_t>(z >> s);
  return mix32(a * 0x9E3779B1u ^ mix32(b * 0x85EBCA77u ^ mix32(c * 0xC2B2AE3Du)));
}
__device__ __forceinline__ uint32_t cell_hash(int x, int y, int z) {
  return mix32(static_cast<uint32_t>(x) * 0x9E3779B1u ^
               mix32(static_cast<uint32_t>(y) * 0x85EBCA77u ^
                     mix32(static_cast<uint32_t>(z) * 0xC2B2AE3Du)));
}

// ---------------------------------------------------------------------------
// slot allocation
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t alloc_inner(const DMap& M) {
  const uint32_t i = atomicAdd(M.ctr + C_INNER, 1u);
  if (i >= M.icap) {
    set_err(M, ERR_POOL_INNER);
    return kNone;
  }
  return i;
}
// Released leaves are reused first (their masks and cells are all zero). The
// free stack is only filled by releaseUnusedMemory, so kernels launched while
// the host knows it is empty skip the probe.
__device__ __forceinline__ uint32_t alloc_leaf(const DMap& M) {
  if (M.has_free && ld_volatile(M.ctr + C_FREE_LEAF) > 0) {
    const int prev = static_cast<int>(atomicSub(M.ctr + C_FREE_LEAF, 1u));
    if (prev > 0) return M.lfree[prev - 1];
    atomicAdd(M.ctr + C_FREE_LEAF, 1u);  // lost the race for the last entry
  }
  const uint32_t i = atomicAdd(M.ctr + C_LEAF, 1u);
  if (i >= M.lcap) {
    set_err(M, ERR_POOL_LEAF);
    return kNone;
  }
  return i;
}

// ---------------------------------------------------------------------------
// root map
// ---------------------------------------------------------------------------
// Read-only lookup (no concurrent inserts in the calling kernel).
__device__ __forceinline__ uint32_t root_find(const DMap& M, int x, int y, int z) {
  uint32_t h = root_hash(M, x, y, z) & M.hmask;
  for (uint32_t p = 0; p <= M.hmask; ++p) {
    const uint4 b = M.buckets[h];
    if (key_eq(b, x, y, z)) return b.w < kPending ? b.w : kNone;
    if (static_cast<int>(b.x) == kEmptyKey) return kNone;
    h = (h + 1) & M.hmask;
  }
  return kNone;
}

// Waits (bounded) until the bucket's inner slot is published; takes over the
// allocation if an earlier attempt failed for lack of pool space.
static __device__ __noinline__ uint32_t root_value_wait(const DMap& M, uint4* b) {
  uint32_t* wp = &b->w;
  unsigned ns = 32;
  for (int it = 0; it < kSpinLimit; ++it) {
    const uint32_t w = ld_volatile(wp);
    if (w < kPending) return w;
    if (w == kNone) {
      if (atomicCAS(wp, kNone, kPending) == kNone) {
        const uint32_t in = alloc_inner(M);
        st_publish(wp, in);
        return in;
      }
      continue;
    }
    if (ld_volatile(M.ctr + C_ERR) & ERR_WAIT) return kNone;
    __nanosleep(ns);
    ns = ns < 1024 ? ns * 2 : 1024;
  }
  set_err(M, ERR_WAIT);
  return kNone;
}

// Get-or-create of the inner node of a root key; kNone on failure (error set).
static __device__ __noinline__ uint32_t root_get_or_create(const DMap& M, int x, int y, int z) {
  const uint4 kEmpty = make_uint4(kNone, kNone, kNone, kNone);
  uint32_t h = root_hash(M, x, y, z) & M.hmask;
  for (uint32_t p = 0; p <= M.hmask; ++p, h = (h + 1) & M.hmask) {
    uint4* b = M.buckets + h;
    uint4 v = ld_volatile4(b);
    if (!key_eq(v, x, y, z)) {
      // A fully written other key has no all-ones component.
      if (static_cast<int>(v.x) != kEmptyKey && static_cast<int>(v.y) != kEmptyKey &&
          static_cast<int>(v.z) != kEmptyKey)
        continue;
      v = cas128(b, kEmpty,
                 make_uint4(static_cast<uint32_t>(x), static_cast<uint32_t>(y),
                            static_cast<uint32_t>(z), kPending));
      if (eq4(v, kEmpty)) {
        const uint32_t in = alloc_inner(M);
        st_publish(&b->w, in);
        atomicAdd(M.ctr + C_ROOTS, 1u);
        return in;
      }
      if (!key_eq(v, x, y, z)) continue;
    }
    if (v.w < kPending) return v.w;
    return root_value_wait(M, b);
  }
  set_err(M, ERR_HASH_FULL);
  return kNone;
}

// Fast path of root_get_or_create for hot loops: up to four probes with plain
// (L1-cacheable) loads. kPending means "take the slow path" -- the key is
// missing, still being created, or the probe chain is long. A stale or torn
// read can only look like one of those (a valid key never has an all-ones
// component), so the slow path always settles it.
__device__ __forceinline__ uint32_t root_probe_fast(const DMap& M, int x, int y, int z) {
  uint32_t h = root_hash(M, x, y, z) & M.hmask;
#pragma unroll 1
  for (int p = 0; p < 4; ++p) {
    const uint4 b = M.buckets[h];
    if (key_eq(b, x, y, z)) return b.w < kPending ? b.w : kPending;
    if (static_cast<int>(b.x) == kEmptyKey) return kPending;
    h = (h + 1) & M.hmask;
  }
  return kPending;
}

// ---------------------------------------------------------------------------
// leaves
// ---------------------------------------------------------------------------
static __device__ __noinline__ uint32_t leaf_get_or_create(const DMap& M, uint32_t in, uint32_t ii,
                                                    int lx, int ly, int lz) {
  uint32_t* slot = M.ichild + static_cast<size_t>(in) * M.isize + ii;
  uint32_t c = ld_volatile(slot);
  unsigned ns = 32;
  for (int it = 0; it < kSpinLimit; ++it) {
    if (c < kPending) return c;
    if (c == kNone) {
      const uint32_t old = atomicCAS(slot, kNone, kPending);
      if (old == kNone) {
        const uint32_t lf = alloc_leaf(M);
        st_publish(slot, lf);
        if (lf != kNone) {  // read only by later kernels (iteration, release)
          M.lkey[lf] = make_int4(lx, ly, lz, static_cast<int>(in));
          atomicOr(M.imask + static_cast<size_t>(in) * M.iwords + (ii >> 6),
                   1ull << (ii & 63));
        }
        return lf;
      }
      c = old;
      continue;
    }
    // another wait of this launch already gave up: the call fails anyway
    if (ld_volatile(M.ctr + C_ERR) & ERR_WAIT) return kNone;
    __nanosleep(ns);
    ns = ns < 1024 ? ns * 2 : 1024;
    c = ld_volatile(slot);
  }
  set_err(M, ERR_WAIT);
  return kNone;
}

// Leaf slot holding coord, or kNone. With create, missing roots and leaves are
// created (Accessor::getLeafGrid, bonxai.hpp:588-621).
__device__ __forceinline__ uint32_t leaf_of(const DMap& M, int x, int y, int z, bool create) {
  const int32_t rm = root_mask(M);
  if (!create) {
    const uint32_t in = root_find(M, x & rm, y & rm, z & rm);
    if (in == kNone) return kNone;
    const uint32_t c = M.ichild[static_cast<size_t>(in) * M.isize + inner_index(M, x, y, z)];
    return c < kPending ? c : kNone;
  }
  const uint32_t in = root_get_or_create(M, x & rm, y & rm, z & rm);
  if (in == kNone) return kNone;
  const int32_t lm = leaf_mask(M);
  return leaf_get_or_create(M, in, inner_index(M, x, y, z), x & lm, y & lm, z & lm);
}

__device__ __forceinline__ unsigned long long* mask_word(const DMap& M, uint32_t lf,
                                                          uint32_t ci) {
  return M.lmask + static_cast<size_t>(lf) * M.lwords + (ci >> 6);
}
__device__ __forceinline__ bool cell_is_on(const DMap& M, uint32_t lf, uint32_t ci) {
  return (*mask_word(M, lf, ci) >> (ci & 63)) & 1ull;
}
// Turns the cell on; returns its previous state (Mask::setOn, mask.hpp:351-357).
__device__ __forceinline__ bool cell_set_on(const DMap& M, uint32_t lf, uint32_t ci) {
  const unsigned long long bit = 1ull << (ci & 63);
  return (atomicOr(mask_word(M, lf, ci), bit) & bit) != 0ull;
}
// Turns a cell on without reading the mask first (the result is unused, so
// this compiles to a fire-and-forget reduction).
__device__ __forceinline__ void cell_or_on(const DMap& M, uint32_t lf, uint32_t ci) {
  atomicOr(mask_word(M, lf, ci), 1ull << (ci & 63));
}
// Turns the cell on, skipping the atomic when a plain read already shows it on.
__device__ __forceinline__ void cell_mark_on(const DMap& M, uint32_t lf, uint32_t ci) {
  unsigned long long* w = mask_word(M, lf, ci);
  const unsigned long long bit = 1ull << (ci & 63);
  if (!(*w & bit)) atomicOr(w, bit);
}

// ---------------------------------------------------------------------------
// ProbabilisticMap::CellT packed as GCC lays it out (probabilistic_map.hpp:44-53):
// update_id = signed bits 0-3, probability_log = signed bits 4-31.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t cell_id(int32_t w) {
  return static_cast<int32_t>(static_cast<uint32_t>(w) << 28) >> 28;
}
__device__ __forceinline__ int32_t cell_prob(int32_t w) { return w >> 4; }
__device__ __forceinline__ int32_t cell_pack(int32_t p, int32_t id) {
  return static_cast<int32_t>((static_cast<uint32_t>(p) << 4) |
                              (static_cast<uint32_t>(id) & 0xFu));
}
__device__ __forceinline__ int32_t wrap_add(int32_t a, int32_t b) {
  return static_cast<int32_t>(static_cast<uint32_t>(a) + static_cast<uint32_t>(b));
}

// ---------------------------------------------------------------------------
// Bresenham in closed form.
//
// RayIterator (probabilistic_map.hpp:162-203) starts every error at 0, adds
// |delta| per step and steps an axis when (error << 1) >= max. By induction
// the number of steps axis b has taken after k iterations is
//     n_b(k) = floor((2 k d_b + max) / (2 max)),
// i.e. k*d_b/max rounded half up, and the cells visited are
//     origin + sign * n(k),  k = 0 .. max-1.
// (tests/test_ray_closed_form.py checks this against the iterative form
// exhaustively for small deltas.) A lane that starts at k0 and advances by W
// keeps (n, r) with r = (2 k d_b + max) mod 2max and adds the constant
// quotient/remainder of 2 W d_b by 2max, so the loop needs no division.
// ---------------------------------------------------------------------------
// q, r = divmod(num, den) for quotients below 2^20, via a float estimate and
// one correction step.
__device__ __forceinline__ void divmod_small(uint32_t num, uint32_t den, float rden,
                                             uint32_t& q, uint32_t& r) {
  uint32_t qe = static_cast<uint32_t>(__fmul_rz(static_cast<float>(num), rden));
  long long rr = static_cast<long long>(num) - static_cast<long long>(qe) * den;
  while (rr < 0) {
    --qe;
    rr += den;
  }
  while (rr >= static_cast<long long>(den)) {
    ++qe;
    rr -= den;
  }
  q = qe;
  r = static_cast<uint32_t>(rr);
}

struct AxisStep {
  uint32_t n, r;  // steps taken, remainder
  uint32_t Q, R;  // increment of (n, r) for k += W
};

__device__ __forceinline__ void axis_init(AxisStep& a, uint32_t d, uint32_t m, uint32_t two_m,
                                          float rtm, uint32_t k0, uint32_t W) {
  divmod_small(2u * k0 * d + m, two_m, rtm, a.n, a.r);
  divmod_small(2u * W * d, two_m, rtm, a.Q, a.R);
}
__device__ __forceinline__ void axis_advance(AxisStep& a, uint32_t two_m) {
  a.n += a.Q;
  a.r += a.R;
  if (a.r >= two_m) {
    a.n += 1;
    a.r -= two_m;
  }
}

// Longest ray handled (cells); the reference's own int32 error term overflows
// at 2^30.
constexpr uint32_t kMaxRayCells = 1u << 26;

}  // namespace bxg
