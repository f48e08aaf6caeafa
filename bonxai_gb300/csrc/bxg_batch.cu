// Batched form: one insertPointCloud scan for each of many independent maps
// per tick, in ONE persistent cooperative launch captured in a CUDA graph.
//
// The per-map scan (bxg_pmap.cu) is four small launches with a host sync; a
// 10k-point scan cannot fill 152 SMs, so many small maps spend their time in
// launch and sync latency. Here every phase covers all scans of the tick:
//
//   phase 0  clear the dedup tables and per-scan counters
//   phase 1  endpoints of every point of every scan (compute_endpoint),
//            lowest index per endpoint cell in the scan's own table
//   phase 2  winners apply their hit/miss and join their scan's ray list
//   phase 3  prefix sum of the ray-list lengths (one global ray index space)
//   phase 4  the ray phase of all scans. Two-phase form (every map has a
//            cube bitmap, bxg_mark.cuh): 4a blocks take tasks of consecutive
//            rays of one scan and mark their cells in that map's bitmap; 4b
//            warps list the marked leaf blocks of every map; 4c groups of 8
//            lanes apply each map's listed blocks. Single-pass
//            form otherwise: groups of W lanes walk rays of all scans
//            (walk_ray), each on its own map's pools. Statistics per scan.
//   phase 5  each map's counters are copied to one read-back block
//
// separated by grid barriers (bounded waits: a barrier that times out sets an
// error word and the kernel returns). Each map keeps its own pools; the tick
// touches no state shared between maps except the read-only descriptors. The
// arithmetic is exactly that of the per-map path (bxg_scan.cuh), so the maps
// are bit-identical to inserting the scans one by one.
#include <algorithm>
#include <cstring>
#include <vector>

#include "bxg_internal.h"
#include "bxg_mark.cuh"
#include "bxg_scan.cuh"

namespace bxg {

constexpr uint32_t kMaxTickScans = 128;

// Layout of the per-tick meta buffer; bytes [0, kBackBytes) are read back.
constexpr size_t kOffBar = 0;                                    // 2 x u32
constexpr size_t kOffErr = 8;                                    // u32
constexpr size_t kOffRayNext = 12;                               // u32
constexpr size_t kOffTime = 16;                                  // [8] u64 phase timestamps
constexpr size_t kOffStats = 80;                                 // [128][4] u64
constexpr size_t kOffCnt = kOffStats + kMaxTickScans * 32;       // [128] u32
constexpr size_t kOffCtr = kOffCnt + kMaxTickScans * 4;          // [128][C_WORDS] u32
constexpr size_t kBackBytes = kOffCtr + kMaxTickScans * C_WORDS * 4;
constexpr size_t kOffPrefix = kBackBytes;                        // [129] u32
constexpr size_t kOffTaskPrefix = kOffPrefix + (kMaxTickScans + 1) * 4;  // [129] u32
constexpr size_t kOffChunk = kOffTaskPrefix + (kMaxTickScans + 1) * 4;   // u32
constexpr size_t kMetaBytes = kOffChunk + 16;
// The tick's neighbourhood of shared-memory leaves around each scan's origin.
constexpr int kTickMarkNB = 2;

struct TickScan {
  DMap M;
  double fx, fy, fz, max_range, mr2, inv_res;
  EpFast fast;                   // float filter of the endpoint math
  int32_t ox, oy, oz, u;
  Opts o;
  unsigned long long pt_begin;   // first point of this scan in the tick's arrays
  unsigned long long tab_begin;  // first bucket of this scan's dedup table
  uint32_t n;                    // points
  uint32_t tmask;                // dedup table size - 1
  int32_t keep_nonfinite;
  uint32_t chunk0;  // first chunk (32 touched words) of this scan's cube in the tick's list phase
  RayCube Q;  // the map's cube bitmap (two-phase ray update)
  LeafDir D;  // the map's kept leaf directory (D.words == nullptr: none)
};

static_assert(sizeof(TickScan) % 8 == 0, "TickScan is copied to shared memory in 8-byte words");

struct TickArgs {
  const uint8_t* pts;  // packed float xyz of all scans
  int4* ep;
  uint4* tab;
  int4* cast;                 // ray list of scan s at cast + pt_begin[s]
  uint32_t* cast_cnt;         // [n_scans]
  unsigned long long* stats;  // [n_scans][4]: points, ray length, visited, updated
  uint32_t* ray_prefix;       // [n_scans + 1]
  uint32_t* bar;              // barrier: arrivals, generation
  uint32_t* err;              // barrier timeout
  uint32_t* ray_next;         // next ray (or mark task) taken in phase 4 (zeroed per tick)
  uint32_t* task_prefix;      // [n_scans + 1] first mark task of each scan
  uint32_t* chunk;            // rays per mark task
  uint32_t* ctr_out;          // [n_scans][C_WORDS]
  unsigned long long* times;  // [8] global-timer stamps at each phase boundary
  uint32_t n_scans;
  uint32_t n_chunks;  // chunks of 32 touched words over all scans' cubes
  unsigned long long total_points;
  unsigned long long total_tab;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier for a cooperative launch (all blocks co-resident). The
// wait is bounded: after 2 s the block records the timeout and returns false,
// and the caller leaves the kernel.
__device__ bool grid_barrier(uint32_t* bar, uint32_t* err) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    const uint32_t gen = ld_acquire(bar + 1);
    __threadfence();
    const uint32_t arrived = atomicAdd(bar, 1u) + 1;
    if (arrived == gridDim.x) {
      bar[0] = 0;
      __threadfence();
      st_release(bar + 1, gen + 1);
    } else {
      const unsigned long long t0 = global_ns();
      unsigned ns = 32;
      while (ld_acquire(bar + 1) == gen) {
        if (global_ns() - t0 > 2000000000ull) {
          atomicOr(err, 1u);
          ok = 0;
          break;
        }
        __nanosleep(ns);
        ns = ns < 256 ? ns * 2 : 256;
      }
    }
    __threadfence();
  }
  __syncthreads();
  __threadfence();  // every thread acquires what other blocks wrote before the barrier
  return ok != 0;
}

__device__ __forceinline__ uint32_t scan_of_point(const TickScan* sc, uint32_t n,
                                                  unsigned long long i) {
  uint32_t lo = 0, hi = n;  // last scan with pt_begin <= i
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (sc[mid].pt_begin <= i) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t scan_of_ray(const uint32_t* prefix, uint32_t n, uint32_t r) {
  uint32_t lo = 0, hi = n;  // last scan with prefix <= r
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (prefix[mid] <= r) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t scan_of_task(const uint32_t* prefix, uint32_t n, uint32_t t) {
  uint32_t lo = 0, hi = n;  // last scan with prefix <= t (scans without tasks are skipped)
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (ld_volatile(prefix + mid) <= t) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t scan_of_chunk(const TickScan* sc, uint32_t n, uint32_t c) {
  uint32_t lo = 0, hi = n;  // last scan with chunk0 <= c
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (sc[mid].chunk0 <= c) lo = mid; else hi = mid;
  }
  return lo;
}

// MARK: phase 4 in the two-phase form (every scan has a cube). Dynamic shared
// memory: the scan table (n_scans entries), then, with MARK, the mark
// neighbourhood (mark_smem_words(kTickMarkNB) words).
template <int W, int U, bool MARK>
__global__ void __launch_bounds__(256, U == 2 ? 3 : 4) k_tick(const TickArgs* __restrict__ argp,
                                                 const TickScan* __restrict__ scans_g) {
  extern __shared__ unsigned long long smem_raw[];
  TickScan* sc = reinterpret_cast<TickScan*>(smem_raw);
  __shared__ uint32_t s_task;
  __shared__ uint32_t s_upd[kMaxTickScans];
  const TickArgs A = *argp;
  const uint32_t ns = A.n_scans;
  uint32_t* smk = reinterpret_cast<uint32_t*>(smem_raw + ns * (sizeof(TickScan) / 8));
  {
    const uint32_t words = ns * (sizeof(TickScan) / 8);
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(scans_g);
    for (uint32_t k = threadIdx.x; k < words; k += blockDim.x) smem_raw[k] = src[k];
  }
  __syncthreads();
  const unsigned lane = threadIdx.x & 31;
  const unsigned long long gtid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  const unsigned long long gsize = gridDim.x * (unsigned long long)blockDim.x;

  auto stamp = [&](int k) {
    if (blockIdx.x == 0 && threadIdx.x == 0) A.times[k] = global_ns();
  };
  stamp(0);
  // phase 0: clear tables and counters
  const uint4 kEmpty = make_uint4(kNone, kNone, kNone, kNone);
  for (unsigned long long k = gtid; k < A.total_tab; k += gsize) A.tab[k] = kEmpty;
  for (unsigned long long k = gtid; k < ns; k += gsize) {
    A.cast_cnt[k] = 0;
    for (int j = 0; j < 4; j++) A.stats[4 * k + j] = 0;
    if (MARK) *sc[k].Q.count = 0u;  // the list phase appends from zero
  }
  if (!grid_barrier(A.bar, A.err)) return;
  stamp(1);

  // phase 1: endpoints
  for (unsigned long long i = gtid; i < A.total_points; i += gsize) {
    const uint32_t s = scan_of_point(sc, ns, i);
    const TickScan& S = sc[s];
    const float* p = reinterpret_cast<const float*>(A.pts) + 3 * i;
    const int4 e = compute_endpoint<float>(p, S.fx, S.fy, S.fz, S.max_range, S.mr2, S.inv_res,
                                           S.keep_nonfinite != 0, &S.fast);
    A.ep[i] = e;
    if (e.w != EP_SKIP)
      dedup_min_insert(A.tab + S.tab_begin, S.tmask, e.x, e.y, e.z,
                       static_cast<uint32_t>(i - S.pt_begin), S.M);
  }
  if (!grid_barrier(A.bar, A.err)) return;
  stamp(2);

  // phase 2: winners (warp-uniform loop for the compaction)
  for (unsigned long long wbase = gtid - lane; wbase < A.total_points; wbase += gsize) {
    const unsigned long long i = wbase + lane;
    const bool in = i < A.total_points;
    uint32_t s = 0;
    bool add = false, valid = false;
    int4 e = make_int4(0, 0, 0, EP_SKIP);
    if (in) {
      s = scan_of_point(sc, ns, i);
      const TickScan& S = sc[s];
      e = A.ep[i];
      valid = e.w != EP_SKIP;
      if (valid && dedup_lookup(A.tab + S.tab_begin, S.tmask, e.x, e.y, e.z) ==
                       static_cast<uint32_t>(i - S.pt_begin))
        add = winner_apply(S.M, e, S.u, S.o);
    }
    const uint32_t s0 = __shfl_sync(0xffffffffu, s, 0);
    const bool uniform = __all_sync(0xffffffffu, !in || s == s0);
    const uint32_t len = add ? chebyshev(sc[s].ox, sc[s].oy, sc[s].oz, e.x, e.y, e.z) : 0;
    if (uniform) {
      const unsigned am = __ballot_sync(0xffffffffu, add);
      const unsigned vm = __ballot_sync(0xffffffffu, valid);
      const unsigned tot = __reduce_add_sync(0xffffffffu, len);
      uint32_t base = 0;
      if (lane == 0) {
        if (vm) atomicAdd(A.stats + 4 * s0 + 0, static_cast<unsigned long long>(__popc(vm)));
        if (tot) atomicAdd(A.stats + 4 * s0 + 1, static_cast<unsigned long long>(tot));
        if (am) base = atomicAdd(A.cast_cnt + s0, static_cast<uint32_t>(__popc(am)));
      }
      base = __shfl_sync(0xffffffffu, base, 0);
      if (add) {
        const uint32_t k = base + __popc(am & ((1u << lane) - 1));
        if (k < sc[s0].n) A.cast[sc[s0].pt_begin + k] = e;
      }
    } else if (in) {  // the warp straddles scans: per-lane counters
      if (valid) atomicAdd(A.stats + 4 * s + 0, 1ull);
      if (add) {
        atomicAdd(A.stats + 4 * s + 1, static_cast<unsigned long long>(len));
        const uint32_t k = atomicAdd(A.cast_cnt + s, 1u);
        if (k < sc[s].n) A.cast[sc[s].pt_begin + k] = e;
      }
    }
  }
  if (!grid_barrier(A.bar, A.err)) return;
  stamp(3);

  // phase 3: one index space over all ray lists (and, with MARK, over the
  // mark tasks: about four per block, at least 64 rays each)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    uint32_t acc = 0;
    for (uint32_t s = 0; s < ns; s++) {
      A.ray_prefix[s] = acc;
      acc += min(ld_volatile(A.cast_cnt + s), sc[s].n);
    }
    A.ray_prefix[ns] = acc;
    if (MARK) {
      const uint32_t chunk = max(64u, (acc + 4u * gridDim.x - 1) / (4u * gridDim.x));
      uint32_t tacc = 0;
      for (uint32_t s = 0; s < ns; s++) {
        A.task_prefix[s] = tacc;
        tacc += (A.ray_prefix[s + 1] - A.ray_prefix[s] + chunk - 1) / chunk;
      }
      A.task_prefix[ns] = tacc;
      *A.chunk = chunk;
    }
  }
  if (!grid_barrier(A.bar, A.err)) return;
  stamp(4);

  // phase 4: rays of all scans
  if (MARK) {
    // 4a: mark
    __shared__ MarkRays<256> s_rays;
    for (int t = threadIdx.x; t < mark_smem_words(kTickMarkNB); t += blockDim.x) smk[t] = 0u;
    const uint32_t n_tasks = ld_volatile(A.task_prefix + ns);
    const uint32_t chunk = ld_volatile(A.chunk);
    for (;;) {
      __syncthreads();
      if (threadIdx.x == 0) s_task = atomicAdd(A.ray_next, 1u);
      __syncthreads();
      const uint32_t t = s_task;
      if (t >= n_tasks) break;
      const uint32_t s = scan_of_task(A.task_prefix, ns, t);
      const TickScan& S = sc[s];
      const uint32_t rays = ld_volatile(A.ray_prefix + s + 1) - ld_volatile(A.ray_prefix + s);
      const uint32_t r0 = (t - ld_volatile(A.task_prefix + s)) * chunk;
      uint32_t visited = 0;
      mark_rays_block<kTickMarkNB, 256>(S.M, S.Q, A.cast + S.pt_begin, r0, min(rays, r0 + chunk),
                                        S.ox, S.oy, S.oz, smk, s_rays, visited);
      visited = __reduce_add_sync(0xffffffffu, visited);
      if (lane == 0 && visited)
        atomicAdd(A.stats + 4 * s + 2, static_cast<unsigned long long>(visited));
    }
    if (!grid_barrier(A.bar, A.err)) return;
    stamp(6);
    // 4b: the marked blocks of every cube onto its list (a warp per 32
    // touched words, all scans in one index space)
    for (uint32_t c = static_cast<uint32_t>(gtid >> 5); c < A.n_chunks;
         c += static_cast<uint32_t>(gsize >> 5)) {
      const uint32_t s = scan_of_chunk(sc, ns, c);
      list_touched(sc[s].M, sc[s].Q, c - sc[s].chunk0);
    }
    if (!grid_barrier(A.bar, A.err)) return;
    stamp(7);
    // 4c: apply, 8 lanes per listed leaf block; each scan's list is taken in
    // a rotated order so that its first entries do not always go to the same
    // groups
    for (uint32_t k = threadIdx.x; k < ns; k += blockDim.x) s_upd[k] = 0u;
    __syncthreads();
    {
      const unsigned sl = lane & (kApplyGroup - 1), gbase = lane & ~unsigned(kApplyGroup - 1);
      const unsigned gmask = ((1u << kApplyGroup) - 1u) << gbase;
      const uint32_t gid = static_cast<uint32_t>(gtid / kApplyGroup);
      const uint32_t ng = static_cast<uint32_t>(gsize / kApplyGroup);
      for (uint32_t s = 0; s < ns; ++s) {
        const TickScan& S = sc[s];
        const uint32_t n = min(ld_volatile(S.Q.count), S.Q.cap);
        uint32_t upd = 0;
        for (uint32_t i = (gid + s * 977u) % ng; i < n; i += ng)
          apply_block(S.M, S.Q, S.Q.list[i], S.u, S.o.miss, S.o.cmin, sl, gbase, gmask, upd,
                      S.D.words ? &S.D : nullptr);
        if (upd) atomicAdd(s_upd + s, upd);
      }
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < ns; k += blockDim.x)
      if (s_upd[k]) atomicAdd(A.stats + 4 * k + 3, static_cast<unsigned long long>(s_upd[k]));
  } else {
    const unsigned sl = lane & (W - 1);
    const unsigned gbase = lane & ~(W - 1);
    const unsigned gmask = (W == 32) ? 0xffffffffu : (((1u << W) - 1u) << gbase);
    const uint32_t total = ld_volatile(A.ray_prefix + ns);
    uint32_t visited = 0, updated = 0, cur = kNone;
    // Rays are taken dynamically (lengths vary widely), kRayChunk consecutive
    // rays per atomic: a tick holds millions of rays, and one atomic per ray
    // on one counter cost 9 % of the ray phase. The leader takes the next
    // chunk before walking the current one.
    constexpr uint32_t kRayChunk = 4;
    uint32_t r = 0;
    if (sl == 0) r = atomicAdd(A.ray_next, kRayChunk);
    r = __shfl_sync(gmask, r, 0, W);
    while (r < total) {
      uint32_t nr = 0;
      if (sl == 0) nr = atomicAdd(A.ray_next, kRayChunk);
      const uint32_t r_end = min(r + kRayChunk, total);
      for (; r < r_end; ++r) {
        const uint32_t s = scan_of_ray(A.ray_prefix, ns, r);
        if (s != cur) {
          if (cur != kNone) {
            const uint32_t v = __reduce_add_sync(gmask, visited), up = __reduce_add_sync(gmask, updated);
            if (sl == 0 && v) {
              atomicAdd(A.stats + 4 * cur + 2, static_cast<unsigned long long>(v));
              atomicAdd(A.stats + 4 * cur + 3, static_cast<unsigned long long>(up));
            }
          }
          visited = updated = 0;
          cur = s;
        }
        const TickScan& S = sc[s];
        const int4 e = A.cast[S.pt_begin + (r - A.ray_prefix[s])];
        if (U == 2)
          walk_ray2<W>(S.M, e, S.ox, S.oy, S.oz, S.u, S.o.miss, S.o.cmin, sl, gbase, gmask,
                       visited, updated);
        else
          walk_ray<W>(S.M, e, S.ox, S.oy, S.oz, S.u, S.o.miss, S.o.cmin, sl, gbase, gmask,
                      visited, updated);
      }
      r = __shfl_sync(gmask, nr, 0, W);
    }
    if (cur != kNone) {
      const uint32_t v = __reduce_add_sync(gmask, visited), up = __reduce_add_sync(gmask, updated);
      if (sl == 0 && v) {
        atomicAdd(A.stats + 4 * cur + 2, static_cast<unsigned long long>(v));
        atomicAdd(A.stats + 4 * cur + 3, static_cast<unsigned long long>(up));
      }
    }
  }
  if (!grid_barrier(A.bar, A.err)) return;
  stamp(5);

  // phase 5: every map's counters into one read-back block
  for (unsigned long long k = gtid; k < static_cast<unsigned long long>(ns) * C_WORDS; k += gsize)
    A.ctr_out[k] = ld_volatile(sc[k / C_WORDS].M.ctr + (k % C_WORDS));
}

}  // namespace bxg

using namespace bxg;

struct bxg_batch_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint32_t rays_per_warp = 1;
  uint32_t ray_unroll = 1;
  int sm_count = 0;
  int grid = 0;       // resident blocks of the single-pass tick
  int grid_mark = 0;  // resident blocks of the two-phase tick
  size_t grid_smem[2] = {0, 0};  // dynamic shared memory the two were sized for
  bool use_graph = true;
  // device buffers
  DevBuf pts, ep, tab, cast, meta, params;
  // pinned host staging
  TickArgs* h_args = nullptr;
  TickScan* h_scans = nullptr;
  unsigned char* h_back = nullptr;  // read-back: err | stats | cast_cnt | ctr_out
  size_t back_bytes = 0;
  // graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool graph_ok = false;
  uint64_t graph_key[7] = {0};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0;
  double phase_ms[6] = {0, 0, 0, 0, 0, 0};  // [5]: the mark part of the ray phase
  uint64_t last_retries = 0, ticks = 0, launches = 0;
  std::string err;
  ~bxg_batch_s() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (h_args) cudaFreeHost(h_args);  // h_scans lives inside this allocation
    if (h_back) cudaFreeHost(h_back);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int bfail(bxg_batch b, int st, const std::string& m) {
  b->err = m;
  return st;
}
#define BB_CUDA(b, call)                                                               \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      cudaGetLastError();                                                              \
      return bfail((b), BXG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    }                                                                                  \
  } while (0)

uint32_t pow2_at_least(uint64_t v) {
  uint32_t p = 64;
  while (p < v) p <<= 1;
  return p;
}

template <int W, int U, bool MARK>
int occupancy_grid(bxg_batch b, size_t smem) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tick<W, U, MARK>, 256, smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per_sm * b->sm_count;
}

// Dynamic shared memory of a tick of ns scans: the scan table, plus the mark
// neighbourhood in the two-phase form.
size_t tick_smem(bool mark, size_t ns) {
  return ns * sizeof(TickScan) + (mark ? size_t(mark_smem_words(kTickMarkNB)) * 4 : 0);
}

template <int W, int U, bool MARK>
cudaError_t launch_tick(bxg_batch b, size_t smem) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(MARK ? b->grid_mark : b->grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = b->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const TickArgs* a = b->params.as<TickArgs>();
  const TickScan* s = reinterpret_cast<const TickScan*>(b->params.as<uint8_t>() + 256);
  return cudaLaunchKernelEx(&cfg, k_tick<W, U, MARK>, a, s);
}

cudaError_t launch_for(bxg_batch b, size_t smem, bool mark) {
  if (mark) return launch_tick<32, 1, true>(b, smem);
  const bool u2 = b->ray_unroll == 2;
  switch (b->rays_per_warp) {
    case 4: return u2 ? launch_tick<8, 2, false>(b, smem) : launch_tick<8, 1, false>(b, smem);
    case 2: return u2 ? launch_tick<16, 2, false>(b, smem) : launch_tick<16, 1, false>(b, smem);
    default: return u2 ? launch_tick<32, 2, false>(b, smem) : launch_tick<32, 1, false>(b, smem);
  }
}

// Enqueues one tick: parameters up, the persistent kernel, results back.
cudaError_t enqueue_tick(bxg_batch b, size_t param_bytes, size_t smem, bool mark) {
  cudaError_t e = cudaMemcpyAsync(b->params.p, b->h_args, param_bytes, cudaMemcpyHostToDevice,
                                  b->stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(b->meta.p, 0, 16, b->stream);  // barrier, error and ray-counter words
  if (e != cudaSuccess) return e;
  e = launch_for(b, smem, mark);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(b->h_back, b->meta.p, kBackBytes, cudaMemcpyDeviceToHost, b->stream);
}

}  // namespace

extern "C" {

int bxg_batch_create(bxg_batch* out, const bxg_config* cfg_in) {
  if (!out) return BXG_ERR_INVALID_ARG;
  *out = nullptr;
  bxg_config cfg;
  bxg_config_default(&cfg);
  if (cfg_in) cfg = *cfg_in;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return BXG_ERR_NO_DEVICE;
  }
  bxg_batch b = new bxg_batch_s();
  if (cfg.device >= 0) cudaSetDevice(cfg.device);
  cudaGetDevice(&b->device);
  cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device);
  b->rays_per_warp = cfg.rays_per_warp == 2 || cfg.rays_per_warp == 4 ? cfg.rays_per_warp : 1;
  b->ray_unroll = cfg.ray_unroll == 2 ? 2 : 1;
  b->use_graph = (cfg.flags & 4u) == 0;  // BXG_FLAG_NO_GRAPH
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return BXG_ERR_CUDA;
  }
  const int smem = int(tick_smem(false, kMaxTickScans));
  cudaFuncSetAttribute(k_tick<32, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaFuncSetAttribute(k_tick<16, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaFuncSetAttribute(k_tick<8, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaFuncSetAttribute(k_tick<32, 2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaFuncSetAttribute(k_tick<16, 2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaFuncSetAttribute(k_tick<8, 2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaFuncSetAttribute(k_tick<32, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(tick_smem(true, kMaxTickScans)));
  cudaGetLastError();
  const size_t pbytes = 256 + kMaxTickScans * sizeof(TickScan);
  if (cudaMallocHost(reinterpret_cast<void**>(&b->h_args), pbytes) != cudaSuccess ||
      b->params.ensure(pbytes) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return BXG_ERR_CUDA;
  }
  b->h_scans = reinterpret_cast<TickScan*>(reinterpret_cast<uint8_t*>(b->h_args) + 256);
  *out = b;
  return BXG_OK;
}

int bxg_batch_destroy(bxg_batch b) {
  delete b;
  return BXG_OK;
}

const char* bxg_batch_last_error(bxg_batch b) { return b ? b->err.c_str() : "null handle"; }

int bxg_batch_insert_f32(bxg_batch b, const bxg_pmap* maps, size_t n_scans, const float* xyz,
                         const uint64_t* offsets, const float* origins, const double* max_ranges,
                         uint64_t* ray_cells) {
  if (!b) return BXG_ERR_INVALID_ARG;
  if (!n_scans) return BXG_OK;
  if (!maps || !xyz || !offsets || !origins || !max_ranges)
    return bfail(b, BXG_ERR_INVALID_ARG, "null argument");
  if (n_scans > kMaxTickScans)
    return bfail(b, BXG_ERR_INVALID_ARG, "at most 128 scans per tick");
  for (size_t s = 0; s < n_scans; s++) {
    if (!maps[s] || maps[s]->core.device != b->device)
      return bfail(b, BXG_ERR_INVALID_ARG, "every map must live on the batch's device");
    for (size_t t = 0; t < s; t++)
      if (maps[t] == maps[s]) return bfail(b, BXG_ERR_INVALID_ARG, "a map appears twice in one tick");
    if (offsets[s + 1] < offsets[s] || offsets[s + 1] - offsets[s] >= 0x7FFFFFFFu)
      return bfail(b, BXG_ERR_INVALID_ARG, "bad offsets");
    if (maps[s]->cast_ub) return bfail(b, BXG_ERR_INVALID_ARG, "a map has queued rays");
  }
  cudaSetDevice(b->device);
  const uint64_t total = offsets[n_scans];

  // Pool headroom for every map (host side, before the graph runs).
  for (size_t s = 0; s < n_scans; s++) {
    bxg_pmap_s* pm = maps[s];
    const uint64_t n = offsets[s + 1] - offsets[s];
    const size_t want = std::max<size_t>({size_t(2) * pm->last_new_leaves, size_t(n / 4), 1024});
    const int st = core_reserve(&pm->core, want, std::max<size_t>(n / 64, 256));
    if (st) return bfail(b, st, pm->core.err);
  }

  // Device buffers (growing them invalidates the captured graph).
  uint64_t tab_total = 0;
  for (size_t s = 0; s < n_scans; s++) tab_total += pow2_at_least(2 * (offsets[s + 1] - offsets[s]));
  const void* dpts = xyz;
  const int pts_dev = ptr_device(xyz);
  // points in another GPU's memory are copied like host points (never read in place)
  const bool host_pts = pts_dev != b->device && pts_dev != kPtrManaged;
  bool realloc = false;
  auto grow = [&](DevBuf& d, size_t bytes) -> cudaError_t {
    if (bytes <= d.cap) return cudaSuccess;
    realloc = true;
    return d.ensure(bytes);
  };
  if (host_pts) BB_CUDA(b, grow(b->pts, total * 12 + 16));
  BB_CUDA(b, grow(b->ep, total * 16 + 16));
  BB_CUDA(b, grow(b->cast, total * 16 + 16));
  BB_CUDA(b, grow(b->tab, tab_total * 16 + 16));
  BB_CUDA(b, grow(b->meta, kMetaBytes));
  if (!b->h_back) {
    BB_CUDA(b, cudaMallocHost(reinterpret_cast<void**>(&b->h_back), kBackBytes));
  }
  if (host_pts) {
    if (pts_dev >= 0)
      BB_CUDA(b, cudaMemcpyPeerAsync(b->pts.p, b->device, xyz, pts_dev, total * 12, b->stream));
    else
      BB_CUDA(b, cudaMemcpyAsync(b->pts.p, xyz, total * 12, cudaMemcpyHostToDevice, b->stream));
    dpts = b->pts.p;
  }

  // Parameters of this tick.
  uint8_t* meta = b->meta.as<uint8_t>();
  TickArgs& A = *b->h_args;
  A.pts = static_cast<const uint8_t*>(dpts);
  A.ep = b->ep.as<int4>();
  A.tab = b->tab.as<uint4>();
  A.cast = b->cast.as<int4>();
  A.bar = reinterpret_cast<uint32_t*>(meta + kOffBar);
  A.err = reinterpret_cast<uint32_t*>(meta + kOffErr);
  A.ray_next = reinterpret_cast<uint32_t*>(meta + kOffRayNext);
  A.stats = reinterpret_cast<unsigned long long*>(meta + kOffStats);
  A.cast_cnt = reinterpret_cast<uint32_t*>(meta + kOffCnt);
  A.ctr_out = reinterpret_cast<uint32_t*>(meta + kOffCtr);
  A.times = reinterpret_cast<unsigned long long*>(meta + kOffTime);
  A.ray_prefix = reinterpret_cast<uint32_t*>(meta + kOffPrefix);
  A.task_prefix = reinterpret_cast<uint32_t*>(meta + kOffTaskPrefix);
  A.chunk = reinterpret_cast<uint32_t*>(meta + kOffChunk);
  A.n_scans = uint32_t(n_scans);
  A.total_points = total;
  A.total_tab = tab_total;
  uint64_t tb = 0;
  for (size_t s = 0; s < n_scans; s++) {
    bxg_pmap_s* pm = maps[s];
    TickScan& S = b->h_scans[s];
    std::memset(&S, 0, sizeof(S));
    S.M = pm->core.dm;
    S.fx = origins[3 * s];
    S.fy = origins[3 * s + 1];
    S.fz = origins[3 * s + 2];
    S.max_range = max_ranges[s];
    S.mr2 = max_ranges[s] * max_ranges[s];
    S.inv_res = pm->core.inv_res;
    S.fast = make_ep_fast(S.fx, S.fy, S.fz, S.max_range, S.inv_res);
    S.ox = static_cast<int>(std::floor(S.fx * pm->core.inv_res));
    S.oy = static_cast<int>(std::floor(S.fy * pm->core.inv_res));
    S.oz = static_cast<int>(std::floor(S.fz * pm->core.inv_res));
    S.u = pm->update_count;
    S.o = Opts{pm->opt.prob_miss_log, pm->opt.prob_hit_log, pm->opt.clamp_min_log,
               pm->opt.clamp_max_log};
    S.pt_begin = offsets[s];
    S.n = uint32_t(offsets[s + 1] - offsets[s]);
    const uint32_t tcap = pow2_at_least(2 * uint64_t(S.n));
    S.tab_begin = tb;
    S.tmask = tcap - 1;
    tb += tcap;
    S.keep_nonfinite = (pm->core.flags & BXG_FLAG_KEEP_NONFINITE) ? 1 : 0;
  }
  // The two-phase ray update when every map can have its cube bitmap (each
  // map's own buffers, zero between scans; growing them synchronises the map).
  bool mark = true;
  for (size_t s = 0; s < n_scans && mark; s++) {
    TickScan& S = b->h_scans[s];
    bool ok = false;
    const int st = cube_for_scan(maps[s], S.ox, S.oy, S.oz, S.max_range, &S.Q, &ok);
    if (st) return bfail(b, st, maps[s]->core.err);
    mark = ok;
  }
  // the list phase's index space: 32 touched words per chunk, scan after scan
  A.n_chunks = 0;
  for (size_t s = 0; s < n_scans && mark; s++) {
    TickScan& S = b->h_scans[s];
    S.chunk0 = A.n_chunks;
    A.n_chunks += (cube_touched_words(S.Q) + 31u) / 32u;
  }
  // each map's kept leaf directory for the apply phase (its memsets go on the
  // batch's stream, ahead of the tick)
  for (size_t s = 0; s < n_scans && mark; s++) {
    TickScan& S = b->h_scans[s];
    maps[s]->dir_reach = S.max_range;
    const int st = leaf_dir_for_scan(maps[s], S.ox, S.oy, S.oz, &S.D, size_t(1) << 23, b->stream);
    maps[s]->dir_reach = 0.0;
    if (st) return bfail(b, st, maps[s]->core.err);
  }
  b->back_bytes = kBackBytes;
  const size_t param_bytes = 256 + n_scans * sizeof(TickScan);
  const size_t smem = tick_smem(mark, n_scans);
  // resident blocks for this shared-memory size (the launch is cooperative)
  if (mark && (!b->grid_mark || b->grid_smem[1] != smem)) {
    b->grid_mark = occupancy_grid<32, 1, true>(b, smem);
    b->grid_smem[1] = smem;
    if (b->grid_mark <= 0) return bfail(b, BXG_ERR_CUDA, "k_tick cannot be resident");
  } else if (!mark && (!b->grid || b->grid_smem[0] != smem)) {
    const bool u2 = b->ray_unroll == 2;
    switch (b->rays_per_warp) {
      case 4: b->grid = u2 ? occupancy_grid<8, 2, false>(b, smem) : occupancy_grid<8, 1, false>(b, smem); break;
      case 2: b->grid = u2 ? occupancy_grid<16, 2, false>(b, smem) : occupancy_grid<16, 1, false>(b, smem); break;
      default: b->grid = u2 ? occupancy_grid<32, 2, false>(b, smem) : occupancy_grid<32, 1, false>(b, smem); break;
    }
    b->grid_smem[0] = smem;
    if (b->grid <= 0) return bfail(b, BXG_ERR_CUDA, "k_tick cannot be resident");
  }

  // Run: the captured graph when its shape matches, else capture it again.
  const uint64_t key[7] = {uint64_t(b->params.p), param_bytes, uint64_t(b->meta.p), b->back_bytes,
                           uint64_t(mark ? b->grid_mark : b->grid), b->rays_per_warp,
                           mark ? 1ull : 0ull};
  cudaEventRecord(b->ev0, b->stream);
  bool ran = false;
  if (b->use_graph) {
    if (!b->graph_ok || realloc || std::memcmp(key, b->graph_key, sizeof(key)) != 0) {
      if (b->exec) cudaGraphExecDestroy(b->exec);
      if (b->graph) cudaGraphDestroy(b->graph);
      b->exec = nullptr;
      b->graph = nullptr;
      b->graph_ok = false;
      if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const cudaError_t e1 = enqueue_tick(b, param_bytes, smem, mark);
        const cudaError_t e2 = cudaStreamEndCapture(b->stream, &b->graph);
        if (e1 == cudaSuccess && e2 == cudaSuccess &&
            cudaGraphInstantiate(&b->exec, b->graph, 0) == cudaSuccess) {
          b->graph_ok = true;
          std::memcpy(b->graph_key, key, sizeof(key));
        }
      }
      cudaGetLastError();
    }
    if (b->graph_ok) {
      BB_CUDA(b, cudaGraphLaunch(b->exec, b->stream));
      ran = true;
    }
  }
  if (!ran) BB_CUDA(b, enqueue_tick(b, param_bytes, smem, mark));
  cudaEventRecord(b->ev1, b->stream);
  BB_CUDA(b, cudaStreamSynchronize(b->stream));
  b->launches++;
  cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
  b->ticks++;

  // Results: barrier health, per-map counters, statistics, ray lists.
  if (*reinterpret_cast<const uint32_t*>(b->h_back + kOffErr))
    return bfail(b, BXG_ERR_WAIT_TIMEOUT, "a grid barrier timed out");
  {
    const unsigned long long* ts = reinterpret_cast<const unsigned long long*>(b->h_back + kOffTime);
    for (int k = 0; k < 5; k++) b->phase_ms[k] = double(ts[k + 1] - ts[k]) * 1e-6;
    b->phase_ms[5] = mark ? double(ts[6] - ts[4]) * 1e-6 : 0.0;
  }
  const unsigned long long* stats =
      reinterpret_cast<const unsigned long long*>(b->h_back + kOffStats);
  const uint32_t* cnt = reinterpret_cast<const uint32_t*>(b->h_back + kOffCnt);
  const uint32_t* ctr = reinterpret_cast<const uint32_t*>(b->h_back + kOffCtr);
  b->last_retries = 0;
  int status = BXG_OK;
  for (size_t s = 0; s < n_scans; s++) {
    bxg_pmap_s* pm = maps[s];
    MapCore* m = &pm->core;
    const uint32_t prev_leaves = m->h_ctr[C_LEAF];
    std::memcpy(m->h_ctr, ctr + s * C_WORDS, C_WORDS * 4);
    m->dm.has_free = m->h_ctr[C_FREE_LEAF] > 0 ? 1u : 0u;
    const uint32_t e = m->h_ctr[C_ERR];
    if (e & (ERR_POOL_INNER | ERR_POOL_LEAF | ERR_HASH_FULL)) {
      b->last_retries++;
      const TickScan& S = b->h_scans[s];
      const int st = pmap_complete_scan(pm, b->cast.as<int4>() + S.pt_begin,
                                        A.cast_cnt + s, S.n, S.ox, S.oy, S.oz, S.u);
      if (st && !status) {
        status = st;
        b->err = m->err;
      }
    } else if (e) {
      const int cs = core_sync(m);  // clears the bits, maps them to a status
      if (!status) {
        status = cs ? cs : BXG_ERR_INVALID_ARG;
        b->err = m->err;
      }
    }
    pm->last_new_leaves = m->h_ctr[C_LEAF] > prev_leaves ? m->h_ctr[C_LEAF] - prev_leaves : 0;
    pm->last_stats[0] = stats[4 * s + 0];
    pm->last_stats[1] = cnt[s];
    pm->last_stats[2] = stats[4 * s + 2];
    pm->last_stats[3] = stats[4 * s + 3];
    pm->last_stats[4] = m->h_ctr[C_LEAF];
    if (ray_cells) ray_cells[s] = stats[4 * s + 0] + stats[4 * s + 1];
    if (++pm->update_count == 4) pm->update_count = 1;
  }
  return status;
}

int bxg_batch_phase_ms(bxg_batch b, double out[6]) {
  if (!b || !out) return BXG_ERR_INVALID_ARG;
  for (int k = 0; k < 6; k++) out[k] = b->phase_ms[k];
  return BXG_OK;
}

int bxg_batch_stats(bxg_batch b, double out[8]) {
  if (!b || !out) return BXG_ERR_INVALID_ARG;
  out[0] = b->last_ms;
  out[1] = b->graph_ok ? 1 : 0;
  out[2] = double(b->last_retries);
  out[3] = double(b->ticks);
  out[4] = double(b->grid_mark ? b->grid_mark : b->grid);
  out[5] = double(b->launches);
  out[6] = b->phase_ms[1];  // endpoints
  out[7] = b->phase_ms[2] + b->phase_ms[4];  // winners + rays
  return BXG_OK;
}

}  // extern "C"
