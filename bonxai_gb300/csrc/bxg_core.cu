// Map lifecycle, node pools and their growth, counters, staging, iteration,
// serialization.
#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "bxg_internal.h"

namespace bxg {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
__global__ void k_fill_u32(uint32_t* p, uint32_t v, size_t n) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x)
    p[i] = v;
}

// Re-inserts the old root buckets into a larger, empty table.
__global__ void k_rehash(const uint4* __restrict__ old_b, uint32_t old_cap, const __grid_constant__ DMap M) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= old_cap) return;
  const uint4 b = old_b[i];
  if (static_cast<int>(b.x) == kEmptyKey) return;
  const uint4 kEmpty = make_uint4(kNone, kNone, kNone, kNone);
  uint32_t h = root_hash(M, int(b.x), int(b.y), int(b.z)) & M.hmask;
  for (uint32_t p = 0; p <= M.hmask; ++p, h = (h + 1) & M.hmask) {
    const uint4 old = cas128(M.buckets + h, kEmpty, b);
    if (eq4(old, kEmpty)) return;
  }
  set_err(M, ERR_HASH_FULL);
}

// Counts active cells: popcount of every leaf mask word.
__global__ void k_count_on(const unsigned long long* __restrict__ lmask, size_t nwords,
                           unsigned long long* out) {
  unsigned long long c = 0;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < nwords;
       i += size_t(gridDim.x) * blockDim.x)
    c += __popcll(lmask[i]);
  c = __reduce_add_sync(0xffffffffu, static_cast<unsigned>(c));
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// forEachCell as a compaction (bonxai.hpp:703-743): one thread per leaf mask
// word writes the coordinates (and values) of its on cells. mode 0 = every
// cell; 1 = ProbabilisticMap cells with probability_log > thr; 2 = < thr.
template <int ESZ>
__global__ void k_dump(const __grid_constant__ DMap M, uint32_t n_leaves, int32_t* __restrict__ out_xyz,
                       uint8_t* __restrict__ out_val, size_t cap,
                       unsigned long long* __restrict__ counter, int mode, int32_t thr) {
  const size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  const uint32_t leaf = static_cast<uint32_t>(t / M.lwords);
  const uint32_t wi = static_cast<uint32_t>(t % M.lwords);
  unsigned long long w = 0;
  int4 key = make_int4(0, 0, 0, -1);
  if (leaf < n_leaves) {
    key = M.lkey[leaf];
    if (key.w != -1) w = M.lmask[static_cast<size_t>(leaf) * M.lwords + wi];
  }
  if (mode != 0 && w) {
    const int32_t* cells = reinterpret_cast<const int32_t*>(M.ldata) +
                           static_cast<size_t>(leaf) * M.lsize + wi * 64;
    unsigned long long f = 0, rest = w;
    while (rest) {
      const int b = __ffsll(static_cast<long long>(rest)) - 1;
      rest &= rest - 1;
      const int32_t p = cell_prob(cells[b]);
      if (mode == 1 ? p > thr : p < thr) f |= 1ull << b;
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
  const int lm = (1 << M.lb) - 1;
  while (w) {
    const int b = __ffsll(static_cast<long long>(w)) - 1;
    w &= w - 1;
    const uint32_t ci = wi * 64 + b;
    if (pos < cap) {
      out_xyz[3 * pos + 0] = key.x | static_cast<int>(ci & lm);
      out_xyz[3 * pos + 1] = key.y | static_cast<int>((ci >> M.lb) & lm);
      out_xyz[3 * pos + 2] = key.z | static_cast<int>((ci >> (2 * M.lb)) & lm);
      if (ESZ > 0 && out_val) {
        const uint8_t* src = M.ldata + (static_cast<size_t>(leaf) * M.lsize + ci) * ESZ;
        uint8_t* dst = out_val + pos * ESZ;
        if (ESZ == 4) {
          *reinterpret_cast<uint32_t*>(dst) = *reinterpret_cast<const uint32_t*>(src);
        } else if (ESZ == 8) {
          *reinterpret_cast<unsigned long long*>(dst) =
              *reinterpret_cast<const unsigned long long*>(src);
        } else {
          for (int k = 0; k < ESZ; k++) dst[k] = src[k];
        }
      }
    }
    pos++;
  }
}

void launch_rehash(MapCore* m, const uint4* old_b, uint32_t old_cap, const DMap& M) {
  if (old_cap) k_rehash<<<(old_cap + 255) / 256, 256, 0, m->stream>>>(old_b, old_cap, M);
}

static thread_local std::string g_create_error;
void set_create_error(const std::string& msg) { g_create_error = msg; }

void launch_dedup_clear(MapCore* m, uint4* tab, uint32_t cap) {
  cudaMemsetAsync(tab, 0xFF, size_t(cap) * sizeof(uint4), m->stream);
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
MapCore::~MapCore() {
  if (device >= 0) cudaSetDevice(device);
  if (stream) cudaStreamSynchronize(stream);
  for (DevBuf* b : {&buckets, &ichild, &imask, &lmask, &ldata, &lkey, &lfree, &ctr, &s_in,
                    &s_in2, &s_out, &s_out2, &s_dedup, &s_dedup2, &s_ep, &s_cast, &s_tmp, &s_dir})
    b->release();
  if (h_ctr) cudaFreeHost(h_ctr);
  if (own_stream && stream) cudaStreamDestroy(stream);
}

int ptr_device(const void* p) {
  if (!p) return kPtrHost;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return kPtrHost;
  }
  if (a.type == cudaMemoryTypeManaged) return kPtrManaged;
  if (a.type == cudaMemoryTypeDevice) return a.device;
  return kPtrHost;
}

bool is_device_ptr(const void* p) { return ptr_device(p) != kPtrHost; }

int set_error(MapCore* m, int status, const std::string& msg) {
  if (m) m->err = msg;
  return status;
}

int cuda_fail(MapCore* m, cudaError_t e, const char* what) {
  cudaGetLastError();
  return set_error(m, BXG_ERR_CUDA,
                   std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

static size_t bytes_inner(const MapCore* m, size_t cap) {
  return cap * (size_t(m->dm.isize) * 4 + size_t(m->dm.iwords) * 8);
}
static size_t bytes_leaf(const MapCore* m, size_t cap) {
  return cap * (size_t(m->dm.lwords) * 8 + size_t(m->dm.lsize) * m->dm.esz + 16 + 4);
}
static size_t bytes_hash(size_t cap) { return cap * 16; }

size_t core_mem_usage(const MapCore* m) {
  return bytes_hash(size_t(m->dm.hmask) + 1) + bytes_inner(m, m->dm.icap) +
         bytes_leaf(m, m->dm.lcap);
}

static int grow_inner(MapCore* m, size_t want) {
  const size_t old = m->dm.icap;
  if (want <= old) return BXG_OK;
  if (want > 0xF0000000u) want = 0xF0000000u;
  if (core_mem_usage(m) + bytes_inner(m, want) - bytes_inner(m, old) > m->budget)
    return set_error(m, BXG_ERR_OUT_OF_POOL, "inner-node pool would exceed the HBM budget");
  DevBuf nc, nm;
  BXG_CUDA(m, nc.ensure(want * m->dm.isize * 4));
  BXG_CUDA(m, nm.ensure(want * m->dm.iwords * 8));
  BXG_CUDA(m, cudaMemsetAsync(nc.p, 0xFF, want * m->dm.isize * 4, m->stream));
  BXG_CUDA(m, cudaMemsetAsync(nm.p, 0, want * m->dm.iwords * 8, m->stream));
  if (old) {
    BXG_CUDA(m, cudaMemcpyAsync(nc.p, m->ichild.p, old * m->dm.isize * 4,
                                cudaMemcpyDeviceToDevice, m->stream));
    BXG_CUDA(m, cudaMemcpyAsync(nm.p, m->imask.p, old * m->dm.iwords * 8,
                                cudaMemcpyDeviceToDevice, m->stream));
  }
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  m->ichild.release();
  m->imask.release();
  m->ichild = nc;
  m->imask = nm;
  nc.p = nm.p = nullptr;
  m->dm.ichild = m->ichild.as<uint32_t>();
  m->dm.imask = m->imask.as<unsigned long long>();
  m->dm.icap = static_cast<uint32_t>(want);
  return BXG_OK;
}

static int grow_leaf(MapCore* m, size_t want) {
  const size_t old = m->dm.lcap;
  if (want <= old) return BXG_OK;
  if (want > 0xF0000000u) want = 0xF0000000u;
  if (core_mem_usage(m) + bytes_leaf(m, want) - bytes_leaf(m, old) > m->budget) {
    // grow as far as the budget allows
    const size_t per = bytes_leaf(m, 1);
    const size_t room = m->budget > core_mem_usage(m) ? m->budget - core_mem_usage(m) : 0;
    const size_t fit = old + room / per;
    if (fit <= old) return set_error(m, BXG_ERR_OUT_OF_POOL, "leaf pool reached the HBM budget");
    want = fit;
  }
  const size_t dbytes = want * m->dm.lsize * size_t(m->dm.esz);
  DevBuf nm, nd, nk, nf;
  BXG_CUDA(m, nm.ensure(want * m->dm.lwords * 8));
  if (dbytes) BXG_CUDA(m, nd.ensure(dbytes));
  BXG_CUDA(m, nk.ensure(want * 16));
  BXG_CUDA(m, nf.ensure(want * 4));
  BXG_CUDA(m, cudaMemsetAsync(nm.p, 0, want * m->dm.lwords * 8, m->stream));
  if (dbytes) BXG_CUDA(m, cudaMemsetAsync(nd.p, 0, dbytes, m->stream));
  BXG_CUDA(m, cudaMemsetAsync(nk.p, 0xFF, want * 16, m->stream));
  if (old) {
    BXG_CUDA(m, cudaMemcpyAsync(nm.p, m->lmask.p, old * m->dm.lwords * 8,
                                cudaMemcpyDeviceToDevice, m->stream));
    if (dbytes)
      BXG_CUDA(m, cudaMemcpyAsync(nd.p, m->ldata.p, old * m->dm.lsize * size_t(m->dm.esz),
                                  cudaMemcpyDeviceToDevice, m->stream));
    BXG_CUDA(m, cudaMemcpyAsync(nk.p, m->lkey.p, old * 16, cudaMemcpyDeviceToDevice, m->stream));
    BXG_CUDA(m, cudaMemcpyAsync(nf.p, m->lfree.p, old * 4, cudaMemcpyDeviceToDevice, m->stream));
  }
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  m->lmask.release();
  m->ldata.release();
  m->lkey.release();
  m->lfree.release();
  m->lmask = nm;
  m->ldata = nd;
  m->lkey = nk;
  m->lfree = nf;
  nm.p = nd.p = nk.p = nf.p = nullptr;
  m->dm.lmask = m->lmask.as<unsigned long long>();
  m->dm.ldata = m->ldata.as<uint8_t>();
  m->dm.lkey = m->lkey.as<int4>();
  m->dm.lfree = m->lfree.as<uint32_t>();
  m->dm.lcap = static_cast<uint32_t>(want);
  return BXG_OK;
}

static int grow_hash(MapCore* m, size_t want) {
  const size_t old = size_t(m->dm.hmask) + 1;
  if (want <= old) return BXG_OK;
  if (core_mem_usage(m) + bytes_hash(want) - bytes_hash(old) > m->budget)
    return set_error(m, BXG_ERR_HASH_FULL, "root hash would exceed the HBM budget");
  DevBuf nb;
  BXG_CUDA(m, nb.ensure(want * 16));
  BXG_CUDA(m, cudaMemsetAsync(nb.p, 0xFF, want * 16, m->stream));
  DMap nd = m->dm;
  nd.buckets = nb.as<uint4>();
  nd.hmask = static_cast<uint32_t>(want - 1);
  k_rehash<<<unsigned((old + 255) / 256), 256, 0, m->stream>>>(m->buckets.as<uint4>(),
                                                               uint32_t(old), nd);
  BXG_LAUNCHED(m);
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  m->buckets.release();
  m->buckets = nb;
  nb.p = nullptr;
  m->dm.buckets = m->buckets.as<uint4>();
  m->dm.hmask = nd.hmask;
  return BXG_OK;
}

int core_init(MapCore* m, double res, int ib, int lb, size_t esz, const bxg_config* cfg_in) {
  bxg_config cfg;
  bxg_config_default(&cfg);
  if (cfg_in) cfg = *cfg_in;
  if (!(res > 0) || ib < 1 || ib > 4 || lb < 1 || lb > 5)
    return set_error(m, BXG_ERR_INVALID_ARG,
                     "voxel size must be > 0, inner_bits in [1,4], leaf_bits in [1,5]");
  if (!(esz == 0 || esz == 1 || esz == 2 || esz == 4 || esz == 8))
    return set_error(m, BXG_ERR_INVALID_ARG, "value_bytes must be 0, 1, 2, 4 or 8");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(m, BXG_ERR_NO_DEVICE, "no CUDA device");
  }
  if (cfg.device >= 0) {
    BXG_CUDA(m, cudaSetDevice(cfg.device));
    m->device = cfg.device;
  } else {
    BXG_CUDA(m, cudaGetDevice(&m->device));
  }
  BXG_CUDA(m, cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, m->device));
  if (cfg.stream) {
    m->stream = static_cast<cudaStream_t>(cfg.stream);
    m->own_stream = false;
  } else {
    BXG_CUDA(m, cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    m->own_stream = true;
  }
  m->flags = cfg.flags;
  m->res = res;
  m->inv_res = 1.0 / res;  // bonxai.hpp:395
  m->budget = cfg.pool_budget_bytes ? cfg.pool_budget_bytes : (size_t(16) << 30);
  m->load_factor = cfg.hash_load_factor > 0 ? cfg.hash_load_factor : 0.5f;
  m->rays_per_warp = cfg.rays_per_warp;
  m->block_size = cfg.block_size;
  m->ray_unroll = cfg.ray_unroll;
  DMap& d = m->dm;
  d.ib = ib;
  d.lb = lb;
  d.isize = 1 << (3 * ib);
  d.iwords = std::max(d.isize / 64, 1);
  d.lsize = 1 << (3 * lb);
  d.lwords = std::max(d.lsize / 64, 1);
  d.esz = static_cast<int32_t>(esz);
  d.icap = d.lcap = 0;
  BXG_CUDA(m, m->ctr.ensure(C_WORDS * 4));
  BXG_CUDA(m, cudaMemsetAsync(m->ctr.p, 0, C_WORDS * 4, m->stream));
  d.ctr = m->ctr.as<uint32_t>();
  BXG_CUDA(m, cudaMallocHost(reinterpret_cast<void**>(&m->h_ctr), C_WORDS * 4));
  std::memset(m->h_ctr, 0, C_WORDS * 4);
  uint32_t hb = cfg.hash_buckets ? cfg.hash_buckets : 4096;
  uint32_t hp = 16;
  while (hp < hb) hp <<= 1;
  BXG_CUDA(m, m->buckets.ensure(size_t(hp) * 16));
  BXG_CUDA(m, cudaMemsetAsync(m->buckets.p, 0xFF, size_t(hp) * 16, m->stream));
  d.buckets = m->buckets.as<uint4>();
  d.hmask = hp - 1;
  m->init_inners = cfg.initial_inners ? cfg.initial_inners : 1024;
  m->init_leaves = cfg.initial_leaves ? cfg.initial_leaves : 4096;
  int st = grow_inner(m, m->init_inners);
  if (st) return st;
  st = grow_leaf(m, m->init_leaves);
  if (st) return st;
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  return BXG_OK;
}

int core_release_pools(MapCore* m) {
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  m->leaf_gen++;
  m->ichild.release();
  m->imask.release();
  m->lmask.release();
  m->ldata.release();
  m->lkey.release();
  m->lfree.release();
  m->dm.icap = m->dm.lcap = 0;
  m->dm.ichild = nullptr;
  m->dm.imask = nullptr;
  m->dm.lmask = nullptr;
  m->dm.ldata = nullptr;
  m->dm.lkey = nullptr;
  m->dm.lfree = nullptr;
  m->dm.has_free = 0;
  int st = grow_inner(m, m->init_inners);
  if (st) return st;
  st = grow_leaf(m, m->init_leaves);
  if (st) return st;
  return core_clear(m);
}

int core_clear(MapCore* m) {
  m->leaf_gen++;
  BXG_CUDA(m, cudaMemsetAsync(m->buckets.p, 0xFF, (size_t(m->dm.hmask) + 1) * 16, m->stream));
  BXG_CUDA(m, cudaMemsetAsync(m->ichild.p, 0xFF, size_t(m->dm.icap) * m->dm.isize * 4,
                              m->stream));
  BXG_CUDA(m, cudaMemsetAsync(m->imask.p, 0, size_t(m->dm.icap) * m->dm.iwords * 8, m->stream));
  BXG_CUDA(m, cudaMemsetAsync(m->lmask.p, 0, size_t(m->dm.lcap) * m->dm.lwords * 8, m->stream));
  if (m->dm.esz)
    BXG_CUDA(m, cudaMemsetAsync(m->ldata.p, 0, size_t(m->dm.lcap) * m->dm.lsize * m->dm.esz,
                                m->stream));
  BXG_CUDA(m, cudaMemsetAsync(m->lkey.p, 0xFF, size_t(m->dm.lcap) * 16, m->stream));
  BXG_CUDA(m, cudaMemsetAsync(m->ctr.p, 0, C_WORDS * 4, m->stream));
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  std::memset(m->h_ctr, 0, C_WORDS * 4);
  return BXG_OK;
}

int core_sync(MapCore* m, uint32_t* err_bits_out) {
  BXG_CUDA(m, cudaMemcpyAsync(m->h_ctr, m->ctr.p, C_WORDS * 4, cudaMemcpyDeviceToHost,
                              m->stream));
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  const uint32_t err = m->h_ctr[C_ERR];
  if (err_bits_out) *err_bits_out = err;
  m->dm.has_free = m->h_ctr[C_FREE_LEAF] > 0 ? 1u : 0u;
  bool fix = false;
  if (m->h_ctr[C_INNER] > m->dm.icap) {
    m->h_ctr[C_INNER] = m->dm.icap;
    fix = true;
  }
  if (m->h_ctr[C_LEAF] > m->dm.lcap) {
    m->h_ctr[C_LEAF] = m->dm.lcap;
    fix = true;
  }
  if (err || fix) {
    m->h_ctr[C_ERR] = 0;
    BXG_CUDA(m, cudaMemcpyAsync(m->ctr.p, m->h_ctr, 4 * 4, cudaMemcpyHostToDevice, m->stream));
    BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  }
  if (!err) return BXG_OK;
  // errors that growing the pools cannot cure come first
  if (err & ERR_WAIT)
    return set_error(m, BXG_ERR_WAIT_TIMEOUT, "a bounded device-side wait gave up");
  if (err & ERR_RAY_TOO_LONG)
    return set_error(m, BXG_ERR_INVALID_ARG, "a ray is longer than 2^26 cells");
  if (err & ERR_SCRATCH) return set_error(m, BXG_ERR_INVALID_ARG, "scratch table overflow");
  if (err & (ERR_POOL_INNER | ERR_POOL_LEAF))
    return set_error(m, BXG_ERR_OUT_OF_POOL, "node pool exhausted");
  if (err & ERR_HASH_FULL) return set_error(m, BXG_ERR_HASH_FULL, "root hash full");
  return set_error(m, BXG_ERR_CUDA, "unknown device error");
}

int core_grow_for(MapCore* m, uint32_t err) {
  int st = BXG_OK;
  if (err & ERR_POOL_INNER) {
    // the counter overshoots by the number of failed requests: a fair estimate
    st = grow_inner(m, std::max<size_t>(size_t(m->dm.icap) * 2, size_t(m->dm.icap) + 1024));
    if (st) return st;
  }
  if (err & ERR_POOL_LEAF) {
    st = grow_leaf(m, std::max<size_t>(size_t(m->dm.lcap) * 2, size_t(m->dm.lcap) + 4096));
    if (st) return st;
  }
  if (err & ERR_HASH_FULL) {
    st = grow_hash(m, (size_t(m->dm.hmask) + 1) * 2);
    if (st) return st;
  }
  if (err & (ERR_WAIT | ERR_RAY_TOO_LONG | ERR_SCRATCH)) return BXG_ERR_INVALID_ARG;
  return BXG_OK;
}

int core_maintain(MapCore* m) {
  // Grow ahead of need so that the next call rarely has to retry.
  const uint32_t roots = m->h_ctr[C_ROOTS], inner = m->h_ctr[C_INNER],
                 leaves = m->h_ctr[C_LEAF];
  const size_t hcap = size_t(m->dm.hmask) + 1;
  if (roots > m->load_factor * hcap) {
    size_t want = hcap * 2;
    while (roots > m->load_factor * want) want *= 2;
    grow_hash(m, want);  // best effort: a full table reports on the next call
  }
  if (inner > 0.75 * m->dm.icap) grow_inner(m, size_t(m->dm.icap) * 2);
  if (leaves > 0.75 * m->dm.lcap) grow_leaf(m, size_t(m->dm.lcap) * 2);
  m->err.clear();
  return BXG_OK;
}

// Headroom before a scan, best effort: a request the HBM budget does not
// allow is skipped (the scan then grows on demand or reports the budget
// itself); only CUDA errors are returned.
int core_reserve(MapCore* m, size_t leaves, size_t inners) {
  const std::string saved = m->err;
  auto soft = [&](int st) -> int {
    if (st == BXG_ERR_OUT_OF_POOL || st == BXG_ERR_HASH_FULL) {
      m->err = saved;
      return BXG_OK;
    }
    return st;
  };
  const size_t lused = m->h_ctr[C_LEAF], lfree = m->h_ctr[C_FREE_LEAF];
  const size_t lavail = (m->dm.lcap > lused ? m->dm.lcap - lused : 0) + lfree;
  if (lavail < leaves) {
    const int st =
        soft(grow_leaf(m, std::max<size_t>(size_t(m->dm.lcap) * 2, lused + leaves)));
    if (st) return st;
  }
  const size_t iused = m->h_ctr[C_INNER];
  if ((m->dm.icap > iused ? m->dm.icap - iused : 0) < inners) {
    const int st =
        soft(grow_inner(m, std::max<size_t>(size_t(m->dm.icap) * 2, iused + inners)));
    if (st) return st;
  }
  const size_t hcap = size_t(m->dm.hmask) + 1;
  if (m->h_ctr[C_ROOTS] + inners > m->load_factor * hcap) {
    size_t want = hcap * 2;
    while (m->h_ctr[C_ROOTS] + inners > m->load_factor * want) want *= 2;
    const int st = soft(grow_hash(m, want));
    if (st) return st;
  }
  return BXG_OK;
}

int core_active_cells(MapCore* m, size_t* out) {
  if (!out) return set_error(m, BXG_ERR_INVALID_ARG, "null output");
  int st = core_sync(m);
  if (st) return st;
  const size_t nwords = size_t(m->h_ctr[C_LEAF]) * m->dm.lwords;
  BXG_CUDA(m, m->s_tmp.ensure(8));
  BXG_CUDA(m, cudaMemsetAsync(m->s_tmp.p, 0, 8, m->stream));
  if (nwords) {
    const unsigned blocks = unsigned(std::min<size_t>((nwords + 255) / 256, 4096));
    k_count_on<<<blocks, 256, 0, m->stream>>>(m->dm.lmask, nwords,
                                              m->s_tmp.as<unsigned long long>());
    BXG_LAUNCHED(m);
  }
  unsigned long long n = 0;
  BXG_CUDA(m, cudaMemcpyAsync(&n, m->s_tmp.p, 8, cudaMemcpyDeviceToHost, m->stream));
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  *out = size_t(n);
  return BXG_OK;
}

int core_node_counts(MapCore* m, size_t* roots, size_t* leaves) {
  int st = core_sync(m);
  if (st) return st;
  if (roots) *roots = m->h_ctr[C_ROOTS];
  if (leaves) *leaves = size_t(m->h_ctr[C_LEAF]) - m->h_ctr[C_FREE_LEAF];
  return BXG_OK;
}

int core_dump(MapCore* m, int32_t* out_xyz, void* out_values, size_t cap, size_t* n_out,
              int mode, int32_t thr) {
  int st = core_sync(m);
  if (st) return st;
  const uint32_t n_leaves = m->h_ctr[C_LEAF];
  const int esz = mode == 0 ? m->dm.esz : 0;
  void* dxyz = nullptr;
  void* dval = nullptr;
  if (cap && out_xyz) {
    st = stage_out(m, m->s_out, out_xyz, cap * 12, &dxyz);
    if (st) return st;
  }
  if (cap && out_values && esz) {
    st = stage_out(m, m->s_out2, out_values, cap * size_t(esz), &dval);
    if (st) return st;
  }
  BXG_CUDA(m, m->s_tmp.ensure(8));
  BXG_CUDA(m, cudaMemsetAsync(m->s_tmp.p, 0, 8, m->stream));
  const size_t threads = size_t(n_leaves) * m->dm.lwords;
  const size_t wcap = dxyz ? cap : 0;
  if (threads) {
    const unsigned blocks = unsigned((threads + 255) / 256);
    auto* cnt = m->s_tmp.as<unsigned long long>();
    auto* xyz = static_cast<int32_t*>(dxyz);
    auto* val = static_cast<uint8_t*>(dval);
    switch (esz) {
      case 0: k_dump<0><<<blocks, 256, 0, m->stream>>>(m->dm, n_leaves, xyz, val, wcap, cnt, mode, thr); break;
      case 1: k_dump<1><<<blocks, 256, 0, m->stream>>>(m->dm, n_leaves, xyz, val, wcap, cnt, mode, thr); break;
      case 2: k_dump<2><<<blocks, 256, 0, m->stream>>>(m->dm, n_leaves, xyz, val, wcap, cnt, mode, thr); break;
      case 4: k_dump<4><<<blocks, 256, 0, m->stream>>>(m->dm, n_leaves, xyz, val, wcap, cnt, mode, thr); break;
      default: k_dump<8><<<blocks, 256, 0, m->stream>>>(m->dm, n_leaves, xyz, val, wcap, cnt, mode, thr); break;
    }
    BXG_LAUNCHED(m);
  }
  unsigned long long n = 0;
  BXG_CUDA(m, cudaMemcpyAsync(&n, m->s_tmp.p, 8, cudaMemcpyDeviceToHost, m->stream));
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  const size_t wrote = std::min<size_t>(size_t(n), wcap);
  if (dxyz) {
    st = stage_out_finish(m, out_xyz, dxyz, wrote * 12);
    if (st) return st;
  }
  if (dval) {
    st = stage_out_finish(m, out_values, dval, wrote * size_t(esz));
    if (st) return st;
  }
  if (n_out) *n_out = size_t(n);
  if (size_t(n) > cap) return set_error(m, BXG_ERR_CAPACITY, "output buffer too small");
  return BXG_OK;
}

int stage_in(MapCore* m, DevBuf& buf, const void* src, size_t bytes, const void** dev) {
  if (!src || !bytes) {
    *dev = src;
    return BXG_OK;
  }
  const int pd = ptr_device(src);
  if (pd == m->device || pd == kPtrManaged) {
    *dev = src;
    return BXG_OK;
  }
  BXG_CUDA(m, buf.ensure(bytes));
  if (pd >= 0)  // memory of another GPU: copied, never dereferenced by our kernels
    BXG_CUDA(m, cudaMemcpyPeerAsync(buf.p, m->device, src, pd, bytes, m->stream));
  else
    BXG_CUDA(m, cudaMemcpyAsync(buf.p, src, bytes, cudaMemcpyHostToDevice, m->stream));
  *dev = buf.p;
  return BXG_OK;
}

int stage_out(MapCore* m, DevBuf& buf, void* dst, size_t bytes, void** dev) {
  if (!dst || !bytes) {
    *dev = nullptr;
    return BXG_OK;
  }
  const int pd = ptr_device(dst);
  if (pd == m->device || pd == kPtrManaged) {
    *dev = dst;
    return BXG_OK;
  }
  BXG_CUDA(m, buf.ensure(bytes));
  *dev = buf.p;
  return BXG_OK;
}

int stage_out_finish(MapCore* m, void* dst, const void* dev, size_t bytes) {
  if (!dst || !bytes || dst == dev) return BXG_OK;
  const int pd = ptr_device(dst);
  if (pd >= 0)
    BXG_CUDA(m, cudaMemcpyPeerAsync(dst, pd, dev, m->device, bytes, m->stream));
  else
    BXG_CUDA(m, cudaMemcpyAsync(dst, dev, bytes, cudaMemcpyDeviceToHost, m->stream));
  BXG_CUDA(m, cudaStreamSynchronize(m->stream));
  return BXG_OK;
}

}  // namespace bxg

// ---------------------------------------------------------------------------
// C ABI: common
// ---------------------------------------------------------------------------
extern "C" {

void bxg_config_default(bxg_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->device = -1;
}

const char* bxg_status_string(int s) {
  switch (s) {
    case BXG_OK: return "ok";
    case BXG_ERR_INVALID_ARG: return "invalid argument";
    case BXG_ERR_OUT_OF_POOL: return "node pool exhausted (HBM budget)";
    case BXG_ERR_HASH_FULL: return "root hash full";
    case BXG_ERR_WAIT_TIMEOUT: return "device wait timed out";
    case BXG_ERR_CUDA: return "CUDA error";
    case BXG_ERR_NO_DEVICE: return "no CUDA device";
    case BXG_ERR_CAPACITY: return "output buffer too small";
    default: return "unknown status";
  }
}

int bxg_version(void) { return 100; }

const char* bxg_last_error(const void* handle) {
  if (!handle) return bxg::g_create_error.c_str();
  return bxg::core_of_handle(handle)->err.c_str();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Serialization in the reference's format (serialization.hpp:77-116):
//   "Bonxai::VoxelGrid<type,inner_bits,leaf_bits>(resolution)\n"
//   uint32 root count; per root: int32 x, y, z; inner mask words; per inner
//   bit set (ascending): leaf mask words, then each on cell's value
//   (ascending cell index).
// Roots are written in ascending (x, y, z) order (the reference writes them in
// its unordered_map's order; any order deserializes to the same grid).
// ---------------------------------------------------------------------------
#include <map>
#include <vector>

namespace {

struct HostImage {
  std::vector<uint4> buckets;
  std::vector<uint64_t> imask;
  std::vector<uint32_t> ichild;
  std::vector<uint64_t> lmask;
  std::vector<uint8_t> ldata;
};

int download(bxg::MapCore* m, HostImage& im) {
  using namespace bxg;
  int st = core_sync(m);
  if (st) return st;
  const size_t hcap = size_t(m->dm.hmask) + 1;
  const size_t ni = std::min<size_t>(m->h_ctr[C_INNER], m->dm.icap);
  const size_t nl = std::min<size_t>(m->h_ctr[C_LEAF], m->dm.lcap);
  im.buckets.resize(hcap);
  im.imask.resize(ni * m->dm.iwords);
  im.ichild.resize(ni * m->dm.isize);
  im.lmask.resize(nl * m->dm.lwords);
  im.ldata.resize(nl * m->dm.lsize * size_t(m->dm.esz));
  BXG_CUDA(m, cudaMemcpy(im.buckets.data(), m->buckets.p, hcap * 16, cudaMemcpyDeviceToHost));
  if (ni) {
    BXG_CUDA(m, cudaMemcpy(im.imask.data(), m->imask.p, im.imask.size() * 8, cudaMemcpyDeviceToHost));
    BXG_CUDA(m, cudaMemcpy(im.ichild.data(), m->ichild.p, im.ichild.size() * 4, cudaMemcpyDeviceToHost));
  }
  if (nl) {
    BXG_CUDA(m, cudaMemcpy(im.lmask.data(), m->lmask.p, im.lmask.size() * 8, cudaMemcpyDeviceToHost));
    if (!im.ldata.empty())
      BXG_CUDA(m, cudaMemcpy(im.ldata.data(), m->ldata.p, im.ldata.size(), cudaMemcpyDeviceToHost));
  }
  return BXG_OK;
}

struct Writer {
  uint8_t* out;
  size_t cap, n = 0;
  void put(const void* p, size_t k) {
    if (out && n + k <= cap) std::memcpy(out + n, p, k);
    n += k;
  }
};

}  // namespace

extern "C" int bxg_grid_serialize(bxg_grid g, const char* type_name, void* out, size_t cap,
                                  size_t* n_out) {
  if (!g || !type_name) return BXG_ERR_INVALID_ARG;
  bxg::MapCore* m = const_cast<bxg::MapCore*>(bxg::core_of_handle(g));
  cudaSetDevice(m->device);
  HostImage im;
  int st = download(m, im);
  if (st) return st;
  const bxg::DMap& d = m->dm;
  std::map<std::array<int32_t, 3>, uint32_t> roots;  // sorted root key -> inner slot
  for (const uint4& b : im.buckets) {
    if (static_cast<int>(b.x) == bxg::kEmptyKey || b.w >= bxg::kPending) continue;
    bool any = false;
    for (int w = 0; w < d.iwords; w++) any |= im.imask[size_t(b.w) * d.iwords + w] != 0;
    if (!any) continue;  // a root whose leaves were all released
    roots[{int32_t(b.x), int32_t(b.y), int32_t(b.z)}] = b.w;
  }
  Writer wr{static_cast<uint8_t*>(out), cap};
  char header[256];
  std::snprintf(header, sizeof(header), "Bonxai::VoxelGrid<%s,%d,%d>(%lf)\n", type_name, d.ib,
                d.lb, m->res);
  wr.put(header, std::strlen(header));
  const uint32_t nroots = uint32_t(roots.size());
  wr.put(&nroots, 4);
  for (const auto& kv : roots) {
    wr.put(kv.first.data(), 12);
    const uint32_t in = kv.second;
    const uint64_t* im_w = im.imask.data() + size_t(in) * d.iwords;
    wr.put(im_w, size_t(d.iwords) * 8);
    for (int iw = 0; iw < d.iwords; iw++) {
      for (uint64_t bits = im_w[iw]; bits; bits &= bits - 1) {
        const uint32_t ii = uint32_t(iw * 64 + __builtin_ctzll(bits));
        const uint32_t lf = im.ichild[size_t(in) * d.isize + ii];
        const uint64_t* lm = im.lmask.data() + size_t(lf) * d.lwords;
        wr.put(lm, size_t(d.lwords) * 8);
        if (!d.esz) continue;
        for (int lw = 0; lw < d.lwords; lw++)
          for (uint64_t cb = lm[lw]; cb; cb &= cb - 1) {
            const uint32_t ci = uint32_t(lw * 64 + __builtin_ctzll(cb));
            wr.put(im.ldata.data() + (size_t(lf) * d.lsize + ci) * d.esz, size_t(d.esz));
          }
      }
    }
  }
  if (n_out) *n_out = wr.n;
  if (out && wr.n > cap) return bxg::set_error(m, BXG_ERR_CAPACITY, "output buffer too small");
  return BXG_OK;
}

extern "C" int bxg_grid_deserialize(bxg_grid g, const void* data, size_t n) {
  if (!g || !data) return BXG_ERR_INVALID_ARG;
  bxg::MapCore* m = const_cast<bxg::MapCore*>(bxg::core_of_handle(g));
  const bxg::DMap& d = m->dm;
  const uint8_t* p = static_cast<const uint8_t*>(data);
  const uint8_t* end = p + n;
  // header line (serialization.hpp:126-151): prefix, type, bits, resolution
  const uint8_t* nl = static_cast<const uint8_t*>(std::memchr(p, '\n', n));
  if (!nl) return bxg::set_error(m, BXG_ERR_INVALID_ARG, "Header wasn't recognized");
  const std::string header(reinterpret_cast<const char*>(p), nl - p);
  if (header.rfind("Bonxai::VoxelGrid<", 0) != 0)
    return bxg::set_error(m, BXG_ERR_INVALID_ARG, "Header wasn't recognized");
  const size_t lt = header.rfind('>');
  const size_t c2 = header.rfind(',', lt);
  const size_t c1 = header.rfind(',', c2 - 1);
  if (lt == std::string::npos || c1 == std::string::npos || c2 == std::string::npos)
    return bxg::set_error(m, BXG_ERR_INVALID_ARG, "Header wasn't recognized");
  const int ib = std::atoi(header.substr(c1 + 1, c2 - c1 - 1).c_str());
  const int lb = std::atoi(header.substr(c2 + 1, lt - c2 - 1).c_str());
  if (ib != d.ib || lb != d.lb)
    return bxg::set_error(m, BXG_ERR_INVALID_ARG, "inner/leaf bits do not match this grid");
  p = nl + 1;
  auto take = [&](void* dst, size_t k) -> bool {
    if (size_t(end - p) < k) return false;
    std::memcpy(dst, p, k);
    p += k;
    return true;
  };
  uint32_t nroots = 0;
  if (!take(&nroots, 4)) return bxg::set_error(m, BXG_ERR_INVALID_ARG, "truncated stream");
  std::vector<int32_t> xyz;
  std::vector<uint8_t> vals;
  std::vector<uint64_t> iw(d.iwords), lw(d.lwords);
  const int im = (1 << d.ib) - 1, lm = (1 << d.lb) - 1;
  for (uint32_t r = 0; r < nroots; r++) {
    int32_t key[3];
    if (!take(key, 12) || !take(iw.data(), iw.size() * 8))
      return bxg::set_error(m, BXG_ERR_INVALID_ARG, "truncated stream");
    for (int a = 0; a < d.iwords; a++)
      for (uint64_t bits = iw[a]; bits; bits &= bits - 1) {
        const int ii = a * 64 + __builtin_ctzll(bits);
        const int xb = key[0] | ((ii & im) << d.lb), yb = key[1] | (((ii >> d.ib) & im) << d.lb),
                  zb = key[2] | (((ii >> (2 * d.ib)) & im) << d.lb);
        if (!take(lw.data(), lw.size() * 8))
          return bxg::set_error(m, BXG_ERR_INVALID_ARG, "truncated stream");
        for (int b = 0; b < d.lwords; b++)
          for (uint64_t cb = lw[b]; cb; cb &= cb - 1) {
            const int ci = b * 64 + __builtin_ctzll(cb);
            xyz.push_back(xb | (ci & lm));
            xyz.push_back(yb | ((ci >> d.lb) & lm));
            xyz.push_back(zb | ((ci >> (2 * d.lb)) & lm));
            if (d.esz) {
              const size_t off = vals.size();
              vals.resize(off + d.esz);
              if (!take(vals.data() + off, d.esz))
                return bxg::set_error(m, BXG_ERR_INVALID_ARG, "truncated stream");
            }
          }
      }
  }
  const size_t cells = xyz.size() / 3;
  if (!cells) return BXG_OK;
  if (d.esz) return bxg_grid_set_values(g, xyz.data(), vals.data(), cells, nullptr);
  return bxg_grid_set_cells_on(g, xyz.data(), cells, nullptr, nullptr);
}
