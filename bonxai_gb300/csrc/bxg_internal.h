// Host-side state shared by the grid and probabilistic-map entry points.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <string>

#include "bonxai_gb300.h"
#include "bxg_device.cuh"

namespace bxg {

// A growable device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    size_t want = cap ? cap : 4096;
    while (want < bytes) want *= 2;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  // Like ensure, but keeps the first `keep` bytes of the old content.
  cudaError_t ensure_keep(size_t bytes, size_t keep, cudaStream_t s) {
    if (bytes <= cap) return cudaSuccess;
    size_t want = cap ? cap : 4096;
    while (want < bytes) want *= 2;
    void* np = nullptr;
    cudaError_t e = cudaMalloc(&np, want);
    if (e != cudaSuccess) return e;
    if (p && keep) {
      e = cudaMemcpyAsync(np, p, keep < cap ? keep : cap, cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) {
        cudaFree(np);
        return e;
      }
    }
    if (p) cudaFree(p);
    p = np;
    cap = want;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  DevBuf() = default;
  DevBuf(const DevBuf&) = default;
  DevBuf& operator=(const DevBuf&) = default;
  ~DevBuf() { release(); }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// One map: pools, counters, stream, scratch and error text.
struct MapCore {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  uint32_t flags = 0;
  double res = 0, inv_res = 0;
  DMap dm{};
  size_t budget = 0;
  size_t init_inners = 0, init_leaves = 0;  // pool sizes at creation
  float load_factor = 0.5f;
  uint32_t rays_per_warp = 0, block_size = 0, ray_unroll = 0;
  // bumped whenever leaf slots may be released (clear, releaseUnusedMemory):
  // caches of coordinate -> slot built before are stale after it
  uint64_t leaf_gen = 0;
  // ray kernel launch shape: block size and one resident wave of blocks
  int ray_wave_bs[2] = {0, 0};
  uint32_t ray_wave_blocks[2] = {0, 0};

  // pools
  DevBuf buckets, ichild, imask, lmask, ldata, lkey, lfree, ctr;
  uint32_t* h_ctr = nullptr;  // pinned mirror of ctr

  // scratch
  DevBuf s_in, s_in2, s_out, s_out2, s_dedup, s_dedup2, s_ep, s_cast, s_tmp;
  // entries of s_dedup known to be empty, from index 0 (the ray kernel clears
  // the table the last endpoint phase used, so the next one needs no memset)
  uint32_t dedup_clean = 0;
  uint32_t dedup_used = 0;  // entries the last endpoint phase used
  DevBuf s_dir;             // leaf directory of the ray kernel (bxg_scan.cuh)

  std::string err;
  uint64_t launches = 0;
  int sm_count = 0;

  ~MapCore();
};

// Pointer kind: the ordinal of the GPU whose memory p is in, kPtrManaged for
// managed memory (usable in place on any device), kPtrHost otherwise.
constexpr int kPtrHost = -1;
constexpr int kPtrManaged = -2;
int ptr_device(const void* p);
bool is_device_ptr(const void* p);

int set_error(MapCore* m, int status, const std::string& msg);
int cuda_fail(MapCore* m, cudaError_t e, const char* what);

// Lifecycle and pools (bxg_core.cu).
int core_init(MapCore* m, double res, int ib, int lb, size_t esz, const bxg_config* cfg);
int core_clear(MapCore* m);
// clear(CLEAR_MEMORY) that also gives the node pools' memory back: the pools
// shrink to their sizes at creation (bonxai.hpp:678-684).
int core_release_pools(MapCore* m);
// Reads the counters back (synchronising the stream) and converts device error
// bits into a status; clears them and repairs overshooting allocation counters.
int core_sync(MapCore* m, uint32_t* err_bits_out = nullptr);
// Grows pools ahead of need (after a sync).
int core_maintain(MapCore* m);
// Grows what the error bits say ran out; returns BXG_OK if a retry may succeed.
int core_grow_for(MapCore* m, uint32_t err_bits);
size_t core_mem_usage(const MapCore* m);
int core_dump(MapCore* m, int32_t* out_xyz, void* out_values, size_t cap, size_t* n_out,
              int filter, int32_t thr);
int core_active_cells(MapCore* m, size_t* out);
int core_node_counts(MapCore* m, size_t* roots, size_t* leaves);

// Staging of caller arrays that may live on the host.
// Returns a device pointer holding `bytes` of `src` (copied if host memory).
int stage_in(MapCore* m, DevBuf& buf, const void* src, size_t bytes, const void** dev);
// Returns a device pointer to write `bytes` into; after the kernels call
// stage_out_finish to copy it to `dst` when dst is host memory.
int stage_out(MapCore* m, DevBuf& buf, void* dst, size_t bytes, void** dev);
int stage_out_finish(MapCore* m, void* dst, const void* dev, size_t bytes);

inline unsigned long long* stats_of(const MapCore* m) {
  return reinterpret_cast<unsigned long long*>(m->ctr.as<uint32_t>() + C_STATS);
}

#define BXG_CUDA(m, call)                                  \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail((m), e_, #call); \
  } while (0)

#define BXG_LAUNCHED(m)                                        \
  do {                                                         \
    (m)->launches++;                                           \
    cudaError_t e_ = cudaGetLastError();                       \
    if (e_ != cudaSuccess) return cuda_fail((m), e_, "launch"); \
  } while (0)

// Shared kernels (bxg_core.cu).
void launch_dedup_clear(MapCore* m, uint4* tab, uint32_t cap);
// Inserts the non-empty buckets of old_b[0..old_cap) into the table of M.
void launch_rehash(MapCore* m, const uint4* old_b, uint32_t old_cap, const DMap& M);
// Text of the last failed create call on this host thread.
void set_create_error(const std::string& msg);
const MapCore* core_of_handle(const void* handle);

}  // namespace bxg

// A ProbabilisticMap handle: a map core plus the scan state of
// probabilistic_map.hpp:127-134.
struct bxg_pmap_s {
  bxg::MapCore core;
  bxg_pmap_options opt{};
  int update_count = 1;      // _update_count (probabilistic_map.hpp:129)
  uint64_t cast_ub = 0;      // upper bound of queued rays on the device
  uint64_t last_stats[8] = {0};
  float last_times[4] = {0};
  float last_query_ms = 0;       // device time of the last lookup kernel (BXG_FLAG_TIMING)
  uint32_t last_new_leaves = 0;  // leaves created by the last scan (pool headroom)
  double dir_reach = 0;          // cells of the coming ray phase lie within this range
  // the leaf directory kept across scans: its cube (leaf coordinates of the
  // corner, side), epoch (1..15) and the leaf generation it was built at
  int dir_x0 = 0, dir_y0 = 0, dir_z0 = 0;
  uint32_t dir_side = 0;
  uint32_t dir_epoch = 0;
  uint64_t dir_gen = 0;
  bool dir_live = false;
  // the ray phase's cube bitmap, list bits and list (bxg_mark.cuh): all zero
  // between scans; sized for cube_blocks leaf blocks
  bxg::DevBuf cube_bits, cube_touch, cube_list;
  size_t cube_blocks = 0;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  ~bxg_pmap_s() {
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
  }
};

namespace bxg {
struct LeafDir;
struct RayCube;
// The cube bitmap of a scan's ray phase from origin cell (ox, oy, oz) whose
// rays end within `reach` (world units) of the origin: *ok = false when the
// scan cannot use one (leaf_bits other than 3, non-finite points kept, a cube
// above the size limit); buffers grow here (cudaMalloc, zeroed).
int cube_for_scan(bxg_pmap_s* pm, int ox, int oy, int oz, double reach, RayCube* Q, bool* ok);
// Sets up the ray walk's leaf directory of a scan (bxg_pmap.cu).
// Memsets (first use, epoch wrap) go to `stream` (nullptr: the map's own).
int leaf_dir_for_scan(bxg_pmap_s* pm, int ox, int oy, int oz, LeafDir* D, size_t max_words,
                      cudaStream_t stream);
// Completes a scan whose endpoints were listed (and possibly applied) by a
// batched tick but whose map ran out of pool: grows the pools and re-runs the
// idempotent endpoint completion and ray phases on the map's own stream.
int pmap_complete_scan(bxg_pmap_s* pm, const int4* d_cast, const uint32_t* d_count,
                       uint32_t cap, int ox, int oy, int oz, int32_t u);
// Grows the map's pools so that the next scan has at least `leaves` free leaf
// slots and the root hash stays under its load factor.
int core_reserve(MapCore* m, size_t leaves, size_t inners);
}  // namespace bxg
