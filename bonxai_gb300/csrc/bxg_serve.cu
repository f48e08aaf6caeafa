// Serving loop: many clients, each with a persistent map on the device,
// sending insertPointCloud, isOccupied and getOccupiedVoxels requests
// (probabilistic_map.hpp:91-124) that are batched continuously.
//
// Requests are queued per map in arrival order. A worker thread forms ticks
// from whatever is queued when the previous tick finishes (continuous
// batching: requests that arrive while a tick runs join the next one). For
// each map a tick takes, in order,
//   the lookups at the head of its queue            ("before" lookups),
//   at most one insert (if a slot and the HBM budget allow),
//   the lookups queued behind that insert            ("after" lookups),
// so every request sees exactly the map state it would see alone. All maps'
// "before" lookups run as one kernel, all inserts as one batched tick
// (bxg_batch.cu), all "after" lookups as one kernel: the work of different
// clients overlaps on the device. A clear request (clear(CLEAR_MEMORY),
// bonxai.hpp:678-684, which can also give the map's pool memory back) takes an
// insert's place in its map's tick and runs before the inserts.
// Admission: insert slots per tick, points per tick, and an HBM budget across
// all maps' node pools. An insert that does not fit the budget stays at the
// head of its map's queue (with the requests behind it) until memory frees up
// -- another map's clear -- and is admitted then; only when it has waited
// past the server's admission timeout does it complete with
// BXG_ERR_OUT_OF_POOL.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bxg_internal.h"

namespace bxg {

struct QueryDesc {
  DMap M;
  int32_t thr;
  int32_t mode;  // 0 occupied, 1 unknown, 2 free
  unsigned long long begin;
  uint32_t n;
  uint32_t pad;
};

__device__ __forceinline__ uint32_t query_of(const QueryDesc* d, uint32_t n, unsigned long long i) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (d[mid].begin <= i) lo = mid; else hi = mid;
  }
  return lo;
}

// isOccupied / isUnknown / isFree (probabilistic_map.cpp:56-75) for the
// lookup requests of many maps in one launch.
__global__ void k_query_multi(const QueryDesc* __restrict__ d, uint32_t nd,
                              const int32_t* __restrict__ xyz, unsigned long long total,
                              uint8_t* __restrict__ out) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < total;
       i += gridDim.x * (unsigned long long)blockDim.x) {
    const QueryDesc& q = d[query_of(d, nd, i)];
    const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    const uint32_t lf = leaf_of(q.M, x, y, z, false);
    bool have = false;
    int32_t p = 0;
    if (lf != kNone) {  // cell word first; the mask only for a zero word (as k_query)
      const uint32_t ci = leaf_index(q.M, x, y, z);
      const int32_t w = reinterpret_cast<const int32_t*>(q.M.ldata)[size_t(lf) * q.M.lsize + ci];
      have = w != 0 || cell_is_on(q.M, lf, ci);
      p = cell_prob(w);
    }
    out[i] = q.mode == 0 ? (have && p > q.thr) : q.mode == 1 ? (have ? p == q.thr : 1)
                                                                : (have && p < q.thr);
  }
}

}  // namespace bxg

using namespace bxg;
using Clock = std::chrono::steady_clock;

namespace {
enum Kind : int { K_INSERT = 0, K_QUERY = 1, K_OCCUPIED = 2, K_CLEAR = 3 };

struct Request {
  uint64_t ticket = 0;
  Kind kind = K_INSERT;
  uint32_t map = 0;
  bool discard = false;
  std::vector<float> pts;
  float origin[3] = {0, 0, 0};
  double max_range = 0;
  std::vector<int32_t> coords;
  int mode = 0;
  // results
  bool done = false;
  int status = BXG_OK;
  uint64_t ray_cells = 0;
  std::vector<uint8_t> answers;
  std::vector<int32_t> occupied;
  Clock::time_point t_submit, t_start, t_done;
  Clock::time_point deadline;  // inserts: admission gives up after this
  uint64_t tick = 0;
};
}  // namespace

struct bxg_server_s {
  int device = 0;
  std::vector<bxg_pmap> maps;
  bxg_batch batch = nullptr;
  cudaStream_t stream = nullptr;
  size_t budget = 0;
  uint32_t max_scans = 128;
  uint64_t max_points = 64ull << 20;
  uint64_t max_lookups = 64ull << 20;
  double admission_timeout_s = 10.0;
  // queues
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::vector<std::deque<Request*>> fifo;
  std::unordered_map<uint64_t, Request*> live;
  uint64_t next_ticket = 1;
  size_t queued = 0, in_flight = 0;
  bool stop = false;
  bool kick = false;  // a submission arrived (wakes a worker waiting on deferred inserts)
  std::thread worker;
  // staging
  DevBuf d_pts, d_xyz, d_ans, d_desc;
  std::vector<float> h_pts;
  std::vector<int32_t> h_xyz;
  std::vector<uint8_t> h_ans;
  // statistics
  std::vector<double> lat_all, lat_ins, lat_q, lat_occ;
  uint64_t completed = 0, n_ins = 0, n_q = 0, n_occ = 0, ticks = 0, rejected = 0;
  uint64_t deferred = 0;  // insert admissions postponed for lack of budget
  uint64_t ray_cells = 0, lookups = 0;
  double busy_s = 0;
  size_t pool_bytes = 0;  // all maps' pools, refreshed by the worker after each tick
  Clock::time_point t_first{}, t_last{};
  bool have_first = false;
  std::string err;

  ~bxg_server_s() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    for (auto& kv : live) delete kv.second;  // every unreleased request is in `live`
    if (batch) bxg_batch_destroy(batch);
    for (bxg_pmap m : maps) bxg_pmap_destroy(m);
    cudaSetDevice(device);
    d_pts.release();
    d_xyz.release();
    d_ans.release();
    d_desc.release();
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

// Runs one group of lookup requests (all maps) in one launch.
int run_lookups(bxg_server_s* s, std::vector<Request*>& qs) {
  std::vector<Request*> look;
  for (Request* r : qs) {
    if (r->kind == K_QUERY) {
      look.push_back(r);
    } else {  // getOccupiedVoxels: one compaction per map
      bxg_pmap m = s->maps[r->map];
      size_t n = 0;
      int st = bxg_pmap_get_occupied(m, nullptr, 0, &n);
      if (st == BXG_OK || st == BXG_ERR_CAPACITY) {
        r->occupied.resize(3 * n);
        size_t got = 0;
        st = n ? bxg_pmap_get_occupied(m, r->occupied.data(), n, &got) : BXG_OK;
        r->occupied.resize(3 * got);
      }
      r->status = st;
    }
  }
  if (look.empty()) return BXG_OK;
  unsigned long long total = 0;
  std::vector<QueryDesc> desc(look.size());
  for (size_t k = 0; k < look.size(); k++) {
    bxg_pmap m = s->maps[look[k]->map];
    std::memset(&desc[k], 0, sizeof(QueryDesc));
    desc[k].M = m->core.dm;
    desc[k].thr = m->opt.occupancy_threshold_log;
    desc[k].mode = look[k]->mode;
    desc[k].begin = total;
    desc[k].n = uint32_t(look[k]->coords.size() / 3);
    total += desc[k].n;
  }
  if (!total) return BXG_OK;
  s->h_xyz.resize(3 * total);
  for (size_t k = 0; k < look.size(); k++)
    std::memcpy(s->h_xyz.data() + 3 * desc[k].begin, look[k]->coords.data(),
                look[k]->coords.size() * 4);
  if (s->d_xyz.ensure(total * 12) != cudaSuccess || s->d_ans.ensure(total) != cudaSuccess ||
      s->d_desc.ensure(desc.size() * sizeof(QueryDesc)) != cudaSuccess) {
    cudaGetLastError();
    return BXG_ERR_CUDA;
  }
  cudaMemcpyAsync(s->d_xyz.p, s->h_xyz.data(), total * 12, cudaMemcpyHostToDevice, s->stream);
  cudaMemcpyAsync(s->d_desc.p, desc.data(), desc.size() * sizeof(QueryDesc),
                  cudaMemcpyHostToDevice, s->stream);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
  const unsigned blocks = unsigned(std::min<unsigned long long>((total + 255) / 256, sms * 16ull));
  k_query_multi<<<blocks, 256, 0, s->stream>>>(s->d_desc.as<QueryDesc>(), uint32_t(desc.size()),
                                               s->d_xyz.as<int32_t>(), total,
                                               s->d_ans.as<uint8_t>());
  s->h_ans.resize(total);
  cudaMemcpyAsync(s->h_ans.data(), s->d_ans.p, total, cudaMemcpyDeviceToHost, s->stream);
  const cudaError_t e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return BXG_ERR_CUDA;
  }
  for (size_t k = 0; k < look.size(); k++) {
    look[k]->answers.assign(s->h_ans.begin() + desc[k].begin,
                            s->h_ans.begin() + desc[k].begin + desc[k].n);
    look[k]->status = BXG_OK;
  }
  s->lookups += total;
  return BXG_OK;
}

size_t pools_bytes(bxg_server_s* s) {
  size_t b = 0;
  for (bxg_pmap m : s->maps) b += core_mem_usage(&m->core);
  return b;
}

// Bytes an insert of n points may add to its map's pools (the leaf headroom
// the batched tick reserves).
size_t insert_need(size_t n) { return (n / 4 + 1024) * (64 + 2048 + 20); }

void worker_loop(bxg_server_s* s) {
  cudaSetDevice(s->device);
  uint32_t rr = 0;         // round-robin start for fairness
  bool idle_wait = false;  // the last tick could only defer inserts
  Clock::time_point wake{};
  // a map's part of a tick: lookups (in `before`), then one insert or clear,
  // then the lookups behind it
  struct MapTick {
    uint32_t map = 0;
    Request* mid = nullptr;
    std::vector<Request*> after;
  };
  for (;;) {
    std::vector<Request*> before;
    std::vector<MapTick> mids;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (idle_wait)
        s->cv_work.wait_until(lk, wake, [&] { return s->stop || s->kick; });
      else
        s->cv_work.wait(lk, [&] { return s->stop || s->queued > 0; });
      s->kick = false;
      if (s->stop && s->queued == 0) return;
      uint64_t pts = 0, looks = 0;
      uint32_t n_ins = 0;
      const uint32_t nm = uint32_t(s->maps.size());
      auto is_mid = [](const Request* r) { return r->kind == K_INSERT || r->kind == K_CLEAR; };
      for (uint32_t j = 0; j < nm; j++) {
        const uint32_t m = (rr + j) % nm;
        auto& q = s->fifo[m];
        while (!q.empty() && !is_mid(q.front()) && looks < s->max_lookups) {
          looks += q.front()->coords.size() / 3;
          before.push_back(q.front());
          q.pop_front();
        }
        if (q.empty() || !is_mid(q.front())) continue;
        Request* r = q.front();
        if (r->kind == K_INSERT) {
          if (n_ins >= s->max_scans || (n_ins && pts + r->pts.size() / 3 > s->max_points))
            continue;
          pts += r->pts.size() / 3;
          n_ins++;
        }
        q.pop_front();
        MapTick mt;
        mt.map = m;
        mt.mid = r;
        while (!q.empty() && !is_mid(q.front()) && looks < s->max_lookups) {
          looks += q.front()->coords.size() / 3;
          mt.after.push_back(q.front());
          q.pop_front();
        }
        mids.push_back(std::move(mt));
      }
      rr = (rr + 1) % std::max<uint32_t>(nm, 1);
      size_t taken = before.size();
      for (auto& mt : mids) taken += 1 + mt.after.size();
      s->queued -= taken;
      s->in_flight += taken;
    }
    const Clock::time_point t0 = Clock::now();
    for (Request* r : before) r->t_start = t0;

    int st = run_lookups(s, before);
    if (st)
      for (Request* r : before) r->status = st;

    // clears first: they can free pool memory for this tick's inserts
    for (auto& mt : mids) {
      if (mt.mid->kind != K_CLEAR) continue;
      bxg_pmap m = s->maps[mt.map];
      m->cast_ub = 0;
      mt.mid->status = mt.mid->mode ? core_release_pools(&m->core) : core_clear(&m->core);
      mt.mid->t_start = t0;
    }
    // admission against the HBM budget; an insert that does not fit waits
    // (it and the requests behind it go back to the head of its queue) until
    // its deadline
    std::vector<MapTick*> admit;
    std::vector<MapTick> deferred;
    size_t used = pools_bytes(s);
    for (auto& mt : mids) {
      Request* r = mt.mid;
      if (r->kind != K_INSERT) continue;
      const size_t need = insert_need(r->pts.size() / 3);
      if (used + need <= s->budget) {
        used += need;
        r->t_start = t0;
        admit.push_back(&mt);
      } else if (t0 >= r->deadline) {
        r->status = BXG_ERR_OUT_OF_POOL;
        r->t_start = t0;
        s->rejected++;
      } else {
        MapTick d;
        d.map = mt.map;
        d.mid = r;
        d.after.swap(mt.after);
        deferred.push_back(std::move(d));
        mt.mid = nullptr;
      }
    }
    if (!admit.empty()) {
      std::vector<bxg_pmap> ms;
      std::vector<uint64_t> off(1, 0);
      std::vector<float> org;
      std::vector<double> mr;
      for (MapTick* mt : admit) {
        Request* r = mt->mid;
        ms.push_back(s->maps[r->map]);
        off.push_back(off.back() + r->pts.size() / 3);
        org.insert(org.end(), r->origin, r->origin + 3);
        mr.push_back(r->max_range);
      }
      s->h_pts.resize(3 * off.back());
      for (size_t k = 0; k < admit.size(); k++)
        std::memcpy(s->h_pts.data() + 3 * off[k], admit[k]->mid->pts.data(),
                    admit[k]->mid->pts.size() * 4);
      std::vector<uint64_t> rc(admit.size(), 0);
      st = bxg_batch_insert_f32(s->batch, ms.data(), ms.size(), s->h_pts.data(), off.data(),
                                org.data(), mr.data(), rc.data());
      for (size_t k = 0; k < admit.size(); k++) {
        admit[k]->mid->status = st;
        admit[k]->mid->ray_cells = rc[k];
        s->ray_cells += rc[k];
      }
      if (st) s->err = bxg_batch_last_error(s->batch);
    }

    std::vector<Request*> after;
    for (auto& mt : mids)
      if (mt.mid)
        for (Request* r : mt.after) {
          r->t_start = t0;
          after.push_back(r);
        }
    st = run_lookups(s, after);
    if (st)
      for (Request* r : after) r->status = st;

    const Clock::time_point t1 = Clock::now();
    const size_t pb = pools_bytes(s);
    size_t done_n = before.size() + after.size();
    for (auto& mt : mids)
      if (mt.mid) done_n++;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->pool_bytes = pb;
      s->busy_s += std::chrono::duration<double>(t1 - t0).count();
      if (done_n) s->ticks++;
      auto finish = [&](Request* r) {
        r->t_done = t1;
        r->done = true;
        r->tick = s->ticks;
        const double lat = ms_between(r->t_submit, r->t_done);
        s->lat_all.push_back(lat);
        if (r->kind == K_INSERT) {
          s->lat_ins.push_back(lat);
          s->n_ins++;
        } else if (r->kind == K_QUERY) {
          s->lat_q.push_back(lat);
          s->n_q++;
        } else if (r->kind == K_OCCUPIED) {
          s->lat_occ.push_back(lat);
          s->n_occ++;
        }
        s->completed++;
        s->t_last = t1;
        if (r->discard) {
          s->live.erase(r->ticket);
          delete r;
        } else {
          r->pts.clear();
          r->pts.shrink_to_fit();
          r->coords.clear();
          r->coords.shrink_to_fit();
        }
      };
      for (Request* r : before) finish(r);
      for (auto& mt : mids)
        if (mt.mid) finish(mt.mid);
      for (Request* r : after) finish(r);
      // deferred inserts and the lookups behind them go back, in order
      Clock::time_point first_deadline = Clock::time_point::max();
      for (auto& d : deferred) {
        auto& q = s->fifo[d.map];
        for (auto it = d.after.rbegin(); it != d.after.rend(); ++it) q.push_front(*it);
        q.push_front(d.mid);
        first_deadline = std::min(first_deadline, d.mid->deadline);
        s->queued += 1 + d.after.size();
        s->in_flight -= 1 + d.after.size();
        s->deferred++;
      }
      s->in_flight -= done_n;
      // only deferred inserts are left: sleep until a submission or the next
      // check (every 50 ms at most, so that a deadline is noticed)
      idle_wait = done_n == 0 && !deferred.empty();
      if (idle_wait) wake = std::min(first_deadline, t1 + std::chrono::milliseconds(50));
    }
    s->cv_done.notify_all();
  }
}

double pct(std::vector<double> v, double p) {
  if (v.empty()) return 0;
  std::sort(v.begin(), v.end());
  const size_t k = std::min(v.size() - 1, size_t(p * (v.size() - 1) + 0.5));
  return v[k];
}

int submit(bxg_server_s* s, Request* r, uint64_t* ticket) {
  if (r->map >= s->maps.size()) {
    delete r;
    s->err = "map index out of range";
    return BXG_ERR_INVALID_ARG;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
      delete r;
      return BXG_ERR_INVALID_ARG;
    }
    r->ticket = s->next_ticket++;
    r->t_submit = Clock::now();
    if (!s->have_first) {
      s->t_first = r->t_submit;
      s->have_first = true;
    }
    if (r->kind == K_INSERT)
      r->deadline = r->t_submit + std::chrono::duration_cast<Clock::duration>(
                                      std::chrono::duration<double>(s->admission_timeout_s));
    s->live[r->ticket] = r;
    s->fifo[r->map].push_back(r);
    s->queued++;
    s->kick = true;
    if (ticket) *ticket = r->ticket;
  }
  s->cv_work.notify_one();
  return BXG_OK;
}

}  // namespace

extern "C" {

void bxg_server_config_default(bxg_server_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->device = -1;
}

int bxg_server_create(bxg_server* out, const double* resolutions, size_t n_maps,
                      const bxg_server_config* cfg_in) {
  if (!out || !resolutions || !n_maps) return BXG_ERR_INVALID_ARG;
  *out = nullptr;
  bxg_server_config cfg;
  bxg_server_config_default(&cfg);
  if (cfg_in) cfg = *cfg_in;
  bxg_server s = new bxg_server_s();
  if (cfg.device >= 0) cudaSetDevice(cfg.device);
  cudaGetDevice(&s->device);
  s->budget = cfg.pool_budget_bytes ? cfg.pool_budget_bytes : (size_t(40) << 30);
  s->max_scans = cfg.max_scans_per_tick ? std::min<uint32_t>(cfg.max_scans_per_tick, 128) : 128;
  if (cfg.max_points_per_tick) s->max_points = cfg.max_points_per_tick;
  if (cfg.max_lookups_per_tick) s->max_lookups = cfg.max_lookups_per_tick;
  if (cfg.admission_timeout_s > 0) s->admission_timeout_s = cfg.admission_timeout_s;
  bxg_config mc;
  bxg_config_default(&mc);
  mc.device = s->device;
  mc.pool_budget_bytes = s->budget;
  mc.flags = cfg.flags;
  mc.initial_leaves = cfg.initial_leaves;
  for (size_t i = 0; i < n_maps; i++) {
    bxg_pmap m = nullptr;
    const int st = bxg_pmap_create(&m, resolutions[i], &mc);
    if (st) {
      delete s;
      return st;
    }
    s->maps.push_back(m);
  }
  bxg_config bc;
  bxg_config_default(&bc);
  bc.device = s->device;
  bc.rays_per_warp = cfg.rays_per_warp;
  bc.ray_unroll = cfg.ray_unroll;
  bc.flags = cfg.flags;
  int st = bxg_batch_create(&s->batch, &bc);
  if (!st && cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    st = BXG_ERR_CUDA;
  }
  if (st) {
    delete s;
    return st;
  }
  s->fifo.resize(n_maps);
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return BXG_OK;
}

int bxg_server_destroy(bxg_server s) {
  delete s;
  return BXG_OK;
}

const char* bxg_server_last_error(bxg_server s) { return s ? s->err.c_str() : "null handle"; }

int bxg_server_insert(bxg_server s, uint32_t map, const float* xyz, size_t n,
                      const float origin[3], double max_range, int discard, uint64_t* ticket) {
  if (!s || (n && !xyz) || !origin) return BXG_ERR_INVALID_ARG;
  Request* r = new Request();
  r->kind = K_INSERT;
  r->map = map;
  r->discard = discard != 0;
  r->pts.assign(xyz, xyz + 3 * n);
  std::memcpy(r->origin, origin, 12);
  r->max_range = max_range;
  return submit(s, r, ticket);
}

int bxg_server_query(bxg_server s, uint32_t map, const int32_t* xyz, size_t n, int mode,
                     int discard, uint64_t* ticket) {
  if (!s || (n && !xyz) || mode < 0 || mode > 2) return BXG_ERR_INVALID_ARG;
  Request* r = new Request();
  r->kind = K_QUERY;
  r->map = map;
  r->mode = mode;
  r->discard = discard != 0;
  r->coords.assign(xyz, xyz + 3 * n);
  return submit(s, r, ticket);
}

int bxg_server_clear(bxg_server s, uint32_t map, int release_memory, int discard,
                     uint64_t* ticket) {
  if (!s) return BXG_ERR_INVALID_ARG;
  Request* r = new Request();
  r->kind = K_CLEAR;
  r->map = map;
  r->mode = release_memory ? 1 : 0;
  r->discard = discard != 0;
  return submit(s, r, ticket);
}

int bxg_server_get_occupied(bxg_server s, uint32_t map, int discard, uint64_t* ticket) {
  if (!s) return BXG_ERR_INVALID_ARG;
  Request* r = new Request();
  r->kind = K_OCCUPIED;
  r->map = map;
  r->discard = discard != 0;
  return submit(s, r, ticket);
}

int bxg_server_wait(bxg_server s, uint64_t ticket, double timeout_s, bxg_server_result* res,
                    void* out, size_t cap) {
  if (!s) return BXG_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->live.find(ticket);
  if (it == s->live.end()) {
    s->err = "unknown ticket (or its result was discarded)";
    return BXG_ERR_INVALID_ARG;
  }
  Request* r = it->second;
  const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                      [&] { return r->done; });
  if (!ok) return BXG_ERR_WAIT_TIMEOUT;
  const size_t n_out = r->kind == K_QUERY ? r->answers.size() : r->occupied.size() / 3;
  if (res) {
    res->status = r->status;
    res->kind = r->kind;
    res->map = r->map;
    res->ray_cells = r->ray_cells;
    res->n_out = n_out;
    res->latency_ms = ms_between(r->t_submit, r->t_done);
    res->queue_ms = ms_between(r->t_submit, r->t_start);
    res->tick = r->tick;
  }
  if (out && cap) {
    if (r->kind == K_QUERY)
      std::memcpy(out, r->answers.data(), std::min(cap, n_out));
    else if (r->kind == K_OCCUPIED)
      std::memcpy(out, r->occupied.data(), std::min(cap, n_out) * 12);
  }
  // A call without an output buffer only reports the result size and keeps
  // the ticket, so that the caller can size a buffer and call again.
  if (out || r->kind == K_INSERT || r->kind == K_CLEAR) {
    s->live.erase(it);
    delete r;
  }
  return BXG_OK;
}

int bxg_server_drain(bxg_server s, double timeout_s) {
  if (!s) return BXG_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                      [&] { return s->queued == 0 && s->in_flight == 0; });
  return ok ? BXG_OK : BXG_ERR_WAIT_TIMEOUT;
}

int bxg_server_stats(bxg_server s, double out[20]) {
  if (!s || !out) return BXG_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  out[0] = double(s->completed);
  out[1] = double(s->n_ins);
  out[2] = double(s->n_q);
  out[3] = double(s->n_occ);
  out[4] = double(s->ticks);
  out[5] = pct(s->lat_all, 0.5);
  out[6] = pct(s->lat_all, 0.99);
  out[7] = pct(s->lat_ins, 0.5);
  out[8] = pct(s->lat_ins, 0.99);
  out[9] = pct(s->lat_q, 0.5);
  out[10] = pct(s->lat_q, 0.99);
  out[11] = double(s->ray_cells);
  out[12] = double(s->lookups);
  out[13] = double(s->rejected);
  out[14] = s->busy_s;
  out[15] = s->have_first ? std::chrono::duration<double>(s->t_last - s->t_first).count() : 0;
  out[16] = pct(s->lat_occ, 0.5);
  out[17] = pct(s->lat_occ, 0.99);
  out[18] = double(s->pool_bytes);
  out[19] = double(s->deferred);
  return BXG_OK;
}

bxg_pmap bxg_server_map(bxg_server s, uint32_t map) {
  if (!s || map >= s->maps.size()) return nullptr;
  return s->maps[map];
}

}  // extern "C"
