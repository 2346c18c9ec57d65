// Mesh request server with continuous batching.
//
// Requests of any size arrive with gcm_server_submit and wait in a bounded
// FIFO.  `lanes` worker threads each own a context and a stream; a free lane
// takes the next request as soon as device memory for it can be reserved
// from the server's pool, so requests that arrive while others run are
// admitted as lanes and memory free up and their kernels overlap on the GPU.
// Memory is admitted exactly (two passes): one pool range holds the
// request's field, device counts, extraction scratch and blend buffer (lent to
// the lane's context, so lanes never allocate or free device memory while
// others run); the field is evaluated, a counting pass gives the vertex total
// (the one readback before the mesh), then the mesh buffers are reserved and
// the mesh pass, its counts and the copies to pinned host memory are enqueued
// together and synchronised once.  Lattices take the fused extraction, CSG
// scenes (sparse surfaces) the windowed one.  With a host pool the mesh's
// device memory is returned at once, so the result's latency is arrival ->
// mesh on the host.
//
// Faults are injected on the host only (tests): failing pool reservations,
// a slow lane, a lane that dies after taking a request (the request goes back
// to the front of the queue and the other lanes serve it).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/gcm.h"
#include "gcm_ctx.h"
#include "pool.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  uint64_t ticket = 0;
  gcm_request req{};
  double t_submit = 0, t_start = 0, t_done = 0;
  gcm_status status = GCM_OK;
  uint32_t lane = 0;
  uint64_t verts = 0, active = 0;
  // device pool ranges
  size_t out_off = 0, out_bytes = 0;
  bool has_out = false;
  // host pool range
  size_t host_off = 0, host_bytes = 0;
  bool has_host = false;
  std::atomic<bool> cancel{false};
  bool done = false;
};

uint64_t field_bytes(const gcm_grid& g) { return (uint64_t)g.nx * g.ny * g.nz * sizeof(float); }
size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }
constexpr size_t kCountsBytes = 64;  // a request's device counts, before its scratch

}  // namespace

struct gcm_server {
  gcm_server_config cfg{};
  Clock::time_point t0;
  // memory
  char* dbase = nullptr;
  char* hbase = nullptr;
  gcm::RangePool dpool, hpool;
  // queue and jobs
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> pending;
  std::deque<Job*> completed;
  std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs;
  uint64_t next_ticket = 1;
  bool stopping = false;
  // lanes
  std::vector<std::thread> threads;
  std::atomic<uint32_t> alive{0};
  // stats
  std::atomic<uint64_t> n_submitted{0}, n_completed{0}, n_rejected{0}, n_cancelled{0}, n_failed{0},
      n_requeued{0}, n_pool_faults{0};
  std::atomic<uint64_t> alloc_seq{0};

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  // Device reservation with the injected failure rule.
  bool dalloc(size_t bytes, size_t* off, Job* j) {
    if ((cfg.fault_flags & GCM_FAULT_POOL_ALLOC) && cfg.fault_param) {
      const uint64_t k = alloc_seq.fetch_add(1) + 1;
      if (k % cfg.fault_param == 0) {
        n_pool_faults.fetch_add(1);
        return false;
      }
    }
    return dpool.alloc_wait(
        bytes, off, [&] { return stopping || j->cancel.load(); }, 60000);
  }

  void finish(Job* j, gcm_status st) {
    j->status = st;
    j->t_done = now();
    {
      std::lock_guard<std::mutex> lock(m);
      j->done = true;
      completed.push_back(j);
    }
    if (st == GCM_OK) n_completed.fetch_add(1);
    else if (st == GCM_ERR_CANCELLED) n_cancelled.fetch_add(1);
    else if (st == GCM_ERR_REJECTED) n_rejected.fetch_add(1);
    else n_failed.fetch_add(1);
    cv_done.notify_all();
  }

  void lane_main(uint32_t lane);
  gcm_status run_job(uint32_t lane, gcm_ctx* ctx, cudaStream_t st, gcm_counts* h_counts, Job* j);
};

gcm_status gcm_server::run_job(uint32_t lane, gcm_ctx* ctx, cudaStream_t st, gcm_counts* h_counts, Job* j) {
  const gcm_request& r = j->req;
  const gcm_grid& g = r.grid;
  // CSG scenes are sparse surfaces: the windowed extraction path
  const bool sparse = r.kind == GCM_REQUEST_CSG;
  ctx->mesh_path = sparse ? GCM_MESH_PATH_SPARSE : GCM_MESH_PATH_AUTO;
  // 1. one pool range for the request's working memory: [field | counts |
  //    scratch | blend buffer], lent to the lane's context, so that no lane
  //    allocates or frees device memory while the others run
  const size_t fb = r.kind == GCM_REQUEST_FIELD ? 0 : align16(field_bytes(g));
  const size_t sb = align16(gcm::extraction_scratch_bytes(ctx, &g, sparse));
  const uint64_t nc = r.kind == GCM_REQUEST_LATTICE && r.lattice.mode == GCM_GRADE_BLEND
                          ? (uint64_t)r.lattice.cx * r.lattice.cy * r.lattice.cz
                          : 0;
  const size_t bb = align16((size_t)nc * GCM_BLEND_WORDS * sizeof(float));
  if (sb == 0) return GCM_ERR_INVALID_ARGUMENT;
  const size_t wbytes = fb + kCountsBytes + sb + bb;
  if (wbytes > dpool.size()) return GCM_ERR_REJECTED;  // can never be admitted
  size_t woff = 0;
  bool has_work = false;
  auto drop_work = [&] {
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    ctx->blend_buf = nullptr;
    ctx->blend_bytes = 0;
    if (has_work) dpool.release(woff, wbytes);
    has_work = false;
  };
  int tries = 0;
  while (!dalloc(wbytes, &woff, j)) {
    if (j->cancel.load() || stopping) return GCM_ERR_CANCELLED;
    if (++tries >= 4) return GCM_ERR_OUT_OF_MEMORY;
  }
  has_work = true;
  char* w = dbase + woff;
  gcm_counts* d_counts = reinterpret_cast<gcm_counts*>(w + fb);
  ctx->scratch = w + fb + kCountsBytes;
  ctx->scratch_bytes = sb;
  ctx->blend_buf = bb ? reinterpret_cast<float*>(w + fb + kCountsBytes + sb) : nullptr;
  ctx->blend_bytes = bb;
  const float* field = r.d_field;
  if (r.kind != GCM_REQUEST_FIELD) {
    float* f = reinterpret_cast<float*>(w);
    const gcm_status s = r.kind == GCM_REQUEST_LATTICE
                             ? gcm_field_lattice(ctx, &r.lattice, g.nx, g.ny, g.nz, f, st)
                             : gcm_field_csg(ctx, r.d_prims, r.n_prims, &r.frame, g.nx, g.ny, g.nz, f, st);
    if (s) {
      cudaStreamSynchronize(st);
      drop_work();
      return s;
    }
    field = f;
  }
  if (j->cancel.load()) {
    cudaStreamSynchronize(st);
    drop_work();
    return GCM_ERR_CANCELLED;
  }
  // 2. exact size: the one readback before the mesh, which admission needs
  gcm_counts c{};
  gcm_status s = gcm_count_field(ctx, field, &g, r.iso, &c, st);
  if (s) {
    cudaStreamSynchronize(st);
    drop_work();
    return s;
  }
  j->verts = c.total_verts;
  j->active = c.active_voxels;
  const size_t obytes = (size_t)std::max<uint64_t>(c.total_verts, 1) * 32;
  if (obytes + wbytes > dpool.size()) {
    drop_work();
    return GCM_ERR_REJECTED;
  }
  tries = 0;
  while (!dalloc(obytes, &j->out_off, j)) {
    if (j->cancel.load() || stopping) {
      drop_work();
      return GCM_ERR_CANCELLED;
    }
    if (++tries >= 4) {
      drop_work();
      return GCM_ERR_OUT_OF_MEMORY;
    }
  }
  j->has_out = true;
  j->out_bytes = obytes;
  float* pos = reinterpret_cast<float*>(dbase + j->out_off);
  float* norm = pos + 4 * std::max<uint64_t>(c.total_verts, 1);
  // 3. mesh and its counts enqueued; the host range is reserved while the
  //    mesh runs, then the copies follow on the stream and one
  //    synchronisation ends the request
  s = gcm_mesh_field_async(ctx, field, &g, r.iso, pos, norm, c.total_verts, d_counts, st);
  cudaError_t e = s ? cudaSuccess : cudaMemcpyAsync(h_counts, d_counts, sizeof(gcm_counts), cudaMemcpyDeviceToHost, st);
  gcm_status host_fail = GCM_OK;
  if (!s && e == cudaSuccess && hbase) {
    if (hpool.alloc_wait(
            obytes, &j->host_off, [&] { return stopping || j->cancel.load(); }, 60000)) {
      j->has_host = true;
      j->host_bytes = obytes;
      const size_t half = (size_t)c.total_verts * 16;
      char* h = hbase + j->host_off;
      e = cudaMemcpyAsync(h, pos, half, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(h + half, norm, half, cudaMemcpyDeviceToHost, st);
    } else {
      host_fail = j->cancel.load() ? GCM_ERR_CANCELLED : GCM_ERR_OUT_OF_MEMORY;
    }
  }
  const cudaError_t es = cudaStreamSynchronize(st);
  drop_work();
  if (s) return s;
  if (e != cudaSuccess || es != cudaSuccess) return GCM_ERR_CUDA;
  if (host_fail) return host_fail;
  if (h_counts->status == GCM_ERR_DEVICE_TIMEOUT) return GCM_ERR_DEVICE_TIMEOUT;
  if (h_counts->status != 0 || h_counts->total_verts != c.total_verts) return GCM_ERR_CUDA;
  if (hbase) {
    dpool.release(j->out_off, j->out_bytes);
    j->has_out = false;
  }
  (void)lane;
  return GCM_OK;
}

void gcm_server::lane_main(uint32_t lane) {
  cudaSetDevice(cfg.device);
  gcm_ctx* ctx = nullptr;
  cudaStream_t st = nullptr;
  gcm_counts* h_counts = nullptr;
  if (gcm_ctx_create(cfg.device, &ctx) != GCM_OK || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMallocHost(reinterpret_cast<void**>(&h_counts), sizeof(gcm_counts)) != cudaSuccess) {
    if (st) cudaStreamDestroy(st);
    if (ctx) gcm_ctx_destroy(ctx);
    alive.fetch_sub(1);
    cv_done.notify_all();
    return;
  }
  ctx->lent = true;  // each request lends the context its scratch from the pool
  while (true) {
    Job* j = nullptr;
    {
      std::unique_lock<std::mutex> lock(m);
      cv_work.wait(lock, [&] { return stopping || !pending.empty(); });
      if (stopping) break;
      j = pending.front();
      pending.pop_front();
    }
    if (lane == 0 && (cfg.fault_flags & GCM_FAULT_LANE_DIES)) {
      // the lane dies holding a request: it goes back to the front of the queue
      {
        std::lock_guard<std::mutex> lock(m);
        pending.push_front(j);
      }
      n_requeued.fetch_add(1);
      cv_work.notify_all();
      break;
    }
    if (lane == 0 && (cfg.fault_flags & GCM_FAULT_SLOW_LANE))
      std::this_thread::sleep_for(std::chrono::milliseconds(cfg.fault_param));
    j->lane = lane;
    j->t_start = now();
    gcm_status s = j->cancel.load() ? GCM_ERR_CANCELLED : run_job(lane, ctx, st, h_counts, j);
    if (s != GCM_OK && j->has_out) {
      dpool.release(j->out_off, j->out_bytes);
      j->has_out = false;
    }
    if (s != GCM_OK && j->has_host) {
      hpool.release(j->host_off, j->host_bytes);
      j->has_host = false;
    }
    finish(j, s);
  }
  if (st) cudaStreamDestroy(st);
  cudaFreeHost(h_counts);
  gcm_ctx_destroy(ctx);  // holds no lent range between requests
  const uint32_t left = alive.fetch_sub(1) - 1;
  if (left == 0) {
    // nothing can serve the queue any more: fail what is left
    std::vector<Job*> orphans;
    {
      std::lock_guard<std::mutex> lock(m);
      orphans.assign(pending.begin(), pending.end());
      pending.clear();
    }
    for (Job* o : orphans) finish(o, GCM_ERR_CUDA);
  }
  cv_done.notify_all();
}

extern "C" {

gcm_status gcm_server_create(const gcm_server_config* cfg, gcm_server** out) {
  if (!cfg || !out || cfg->lanes == 0 || cfg->lanes > 64 || cfg->queue_capacity == 0 || cfg->device_pool_bytes == 0)
    return GCM_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (cudaSetDevice(cfg->device) != cudaSuccess) return GCM_ERR_INVALID_ARGUMENT;
  auto* s = new gcm_server();
  s->cfg = *cfg;
  s->t0 = Clock::now();
  if (cudaMalloc(reinterpret_cast<void**>(&s->dbase), cfg->device_pool_bytes) != cudaSuccess) {
    delete s;
    return GCM_ERR_OUT_OF_MEMORY;
  }
  s->dpool.reset(cfg->device_pool_bytes);
  if (cfg->host_pool_bytes) {
    if (cudaMallocHost(reinterpret_cast<void**>(&s->hbase), cfg->host_pool_bytes) != cudaSuccess) {
      cudaFree(s->dbase);
      delete s;
      return GCM_ERR_OUT_OF_MEMORY;
    }
    s->hpool.reset(cfg->host_pool_bytes);
  }
  s->alive.store(cfg->lanes);
  for (uint32_t i = 0; i < cfg->lanes; ++i) s->threads.emplace_back([s, i] { s->lane_main(i); });
  *out = s;
  return GCM_OK;
}

gcm_status gcm_server_destroy(gcm_server* s) {
  if (!s) return GCM_OK;
  {
    std::lock_guard<std::mutex> lock(s->m);
    s->stopping = true;
  }
  s->cv_work.notify_all();
  s->dpool.wake();
  s->hpool.wake();
  for (auto& t : s->threads) t.join();
  if (s->dbase) cudaFree(s->dbase);
  if (s->hbase) cudaFreeHost(s->hbase);
  delete s;
  return GCM_OK;
}

double gcm_server_now(const gcm_server* s) { return s ? s->now() : 0.0; }

gcm_status gcm_server_submit(gcm_server* s, const gcm_request* req, uint64_t* h_ticket) {
  if (!s || !req || !h_ticket) return GCM_ERR_INVALID_ARGUMENT;
  const gcm_grid& g = req->grid;
  if (g.nx < 2 || g.ny < 2 || g.nz < 2 || req->kind > GCM_REQUEST_FIELD) return GCM_ERR_INVALID_ARGUMENT;
  if (req->kind == GCM_REQUEST_FIELD && !req->d_field) return GCM_ERR_INVALID_ARGUMENT;
  if (req->kind == GCM_REQUEST_CSG && (!req->d_prims || req->n_prims == 0)) return GCM_ERR_INVALID_ARGUMENT;
  // a request whose field alone exceeds the pool can never be admitted
  if (req->kind != GCM_REQUEST_FIELD && field_bytes(g) + 32 > s->dpool.size()) {
    s->n_rejected.fetch_add(1);
    return GCM_ERR_REJECTED;
  }
  auto j = std::make_unique<Job>();
  j->req = *req;
  j->t_submit = s->now();
  {
    std::lock_guard<std::mutex> lock(s->m);
    if (s->alive.load() == 0) return GCM_ERR_CUDA;
    if (s->pending.size() >= s->cfg.queue_capacity) return GCM_ERR_BUSY;
    j->ticket = s->next_ticket++;
    *h_ticket = j->ticket;
    s->pending.push_back(j.get());
    s->jobs.emplace(j->ticket, std::move(j));
  }
  s->n_submitted.fetch_add(1);
  s->cv_work.notify_one();
  return GCM_OK;
}

gcm_status gcm_server_poll(gcm_server* s, gcm_result* out, uint32_t max, uint32_t* n_out, uint64_t timeout_us) {
  if (!s || !out || !n_out) return GCM_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lock(s->m);
  if (s->completed.empty() && timeout_us)
    s->cv_done.wait_for(lock, std::chrono::microseconds(timeout_us), [&] { return !s->completed.empty(); });
  uint32_t n = 0;
  while (n < max && !s->completed.empty()) {
    Job* j = s->completed.front();
    s->completed.pop_front();
    gcm_result& r = out[n++];
    std::memset(&r, 0, sizeof(r));
    r.ticket = j->ticket;
    r.user_tag = j->req.user_tag;
    r.status = j->status;
    r.lane = j->lane;
    r.total_verts = j->verts;
    r.active_voxels = j->active;
    if (j->status == GCM_OK) {
      const char* base = j->has_host ? s->hbase + j->host_off : s->dbase + j->out_off;
      r.pos = reinterpret_cast<const float*>(base);
      r.norm = reinterpret_cast<const float*>(base + (size_t)std::max<uint64_t>(j->verts, 1) * 16);
      r.on_host = j->has_host ? 1 : 0;
    }
    r.t_submit = j->t_submit;
    r.t_start = j->t_start;
    r.t_done = j->t_done;
  }
  *n_out = n;
  return GCM_OK;
}

gcm_status gcm_server_release(gcm_server* s, uint64_t ticket) {
  if (!s) return GCM_ERR_INVALID_ARGUMENT;
  std::unique_ptr<Job> j;
  {
    std::lock_guard<std::mutex> lock(s->m);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end() || !it->second->done) return GCM_ERR_INVALID_ARGUMENT;
    // not yet handed out by poll: drop it from the completed list
    auto& c = s->completed;
    c.erase(std::remove(c.begin(), c.end(), it->second.get()), c.end());
    j = std::move(it->second);
    s->jobs.erase(it);
  }
  if (j->has_out) s->dpool.release(j->out_off, j->out_bytes);
  if (j->has_host) s->hpool.release(j->host_off, j->host_bytes);
  return GCM_OK;
}

gcm_status gcm_server_cancel(gcm_server* s, uint64_t ticket) {
  if (!s) return GCM_ERR_INVALID_ARGUMENT;
  Job* j = nullptr;
  bool was_pending = false;
  {
    std::lock_guard<std::mutex> lock(s->m);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return GCM_ERR_INVALID_ARGUMENT;
    j = it->second.get();
    if (j->done) return GCM_OK;
    j->cancel.store(true);
    auto pit = std::find(s->pending.begin(), s->pending.end(), j);
    if (pit != s->pending.end()) {
      s->pending.erase(pit);
      was_pending = true;
    }
  }
  s->dpool.wake();
  s->hpool.wake();
  if (was_pending) s->finish(j, GCM_ERR_CANCELLED);
  return GCM_OK;
}

gcm_status gcm_server_get_stats(gcm_server* s, gcm_server_stats* out) {
  if (!s || !out) return GCM_ERR_INVALID_ARGUMENT;
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->n_submitted.load();
  out->completed = s->n_completed.load();
  out->rejected = s->n_rejected.load();
  out->cancelled = s->n_cancelled.load();
  out->failed = s->n_failed.load();
  out->requeued = s->n_requeued.load();
  out->pool_faults = s->n_pool_faults.load();
  out->device_pool_peak = s->dpool.peak();
  out->host_pool_peak = s->hpool.peak();
  out->device_pool_used = s->dpool.used();
  out->lanes_alive = s->alive.load();
  {
    std::lock_guard<std::mutex> lock(s->m);
    out->pending = (uint32_t)s->pending.size();
  }
  return GCM_OK;
}

// Host-only exercise of the pool allocator (no GPU): runs `n` operations on a
// pool of `size` bytes; op[i] > 0 reserves op[i] bytes, op[i] < 0 releases the
// reservation made by operation -op[i]-1.  result[i] = offset, or -1 when a
// reservation failed.  Returns the number of free ranges left.
int64_t gcm_test_pool_script(uint64_t size, const int64_t* op, int64_t* result, uint32_t n) {
  gcm::RangePool pool(size);
  std::vector<size_t> off(n, 0), len(n, 0);
  for (uint32_t i = 0; i < n; ++i) {
    if (op[i] > 0) {
      size_t o = 0;
      if (pool.try_alloc((size_t)op[i], &o)) {
        off[i] = o;
        len[i] = (size_t)op[i];
        result[i] = (int64_t)o;
      } else {
        result[i] = -1;
      }
    } else {
      const int64_t k = -op[i] - 1;
      if (k >= 0 && k < (int64_t)i && len[k]) {
        pool.release(off[k], len[k]);
        len[k] = 0;
      }
      result[i] = 0;
    }
  }
  return (int64_t)pool.free_ranges();
}

}  // extern "C"
