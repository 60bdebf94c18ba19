// Continuous-batching request server over the field, mesh and energy paths.
//
// No reference counterpart: the reference runs one driver per job.  Requests
// (field, field + mesh, energy + gradient) are submitted from any host
// thread.  A dispatcher admits them as soon as a worker slot is free and
// their device-memory estimate fits the HBM budget, looking past a request
// that does not fit yet (up to `lookahead` places, so small requests flow
// around a large one without starving it for long).  Each worker owns a
// context (private scratch) and a stream, so admitted requests run
// concurrently on the device; a request admitted while others run overlaps
// with them.  Results are copied to caller buffers; latencies are measured
// from submission to completion on the host clock.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/quijibo_gpu.h"
#include "qj_ctx.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  int64_t ticket;
  qjg_request req;
  // owned copies of the inputs
  std::vector<double> top_roots, top_powers, bot_roots, bot_powers, xyz, target, params;
  int64_t est_bytes = 0;
  Clock::time_point t_submit, t_admit, t_done;
  qjg_result res;
};

int64_t estimate_bytes(const qjg_request& r) {
  const int64_t vox = (int64_t)r.grid.res[0] * r.grid.res[1] * r.grid.res[2];
  const int64_t slab = (int64_t)r.grid.res[0] * r.grid.res[1];
  switch (r.kind) {
    case QJG_REQ_FIELD:
      return vox * (8 + 4 + (r.precision == QJG_FP32_REFINE ? 4 : 0)) + (1 << 20);
    case QJG_REQ_MESH: {
      const int64_t nz = 64;
      return slab * (nz + 2) * (8 + 1 + 1 + 4 + 12) + r.vert_cap * 36 + r.tri_cap * 24 + (1 << 20);
    }
    default:
      return r.n_samples * 40 + (1 << 20);
  }
}

}  // namespace

struct qjg_server {
  int device = 0;
  int64_t budget = 0;
  int lookahead = 16;
  std::mutex mu;
  std::condition_variable cv_dispatch, cv_done;
  std::deque<std::shared_ptr<Job>> waiting;
  std::map<int64_t, std::shared_ptr<Job>> jobs;
  int64_t next_ticket = 1;
  int64_t in_use = 0;
  bool stop = false;
  std::vector<char> idle;  // worker w waits with an empty queue
  std::vector<std::thread> threads;
  std::vector<std::deque<std::shared_ptr<Job>>> worker_q;
  std::vector<std::condition_variable> worker_cv;
  std::vector<double> latencies_ms;
  int64_t completed = 0, failed = 0;
  int64_t peak_in_use = 0;
  int running = 0, peak_running = 0;
  Clock::time_point t_created = Clock::now();
  Clock::time_point t_first, t_last;
  bool any = false;

  explicit qjg_server(int workers) : idle(workers, 0), worker_q(workers), worker_cv(workers) {}
};

namespace {

void run_job(qjg_ctx* ctx, cudaStream_t s, Job& j) {
  qjg_request& r = j.req;
  qjg_result& out = j.res;
  int rc = QJG_OK;
  qjg_rootset h = -1;
  if (r.kind == QJG_REQ_FIELD || r.kind == QJG_REQ_MESH) {
    rc = qjg_rootset_upload(ctx, r.n_top, j.top_roots.data(), j.top_powers.data(), r.sigma_top,
                            r.n_bot, j.bot_roots.empty() ? nullptr : j.bot_roots.data(),
                            j.bot_powers.empty() ? nullptr : j.bot_powers.data(), r.sigma_bot,
                            r.scale, &h);
  }
  qjg_iter it = {};
  it.max_it = r.max_it;
  it.precision = r.precision;
  it.refine_pow = QJG_REFINE_INT;
  it.escape = r.escape;
  it.band_h = 2.0;
  it.field_tol = 1e-3;
  if (rc == QJG_OK && r.kind == QJG_REQ_FIELD) {
    const int64_t vox = (int64_t)r.grid.res[0] * r.grid.res[1] * r.grid.res[2];
    double* d_field = nullptr;
    if (cudaMallocAsync((void**)&d_field, vox * sizeof(double), s) != cudaSuccess) rc = QJG_ERR_NOMEM;
    if (rc == QJG_OK) rc = qjg_field(ctx, h, &r.grid, &it, 0, r.grid.res[2], d_field, nullptr, s);
    qjg_field_stats fs = {};
    if (rc == QJG_OK) rc = qjg_field_stats_read(ctx, s, &fs);
    if (rc == QJG_OK && r.out_field &&
        cudaMemcpyAsync(r.out_field, d_field, vox * sizeof(double), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess)
      rc = QJG_ERR_CUDA;
    if (d_field) cudaFreeAsync(d_field, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && rc == QJG_OK) rc = QJG_ERR_CUDA;
    out.voxel_iters = fs.voxel_iters;
    out.refined = fs.refined;
  } else if (rc == QJG_OK && r.kind == QJG_REQ_MESH) {
    double* v64 = nullptr;
    int32_t* tris = nullptr;
    int64_t vcap = std::max<int64_t>(r.vert_cap, 1), tcap = std::max<int64_t>(r.tri_cap, 1);
    if (cudaMallocAsync((void**)&v64, vcap * 3 * sizeof(double), s) != cudaSuccess ||
        cudaMallocAsync((void**)&tris, tcap * 3 * sizeof(int32_t), s) != cudaSuccess)
      rc = QJG_ERR_NOMEM;
    qjg_mesh_stats ms = {};
    if (rc == QJG_OK)
      rc = qjg_mesh_stream(ctx, h, &r.grid, &it, r.iso, 0, v64, nullptr, vcap, tris, tcap, &ms, s);
    out.n_verts = ms.n_verts;
    out.n_tris = ms.n_tris;
    out.voxel_iters = ms.field.voxel_iters;
    out.refined = ms.field.refined;
    if (rc == QJG_OK && r.out_verts &&
        cudaMemcpyAsync(r.out_verts, v64, ms.n_verts * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                        s) != cudaSuccess)
      rc = QJG_ERR_CUDA;
    if (rc == QJG_OK && r.out_tris &&
        cudaMemcpyAsync(r.out_tris, tris, ms.n_tris * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                        s) != cudaSuccess)
      rc = QJG_ERR_CUDA;
    if (v64) cudaFreeAsync(v64, s);
    if (tris) cudaFreeAsync(tris, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && rc == QJG_OK) rc = QJG_ERR_CUDA;
  } else if (rc == QJG_OK && r.kind == QJG_REQ_ENERGY) {
    const int64_t P = 5 * (r.n_top + r.n_bot) + 1;
    double *d_p = nullptr, *d_x = nullptr, *d_t = nullptr, *d_g = nullptr;
    if (cudaMallocAsync((void**)&d_p, P * sizeof(double), s) != cudaSuccess ||
        cudaMallocAsync((void**)&d_g, P * sizeof(double), s) != cudaSuccess ||
        cudaMallocAsync((void**)&d_x, std::max<int64_t>(r.n_samples, 1) * 3 * sizeof(double), s) != cudaSuccess ||
        cudaMallocAsync((void**)&d_t, std::max<int64_t>(r.n_samples, 1) * sizeof(double), s) != cudaSuccess)
      rc = QJG_ERR_NOMEM;
    if (rc == QJG_OK &&
        (cudaMemcpyAsync(d_p, j.params.data(), P * sizeof(double), cudaMemcpyHostToDevice, s) ||
         cudaMemcpyAsync(d_x, j.xyz.data(), r.n_samples * 3 * sizeof(double), cudaMemcpyHostToDevice, s) ||
         cudaMemcpyAsync(d_t, j.target.data(), r.n_samples * sizeof(double), cudaMemcpyHostToDevice, s)))
      rc = QJG_ERR_CUDA;
    double e = 0;
    if (rc == QJG_OK)
      rc = qjg_energy_backward(ctx, d_p, r.n_top, r.n_bot, r.n_samples, d_x, d_t, r.grid.slice,
                               r.max_it, r.escape, r.d_sat,
                               r.precision == QJG_FP64 ? QJG_FP64 : QJG_FP32, &e, d_g, s);
    out.energy = e;
    if (rc == QJG_OK && r.out_grad &&
        cudaMemcpyAsync(r.out_grad, d_g, P * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
      rc = QJG_ERR_CUDA;
    for (double* ptr : {d_p, d_x, d_t, d_g})
      if (ptr) cudaFreeAsync(ptr, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && rc == QJG_OK) rc = QJG_ERR_CUDA;
  }
  if (h >= 0) qjg_rootset_free(ctx, h);
  out.error = rc;
}

void worker_main(qjg_server* srv, int w) {
  qjg_ctx* ctx = nullptr;
  cudaSetDevice(srv->device);
  const int crc = qjg_create(srv->device, &ctx);
  cudaStream_t s = nullptr;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  for (;;) {
    std::shared_ptr<Job> j;
    {
      std::unique_lock<std::mutex> lk(srv->mu);
      srv->idle[w] = 1;
      srv->cv_dispatch.notify_one();
      srv->worker_cv[w].wait(lk, [&] { return srv->stop || !srv->worker_q[w].empty(); });
      srv->idle[w] = 0;
      if (srv->worker_q[w].empty()) break;  // stopping
      j = srv->worker_q[w].front();
      srv->worker_q[w].pop_front();
      j->res.status = QJG_STATUS_RUNNING;
    }
    if (crc != QJG_OK)
      j->res.error = crc;
    else
      run_job(ctx, s, *j);
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      j->t_done = Clock::now();
      j->res.status = j->res.error == QJG_OK ? QJG_STATUS_DONE : QJG_STATUS_FAILED;
      j->res.latency_ms = std::chrono::duration<double, std::milli>(j->t_done - j->t_submit).count();
      j->res.queue_ms = std::chrono::duration<double, std::milli>(j->t_admit - j->t_submit).count();
      j->res.run_ms = std::chrono::duration<double, std::milli>(j->t_done - j->t_admit).count();
      srv->in_use -= j->est_bytes;
      srv->running--;
      j->res.t_admit_ms = std::chrono::duration<double, std::milli>(j->t_admit - srv->t_created).count();
      j->res.t_done_ms = std::chrono::duration<double, std::milli>(j->t_done - srv->t_created).count();
      if (j->res.error == QJG_OK) {
        srv->completed++;
        srv->latencies_ms.push_back(j->res.latency_ms);
      } else {
        srv->failed++;
      }
      srv->t_last = j->t_done;
      srv->cv_done.notify_all();
      srv->cv_dispatch.notify_one();
    }
  }
  if (s) cudaStreamDestroy(s);
  if (ctx) qjg_destroy(ctx);
}

void dispatcher_main(qjg_server* srv) {
  std::unique_lock<std::mutex> lk(srv->mu);
  const int nw = (int)srv->worker_q.size();
  for (;;) {
    // admit while a worker is idle and the head (or a request within the
    // lookahead window) fits the budget
    bool admitted = false;
    int w = -1;
    for (int k = 0; k < nw; k++)
      if (srv->idle[k] && srv->worker_q[k].empty()) {
        w = k;
        break;
      }
    if (w >= 0 && !srv->waiting.empty()) {
      const int look = std::min<int>(srv->lookahead, (int)srv->waiting.size());
      for (int i = 0; i < look; i++) {
        auto job = srv->waiting[i];
        // a request larger than the whole budget runs alone
        if (srv->in_use + job->est_bytes <= srv->budget || srv->in_use == 0) {
          srv->waiting.erase(srv->waiting.begin() + i);
          srv->in_use += job->est_bytes;
          srv->peak_in_use = std::max(srv->peak_in_use, srv->in_use);
          srv->running++;
          srv->peak_running = std::max(srv->peak_running, srv->running);
          job->t_admit = Clock::now();
          srv->worker_q[w].push_back(job);
          srv->worker_cv[w].notify_one();
          admitted = true;
          break;
        }
      }
    }
    if (admitted) continue;
    if (srv->stop && srv->waiting.empty()) break;
    srv->cv_dispatch.wait(lk);
  }
}

}  // namespace

extern "C" {

int qjg_server_create(int device, int32_t workers, int64_t hbm_budget_bytes, qjg_server** out) {
  if (!out || workers < 1 || workers > 64 || hbm_budget_bytes <= 0) return QJG_ERR_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return QJG_ERR_CUDA;
  qjg_server* srv = new qjg_server(workers);
  srv->device = device;
  srv->budget = hbm_budget_bytes;
  for (int w = 0; w < workers; w++) srv->threads.emplace_back(worker_main, srv, w);
  srv->threads.emplace_back(dispatcher_main, srv);
  *out = srv;
  return QJG_OK;
}

int qjg_server_submit(qjg_server* srv, const qjg_request* req, int64_t* ticket) {
  if (!srv || !req || !ticket) return QJG_ERR_ARG;
  if (req->kind != QJG_REQ_FIELD && req->kind != QJG_REQ_MESH && req->kind != QJG_REQ_ENERGY)
    return QJG_ERR_ARG;
  if (req->n_top < 1 || req->n_bot < 0 || req->n_top + req->n_bot > QJG_MAX_ROOTS) return QJG_ERR_ARG;
  auto j = std::make_shared<Job>();
  j->req = *req;
  const int nt = req->n_top, nb = req->n_bot;
  if (req->kind == QJG_REQ_ENERGY) {
    if (!req->params || req->n_samples < 0 || (req->n_samples > 0 && (!req->xyz || !req->target)))
      return QJG_ERR_ARG;
    j->params.assign(req->params, req->params + 5 * (nt + nb) + 1);
    j->xyz.assign(req->xyz, req->xyz + 3 * req->n_samples);
    j->target.assign(req->target, req->target + req->n_samples);
  } else {
    if (!req->top_roots || !req->top_powers || (nb > 0 && (!req->bot_roots || !req->bot_powers)))
      return QJG_ERR_ARG;
    j->top_roots.assign(req->top_roots, req->top_roots + 4 * nt);
    j->top_powers.assign(req->top_powers, req->top_powers + nt);
    if (nb) {
      j->bot_roots.assign(req->bot_roots, req->bot_roots + 4 * nb);
      j->bot_powers.assign(req->bot_powers, req->bot_powers + nb);
    }
  }
  j->est_bytes = estimate_bytes(*req);
  std::memset(&j->res, 0, sizeof j->res);
  j->res.status = QJG_STATUS_QUEUED;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    j->ticket = srv->next_ticket++;
    j->t_submit = Clock::now();
    if (!srv->any) {
      srv->t_first = j->t_submit;
      srv->any = true;
    }
    srv->jobs[j->ticket] = j;
    srv->waiting.push_back(j);
    *ticket = j->ticket;
  }
  srv->cv_dispatch.notify_one();
  return QJG_OK;
}

int qjg_server_poll(qjg_server* srv, int64_t ticket, qjg_result* out) {
  if (!srv || !out) return QJG_ERR_ARG;
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->jobs.find(ticket);
  if (it == srv->jobs.end()) return QJG_ERR_HANDLE;
  *out = it->second->res;
  return QJG_OK;
}

int qjg_server_wait(qjg_server* srv, int64_t ticket, qjg_result* out) {
  if (!srv) return QJG_ERR_ARG;
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->jobs.find(ticket);
  if (it == srv->jobs.end()) return QJG_ERR_HANDLE;
  auto j = it->second;
  srv->cv_done.wait(lk, [&] {
    return j->res.status == QJG_STATUS_DONE || j->res.status == QJG_STATUS_FAILED;
  });
  if (out) *out = j->res;
  srv->jobs.erase(ticket);
  return QJG_OK;
}

int qjg_server_drain(qjg_server* srv) {
  if (!srv) return QJG_ERR_ARG;
  std::unique_lock<std::mutex> lk(srv->mu);
  srv->cv_done.wait(lk, [&] {
    if (!srv->waiting.empty()) return false;
    for (auto& q : srv->worker_q)
      if (!q.empty()) return false;
    for (auto& kv : srv->jobs)
      if (kv.second->res.status == QJG_STATUS_QUEUED || kv.second->res.status == QJG_STATUS_RUNNING)
        return false;
    return true;
  });
  return QJG_OK;
}

int qjg_server_read_stats(qjg_server* srv, qjg_server_stats* out) {
  if (!srv || !out) return QJG_ERR_ARG;
  std::lock_guard<std::mutex> lk(srv->mu);
  std::vector<double> l = srv->latencies_ms;
  std::sort(l.begin(), l.end());
  auto pct = [&](double p) {
    if (l.empty()) return 0.0;
    const size_t k = (size_t)std::min<double>(l.size() - 1, std::ceil(p * l.size()) - 1);
    return l[k];
  };
  out->completed = srv->completed;
  out->failed = srv->failed;
  out->p50_ms = pct(0.50);
  out->p99_ms = pct(0.99);
  out->max_ms = l.empty() ? 0.0 : l.back();
  out->span_s = srv->any ? std::chrono::duration<double>(srv->t_last - srv->t_first).count() : 0.0;
  out->in_use_bytes = srv->in_use;
  out->peak_in_use_bytes = srv->peak_in_use;
  out->peak_running = srv->peak_running;
  return QJG_OK;
}

void qjg_server_destroy(qjg_server* srv) {
  if (!srv) return;
  qjg_server_drain(srv);
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv_dispatch.notify_all();
  for (auto& cv : srv->worker_cv) cv.notify_all();
  for (auto& t : srv->threads) t.join();
  delete srv;
}

}  // extern "C"
