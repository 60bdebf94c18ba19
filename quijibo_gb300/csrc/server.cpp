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
// with them.  Small field requests in the precision form go to a batch
// worker: all that wait when it frees up run as one multi-request pass (one
// tile queue over every item, field.cu's batch kernels), replayed from a
// CUDA graph captured on the first batch, with the batch table rewritten in
// place each time.  Small mesh requests of the same form take their field
// from that pass too (an item of the batch); the field is copied out of the
// arena and the request goes back to the dispatcher, which hands it to a
// worker to mesh (so meshes still overlap one another).  Results are copied
// to caller buffers; latencies are measured from submission to completion
// on the host clock.
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
#include "qj_kernels.h"

namespace {

using Clock = std::chrono::steady_clock;

// Largest mesh request (voxels) whose field joins the field batch pass.
constexpr int64_t kMeshBatchVoxels = 1ll << 22;

struct Job {
  int64_t ticket;
  qjg_request req;
  // owned copies of the inputs
  std::vector<double> top_roots, top_powers, bot_roots, bot_powers, xyz, target, params;
  int64_t est_bytes = 0;
  int64_t voxels = 0;
  bool batchable = false;   // field (or mesh) request for the field batch worker
  bool mbatch = false;      // a mesh request whose field runs in the field batch
  bool staged = false;      // ... whose field has run: a worker meshes d_staged
  double* d_staged = nullptr;  // that field (X*Y*Z doubles, freed by the worker)
  bool ebatchable = false;  // FP32 energy request for the energy batch worker
  Clock::time_point t_submit, t_admit, t_done;
  qjg_result res;
};

// Device and pinned host buffers of the batch worker, and its graph.
struct FieldBatcher {
  int64_t cap = 0;  // voxels per batch (sum over items)
  cudaStream_t s = nullptr;
  qj::BatchTable* d_tab = nullptr;
  qj::MapParams* d_maps = nullptr;
  double* d_arena = nullptr;
  uint32_t *d_list = nullptr, *d_sorted = nullptr, *d_ff = nullptr;
  uint8_t* d_keys = nullptr;
  unsigned* d_hist = nullptr;
  qj::BatchCounts* d_counts = nullptr;
  qj::DevStats* d_st = nullptr;
  qj::BatchTable* h_tab = nullptr;
  qj::MapParams* h_maps = nullptr;
  qj::BatchCounts* h_counts = nullptr;
  qj::BatchShapes sh{};
  cudaGraphExec_t exec = nullptr;
  bool ok = false;

  int init(int64_t voxels) {
    cap = voxels;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return QJG_ERR_CUDA;
    const size_t n = (size_t)cap;
    if (cudaMalloc((void**)&d_tab, sizeof(qj::BatchTable)) ||
        cudaMalloc((void**)&d_maps, qj::BATCH_MAX * sizeof(qj::MapParams)) ||
        cudaMalloc((void**)&d_arena, n * sizeof(double)) ||
        cudaMalloc((void**)&d_list, n * sizeof(uint32_t)) ||
        cudaMalloc((void**)&d_sorted, n * sizeof(uint32_t)) ||
        cudaMalloc((void**)&d_ff, n * sizeof(uint32_t)) || cudaMalloc((void**)&d_keys, n) ||
        cudaMalloc((void**)&d_hist, qj::REFINE_KEYS * sizeof(unsigned)) ||
        cudaMalloc((void**)&d_counts, qj::BATCH_MAX * sizeof(qj::BatchCounts)) ||
        cudaMalloc((void**)&d_st, sizeof(qj::DevStats)) ||
        cudaMallocHost((void**)&h_tab, sizeof(qj::BatchTable)) ||
        cudaMallocHost((void**)&h_maps, qj::BATCH_MAX * sizeof(qj::MapParams)) ||
        cudaMallocHost((void**)&h_counts, qj::BATCH_MAX * sizeof(qj::BatchCounts)))
      return QJG_ERR_NOMEM;
    sh = qj::batch_shapes();
    ok = true;
    return QJG_OK;
  }

  ~FieldBatcher() {
    if (exec) cudaGraphExecDestroy(exec);
    for (void* p : {(void*)d_tab, (void*)d_maps, (void*)d_arena, (void*)d_list, (void*)d_sorted,
                    (void*)d_ff, (void*)d_keys, (void*)d_hist, (void*)d_counts, (void*)d_st})
      if (p) cudaFree(p);
    for (void* p : {(void*)h_tab, (void*)h_maps, (void*)h_counts})
      if (p) cudaFreeHost(p);
    if (s) cudaStreamDestroy(s);
  }

  qj::BatchBuffers buffers() const {
    qj::BatchBuffers b;
    b.tab = d_tab;
    b.maps = d_maps;
    b.rl = {d_list, d_keys, d_ff};
    b.sorted = d_sorted;
    b.hist = d_hist;
    b.counts = d_counts;
    b.st = d_st;
    return b;
  }

  // One pass over `jobs` (each batchable; their voxels sum to <= cap); the
  // fields of the mesh jobs among them are copied to their own device
  // buffers (Job::d_staged).  Returns the pass's status; a mesh job whose
  // copy failed has its own status in its result.
  int run(std::vector<std::shared_ptr<Job>>& jobs);
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
    default: {
      // inputs and gradient, per-sample results and sort, checkpoints every
      // 8 steps (16 B each), partial rows of the sums
      const int64_t nck = r.max_it > 0 ? (r.max_it - 1) / 8 + 1 : 0;
      const int64_t slots = 5 * (int64_t)(r.n_top + r.n_bot) + 3;
      return r.n_samples * (32 + 48 + 16 * nck) + (r.n_samples / 32 + 1) * slots * 8 + (1 << 20);
    }
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

  // batch worker
  std::unique_ptr<FieldBatcher> batcher;
  int64_t batch_cap = 0;  // 0: no batch worker
  bool batch_idle = false;
  std::vector<std::shared_ptr<Job>> batch_q;
  std::condition_variable batch_cv;
  int64_t batched = 0, batches = 0, max_batch = 0, mesh_batched = 0;

  // energy batch worker
  bool ebatch_on = false;
  bool ebatch_idle = false;
  std::vector<std::shared_ptr<Job>> ebatch_q;
  std::condition_variable ebatch_cv;
  int64_t ebatched = 0, ebatches = 0, max_ebatch = 0;

  explicit qjg_server(int workers) : idle(workers, 0), worker_q(workers), worker_cv(workers) {}
};

namespace {

void mesh_from_field(qjg_ctx* mctx, cudaStream_t s, Job& j, const double* d_field);

void run_job(qjg_ctx* ctx, cudaStream_t s, Job& j) {
  qjg_request& r = j.req;
  qjg_result& out = j.res;
  if (j.staged) {
    // a mesh whose field the batch pass computed
    mesh_from_field(ctx, s, j, j.d_staged);
    cudaFreeAsync(j.d_staged, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && out.error == QJG_OK) out.error = QJG_ERR_CUDA;
    j.d_staged = nullptr;
    return;
  }
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
  it.rel_tol = r.precision == QJG_FP32_REFINE ? r.rel_tol : 0.0;
  if (rc == QJG_OK && r.kind == QJG_REQ_FIELD) {
    const int64_t vox = (int64_t)r.grid.res[0] * r.grid.res[1] * r.grid.res[2];
    double* d_field = nullptr;
    if (qj_malloc_async(ctx, &d_field, vox * sizeof(double), s) != cudaSuccess) rc = QJG_ERR_NOMEM;
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
    if (qj_malloc_async(ctx, &v64, vcap * 3 * sizeof(double), s) != cudaSuccess ||
        qj_malloc_async(ctx, &tris, tcap * 3 * sizeof(int32_t), s) != cudaSuccess)
      rc = QJG_ERR_NOMEM;
    qjg_mesh_stats ms = {};
    // meshes up to 2^24 voxels run as the fixed launch sequence (one wait at
    // the end instead of host reads between slabs; the context's buffers are
    // sized to the request's capacities, so larger meshes keep the path whose
    // buffers grow with the actual counts); a mesh that outgrows its
    // capacities is re-run on that path for the counts it needs
    const int64_t vox = (int64_t)r.grid.res[0] * r.grid.res[1] * r.grid.res[2];
    const bool fixed = vox <= (int64_t)1 << 24;
    if (rc == QJG_OK && fixed) {
      rc = qjg_mesh_prepare(ctx, &r.grid, 0, vcap, tcap);
      if (rc == QJG_OK)
        rc = qjg_mesh_stream_async(ctx, h, &r.grid, &it, r.iso, 0, v64, nullptr, vcap, tris, tcap, s);
      if (rc == QJG_OK) rc = cudaStreamSynchronize(s) == cudaSuccess ? QJG_OK : QJG_ERR_CUDA;
      if (rc == QJG_OK) rc = qjg_mesh_async_result(ctx, &ms);
    }
    if ((rc == QJG_OK && !fixed) || rc == QJG_ERR_CAPACITY)
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
    if (qj_malloc_async(ctx, &d_p, P * sizeof(double), s) != cudaSuccess ||
        qj_malloc_async(ctx, &d_g, P * sizeof(double), s) != cudaSuccess ||
        qj_malloc_async(ctx, &d_x, std::max<int64_t>(r.n_samples, 1) * 3 * sizeof(double), s) != cudaSuccess ||
        qj_malloc_async(ctx, &d_t, std::max<int64_t>(r.n_samples, 1) * sizeof(double), s) != cudaSuccess)
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

// Completion bookkeeping of one job (srv->mu held).
void finish_job(qjg_server* srv, Job& j, Clock::time_point now) {
  j.t_done = now;
  j.res.status = j.res.error == QJG_OK ? QJG_STATUS_DONE : QJG_STATUS_FAILED;
  j.res.latency_ms = std::chrono::duration<double, std::milli>(j.t_done - j.t_submit).count();
  j.res.queue_ms = std::chrono::duration<double, std::milli>(j.t_admit - j.t_submit).count();
  j.res.run_ms = std::chrono::duration<double, std::milli>(j.t_done - j.t_admit).count();
  srv->in_use -= j.est_bytes;
  srv->running--;
  j.res.t_admit_ms = std::chrono::duration<double, std::milli>(j.t_admit - srv->t_created).count();
  j.res.t_done_ms = std::chrono::duration<double, std::milli>(j.t_done - srv->t_created).count();
  if (j.res.error == QJG_OK) {
    srv->completed++;
    srv->latencies_ms.push_back(j.res.latency_ms);
  } else {
    srv->failed++;
  }
  srv->t_last = j.t_done;
}

void worker_main(qjg_server* srv, int w) {
  qjg_ctx* ctx = nullptr;
  cudaSetDevice(srv->device);
  const int crc = qjg_create(srv->device, &ctx);
  // requests' buffers go back to the device when a request ends, so that
  // the HBM budget of admitted requests is what the workers hold
  if (crc == QJG_OK) qj_pool_keep(ctx, false);
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
      finish_job(srv, *j, Clock::now());
      srv->cv_done.notify_all();
      srv->cv_dispatch.notify_one();
    }
  }
  if (s) cudaStreamDestroy(s);
  if (ctx) qjg_destroy(ctx);
}

// The mesh of a mesh job from its field computed by the batch pass
// (d_field): the bisection evaluates the map as the streaming mesher does,
// so the vertices and triangles are the ones qjg_mesh_stream gives for the
// request.
void mesh_from_field(qjg_ctx* mctx, cudaStream_t s, Job& j, const double* d_field) {
  qjg_request& r = j.req;
  qjg_result& out = j.res;
  qjg_rootset h = -1;
  int rc = qjg_rootset_upload(mctx, r.n_top, j.top_roots.data(), j.top_powers.data(), r.sigma_top,
                              r.n_bot, j.bot_roots.empty() ? nullptr : j.bot_roots.data(),
                              j.bot_powers.empty() ? nullptr : j.bot_powers.data(), r.sigma_bot,
                              r.scale, &h);
  qjg_iter it = {};
  it.max_it = r.max_it;
  it.precision = r.precision;
  it.refine_pow = QJG_REFINE_INT;
  it.escape = r.escape;
  it.band_h = 2.0;
  it.field_tol = 1e-3;
  it.rel_tol = r.precision == QJG_FP32_REFINE ? r.rel_tol : 0.0;
  double* v64 = nullptr;
  int32_t* tris = nullptr;
  const int64_t vcap = std::max<int64_t>(r.vert_cap, 1), tcap = std::max<int64_t>(r.tri_cap, 1);
  if (rc == QJG_OK && (qj_malloc_async(mctx, &v64, vcap * 3 * sizeof(double), s) != cudaSuccess ||
                       qj_malloc_async(mctx, &tris, tcap * 3 * sizeof(int32_t), s) != cudaSuccess))
    rc = QJG_ERR_NOMEM;
  qjg_mesh_stats ms = {};
  if (rc == QJG_OK)
    rc = qjg_mesh_field(mctx, h, &r.grid, &it, d_field, QJG_EDGE_BISECT, r.iso, 0, v64, nullptr,
                        vcap, tris, tcap, &ms, s);
  // a mesh that outgrows its capacities reports the counts it needs
  out.n_verts = ms.n_verts;
  out.n_tris = ms.n_tris;
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
  if (h >= 0) qjg_rootset_free(mctx, h);
  out.error = rc;
}

int FieldBatcher::run(std::vector<std::shared_ptr<Job>>& jobs) {
  const int n = (int)jobs.size();
  int64_t off = 0, tiles = 0;
  h_tab->n = n;
  for (int k = 0; k < n; k++) {
    const qjg_request& r = jobs[k]->req;
    const Job& j = *jobs[k];
    if (qj_fill_map(&h_maps[k], r.n_top, j.top_roots.data(), j.top_powers.data(), r.sigma_top,
                    r.n_bot, j.bot_roots.empty() ? nullptr : j.bot_roots.data(),
                    j.bot_powers.empty() ? nullptr : j.bot_powers.data(), r.sigma_bot,
                    r.scale) >= 0)
      return QJG_ERR_ARG;
    qjg_iter it = {};
    it.max_it = r.max_it;
    it.precision = r.precision;
    it.refine_pow = QJG_REFINE_INT;
    it.want_de = 1;
    it.escape = r.escape;
    it.band_h = 2.0;
    it.field_tol = 1e-3;
    it.rel_tol = r.precision == QJG_FP32_REFINE ? r.rel_tol : 0.0;
    qj::BatchItem& b = h_tab->items[k];
    b.g = qj_grid_params(&r.grid, 0, r.grid.res[2]);
    b.it = qj_iter_params(&it, &r.grid);
    b.field = d_arena + off;
    b.de = nullptr;
    b.tile0 = tiles;
    b.refine = r.precision == QJG_FP32_REFINE ? 1 : 0;
    b.pad_ = 0;
    off += j.voxels;
    tiles += qj::batch_item_tiles(r.grid.res[0], r.grid.res[1], r.grid.res[2]);
  }
  h_tab->total_tiles = tiles;
  if (cudaMemcpyAsync(d_maps, h_maps, (size_t)n * sizeof(qj::MapParams), cudaMemcpyHostToDevice,
                      s) ||
      cudaMemcpyAsync(d_tab, h_tab, sizeof(qj::BatchTable), cudaMemcpyHostToDevice, s))
    return QJG_ERR_CUDA;
  if (!exec) {
    // the pass reads the table from d_tab and every count from the device,
    // so one capture serves every batch
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) return QJG_ERR_CUDA;
    const cudaError_t le = qj::launch_field_batch(buffers(), sh, s);
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (le || ce || !graph) return QJG_ERR_CUDA;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie) {
      exec = nullptr;
      return QJG_ERR_CUDA;
    }
  }
  if (cudaGraphLaunch(exec, s)) return QJG_ERR_CUDA;
  if (cudaMemcpyAsync(h_counts, d_counts, (size_t)n * sizeof(qj::BatchCounts),
                      cudaMemcpyDeviceToHost, s))
    return QJG_ERR_CUDA;
  off = 0;
  for (int k = 0; k < n; k++) {
    Job& j = *jobs[k];
    if (!j.mbatch && j.req.out_field &&
        cudaMemcpyAsync(j.req.out_field, d_arena + off, (size_t)j.voxels * sizeof(double),
                        cudaMemcpyDeviceToHost, s))
      return QJG_ERR_CUDA;
    off += j.voxels;
  }
  if (cudaStreamSynchronize(s)) return QJG_ERR_CUDA;
  for (int k = 0; k < n; k++) jobs[k]->res.voxel_iters = (int64_t)h_counts[k].voxel_iters;
  // the mesh jobs' fields out of the arena (the next pass reuses it)
  off = 0;
  for (int k = 0; k < n; k++) {
    Job& j = *jobs[k];
    if (j.mbatch) {
      const size_t bytes = (size_t)j.voxels * sizeof(double);
      if (cudaMallocAsync((void**)&j.d_staged, bytes, s) != cudaSuccess) {
        j.d_staged = nullptr;
        j.res.error = QJG_ERR_NOMEM;
      } else if (cudaMemcpyAsync(j.d_staged, d_arena + off, bytes, cudaMemcpyDeviceToDevice, s) !=
                 cudaSuccess) {
        j.res.error = QJG_ERR_CUDA;
      }
    }
    off += j.voxels;
  }
  if (cudaStreamSynchronize(s)) return QJG_ERR_CUDA;
  return QJG_OK;
}

void batch_main(qjg_server* srv) {
  cudaSetDevice(srv->device);
  for (;;) {
    std::vector<std::shared_ptr<Job>> jobs;
    {
      std::unique_lock<std::mutex> lk(srv->mu);
      srv->batch_idle = true;
      srv->cv_dispatch.notify_one();
      srv->batch_cv.wait(lk, [&] { return srv->stop || !srv->batch_q.empty(); });
      srv->batch_idle = false;
      if (srv->batch_q.empty()) break;  // stopping
      jobs.swap(srv->batch_q);
      for (auto& j : jobs) j->res.status = QJG_STATUS_RUNNING;
    }
    const int rc = srv->batcher->run(jobs);
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      const Clock::time_point now = Clock::now();
      srv->batches++;
      srv->batched += (int64_t)jobs.size();
      srv->max_batch = std::max<int64_t>(srv->max_batch, (int64_t)jobs.size());
      for (auto& j : jobs) {
        // a failed pass fails every job; after it, a mesh job has its own status
        if (rc != QJG_OK) j->res.error = rc;
        if (j->mbatch) {
          srv->mesh_batched++;
          j->mbatch = false;
          if (j->res.error == QJG_OK && j->d_staged) {
            // to the front of the queue: a worker meshes it (its bytes stay
            // counted in the budget from its admission to the batch)
            j->staged = true;
            srv->running--;
            srv->waiting.push_front(j);
            continue;
          }
          if (j->d_staged) cudaFree(j->d_staged);
          j->d_staged = nullptr;
        }
        finish_job(srv, *j, now);
      }
      srv->cv_done.notify_all();
      srv->cv_dispatch.notify_all();
    }
  }
}

// One pass over FP32 energy + gradient jobs: their inputs to the device,
// qjg_energy_backward_batch, the gradients back.
int run_energy_batch(qjg_ctx* ctx, cudaStream_t s, std::vector<std::shared_ptr<Job>>& jobs) {
  const int K = (int)jobs.size();
  int64_t doubles = 0;
  for (auto& j : jobs) {
    const qjg_request& r = j->req;
    doubles += 2 * (5 * (int64_t)(r.n_top + r.n_bot) + 1) + 4 * r.n_samples;
  }
  double* arena = nullptr;
  if (qj_malloc_async(ctx, &arena, (size_t)std::max<int64_t>(doubles, 1) * sizeof(double), s))
    return QJG_ERR_NOMEM;
  std::vector<qjg_energy_item> items((size_t)K);
  int rc = QJG_OK;
  double* at = arena;
  for (int k = 0; k < K && rc == QJG_OK; k++) {
    Job& j = *jobs[(size_t)k];
    const qjg_request& r = j.req;
    const int64_t P = 5 * (int64_t)(r.n_top + r.n_bot) + 1;
    qjg_energy_item& it = items[(size_t)k];
    std::memset(&it, 0, sizeof it);
    double* dp = at;
    double* dg = dp + P;
    double* dx = dg + P;
    double* dt = dx + 3 * r.n_samples;
    at = dt + r.n_samples;
    if (cudaMemcpyAsync(dp, j.params.data(), P * sizeof(double), cudaMemcpyHostToDevice, s) ||
        (r.n_samples &&
         (cudaMemcpyAsync(dx, j.xyz.data(), 3 * r.n_samples * sizeof(double), cudaMemcpyHostToDevice, s) ||
          cudaMemcpyAsync(dt, j.target.data(), r.n_samples * sizeof(double), cudaMemcpyHostToDevice, s))))
      rc = QJG_ERR_CUDA;
    it.d_params = dp;
    it.n_top = r.n_top;
    it.n_bot = r.n_bot;
    it.n = r.n_samples;
    it.d_xyz = dx;
    it.d_target = dt;
    it.slice = r.grid.slice;
    it.max_it = r.max_it;
    it.escape = r.escape;
    it.d_sat = r.d_sat;
    it.d_grad = dg;
  }
  if (rc == QJG_OK) rc = qjg_energy_backward_batch(ctx, K, items.data(), s);
  for (int k = 0; k < K && rc == QJG_OK; k++) {
    Job& j = *jobs[(size_t)k];
    j.res.energy = items[(size_t)k].energy;
    const int64_t P = 5 * (int64_t)(j.req.n_top + j.req.n_bot) + 1;
    if (j.req.out_grad && cudaMemcpyAsync(j.req.out_grad, items[(size_t)k].d_grad, P * sizeof(double),
                                          cudaMemcpyDeviceToHost, s))
      rc = QJG_ERR_CUDA;
  }
  cudaFreeAsync(arena, s);
  if (cudaStreamSynchronize(s) != cudaSuccess && rc == QJG_OK) rc = QJG_ERR_CUDA;
  return rc;
}

void ebatch_main(qjg_server* srv) {
  cudaSetDevice(srv->device);
  qjg_ctx* ctx = nullptr;
  const int crc = qjg_create(srv->device, &ctx);
  if (crc == QJG_OK) qj_pool_keep(ctx, false);
  cudaStream_t s = nullptr;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  for (;;) {
    std::vector<std::shared_ptr<Job>> jobs;
    {
      std::unique_lock<std::mutex> lk(srv->mu);
      srv->ebatch_idle = true;
      srv->cv_dispatch.notify_one();
      srv->ebatch_cv.wait(lk, [&] { return srv->stop || !srv->ebatch_q.empty(); });
      srv->ebatch_idle = false;
      if (srv->ebatch_q.empty()) break;  // stopping
      jobs.swap(srv->ebatch_q);
      for (auto& j : jobs) j->res.status = QJG_STATUS_RUNNING;
    }
    const int rc = crc != QJG_OK ? crc : run_energy_batch(ctx, s, jobs);
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      const Clock::time_point now = Clock::now();
      srv->ebatches++;
      srv->ebatched += (int64_t)jobs.size();
      srv->max_ebatch = std::max<int64_t>(srv->max_ebatch, (int64_t)jobs.size());
      for (auto& j : jobs) {
        j->res.error = rc;
        finish_job(srv, *j, now);
      }
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
    bool admitted = false;
    // the batch worker takes every batchable request waiting when it is free
    if (srv->batcher && srv->batch_idle && srv->batch_q.empty()) {
      int64_t vox = 0;
      for (size_t i = 0; i < srv->waiting.size() && (int)srv->batch_q.size() < qj::BATCH_MAX;) {
        auto job = srv->waiting[i];
        // a mesh job's mesher buffers count against the budget
        const bool fits = srv->in_use + job->est_bytes <= srv->budget || srv->in_use == 0;
        if (!job->batchable || job->staged || vox + job->voxels > srv->batch_cap || !fits) {
          i++;
          continue;
        }
        srv->waiting.erase(srv->waiting.begin() + (long)i);
        vox += job->voxels;
        srv->in_use += job->est_bytes;
        srv->peak_in_use = std::max(srv->peak_in_use, srv->in_use);
        job->t_admit = Clock::now();
        srv->batch_q.push_back(job);
        srv->running++;
      }
      if (!srv->batch_q.empty()) {
        srv->peak_running = std::max(srv->peak_running, srv->running);
        srv->batch_idle = false;
        srv->batch_cv.notify_one();
        admitted = true;
      }
    }
    // the energy batch worker takes the FP32 energy requests waiting when it
    // is free (up to BATCH_MAX items and 2^23 samples) that fit the budget
    if (srv->ebatch_on && srv->ebatch_idle && srv->ebatch_q.empty()) {
      int64_t samples = 0;
      for (size_t i = 0; i < srv->waiting.size() && (int)srv->ebatch_q.size() < qj::BATCH_MAX;) {
        auto job = srv->waiting[i];
        const bool fits = srv->in_use + job->est_bytes <= srv->budget || srv->in_use == 0;
        const bool room = srv->ebatch_q.empty() || samples + job->req.n_samples <= (1ll << 23);
        if (!job->ebatchable || !room || !fits) {
          i++;
          continue;
        }
        srv->waiting.erase(srv->waiting.begin() + (long)i);
        samples += job->req.n_samples;
        srv->in_use += job->est_bytes;
        srv->peak_in_use = std::max(srv->peak_in_use, srv->in_use);
        job->t_admit = Clock::now();
        srv->ebatch_q.push_back(job);
        srv->running++;
      }
      if (!srv->ebatch_q.empty()) {
        srv->peak_running = std::max(srv->peak_running, srv->running);
        srv->ebatch_idle = false;
        srv->ebatch_cv.notify_one();
        admitted = true;
      }
    }
    // admit while a worker is idle and the head (or a request within the
    // lookahead window) fits the budget
    int w = -1;
    for (int k = 0; k < nw; k++)
      if (srv->idle[k] && srv->worker_q[k].empty()) {
        w = k;
        break;
      }
    if (w >= 0 && !srv->waiting.empty()) {
      int seen = 0;
      for (size_t i = 0; i < srv->waiting.size() && seen < srv->lookahead; i++) {
        auto job = srv->waiting[i];
        if (job->batchable && !job->staged && srv->batcher) continue;  // the batch worker's
        if (job->ebatchable && srv->ebatch_on) continue;  // the energy batch worker's
        seen++;
        // a request larger than the whole budget runs alone; a staged mesh
        // has been counted since its admission to the batch
        if (job->staged || srv->in_use + job->est_bytes <= srv->budget || srv->in_use == 0) {
          srv->waiting.erase(srv->waiting.begin() + (long)i);
          if (!job->staged) srv->in_use += job->est_bytes;
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
  // the batch worker's arena (FP64 outputs, lists; ~21 B per voxel) is set
  // aside from the budget when the budget holds at least four times it
  const int64_t cap = 1ll << 25;
  const int64_t arena = cap * 21 + (int64_t)qj::BATCH_MAX * (int64_t)sizeof(qj::MapParams);
  if (hbm_budget_bytes >= 4 * arena) {
    cudaSetDevice(device);
    std::unique_ptr<FieldBatcher> fb(new FieldBatcher());
    if (fb->init(cap) == QJG_OK) {
      srv->batcher = std::move(fb);
      srv->batch_cap = cap;
      srv->budget -= arena;
    } else {
      cudaGetLastError();
    }
  }
  for (int w = 0; w < workers; w++) srv->threads.emplace_back(worker_main, srv, w);
  if (srv->batcher) srv->threads.emplace_back(batch_main, srv);
  srv->ebatch_on = true;
  srv->threads.emplace_back(ebatch_main, srv);
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
  j->voxels = (int64_t)req->grid.res[0] * req->grid.res[1] * req->grid.res[2];
  if ((req->kind == QJG_REQ_FIELD || req->kind == QJG_REQ_MESH) && req->precision != QJG_FP64 &&
      req->grid.res[0] > 0 &&
      req->grid.res[1] > 0 && req->grid.res[2] > 0 && j->voxels <= srv->batch_cap &&
      j->voxels <= qj::BATCH_ITEM_VOXELS && req->max_it >= 0 && req->escape > 0) {
    // batch items take integer effective exponents (the double-float head and
    // the FP64 pass by products)
    bool ints = true;
    for (int i = 0; i < nt + nb && ints; i++) {
      const double e = (i < nt ? req->sigma_top * req->top_powers[i]
                               : req->sigma_bot * req->bot_powers[i - nt]);
      ints = e == std::floor(e) && e >= 1 && e <= QJ_MAX_INT_EXP;
    }
    // meshes join the batch up to kMeshBatchVoxels, so that a large mesh
    // field does not hold up the small fields of its pass
    const bool mesh = req->kind == QJG_REQ_MESH;
    j->batchable = ints && (!mesh || j->voxels <= kMeshBatchVoxels);
    j->mbatch = j->batchable && mesh;
    // a field lives inside the batch arena; a mesh job keeps its mesher's
    // part and the copy of its field
    if (j->batchable && !mesh) j->est_bytes = 0;
    if (j->mbatch) j->est_bytes += j->voxels * (int64_t)sizeof(double);
  }
  j->ebatchable = req->kind == QJG_REQ_ENERGY && req->precision != QJG_FP64 &&
                  req->max_it >= 0 && req->escape > 0;
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
    if (!srv->batch_q.empty() || !srv->ebatch_q.empty()) return false;
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
  out->pad_ = 0;
  out->batched = srv->batched;
  out->batches = srv->batches;
  out->max_batch = srv->max_batch;
  out->energy_batched = srv->ebatched;
  out->energy_batches = srv->ebatches;
  out->max_energy_batch = srv->max_ebatch;
  out->mesh_batched = srv->mesh_batched;
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
  srv->batch_cv.notify_all();
  srv->ebatch_cv.notify_all();
  for (auto& cv : srv->worker_cv) cv.notify_all();
  for (auto& t : srv->threads) t.join();
  srv->batcher.reset();
  delete srv;
}

}  // extern "C"
