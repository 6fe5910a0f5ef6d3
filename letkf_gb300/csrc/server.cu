// server.cu -- continuous-batching analysis server on one device.
//
// Jobs (a regional sweep or a Lorenz-96 ring analysis) are queued as they
// arrive.  `nslots` worker threads each own a CUDA stream and take the job at
// the head of the queue as soon as its device footprint fits the budget, so
// jobs that arrive while others run start at once and overlap with them on
// the device; each sweep launch is capped at 1/nslots of the resident CTAs so
// the slots share the SMs instead of queueing behind one persistent grid.
// Domains with a key keep their device state (points, observations, ensemble
// buffers) between jobs; idle ones are released oldest first when a new job
// needs the memory.  Admission is strictly in arrival order.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "letkf_gpu.h"

namespace letkf {

int cuda_status(cudaError_t e);
void note_launch();

__global__ void srv_iota1(int n, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i + 1;
}

__global__ void srv_fill(int n, double v, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = v;
}

template <typename S, typename D>
__global__ void srv_convert(int64_t n, const S* __restrict__ a, D* __restrict__ b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (D)a[i];
}

template <typename S, typename D>
static void convert(int64_t n, const S* a, D* b, cudaStream_t s) {
  if (n <= 0) return;
  srv_convert<S, D><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, a, b);
  note_launch();
}

// resident device state of a Lorenz-96 domain
struct L96State {
  int nx = 0, ny = 0, ne = 0;
  int *cell = nullptr, *pix = nullptr, *nobsl = nullptr, *status = nullptr;
  int64_t* offs = nullptr;
  double *hdxf = nullptr, *dep = nullptr, *xb = nullptr, *xa = nullptr, *infl = nullptr, *trans = nullptr;
};

static size_t l96_bound_rows(const letkf_job_desc& j) {
  // an observation is selected by at most 2 ceil(xmaxloc) + 1 points
  const double xmaxloc = j.xlocal * 2.0 * std::sqrt(10.0 / 3.0);
  const double reach = 2.0 * std::ceil(xmaxloc) + 1.0;
  const double per = std::min<double>(reach, (double)j.npts);
  return (size_t)((double)j.nobs * per) + 1;
}

static size_t l96_footprint(const letkf_job_desc& j) {
  const size_t nx = (size_t)j.npts, ny = (size_t)j.nobs, ne = (size_t)j.ne;
  size_t b = ny * (4 + ne * 8 + 8) + nx * (4 + 4 + 4 + 8 * 3 + 8 * ne * 2 + ne * ne * 8) + 8 * (nx + 1);
  const size_t rows = l96_bound_rows(j);
  b += rows * (4 + 8 * 3 + ne * 8);                                    // lists and gathered rows
  if (j.precision == LETKF_PREC_MIXED) b += rows * (3 * 4 + ne * 4) + nx * ne * ne * 4;
  b += 16 * (nx + 1) + ny * 16 + 8192;                                 // search buckets and scan scratch
  return b;
}

static int l96_alloc(L96State* st, const letkf_job_desc& j, cudaStream_t s) {
  st->nx = j.npts;
  st->ny = j.nobs;
  st->ne = j.ne;
  const size_t nx = (size_t)j.npts, ny = (size_t)std::max(j.nobs, 1), ne = (size_t)j.ne;
  bool ok = true;
  auto A = [&](auto** p, size_t bytes) { ok = ok && cudaMallocAsync((void**)p, bytes, s) == cudaSuccess; };
  A(&st->cell, ny * 4);
  A(&st->hdxf, ny * ne * 8);
  A(&st->dep, ny * 8);
  A(&st->pix, nx * 4);
  A(&st->nobsl, nx * 4);
  A(&st->status, nx * 4);
  A(&st->offs, (nx + 1) * 8);
  A(&st->xb, nx * ne * 8);
  A(&st->xa, nx * ne * 8);
  A(&st->infl, nx * 8);
  A(&st->trans, nx * ne * ne * 8);
  if (!ok) return LETKF_ERR_CUDA;
  srv_iota1<<<(unsigned)((nx + 255) / 256), 256, 0, s>>>(j.npts, st->pix);
  note_launch();
  return LETKF_OK;
}

static void l96_free(L96State* st, cudaStream_t s) {
  void* p[] = {st->cell, st->hdxf, st->dep, st->pix, st->nobsl, st->status, st->offs, st->xb, st->xa, st->infl,
               st->trans};
  for (void* q : p)
    if (q) cudaFreeAsync(q, s);
  *st = L96State();
}

static int l96_run(L96State* st, const letkf_job_desc& j, cudaStream_t s) {
  const int nx = j.npts, ny = j.nobs, ne = j.ne;
  int rc = LETKF_OK;
  auto C = [&](int r) {
    if (rc == LETKF_OK && r != LETKF_OK) rc = r;
  };
  if (ny > 0) {
    C(cuda_status(cudaMemcpyAsync(st->cell, j.obs_cell, sizeof(int) * ny, cudaMemcpyHostToDevice, s)));
    C(cuda_status(cudaMemcpyAsync(st->hdxf, j.hdxf, sizeof(double) * ny * ne, cudaMemcpyHostToDevice, s)));
    C(cuda_status(cudaMemcpyAsync(st->dep, j.dep, sizeof(double) * ny, cudaMemcpyHostToDevice, s)));
  }
  C(cuda_status(cudaMemcpyAsync(st->xb, j.xb, sizeof(double) * (size_t)nx * ne, cudaMemcpyHostToDevice, s)));
  if (j.infl) {
    C(cuda_status(cudaMemcpyAsync(st->infl, j.infl, sizeof(double) * nx, cudaMemcpyHostToDevice, s)));
  } else {
    srv_fill<<<(nx + 255) / 256, 256, 0, s>>>(nx, j.msw_infl > 0.0 ? j.msw_infl : 1.0, st->infl);
    note_launch();
  }
  C(letkf_search_l96(nx, ny, st->cell, nx, st->pix, j.xlocal, 0.0, -1.0, j.obserr, nullptr, st->nobsl, nullptr,
                     nullptr, nullptr, s));
  C(letkf_exclusive_scan(nx, st->nobsl, st->offs, s));
  int64_t total = 0;
  C(cuda_status(cudaMemcpyAsync(&total, st->offs + nx, sizeof(int64_t), cudaMemcpyDeviceToHost, s)));
  C(cuda_status(cudaStreamSynchronize(s)));
  if (rc != LETKF_OK) return rc;
  const size_t nr = (size_t)std::max<int64_t>(total, 1);
  int* idx = nullptr;
  double *rloc = nullptr, *rdiag = nullptr, *rows = nullptr, *dl = nullptr;
  float *r32 = nullptr, *t32 = nullptr;
  bool ok = cudaMallocAsync((void**)&idx, nr * 4, s) == cudaSuccess &&
            cudaMallocAsync((void**)&rloc, nr * 8, s) == cudaSuccess &&
            cudaMallocAsync((void**)&rdiag, nr * 8, s) == cudaSuccess &&
            cudaMallocAsync((void**)&rows, nr * ne * 8, s) == cudaSuccess &&
            cudaMallocAsync((void**)&dl, nr * 8, s) == cudaSuccess;
  if (ok && j.precision == LETKF_PREC_MIXED)
    ok = cudaMallocAsync((void**)&r32, nr * (ne + 3) * 4, s) == cudaSuccess &&
         cudaMallocAsync((void**)&t32, (size_t)nx * ne * ne * 4, s) == cudaSuccess;
  if (!ok) rc = LETKF_ERR_CUDA;
  C(letkf_search_l96(nx, ny, st->cell, nx, st->pix, j.xlocal, 0.0, -1.0, j.obserr, st->offs, nullptr, idx, rloc,
                     rdiag, s));
  if (total > 0) C(letkf_gather_rows(ne, total, idx, st->hdxf, st->dep, 8, rows, dl, s));
  if (rc == LETKF_OK) {
    if (j.precision == LETKF_PREC_F64) {
      C(letkf_core_batch_f64(ne, nx, st->offs, rows, rdiag, rloc, dl, st->infl, st->trans, nullptr, nullptr, 0, 0.0,
                             st->status, s));
    } else {
      float *rw = r32, *rd = r32 + nr * ne, *rl = rd + nr, *dp = rl + nr;
      convert<double, float>((int64_t)nr * ne, rows, rw, s);
      convert<double, float>((int64_t)nr, rdiag, rd, s);
      convert<double, float>((int64_t)nr, rloc, rl, s);
      convert<double, float>((int64_t)nr, dl, dp, s);
      C(letkf_core_batch_mixed(ne, nx, st->offs, rw, rd, rl, dp, st->infl, t32, nullptr, 0, 0.0, st->status, s));
      convert<float, double>((int64_t)nx * ne * ne, t32, st->trans, s);
    }
  }
  if (rc == LETKF_OK && j.msw_infl > 0.0) {
    srv_fill<<<(nx + 255) / 256, 256, 0, s>>>(nx, j.msw_infl, st->infl);
    note_launch();
  }
  if (rc == LETKF_OK) C(letkf_update_f64(ne, nx, 1, st->xb, st->trans, nullptr, st->xa, s));
  if (rc == LETKF_OK)
    C(cuda_status(cudaMemcpyAsync(j.xa, st->xa, sizeof(double) * (size_t)nx * ne, cudaMemcpyDeviceToHost, s)));
  if (rc == LETKF_OK && j.infl)
    C(cuda_status(cudaMemcpyAsync(j.infl, st->infl, sizeof(double) * nx, cudaMemcpyDeviceToHost, s)));
  std::vector<int> stat((size_t)nx);
  if (rc == LETKF_OK)
    C(cuda_status(cudaMemcpyAsync(stat.data(), st->status, sizeof(int) * nx, cudaMemcpyDeviceToHost, s)));
  void* tmp[] = {idx, rloc, rdiag, rows, dl, r32, t32};
  for (void* q : tmp)
    if (q) cudaFreeAsync(q, s);
  C(cuda_status(cudaStreamSynchronize(s)));
  if (rc == LETKF_OK)
    for (int p = 0; p < nx; p++)
      if (stat[p] != LETKF_OK) return stat[p];
  return rc;
}

}  // namespace letkf

using namespace letkf;

struct Domain {
  int64_t key = -1;
  int kind = 0;
  letkf_job_desc shape;  // dimensions the state was built for
  letkf_sweep_t sweep = nullptr;
  L96State l96;
  bool l96_ready = false;
  size_t bytes = 0;
  bool busy = false;
  uint64_t last_use = 0;
};

struct JobRec {
  letkf_job_desc d;
  letkf_job_result r;
  bool done = false;
};

struct letkf_server_s {
  letkf_server_desc d;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<int64_t> queue;
  std::map<int64_t, JobRec> jobs;
  std::map<int64_t, Domain*> domains;
  std::vector<std::thread> workers;
  cudaStream_t rel = nullptr;  // frees of released domains
  int64_t next_id = 0;
  size_t used = 0, peak = 0;
  int running = 0;
  bool stop = false;
  uint64_t tick = 0;
  std::vector<double> latencies;
  double first_submit = -1.0, last_done = 0.0;
  int64_t points_done = 0, failed = 0;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

static bool same_shape(const letkf_job_desc& a, const letkf_job_desc& b) {
  return a.kind == b.kind && a.ne == b.ne && a.nv == b.nv && a.npts == b.npts && a.nlon == b.nlon &&
         a.nlat == b.nlat && a.precision == b.precision && (a.kind != LETKF_JOB_L96 || a.nobs == b.nobs);
}

static size_t job_footprint(const letkf_job_desc& j) {
  if (j.kind == LETKF_JOB_L96) return l96_footprint(j);
  letkf_sweep_desc sd;
  memset(&sd, 0, sizeof(sd));
  sd.ne = j.ne;
  sd.nv = j.nv;
  sd.nlon = j.nlon;
  sd.nlat = j.nlat;
  sd.npts = j.npts;
  sd.precision = j.precision;
  size_t b = 0;
  letkf_sweep_footprint(&sd, j.nobs, &b);
  return b;
}

// the domain's jobs have all finished (each job ends with a stream sync)
static void release_domain(letkf_server_s* S, Domain* dm) {
  if (dm->sweep) letkf_sweep_destroy(dm->sweep);
  if (dm->l96_ready) {
    l96_free(&dm->l96, S->rel);
    cudaStreamSynchronize(S->rel);
  }
  delete dm;
}

// run one job on the worker's stream; dm is the job's (possibly new) domain
static int run_job(letkf_server_s* S, const letkf_job_desc& j, Domain* dm, cudaStream_t s) {
  if (j.kind == LETKF_JOB_L96) {
    if (!dm->l96_ready) {
      dm->l96_ready = true;
      int rc = l96_alloc(&dm->l96, j, s);
      if (rc != LETKF_OK) return rc;
    }
    return l96_run(&dm->l96, j, s);
  }
  int rc = LETKF_OK;
  if (!dm->sweep) {
    letkf_sweep_desc sd;
    memset(&sd, 0, sizeof(sd));
    sd.ne = j.ne;
    sd.nv = j.nv;
    sd.nlon = j.nlon;
    sd.nlat = j.nlat;
    sd.npts = j.npts;
    sd.precision = j.precision;
    memcpy(sd.params, j.params, sizeof(sd.params));
    sd.minfl = j.minfl;
    rc = letkf_sweep_create(&dm->sweep, &sd);
    if (rc != LETKF_OK) return rc;
    rc = letkf_sweep_set_points(dm->sweep, j.pri, j.prj, j.prlev, nullptr, 4);
    if (rc != LETKF_OK) return rc;
  }
  letkf_sweep_t h = dm->sweep;
  rc = letkf_sweep_set_obs(h, j.nobs, j.ori, j.orj, j.olev, j.odat, j.oerr, j.dep, j.ocls, nullptr, nullptr, 0,
                           j.hdxf, j.precision == LETKF_PREC_MIXED);
  if (rc == LETKF_OK) rc = letkf_sweep_set_background(h, j.xb, 0);
  if (rc == LETKF_OK && j.infl) rc = letkf_sweep_set_inflation(h, j.infl, 0);
  if (rc == LETKF_OK && !j.infl) {
    std::vector<double> one((size_t)j.npts, 1.0);
    rc = letkf_sweep_set_inflation(h, one.data(), 0);
  }
  if (rc == LETKF_OK) rc = letkf_sweep_set_option(h, LETKF_OPT_GRID_SHARE, S->d.nslots);
  if (rc == LETKF_OK) rc = letkf_sweep_run(h, s);
  if (rc == LETKF_OK) rc = letkf_sweep_get_analysis(h, j.xa, 0);
  std::vector<int> stat((size_t)j.npts);
  if (rc == LETKF_OK) rc = letkf_sweep_get_diagnostics(h, j.infl, nullptr, stat.data(), nullptr);
  if (rc == LETKF_OK)
    for (int p = 0; p < j.npts; p++)
      if (stat[p] != LETKF_OK) return stat[p];
  return rc;
}

// under S->mu: make room for `need` bytes by releasing idle domains, oldest first
static bool make_room(letkf_server_s* S, size_t need, int64_t keep_key, std::vector<Domain*>* victims) {
  while (S->used + need > S->d.hbm_budget) {
    Domain* best = nullptr;
    for (auto& kv : S->domains)
      if (!kv.second->busy && kv.first != keep_key && (!best || kv.second->last_use < best->last_use))
        best = kv.second;
    if (!best) return false;
    S->domains.erase(best->key);
    S->used -= best->bytes;
    victims->push_back(best);
  }
  return true;
}

static void worker_main(letkf_server_s* S) {
  cudaSetDevice(S->d.device);
  cudaStream_t s = nullptr;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    int64_t id = -1;
    Domain* dm = nullptr;
    size_t charge = 0;
    std::vector<Domain*> victims;
    while (id < 0) {
      if (S->queue.empty()) {
        if (S->stop) break;
        S->cv_work.wait(lk);
        continue;
      }
      const int64_t head = S->queue.front();
      JobRec& jr = S->jobs[head];
      const letkf_job_desc& j = jr.d;
      auto it = j.domain >= 0 ? S->domains.find(j.domain) : S->domains.end();
      Domain* cur = it != S->domains.end() ? it->second : nullptr;
      if (cur && cur->busy) {  // the domain's previous job is still on the device
        S->cv_work.wait(lk);
        continue;
      }
      const size_t fp = job_footprint(j);
      const bool reuse = cur && same_shape(cur->shape, j);
      const size_t have = reuse ? cur->bytes : 0;
      const size_t need = fp > have ? fp - have : 0;
      if (fp > S->d.hbm_budget) {  // can never fit
        S->queue.pop_front();
        jr.r.status = LETKF_ERR_CAPACITY;
        jr.r.t_start = jr.r.t_done = S->now();
        jr.done = true;
        S->failed++;
        S->cv_done.notify_all();
        continue;
      }
      if (cur && !reuse) {  // same key, new shape: drop the old state
        S->domains.erase(cur->key);
        S->used -= cur->bytes;
        victims.push_back(cur);
        cur = nullptr;
      }
      if (!make_room(S, need, j.domain, &victims)) {
        // wait for running jobs to finish (memory frees) before trying again
        if (!victims.empty()) break;
        S->cv_work.wait(lk);
        continue;
      }
      S->queue.pop_front();
      id = head;
      if (!cur) {
        cur = new Domain();
        cur->key = j.domain;
        cur->kind = j.kind;
        cur->shape = j;
        if (j.domain >= 0) S->domains[j.domain] = cur;
      }
      const size_t before = cur->bytes;
      cur->bytes = std::max(before, fp);
      S->used += cur->bytes - before;
      cur->busy = true;
      dm = cur;
      charge = cur->bytes;
      S->peak = std::max(S->peak, S->used);
      jr.r.t_start = S->now();
      jr.r.device_bytes = charge;
      S->running++;
    }
    if (id < 0 && victims.empty()) break;  // stopping and nothing queued
    letkf_job_desc jd{};
    if (id >= 0) jd = S->jobs[id].d;  // copied under the lock: submits insert into the map meanwhile
    lk.unlock();
    for (Domain* v : victims) release_domain(S, v);
    int rc = LETKF_OK;
    if (id >= 0) rc = run_job(S, jd, dm, s);
    lk.lock();
    if (id < 0) continue;
    JobRec& jr = S->jobs[id];
    jr.r.status = rc;
    jr.r.t_done = S->now();
    jr.done = true;
    S->running--;
    dm->busy = false;
    dm->last_use = ++S->tick;
    if (rc == LETKF_OK) {
      S->latencies.push_back(jr.r.t_done - jr.r.t_submit);
      S->points_done += jr.d.npts;
      S->last_done = std::max(S->last_done, jr.r.t_done);
    } else {
      S->failed++;
    }
    Domain* drop = nullptr;
    if (jr.d.domain < 0 || rc != LETKF_OK) {
      if (jr.d.domain >= 0) S->domains.erase(jr.d.domain);
      S->used -= dm->bytes;
      drop = dm;
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
    if (drop) {
      lk.unlock();
      release_domain(S, drop);
      lk.lock();
    }
  }
  lk.unlock();
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
}

extern "C" {

int letkf_server_create(letkf_server_t* out, const letkf_server_desc* d) {
  if (!out || !d || d->nslots < 1 || d->nslots > 16 || d->device < 0) return LETKF_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return LETKF_ERR_NOGPU;
  }
  if (d->device >= ndev) return LETKF_ERR_ARG;
  if (cudaSetDevice(d->device) != cudaSuccess) return LETKF_ERR_CUDA;
  letkf_server_s* S = new letkf_server_s();
  S->d = *d;
  S->t0 = std::chrono::steady_clock::now();
  if (S->d.hbm_budget == 0) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    S->d.hbm_budget = fr / 10 * 8;
  }
  if (cudaStreamCreateWithFlags(&S->rel, cudaStreamNonBlocking) != cudaSuccess) {
    delete S;
    return LETKF_ERR_CUDA;
  }
  for (int i = 0; i < d->nslots; i++) S->workers.emplace_back(worker_main, S);
  *out = S;
  return LETKF_OK;
}

static bool valid_job(const letkf_job_desc* j) {
  if (j->ne < 2 || j->ne > LETKF_MAX_NE || j->npts < 1 || j->nobs < 0 || !j->xb || !j->xa) return false;
  if (j->precision != LETKF_PREC_F64 && j->precision != LETKF_PREC_MIXED) return false;
  if (j->nobs > 0 && (!j->hdxf || !j->dep)) return false;
  if (j->kind == LETKF_JOB_L96) return j->nv == 1 && (j->nobs == 0 || j->obs_cell) && j->xlocal > 0.0;
  if (j->kind != LETKF_JOB_SCALE_SWEEP) return false;
  if (j->nv < 1 || j->nv > 8 || j->nlon < 1 || j->nlat < 1 || !j->pri || !j->prj || !j->prlev) return false;
  return j->nobs == 0 || (j->ori && j->orj && j->olev && j->odat && j->oerr && j->ocls);
}

int letkf_server_submit(letkf_server_t S, const letkf_job_desc* job, int64_t* job_id) {
  if (!S || !job || !job_id) return LETKF_ERR_ARG;
  if (!valid_job(job)) return LETKF_ERR_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  if (S->stop) return LETKF_ERR_ARG;
  const int64_t id = S->next_id++;
  JobRec& jr = S->jobs[id];
  jr.d = *job;
  jr.r.status = LETKF_PENDING;
  jr.r.t_submit = S->now();
  if (S->first_submit < 0.0) S->first_submit = jr.r.t_submit;
  S->queue.push_back(id);
  *job_id = id;
  S->cv_work.notify_all();
  return LETKF_OK;
}

int letkf_server_wait(letkf_server_t S, int64_t id, double timeout_s, letkf_job_result* res) {
  if (!S) return LETKF_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->jobs.find(id);
  if (it == S->jobs.end()) return LETKF_ERR_ARG;
  auto done = [&] { return it->second.done; };
  if (timeout_s < 0.0) S->cv_done.wait(lk, done);
  else S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done);
  if (res) *res = it->second.r;
  if (!it->second.done) return LETKF_PENDING;
  // the result has been handed out: release the record, so a long-lived
  // server keeps only unfinished and unclaimed jobs
  const int st = it->second.r.status;
  S->jobs.erase(it);
  return st;
}

int letkf_server_stats_get(letkf_server_t S, letkf_server_stats* st) {
  if (!S || !st) return LETKF_ERR_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  memset(st, 0, sizeof(*st));
  st->submitted = S->next_id;
  st->completed = (int64_t)S->latencies.size();
  st->failed = S->failed;
  std::vector<double> l = S->latencies;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    auto q = [&](double f) {
      const double pos = f * (double)(l.size() - 1);
      const size_t i = (size_t)pos;
      const double w = pos - (double)i;
      return i + 1 < l.size() ? l[i] * (1.0 - w) + l[i + 1] * w : l[i];
    };
    st->p50_latency_s = q(0.50);
    st->p99_latency_s = q(0.99);
    const double span = S->last_done - S->first_submit;
    st->points_per_s = span > 0.0 ? (double)S->points_done / span : 0.0;
  }
  st->peak_bytes = S->peak;
  st->resident_domains = (int)S->domains.size();
  return LETKF_OK;
}

int letkf_server_destroy(letkf_server_t S) {
  if (!S) return LETKF_OK;
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stop = true;
    S->cv_work.notify_all();
  }
  for (auto& t : S->workers) t.join();
  cudaSetDevice(S->d.device);
  for (auto& kv : S->domains) release_domain(S, kv.second);
  cudaStreamDestroy(S->rel);
  delete S;
  return LETKF_OK;
}

}  // extern "C"
