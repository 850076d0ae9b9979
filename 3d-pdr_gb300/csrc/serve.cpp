// serve.cpp -- a serving loop for batched chemistry requests.
//
// There is no counterpart in the reference: it is the service around the
// chemistry path that a client calls with blocks of cells (physical
// conditions plus initial abundances) and gets abundances back.  Design:
//   * one lane per network: a dispatcher thread, a CUDA stream, a solver
//     instance (pdr_solver, own scratch) and pinned staging plus device
//     buffers for max_batch_cells cells, all allocated when the server is
//     created -- nothing is allocated while serving;
//   * FIFO admission with continuous batching: whenever a lane is free it
//     takes every queued request of its network, in arrival order, that fits
//     the remaining batch capacity, packs them into one launch (per-cell end
//     times) and returns each request's cells when the launch completes;
//   * lanes of different networks run concurrently on their own streams.  A
//     persistent launch holds its SMs until its last cell is done, so by
//     default a lane's launch spans every SM only when no other lane is
//     running and an equal share with the running lanes otherwise
//     (pdr_solver_set_max_sms).
// Each cell is integrated independently, so a request's results do not depend
// on what it was batched with.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pdr_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  pdr_serve_request r;
  Clock::time_point submitted, finished;
  bool done = false;
  int result = 0;
};

struct Lane {
  pdr_net *net = nullptr;
  pdr_solver *solver = nullptr;
  cudaStream_t stream = nullptr;
  int nspec = 0, nreac = 0;
  // pinned staging and device buffers, max_batch_cells cells each
  double *h_nH = nullptr, *h_T = nullptr, *h_Td = nullptr, *h_rad = nullptr, *h_AV = nullptr, *h_col = nullptr,
         *h_ab = nullptr, *h_tend = nullptr;
  int *h_status = nullptr;
  double *d_nH = nullptr, *d_T = nullptr, *d_Td = nullptr, *d_rad = nullptr, *d_AV = nullptr, *d_col = nullptr,
         *d_ab = nullptr, *d_tend = nullptr, *d_rate = nullptr;
  int *d_status = nullptr, *d_rstatus = nullptr;
  std::deque<Req *> queue;
  std::thread thread;
  long long batches = 0, cells = 0;
};

}  // namespace

struct pdr_server {
  pdr_phys phys;
  pdr_server_opts opts;
  std::vector<Lane> lanes;
  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  bool stop = false;
  long long next_ticket = 1;
  std::unordered_map<long long, Req *> reqs;
  int device = 0, sms = 0;
  int running = 0;   // lanes with a launch in flight
};

namespace {

int alloc_lane(pdr_server *s, Lane &L) {
  const size_t n = (size_t)s->opts.max_batch_cells, nr = (size_t)s->opts.nrays;
  auto dev = [&](void **p, size_t bytes) { return cudaMalloc(p, bytes); };
  auto host = [&](void **p, size_t bytes) { return cudaHostAlloc(p, bytes, cudaHostAllocDefault); };
  cudaError_t e = cudaSuccess;
  if ((e = host((void **)&L.h_nH, 8 * n)) || (e = host((void **)&L.h_T, 8 * n)) || (e = host((void **)&L.h_Td, 8 * n)) ||
      (e = host((void **)&L.h_rad, 8 * n * nr)) || (e = host((void **)&L.h_AV, 8 * n * nr)) ||
      (e = host((void **)&L.h_col, 8 * n * nr * 5)) || (e = host((void **)&L.h_ab, 8 * n * L.nspec)) ||
      (e = host((void **)&L.h_tend, 8 * n)) || (e = host((void **)&L.h_status, 4 * n)))
    return pdr::cuda_fail(e, "pdr_server_create: pinned staging");
  if ((e = dev((void **)&L.d_nH, 8 * n)) || (e = dev((void **)&L.d_T, 8 * n)) || (e = dev((void **)&L.d_Td, 8 * n)) ||
      (e = dev((void **)&L.d_rad, 8 * n * nr)) || (e = dev((void **)&L.d_AV, 8 * n * nr)) ||
      (e = dev((void **)&L.d_col, 8 * n * nr * 5)) || (e = dev((void **)&L.d_ab, 8 * n * L.nspec)) ||
      (e = dev((void **)&L.d_tend, 8 * n)) || (e = dev((void **)&L.d_rate, 8 * n * L.nreac)) ||
      (e = dev((void **)&L.d_status, 4 * n)) || (e = dev((void **)&L.d_rstatus, 4 * n)))
    return pdr::cuda_fail(e, "pdr_server_create: device buffers");
  if ((e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking)))
    return pdr::cuda_fail(e, "pdr_server_create: stream");
  return 0;
}

void free_lane(Lane &L) {
  for (void *p : {(void *)L.h_nH, (void *)L.h_T, (void *)L.h_Td, (void *)L.h_rad, (void *)L.h_AV, (void *)L.h_col,
                  (void *)L.h_ab, (void *)L.h_tend, (void *)L.h_status})
    if (p) cudaFreeHost(p);
  for (void *p : {(void *)L.d_nH, (void *)L.d_T, (void *)L.d_Td, (void *)L.d_rad, (void *)L.d_AV, (void *)L.d_col,
                  (void *)L.d_ab, (void *)L.d_tend, (void *)L.d_rate, (void *)L.d_status, (void *)L.d_rstatus})
    if (p) cudaFree(p);
  if (L.solver) pdr_solver_free(L.solver);
  if (L.stream) cudaStreamDestroy(L.stream);
}

// one launch over the packed requests: rates, then the batched solve
int run_batch(pdr_server *s, Lane &L, const std::vector<Req *> &batch) {
  const int nr = s->opts.nrays;
  size_t off = 0;
  for (Req *q : batch) {
    const pdr_serve_request &r = q->r;
    const size_t n = (size_t)r.ncell;
    std::memcpy(L.h_nH + off, r.n_H, 8 * n);
    std::memcpy(L.h_T + off, r.T, 8 * n);
    std::memcpy(L.h_Td + off, r.Tdust, 8 * n);
    std::memcpy(L.h_rad + off * nr, r.rad_surface, 8 * n * nr);
    std::memcpy(L.h_AV + off * nr, r.AV, 8 * n * nr);
    std::memcpy(L.h_col + off * nr * 5, r.column5, 8 * n * nr * 5);
    std::memcpy(L.h_ab + off * L.nspec, r.abundance, 8 * n * L.nspec);
    for (size_t i = 0; i < n; i++) L.h_tend[off + i] = r.t_end_yr;
    off += n;
  }
  const int n = (int)off;
  cudaStream_t st = L.stream;
  cudaError_t e = cudaSuccess;
  auto h2d = [&](void *d, const void *h, size_t bytes) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
  };
  h2d(L.d_nH, L.h_nH, 8 * (size_t)n);
  h2d(L.d_T, L.h_T, 8 * (size_t)n);
  h2d(L.d_Td, L.h_Td, 8 * (size_t)n);
  h2d(L.d_rad, L.h_rad, 8 * (size_t)n * nr);
  h2d(L.d_AV, L.h_AV, 8 * (size_t)n * nr);
  h2d(L.d_col, L.h_col, 8 * (size_t)n * nr * 5);
  h2d(L.d_ab, L.h_ab, 8 * (size_t)n * L.nspec);
  h2d(L.d_tend, L.h_tend, 8 * (size_t)n);
  if (e != cudaSuccess) return pdr::cuda_fail(e, "pdr_server: host-to-device copy");
  int rc = pdr_rates_batched(L.net, &s->phys, n, nr, L.d_T, L.d_Td, L.d_rad, L.d_AV, L.d_col, L.d_rate, L.d_rstatus,
                             st);
  if (rc) return rc;
  rc = pdr_solver_run(L.solver, n, L.d_ab, L.d_rate, L.d_nH, L.d_tend, L.d_status, nullptr, st);
  if (rc) return rc;
  if ((e = cudaMemcpyAsync(L.h_ab, L.d_ab, 8 * (size_t)n * L.nspec, cudaMemcpyDeviceToHost, st)) ||
      (e = cudaMemcpyAsync(L.h_status, L.d_status, 4 * (size_t)n, cudaMemcpyDeviceToHost, st)) ||
      (e = cudaStreamSynchronize(st)))
    return pdr::cuda_fail(e, "pdr_server: device-to-host copy");
  off = 0;
  for (Req *q : batch) {
    const size_t m = (size_t)q->r.ncell;
    std::memcpy(q->r.abundance, L.h_ab + off * L.nspec, 8 * m * L.nspec);
    int res = 0;
    for (size_t i = 0; i < m; i++) {
      if (q->r.status) q->r.status[i] = L.h_status[off + i];
      if (L.h_status[off + i] != 0) res = L.h_status[off + i];
    }
    q->result = res;
    off += m;
  }
  return 0;
}

void lane_loop(pdr_server *s, int li) {
  Lane &L = s->lanes[li];
  cudaSetDevice(s->device);
  for (;;) {
    std::vector<Req *> batch;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->work_cv.wait(lk, [&] { return s->stop || !L.queue.empty(); });
      if (L.queue.empty()) return;   // stopping
      int cells = 0;
      while (!L.queue.empty() && (batch.empty() || cells + L.queue.front()->r.ncell <= s->opts.max_batch_cells)) {
        cells += L.queue.front()->r.ncell;
        batch.push_back(L.queue.front());
        L.queue.pop_front();
      }
      // SM share of this launch: all SMs when the other lanes are idle, else
      // an equal share with the lanes that are running
      if (s->opts.partition_sms && s->lanes.size() > 1)
        pdr_solver_set_max_sms(L.solver, s->running == 0 ? 0 : std::max(1, s->sms / (s->running + 1)));
      s->running++;
    }
    const int rc = run_batch(s, L, batch);
    const Clock::time_point t = Clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->running--;
      for (Req *q : batch) {
        if (rc) q->result = rc;
        q->finished = t;
        q->done = true;
        L.cells += q->r.ncell;
      }
      L.batches++;
    }
    s->done_cv.notify_all();
  }
}

}  // namespace

extern "C" {

void pdr_server_opts_default(pdr_server_opts *o) {
  if (!o) return;
  o->max_batch_cells = 65536;
  o->nrays = 12;
  o->precision = PDR_MIXED;
  o->partition_sms = 1;
}

int pdr_server_create(pdr_net *const *nets, int nnet, const pdr_phys *phys, const pdr_server_opts *opts,
                      pdr_server **out) {
  if (!nets || nnet <= 0 || !phys || !out) {
    pdr::set_error("pdr_server_create: invalid argument");
    return PDR_E_ARG;
  }
  *out = nullptr;
  pdr_server *s = new pdr_server();
  s->phys = *phys;
  pdr_server_opts_default(&s->opts);
  if (opts) s->opts = *opts;
  if (s->opts.max_batch_cells <= 0 || s->opts.nrays <= 0) {
    delete s;
    pdr::set_error("pdr_server_create: invalid options");
    return PDR_E_ARG;
  }
  cudaGetDevice(&s->device);
  cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
  s->lanes.resize(nnet);
  int rc = 0;
  for (int i = 0; i < nnet && !rc; i++) {
    Lane &L = s->lanes[i];
    L.net = nets[i];
    if (!L.net) { rc = PDR_E_ARG; pdr::set_error("pdr_server_create: null network"); break; }
    L.nspec = L.net->host.nspec;
    L.nreac = L.net->host.nreac;
    rc = alloc_lane(s, L);
    if (rc) break;
    pdr_chem_opts o;
    pdr_chem_opts_default(&o);
    o.precision = s->opts.precision;
    rc = pdr_solver_create(L.net, s->opts.max_batch_cells, &o, &L.solver);
  }
  // one warm-up cell per lane: kernel attributes and device tables are set up
  // now, not inside the first request's latency
  for (int i = 0; i < nnet && !rc; i++) {
    Lane &L = s->lanes[i];
    const int nr = s->opts.nrays;
    std::vector<double> ab(L.nspec, 1e-20);
    ab[0] = 1.0;
    pdr_serve_request r{};
    r.network = i; r.ncell = 1; r.t_end_yr = 1.0;
    std::vector<double> nH(1, 1e3), T(1, 50.0), Td(1, 15.0), rad(nr, 1.0), AV(nr, 1.0), col(nr * 5, 1e15);
    r.n_H = nH.data(); r.T = T.data(); r.Tdust = Td.data(); r.rad_surface = rad.data(); r.AV = AV.data();
    r.column5 = col.data(); r.abundance = ab.data(); r.status = nullptr;
    Req q;
    q.r = r;
    rc = run_batch(s, L, {&q});
  }
  if (rc) {
    for (Lane &L : s->lanes) free_lane(L);
    delete s;
    return rc;
  }
  for (int i = 0; i < nnet; i++) s->lanes[i].thread = std::thread(lane_loop, s, i);
  *out = s;
  return 0;
}

int pdr_server_submit(pdr_server *s, const pdr_serve_request *r, long long *ticket) {
  if (!s || !r || !ticket || r->network < 0 || r->network >= (int)s->lanes.size() || r->ncell <= 0 ||
      r->ncell > s->opts.max_batch_cells || !r->n_H || !r->T || !r->Tdust || !r->rad_surface || !r->AV ||
      !r->column5 || !r->abundance || !(r->t_end_yr > 0.0)) {
    pdr::set_error("pdr_server_submit: invalid request (ncell above max_batch_cells?)");
    return PDR_E_ARG;
  }
  Req *q = new Req();
  q->r = *r;
  q->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    *ticket = s->next_ticket++;
    s->reqs[*ticket] = q;
    s->lanes[r->network].queue.push_back(q);
  }
  s->work_cv.notify_all();
  return 0;
}

int pdr_server_wait(pdr_server *s, long long ticket, double *latency_ms) {
  if (!s) return PDR_E_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) {
    pdr::set_error("pdr_server_wait: unknown ticket");
    return PDR_E_ARG;
  }
  Req *q = it->second;
  s->done_cv.wait(lk, [&] { return q->done; });
  if (latency_ms) latency_ms[0] = std::chrono::duration<double, std::milli>(q->finished - q->submitted).count();
  const int res = q->result;
  s->reqs.erase(it);
  delete q;
  return res;
}

int pdr_server_stats(pdr_server *s, int lane, long long *batches, long long *cells) {
  if (!s || lane < 0 || lane >= (int)s->lanes.size()) return PDR_E_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (batches) *batches = s->lanes[lane].batches;
  if (cells) *cells = s->lanes[lane].cells;
  return 0;
}

void pdr_server_free(pdr_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->work_cv.notify_all();
  for (Lane &L : s->lanes)
    if (L.thread.joinable()) L.thread.join();
  for (Lane &L : s->lanes) free_lane(L);
  for (auto &kv : s->reqs) delete kv.second;
  delete s;
}

}  // extern "C"
