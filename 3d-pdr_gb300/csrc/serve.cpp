// serve.cpp -- a serving loop for batched chemistry requests.
//
// There is no counterpart in the reference: it is the service around the
// chemistry path that a client calls with blocks of cells (physical
// conditions plus initial abundances) and gets abundances back.  Design:
//   * one lane per network, each with slots_per_lane launch slots: a worker
//     thread, a CUDA stream, a solver instance (pdr_solver, own scratch) and
//     pinned staging plus device buffers for max_batch_cells cells, all
//     allocated when the server is created -- nothing is allocated while
//     serving;
//   * continuous batching at slot level: a free slot takes every queued
//     request of its network that fits its buffers, in arrival order, and runs
//     them as one launch (rates, then the batched solve with per-cell end
//     times); a request that arrives while other launches are on the GPU
//     starts at once on another free slot, without waiting for them to drain;
//   * SM sharing: persistent launches would hold their SMs until their last
//     cell, so a new launch is sized for an equal share of the SMs with the
//     launches in flight, and those are told to shrink to that share
//     (pdr_solver_limit_sms, a 4-byte copy on a control stream): their blocks
//     beyond it stop taking cells at the next cell boundary and the hardware
//     hands those SMs to the new launch.  A persistent launch cannot widen its
//     grid again, so a batch is solved in chunks of about sixteen waves, each
//     launched with the share of the moment: once the newcomers finish, the
//     next chunk takes their SMs back;
//   * admission by device-memory footprint: requests whose bytes (inputs, rate
//     constants, outputs per cell) would push the admitted-and-unfinished total
//     over the budget are refused with PDR_E_BUSY.
// Each cell is integrated independently, so a request's results do not depend
// on what it was batched or overlapped with.
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

#include "pdr_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  pdr_serve_request r;
  Clock::time_point submitted, finished;
  double bytes = 0.0;
  bool done = false;
  int result = 0;
};

struct Slot {
  pdr_solver *solver = nullptr;
  cudaStream_t stream = nullptr;
  // pinned staging and device buffers, max_batch_cells cells each
  double *h_nH = nullptr, *h_T = nullptr, *h_Td = nullptr, *h_rad = nullptr, *h_AV = nullptr, *h_col = nullptr,
         *h_ab = nullptr, *h_tend = nullptr;
  int *h_status = nullptr;
  double *d_nH = nullptr, *d_T = nullptr, *d_Td = nullptr, *d_rad = nullptr, *d_AV = nullptr, *d_col = nullptr,
         *d_ab = nullptr, *d_tend = nullptr, *d_rate = nullptr;
  int *d_status = nullptr, *d_rstatus = nullptr;
  std::thread thread;
  bool running = false;
  // SMs this slot's launch may keep: written under the server lock, read by
  // the slot's own thread between chunks without it
  std::atomic<int> share{0};
};

struct Lane {
  pdr_net *net = nullptr;
  int nspec = 0, nreac = 0;
  double cell_bytes = 0.0;
  int cells_per_sm = 0;   // cells one SM holds at once (16 warps, or 2 blocks of the block integrator)
  std::vector<std::unique_ptr<Slot>> slots;
  std::deque<Req *> queue;
  long long batches = 0, cells = 0;
};

}  // namespace

struct pdr_server {
  pdr_phys phys;
  pdr_server_opts opts;
  std::deque<Lane> lanes;   // (a deque: a Lane is not copyable)
  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  bool stop = false;
  long long next_ticket = 1;
  std::unordered_map<long long, Req *> reqs;
  int device = 0, sms = 0;
  int running = 0;            // launches in flight
  double admitted_bytes = 0.0, budget_bytes = 0.0;
  cudaStream_t control = nullptr;   // the SM-allowance copies
};

namespace {

int alloc_slot(pdr_server *s, Lane &L, Slot &S) {
  const size_t n = (size_t)s->opts.max_batch_cells, nr = (size_t)s->opts.nrays;
  auto dev = [&](void **p, size_t bytes) { return cudaMalloc(p, bytes); };
  auto host = [&](void **p, size_t bytes) { return cudaHostAlloc(p, bytes, cudaHostAllocDefault); };
  cudaError_t e = cudaSuccess;
  if ((e = host((void **)&S.h_nH, 8 * n)) || (e = host((void **)&S.h_T, 8 * n)) || (e = host((void **)&S.h_Td, 8 * n)) ||
      (e = host((void **)&S.h_rad, 8 * n * nr)) || (e = host((void **)&S.h_AV, 8 * n * nr)) ||
      (e = host((void **)&S.h_col, 8 * n * nr * 5)) || (e = host((void **)&S.h_ab, 8 * n * L.nspec)) ||
      (e = host((void **)&S.h_tend, 8 * n)) || (e = host((void **)&S.h_status, 4 * n)))
    return pdr::cuda_fail(e, "pdr_server_create: pinned staging");
  if ((e = dev((void **)&S.d_nH, 8 * n)) || (e = dev((void **)&S.d_T, 8 * n)) || (e = dev((void **)&S.d_Td, 8 * n)) ||
      (e = dev((void **)&S.d_rad, 8 * n * nr)) || (e = dev((void **)&S.d_AV, 8 * n * nr)) ||
      (e = dev((void **)&S.d_col, 8 * n * nr * 5)) || (e = dev((void **)&S.d_ab, 8 * n * L.nspec)) ||
      (e = dev((void **)&S.d_tend, 8 * n)) || (e = dev((void **)&S.d_rate, 8 * n * L.nreac)) ||
      (e = dev((void **)&S.d_status, 4 * n)) || (e = dev((void **)&S.d_rstatus, 4 * n)))
    return pdr::cuda_fail(e, "pdr_server_create: device buffers");
  if ((e = cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking)))
    return pdr::cuda_fail(e, "pdr_server_create: stream");
  pdr_chem_opts o;
  pdr_chem_opts_default(&o);
  o.precision = s->opts.precision;
  return pdr_solver_create(L.net, s->opts.max_batch_cells, &o, &S.solver);
}

void free_slot(Slot &S) {
  for (void *p : {(void *)S.h_nH, (void *)S.h_T, (void *)S.h_Td, (void *)S.h_rad, (void *)S.h_AV, (void *)S.h_col,
                  (void *)S.h_ab, (void *)S.h_tend, (void *)S.h_status})
    if (p) cudaFreeHost(p);
  for (void *p : {(void *)S.d_nH, (void *)S.d_T, (void *)S.d_Td, (void *)S.d_rad, (void *)S.d_AV, (void *)S.d_col,
                  (void *)S.d_ab, (void *)S.d_tend, (void *)S.d_rate, (void *)S.d_status, (void *)S.d_rstatus})
    if (p) cudaFree(p);
  if (S.solver) pdr_solver_free(S.solver);
  if (S.stream) cudaStreamDestroy(S.stream);
}

int claim_sms(pdr_server *s, Slot &me, bool counted = false);

// the packed requests: rates, then the batched solve
int run_batch(pdr_server *s, Lane &L, Slot &S, const std::vector<Req *> &batch) {
  const int nr = s->opts.nrays;
  size_t off = 0;
  for (Req *q : batch) {
    const pdr_serve_request &r = q->r;
    const size_t n = (size_t)r.ncell;
    std::memcpy(S.h_nH + off, r.n_H, 8 * n);
    std::memcpy(S.h_T + off, r.T, 8 * n);
    std::memcpy(S.h_Td + off, r.Tdust, 8 * n);
    std::memcpy(S.h_rad + off * nr, r.rad_surface, 8 * n * nr);
    std::memcpy(S.h_AV + off * nr, r.AV, 8 * n * nr);
    std::memcpy(S.h_col + off * nr * 5, r.column5, 8 * n * nr * 5);
    std::memcpy(S.h_ab + off * L.nspec, r.abundance, 8 * n * L.nspec);
    for (size_t i = 0; i < n; i++) S.h_tend[off + i] = r.t_end_yr;
    off += n;
  }
  const int n = (int)off;
  cudaStream_t st = S.stream;
  cudaError_t e = cudaSuccess;
  auto h2d = [&](void *d, const void *h, size_t bytes) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
  };
  h2d(S.d_nH, S.h_nH, 8 * (size_t)n);
  h2d(S.d_T, S.h_T, 8 * (size_t)n);
  h2d(S.d_Td, S.h_Td, 8 * (size_t)n);
  h2d(S.d_rad, S.h_rad, 8 * (size_t)n * nr);
  h2d(S.d_AV, S.h_AV, 8 * (size_t)n * nr);
  h2d(S.d_col, S.h_col, 8 * (size_t)n * nr * 5);
  h2d(S.d_ab, S.h_ab, 8 * (size_t)n * L.nspec);
  h2d(S.d_tend, S.h_tend, 8 * (size_t)n);
  if (e != cudaSuccess) return pdr::cuda_fail(e, "pdr_server: host-to-device copy");
  int rc = pdr_rates_batched(L.net, &s->phys, n, nr, S.d_T, S.d_Td, S.d_rad, S.d_AV, S.d_col, S.d_rate, S.d_rstatus,
                             st);
  if (rc) return rc;
  // the solve in chunks of about sixteen waves at the slot's share
  for (int c0 = 0; c0 < n && !rc;) {
    int m = n - c0;
    if (c0 > 0 && s->opts.partition_sms) {
      std::lock_guard<std::mutex> lk(s->mu);
      const int share = claim_sms(s, S, true);
      pdr_solver_set_max_sms(S.solver, share);
    }
    // (a slot outside slot_loop -- the warm-up at creation -- has no share yet:
    // it counts as the whole device; every chunk holds at least one cell)
    const int sh = S.share.load(std::memory_order_relaxed);
    if (s->opts.partition_sms) m = std::min(m, std::max(1, 16 * (sh > 0 ? sh : s->sms) * L.cells_per_sm));
    rc = pdr_solver_run(S.solver, m, S.d_ab + (size_t)c0 * L.nspec, S.d_rate + (size_t)c0 * L.nreac, S.d_nH + c0,
                        S.d_tend + c0, S.d_status + c0, nullptr, st);
    c0 += m;
  }
  if (rc) return rc;
  if ((e = cudaMemcpyAsync(S.h_ab, S.d_ab, 8 * (size_t)n * L.nspec, cudaMemcpyDeviceToHost, st)) ||
      (e = cudaMemcpyAsync(S.h_status, S.d_status, 4 * (size_t)n, cudaMemcpyDeviceToHost, st)) ||
      (e = cudaStreamSynchronize(st)))
    return pdr::cuda_fail(e, "pdr_server: device-to-host copy");
  off = 0;
  for (Req *q : batch) {
    const size_t m = (size_t)q->r.ncell;
    std::memcpy(q->r.abundance, S.h_ab + off * L.nspec, 8 * m * L.nspec);
    int res = 0;
    for (size_t i = 0; i < m; i++) {
      if (q->r.status) q->r.status[i] = S.h_status[off + i];
      if (S.h_status[off + i] != 0) res = S.h_status[off + i];
    }
    q->result = res;
    off += m;
  }
  return 0;
}

// Called with the server lock held: the SMs of a launch that is about to
// start, and the shrinking of the launches in flight to the same share.
// `counted`: this slot is already among the running ones (a later chunk).
int claim_sms(pdr_server *s, Slot &me, bool counted) {
  if (!s->opts.partition_sms) return 0;
  const int share = std::max(1, s->sms / std::max(1, s->running + (counted ? 0 : 1)));
  for (Lane &L : s->lanes)
    for (auto &sp : L.slots) {
      Slot &o = *sp;
      if (&o == &me || !o.running || o.share.load(std::memory_order_relaxed) <= share) continue;
      o.share.store(share, std::memory_order_relaxed);
      pdr_solver_limit_sms(o.solver, share, s->control);
    }
  me.share.store(share, std::memory_order_relaxed);
  return share;
}

void slot_loop(pdr_server *s, int li, int si) {
  Lane &L = s->lanes[li];
  Slot &S = *L.slots[si];
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
      const int share = claim_sms(s, S);
      pdr_solver_set_max_sms(S.solver, share);
      S.running = true;
      s->running++;
    }
    const int rc = run_batch(s, L, S, batch);
    const Clock::time_point t = Clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->running--;
      S.running = false;
      for (Req *q : batch) {
        if (rc) q->result = rc;
        q->finished = t;
        q->done = true;
        s->admitted_bytes -= q->bytes;
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
  o->slots_per_lane = 4;
  o->hbm_budget_mb = 0.0;
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
  if (s->opts.max_batch_cells <= 0 || s->opts.nrays <= 0 || s->opts.slots_per_lane < 1 ||
      s->opts.slots_per_lane > 64 || !(s->opts.hbm_budget_mb >= 0.0)) {
    delete s;
    pdr::set_error("pdr_server_create: invalid options");
    return PDR_E_ARG;
  }
  cudaGetDevice(&s->device);
  cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
  s->lanes.resize(nnet);
  int rc = 0;
  cudaError_t e = cudaStreamCreateWithFlags(&s->control, cudaStreamNonBlocking);
  if (e != cudaSuccess) rc = pdr::cuda_fail(e, "pdr_server_create: control stream");
  double capacity = 0.0;
  const double nr = s->opts.nrays;
  for (int i = 0; i < nnet && !rc; i++) {
    Lane &L = s->lanes[i];
    L.net = nets[i];
    if (!L.net) { rc = PDR_E_ARG; pdr::set_error("pdr_server_create: null network"); break; }
    L.nspec = L.net->host.nspec;
    L.nreac = L.net->host.nreac;
    // device bytes per cell: n_H, T, T_dust, end time, per-ray field, A_V and
    // five columns, abundances, rate constants, two status words
    L.cell_bytes = 8.0 * (4 + 7 * nr + L.nspec + L.nreac) + 8.0;
    {
      pdr_chem_opts o;
      pdr_chem_opts_default(&o);
      o.precision = s->opts.precision;
      L.cells_per_sm = pdr::uses_warp_path(L.net, o) ? 16 : 2;
    }
    for (int k = 0; k < s->opts.slots_per_lane && !rc; k++) {
      L.slots.emplace_back(new Slot());
      rc = alloc_slot(s, L, *L.slots.back());
    }
    capacity += L.cell_bytes * s->opts.max_batch_cells * s->opts.slots_per_lane;
  }
  s->budget_bytes = s->opts.hbm_budget_mb > 0.0 ? s->opts.hbm_budget_mb * 1048576.0 : capacity;
  // one warm-up cell per slot: kernel attributes and device tables are set up
  // now, not inside the first request's latency
  for (int i = 0; i < nnet && !rc; i++) {
    Lane &L = s->lanes[i];
    const int nrays = s->opts.nrays;
    for (auto &sp : L.slots) {
      if (rc) break;
      std::vector<double> ab(L.nspec, 1e-20);
      ab[0] = 1.0;
      pdr_serve_request r{};
      r.network = i; r.ncell = 1; r.t_end_yr = 1.0;
      std::vector<double> nH(1, 1e3), T(1, 50.0), Td(1, 15.0), rad(nrays, 1.0), AV(nrays, 1.0), col(nrays * 5, 1e15);
      r.n_H = nH.data(); r.T = T.data(); r.Tdust = Td.data(); r.rad_surface = rad.data(); r.AV = AV.data();
      r.column5 = col.data(); r.abundance = ab.data(); r.status = nullptr;
      Req q;
      q.r = r;
      rc = run_batch(s, L, *sp, {&q});
    }
  }
  if (rc) {
    for (Lane &L : s->lanes)
      for (auto &sp : L.slots) free_slot(*sp);
    if (s->control) cudaStreamDestroy(s->control);
    delete s;
    return rc;
  }
  for (int i = 0; i < nnet; i++)
    for (int k = 0; k < (int)s->lanes[i].slots.size(); k++)
      s->lanes[i].slots[k]->thread = std::thread(slot_loop, s, i, k);
  *out = s;
  return 0;
}

int pdr_server_footprint(pdr_server *s, int network, int ncell, double *bytes) {
  if (!s || !bytes || network < 0 || network >= (int)s->lanes.size() || ncell < 0) {
    pdr::set_error("pdr_server_footprint: invalid argument");
    return PDR_E_ARG;
  }
  *bytes = s->lanes[network].cell_bytes * ncell;
  return 0;
}

int pdr_server_submit(pdr_server *s, const pdr_serve_request *r, long long *ticket) {
  if (!s || !r || !ticket || r->network < 0 || r->network >= (int)s->lanes.size() || r->ncell <= 0 ||
      r->ncell > s->opts.max_batch_cells || !r->n_H || !r->T || !r->Tdust || !r->rad_surface || !r->AV ||
      !r->column5 || !r->abundance || !(r->t_end_yr > 0.0)) {
    pdr::set_error("pdr_server_submit: invalid request (ncell above max_batch_cells?)");
    return PDR_E_ARG;
  }
  const double bytes = s->lanes[r->network].cell_bytes * r->ncell;
  Req *q = new Req();
  q->r = *r;
  q->bytes = bytes;
  q->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    // admission by footprint; a request alone above the budget is still
    // admitted when nothing else is, so that it can ever run
    if (s->admitted_bytes > 0.0 && s->admitted_bytes + bytes > s->budget_bytes) {
      delete q;
      pdr::set_error("pdr_server_submit: the request would exceed the device-memory budget; retry later");
      return PDR_E_BUSY;
    }
    s->admitted_bytes += bytes;
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
    for (auto &sp : L.slots)
      if (sp->thread.joinable()) sp->thread.join();
  for (Lane &L : s->lanes)
    for (auto &sp : L.slots) free_slot(*sp);
  for (auto &kv : s->reqs) delete kv.second;
  if (s->control) cudaStreamDestroy(s->control);
  delete s;
}

}  // extern "C"
