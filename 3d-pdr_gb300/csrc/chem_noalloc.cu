// chem_noalloc.cu -- an allocation-free variant of pdr_chem_solve_batched.
//
// Some callers cannot call cudaMalloc: a 3D-PDR rank embedded in a larger
// application whose device memory is owned and capped by another framework's
// pool, or a serving loop that must not allocate once it is running, because a
// cudaMalloc can synchronise the device and stall the streams of other
// requests.  This entry point keeps the solver's only scratch -- the
// work-queue cursors and the list of cells the mixed form re-solves in FP64 --
// in a file-scope device array of fixed size instead of the per-device pool
// that pdr_chem_solve_batched grows with cudaMalloc.  The caller still passes
// every input and output buffer.
//
// Limits and rules:
//   * at most kNoAllocMaxCells cells per call (larger calls are rejected);
//   * the array (about 1 MiB) exists on every GPU that loads the library,
//     until the process exits;
//   * every call on a device shares that one array: calls whose work overlaps
//     on the GPU (different streams, or host threads) race and must be
//     serialised by the caller; each call clears the cursors it needs;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current), so make that first call
//     before any stream capture.
#include <mutex>

#include "pdr_internal.h"

namespace pdr {

int launch_chem_warp(const pdr_net *net, int ncell, double *ab, const double *rate, const double *dens,
                     const double *tend, const pdr_chem_opts &o, int *status, int *stats, int *queue,
                     int *fb_list, int *fb_count, const int *cell_list, const int *total_ptr, bool mixed,
                     int sm_count, cudaStream_t st, const int *sm_limit = nullptr);

namespace {

constexpr int kNoAllocMaxCells = 262144;
constexpr int kCounters = 16;   // [0] queue, [1] redo queue, [2] redo count, rest spare

// [kCounters] cursors, then the FP64 redo list of up to kNoAllocMaxCells cells
static __device__ __align__(256) int g_noalloc_scratch[kCounters + kNoAllocMaxCells];

std::mutex g_noalloc_mu;
int *g_noalloc_addr[64] = {nullptr};

// device address of g_noalloc_scratch on `dev` (the current device)
int noalloc_scratch(int dev, int **out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  int *&p = g_noalloc_addr[dev & 63];
  if (!p) {
    void *addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
    p = static_cast<int *>(addr);
  }
  *out = p;
  return 0;
}

}  // namespace
}  // namespace pdr

using namespace pdr;

extern "C" int pdr_chem_solve_batched_noalloc(const pdr_net *net, int ncell, double *d_abundance,
                                              const double *d_rate, const double *d_density,
                                              const double *d_t_end_yr, const pdr_chem_opts *opts,
                                              int *d_status, int *d_stats, void *stream) {
  if (!net || ncell < 0 || !d_abundance || !d_rate || !d_density || !d_status) {
    set_error("pdr_chem_solve_batched_noalloc: invalid argument");
    return PDR_E_ARG;
  }
  if (ncell > kNoAllocMaxCells) {
    set_error("pdr_chem_solve_batched_noalloc: " + std::to_string(ncell) + " cells exceed the static scratch of " +
              std::to_string(kNoAllocMaxCells) + " cells; use pdr_chem_solve_batched or split the call");
    return PDR_E_ARG;
  }
  if (ncell == 0) return 0;
  pdr_chem_opts o;
  pdr_chem_opts_default(&o);
  if (opts) o = *opts;
  // the same option checks as pdr_chem_solve_batched
  int rc = check_opts(net, o, "pdr_chem_solve_batched_noalloc");
  if (rc) return rc;
  if (!uses_warp_path(net, o)) {
    // the block integrator needs per-block scratch that scales with the grid
    set_error("pdr_chem_solve_batched_noalloc: only the warp integrator (networks of 32 ODE species) "
              "runs without allocation");
    return PDR_E_NET;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  int *scratch = nullptr;
  rc = noalloc_scratch(dev, &scratch);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // the array keeps the previous call's contents: clear the cursors and the redo count
  e = cudaMemsetAsync(scratch, 0, kCounters * sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(no-alloc scratch)");
  int *queue = scratch + 0, *redo_queue = scratch + 1, *redo_count = scratch + 2, *redo = scratch + kCounters;
  const bool mixed = (o.precision == PDR_MIXED);
  const int sm_use = eff_sms(o, sms);   // opts.max_sms, as pdr_chem_solve_batched applies it
  rc = launch_chem_warp(net, ncell, d_abundance, d_rate, d_density, d_t_end_yr, o, d_status, d_stats, queue,
                        redo, redo_count, nullptr, nullptr, mixed, sm_use, st);
  if (rc) return rc;
  if (mixed)
    rc = launch_chem_warp(net, ncell, d_abundance, d_rate, d_density, d_t_end_yr, o, d_status, d_stats,
                          redo_queue, nullptr, nullptr, redo, redo_count, false, sm_use, st);
  return rc;
}
