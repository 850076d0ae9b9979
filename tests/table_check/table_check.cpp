// Host check of the chemistry tables that pdr_net.cpp builds for the two
// integrators (warp tables, 32 lanes; block tables, G lanes): the device
// allocations are redirected to host memory, then the table-driven RHS (the
// pair-operand terms with merged rate constants, the balanced chunks and
// their partial sums) and the term-parallel Jacobian assembly are replayed on
// the CPU the way the kernels run them and compared with a direct evaluation
// from the stoichiometry on seeded states.
// Usage: table_check <data dir> <network>...; exit 0 when every check holds.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

static cudaError_t host_malloc(void **p, size_t n) {
  *p = std::malloc(n ? n : 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
static cudaError_t host_copy(void *d, const void *s, size_t n, cudaMemcpyKind) {
  std::memcpy(d, s, n);
  return cudaSuccess;
}
#define cudaMalloc(p, n) host_malloc((void **)(p), (n))
#define cudaMemcpy(d, s, n, k) host_copy((d), (s), (n), (k))
#include "../../3d-pdr_gb300/csrc/pdr_net.cpp"
#undef cudaMalloc
#undef cudaMemcpy

#include <cmath>
#include <cstdio>
#include <random>

namespace pdr {
int cuda_fail(cudaError_t, const char *) { return -1; }
void set_error(const std::string &) {}
}  // namespace pdr

using namespace pdr;

struct Direct {
  std::vector<double> f, scale, J, jscale;   // J: [neq][neq+1]
};

// f and J from the stoichiometry: phi_r = kn_r x_a x_b, f_i = sum nu phi_r,
// J_ij = sum nu dphi_r/dx_j (column neq: x_e), the term-magnitude sums as scales
static Direct direct(const HostNet &h, const std::vector<Term> &terms, const std::vector<double> &kn,
                     const std::vector<double> &xs) {
  const int n = h.neq, ONE = n + 1;
  Direct d;
  d.f.assign(n, 0.0);
  d.scale.assign(n, 0.0);
  d.J.assign((size_t)n * (n + 1), 0.0);
  d.jscale.assign(n, 0.0);
  for (const Term &t : terms) {
    const int r = t.r, a = h.ra[r], b = (h.ode_kind[r] == ODE_BI) ? h.rb[r] : ONE;
    const double phi = kn[r] * xs[a] * xs[b];
    d.f[t.i] += t.nu * phi;
    d.scale[t.i] += std::fabs(t.nu * phi);
    const double da = t.nu * kn[r] * xs[b], db = t.nu * kn[r] * xs[a];
    d.J[(size_t)t.i * (n + 1) + a] += da;
    d.jscale[t.i] += std::fabs(da);
    if (b != ONE) {
      d.J[(size_t)t.i * (n + 1) + b] += db;
      d.jscale[t.i] += std::fabs(db);
    }
  }
  return d;
}

static int check_tables(const HostNet &h, const std::vector<Term> &terms, const WarpTables &T, const char *which,
                        std::mt19937_64 &rng) {
  const int n = h.neq, G = T.lanes, ONE = n + 1;
  int bad = 0;
  std::uniform_real_distribution<double> U(0.0, 1.0);
  for (int trial = 0; trial < 8; trial++) {
    // state: abundances log-uniform 1e-20..1, rates log-uniform 1e-20..1e-8, n_H 1e2..1e5
    std::vector<double> x(n), rate(h.nreac);
    for (auto &v : x) v = std::pow(10.0, -20.0 * U(rng));
    for (auto &v : rate) v = std::pow(10.0, -8.0 - 12.0 * U(rng));
    const double nH = std::pow(10.0, 2.0 + 3.0 * U(rng));
    double xe = 0.0;
    for (int j = 0; j < n; j++) xe += h.xe[j] * x[j];
    std::vector<double> xs(x);
    xs.push_back(xe);    // slot n: x_e
    xs.push_back(1.0);   // slot n+1: the constant
    // per-cell rate constants as the kernels load them
    std::vector<double> kn(T.nkn + 1, 0.0);
    for (int r = 0; r < T.nreac; r++) kn[r] = rate[r] * (T.nh_mask[r] != 0.0 ? nH : 1.0);
    for (int e = 0; e < T.nkext; e++) {
      double k = 0.0;
      for (int q = T.kext_ptr[e]; q < T.kext_ptr[e + 1]; q++) k = std::fma((double)T.kext_rn[q].y, kn[T.kext_rn[q].x], k);
      kn[T.nreac + e] = k;
    }
    const Direct d = direct(h, terms, kn, xs);
    // the table RHS: operands, terms by chunk with flushes, partial sums per species
    std::vector<double> P(T.nop);
    for (int j = 0; j < n + 2; j++) P[j] = xs[j];
    for (int p = 0; p < T.npairs; p++) P[n + 2 + p] = P[T.pairs[p].x] * P[T.pairs[p].y];
    std::vector<double> part(T.nparts + 1, 0.0);
    for (int l = 0; l < G; l++) {
      double s = 0.0;
      for (int t = 0; t < T.rhs_len; t++) {
        const int2 dd = T.rhs_t[t * G + l];
        const int ki = dd.x & 0xffff, op = dd.y & 0x7fffffff, fl = (int)((unsigned)dd.x >> 16) - 1;
        if (ki > T.nkn || op >= T.nop || fl >= T.nparts) return 1000;
        const double k = (dd.y & (int)0x80000000u) ? -kn[ki] : kn[ki];
        s = std::fma(k, P[op], s);
        if (fl >= 0) { part[fl] = s; s = 0.0; }
      }
    }
    for (int i = 0; i < n; i++) {
      double f = 0.0;
      for (int k = 0; k < T.plist_len; k++) f += part[T.plist[k * G + i]];
      if (std::fabs(f - d.f[i]) > 1e-14 * d.scale[i] + 1e-300) {
        if (bad < 5) std::printf("%s RHS species %d: %.17g vs %.17g (scale %.3g)\n", which, i, f, d.f[i], d.scale[i]);
        bad++;
      }
    }
    // the term-parallel Jacobian assembly (FP64 form)
    std::vector<double> Da(T.nreac), Db(T.nreac);
    for (int r = 0; r < T.nreac; r++) {
      const int2 ab = T.rab[r];
      Da[r] = kn[r] * xs[ab.y];
      Db[r] = (ab.y == ONE) ? 0.0 : kn[r] * xs[ab.x];
    }
    std::vector<double> J((size_t)n * (n + 1), 0.0), slots(2 * G + 8 * n + 64, 0.0);
    for (int c = 0; c < G; c++) {
      double s = 0.0;
      for (int t = 0; t < T.hlen; t++) {
        const int2 xy = T.h_xy[t * G + c];
        const int x = xy.x, y = xy.y, r = x & 0xffff, kind = (x >> 17) & 3;
        const double nu = T.h_nu[t * G + c];
        if ((double)(x >> 19) != nu || kind == 3 || r >= T.nreac) return 1001;
        s = std::fma(nu, (x & 0x10000) ? Db[r] : Da[r], s);
        if (kind == 1) {
          const int row = y & 0xff, col = (y >> 8) & 0xff;
          if (row >= n || col > n) return 1002;
          J[(size_t)row * (n + 1) + col] = s;
          s = 0.0;
        } else if (kind == 2) {
          if ((y >> 16) >= (int)slots.size()) return 1003;
          slots[y >> 16] = s;
          s = 0.0;
        }
      }
    }
    for (int b = 0; b < T.nbnd; b++) {
      const int tt = T.bnd_t[b], ss = T.bnd_s[b];
      double acc = 0.0;
      for (int q = ss & 0xffff; q < (ss >> 16); q++) acc += slots[q];
      J[(size_t)(tt & 0xff) * (n + 1) + ((tt >> 8) & 0xff)] = acc;
    }
    for (int i = 0; i < n; i++)
      for (int j = 0; j <= n; j++) {
        const double g = J[(size_t)i * (n + 1) + j], w = d.J[(size_t)i * (n + 1) + j];
        if (std::fabs(g - w) > 1e-14 * d.jscale[i] + 1e-300) {
          if (bad < 5) std::printf("%s J(%d,%d): %.17g vs %.17g\n", which, i, j, g, w);
          bad++;
        }
      }
  }
  return bad;
}

static int check_network(const std::string &dir, const std::string &name) {
  pdr_net net;
  std::string err = load_network((dir + "/species_" + name + ".d").c_str(), (dir + "/rates_" + name + ".d").c_str(),
                                 (dir + "/layout_" + name + ".d").c_str(), net.host);
  if (!err.empty()) { std::printf("%s: load: %s\n", name.c_str(), err.c_str()); return 1; }
  const int rc = build_device_tables(&net);
  if (rc != 0) { std::printf("%s: build_device_tables %d\n", name.c_str(), rc); return 1; }
  const auto terms = stoichiometry(net.host);
  std::mt19937_64 rng(20261204u);
  int bad = 0;
  if (net.host.neq <= kWarp) {
    if (!net.warp_ok) { std::printf("%s: no warp tables\n", name.c_str()); return 1; }
    bad += check_tables(net.host, terms, net.warp, "warp", rng);
  }
  if (!net.cta_ok) { std::printf("%s: no block tables\n", name.c_str()); return 1; }
  bad += check_tables(net.host, terms, net.cta, "block", rng);
  std::printf("%s: neq %d nreac %d warp %s (rhs_len %d) block lanes %d (rhs_len %d, hlen %d): %s\n", name.c_str(),
              net.host.neq, net.host.nreac, net.warp_ok ? "yes" : "no", net.warp.rhs_len, net.cta.lanes,
              net.cta.rhs_len, net.cta.hlen, bad ? "MISMATCH" : "ok");
  return bad;
}

int main(int argc, char **argv) {
  if (argc < 3) { std::printf("usage: table_check <data dir> <network>...\n"); return 2; }
  int bad = 0;
  for (int i = 2; i < argc; i++) bad += check_network(argv[1], argv[i]);
  return bad ? 1 : 0;
}
