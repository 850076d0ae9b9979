// Host check of the block integrator's sparse bordered Newton matrix plan
// (pdr_net.cpp sparse_plan): for each network given on the command line,
//   * the plan's structure: leaf rows in dependency-level order, the fill
//     closed (every update of the elimination lands on a stored entry), every
//     Jacobian entry and diagonal located, the x_e row's entries located;
//   * its numbers: random matrices over the network's Jacobian pattern,
//     factorised and solved the way the device does it (leaf rows by level
//     without pivoting, the trailing rows' leaf part, the dense block with
//     partial pivoting, then the substitutions), in FP64, against a dense
//     Gaussian elimination of the chain-rule system I - gamma (J0 + d c^T).
// Usage: sparse_plan_check <data dir> <network>...; exit 0 when every check holds.
#include "../../3d-pdr_gb300/csrc/pdr_net.cpp"

#include <random>

namespace pdr {
int cuda_fail(cudaError_t, const char *) { return -1; }
void set_error(const std::string &) {}
}  // namespace pdr

using namespace pdr;

static int check_network(const std::string &dir, const std::string &name) {
  HostNet h;
  std::string err = load_network((dir + "/species_" + name + ".d").c_str(), (dir + "/rates_" + name + ".d").c_str(),
                                 (dir + "/layout_" + name + ".d").c_str(), h);
  if (!err.empty()) { std::printf("%s: load: %s\n", name.c_str(), err.c_str()); return 1; }
  const int n = h.neq, ONE = n + 1;
  // the Jacobian entries the term-parallel assembly stores (columns: slots and x_e)
  std::vector<std::pair<int, int>> ent;
  for (auto &t : stoichiometry(h)) {
    if (h.ode_kind[t.r] == ODE_XRAY) continue;
    const int a = h.ra[t.r], b = (h.ode_kind[t.r] == ODE_BI) ? h.rb[t.r] : ONE;
    if (a <= n) ent.push_back({t.i, a});
    if (b <= n) ent.push_back({t.i, b});
  }
  SparsePlan sp;
  const int G = std::max(64, (n + 31) / 32 * 32);
  if (!sparse_plan(n, ent, h.xe, G, sp)) { std::printf("%s: no plan\n", name.c_str()); return 1; }
  const int N = sp.N, a = sp.a, m = sp.m, ldb = sp.ldb;
  int bad = 0;
  // structure
  if (N != n + 1 || a + m != N || (int)sp.a_ptr.size() != a + 1 || (int)sp.b_ptr.size() != m + 1) bad++;
  for (int i = 0; i < N; i++)
    if (sp.perm[sp.iperm[i]] != i) bad++;
  std::vector<int> lev(a, 0);
  for (int l = 0; l + 1 < (int)sp.lev_ptr.size(); l++)
    for (int r = sp.lev_ptr[l]; r < sp.lev_ptr[l + 1]; r++) lev[r] = l;
  for (int r = 0; r < a; r++) {
    if (sp.a_col[sp.a_diag[r]] != r) bad++;
    for (int p = sp.a_ptr[r]; p < sp.a_ptr[r + 1]; p++) {
      if (p > sp.a_ptr[r] && sp.a_col[p] <= sp.a_col[p - 1]) bad++;   // ascending
      if (p < sp.a_diag[r] && lev[sp.a_col[p]] >= lev[r]) bad++;      // deps on earlier levels
    }
    for (int p = sp.a_ptr[r]; p < sp.a_diag[r]; p++) {                // closed fill
      const int k = sp.a_col[p];
      for (int u = sp.a_diag[k] + 1; u < sp.a_ptr[k + 1]; u++)
        if (sp.loc(r, sp.a_col[u]) < 0) bad++;
    }
  }
  for (int t = 0; t < m; t++)
    for (int p = sp.b_ptr[t]; p < sp.b_ptr[t + 1]; p++) {
      const int k = sp.b_col[p];
      for (int u = sp.a_diag[k] + 1; u < sp.a_ptr[k + 1]; u++)
        if (sp.loc(a + t, sp.a_col[u]) < 0) bad++;
    }
  std::vector<int> ul(a, -1);
  for (int l = 0; l + 1 < (int)sp.ul_ptr.size(); l++)
    for (int i = sp.ul_ptr[l]; i < sp.ul_ptr[l + 1]; i++) ul[sp.ul_rows[i]] = l;
  for (int r = 0; r < a; r++) {
    if (ul[r] < 0) bad++;
    for (int p = sp.a_diag[r] + 1; p < sp.a_ptr[r + 1]; p++)
      if (sp.a_col[p] < a && ul[sp.a_col[p]] >= ul[r]) bad++;
  }
  for (auto &e : ent)
    if (sp.loc(sp.iperm[e.first], sp.iperm[e.second]) < 0) bad++;
  for (int j = 0; j < n; j++)
    if ((h.xe[j] != 0) != (sp.e_loc[j] >= 0)) bad++;
  if (bad) { std::printf("%s: %d structural faults\n", name.c_str(), bad); return 1; }
  // numbers
  std::mt19937_64 rng(5);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  double worst = 0.0;
  for (int trial = 0; trial < 20; trial++) {
    std::vector<double> J((size_t)n * (n + 1), 0.0);
    for (auto &e : ent) J[(size_t)e.first * (n + 1) + e.second] = U(rng) * std::pow(10.0, U(rng));
    const double gam = std::pow(10.0, 2.0 * U(rng) - 1.0);
    std::vector<double> S(sp.total, 0.0);
    for (int i = 0; i < n; i++)
      for (int j = 0; j <= n; j++)
        if (J[(size_t)i * (n + 1) + j] != 0.0) S[sp.loc(sp.iperm[i], sp.iperm[j])] = -gam * J[(size_t)i * (n + 1) + j];
    for (int i = 0; i < N; i++) S[sp.diag_loc[i]] += 1.0;
    for (int j = 0; j < n; j++)
      if (sp.e_loc[j] >= 0) S[sp.e_loc[j]] = -h.xe[j];
    std::vector<double> dinv(std::max(a, 1)), w(N);
    for (int r = 0; r < a; r++) {   // rows are in level order
      for (int p = sp.a_ptr[r]; p < sp.a_ptr[r + 1]; p++) w[sp.a_col[p]] = S[p];
      for (int p = sp.a_ptr[r]; p < sp.a_diag[r]; p++) {
        const int k = sp.a_col[p];
        const double lk = w[k] * dinv[k];
        for (int u = sp.a_diag[k] + 1; u < sp.a_ptr[k + 1]; u++) w[sp.a_col[u]] -= lk * S[u];
        S[p] = lk;
      }
      for (int p = sp.a_diag[r]; p < sp.a_ptr[r + 1]; p++) S[p] = w[sp.a_col[p]];
      dinv[r] = 1.0 / w[r];
    }
    double *D = S.data() + sp.off_d;
    for (int t = 0; t < m; t++) {
      for (int p = sp.b_ptr[t]; p < sp.b_ptr[t + 1]; p++) w[sp.b_col[p]] = S[sp.off_ba + p];
      for (int p = sp.b_ptr[t]; p < sp.b_ptr[t + 1]; p++) {
        const int k = sp.b_col[p];
        const double lk = w[k] * dinv[k];
        for (int u = sp.a_diag[k] + 1; u < sp.a_ptr[k + 1]; u++) {
          const int j = sp.a_col[u];
          if (j < a) w[j] -= lk * S[u];
          else D[(size_t)(j - a) * ldb + t] -= lk * S[u];
        }
        S[sp.off_ba + p] = lk;
      }
    }
    auto Mx = [&](int i, int j) -> double & { return D[(size_t)j * ldb + i]; };
    std::vector<int> perm(m), step(m, -1);
    for (int k = 0; k < m; k++) {
      int p = -1;
      double best = -1.0;
      for (int i = 0; i < m; i++)
        if (step[i] < 0 && std::fabs(Mx(i, k)) > best) { best = std::fabs(Mx(i, k)); p = i; }
      perm[k] = p;
      step[p] = k;
      for (int i = 0; i < m; i++)
        if (step[i] < 0) {
          const double l = Mx(i, k) / Mx(p, k);
          Mx(i, k) = l;
          for (int j = k + 1; j < m; j++) Mx(i, j) -= l * Mx(p, j);
        }
    }
    std::vector<double> b(n), yv(N);
    for (int i = 0; i < n; i++) b[i] = U(rng);
    for (int i = 0; i < n; i++) yv[sp.iperm[i]] = b[i];
    yv[sp.iperm[n]] = 0.0;
    for (int r = 0; r < a; r++)
      for (int p = sp.a_ptr[r]; p < sp.a_diag[r]; p++) yv[r] -= S[p] * yv[sp.a_col[p]];
    std::vector<double> bt(m), y(m), x(m);
    for (int t = 0; t < m; t++) {
      double s = yv[a + t];
      for (int p = sp.b_ptr[t]; p < sp.b_ptr[t + 1]; p++) s -= S[sp.off_ba + p] * yv[sp.b_col[p]];
      bt[t] = s;
    }
    for (int k = 0; k < m; k++) {
      double s = bt[perm[k]];
      for (int t = 0; t < k; t++) s -= Mx(perm[k], t) * y[t];
      y[k] = s;
    }
    for (int k = m - 1; k >= 0; k--) {
      double s = y[k];
      for (int t = k + 1; t < m; t++) s -= Mx(perm[k], t) * x[t];
      x[k] = s / Mx(perm[k], k);
    }
    for (int t = 0; t < m; t++) yv[a + t] = x[t];
    for (int l = 0; l + 1 < (int)sp.ul_ptr.size(); l++)
      for (int i = sp.ul_ptr[l]; i < sp.ul_ptr[l + 1]; i++) {
        const int r = sp.ul_rows[i];
        double s = yv[r];
        for (int p = sp.a_diag[r] + 1; p < sp.a_ptr[r + 1]; p++) s -= S[p] * yv[sp.a_col[p]];
        yv[r] = s * dinv[r];
      }
    // the chain-rule system, dense elimination with partial pivoting
    std::vector<double> Mc((size_t)n * n), rb = b, xr(n);
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        Mc[(size_t)i * n + j] = (i == j ? 1.0 : 0.0) -
                                gam * (J[(size_t)i * (n + 1) + j] + J[(size_t)i * (n + 1) + n] * h.xe[j]);
    for (int k = 0; k < n; k++) {
      int p = k;
      for (int i = k + 1; i < n; i++)
        if (std::fabs(Mc[(size_t)i * n + k]) > std::fabs(Mc[(size_t)p * n + k])) p = i;
      if (p != k) {
        for (int j = 0; j < n; j++) std::swap(Mc[(size_t)k * n + j], Mc[(size_t)p * n + j]);
        std::swap(rb[k], rb[p]);
      }
      for (int i = k + 1; i < n; i++) {
        const double l = Mc[(size_t)i * n + k] / Mc[(size_t)k * n + k];
        for (int j = k; j < n; j++) Mc[(size_t)i * n + j] -= l * Mc[(size_t)k * n + j];
        rb[i] -= l * rb[k];
      }
    }
    for (int k = n - 1; k >= 0; k--) {
      double s = rb[k];
      for (int j = k + 1; j < n; j++) s -= Mc[(size_t)k * n + j] * xr[j];
      xr[k] = s / Mc[(size_t)k * n + k];
    }
    double mx = 0.0, er = 0.0;
    for (int i = 0; i < n; i++) {
      mx = std::max(mx, std::fabs(xr[i]));
      er = std::max(er, std::fabs(xr[i] - yv[sp.iperm[i]]));
    }
    worst = std::max(worst, er / mx);
  }
  std::printf("%s: N %d leaf %d levels %zu dense %d storage %d; bordered vs chain-rule solve %.2e\n", name.c_str(),
              N, a, sp.lev_ptr.size() - 1, m, sp.total, worst);
  return worst < 1e-9 ? 0 : 2;
}

int main(int argc, char **argv) {
  if (argc < 3) return 64;
  int rc = 0;
  for (int i = 2; i < argc; i++) rc |= check_network(argv[1], argv[i]);
  return rc;
}
