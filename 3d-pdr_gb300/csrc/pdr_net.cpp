// pdr_net.cpp -- network loader and device-table builder.
//
// Parses the reference's network files with the semantics of
// read_species.F90:15-194 and read_rates.F90:9-95 (CSV records, empty fields
// keep their blank/zero initial values, consecutive identical reactions form a
// duplicate group whose RTMIN is moved to the previous RTMAX, :61-74), classifies
// every reaction the way calc_reac_rates.F90:53-112 dispatches it, and builds the
// tables the kernels read: reactant slots per reaction, the net stoichiometry as
// per-species term lists, and their balanced split over the 32 lanes of a warp.
#include <algorithm>
#include <bitset>
#include <limits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>

#include "pdr_internal.h"

namespace pdr {

static std::string trim(const std::string &s) {
  size_t b = s.find_first_not_of(" \t\r\n"), e = s.find_last_not_of(" \t\r\n");
  return b == std::string::npos ? std::string() : s.substr(b, e - b + 1);
}

static std::vector<std::string> csv(const std::string &line) {
  std::vector<std::string> f;
  std::string cur;
  for (char c : line) {
    if (c == ',') { f.push_back(trim(cur)); cur.clear(); }
    else cur.push_back(c);
  }
  f.push_back(trim(cur));
  return f;
}

static std::vector<std::string> records(const char *path, std::string &err) {
  std::vector<std::string> out;
  std::ifstream in(path);
  if (!in) { err = std::string("cannot open ") + path; return out; }
  std::string line;
  while (std::getline(in, line))
    if (!trim(line).empty()) out.push_back(line);
  return out;
}

static double num(const std::string &s) { return s.empty() ? 0.0 : std::strtod(s.c_str(), nullptr); }

static int name_charge(const std::string &s) {
  if (s == "e-" || s == "ELECTR") return -1;
  int q = 0;
  for (char c : s) q += (c == '+') - (c == '-');
  return q;
}

std::string load_network(const char *species, const char *rates, const char *layout, HostNet &net) {
  std::string err;
  auto sp = records(species, err);
  if (!err.empty()) return err;
  for (auto &r : sp) {
    auto f = csv(r);
    if (f.size() < 4) return "bad species record";
    net.spec.push_back(f[1]);
  }
  net.nspec = (int)net.spec.size();
  net.neq = net.nspec - 1;
  if (net.nspec < 2 || (net.spec.back() != "e-" && net.spec.back() != "ELECTR"))
    return "the electron must be the last species (calculate_abundances.c:67)";
  net.slot.assign(net.spec.begin(), net.spec.end() - 1);
  net.xe.resize(net.neq);
  for (int i = 0; i < net.neq; i++) net.xe[i] = name_charge(net.spec[i]);
  if (layout) {
    auto ly = records(layout, err);
    if (!err.empty()) return err;
    if ((int)ly.size() != net.neq) return "layout slot count does not match the species file";
    for (auto &r : ly) {
      auto f = csv(r);
      if (f.size() < 4) return "bad layout record";
      int s = std::atoi(f[0].c_str()) - 1;
      if (s < 0 || s >= net.neq || f[1] != net.spec[s]) return "layout does not match the species file";
      net.slot[s] = f[2];
      net.xe[s] = std::atoi(f[3].c_str());
    }
  }
  std::map<std::string, int> slot_of;
  for (int i = 0; i < net.neq; i++) slot_of[net.slot[i]] = i;
  slot_of[net.spec.back()] = net.neq;  // electron

  auto rr = records(rates, err);
  if (!err.empty()) return err;
  net.nreac = (int)rr.size();
  const int n = net.nreac;
  net.reac.resize(n); net.prod.resize(n);
  net.alpha.resize(n); net.beta.resize(n); net.gamma.resize(n);
  net.rtmin.resize(n); net.rtmax.resize(n); net.dup.assign(n, 0);
  net.ode_kind.resize(n); net.rate_kind.resize(n); net.ra.resize(n); net.rb.resize(n);
  net.pidx.resize(n);
  for (int i = 0; i < n; i++) {
    auto f = csv(rr[i]);
    if (f.size() < 14) return "bad rate record " + std::to_string(i + 1);
    for (int k = 0; k < 3; k++) net.reac[i][k] = f[1 + k];
    for (int k = 0; k < 4; k++) net.prod[i][k] = f[4 + k];
    net.alpha[i] = num(f[8]); net.beta[i] = num(f[9]); net.gamma[i] = num(f[10]);
    net.rtmin[i] = num(f[12]); net.rtmax[i] = num(f[13]);
    if (i > 0 && net.reac[i] == net.reac[i - 1] && net.prod[i] == net.prod[i - 1]) {
      if (net.dup[i - 1] == 0) net.dup[i - 1] = 1;
      net.dup[i] = net.dup[i - 1] + 1;
      net.rtmin[i] = net.rtmax[i - 1];
    }
  }
  auto is = [](const std::string &a, const char *b) { return a == b; };
  for (int i = 0; i < n; i++) {
    const auto &R = net.reac[i];
    const auto &P = net.prod[i];
    const std::string &r2 = R[1];
    bool xray = is(r2, "XRAY") || is(r2, "XRSEC") || is(r2, "XRLYA") || is(r2, "XRPHOT");
    bool uni = is(r2, "PHOTON") || is(r2, "CRP") || is(r2, "CRPHOT") || r2.empty() ||
               is(r2, "FREEZE") || is(r2, "ELFRZE") || is(r2, "CRH") || is(r2, "PHOTD") ||
               is(r2, "THERM") || (!r2.empty() && r2[0] == '#');
    auto sl = [&](const std::string &s) { auto it = slot_of.find(s); return it == slot_of.end() ? -1 : it->second; };
    net.ra[i] = sl(R[0]);
    net.rb[i] = -1;
    if (xray) net.ode_kind[i] = ODE_XRAY;
    else if (R[2] == "#") net.ode_kind[i] = ODE_GRAINH2;
    else if (uni) net.ode_kind[i] = ODE_UNI;
    else { net.ode_kind[i] = ODE_BI; net.rb[i] = sl(R[1]); }
    if (net.ra[i] < 0 || (net.ode_kind[i] == ODE_BI && net.rb[i] < 0))
      return "reaction " + std::to_string(i + 1) + ": reactant is not a species";
    for (int k = 0; k < 4; k++) net.pidx[i][k] = sl(P[k]);
    auto anyP = [&](const char *s) { for (auto &p : P) if (p == s) return true; return false; };
    int k;
    if (is(r2, "PHOTON")) {
      if (is(R[0], "H2") && R[2].empty()) k = RK_PHOTO_H2;
      else if (is(R[0], "HD") && R[2].empty()) k = RK_PHOTO_HD;
      else if (is(R[0], "CO") && R[2].empty() && anyP("C") && anyP("O")) k = RK_PHOTO_CO;
      else if (is(R[0], "C") && R[2].empty() &&
               ((is(P[0], "C+") && is(P[1], "e-")) || (is(P[0], "e-") && is(P[1], "C+"))))
        k = RK_PHOTO_CI;
      else if (is(R[0], "S") && R[2].empty() &&
               ((is(P[0], "S+") && is(P[1], "e-")) || (is(P[0], "e-") && is(P[1], "S+"))))
        k = RK_PHOTO_SI;
      else k = RK_PHOTO;
    } else if (is(r2, "CRP")) k = RK_CRP;
    else if (is(r2, "CRPHOT")) k = RK_CRPHOT;
    else if (is(r2, "FREEZE")) k = RK_FREEZE;
    else if (is(r2, "ELFRZE")) k = RK_ELFRZE;
    else if (is(r2, "CRH")) k = RK_CRH;
    else if (is(r2, "PHOTD")) k = RK_PHOTD;
    else if (is(r2, "THERM")) k = RK_THERM;
    else if (!r2.empty() && r2[0] == '#') k = RK_GRAIN;
    else if (xray) k = RK_XRAY;
    else {
      bool h2f = is(R[0], "H") && is(R[1], "H") && (R[2].empty() || is(R[2], "#")) && is(P[0], "H2") &&
                 (P[1].empty() || is(P[1], "#"));
      bool pah = false;
      for (auto &x : R) pah |= is(x, "PAH") || is(x, "PAH0") || is(x, "PAH+") || is(x, "PAH-");
      k = h2f ? RK_H2FORM : (pah ? RK_PAH : RK_THERMAL);
    }
    net.rate_kind[i] = k;
    if (k == RK_H2FORM) net.nr[0] = i + 1;
    if (k == RK_PHOTO_H2 && is(P[0], "H") && is(P[1], "H")) net.nr[1] = i + 1;
    if (k == RK_PHOTO_HD && anyP("H") && anyP("D")) net.nr[2] = i + 1;
    if (k == RK_PHOTO_CO) net.nr[3] = i + 1;
    if (k == RK_PHOTO_CI) net.nr[4] = i + 1;
    if (k == RK_PHOTO_SI) net.nr[5] = i + 1;
  }
  return std::string();
}

// net stoichiometry nu_{i,r} of every ODE slot, sorted by slot then reaction
struct Term { int i, r; double nu; };

static std::vector<Term> stoichiometry(const HostNet &net) {
  std::vector<Term> t;
  for (int r = 0; r < net.nreac; r++) {
    if (net.ode_kind[r] == ODE_XRAY) continue;
    std::map<int, double> nu;
    for (int k = 0; k < 4; k++)
      if (net.pidx[r][k] >= 0 && net.pidx[r][k] < net.neq) nu[net.pidx[r][k]] += 1.0;
    nu[net.ra[r]] -= 1.0;
    if (net.ode_kind[r] == ODE_BI) nu[net.rb[r]] -= 1.0;
    if (net.ode_kind[r] == ODE_GRAINH2) nu[net.ra[r]] -= 1.0;
    for (auto &kv : nu)
      if (kv.first < net.neq && kv.second != 0.0) t.push_back({kv.first, r, kv.second});
  }
  std::stable_sort(t.begin(), t.end(), [](const Term &a, const Term &b) {
    return a.i != b.i ? a.i < b.i : a.r < b.r;
  });
  return t;
}

template <class T>
static T *upload(pdr_net *net, const std::vector<T> &v, int &rc) {
  if (v.empty()) return nullptr;
  T *d = nullptr;
  cudaError_t e = cudaMalloc(&d, v.size() * sizeof(T));
  if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMalloc(network tables)"); return nullptr; }
  net->allocations.push_back(d);
  e = cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpy(network tables)");
  return d;
}

// ---- sparse Newton matrix of the block integrator (mixed form) ----
//
// The chain rule through x_e = sum_j c_j x_j adds (df/dx_e) c^T to the
// Jacobian: a rank-one term that fills the rows of every species with an
// electron reaction in the columns of every charged species (two thirds of
// the full network's 214 x 214 entries).  Keeping x_e as an unknown of its
// own, with the linearised constraint x_e - c^T x = 0 as an extra row, gives
// the same Newton correction from a matrix with a seventh of the entries.
// This plan orders the unknowns (minimum degree), computes the fill of the
// factorisation in that order, splits the rows into packed "leaf" rows and a
// dense trailing block, and maps every Jacobian entry to its storage location.
struct SparsePlan {
  int N = 0, a = 0, m = 0, ldb = 0, off_ba = 0, off_d = 0, total = 0;
  std::vector<int> perm, iperm, a_ptr, a_diag, lev_ptr, ul_rows, ul_ptr, b_ptr, diag_loc, e_loc;
  std::vector<unsigned short> a_col, b_col;
  std::vector<std::bitset<256>> F;   // filled pattern in elimination order
  // storage location of entry (unknown i, unknown j), -1 outside the pattern
  int loc(int i, int j) const {
    if (i < a) {
      for (int p = a_ptr[i]; p < a_ptr[i + 1]; p++)
        if (a_col[p] == j) return p;
      return -1;
    }
    const int t = i - a;
    if (j < a) {
      for (int p = b_ptr[t]; p < b_ptr[t + 1]; p++)
        if (b_col[p] == j) return off_ba + p;
      return -1;
    }
    return off_d + (j - a) * ldb + t;
  }
};

using Bits = std::bitset<256>;

// symbolic LU fill without pivoting of pattern P (rows as bitsets)
static std::vector<Bits> symbolic_fill(std::vector<Bits> F) {
  const int N = (int)F.size();
  for (int k = 0; k < N; k++) {
    Bits right = F[k];
    for (int j = 0; j <= k; j++) right.reset(j);
    for (int i = k + 1; i < N; i++)
      if (F[i].test(k)) F[i] |= right;
  }
  return F;
}

// pattern entries (row, column) over slots (species 0..neq-1, x_e = neq);
// G threads per block (for the cost model)
static bool sparse_plan(int neq, const std::vector<std::pair<int, int>> &entries, const std::vector<int> &xe,
                        int G, SparsePlan &sp) {
  const int N = neq + 1;
  if (N > 256) return false;
  std::vector<Bits> P(N);
  for (int i = 0; i < N; i++) P[i].set(i);
  for (auto &e : entries) P[e.first].set(e.second);
  for (int j = 0; j < neq; j++)
    if (xe[j] != 0) P[neq].set(j);
  // minimum-degree order on the symmetrised pattern (ties: lowest slot)
  std::vector<int> order;
  {
    std::vector<Bits> adj(N);
    for (int i = 0; i < N; i++)
      for (int j = 0; j < N; j++)
        if (i != j && (P[i].test(j) || P[j].test(i))) adj[i].set(j);
    Bits alive;
    for (int i = 0; i < N; i++) alive.set(i);
    for (int step = 0; step < N; step++) {
      int best = -1;
      size_t bd = 0;
      for (int v = 0; v < N; v++) {
        if (!alive.test(v)) continue;
        const size_t d = (adj[v] & alive).count();
        if (best < 0 || d < bd) { best = v; bd = d; }
      }
      order.push_back(best);
      alive.reset(best);
      const Bits nb = adj[best] & alive;
      for (int u = 0; u < N; u++)
        if (nb.test(u)) { adj[u] |= nb; adj[u].reset(u); }
    }
  }
  auto permuted = [&](const std::vector<int> &ord) {
    std::vector<Bits> Q(N);
    for (int i = 0; i < N; i++)
      for (int j = 0; j < N; j++)
        if (P[ord[i]].test(ord[j])) Q[i].set(j);
    return symbolic_fill(Q);
  };
  std::vector<Bits> F = permuted(order);
  // L-dependency level of each row: 1 + the deepest row it reads
  std::vector<int> lev(N, 1);
  int maxlev = 0;
  for (int i = 0; i < N; i++) {
    for (int k = 0; k < i; k++)
      if (F[i].test(k)) lev[i] = std::max(lev[i], lev[k] + 1);
    maxlev = std::max(maxlev, lev[i]);
  }
  // split: the rows of levels <= s are leaf rows.  Cost model per
  // factorisation: the dense block's FMAs spread over G threads, a block
  // barrier per dense column and per leaf level, and the longest leaf row
  // (one thread each) of every level
  std::vector<int> ucount(N, 0);
  for (int k = 0; k < N; k++)
    for (int j = k + 1; j < N; j++) ucount[k] += F[k].test(j);
  int best_s = 0;
  double best_cost = 0.0;
  for (int s = 0; s <= maxlev; s++) {
    int a = 0;
    double rowwork = 0.0;
    std::vector<double> lw(s + 1, 0.0);
    for (int i = 0; i < N; i++)
      if (lev[i] <= s) {
        a++;
        double w = 0.0;
        for (int k = 0; k < i; k++)
          if (F[i].test(k)) w += 1 + ucount[k];
        lw[lev[i]] = std::max(lw[lev[i]], w);
      }
    for (double w : lw) rowwork += w;
    const double m = N - a;
    const double cost = 4.0 * (2.0 / 3.0) * m * m * m / G + 250.0 * (m + s) + 12.0 * rowwork;
    if (s == 0 || cost < best_cost) { best_cost = cost; best_s = s; }
  }
  // final order: leaf rows by level (rows of one level are independent, so
  // this keeps the fill), then the trailing rows in minimum-degree order
  std::vector<int> idx;
  for (int l = 1; l <= best_s; l++)
    for (int i = 0; i < N; i++)
      if (lev[i] == l) idx.push_back(i);
  const int a = (int)idx.size();
  for (int i = 0; i < N; i++)
    if (lev[i] > best_s) idx.push_back(i);
  std::vector<int> ord2(N);
  for (int i = 0; i < N; i++) ord2[i] = order[idx[i]];
  F = permuted(ord2);
  const int m = N - a;
  for (int i = a; i < N; i++)
    for (int j = a; j < N; j++) F[i].set(j);   // the trailing block is stored dense
  sp.N = N;
  sp.a = a;
  sp.m = m;
  sp.ldb = m | 1;
  sp.perm = ord2;
  sp.iperm.assign(N, 0);
  for (int i = 0; i < N; i++) sp.iperm[ord2[i]] = i;
  // leaf rows, packed; their levels
  sp.a_ptr.assign(1, 0);
  sp.lev_ptr.assign(1, 0);
  std::vector<int> lev2(N, 1);
  for (int i = 0; i < a; i++) {
    for (int k = 0; k < i; k++)
      if (F[i].test(k)) lev2[i] = std::max(lev2[i], lev2[k] + 1);
    for (int j = 0; j < N; j++)
      if (F[i].test(j)) {
        if (j == i) sp.a_diag.push_back((int)sp.a_col.size());
        sp.a_col.push_back((unsigned short)j);
      }
    sp.a_ptr.push_back((int)sp.a_col.size());
  }
  for (int i = 0; i < a; i++) {
    if (i > 0 && lev2[i] < lev2[i - 1]) return false;   // rows must be in level order
    if (i == 0 || lev2[i] != lev2[i - 1]) {
      if (i > 0) sp.lev_ptr.push_back(i);
    }
  }
  if (a > 0) sp.lev_ptr.push_back(a);
  // U-dependency levels of the leaf rows (backward substitution)
  std::vector<int> ul(a, 1);
  int maxul = 0;
  for (int i = a - 1; i >= 0; i--) {
    for (int j = i + 1; j < a; j++)
      if (F[i].test(j)) ul[i] = std::max(ul[i], ul[j] + 1);
    maxul = std::max(maxul, ul[i]);
  }
  sp.ul_ptr.assign(1, 0);
  for (int l = 1; l <= maxul; l++) {
    for (int i = 0; i < a; i++)
      if (ul[i] == l) sp.ul_rows.push_back(i);
    sp.ul_ptr.push_back((int)sp.ul_rows.size());
  }
  // trailing rows: leaf-column entries packed, then the dense block
  sp.b_ptr.assign(1, 0);
  for (int i = a; i < N; i++) {
    for (int j = 0; j < a; j++)
      if (F[i].test(j)) sp.b_col.push_back((unsigned short)j);
    sp.b_ptr.push_back((int)sp.b_col.size());
  }
  sp.off_ba = (int)sp.a_col.size();
  sp.off_d = (sp.off_ba + (int)sp.b_col.size() + 3) & ~3;
  sp.total = sp.off_d + m * sp.ldb;
  if (sp.total >= 65536) return false;
  sp.F = F;
  sp.diag_loc.assign(N, -1);
  for (int i = 0; i < N; i++) sp.diag_loc[i] = sp.loc(i, i);
  sp.e_loc.assign(neq, -1);
  for (int j = 0; j < neq; j++)
    if (xe[j] != 0) sp.e_loc[j] = sp.loc(sp.iperm[neq], sp.iperm[j]);
  for (int v : sp.diag_loc)
    if (v < 0) return false;
  return true;
}

int build_device_tables(pdr_net *net) {
  const HostNet &h = net->host;
  int rc = 0;
  // ---- rate evaluator tables ----
  {
    std::vector<int> kind(h.rate_kind), dup(h.dup), dn(h.nreac), flags(h.nreac, 0);
    for (int i = 0; i < h.nreac; i++) {
      dn[i] = (i + 1 < h.nreac) ? h.dup[i + 1] : -1;
      if (!h.reac[i][0].empty() && h.reac[i][0][0] == 'G') flags[i] |= 1;
    }
    net->rates.nreac = h.nreac;
    net->rates.kind = upload(net, kind, rc);
    net->rates.dup = upload(net, dup, rc);
    net->rates.dup_next = upload(net, dn, rc);
    net->rates.alpha = upload(net, h.alpha, rc);
    net->rates.beta = upload(net, h.beta, rc);
    net->rates.gamma = upload(net, h.gamma, rc);
    net->rates.rtmin = upload(net, h.rtmin, rc);
    net->rates.rtmax = upload(net, h.rtmax, rc);
    net->rates.flags = upload(net, flags, rc);
    std::vector<int> ray, other;
    auto ray_kind = [](int k) {
      return k == RK_PHOTO_H2 || k == RK_PHOTO_HD || k == RK_PHOTO_CO || k == RK_PHOTO_CI || k == RK_PHOTO_SI ||
             k == RK_PHOTO || k == RK_PHOTD;
    };
    for (int i = 0; i < h.nreac; i++) (ray_kind(h.rate_kind[i]) ? ray : other).push_back(i);
    auto by_kind = [&](int x, int y) { return h.rate_kind[x] < h.rate_kind[y]; };
    std::stable_sort(ray.begin(), ray.end(), by_kind);
    std::stable_sort(other.begin(), other.end(), by_kind);
    net->rates.nray = (int)ray.size();
    net->rates.nother = (int)other.size();
    net->rates.ray_reac = upload(net, ray, rc);
    net->rates.other_reac = upload(net, other, rc);
  }
  // ---- chemistry tables ----
  const int neq = h.neq;
  const int E = neq, ONE = neq + 1;
  std::vector<int2> rab(h.nreac);
  std::vector<double> nhm(h.nreac);
  for (int r = 0; r < h.nreac; r++) {
    int a = h.ra[r], b = (h.ode_kind[r] == ODE_BI) ? h.rb[r] : ONE;
    if (h.ode_kind[r] == ODE_XRAY) { a = ONE; b = ONE; }
    rab[r] = make_int2(a == neq ? E : a, b);
    nhm[r] = (h.ode_kind[r] == ODE_BI || h.ode_kind[r] == ODE_GRAINH2) ? 1.0 : 0.0;
  }
  auto terms = stoichiometry(h);
  // the packed term tables hold a reaction in 16 bits and a slot in 8: larger
  // networks get no integrator tables (the solve entry points reject them)
  if (h.nreac >= 65536 || neq + 2 > 255) return rc;
  auto build = [&](int G, WarpTables &w, size_t max_merged) -> int {
    w.neq = neq;
    w.nreac = h.nreac;
    w.lanes = G;
    const int T = (int)terms.size();
    // RHS operands: the slot values themselves (one-body reactions, whose
    // flux is kn x_a) and the product x_a x_b of every distinct reactant pair
    // of the two-body reactions, formed once per RHS evaluation.  A term is
    // then one FMA, s += (nu kn_r) * operand, with nu kn_r taken from the
    // per-cell rate constants: nu = +-1 is a sign flip of kn_r (an integer
    // operation), |nu| > 1 reads an extra constant |nu| kn_r made once per cell.
    std::vector<int> op_of(h.nreac, ONE);
    std::map<std::pair<int, int>, int> pair_index;
    std::vector<int2> pairs;
    for (int r = 0; r < h.nreac; r++) {
      if (h.ode_kind[r] == ODE_XRAY) continue;
      const int2 ab = rab[r];
      if (h.ode_kind[r] == ODE_BI) {
        const std::pair<int, int> key(std::min(ab.x, ab.y), std::max(ab.x, ab.y));
        auto it = pair_index.find(key);
        if (it == pair_index.end()) {
          it = pair_index.emplace(key, (int)pairs.size()).first;
          pairs.push_back(make_int2(key.first, key.second));
        }
        op_of[r] = neq + 2 + it->second;
      } else {
        op_of[r] = ab.x;
      }
    }
    for (auto &t : terms)
      if (std::fabs(t.nu) != std::floor(std::fabs(t.nu)) || std::fabs(t.nu) > 64) return PDR_E_NET;
    // Terms of one species that share an operand (reactions with the same
    // reactants and different products) are merged: their coefficient
    // sum_r nu_r kn_r is formed once per cell as an extra rate constant
    // (kn[nreac + e], summed in reaction order), so the RHS takes one FMA for
    // them.  A single term with nu = +-1 reads kn_r with the sign bit flipped;
    // any other single term reads an extra constant nu kn_r.
    struct MTerm { int i, op, kidx; bool neg; };
    std::vector<MTerm> mt;
    std::vector<int> kext_ptr(1, 0);
    std::vector<int2> kext_rn;   // (reaction, nu) of the extras' summands
    auto extra = [&](const std::vector<int> &ts) {
      for (int t : ts) kext_rn.push_back(make_int2(terms[t].r, (int)terms[t].nu));
      kext_ptr.push_back((int)kext_rn.size());
      return h.nreac + (int)kext_ptr.size() - 2;
    };
    // the groups of terms (one species, one operand), in species order and
    // operand order of first appearance
    struct Group { int i, op; std::vector<int> ts; };
    std::vector<Group> groups;
    for (int t0 = 0; t0 < T;) {
      const int i = terms[t0].i;
      int t1 = t0;
      while (t1 < T && terms[t1].i == i) t1++;
      std::map<int, int> at;
      for (int t = t0; t < t1; t++) {
        const int op = op_of[terms[t].r];
        auto it = at.find(op);
        if (it == at.end()) {
          at[op] = (int)groups.size();
          groups.push_back({i, op, {t}});
        } else {
          groups[it->second].ts.push_back(t);
        }
      }
      t0 = t1;
    }
    // every extra rate constant costs 8 bytes of a warp integrator's shared
    // memory: the largest groups are merged first, up to max_merged of them
    std::vector<int> by_size;
    for (int g = 0; g < (int)groups.size(); g++)
      if (groups[g].ts.size() > 1) by_size.push_back(g);
    std::stable_sort(by_size.begin(), by_size.end(),
                     [&](int a, int b) { return groups[a].ts.size() > groups[b].ts.size(); });
    std::vector<char> merge(groups.size(), 0);
    for (size_t k = 0; k < by_size.size() && k < max_merged; k++) merge[by_size[k]] = 1;
    for (int g = 0; g < (int)groups.size(); g++) {
      const Group &gr = groups[g];
      if (merge[g]) {
        mt.push_back({gr.i, gr.op, extra(gr.ts), false});
        continue;
      }
      for (int t : gr.ts) {
        if (std::fabs(terms[t].nu) == 1.0) mt.push_back({gr.i, gr.op, terms[t].r, terms[t].nu < 0});
        else mt.push_back({gr.i, gr.op, extra({t}), false});
      }
    }
    const int M = (int)mt.size();
    // the merged term list cut into G balanced chunks; a chunk flushes its
    // running sum into a partial slot whenever the species changes
    w.rhs_len = std::max(1, (M + G - 1) / G);
    std::vector<int2> rt(w.rhs_len * G, make_int2(0, ONE));
    std::vector<std::vector<int>> parts(G);
    int slot = 0;
    for (int l = 0; l < G; l++) {
      int b = l * w.rhs_len, e = std::min(M, b + w.rhs_len);
      for (int t = b; t < e; t++) {
        int k = t - b, fl = -1;
        if (t + 1 == e || mt[t + 1].i != mt[t].i) {
          fl = slot;
          parts[mt[t].i].push_back(slot);
          slot++;
        }
        rt[k * G + l] = make_int2(mt[t].kidx | ((fl + 1) << 16), mt[t].op | (mt[t].neg ? (int)0x80000000u : 0));
      }
    }
    // padding terms read the constant-zero rate slot nkn (kn is zero-filled there)
    const int nkext = (int)kext_ptr.size() - 1;
    const int nkn = h.nreac + nkext;
    for (int l = 0; l < G; l++) {
      int b = l * w.rhs_len, e = std::min(M, b + w.rhs_len);
      for (int t = std::max(e, b); t < b + w.rhs_len; t++) rt[(t - b) * G + l] = make_int2(nkn, ONE);
    }
    if (slot + 1 >= 65536 || nkn + 1 >= 65536) return PDR_E_NET;
    w.nkn = nkn;
    w.nkext = nkext;
    w.npairs = (int)pairs.size();
    w.nop = neq + 2 + w.npairs;
    w.nparts = slot;
    w.plist_len = 1;
    for (auto &p : parts) w.plist_len = std::max<int>(w.plist_len, (int)p.size());
    std::vector<int> pl(w.plist_len * G, slot /* zero slot */);
    for (int i = 0; i < G; i++)
      for (size_t k = 0; k < parts[i].size(); k++) pl[k * G + i] = parts[i][k];
    // per-species Jacobian term lists
    std::vector<std::vector<Term>> per(G);
    for (auto &t : terms) per[t.i].push_back(t);
    w.jac_len = 1;
    for (auto &p : per) w.jac_len = std::max<int>(w.jac_len, (int)p.size());
    std::vector<int> jr(w.jac_len * G, 0);   // reaction | a << 16 | b << 24
    std::vector<double> jn(w.jac_len * G, 0.0);
    std::vector<float> jnf(w.jac_len * G, 0.0f);
    for (int i = 0; i < G; i++)
      for (size_t k = 0; k < per[i].size(); k++) {
        const int r = per[i][k].r;
        jr[k * G + i] = r | (rab[r].x << 16) | (rab[r].y << 24);
        jn[k * G + i] = per[i][k].nu;
        jnf[k * G + i] = (float)per[i][k].nu;
      }
    std::vector<double> xe(G, 0.0);
    for (int i = 0; i < neq; i++) xe[i] = h.xe[i];
    // term-parallel Jacobian tables (both integrators)
    std::vector<int2> hxy;
    std::vector<int> bt, bs;
    SparsePlan plan;
    std::vector<double> hn;
    {
      struct Half { int i, col, r, which; double nu; };
      std::vector<Half> hs;
      for (auto &t : terms) {
        const int2 ab = rab[t.r];
        if (ab.x <= neq) hs.push_back({t.i, ab.x, t.r, 0, t.nu});   // column a: Da
        if (ab.y <= neq) hs.push_back({t.i, ab.y, t.r, 1, t.nu});   // column b: Db
      }
      std::stable_sort(hs.begin(), hs.end(), [](const Half &x, const Half &y) {
        if (x.i != y.i) return x.i < y.i;
        if (x.col != y.col) return x.col < y.col;
        if (x.r != y.r) return x.r < y.r;
        return x.which < y.which;
      });
      const int H = (int)hs.size();
      // the block integrator's sparse Newton matrix: entry locations
      if (G > kWarp) {
        std::vector<std::pair<int, int>> ent;
        for (auto &x : hs) ent.push_back({x.i, x.col});
        w.sp.ok = sparse_plan(neq, ent, h.xe, G, plan) ? 1 : 0;
      }
      auto sp_loc = [&](int i, int col) -> unsigned {
        if (!w.sp.ok) return 0u;
        const int l = plan.loc(plan.iperm[i], plan.iperm[col]);
        if (l < 0) w.sp.ok = 0;
        return l < 0 ? 0u : (unsigned)l;
      };
      w.hlen = std::max(1, (H + G - 1) / G);
      hxy.assign((size_t)w.hlen * G, int2{0, 0});
      hn.assign((size_t)w.hlen * G, 0.0);
      // an entry's runs: the chunks holding it, in order
      int slot = 0;
      for (int e0 = 0; e0 < H;) {
        int e1 = e0;
        while (e1 < H && hs[e1].i == hs[e0].i && hs[e1].col == hs[e0].col) e1++;
        const int c0 = e0 / w.hlen, c1 = (e1 - 1) / w.hlen;
        const int first_slot = slot;
        for (int c = c0; c <= c1; c++) {
          const int b = std::max(e0, c * w.hlen), e = std::min(e1, (c + 1) * w.hlen);
          for (int k = b; k < e; k++) {
            const int t = k - c * w.hlen;
            int kind = 0, sl = 0;
            if (k + 1 == e) {
              kind = (c0 == c1) ? 1 : 2;
              if (kind == 2) sl = slot++;
            }
            // nu, a stoichiometric count, rides in the high bits as a signed integer
            const int nu_i = (int)hs[k].nu;
            if ((double)nu_i != hs[k].nu || nu_i < -4096 || nu_i > 4095 || hs[k].r > 0xffff) return PDR_E_NET;
            hxy[(size_t)t * G + c].x = (int)((unsigned)hs[k].r | ((unsigned)hs[k].which << 16) | ((unsigned)kind << 17) |
                                             ((unsigned)nu_i << 19));
            // kind 1 (a store): the entry's sparse location; kind 2: its slot
            const unsigned hi = (kind == 1) ? sp_loc(hs[k].i, hs[k].col) : (unsigned)sl;
            hxy[(size_t)t * G + c].y = (int)((unsigned)hs[k].i | ((unsigned)hs[k].col << 8) | (hi << 16));
            hn[(size_t)t * G + c] = hs[k].nu;
          }
        }
        if (c0 != c1) {
          bt.push_back((int)((unsigned)hs[e0].i | ((unsigned)hs[e0].col << 8) | (sp_loc(hs[e0].i, hs[e0].col) << 16)));
          bs.push_back(first_slot | (slot << 16));
        }
        e0 = e1;
      }
      // the slots live in the block integrator's LU panel buffer (8 x neq
      // values) and in the warp integrator's RHS partial-sum buffer (nparts
      // values, free during the assembly); a run crosses at most G-1 chunk
      // boundaries in all
      if (neq + 1 > 255) return PDR_E_NET;
      if (G > kWarp ? slot > 8 * neq : slot > w.nparts) return PDR_E_NET;
      w.nbnd = (int)bt.size();
    }
    int rc2 = 0;
    w.rab = upload(net, rab, rc2);
    w.nh_mask = upload(net, nhm, rc2);
    w.rhs_t = upload(net, rt, rc2);
    w.pairs = upload(net, pairs, rc2);
    w.kext_ptr = upload(net, kext_ptr, rc2);
    w.kext_rn = upload(net, kext_rn, rc2);
    w.plist = upload(net, pl, rc2);
    w.jac_rab = upload(net, jr, rc2);
    w.jac_nu = upload(net, jn, rc2);
    w.jac_nu_f = upload(net, jnf, rc2);
    w.xe_coef = upload(net, xe, rc2);
    {
      std::vector<float> xef(xe.begin(), xe.end());
      w.xe_coef_f = upload(net, xef, rc2);
    }
    {
      w.h_xy = upload(net, hxy, rc2);
      w.h_nu = upload(net, hn, rc2);
      if (!bt.empty()) {
        w.bnd_t = upload(net, bt, rc2);
        w.bnd_s = upload(net, bs, rc2);
      }
    }
    if (w.sp.ok) {
      auto &d = w.sp;
      d.N = plan.N; d.a = plan.a; d.m = plan.m; d.ldb = plan.ldb;
      d.off_ba = plan.off_ba; d.off_d = plan.off_d; d.total = plan.total;
      d.nnz_b = (int)plan.b_col.size();
      d.nlev = (int)plan.lev_ptr.size() - 1;
      d.nul = (int)plan.ul_ptr.size() - 1;
      d.perm = upload(net, plan.perm, rc2);
      d.iperm = upload(net, plan.iperm, rc2);
      d.a_ptr = upload(net, plan.a_ptr, rc2);
      d.a_col = upload(net, plan.a_col, rc2);
      d.a_diag = upload(net, plan.a_diag, rc2);
      d.lev_ptr = upload(net, plan.lev_ptr, rc2);
      d.ul_rows = upload(net, plan.ul_rows, rc2);
      d.ul_ptr = upload(net, plan.ul_ptr, rc2);
      d.b_ptr = upload(net, plan.b_ptr, rc2);
      d.b_col = upload(net, plan.b_col, rc2);
      d.diag_loc = upload(net, plan.diag_loc, rc2);
      d.e_loc = upload(net, plan.e_loc, rc2);
    }
    return rc2;
  };
  if (neq <= kWarp) {
    // a warp integrator keeps its rate constants in shared memory: at most 96
    // merged groups keep the mixed form at 16 warps per SM
    const int e = build(kWarp, net->warp, 96);
    if (e) rc = e;
    net->warp_ok = (e == 0);
  }
  {
    const int G = std::max(64, (neq + kWarp - 1) / kWarp * kWarp);
    // the block integrator keeps its rate constants in global memory
    const int e = build(G, net->cta, std::numeric_limits<size_t>::max());
    if (e) rc = e;
    net->cta_ok = (e == 0);
  }
  return rc;
}

}  // namespace pdr
