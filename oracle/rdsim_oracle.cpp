// rdsim_oracle.cpp -- CPU float64 restatement of PyRDSim's simulation step.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU engine is
// checked against; it is linked by tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py, never by the product path.
//
// Every function follows pyrdsim/pyrdsim.pyx (cited as pyx:<line>) with the
// same float64 operation order.  Build with -ffp-contract=off.
#include "rdsim_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <random>
#include <set>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

struct Geom {
  double d;
  double hat[RDSIM_MAX_DIM];  // unit vector from the lower to the higher index
};

struct BondF {
  int i1, i2;
  double k, r0;
};
struct AngleF {
  int i1, i2, i3;
  double k0, theta0, thr;
  int pi;  // +1 if theta0 == pi (np.isclose, pyx:1333-1338), else -1
};

}  // namespace

struct oracle_handle {
  int D = 0, N = 0, T = 0, M = 0;
  double L[RDSIM_MAX_DIM] = {0}, periodic[RDSIM_MAX_DIM] = {0};
  double dt = 0, rs = 0;
  int ratio = 2, freq = 10, angle_is_pi = -1;
  bool quirk = false;
  std::vector<double> x, a, tau, fp, npf;
  std::vector<int> types, mol, first;
  std::vector<rdsim_interaction> inter;
  std::vector<rdsim_reaction> rx;
  std::vector<rdsim_template> tmpl;
  std::vector<rdsim_term> terms;
  bool partner[RDSIM_MAX_TYPES][RDSIM_MAX_TYPES];
  bool has_partner[RDSIM_MAX_TYPES];
  // neighbour lists: half lists (j > i), ascending
  std::vector<std::set<int>> bonded;       // bonded_neighbor_list
  std::vector<std::set<int>> bonded_init;  // its value after pyx:1268
  std::vector<std::vector<int>> nl;
  std::unordered_map<uint64_t, Geom> geom;  // d_xx / xx_hat of (i<j)
  std::vector<BondF> bonds;
  std::vector<AngleF> angles;
  // cells (pyx:1415-1446)
  double cl[RDSIM_MAX_DIM] = {0};
  int nc[RDSIM_MAX_DIM] = {0}, pbc_nc[RDSIM_MAX_DIM] = {0};
  std::vector<int> cell_id;
  double min_dist = INFINITY;
  std::vector<double> rates, total;
  std::mt19937 gen;
  int64_t step = 0;
  // first error
  int err_code = 0;
  int64_t err_particle = -1, err_step = -1;
  int err_dim = -1;
  double err_value = 0;

  uint64_t key(int i, int j) const { return (uint64_t)i * (uint64_t)N + (uint64_t)j; }

  // xx_hat[i, j, k] (unit vector from i to j) and d_xx[i, j]
  const Geom* g(int i, int j) const {
    auto it = geom.find(i < j ? key(i, j) : key(j, i));
    return it == geom.end() ? nullptr : &it->second;
  }
  double hat(int i, int j, int k) const {
    const Geom* p = g(i, j);
    if (!p) return 0.0;
    return i < j ? p->hat[k] : -p->hat[k];
  }
  double dxx(int i, int j) const {
    const Geom* p = g(i, j);
    return p ? p->d : 0.0;
  }

  double normal() {  // pyx:71-77
    std::normal_distribution<double> dist(0.0, 1.0);
    return dist(gen);
  }
  double uniform() {  // pyx:79-85
    std::uniform_real_distribution<double> dist(0.0, 1.0);
    return dist(gen);
  }

  // pyx:1415-1446
  void set_up_cells() {
    double r = (double)ratio;
    for (int k = 0; k < D; k++) {
      int l = 1;
      while (L[k] / (double)(l + 1) >= rs / r) l += 1;
      cl[k] = L[k] / (double)l;
      nc[k] = l;
      pbc_nc[k] = l - ratio;
    }
  }

  // pyx:1268-1408 (bonded_neighbor_list and the bonded force terms)
  int set_up_bonded() {
    bonded.assign(N, {});
    bonds.clear();
    angles.clear();
    std::map<int, int> by_id;
    for (int t = 0; t < (int)tmpl.size(); t++) by_id[tmpl[t].molecule_id] = t;
    for (int m = 0; m < M; m++) {
      int j = first[m];
      int mid = mol[3 * j + 2];
      auto it = by_id.find(mid);
      if (it == by_id.end())
        return fail(RDSIM_ERR_ARG, "molecule id " + std::to_string(mid) + " has no definition");
      const rdsim_template& tp = tmpl[it->second];
      for (int q = 0; q < tp.n_terms; q++) {
        const rdsim_term& tm = terms[tp.first_term + q];
        if (tm.kind == RDSIM_TERM_BOND) {
          int i1 = tm.i + j, i2 = tm.j + j;
          bonds.push_back({i1, i2, tm.k0, tm.p0});
          bonded[std::min(i1, i2)].insert(std::max(i1, i2));
        } else if (tm.kind == RDSIM_TERM_ANGLE) {
          int i1 = tm.i + j, i2 = tm.j + j, i3 = tm.k + j;
          angles.push_back({i1, i2, i3, tm.k0, tm.p0, tm.p0 - 0.1,
                            std::fabs(tm.p0 - M_PI) <= 1e-5 + 1e-5 * M_PI ? 1 : -1});
          bonded[std::min(i1, i2)].insert(std::max(i1, i2));
          bonded[std::min(i2, i3)].insert(std::max(i2, i3));
        }
      }
    }
    bonded_init = bonded;
    return 0;
  }

  // pyx:1590-1652, over a candidate list
  void calculate_distances(const std::vector<std::vector<int>>& lst) {
    double md = INFINITY;
    for (int i1 = 0; i1 < N; i1++) {
      for (int i2 : lst[i1]) {
        Geom gm;
        double xx[RDSIM_MAX_DIM];
        double dl = 0;
        for (int k = 0; k < D; k++) {
          double v = x[(size_t)i2 * D + k] - x[(size_t)i1 * D + k];
          if (periodic[k] > 0) v = v - L[k] * std::round(v / L[k]);
          dl += std::pow(v, 2.0);
          xx[k] = v;
        }
        dl = std::sqrt(dl);
        if (dl < md && mol[3 * i1] != mol[3 * i2]) md = dl;
        gm.d = dl;
        for (int k = 0; k < D; k++) gm.hat[k] = xx[k] / dl;
        geom[key(i1, i2)] = gm;
      }
    }
    min_dist = md;
  }

  bool is_partner(int ti, int tj) const {
    if (ti < 0 || tj < 0 || ti >= RDSIM_MAX_TYPES || tj >= RDSIM_MAX_TYPES) return false;
    if (!has_partner[tj]) return false;
    return partner[tj][ti];
  }

  // pyx:1448-1587
  void create_neighbor_list() {
    for (int i = 0; i < N; i++)
      for (int k = 0; k < D; k++)
        cell_id[(size_t)i * D + k] = (int)std::floor(x[(size_t)i * D + k] / cl[k]);
    std::vector<std::set<int>>& cand_src = quirk ? bonded : bonded_init;
    std::vector<std::set<int>> cand_local;
    if (!quirk) cand_local = bonded_init;
    std::vector<std::set<int>>& cand = quirk ? cand_src : cand_local;
    // bucket particles by cell tuple; enumerate allowed partner cells per dim
    std::map<std::vector<int>, std::vector<int>> buckets;
    std::vector<std::set<int>> values(D);
    for (int i = 0; i < N; i++) {
      std::vector<int> c(cell_id.begin() + (size_t)i * D, cell_id.begin() + (size_t)(i + 1) * D);
      buckets[c].push_back(i);
      for (int k = 0; k < D; k++) values[k].insert(c[k]);
    }
    for (int i = 0; i < N; i++) {
      int ti = types[i];
      std::vector<std::vector<int>> allowed(D);
      for (int k = 0; k < D; k++) {
        int ci = cell_id[(size_t)i * D + k];
        for (int v : values[k]) {
          int dc = v - ci;
          if (dc < 0) dc = -dc;
          bool ok;
          if (dc <= ratio) ok = true;
          else if (periodic[k] > 0) ok = !(dc < pbc_nc[k]);
          else ok = false;
          if (ok) allowed[k].push_back(v);
        }
      }
      std::vector<int> idx(D, 0), c(D);
      bool empty = false;
      for (int k = 0; k < D; k++) empty |= allowed[k].empty();
      if (empty) continue;
      while (true) {
        for (int k = 0; k < D; k++) c[k] = allowed[k][idx[k]];
        auto it = buckets.find(c);
        if (it != buckets.end()) {
          for (int j : it->second) {
            if (j <= i) continue;
            if (mol[3 * i] == mol[3 * j]) continue;  // pyx:1523
            if (!is_partner(ti, types[j])) continue; // pyx:1529-1534
            cand[i].insert(j);                        // pyx:1567
          }
        }
        int k = 0;
        while (k < D && ++idx[k] == (int)allowed[k].size()) idx[k++] = 0;
        if (k == D) break;
      }
    }
    std::vector<std::vector<int>> lst(N);
    for (int i = 0; i < N; i++) lst[i].assign(cand[i].begin(), cand[i].end());
    calculate_distances(lst);  // pyx:1572
    nl.assign(N, {});
    for (int i = 0; i < N; i++)  // pyx:1578-1586
      for (int j : lst[i])
        if (!(dxx(i, j) > rs)) nl[i].push_back(j);
  }

  // pyx:1068-1130: force magnitude of one pair law
  static double law(const rdsim_interaction& it, double r) {
    switch (it.law) {
      case RDSIM_LAW_LJ: {
        double n = (double)it.n;
        double r6 = std::pow(it.r0 / r, n);
        return -2. * n * it.u0 / r * r6 * (r6 - 1.);
      }
      case RDSIM_LAW_TANH: {
        double a_inv = 1. / it.a;
        return it.u0 * (1. - std::pow(std::tanh((r - it.r0) * a_inv), 2.0)) * a_inv / 2.;
      }
      case RDSIM_LAW_YUKAWA:
        return -it.u0 * (1. + it.r0 / r) * std::exp(-r / it.r0) / (r * it.r0);
      case RDSIM_LAW_HARMONIC:
        return it.u0 * r;
      case RDSIM_LAW_PIECEWISE_LINEAR: {
        double r_inner = it.r0 - it.dr;
        double slope = it.u0 / it.dr;
        if (r < r_inner) return 0.0;
        return slope;
      }
    }
    return 0.0;
  }

  int update_drifts() {  // pyx:1941-2067
    std::fill(a.begin(), a.end(), 0.0);
    for (const rdsim_interaction& it : inter) {
      if (it.law == RDSIM_LAW_WALL || it.law == RDSIM_LAW_WALL93) {
        int p = it.type_a, d = it.type_b;
        for (int i1 = 0; i1 < N; i1++) {
          if (types[i1] != p) continue;
          double xv = x[(size_t)i1 * D + d], f;
          if (it.law == RDSIM_LAW_WALL) {  // pyx:1132-1145
            double a_inv = 1. / it.a;
            f = it.u0 * (1. - std::pow(std::tanh((xv - it.r0) * a_inv), 2.0)) * a_inv / 2.;
          } else {  // 9-3 wall: f = dU/dy, U = u0[(2/15)(r0/y)^9 - (r0/y)^3], y <= rc
            if (xv > it.rc) continue;
            double s = it.r0 / xv, s3 = s * s * s, s9 = s3 * s3 * s3;
            f = it.u0 / xv * (-1.2 * s9 + 3.0 * s3);
          }
          a[(size_t)i1 * D + d] += -f;
        }
        continue;
      }
      int p1_ = it.type_a, p2_ = it.type_b;
      double rc = (it.law == RDSIM_LAW_PIECEWISE_LINEAR) ? it.r0 : it.rc;  // pyx:1058
      for (int i1 = 0; i1 < N; i1++) {
        for (int i2 : nl[i1]) {
          if (mol[3 * i1] == mol[3 * i2]) continue;
          int p1, p2;
          if (types[i1] < types[i2]) { p1 = types[i1]; p2 = types[i2]; }
          else { p1 = types[i2]; p2 = types[i1]; }
          if (!(p1 == p1_ && p2 == p2_)) continue;
          double r = dxx(i1, i2);
          if (r > rc) continue;
          double f = law(it, r);
          for (int k = 0; k < D; k++) {
            double h = hat(i1, i2, k);
            a[(size_t)i1 * D + k] += f * h;
            a[(size_t)i2 * D + k] += -f * h;
          }
        }
      }
    }
    for (const BondF& b : bonds) {  // pyx:2037-2047
      double f = b.k * (dxx(b.i1, b.i2) - b.r0);
      for (int k = 0; k < D; k++) {
        double h = hat(b.i1, b.i2, k);
        a[(size_t)b.i1 * D + k] += f * h;
        a[(size_t)b.i2 * D + k] += -f * h;
      }
    }
    for (const AngleF& an : angles) {  // pyx:2052-2066 with pyx:1341-1407
      int i1 = an.i1, i2 = an.i2, i3 = an.i3;
      double h = 0.;
      for (int k = 0; k < D; k++) h += hat(i2, i1, k) * hat(i2, i3, k);
      double theta;
      if (h < -1.) {
        if (h < -1.0000001) {
          char buf[160];
          snprintf(buf, sizeof buf,
                   "Inner product of units vectors is smaller than -1. Value = %.17g", h);
          g_err = buf;
          if (!err_code) { err_code = RDSIM_ERR_ANGLE_DOMAIN; err_value = h; err_step = step; }
          return RDSIM_ERR_ANGLE_DOMAIN;
        }
        h = -1.;
        theta = M_PI;
      } else {
        theta = std::acos(h);
      }
      double prefac;
      // angle_is_pi == 0: each term's own flag instead of the late-bound one
      if (angle_is_pi != 0 ? angle_is_pi > 0 : an.pi > 0) {
        if (theta < an.thr)
          prefac = an.k0 * (theta - an.theta0) / (std::sqrt(1. - std::pow(h, 2.0)));
        else
          prefac = -an.k0 / (1. - std::pow(theta - an.theta0, 2.0) / 6. +
                             std::pow(theta - an.theta0, 4.0) / (120.));
      } else {
        prefac = an.k0 * (theta - an.theta0) / (std::sqrt(1. - std::pow(h, 2.0)));
      }
      for (int k = 0; k < D; k++) {
        double f = prefac / dxx(i2, i1) * (hat(i2, i3, k) - h * hat(i2, i1, k));
        a[(size_t)i1 * D + k] += f;
        a[(size_t)i2 * D + k] -= f;
        f = prefac / dxx(i2, i3) * (hat(i2, i1, k) - h * hat(i2, i3, k));
        a[(size_t)i3 * D + k] += f;
        a[(size_t)i2 * D + k] -= f;
      }
    }
    return 0;
  }

  void compute_rates() {  // pyx:2091-2206
    int R = (int)rx.size();
    std::fill(rates.begin(), rates.end(), 0.0);
    std::fill(total.begin(), total.end(), 0.0);
    for (int i = 0; i < R; i++) {
      const rdsim_reaction& r = rx[i];
      double* ri = &rates[(size_t)i * N];
      if (r.kind == RDSIM_RX_LINEAR) {
        for (int j = 0; j < N; j++)
          if (types[j] == r.reactant) { ri[j] = r.rate; total[j] += r.rate; }
      } else if (r.kind == RDSIM_RX_CATALYZED) {
        for (int j = 0; j < N; j++) {
          if (types[j] == r.reactant)
            for (int k : nl[j])
              if (types[k] == r.catalyst && dxx(j, k) < r.r0) { ri[j] += r.rate; total[j] += r.rate; }
          if (types[j] == r.catalyst)
            for (int k : nl[j])
              if (types[k] == r.reactant && dxx(j, k) < r.r0) { ri[k] += r.rate; total[k] += r.rate; }
        }
      } else if (r.kind == RDSIM_RX_INHIBITED) {
        int inh = r.inhibitor, inh2 = r.inhibitor2;
        for (int j = 0; j < N; j++) ri[j] = (types[j] == r.reactant) ? r.rate : 0.;
        for (int j = 0; j < N; j++) {
          int tj = types[j];
          if (tj == r.reactant)
            for (int k : nl[j])
              if ((types[k] == inh) || (types[k] == inh2))
                if (dxx(j, k) < r.r0) ri[j] -= r.rate_decrease;
          if ((tj == inh) || (tj == inh2))
            for (int k : nl[j])
              if (types[k] == r.reactant)
                if (dxx(j, k) < r.r0) ri[k] -= r.rate_decrease;
        }
        for (int j = 0; j < N; j++) {
          if (ri[j] < 0) ri[j] = 0.;
          total[j] += ri[j];
        }
      }
    }
  }

  void reaction_step(int mode, const double* u1, const double* u2) {  // pyx:2070-2223
    compute_rates();
    int R = (int)rx.size();
    for (int i = 0; i < N; i++) {
      double tr = total[i];
      double v1 = (mode & ORACLE_STREAM) ? uniform() : (u1 ? u1[i] : 1.0);
      if ((dt * tr) > v1) {
        double u = (mode & ORACLE_STREAM) ? uniform() : (u2 ? u2[i] : 1.0);
        double s = 0.;
        for (int j = 0; j < R; j++) {
          s += rates[(size_t)j * N + i] / tr;
          if (s >= u) { types[i] = rx[j].product; break; }
        }
      }
    }
  }

  void update_positions(int mode, const double* xi) {  // pyx:2225-2250
    double inc = (mode & ORACLE_NO_NOISE) ? 0. : 1.;
    for (int j = 0; j < N; j++) {
      int t = types[j];
      for (int k = 0; k < D; k++) {
        size_t q = (size_t)j * D + k;
        x[q] += fp[t] * a[q];
        double xin = (mode & ORACLE_STREAM) ? normal() : (xi ? xi[q] : 0.0);
        x[q] += inc * npf[t] * xin;
      }
    }
  }

  int apply_boundary_conditions() {  // pyx:2253-2292
    for (int j = 0; j < N; j++) {
      for (int k = 0; k < D; k++) {
        double& v = x[(size_t)j * D + k];
        if (periodic[k] < 0) {
          if (v > L[k]) v -= 2 * (v - L[k]);
          if (v < 0.) v -= 2 * v;
        } else {
          double r = std::fmod(v, L[k]);
          r += (double)((r != 0) & ((r < 0) ^ (L[k] < 0))) * L[k];
          v = r;
        }
        if ((v < 0) || (v > L[k])) {
          char buf[200];
          snprintf(buf, sizeof buf,
                   "x[%d,%d] = %.17g out of bounds. Maybe the timestep is too large "
                   "for the given the interaction parameters?", j, k, v);
          g_err = buf;
          if (!err_code) {
            err_code = RDSIM_ERR_OUT_OF_BOUNDS; err_particle = j; err_dim = k;
            err_value = v; err_step = step;
          }
          return RDSIM_ERR_OUT_OF_BOUNDS;
        }
      }
    }
    return 0;
  }
};

extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }

int oracle_create(const rdsim_system* s, int32_t history_quirk, oracle_handle** out) {
  if (!s || !out) return fail(RDSIM_ERR_ARG, "null argument");
  if (s->n_dim < 1 || s->n_dim > RDSIM_MAX_DIM) return fail(RDSIM_ERR_ARG, "n_dim out of range");
  if (s->n_particles <= 0) return fail(RDSIM_ERR_ARG, "no particles");
  auto* h = new oracle_handle();
  h->D = s->n_dim; h->N = s->n_particles; h->T = s->n_types; h->M = s->n_molecules;
  for (int k = 0; k < h->D; k++) { h->L[k] = s->L[k]; h->periodic[k] = s->periodic[k]; }
  h->dt = s->dt; h->rs = s->rs; h->ratio = s->cell_length_ratio;
  h->freq = s->neighbor_list_update_frequency; h->angle_is_pi = s->angle_is_pi;
  h->quirk = history_quirk != 0;
  h->tau.assign(s->tau_by_tauD, s->tau_by_tauD + s->n_types);
  h->fp.resize(h->T); h->npf.resize(h->T);
  for (int t = 0; t < h->T; t++) {  // pyx:488-496
    if (h->tau[t] < 0) { h->fp[t] = 0.; h->npf[t] = 0.; }
    else { h->npf[t] = std::sqrt(2. * h->dt * h->tau[t]); h->fp[t] = h->dt * h->tau[t]; }
  }
  h->inter.assign(s->interactions, s->interactions + s->n_interactions);
  h->rx.assign(s->reactions, s->reactions + s->n_reactions);
  h->tmpl.assign(s->templates, s->templates + s->n_templates);
  h->terms.assign(s->terms, s->terms + s->n_terms);
  std::memset(h->partner, 0, sizeof h->partner);
  std::memset(h->has_partner, 0, sizeof h->has_partner);
  auto add = [&](int i0, int i1) -> bool {  // pyx:1234-1263
    if (i0 < 0 || i1 < 0 || i0 >= RDSIM_MAX_TYPES || i1 >= RDSIM_MAX_TYPES) return false;
    h->partner[i0][i1] = h->partner[i1][i0] = true;
    h->has_partner[i0] = h->has_partner[i1] = true;
    return true;
  };
  for (const auto& it : h->inter)
    if (it.law != RDSIM_LAW_WALL && it.law != RDSIM_LAW_WALL93)
      if (!add(it.type_a, it.type_b)) { delete h; return fail(RDSIM_ERR_ARG, "type out of range"); }
  for (const auto& r : h->rx) {
    if (r.kind == RDSIM_RX_CATALYZED) add(r.reactant, r.catalyst);
    else if (r.kind == RDSIM_RX_INHIBITED) {
      add(r.reactant, r.inhibitor);
      if (r.inhibitor2 >= 0) add(r.reactant, r.inhibitor2);
    }
  }
  h->x.assign(s->x, s->x + (size_t)h->N * h->D);
  h->a.assign((size_t)h->N * h->D, 0.0);
  h->types.assign(s->particle_types, s->particle_types + h->N);
  h->mol.assign(s->molecule_ids, s->molecule_ids + (size_t)3 * h->N);
  h->first.assign(s->first_index_of_molecule, s->first_index_of_molecule + h->M);
  for (int t : h->types)
    if (t < 0 || t >= h->T) { delete h; return fail(RDSIM_ERR_ARG, "particle type without tau_by_tauD"); }
  h->cell_id.assign((size_t)h->N * h->D, 0);
  h->rates.assign((size_t)h->rx.size() * h->N, 0.0);
  h->total.assign(h->N, 0.0);
  h->gen = std::mt19937((std::mt19937::result_type)s->seed);  // pyx:87-108
  h->set_up_cells();
  int rc = h->set_up_bonded();
  if (rc) { delete h; return rc; }
  h->create_neighbor_list();  // pyx:2398
  rc = h->update_drifts();    // pyx:2401
  if (rc) { delete h; return rc; }
  *out = h;
  return 0;
}

int oracle_destroy(oracle_handle* h) { delete h; return 0; }

int oracle_step(oracle_handle* h, int32_t n_steps, int32_t flags, const double* xi,
                const double* u1, const double* u2) {
  size_t ND = (size_t)h->N * h->D;
  for (int s = 0; s < n_steps; s++) {  // pyx:2410-2426 -> 2296-2322
    h->step += 1;
    const double* xs = xi ? xi + (size_t)s * ND : nullptr;
    const double* a1 = u1 ? u1 + (size_t)s * h->N : nullptr;
    const double* a2 = u2 ? u2 + (size_t)s * h->N : nullptr;
    h->update_positions(flags, xs);
    int rc = h->apply_boundary_conditions();
    if (rc) return rc;
    if (h->step % h->freq == 0) h->create_neighbor_list();
    else {
      std::vector<std::vector<int>> lst = h->nl;
      h->calculate_distances(lst);
    }
    h->reaction_step(flags, a1, a2);
    rc = h->update_drifts();
    if (rc) return rc;
  }
  return 0;
}

int oracle_set_state(oracle_handle* h, const double* x, const int32_t* types) {
  if (x) h->x.assign(x, x + (size_t)h->N * h->D);
  if (types) h->types.assign(types, types + h->N);
  h->create_neighbor_list();
  return h->update_drifts();
}

int oracle_get_state(oracle_handle* h, double* x, int32_t* types) {
  if (x) std::memcpy(x, h->x.data(), sizeof(double) * h->x.size());
  if (types) for (int i = 0; i < h->N; i++) types[i] = h->types[i];
  return 0;
}

int oracle_get_drift(oracle_handle* h, double* a) {
  std::memcpy(a, h->a.data(), sizeof(double) * h->a.size());
  return 0;
}

int oracle_get_reaction_rates(oracle_handle* h, int32_t recompute, double* total) {
  if (recompute) h->compute_rates();
  std::memcpy(total, h->total.data(), sizeof(double) * h->N);
  return 0;
}

int oracle_get_pairs(oracle_handle* h, int32_t* pairs, int64_t cap, int64_t* n_pairs) {
  int64_t n = 0;
  for (int i = 0; i < h->N; i++) n += (int64_t)h->nl[i].size();
  *n_pairs = n;
  if (n > cap) return fail(RDSIM_ERR_CAPACITY, "pair buffer too small");
  int64_t p = 0;
  for (int i = 0; i < h->N; i++)
    for (int j : h->nl[i]) { pairs[2 * p] = i; pairs[2 * p + 1] = j; p++; }
  return 0;
}

int oracle_get_cell_ids(oracle_handle* h, int32_t* cell_ids) {
  for (size_t q = 0; q < h->cell_id.size(); q++) cell_ids[q] = h->cell_id[q];
  return 0;
}

int oracle_get_min_dist(oracle_handle* h, double* md) { *md = h->min_dist; return 0; }

int oracle_get_error(oracle_handle* h, int32_t* code, int64_t* particle, int32_t* dim,
                     double* value, int64_t* step) {
  *code = h->err_code; *particle = h->err_particle; *dim = h->err_dim;
  *value = h->err_value; *step = h->err_step;
  h->err_code = 0;
  return 0;
}

int oracle_set_step(oracle_handle* h, int64_t step) { h->step = step; return 0; }

// Potentials of the force laws above, truncated where the force stops
// (observables; the reference has none).  Returns U; f = dU/dr as law().
static double potential(const rdsim_interaction& it, double r) {
  switch (it.law) {
    case RDSIM_LAW_LJ: {
      double s = std::pow(it.r0 / r, (double)it.n);
      return it.u0 * s * (s - 2.);
    }
    case RDSIM_LAW_TANH:
      return it.u0 / 2. * (std::tanh((r - it.r0) / it.a) - 1.);
    case RDSIM_LAW_YUKAWA:
      return it.u0 * std::exp(-r / it.r0) / r;
    case RDSIM_LAW_HARMONIC:
      return it.u0 * r * r / 2.;
    case RDSIM_LAW_PIECEWISE_LINEAR:
      if (r < it.r0 - it.dr) return -it.u0;
      return it.u0 / it.dr * (r - it.r0);
  }
  return 0.0;
}

// Energies, virial and counts of rdsim_get_observables over the oracle's own
// neighbour list, in the loop order of update_drifts (pyx:1941-2067).
int oracle_get_observables(oracle_handle* h, rdsim_observables* out) {
  std::memset(out, 0, sizeof *out);
  const int N = h->N, D = h->D;
  std::set<uint64_t> in_range;
  for (const rdsim_interaction& it : h->inter) {
    if (it.law == RDSIM_LAW_WALL || it.law == RDSIM_LAW_WALL93) {
      for (int i = 0; i < N; i++) {
        if (h->types[i] != it.type_a) continue;
        double y = h->x[(size_t)i * D + it.type_b];
        if (it.law == RDSIM_LAW_WALL) {
          out->wall_energy += it.u0 / 2. * (std::tanh((y - it.r0) / it.a) - 1.);
        } else if (!(y > it.rc)) {
          double q = it.r0 / y, q3 = q * q * q, q9 = q3 * q3 * q3;
          out->wall_energy += it.u0 * (2. / 15. * q9 - q3);
        }
      }
      continue;
    }
    double rc = (it.law == RDSIM_LAW_PIECEWISE_LINEAR) ? it.r0 : it.rc;
    for (int i1 = 0; i1 < N; i1++) {
      for (int i2 : h->nl[i1]) {
        if (h->mol[3 * i1] == h->mol[3 * i2]) continue;
        int p1 = std::min(h->types[i1], h->types[i2]);
        int p2 = std::max(h->types[i1], h->types[i2]);
        if (!(p1 == it.type_a && p2 == it.type_b)) continue;
        double r = h->dxx(i1, i2);
        if (r > rc) continue;
        out->pair_energy += potential(it, r);
        out->virial += -r * oracle_handle::law(it, r);
        in_range.insert(h->key(std::min(i1, i2), std::max(i1, i2)));
      }
    }
  }
  for (const BondF& b : h->bonds) {
    double d = h->dxx(b.i1, b.i2);
    out->bond_energy += b.k * (d - b.r0) * (d - b.r0) / 2.;
    out->virial += -d * b.k * (d - b.r0);
  }
  for (const AngleF& an : h->angles) {
    double c = 0.;
    for (int k = 0; k < D; k++) c += h->hat(an.i2, an.i1, k) * h->hat(an.i2, an.i3, k);
    double theta = c <= -1. ? M_PI : (c >= 1. ? 0. : std::acos(c));
    out->angle_energy += an.k0 * (theta - an.theta0) * (theta - an.theta0) / 2.;
  }
  out->min_distance = h->min_dist;
  out->n_pairs = (int64_t)in_range.size();
  out->n_particles = N;
  for (int i = 0; i < N; i++)
    if (h->types[i] >= 0 && h->types[i] < RDSIM_MAX_TYPES) out->type_counts[h->types[i]] += 1;
  return 0;
}

// Pair-distance histogram of rdsim_get_rdf over all pairs (i < j).
int oracle_get_rdf(oracle_handle* h, int32_t type_a, int32_t type_b, double r_max,
                   int32_t n_bins, int32_t flags, int64_t* counts) {
  if (n_bins < 1 || !(r_max > 0)) return fail(RDSIM_ERR_ARG, "bad histogram");
  const int N = h->N, D = h->D;
  const double w = r_max / n_bins;
  auto is = [](int t, int want) { return want < 0 || t == want; };
  for (int b = 0; b < n_bins; b++) counts[b] = 0;
  for (int i = 0; i < N; i++) {
    int ti = h->types[i];
    for (int j = i + 1; j < N; j++) {
      int tj = h->types[j];
      if (!((is(ti, type_a) && is(tj, type_b)) || (is(ti, type_b) && is(tj, type_a)))) continue;
      if ((flags & RDSIM_RDF_OTHER_MOLECULES) && h->mol[3 * i] == h->mol[3 * j]) continue;
      double d2 = 0.;
      for (int k = 0; k < D; k++) {
        double v = h->x[(size_t)j * D + k] - h->x[(size_t)i * D + k];
        if (h->periodic[k] > 0) v = v - h->L[k] * std::round(v / h->L[k]);
        d2 += v * v;
      }
      double r = std::sqrt(d2);
      if (!(r < r_max)) continue;
      int b = (int)std::floor(r / w);
      counts[b < n_bins ? b : n_bins - 1] += 1;
    }
  }
  return 0;
}

}  // extern "C"
