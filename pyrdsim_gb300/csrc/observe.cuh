// observe.cuh -- float64 observables of one system at the current state.
//
// k_observe: one thread per particle (sorted order) sums, in float64, the
// pair energies and virials of its Verlet-list row (each pair once, by the
// lower sorted index), its wall energies and the bonded terms it heads
// (bond or angle whose first atom it is), and takes the minimum listed
// partner distance; a block reduction writes one partial per CTA.
// k_observe_sum adds the partials in a fixed order (deterministic results).
// Counts (pairs in range, particles per type) are integer atomics.
//
// k_rdf: pair-distance histogram.  Particles are binned in the cells of the
// last rebuild and have moved by at most delta since, so every pair closer
// than r_max now lies within a stencil of h cells, h = floor((r_max +
// 2 delta) / cell length) + 1 per dimension (all cells once where the
// stencil would wrap onto itself).  One shared-memory histogram per CTA.
#pragma once

#include "list.cuh"

namespace rd {

constexpr int OBS_BLOCK = 128;
constexpr int OBS_NSUM = 6;  // pair, wall, bond, angle energy, virial, min distance
constexpr int RDF_MAX_BINS = 8192;

struct ObsArgs {
  const rdsim_interaction* laws;   // float64 parameters, same order as Args::laws
  const rdsim_interaction* walls;  // same order as Args::walls
  const rdsim_term* terms;         // same order as Args::terms
  double* part;                    // [CTAs][OBS_NSUM]
  double* sums;                    // [OBS_NSUM] results of k_observe_sum
  unsigned long long* counts;      // [1 + MAXT]: pairs in range, particles per type
  int sys, tpp, nblocks, pad;
};

// Potential U and force magnitude f = dU/dr of one pair law at float64
// distance r; f follows pyrdsim.pyx:1068-1130.
__device__ inline double law_potential(const rdsim_interaction& it, double r, double& f) {
  switch (it.law) {
    case RDSIM_LAW_LJ: {
      const double s = pow(it.r0 / r, (double)it.n);
      f = -2.0 * it.n * it.u0 / r * s * (s - 1.0);
      return it.u0 * s * (s - 2.0);
    }
    case RDSIM_LAW_TANH: {
      const double t = tanh((r - it.r0) / it.a);
      f = it.u0 * (1.0 - t * t) / (2.0 * it.a);
      return 0.5 * it.u0 * (t - 1.0);
    }
    case RDSIM_LAW_YUKAWA: {
      const double e = exp(-r / it.r0);
      f = -it.u0 * (1.0 + it.r0 / r) * e / (r * it.r0);
      return it.u0 * e / r;
    }
    case RDSIM_LAW_HARMONIC:
      f = it.u0 * r;
      return 0.5 * it.u0 * r * r;
    case RDSIM_LAW_PIECEWISE_LINEAR:
      if (r < it.r0 - it.dr) {
        f = 0.0;
        return -it.u0;
      }
      f = it.u0 / it.dr;
      return f * (r - it.r0);
  }
  f = 0.0;
  return 0.0;
}

// Wall potential at coordinate y (pyrdsim.pyx:1132-1145; 9-3 wall cut at rc).
__device__ inline double wall_potential(const rdsim_interaction& w, double y) {
  if (w.law == RDSIM_LAW_WALL) return 0.5 * w.u0 * (tanh((y - w.r0) / w.a) - 1.0);
  if (y > w.rc) return 0.0;
  const double s = w.r0 / y, s3 = s * s * s, s9 = s3 * s3 * s3;
  return w.u0 * (2.0 / 15.0 * s9 - s3);
}

// Minimum-image vector x_j - x_i and distance in float64, with the same
// operations as exact_dist (pyrdsim.pyx:1619-1633).
template <int D>
__device__ inline double exact_vec(const SysDev& s, const Args& a, int gi, int gj, double* v) {
  double d2 = 0.0;
#pragma unroll
  for (int k = 0; k < D; k++) {
    const double xi = fixed_to_double(s, k, a.xh[k][gi], a.xl[k][gi]);
    const double xj = fixed_to_double(s, k, a.xh[k][gj], a.xl[k][gj]);
    double d = __dsub_rn(xj, xi);
    if (((s.periodic >> k) & 1) && !(fabs(d) < 0.49 * s.L[k]))
      d = __dsub_rn(d, __dmul_rn(s.L[k], round(__ddiv_rn(d, s.L[k]))));
    v[k] = d;
    d2 = __dadd_rn(d2, __dmul_rn(d, d));
  }
  return __dsqrt_rn(d2);
}

// Sum (or minimum, q == OBS_NSUM - 1) of OBS_NSUM values over the CTA;
// thread 0 receives the result.
template <int NT>
__device__ inline void block_reduce(double* v) {
  __shared__ double red[NT / 32][OBS_NSUM];
#pragma unroll
  for (int q = 0; q < OBS_NSUM; q++)
    for (int o = 16; o > 0; o >>= 1) {
      const double u = __shfl_down_sync(0xffffffffu, v[q], o);
      v[q] = q == OBS_NSUM - 1 ? fmin(v[q], u) : v[q] + u;
    }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int q = 0; q < OBS_NSUM; q++) red[w][q] = v[q];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int ww = 1; ww < NT / 32; ww++)
#pragma unroll
      for (int q = 0; q < OBS_NSUM; q++)
        v[q] = q == OBS_NSUM - 1 ? fmin(v[q], red[ww][q]) : v[q] + red[ww][q];
}

template <int D>
__global__ void __launch_bounds__(OBS_BLOCK) k_observe(Args a, ObsArgs o) {
  __shared__ unsigned int stype[MAXT];
  __shared__ unsigned int spairs;
  const SysDev& s = a.sys[o.sys];
  if (threadIdx.x < MAXT) stype[threadIdx.x] = 0u;
  if (threadIdx.x == 0) spairs = 0u;
  __syncthreads();
  double v[OBS_NSUM] = {0.0, 0.0, 0.0, 0.0, 0.0, INFINITY};
  const int i = s.p0 + (int)blockIdx.x * OBS_BLOCK + (int)threadIdx.x;
  if (i < s.p0 + s.n) {
    const uint32_t mi = a.meta[i];
    const int ti = mi & 0xff;
    atomicAdd(&stype[ti], 1u);
    unsigned int npairs = 0;
    // listed pairs (both directions are listed; the lower index sums)
    auto visit = [&](int ent) {
      if (ent & LIST_SAME_MOL) return;
      const int j = ent;
      double dv[3];
      const double r = exact_vec<D>(s, a, i, j, dv);
      v[5] = fmin(v[5], r);
      if (j < i) return;
      const int tj = a.meta[j] & 0xff;
      const unsigned int pp = s.ppair[ti * MAXT + tj];
      const int nl = pp & 31, l0 = (pp >> 5) & 0x3ff;
      bool in_range = false;
      for (int l = l0; l < l0 + nl; l++) {
        const rdsim_interaction& L = o.laws[s.law0 + l];
        const double rc = L.law == RDSIM_LAW_PIECEWISE_LINEAR ? L.r0 : L.rc;
        if (r > rc) continue;  // pyrdsim.pyx:1988-2030
        double f;
        v[0] += law_potential(L, r, f);
        v[4] -= r * f;
        in_range = true;
      }
      npairs += in_range ? 1u : 0u;
    };
    const int cnt = a.ncnt[i];
    if (cnt <= a.W) {
      for (int e = 0; e < cnt; e++)
        visit(a.nbr[((e / o.tpp) * a.npad + i) * o.tpp + e % o.tpp]);
    } else {
      row_scan<D, 1>(s, a, i, 0, [&](int, int ent) { visit(ent); });
    }
    if (npairs) atomicAdd(&spairs, npairs);
    // walls
    for (int w = 0; w < s.nwalls; w++) {
      const rdsim_interaction& W = o.walls[s.wall0 + w];
      if (W.type_a != ti) continue;
      const int d = W.type_b;
      v[1] += wall_potential(W, fixed_to_double(s, d, a.xh[d][i], a.xl[d][i]));
    }
    // bonded terms headed by this particle (role 0: it is atom i of the term)
    const int tm = mi >> 24;
    if (tm != 0xff) {
      const TmplDev& T = a.tmpl[tm];
      const int loc = (mi >> 16) & 0xff;
      const int mbase = a.pid[i] - loc;
      for (int e = a.atomterm[T.atom0 + loc]; e < a.atomterm[T.atom0 + loc + 1]; e++) {
        const int code = a.atomterm[e];
        if (code & 3) continue;
        const TermDev& tr = a.terms[code >> 2];
        const rdsim_term& ot = o.terms[code >> 2];
        if (tr.kind == RDSIM_TERM_BOND) {
          double dv[3];
          const double d = exact_vec<D>(s, a, i, a.slot_of[mbase + tr.j], dv);
          const double f = ot.k0 * (d - ot.p0);
          v[2] += 0.5 * f * (d - ot.p0);
          v[4] -= d * f;
        } else {
          // theta from the unit vectors as pyrdsim.pyx:1341-1364 forms them
          const int s2 = a.slot_of[mbase + tr.j], s3 = a.slot_of[mbase + tr.k];
          double v1[3], v2[3];
          const double d21 = exact_vec<D>(s, a, s2, i, v1);
          const double d23 = exact_vec<D>(s, a, s2, s3, v2);
          double c = 0.0;
#pragma unroll
          for (int k = 0; k < D; k++) c += (v1[k] / d21) * (v2[k] / d23);
          const double theta = c <= -1.0 ? 3.141592653589793 : (c >= 1.0 ? 0.0 : acos(c));
          v[3] += 0.5 * ot.k0 * (theta - ot.p0) * (theta - ot.p0);
        }
      }
    }
  }
  block_reduce<OBS_BLOCK>(v);
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < OBS_NSUM; q++) o.part[(size_t)blockIdx.x * OBS_NSUM + q] = v[q];
    if (spairs) atomicAdd(o.counts, (unsigned long long)spairs);
  }
  if (threadIdx.x < MAXT && stype[threadIdx.x])
    atomicAdd(o.counts + 1 + threadIdx.x, (unsigned long long)stype[threadIdx.x]);
}

// One CTA: thread t adds the partials of CTAs t, t + 128, ... in order, then
// the fixed-shape block reduction.
__global__ void __launch_bounds__(OBS_BLOCK) k_observe_sum(ObsArgs o) {
  double v[OBS_NSUM] = {0.0, 0.0, 0.0, 0.0, 0.0, INFINITY};
  for (int b = threadIdx.x; b < o.nblocks; b += OBS_BLOCK)
#pragma unroll
    for (int q = 0; q < OBS_NSUM; q++) {
      const double u = o.part[(size_t)b * OBS_NSUM + q];
      v[q] = q == OBS_NSUM - 1 ? fmin(v[q], u) : v[q] + u;
    }
  block_reduce<OBS_BLOCK>(v);
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < OBS_NSUM; q++) o.sums[q] = v[q];
}

struct RdfArgs {
  unsigned long long* counts;  // [nbins]
  double r_max, width;         // bin width r_max / nbins
  float r2_hi;                 // float32 bound of r_max^2 (guard band)
  int sys, type_a, type_b, nbins, flags;
  int h[3];                    // stencil half-width in cells
};

__device__ inline bool type_is(int t, int want) { return want < 0 || t == want; }

template <int D>
__global__ void __launch_bounds__(OBS_BLOCK) k_rdf(Args a, RdfArgs o) {
  __shared__ unsigned int hist[RDF_MAX_BINS];
  for (int b = threadIdx.x; b < o.nbins; b += OBS_BLOCK) hist[b] = 0u;
  __syncthreads();
  const SysDev& s = a.sys[o.sys];
  const int i = s.p0 + (int)blockIdx.x * OBS_BLOCK + (int)threadIdx.x;
  if (i < s.p0 + s.n) {
    const int ti = a.meta[i] & 0xff;
    if (type_is(ti, o.type_a) || type_is(ti, o.type_b)) {
      const int moli = a.mol[i];
      int c[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
      bool all[3] = {true, true, true};
      uint32_t xi[3] = {0u, 0u, 0u};
#pragma unroll
      for (int k = 0; k < D; k++) {
        xi[k] = a.xh[k][i];
        c[k] = cell_coord(s, k, a.xr[k][i]);
        const bool per = (s.periodic >> k) & 1;
        all[k] = per && 2 * o.h[k] + 1 >= s.nc[k];
        if (all[k]) {
          lo[k] = 0;
          hi[k] = s.nc[k] - 1;
        } else if (per) {
          lo[k] = c[k] - o.h[k];
          hi[k] = c[k] + o.h[k];
        } else {
          lo[k] = max(c[k] - o.h[k], 0);
          hi[k] = min(c[k] + o.h[k], s.nc[k] - 1);
        }
      }
      for (int cz = lo[2]; cz <= hi[2]; cz++)
        for (int cy = lo[1]; cy <= hi[1]; cy++)
          for (int cx = lo[0]; cx <= hi[0]; cx++) {
            const int cc[3] = {cx, cy, cz};
            int g = 0, mult = 1;
#pragma unroll
            for (int k = 0; k < D; k++) {
              int ck = cc[k];
              if (ck < 0) ck += s.nc[k];
              else if (ck >= s.nc[k]) ck -= s.nc[k];
              g += ck * mult;
              mult *= s.nc[k];
            }
            const int jb = a.cell_start[s.c0 + g], je = a.cell_start[s.c0 + g + 1];
            for (int j = max(jb, i + 1); j < je; j++) {
              const int tj = a.meta[j] & 0xff;
              if (!((type_is(ti, o.type_a) && type_is(tj, o.type_b)) ||
                    (type_is(ti, o.type_b) && type_is(tj, o.type_a))))
                continue;
              if ((o.flags & RDSIM_RDF_OTHER_MOLECULES) && a.mol[j] == moli) continue;
              float r2 = 0.f;
#pragma unroll
              for (int k = 0; k < D; k++) {
                const float d = (float)(int)(a.xh[k][j] - xi[k]) * s.unit_hi[k];
                r2 += d * d;
              }
              if (r2 > o.r2_hi) continue;
              const double r = exact_dist<D>(s, a, i, j);
              if (!(r < o.r_max)) continue;
              const int b = min((int)floor(__ddiv_rn(r, o.width)), o.nbins - 1);
              atomicAdd(&hist[b], 1u);
            }
          }
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < o.nbins; b += OBS_BLOCK)
    if (hist[b]) atomicAdd(o.counts + b, (unsigned long long)hist[b]);
}

}  // namespace rd
