// force64.cuh -- the drift kernel in float64: the reference's own precision
// (pyrdsim.pyx:1941-2067 with the laws of 1068-1145, the EM update of
// 2225-2250), for the "plain method" that wants float64 forces.
//
// Same structure as k_force_l (list.cuh): a CTA per run of particles, TPP
// lanes per particle walking its Verlet-list row, then one thread per
// particle for walls, bonded terms, the drift store and the fused
// Euler-Maruyama update.  Differences: pair displacements are the full 64-bit
// fixed-point differences converted to float64 (exact to the double's 53
// bits); the laws, walls and bonded terms are evaluated in float64 from the
// deck's float64 parameters with the reference's formulas (angles by acos
// with its domain check and the theta0 == pi expansion); the drift is kept
// in float64; the position increment dt D a + sqrt(2 dt D) xi is formed in
// float64 and rounded once to fixed units.  Cutoffs are decided on the
// float64 r^2 except within 1e-12 relative of rc, where the distance is
// recomputed exactly as the reference computes it (exact_dist).
#pragma once

#include "list.cuh"

namespace rd {

// A list entry with the neighbour's full fixed-point words.
struct NbF {
  uint32_t h[3], l[3];
  uint32_t m;
  int v;
};

template <int D>
__device__ inline NbF gather_full(const Args& a, int v) {
  NbF n;
  const int j = v & 0x7fffffff;
  n.v = v;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    n.h[k] = k < D ? a.xh[k][j] : 0u;
    n.l[k] = k < D ? a.xl[k][j] : 0u;
  }
  n.m = a.meta[j];
  return n;
}

// for_entries (list.cuh) with full-word gathers.
template <int D, int TPP, class Fn>
__device__ inline void for_entries_full(const SysDev& s, const Args& a, int i, int lane, int cnt,
                                        Fn&& fn) {
  constexpr int B = RD_LIST_BATCH;
  if (cnt <= a.W) {
    for (int e0 = lane; e0 < cnt; e0 += B * TPP) {
      int v[B];
#pragma unroll
      for (int u = 0; u < B; u++) {
        const int e = e0 + u * TPP;
        v[u] = e < cnt ? a.nbr[ell_index<TPP>(e, i, a.npad)] : i;
      }
      NbF nb[B];
#pragma unroll
      for (int u = 0; u < B; u++) nb[u] = gather_full<D>(a, v[u]);
#pragma unroll
      for (int u = 0; u < B; u++)
        if (e0 + u * TPP < cnt) fn(nb[u]);
    }
  } else {
    row_scan<D, TPP>(s, a, i, lane, [&](int, int v) { fn(gather_full<D>(a, v)); });
  }
}

__device__ inline unsigned long long fixed_word(uint32_t h, uint32_t l) {
  return ((unsigned long long)h << 32) | l;
}

// Float64 displacement x_j - x_i along dimension k (minimum image in periodic
// dimensions).
__device__ inline double disp_d(const SysDev& s, const Args& a, int k, int gi, int gj) {
  const unsigned long long Xi = fixed_word(a.xh[k][gi], a.xl[k][gi]);
  const unsigned long long Xj = fixed_word(a.xh[k][gj], a.xl[k][gj]);
  return __ll2double_rn((long long)(Xj - Xi)) * s.unit_d[k];
}

// f / r of one law at squared distance r2 in float64 (pyrdsim.pyx:1068-1130).
__device__ inline double law_over_r_d(const rdsim_interaction& O, double r2) {
  const double r = sqrt(r2);
  switch (O.law) {
    case RDSIM_LAW_LJ: {  // f = -2 n u0 / r * s (s - 1), s = (r0/r)^n
      const double b = O.r0 / r;
      double sn = 1.0;
      for (int e = 0; e < O.n; e++) sn *= b;
      return -2.0 * O.n * O.u0 / r * sn * (sn - 1.0) / r;
    }
    case RDSIM_LAW_TANH: {  // f = u0 (1 - tanh^2((r - r0)/a)) / (2a)
      const double t = tanh((r - O.r0) / O.a);
      return O.u0 * (1.0 - t * t) / O.a / 2.0 / r;
    }
    case RDSIM_LAW_YUKAWA:  // f = -u0 (1 + r0/r) exp(-r/r0) / (r r0)
      return -O.u0 * (1.0 + O.r0 / r) * exp(-r / O.r0) / (r * O.r0) / r;
    case RDSIM_LAW_HARMONIC:  // f = u0 r
      return O.u0;
    case RDSIM_LAW_PIECEWISE_LINEAR:  // f = u0/dr for r >= r0 - dr (checked by the caller)
      return O.u0 / O.dr / r;
  }
  return 0.0;
}

// f / r summed over the laws of one type pair at squared distance r2; the
// reference's distance decides within 1e-12 of a threshold.
template <int D>
__device__ inline double pair_force_d(const SysDev& s, const PairLaw* laws,
                                      const rdsim_interaction* ol, const Args& a, int gi, int gj,
                                      unsigned int pp, double r2) {
  const int nl = pp & 31, l0 = (pp >> 5) & 0x3ff;
  double fr = 0.0, dexact = -1.0;
  for (int l = l0; l < l0 + nl; l++) {
    const PairLaw& L = laws[l];
    const double rc2 = L.rc * L.rc;
    if (r2 > rc2 * (1.0 + 1e-12)) continue;
    if (r2 >= rc2 * (1.0 - 1e-12)) {
      if (dexact < 0) dexact = exact_dist<D>(s, a, gi, gj);
      if (dexact > L.rc) continue;
    }
    if (L.law == RDSIM_LAW_PIECEWISE_LINEAR && L.rin > 0.0) {
      const double ri2 = L.rin * L.rin;
      if (r2 < ri2 * (1.0 - 1e-12)) continue;
      if (r2 <= ri2 * (1.0 + 1e-12)) {
        if (dexact < 0) dexact = exact_dist<D>(s, a, gi, gj);
        if (dexact < L.rin) continue;
      }
    }
    fr += law_over_r_d(ol[l], r2);
  }
  return fr;
}

// Bonded terms of one particle in float64 (pyrdsim.pyx:2037-2066 with the
// angle closure of 1341-1407), gathered through slot_of like bonded_terms.
template <int D>
__device__ inline void bonded_terms_d(const SysDev& s, const Args& a, int gi, int pid, uint32_t mi,
                                      double* acc) {
  const int tm = mi >> 24;
  if (tm == 0xff) return;
  const TmplDev& T = a.tmpl[tm];
  const int loc = (mi >> 16) & 0xff;
  const int mbase = pid - loc;
  for (int e = a.atomterm[T.atom0 + loc]; e < a.atomterm[T.atom0 + loc + 1]; e++) {
    const int code = a.atomterm[e];
    const TermDev& tr = a.terms[code >> 2];
    const rdsim_term& O = a.oterms[code >> 2];
    const int role = code & 3;
    if (tr.kind == RDSIM_TERM_BOND) {  // f = U0 (d - r0) along the bond
      const int other = a.slot_of[mbase + (role == 0 ? tr.j : tr.i)];
      double v[3], d2 = 0.0;
#pragma unroll
      for (int k = 0; k < D; k++) {
        v[k] = disp_d(s, a, k, gi, other);
        d2 += v[k] * v[k];
      }
      const double d = sqrt(d2);
      const double f = O.k0 * (d - O.p0) / d;
#pragma unroll
      for (int k = 0; k < D; k++) acc[k] += f * v[k];
    } else {
      const int s1 = a.slot_of[mbase + tr.i], s2 = a.slot_of[mbase + tr.j],
                s3 = a.slot_of[mbase + tr.k];
      double u1[3], u2[3], n1 = 0.0, n2 = 0.0;
#pragma unroll
      for (int k = 0; k < D; k++) {
        u1[k] = disp_d(s, a, k, s2, s1);
        u2[k] = disp_d(s, a, k, s2, s3);
        n1 += u1[k] * u1[k];
        n2 += u2[k] * u2[k];
      }
      const double d21 = sqrt(n1), d23 = sqrt(n2);
      double h = 0.0;
#pragma unroll
      for (int k = 0; k < D; k++) {
        u1[k] /= d21;
        u2[k] /= d23;
        h += u1[k] * u2[k];
      }
      double theta;
      if (h < -1.0) {  // pyrdsim.pyx:1359-1369
        if (h < -1.0000001) record_error(a.err, RDSIM_ERR_ANGLE_DOMAIN, pid, -1, h, eff_step(a));
        h = -1.0;
        theta = 3.141592653589793;
      } else {
        theta = acos(h);
      }
      // the expansion about pi: all angles follow the flag of the last angle
      // defined (pyrdsim.pyx:1401), or each its own with angle_is_pi == 0
      const bool pi_branch = s.angle_is_pi != 0 ? s.angle_is_pi > 0 : tr.pi > 0.f;
      double prefac;
      if (pi_branch && !(theta < O.p0 - 0.1)) {
        const double dt_ = theta - O.p0, q2 = dt_ * dt_;
        prefac = -O.k0 / (1.0 - q2 / 6.0 + q2 * q2 / 120.0);
      } else {
        prefac = O.k0 * (theta - O.p0) / sqrt(1.0 - h * h);
      }
#pragma unroll
      for (int k = 0; k < D; k++) {
        const double f1 = prefac / d21 * (u2[k] - h * u1[k]);
        const double f3 = prefac / d23 * (u1[k] - h * u2[k]);
        acc[k] += role == 0 ? f1 : (role == 2 ? f3 : -(f1 + f3));
      }
    }
  }
}

// Euler-Maruyama update in float64: the increment dt D a + sqrt(2 dt D) xi
// rounded once to fixed units, then advance() (wrap or reflect).  Philox
// normals are float32 (the injected ones float64).
template <int D>
__device__ inline void em_update_d(const SysDev& s, const Args& a, int sysi, int gi, int pid,
                                   int type, const double* acc, long long em_step, int flags,
                                   const U4* w0) {
  double xi[3] = {0.0, 0.0, 0.0};
  if (!(flags & F_NO_NOISE)) {
    if (flags & F_INJECT) {
#pragma unroll
      for (int k = 0; k < D; k++) xi[k] = a.xi[(size_t)pid * D + k];
    } else {
      float xf[3] = {0.f, 0.f, 0.f};
      gaussians<D>(w0 ? *w0 : noise_words(s.seed, em_step, pid, 0u), xf);
#pragma unroll
      for (int k = 0; k < D; k++) xi[k] = xf[k];
    }
  }
  const double* td = a.typed + (size_t)sysi * 2 * MAXT;
  const double fp = td[type], np = td[MAXT + type];
#pragma unroll
  for (int k = 0; k < D; k++) {
    const double dl = fp * acc[k] + np * xi[k];
    const double v = dl * s.inv_unit_d[k];
    long long d = 0;
    // the bound of delta_fixed: |d| < 2^61 (advance() needs |d| < 2^62)
    if (!(fabs(v) < 2.3e18)) record_error(a.err, RDSIM_ERR_NONFINITE, pid, k, dl, em_step);
    else d = __double2ll_rn(v);
    advance(s, a, gi, pid, k, d, em_step);
  }
}

// Per-particle tail in float64: walls (pyrdsim.pyx:1979-1986), bonded terms,
// drift store, finiteness and skin checks, fused Euler-Maruyama update.
template <int D>
__device__ inline void force_tail_d(const SysDev& s, const WallLaw* walls,
                                    const rdsim_interaction* ow, const Args& a, int sysi, int gi,
                                    int pid, const uint32_t* xo_h, uint32_t mi, double* acc,
                                    const U4* w0) {
  const int ti = mi & 0xff;
  for (int w = 0; w < s.nwalls; w++) {
    const WallLaw& W = walls[w];
    if (W.type != ti) continue;
    const rdsim_interaction& O = ow[w];
    uint32_t h = xo_h[0];
#pragma unroll
    for (int k = 1; k < D; k++)
      if (k == W.dim) h = xo_h[k];
    const double x = fixed_to_double(s, W.dim, h, a.xl[W.dim][gi]);
    double f;
    if (W.law == RDSIM_LAW_WALL) {
      const double t = tanh((x - O.r0) / O.a);
      f = O.u0 * (1.0 - t * t) / O.a / 2.0;
    } else {
      if (x > O.rc) continue;
      const double sr = O.r0 / x, s3 = sr * sr * sr, s9 = s3 * s3 * s3;
      f = O.u0 / x * (-1.2 * s9 + 3.0 * s3);
    }
#pragma unroll
    for (int k = 0; k < D; k++)
      if (k == W.dim) acc[k] += -f;
  }
  bonded_terms_d<D>(s, a, gi, pid, mi, acc);
  if (a.flags & F_STORE_DRIFT) {
#pragma unroll
    for (int k = 0; k < D; k++) a.drift_d[k][gi] = acc[k];
  }
#pragma unroll
  for (int k = 0; k < D; k++)
    if (!isfinite(acc[k])) record_error(a.err, RDSIM_ERR_NONFINITE, pid, k, acc[k], eff_step(a));
  if (a.flags & F_CHECK_SKIN) {
    float rel2 = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) {
      const float rel = (float)(int)(xo_h[k] - a.xr[k][gi]) * s.unit_hi[k];
      rel2 += rel * rel;
    }
    if (rel2 > s.delta * s.delta)
      record_error(a.err, RDSIM_ERR_SKIN, pid, -1, (double)sqrtf(rel2), eff_step(a));
  }
  if (a.flags & F_EM) em_update_d<D>(s, a, sysi, gi, pid, ti, acc, eff_em_step(a), a.flags, w0);
}

// Drift kernel in float64.  Phase A: TPP lanes per particle sum the pair
// drift over its list entries; phase B: one thread per particle.
template <int D, int TPP>
__global__ void __launch_bounds__(LBLOCK) k_force_d(Args a) {
  constexpr int PER = LBLOCK / TPP;
  constexpr int NO = MAXI * (int)(sizeof(rdsim_interaction) / 4);
  __shared__ ListShared sh;
  __shared__ rdsim_interaction olaw[MAXI];
  __shared__ double sacc[3][PER];
  pdl_trigger();
  const Chunk ch = chunk_of<PER>(a);
  const int tid = threadIdx.x, g = tid / TPP, lane = tid % TPP;
  const bool active = g < ch.cnt;
  const int i = ch.beg + (active ? g : 0);
  {
    WordLoad<NO> lo;
    const int no = ch.nlaws * (int)(sizeof(rdsim_interaction) / 4);
    lo.load(reinterpret_cast<const int*>(a.olaws + ch.law0), no);
    list_tables<true, true, false>(sh, a, ch);
    lo.store(reinterpret_cast<int*>(olaw), no);
  }
  pdl_wait();
  const int cnt = a.ncnt[i];
  unsigned long long Xo[3] = {0ull, 0ull, 0ull};
#pragma unroll
  for (int k = 0; k < D; k++) Xo[k] = fixed_word(a.xh[k][i], a.xl[k][i]);
  const uint32_t mi = a.meta[i];
  prefetch_rows<TPP>(a, ch, cnt, active);
  __syncthreads();
  const SysDev& s = sh.sys;
  double acc[3] = {0.0, 0.0, 0.0};
  if (active && s.R2 > 0.f) {
    const int ti = mi & 0xff;
    for_entries_full<D, TPP>(s, a, i, lane, cnt, [&](const NbF& nb) {
      if (nb.v < 0) return;  // same molecule: reactions only
      double dx[3], r2 = 0.0;
#pragma unroll
      for (int k = 0; k < D; k++) {
        dx[k] = __ll2double_rn((long long)(fixed_word(nb.h[k], nb.l[k]) - Xo[k])) * s.unit_d[k];
        r2 += dx[k] * dx[k];
      }
      const int tj = nb.m & 0xff;
      if (!(r2 < (double)s.prc2[ti * MAXT + tj])) return;  // beyond every law of the pair
      const unsigned int pp = s.ppair[ti * MAXT + tj];
      const double fr = pair_force_d<D>(s, sh.laws, olaw, a, i, nb.v, pp, r2);
#pragma unroll
      for (int k = 0; k < D; k++) acc[k] += fr * dx[k];
    });
  }
#pragma unroll
  for (int o = TPP >> 1; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < D; k++) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
  }
  if (active && lane == 0) {
#pragma unroll
    for (int k = 0; k < D; k++) sacc[k][g] = acc[k];
  }
  __syncthreads();
  const int ib = ch.beg + tid;
  bool listed = false;
  int4 rec = make_int4(0, 0, 0, 0);
  if (tid < ch.cnt) {
    uint32_t xb[3] = {0u, 0u, 0u};
#pragma unroll
    for (int k = 0; k < D; k++) xb[k] = a.xh[k][ib];
    double accb[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < D; k++) accb[k] = sacc[k][tid];
    const uint32_t mb = a.meta[ib];
    const int pid = a.pid[ib];
    const bool words = (a.flags & F_RX_NEXT) ||
                       ((a.flags & F_EM) && !(a.flags & (F_NO_NOISE | F_INJECT)));
    U4 w0 = {0u, 0u, 0u, 0u};
    if (words) w0 = noise_words(s.seed, eff_em_step(a), pid, 0u);
    force_tail_d<D>(s, sh.walls, a.owalls + ch.wall0, a, ch.sys, ib, pid, xb, mb, accb,
                    words ? &w0 : nullptr);
    if (a.flags & F_RX_NEXT) {
      a.meta_out[ib] = mb;
      rec = make_int4(ib, (int)mb, a.ncnt[ib], pid);
      listed = rx_may_react<D>(s, (int)(mb & 0xff), rec.z, pid, eff_em_step(a), &w0);
    }
  }
  if (a.flags & F_RX_NEXT) {
    const unsigned int bal = __ballot_sync(0xffffffffu, listed);
    if (bal) {
      const int lane32 = threadIdx.x & 31, leader = __ffs(bal) - 1;
      const int p = rx_slot(eff_em_step(a));
      int base = 0;
      if (lane32 == leader) base = atomicAdd(a.rx_count + p, __popc(bal));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (listed) a.rx_list[(size_t)p * a.npad + base + __popc(bal & ((1u << lane32) - 1u))] = rec;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.rx_count[rx_slot(eff_step(a) + 2)] = 0;
}

// Stand-alone float64 EM update of every particle (first step of a call).
template <int D>
__global__ void k_em_d(Args a, const int* sid) {
  pdl_trigger();
  pdl_wait();
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= a.n_total) return;
  const int sysi = sid[gi];
  const SysDev& s = a.sys[sysi];
  double acc[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < D; k++) acc[k] = a.drift_d[k][gi];
  em_update_d<D>(s, a, sysi, gi, a.pid[gi], a.meta[gi] & 0xff, acc, a.em_step, a.flags, nullptr);
}

}  // namespace rd
