// kernels.cuh -- sm_103a device code of the simulation step shared by the
// list kernels (list.cuh): pair laws, walls, bonded terms, Euler-Maruyama
// update, reaction propensities and draws, and the cell-list rebuild.
//
//   k_bin / k_scan_* / k_scatter / k_order : cell-list rebuild, a warp-
//       aggregated counting sort of all systems' particles into cells
//       (replaces create_neighbor_list, pyrdsim.pyx:1448-1587)
//   k_em<D>         : stand-alone Euler-Maruyama update
//   hooks           : reference cell ids, neighbour pairs, snapshots
#pragma once

#include <cuda_runtime.h>

#include "device.cuh"

namespace rd {

__device__ inline void record_error(ErrDev* e, int code, long long particle, int dim,
                                    double value, long long step) {
  if (atomicCAS(&e->code, 0, code) == 0) {
    e->particle = particle;
    e->dim = dim;
    e->value = value;
    e->step = step;
  }
}

// Programmatic dependent launch: pdl_trigger lets the next kernel of the
// stream be scheduled while this one runs; pdl_wait blocks until the kernels
// before this one have completed and their writes are visible.  Every kernel
// waits before it touches memory that earlier work writes; only tables
// written at create time are read before the wait.  Without the launch
// attribute both are no-ops.
__device__ inline void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ inline void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// The step the CTA of a period kernel is at (F_PERIOD): its drift of step n
// performs the update of step n + 1.
static __shared__ long long period_step;

__device__ inline long long eff_step(const Args& a) {
  if (a.flags & F_PERIOD) return period_step;
  return a.step_base ? *a.step_base + a.step : a.step;
}
__device__ inline long long eff_em_step(const Args& a) {
  if (a.flags & F_PERIOD) return period_step + 1;
  return a.step_base ? *a.step_base + a.em_step : a.em_step;
}

static __global__ void k_set_counter(long long* c, long long v, int add) {
  pdl_trigger();
  pdl_wait();
  if (add) *c += v;
  else *c = v;
}

// Cell coordinate along dimension k of high word h: floor(h nc / 2^32) in
// periodic dimensions, floor(h nc / 2^30) in reflecting ones (their high
// words span [0, 2^30]; x = L falls into the last cell) -- shifts, no 64-bit
// division.  Reflecting dimensions hold signed values (an initial position
// may lie below 0 until the first boundary step); those count as cell 0.
__device__ inline int cell_coord(const SysDev& s, int k, uint32_t h) {
  unsigned long long v = h;
  if (!((s.periodic >> k) & 1) && (int)h < 0) v = 0;
  const int c = (int)((v * (unsigned long long)s.nc[k]) >> s.hshift[k]);
  return c >= s.nc[k] ? s.nc[k] - 1 : c;
}

__device__ inline double fixed_to_double(const SysDev& s, int k, uint32_t h, uint32_t l) {
  unsigned long long X = ((unsigned long long)h << 32) | l;
  if ((s.periodic >> k) & 1) return __dmul_rn(__ull2double_rn(X), s.unit_d[k]);
  return __dmul_rn(__ll2double_rn((long long)X), s.unit_d[k]);
}

// Binary significand and exponent of a finite non-zero double: |v| = m 2^e
// with m in [2^52, 2^53).
__host__ __device__ inline unsigned long long significand(double v, int* e) {
  int ex = 0;
  const double f = frexp(fabs(v), &ex);
  *e = ex - 53;
  return (unsigned long long)ldexp(f, 53);
}

// float64 -> 64-bit fixed point, exactly: periodic dimensions give
// round(frac(x / L) * 2^64) mod 2^64 (x taken modulo L; halves round up),
// reflecting ones llround(x / L * Si).  128-bit integer arithmetic on the
// significands, so every host and the device give the same value.  False
// for a non-finite x.
__host__ __device__ inline bool fixed_from_double(double x, double L, bool periodic,
                                                  long long Si, unsigned long long* out) {
  typedef unsigned __int128 u128;
  if (!(x - x == 0.0)) return false;  // inf or nan
  int eL = 0;
  const u128 mL = significand(L, &eL);
  if (periodic) {
    const double f = fmod(x, L);  // exact, |f| < L, the sign of x
    if (f == 0.0) {
      *out = 0ull;
      return true;
    }
    int ef = 0;
    const u128 mf = significand(f, &ef);
    // y = |f| 2^64 / L = mf 2^s / mL with s <= 64 (|f| < L)
    const int sh = ef + 64 - eL;
    u128 N = 0, Dn = 1;
    if (sh >= 0) {
      N = mf << sh;
      Dn = mL;
    } else if (-sh < 70) {
      N = mf;
      Dn = mL << (-sh);
    }
    // f >= 0: floor(y + 1/2); f < 0: 2^64 - ceil(y - 1/2)
    const bool neg = f < 0.0;
    const u128 q = neg ? (2 * N + Dn - 1) / (2 * Dn) : (2 * N + Dn) / (2 * Dn);
    const unsigned long long X = (unsigned long long)q;
    *out = neg ? 0ull - X : X;
    return true;
  }
  if (x == 0.0) {
    *out = 0ull;
    return true;
  }
  int ea = 0;
  const u128 ma = significand(x, &ea);
  // y = |x| Si / L = ma Si 2^s / mL with s <= 1 (|x| <= L (1 + 1e-9))
  const int sh = ea - eL;
  const u128 N0 = ma * (u128)(unsigned long long)Si;
  u128 N = 0, Dn = 1;
  if (sh >= 0) {
    N = N0 << sh;
    Dn = mL;
  } else if (-sh < 74) {
    N = N0;
    Dn = mL << (-sh);
  }
  const long long q = (long long)((2 * N + Dn) / (2 * Dn));  // half away from zero
  *out = (unsigned long long)(x < 0.0 ? -q : q);
  return true;
}

// Words that other CTAs of a running period kernel write (positions and
// type words of other particles) are read there with strong relaxed loads
// (coherent at GPU scope, not cached in L1), so that no acquire fence has
// to invalidate the SM's L1, which holds the list rows and the CTA's own
// words.  Elsewhere plain loads.  RD_PERIOD_CG: 0 plain loads after an
// acquire fence, 1 ld.global.cg, 2 ld.relaxed.gpu.
#ifndef RD_PERIOD_CG
#define RD_PERIOD_CG 2
#endif
__device__ inline uint32_t ldw(const Args& a, const uint32_t* p) {
#if RD_PERIOD_CG == 1
  if (a.flags & F_PERIOD) return __ldcg(p);
#elif RD_PERIOD_CG == 2
  if (a.flags & F_PERIOD) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
  }
#endif
  return *p;
}

// Distance of two particles exactly as pyrdsim.pyx:1619-1633 computes it
// (float64, C round() minimum image, pow(v, 2) summed in dimension order).
template <int D>
__device__ double exact_dist(const SysDev& s, const Args& a, int gi, int gj) {
  double d2 = 0.0;
#pragma unroll
  for (int k = 0; k < D; k++) {
    double xi = fixed_to_double(s, k, ldw(a, a.xh[k] + gi), ldw(a, a.xl[k] + gi));
    double xj = fixed_to_double(s, k, ldw(a, a.xh[k] + gj), ldw(a, a.xl[k] + gj));
    double v = __dsub_rn(xj, xi);
    // minimum image; round(v / L) is 0 whenever |v| < 0.49 L, which holds for
    // every pair of adjacent cells except in boxes of three cells or fewer
    if (((s.periodic >> k) & 1) && !(fabs(v) < 0.49 * s.L[k]))
      v = __dsub_rn(v, __dmul_rn(s.L[k], round(__ddiv_rn(v, s.L[k]))));
    d2 = __dadd_rn(d2, __dmul_rn(v, v));
  }
  return __dsqrt_rn(d2);
}

// Reciprocal of r2 > 0: the hardware approximation and one Newton step
// (within about one ulp).
__device__ inline float recip(float r2) {
  float w;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(w) : "f"(r2));
  return fmaf(w, fmaf(-r2, w, 1.0f), w);
}

// f / r of the Lennard-Jones n = 6 law, g(w) = c0 s (s - 1) w with w = 1/r^2
// and s = (c1 w)^3.  The law amplifies the relative error of w about
// sevenfold (g ~ w^7 near contact), so the rounding of w is removed to first
// order: with eta = w r2 - 1 (exact by fma), g(w / (1 + eta)) =
// g(w) - eta w g'(w) and w g'(w) = c0 s (7 s - 4) w.
__device__ inline float lj6_over_r(float c0, float c1, float r2, float w) {
  const float eta = fmaf(w, r2, -1.0f);
  const float q = c1 * w;  // (r0/r)^2
  const float s = q * q * q;
  const float cs = c0 * s;
  const float g = cs * (s - 1.0f) * w;
  return fmaf(-eta, cs * fmaf(7.0f, s, -4.0f) * w, g);
}

// A 128-bit unsigned integer rounded to the nearest float32: the top 64
// significant bits, with the bits below them folded into a sticky bit (which
// lies far below float32's rounding position), converted once.
__device__ inline float u128_to_float(unsigned __int128 v) {
  const unsigned long long hi = (unsigned long long)(v >> 64);
  if (hi == 0ull) return __ull2float_rn((unsigned long long)v);
  const int sh = 64 - __clzll((long long)hi);
  const unsigned long long top = (unsigned long long)(v >> sh);
  const unsigned long long sticky = ((unsigned long long)v << (64 - sh)) != 0ull ? 1ull : 0ull;
  return ldexpf(__ull2float_rn(top | sticky), sh);
}

// Displacement x_j - x_i along dimension k from the full fixed-point words
// (minimum image in periodic dimensions), rounded once to float32 before the
// unit is applied: bonded terms, whose partners may lie anywhere in the box.
__device__ inline float disp_full(const SysDev& s, const Args& a, int k, int gi, int gj) {
  const unsigned long long Xi = ((unsigned long long)ldw(a, a.xh[k] + gi) << 32) | ldw(a, a.xl[k] + gi);
  const unsigned long long Xj = ((unsigned long long)ldw(a, a.xh[k] + gj) << 32) | ldw(a, a.xl[k] + gj);
  return __ll2float_rn((long long)(Xj - Xi)) * s.unitf[k];
}

// f / r of one pair law at squared distance r2 (float32); inv_r2 = recip(r2).
__device__ inline float eval_pair(const PairLaw& L, float r2, float inv_r2) {
  switch (L.law) {
    case RDSIM_LAW_LJ: {  // f = -2 n u0 / r * s (s - 1), s = (r0/r)^n
      if (L.n == 6) return lj6_over_r(L.c0, L.c1, r2, inv_r2);
      const float q = L.c1 * inv_r2;  // (r0/r)^2
      float s;
      if ((L.n & 1) == 0) {
        s = 1.0f;
        for (int e = 0; e < (L.n >> 1); e++) s *= q;
      } else {
        const float b = sqrtf(q);
        s = 1.0f;
        for (int e = 0; e < L.n; e++) s *= b;
      }
      return L.c0 * s * (s - 1.0f) * inv_r2;
    }
    case RDSIM_LAW_TANH: {  // f = u0 (1 - tanh^2 z) / (2a), z = (r - r0)/a
      const float ir = rsqrtf(r2);
      const float z = (r2 * ir - L.c1) * L.c2;
      const float e = expf(-2.0f * fabsf(z));
      return L.c0 * 4.0f * e / ((1.0f + e) * (1.0f + e)) * ir;
    }
    case RDSIM_LAW_YUKAWA: {  // f = -u0 (1 + r0/r) exp(-r/r0) / (r r0)
      const float ir = rsqrtf(r2);
      return L.c0 * (1.0f + L.c1 * ir) * expf(-r2 * ir * L.c2) * inv_r2;
    }
    case RDSIM_LAW_HARMONIC:  // f = u0 r
      return L.c0;
    case RDSIM_LAW_PIECEWISE_LINEAR:  // f = u0/dr for r >= r0 - dr
      return L.c0 * rsqrtf(r2);
  }
  return 0.0f;
}

// f / r summed over the laws of one type pair (pp = first << 5 | count) at
// squared distance r2; near a cutoff the float64 distance decides
// (pyrdsim.pyx:1988-2030).  gi, gj: sorted indices of the pair.
template <int D>
__device__ inline float pair_force(const SysDev& s, const PairLaw* laws, const Args& a, int gi,
                                   int gj, unsigned int pp, float r2) {
  const int nl = pp & 31, l0 = (pp >> 5) & 0x3ff;
  const float inv_r2 = recip(r2);
  float fr = 0.f;
  double dexact = -1.0;
  for (int l = l0; l < l0 + nl; l++) {
    const PairLaw& L = laws[l];
    if (r2 > L.rc2_hi) continue;
    if (r2 >= L.rc2_lo) {
      if (dexact < 0) dexact = exact_dist<D>(s, a, gi, gj);
      if (dexact > L.rc) continue;
    }
    if (L.law == RDSIM_LAW_PIECEWISE_LINEAR) {
      if (r2 < L.in2_lo) continue;
      if (r2 <= L.in2_hi) {
        if (dexact < 0) dexact = exact_dist<D>(s, a, gi, gj);
        if (dexact < L.rin) continue;
      }
    }
    fr += eval_pair(L, r2, inv_r2);
  }
  return fr;
}

// Block-wide copies of words from global to shared memory (blockDim.x ==
// NT).  All loads are issued before any store: through generic pointers
// the compiler could not otherwise move a load past the previous iteration's
// store, and every iteration would wait a full memory round trip.
template <int MAXN, int NT = BLOCK>
struct WordLoad {
  static constexpr int IT = MAXN > 0 ? (MAXN + NT - 1) / NT : 1;
  int v[IT];
  __device__ inline void load(const int* __restrict__ src, int n) {
#pragma unroll
    for (int u = 0; u < IT; u++) {
      const int q = (int)threadIdx.x + u * NT;
      v[u] = q < n ? __ldg(src + q) : 0;
    }
  }
  __device__ inline void store(int* __restrict__ dst, int n) const {
#pragma unroll
    for (int u = 0; u < IT; u++) {
      const int q = (int)threadIdx.x + u * NT;
      if (q < n) dst[q] = v[u];
    }
  }
};

__device__ inline long long delta_fixed(float d, float inv_unit_hi, bool* bad) {
  float v = d * inv_unit_hi;
  // non-finite, or beyond 2^29 high units (an eighth of a periodic box, half
  // a reflecting one): |result| < 2^62, which advance() relies on
  if (!(fabsf(v) < 536870912.0f)) {
    *bad = true;
    return 0;
  }
  float fl = floorf(v);
  int hi = (int)fl;
  float frac = v - fl;
  unsigned int lo = __float2uint_rn(frac * 4294967296.0f);
  return (long long)hi * 4294967296LL + (long long)lo;
}

__device__ inline double uniform53(uint32_t hi, uint32_t lo) {
  unsigned long long m = (((unsigned long long)hi << 32) | lo) >> 11;
  return __dadd_rn(__dmul_rn(__ull2double_rn(m), 1.1102230246251565e-16), 5.551115123125783e-17);
}

// Counter-based draws of one particle at one step.  The tag-0 words give
// the Gaussian increments (x, y; for D == 3 also z, w); the reaction
// uniforms take u1 from tag-0 (z, w) for D <= 2 and from tag-1 (x, y) for
// D == 3, and u2 from the other tag-1 pair.  w0 may hold the tag-0 words
// of the step already.
template <int D>
__device__ inline void u1_words(unsigned long long seed, long long step, int pid, const U4* w0,
                                uint32_t& hi, uint32_t& lo) {
  if (D <= 2) {
    const U4 w = w0 ? *w0 : noise_words(seed, step, pid, 0u);
    hi = w.z;
    lo = w.w;
  } else {
    const U4 w = noise_words(seed, step, pid, 1u);
    hi = w.x;
    lo = w.y;
  }
}

template <int D>
__device__ inline void u2_words(unsigned long long seed, long long step, int pid, uint32_t& hi,
                                uint32_t& lo) {
  const U4 w = noise_words(seed, step, pid, 1u);
  hi = D <= 2 ? w.x : w.z;
  lo = D <= 2 ? w.y : w.w;
}

// Float32 bounds [lo, hi] of uniform53(w_hi, w_lo): its top 24 bits.
__device__ inline void uniform_bounds(uint32_t whi, float& lo, float& hi) {
  lo = (float)(whi >> 8) * 5.9604644775390625e-08f;
  hi = (float)((whi >> 8) + 1u) * 5.9604644775390625e-08f;
}

template <int D>
__device__ inline void gaussians(const U4& w, float* xi) {
  float ua = (float)w.x * 2.3283064365386963e-10f + 1.1641532182693481e-10f;
  float r = sqrtf(-2.0f * logf(ua));
  float sn, cs;
  sincospif(2.0f * ((float)w.y * 2.3283064365386963e-10f), &sn, &cs);
  xi[0] = r * cs;
  if (D > 1) xi[1] = r * sn;
  if (D > 2) {
    float ub = (float)w.z * 2.3283064365386963e-10f + 1.1641532182693481e-10f;
    float r2 = sqrtf(-2.0f * logf(ub));
    float s2, c2;
    sincospif(2.0f * ((float)w.w * 2.3283064365386963e-10f), &s2, &c2);
    xi[2] = r2 * c2;
  }
}

// Advances coordinate k of particle gi by d fixed units (|d| < 2^62) and
// applies the boundary condition (pyrdsim.pyx:2253-2292): an exact wrap in
// periodic dimensions, a reflection at 0 and L in reflecting ones, where X
// lies in [-S, S] (S = 2^62), so X + d and the reflections stay within
// int64.  Writes the high, low and pair words.
// X: the coordinate's current fixed-point value.
__device__ inline void advance_x(const SysDev& s, const Args& a, int gi, int pid, int k,
                                 long long d, long long em_step, unsigned long long X) {
  if ((s.periodic >> k) & 1) {
    X += (unsigned long long)d;
  } else {
    // reflect (pyrdsim.pyx:2275-2280)
    long long Xs = (long long)X + d;
    const long long Si = s.Si[k];
    if (Xs > Si) Xs = Si - (Xs - Si);
    if (Xs < 0) Xs = -Xs;
    if (Xs < 0 || Xs > Si) {
      record_error(a.err, RDSIM_ERR_OUT_OF_BOUNDS, pid, k,
                   __dmul_rn(__ll2double_rn((long long)(Xs > Si ? Si : 0)), s.unit_d[k]) +
                       __dmul_rn(__ll2double_rn((long long)(Xs > Si ? Xs - Si : Xs)),
                                 s.unit_d[k]),
                   em_step);
      Xs = Xs < 0 ? 0 : Si;
    }
    X = (unsigned long long)(long long)Xs;
  }
  a.xh_out[k][gi] = (uint32_t)(X >> 32);
  a.xl_out[k][gi] = (uint32_t)X;
  a.xp_out[k][gi] = (uint32_t)(X >> s.ps[k]);
}

__device__ inline void advance(const SysDev& s, const Args& a, int gi, int pid, int k,
                               long long d, long long em_step) {
  advance_x(s, a, gi, pid, k, d, em_step,
            ((unsigned long long)a.xh[k][gi] << 32) | a.xl[k][gi]);
}

// The words of one particle that its per-particle tail reads, loaded by the
// caller: current high and low words, high words at the last rebuild, and
// (optionally) its standard normals of the update.
struct TailIn {
  uint32_t xh[3], xl[3], xr[3];
  const float* xi;                // nullptr: drawn from w0 / Philox / xi buffer
};

// Euler-Maruyama update + boundary conditions of one particle in fixed point
// (pyrdsim.pyx:2240-2292): x += dt D a + sqrt(2 dt D) xi, then reflect or wrap.
template <int D>
__device__ inline void em_update_in(const SysDev& s, const Args& a, int gi, int pid, int type,
                                    const float* acc, long long em_step, int flags,
                                    const U4* w0, const TailIn& t) {
  float xi[3] = {0.f, 0.f, 0.f};
  if (!(flags & F_NO_NOISE)) {
    if (t.xi) {
#pragma unroll
      for (int k = 0; k < D; k++) xi[k] = t.xi[k];
    } else if (flags & F_INJECT) {
#pragma unroll
      for (int k = 0; k < D; k++) xi[k] = (float)a.xi[(size_t)pid * D + k];
    } else {
      gaussians<D>(w0 ? *w0 : noise_words(s.seed, em_step, pid, 0u), xi);
    }
  }
  const float fp = s.fp[type], np = s.npf[type];
#pragma unroll
  for (int k = 0; k < D; k++) {
    bool bad = false;
    float dl = fp * acc[k] + np * xi[k];
    long long d = delta_fixed(dl, s.inv_unit_hi[k], &bad);
    if (bad) record_error(a.err, RDSIM_ERR_NONFINITE, pid, k, (double)dl, em_step);
    advance_x(s, a, gi, pid, k, d, em_step, ((unsigned long long)t.xh[k] << 32) | t.xl[k]);
  }
}

template <int D>
__device__ inline TailIn tail_load(const Args& a, int gi) {
  TailIn t;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    t.xh[k] = k < D ? a.xh[k][gi] : 0u;
    t.xl[k] = k < D ? a.xl[k][gi] : 0u;
    t.xr[k] = k < D ? a.xr[k][gi] : 0u;
  }
  t.xi = nullptr;
  return t;
}

template <int D>
__device__ inline void em_update(const SysDev& s, const Args& a, int gi, int pid, int type,
                                 const float* acc, long long em_step, int flags,
                                 const U4* w0 = nullptr) {
  em_update_in<D>(s, a, gi, pid, type, acc, em_step, flags, w0, tail_load<D>(a, gi));
}

// ---------------------------------------------------------------------------
// Bonded terms of one particle (pyrdsim.pyx:2037-2066), gathered: the
// particle evaluates every bond and angle it takes part in, reading its
// partners' positions through slot_of (caller index -> sorted slot).
template <int D>
__device__ inline void bonded_terms(const SysDev& s, const Args& a, int gi, int pid, uint32_t mi,
                                    float* acc) {
  const int tm = mi >> 24;
  if (tm == 0xff) return;
  const TmplDev& T = a.tmpl[tm];
  const int loc = (mi >> 16) & 0xff;
  const int mbase = pid - loc;
  float xo[3];
  for (int e = a.atomterm[T.atom0 + loc]; e < a.atomterm[T.atom0 + loc + 1]; e++) {
    const int code = a.atomterm[e];
    const TermDev& tr = a.terms[code >> 2];
    const int role = code & 3;
    if (tr.kind == RDSIM_TERM_BOND) {
      const int other = a.slot_of[mbase + (role == 0 ? tr.j : tr.i)];
      // f = k (d - r0) / d (pyrdsim.pyx:2037-2047).  A stiff bond near rest
      // cancels in d - r0: where every dimension has the same fixed unit,
      // d^2 - r0^2 is formed exactly in 128-bit integers (units unit^2) and
      // d - r0 = (d^2 - r0^2) / (d + r0) keeps float32 precision relative
      // to itself.  Otherwise the full-word float32 displacement is used.
      float f;
      if (s.bond128) {
        unsigned __int128 S2 = 0;
#pragma unroll
        for (int k = 0; k < D; k++) {
          const unsigned long long Xi = ((unsigned long long)a.xh[k][gi] << 32) | a.xl[k][gi];
          const unsigned long long Xj =
              ((unsigned long long)ldw(a, a.xh[k] + other) << 32) | ldw(a, a.xl[k] + other);
          const long long dd = (long long)(Xj - Xi);
          const unsigned long long m = dd < 0 ? 0ull - (unsigned long long)dd : (unsigned long long)dd;
          S2 += (unsigned __int128)m * m;
          xo[k] = __ll2float_rn(dd) * s.unitf[k];
        }
        const unsigned __int128 R0 = ((unsigned __int128)tr.r0q_hi << 64) | tr.r0q_lo;
        const bool longer = S2 >= R0;
        const float ex = u128_to_float(longer ? S2 - R0 : R0 - S2) * s.unit2f;
        const float d = sqrtf(u128_to_float(S2) * s.unit2f);
        const float dmr = (longer ? ex : -ex) / (d + tr.p0);
        f = tr.k0 * dmr / d;
      } else {
        float d2 = 0.f;
#pragma unroll
        for (int k = 0; k < D; k++) {
          xo[k] = disp_full(s, a, k, gi, other);
          d2 = fmaf(xo[k], xo[k], d2);
        }
        const float d = sqrtf(d2);
        f = tr.k0 * (d - tr.p0) / d;
      }
#pragma unroll
      for (int k = 0; k < D; k++) acc[k] += f * xo[k];
    } else {
      const int s1 = a.slot_of[mbase + tr.i], s2 = a.slot_of[mbase + tr.j],
                s3 = a.slot_of[mbase + tr.k];
      float v1[3], v2[3], n1 = 0.f, n2 = 0.f;
#pragma unroll
      for (int k = 0; k < D; k++) {
        v1[k] = disp_full(s, a, k, s2, s1);
        v2[k] = disp_full(s, a, k, s2, s3);
        n1 = fmaf(v1[k], v1[k], n1);
        n2 = fmaf(v2[k], v2[k], n2);
      }
      const float d21 = sqrtf(n1), d23 = sqrtf(n2);
      float c = 0.f, sn;
#pragma unroll
      for (int k = 0; k < D; k++) {
        v1[k] /= d21;
        v2[k] /= d23;
        c += v1[k] * v2[k];
      }
      if (D == 2) {
        sn = fabsf(v1[0] * v2[1] - v1[1] * v2[0]);
      } else if (D == 3) {
        const float cx = v1[1] * v2[2] - v1[2] * v2[1];
        const float cy = v1[2] * v2[0] - v1[0] * v2[2];
        const float cz = v1[0] * v2[1] - v1[1] * v2[0];
        sn = sqrtf(cx * cx + cy * cy + cz * cz);
      } else {
        sn = 0.f;
      }
      // theta from atan2(|u1 x u2|, u1.u2): well conditioned near 0 and pi,
      // where acos(h) loses half its digits in float32
      const float theta = atan2f(sn, c);
      float prefac;
      // the expansion about pi: all angles follow the flag of the last angle
      // defined (pyrdsim.pyx:1401), or each its own with angle_is_pi == 0
      const bool pi_branch = s.angle_is_pi != 0 ? s.angle_is_pi > 0 : tr.pi > 0.f;
      if (pi_branch && !(theta < tr.thr)) {
        const float dt_ = theta - tr.p0, d2_ = dt_ * dt_;
        prefac = -tr.k0 / (1.0f - d2_ / 6.0f + d2_ * d2_ / 120.0f);
      } else {
        prefac = tr.k0 * (theta - tr.p0) / sn;
      }
#pragma unroll
      for (int k = 0; k < D; k++) {
        const float f1 = prefac / d21 * (v2[k] - c * v1[k]);
        const float f3 = prefac / d23 * (v1[k] - c * v2[k]);
        acc[k] += role == 0 ? f1 : (role == 2 ? f3 : -(f1 + f3));
      }
    }
  }
}

// Per-particle tail of the drift kernels, on one thread per particle: walls
// (pyrdsim.pyx:1979-1986), bonded terms, drift store, finiteness and skin
// checks, and the fused Euler-Maruyama update.  acc holds the pair drift.
template <int D>
__device__ inline void force_tail_in(const SysDev& s, const WallLaw* walls, const Args& a, int gi,
                                     int pid, const TailIn& t, uint32_t mi, float* acc,
                                     const U4* w0 = nullptr) {
  const uint32_t* xo_h = t.xh;
  const int ti = mi & 0xff;
  // walls (pyrdsim.pyx:1979-1986)
  for (int w = 0; w < s.nwalls; w++) {
    const WallLaw& W = walls[w];
    if (W.type != ti) continue;
    uint32_t h = xo_h[0];
#pragma unroll
    for (int k = 1; k < D; k++)
      if (k == W.dim) h = xo_h[k];
    float f;
    if (W.law == RDSIM_LAW_WALL) {
      const float z = (float)((long long)h - W.hr0) * s.unit_hi[W.dim] * W.c2;
      const float e = expf(-2.0f * fabsf(z));
      f = W.c0 * 4.0f * e / ((1.0f + e) * (1.0f + e));
    } else {
      // the high word alone first (it is at most the coordinate): all but
      // the particles near the wall stop here
      const float yh = (((s.periodic >> W.dim) & 1) ? (float)h : (float)(int)h) *
                       s.unit_hi[W.dim];
      if (yh > W.rc_hi) continue;
      // the full coordinate; reflecting ones are signed (an initial
      // position may lie below 0)
      uint32_t l = t.xl[0];
#pragma unroll
      for (int k = 1; k < D; k++)
        if (k == W.dim) l = t.xl[k];
      const unsigned long long X = ((unsigned long long)h << 32) | l;
      const float y = (((s.periodic >> W.dim) & 1) ? __ull2float_rn(X)
                                                    : __ll2float_rn((long long)X)) *
                      s.unitf[W.dim];
      if (y > W.rc_hi) continue;
      if (y >= W.rc_lo) {
        const double yd = fixed_to_double(s, W.dim, h, l);
        if (yd > W.rc) continue;
      }
      const float sr = W.c1 / y, s3 = sr * sr * sr, s9 = s3 * s3 * s3;
      f = W.c0 / y * (-1.2f * s9 + 3.0f * s3);
    }
#pragma unroll
    for (int k = 0; k < D; k++)
      if (k == W.dim) acc[k] += -f;
  }
  bonded_terms<D>(s, a, gi, pid, mi, acc);
  if (a.flags & F_STORE_DRIFT) {
#pragma unroll
    for (int k = 0; k < D; k++) a.drift[k][gi] = acc[k];
  }
#pragma unroll
  for (int k = 0; k < D; k++)
    if (!isfinite(acc[k])) record_error(a.err, RDSIM_ERR_NONFINITE, pid, k, (double)acc[k], eff_step(a));
  if (a.flags & F_CHECK_SKIN) {
    // displacement since the last rebuild: keeps every pair within range in
    // adjacent cells, in the Verlet list and within rs of each other at that
    // rebuild
    float rel2 = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) {
      const float rel = (float)(int)(xo_h[k] - t.xr[k]) * s.unit_hi[k];
      rel2 += rel * rel;
    }
    if (rel2 > s.delta * s.delta)
      record_error(a.err, RDSIM_ERR_SKIN, pid, -1, (double)sqrtf(rel2), eff_step(a));
  }
  if (a.flags & F_EM) em_update_in<D>(s, a, gi, pid, ti, acc, eff_em_step(a), a.flags, w0, t);
}

// The same with the words loaded here (xo_h: the current high words).
template <int D>
__device__ inline void force_tail(const SysDev& s, const WallLaw* walls, const Args& a, int gi,
                                  int pid, const uint32_t* xo_h, uint32_t mi, float* acc,
                                  const U4* w0 = nullptr) {
  TailIn t = tail_load<D>(a, gi);
#pragma unroll
  for (int k = 0; k < D; k++) t.xh[k] = xo_h[k];
  force_tail_in<D>(s, walls, a, gi, pid, t, mi, acc, w0);
}

// ---------------------------------------------------------------------------
// Propensity of one reaction for a particle of type ti with c counted
// neighbours (pyrdsim.pyx:2091-2206).
__device__ inline double rx_rate(const RxDev& R, int ti, int c) {
  double v = 0.0;  // reaction_rates[r, particle]
  if (R.reactant != ti) return v;
  if (R.kind == RDSIM_RX_LINEAR) return R.rate;
  if (R.kind == RDSIM_RX_CATALYZED) {
    for (int e = 0; e < c; e++) v = __dadd_rn(v, R.rate);
    return v;
  }
  v = R.rate;
  for (int e = 0; e < c; e++) v = __dsub_rn(v, R.dec);
  return v < 0 ? 0.0 : v;
}

// Float64 total propensity of a type-ti particle (pyrdsim.pyx:2091-2206,
// file order, repeated additions).
__device__ inline double rx_total(const SysDev& s, const RxDev* rx, int ti, const uint32_t* cw) {
  double total = 0.0;
  for (int r = 0; r < s.nrx; r++) {
    const RxDev& R = rx[r];
    if (R.reactant != ti) continue;
    const int c = (cw[r >> 1] >> (16 * (r & 1))) & 0xffff;
    if (R.kind == RDSIM_RX_LINEAR) {
      total = __dadd_rn(total, R.rate);
    } else if (R.kind == RDSIM_RX_CATALYZED) {
      for (int e = 0; e < c; e++) total = __dadd_rn(total, R.rate);
    } else {
      total = __dadd_rn(total, rx_rate(R, ti, c));
    }
  }
  return total;
}

// Per-particle tail of the reaction kernels, on one thread per particle:
// propensities in file order, the draw and the new type
// (pyrdsim.pyx:2091-2222).  cw holds the neighbour counts of the
// neighbour-dependent reactions, two 16-bit counters per word; pid is the
// particle's caller index.  The reference decides in float64; when every
// reaction of the type adds a non-negative term (linear, catalysed), the
// two comparisons are first made in float32 against the bounds of the
// uniforms with a relative margin of 4e-6 (the float32 sums err by less than
// 1e-6), and only an undecided comparison is redone in float64.
// react_decide returns the new type of a type-ti particle (caller index pid)
// at the kernel's step; react_tail writes it (or, with F_RATES_ONLY, the
// total propensity).
template <int D>
__device__ inline int react_decide(const SysDev& s, const RxDev* rx, const Args& a, int pid,
                                   int ti, const uint32_t* cw, const U4* w0 = nullptr) {
  int newt = ti;
  const bool any = (s.rx_any_mask >> ti) & 1;
  if (any) {  // pyrdsim.pyx:2211-2222
    const long long step = eff_step(a);
    const bool inject = (a.flags & F_INJECT) != 0;
    // the uniforms and their float32 bounds
    uint32_t h1 = 0, l1 = 0;
    float u1lo, u1hi;
    if (inject) {
      u1lo = __double2float_rd(a.u1[pid]);
      u1hi = __double2float_ru(a.u1[pid]);
    } else {
      u1_words<D>(s.seed, step, pid, w0, h1, l1);
      uniform_bounds(h1, u1lo, u1hi);
    }
    const bool screen = (s.rx_screen_mask >> ti) & 1;
    float tf = 0.f;
    int fires = -1;  // -1: undecided
    constexpr float M = 4e-6f;
    if (screen) {
      for (int r = 0; r < s.nrx; r++) {
        const RxDev& R = rx[r];
        if (R.reactant != ti) continue;
        const int c = (cw[r >> 1] >> (16 * (r & 1))) & 0xffff;
        tf += R.kind == RDSIM_RX_LINEAR ? R.ratef : R.ratef * (float)c;
      }
      const float p = s.dtf * tf;
      if (p * (1.0f + M) < u1lo) fires = 0;
      else if (p * (1.0f - M) > u1hi) fires = 1;
    }
    double total = -1.0;
    if (fires < 0) {
      total = rx_total(s, rx, ti, cw);
      const double u1 = inject ? a.u1[pid] : uniform53(h1, l1);
      fires = __dmul_rn(s.dt, total) > u1 ? 1 : 0;
    }
    if (fires) {
      uint32_t h2 = 0, l2 = 0;
      float u2lo, u2hi;
      if (inject) {
        u2lo = __double2float_rd(a.u2[pid]);
        u2hi = __double2float_ru(a.u2[pid]);
      } else {
        u2_words<D>(s.seed, step, pid, h2, l2);
        uniform_bounds(h2, u2lo, u2hi);
      }
      int pick = -1;  // reaction index; -1 undecided, nrx: none
      if (screen && tf > 0.f) {
        float acc = 0.f;
        for (int r = 0; r < s.nrx && pick < 0; r++) {
          const RxDev& R = rx[r];
          float rf = 0.f;
          if (R.reactant == ti) {
            const int c = (cw[r >> 1] >> (16 * (r & 1))) & 0xffff;
            rf = R.kind == RDSIM_RX_LINEAR ? R.ratef : R.ratef * (float)c;
          }
          acc += rf / tf;
          if (acc * (1.0f + M) < u2lo) continue;  // not reached yet
          if (acc * (1.0f - M) >= u2hi) pick = r;
          else break;  // undecided
        }
        if (pick < 0 && acc * (1.0f + M) < u2lo) pick = s.nrx;  // no product reached
      }
      if (pick < 0) {  // exact selection (pyrdsim.pyx:2216-2222)
        if (total < 0.0) total = rx_total(s, rx, ti, cw);
        const double u2 = inject ? a.u2[pid] : uniform53(h2, l2);
        double accu = 0.0;
        pick = s.nrx;
        for (int r = 0; r < s.nrx; r++) {
          const RxDev& R = rx[r];
          const int c = (cw[r >> 1] >> (16 * (r & 1))) & 0xffff;
          accu = __dadd_rn(accu, __ddiv_rn(rx_rate(R, ti, c), total));
          if (accu >= u2) {
            pick = r;
            break;
          }
        }
      }
      if (pick < s.nrx) newt = rx[pick].product;
    }
  }
  return newt;
}

template <int D>
__device__ inline void react_tail(const SysDev& s, const RxDev* rx, const Args& a, int gi,
                                  int pid, uint32_t mi, const uint32_t* cw) {
  const int ti = mi & 0xff;
  if (a.flags & F_RATES_ONLY) {
    a.rates_out[pid] = ((s.rx_any_mask >> ti) & 1) ? rx_total(s, rx, ti, cw) : 0.0;
    return;
  }
  a.meta_out[gi] = (mi & 0xffffff00u) | (uint32_t)react_decide<D>(s, rx, a, pid, ti, cw);
}

// ---------------------------------------------------------------------------
// Stand-alone EM update of every particle (first step of a call).
template <int D>
__global__ void k_em(Args a, const int* sid) {
  pdl_trigger();
  pdl_wait();
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= a.n_total) return;
  const SysDev& s = a.sys[sid[gi]];
  float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int k = 0; k < D; k++) acc[k] = a.drift[k][gi];
  em_update<D>(s, a, gi, a.pid[gi], a.meta[gi] & 0xff, acc, a.em_step, a.flags);
}

// ---------------------------------------------------------------------------
// Cell-list rebuild.
// ctr (graph replays): the device step counter, advanced here by `add` at
// the start of a rebuild period (the kernels that read it run after this one).
template <int D>
__global__ void k_bin(const SysDev* sysv, const int* sid, const uint32_t* x0, const uint32_t* x1,
                      const uint32_t* x2, int n, int* cell_of, int* rank_of, int* count,
                      long long* ctr, long long add) {
  pdl_trigger();
  pdl_wait();
  if (ctr && blockIdx.x == 0 && threadIdx.x == 0) *ctr += add;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool valid = i < n;
  int gcell = -1 - lane;
  if (valid) {
    const SysDev& s = sysv[sid[i]];
    const uint32_t* xs[3] = {x0, x1, x2};
    int g = 0, mult = 1;
#pragma unroll
    for (int k = 0; k < D; k++) {
      g += cell_coord(s, k, xs[k][i]) * mult;
      mult *= s.nc[k];
    }
    gcell = s.c0 + g;
  }
  const unsigned int peers = __match_any_sync(0xffffffffu, gcell);
  const int leader = __ffs(peers) - 1;
  int base = 0;
  if (valid && lane == leader) base = atomicAdd(&count[gcell], __popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (valid) {
    cell_of[i] = gcell;
    rank_of[i] = base + __popc(peers & ((1u << lane) - 1u));
  }
}

// Exclusive scan of count[0..n) into start[0..n]; two passes, no waits.
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = 256 * SCAN_ITEMS;

// The same in one CTA when n <= SCAN1_T * SCAN1_I (one launch instead of
// two).  Warp w owns the contiguous segment [w * seg, (w + 1) * seg), loaded
// 32 items per instruction (coalesced) into registers; the warp totals are
// scanned across the CTA, then every warp scans its segment with shuffles.
constexpr int SCAN1_T = 1024;
constexpr int SCAN1_I = 32;

static __global__ void __launch_bounds__(SCAN1_T) k_scan_one(const int* count, int n, int* start) {
  pdl_trigger();
  pdl_wait();
  __shared__ int ws[SCAN1_T / 32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int seg = (((n + SCAN1_T / 32 - 1) / (SCAN1_T / 32)) + 31) & ~31;  // items per warp
  const int base = w * seg;
  int v[SCAN1_I], sum = 0;
#pragma unroll
  for (int it = 0; it < SCAN1_I; it++) {
    const int q = base + it * 32 + lane;
    v[it] = (it * 32 < seg && q < n) ? count[q] : 0;
    sum += v[it];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) ws[w] = sum;
  __syncthreads();
  if (w == 0) {
    const int x0 = ws[lane];
    int x = x0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    ws[lane] = x - x0;  // exclusive
    if (lane == 31 && tid == 31) start[n] = x;  // the total
  }
  __syncthreads();
  int run = ws[w];
#pragma unroll
  for (int it = 0; it < SCAN1_I; it++) {
    if (it * 32 >= seg) break;
    int x = v[it];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    const int q = base + it * 32 + lane;
    if (q < n) start[q] = run + x - v[it];
    run += __shfl_sync(0xffffffffu, x, 31);
  }
}

static __global__ void k_scan_partial(const int* count, int n, int* bsum) {
  pdl_trigger();
  pdl_wait();
  __shared__ int ws[8];
  const int base = blockIdx.x * SCAN_TILE;
  int s = 0;
  for (int e = threadIdx.x; e < SCAN_TILE; e += 256) {
    int q = base + e;
    if (q < n) s += count[q];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < 8; w++) t += ws[w];
    bsum[blockIdx.x] = t;
  }
}

static __global__ void k_scan_final(const int* count, int n, const int* bsum, int* start) {
  pdl_trigger();
  pdl_wait();
  __shared__ int ws[8];
  __shared__ int prefix;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  int p = 0;
  for (int b = tid; b < (int)blockIdx.x; b += 256) p += bsum[b];
  for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
  if (lane == 0) ws[w] = p;
  __syncthreads();
  if (tid == 0) {
    int t = 0;
    for (int q = 0; q < 8; q++) t += ws[q];
    prefix = t;
  }
  __syncthreads();
  const int base = blockIdx.x * SCAN_TILE + tid * SCAN_ITEMS;
  int v[SCAN_ITEMS], sum = 0;
#pragma unroll
  for (int e = 0; e < SCAN_ITEMS; e++) {
    v[e] = (base + e < n) ? count[base + e] : 0;
    sum += v[e];
  }
  int inc = sum;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  __syncthreads();
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  int off = prefix;
  for (int q = 0; q < w; q++) off += ws[q];
  int run = off + inc - sum;
#pragma unroll
  for (int e = 0; e < SCAN_ITEMS; e++) {
    if (base + e < n) start[base + e] = run;
    run += v[e];
  }
  // items past n count as zero, so the last thread of the grid holds the total
  if (blockIdx.x == gridDim.x - 1 && tid == 255) start[n] = run;
}

// Also zeroes the cell counts (consumed by the scans) for the next rebuild.
static __global__ void k_scatter(const int* cell_of, const int* rank_of, const int* start, int n,
                          int* tmp, int* count, int ncells) {
  pdl_trigger();
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (int q = i; q < ncells; q += gridDim.x * blockDim.x) count[q] = 0;
  if (i >= n) return;
  tmp[start[cell_of[i]] + rank_of[i]] = i;
}

// Deterministic order inside each cell (by caller index), then gather every
// per-particle array into its final slot.  Records types at this rebuild.
struct OrderOut {
  int* mol;
  int* pid;
  uint32_t* xr[3];
  int* slot_of;
};

template <int D>
__global__ void k_order(Args a, OrderOut o, const int* tmp, const int* cell_of,
                        const int* start, int n) {
  pdl_trigger();
  pdl_wait();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int old = tmp[k];
  const int g = cell_of[old];
  const int b = start[g], e = start[g + 1];
  const int myid = a.pid[old];
  int fin = k;
  if (e - b <= 1024) {  // larger cells keep the atomic order
    int r = 0;
    for (int q = b; q < e; q++) r += a.pid[tmp[q]] < myid ? 1 : 0;
    fin = b + r;
  }
#pragma unroll
  for (int d = 0; d < D; d++) {
    const uint32_t h = a.xh[d][old];
    a.xh_out[d][fin] = h;
    a.xl_out[d][fin] = a.xl[d][old];
    a.xp_out[d][fin] = a.xp[d][old];
    o.xr[d][fin] = h;
  }
  const uint32_t m = a.meta[old];
  a.meta_out[fin] = (m & 0xffff00ffu) | ((m & 0xffu) << 8);
  o.mol[fin] = a.mol[old];
  o.pid[fin] = myid;
  o.slot_of[myid] = fin;
}

// ---------------------------------------------------------------------------
// Hooks (tests and reports).
template <int D>
__global__ void k_to_double(const SysDev* sysv, const int* sid, Args a, double* x, int* types) {
  pdl_trigger();
  pdl_wait();
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= a.n_total) return;
  const SysDev& s = sysv[sid[gi]];
  const int pid = a.pid[gi];
#pragma unroll
  for (int k = 0; k < D; k++) x[(size_t)pid * D + k] = fixed_to_double(s, k, a.xh[k][gi], a.xl[k][gi]);
  if (types) types[pid] = a.meta[gi] & 0xff;
}

// State upload: caller-order float64 positions x and types -> the fixed-point
// arrays (slot = caller index), meta and molecule words.  bad receives the
// first problem: 1 reflecting position outside [-L, L], 2 non-finite
// position, 3 type without a tau_by_tauD entry.
struct StateOut {
  uint32_t* xh[3];
  uint32_t* xl[3];
  uint32_t* xp[3];
  uint32_t* meta;
  int* mol;
  int* pid;
  int n;
};

template <int D>
__global__ void k_from_double(const SysDev* sysv, const int* sid, const double* x,
                              const int* types, const uint32_t* meta_static,
                              const int* mol_static, StateOut a, int* bad) {
  pdl_trigger();
  pdl_wait();
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= a.n) return;
  const SysDev& s = sysv[sid[gi]];
#pragma unroll
  for (int k = 0; k < D; k++) {
    const double v = x[(size_t)gi * D + k];
    const bool per = (s.periodic >> k) & 1;
    if (!per && !(v >= -s.L[k] && v <= s.L[k] * (1.0 + 1e-9))) {
      atomicCAS(bad, 0, 1);
      return;
    }
    unsigned long long X = 0;
    if (!fixed_from_double(v, s.L[k], per, s.Si[k], &X)) {
      atomicCAS(bad, 0, 2);
      return;
    }
    a.xh[k][gi] = (uint32_t)(X >> 32);
    a.xl[k][gi] = (uint32_t)X;
    a.xp[k][gi] = (uint32_t)(X >> s.ps[k]);
  }
  const int t = types[gi];
  if (t < 0 || t >= s.ntypes) {
    atomicCAS(bad, 0, 3);
    return;
  }
  a.meta[gi] = meta_static[gi] | (uint32_t)t | ((uint32_t)t << 8);
  a.mol[gi] = mol_static[gi];
  a.pid[gi] = gi;
}

// trajectory frame: positions (float64) and types in caller order
template <int D>
__global__ void k_snapshot(const SysDev* sysv, const int* sid, Args a, double* fx, int* ft) {
  pdl_trigger();
  pdl_wait();
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= a.n_total) return;
  const SysDev& s = sysv[sid[gi]];
  const int pid = a.pid[gi];
#pragma unroll
  for (int k = 0; k < D; k++) fx[(size_t)pid * D + k] = fixed_to_double(s, k, a.xh[k][gi], a.xl[k][gi]);
  ft[pid] = a.meta[gi] & 0xff;
}

// reference cell ids floor(x / cl) (pyrdsim.pyx:1506-1508) of one system
template <int D>
__global__ void k_ref_cells(const SysDev* sysv, int sys, Args a, const double* cl, int p0, int n,
                            int pid0, int* out) {
  pdl_trigger();
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const SysDev& s = sysv[sys];
  const int gi = p0 + i;
  const int pid = a.pid[gi] - pid0;
#pragma unroll
  for (int k = 0; k < D; k++) {
    double x = fixed_to_double(s, k, a.xh[k][gi], a.xl[k][gi]);
    out[(size_t)pid * D + k] = (int)floor(__ddiv_rn(x, cl[k]));
  }
}

// neighbour list as the reference would rebuild it now (pyrdsim.pyx:1448-1587):
// bonded-list pairs plus partner-type pairs of different molecules, d <= rs.
template <int D>
__global__ void k_pairs(const SysDev* sysv, int sys, Args a, const TmplDev* tmpl, double rs,
                        float rs2_hi, int p0, int n, int pid0, int* out, unsigned long long cap,
                        unsigned long long* count) {
  pdl_trigger();
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const SysDev& s = sysv[sys];
  const int gi = p0 + i;
  const uint32_t mi = a.meta[gi];
  const int pi = a.pid[gi] - pid0;
  const int ti = mi & 0xff, loci = (mi >> 16) & 0xff, tmi = mi >> 24;
  const uint32_t bmask = tmi != 0xff ? tmpl[tmi].bondmask[loci] : 0u;
  for (int j = 0; j < n; j++) {
    const int gj = p0 + j;
    const int pj = a.pid[gj] - pid0;
    if (pj <= pi) continue;
    const uint32_t mj = a.meta[gj];
    bool listed;
    if (a.mol[gj] == a.mol[gi]) listed = (bmask >> ((mj >> 16) & 31)) & 1;
    else listed = (s.partner[ti] >> (mj & 0xff)) & 1;
    if (!listed) continue;
    float r2 = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) {
      float dx = (float)(int)(a.xh[k][gj] - a.xh[k][gi]) * s.unit_hi[k];
      r2 += dx * dx;
    }
    if (r2 > rs2_hi) continue;
    if (exact_dist<D>(s, a, gi, gj) > rs) continue;
    unsigned long long slot = atomicAdd(count, 1ull);
    if (slot < cap) {
      out[2 * slot] = pi;
      out[2 * slot + 1] = pj;
    }
  }
}

}  // namespace rd
