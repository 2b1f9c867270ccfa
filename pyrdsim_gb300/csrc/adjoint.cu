// adjoint.cu -- float64 reaction-free steps, a trajectory loss and its
// discrete adjoint (gradients with respect to the initial positions and the
// pair-law parameters), for include/rdsim_adjoint.h.
//
// Every state is binned into cells (counting sort, then each cell's members
// in index order) and gets a neighbour list: the particles of the 3^D
// cells around each particle that pass a float32 distance screen, in a fixed
// order, so all sums run in a fixed order and results are deterministic.
// The float64 kernels walk the lists with four lanes per particle: float64
// issue is scarce on this GPU (1/64 of float32), and a compact list keeps
// the lanes of a warp busy with pairs inside the cutoff.  Forward (k_adj_step): pair drift of pyrdsim.pyx:1941-2067 for
// Lennard-Jones and Yukawa laws (pyrdsim.pyx:1068-1130), the loss terms of
// the state, and the Euler-Maruyama update with injected noise and periodic
// wrap (pyrdsim.pyx:2225-2292).  Backward (k_adj_back): for state x_n and
// w = c * lambda_{n+1},
//   lambda_n = g_n + lambda_{n+1} + sum_j K_ij (w_j - w_i),
//   K_ij = f' rhat rhat^T + (f / r) (I - rhat rhat^T),
// (f = dU/dr; a_i = sum_j f rhat_ij, so d a_i / d x_j = K_ij), the loss
// gradient g_n, and the parameter gradients sum over pairs of
// df/dtheta rhat . (w_i - w_j) plus the loss's own dependence.  States of
// the backward pass are recomputed segment by segment from checkpoints.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/rdsim_adjoint.h"

namespace {

constexpr int MAXT = RDSIM_MAX_TYPES;
constexpr int MAXL = RDSIM_ADJ_MAX_LAWS;
constexpr int NG = 2 * MAXL;  // parameter gradients: (u0, r0) per law
constexpr int BLK = 128;
constexpr int SCAN_T = 1024;

thread_local std::string g_err;

int fail(int code, const std::string& m) {
  g_err = m;
  return code;
}

#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return fail(RDSIM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct Law {
  int law, n;
  double u0, r0, rc, ir0;       // ir0 = 1 / r0
  double Uc, dUc_du0, dUc_dr0;  // energy at rc and its parameter derivatives
};

struct AdjArgs {
  int N, D, nlaws;
  int nc[3], ncell;
  double L[3], cellinv[3];
  float Lf[3], Linvf[3];
  double rc2max;                // largest law cutoff^2: list entries beyond skip
  float cut2f;                  // float32 screen of the list in use
  float move2f;                 // displacement^2 allowed while a list is reused                  // float32 screen: above the largest rc^2
  double c[MAXT], s[MAXT];      // dt D and sqrt(2 dt D) per type
  double wU, wW;                // loss weights 1/K and 1/(K d V)
  unsigned char lawmask[MAXT * MAXT];  // bit l: law l applies to (ti, tj)
  Law laws[MAXL];
};

enum { F_STEP = 1, F_LOSS = 2 };
constexpr int TPP = 4;  // lanes per particle in the pair kernels

// Pair terms of one law at distance r < rc (ir = 1 / r): U (unshifted),
// f = dU/dr, fp = d2U/dr2, and the derivatives of U and f by (u0, r0).
struct PairEval {
  double U, f, fp, dU[2], df[2];
};

__host__ __device__ inline double lj_power(double q, int n) {
  // (r0 / r)^n from q = r0 / r
  if (n == 6) {
    const double q2 = q * q;
    return q2 * q2 * q2;
  }
  double s = 1.0;
  for (int e = 0; e < n; e++) s *= q;
  return s;
}

__host__ __device__ inline PairEval eval_law(const Law& w, double r, double ir) {
  PairEval p;
  if (w.law == RDSIM_LAW_LJ) {
    // U = u0 (s^2 - 2 s), s = (r0/r)^n; f = -2 n u0 s (s - 1) / r
    const double n = (double)w.n;
    const double s = lj_power(w.r0 * ir, w.n);
    const double t = 2.0 * n * s * ir;
    p.U = w.u0 * s * (s - 2.0);
    p.f = -w.u0 * t * (s - 1.0);
    p.fp = w.u0 * t * ((2.0 * n + 1.0) * s - (n + 1.0)) * ir;
    p.dU[0] = s * (s - 2.0);
    p.df[0] = -t * (s - 1.0);
    // ds/dr0 = n s / r0
    p.dU[1] = 2.0 * n * w.u0 * s * (s - 1.0) * w.ir0;
    p.df[1] = -w.u0 * t * n * (2.0 * s - 1.0) * w.ir0;
  } else {
    // Yukawa: U = u0 e / r, e = exp(-r / r0)
    const double e = exp(-r * w.ir0);
    const double ir0 = w.ir0;
    const double h = ir * ir0 + ir * ir;
    p.U = w.u0 * e * ir;
    p.f = -w.u0 * e * h;
    p.fp = w.u0 * e * ir * (ir0 * ir0 + 2.0 * ir * ir0 + 2.0 * ir * ir);
    p.dU[0] = e * ir;
    p.df[0] = -e * h;
    p.dU[1] = w.u0 * e * ir0 * ir0;
    p.df[1] = -w.u0 * e * ir0 * ir0 * ir0;
  }
  return p;
}

// Cell of coordinate x along k, wrapped into [0, nc) (positions on or
// outside the box edge map to their periodic image's cell).
__device__ inline int cell_of(const AdjArgs& g, int k, double x) {
  int c = (int)floor(x * g.cellinv[k]) % g.nc[k];
  return c < 0 ? c + g.nc[k] : c;
}

template <int D>
__global__ void k_bin(AdjArgs g, const double* __restrict__ x, int* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.N) return;
  int c = 0, mult = 1;
#pragma unroll
  for (int k = 0; k < D; k++) {
    c += cell_of(g, k, x[(size_t)i * D + k]) * mult;
    mult *= g.nc[k];
  }
  atomicAdd(count + c, 1);
}

// Exclusive scan of count[0..n) into start[0..n] and cursor[0..n), one CTA.
__global__ void __launch_bounds__(SCAN_T) k_scan(const int* __restrict__ count, int n,
                                                 int* __restrict__ start, int* __restrict__ cursor) {
  __shared__ int wsum[SCAN_T / 32];
  const int t = threadIdx.x;
  const int chunk = (n + SCAN_T - 1) / SCAN_T;
  const int b = min(t * chunk, n), e = min(b + chunk, n);
  int sum = 0;
  for (int q = b; q < e; q++) sum += count[q];
  // block exclusive scan of the per-thread sums
  int v = sum;
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, o);
    if ((t & 31) >= o) v += u;
  }
  if ((t & 31) == 31) wsum[t >> 5] = v;
  __syncthreads();
  if (t < 32) {
    int w = wsum[t];
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, w, o);
      if (t >= o) w += u;
    }
    wsum[t] = w;  // inclusive over warps
  }
  __syncthreads();
  int run = v - sum + ((t >> 5) > 0 ? wsum[(t >> 5) - 1] : 0);
  for (int q = b; q < e; q++) {
    start[q] = run;
    cursor[q] = run;
    run += count[q];
  }
  if (t == SCAN_T - 1) start[n] = run;
}

template <int D>
__global__ void k_fill(AdjArgs g, const double* __restrict__ x, int* __restrict__ cursor,
                       int* __restrict__ idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.N) return;
  int c = 0, mult = 1;
#pragma unroll
  for (int k = 0; k < D; k++) {
    c += cell_of(g, k, x[(size_t)i * D + k]) * mult;
    mult *= g.nc[k];
  }
  idx[atomicAdd(cursor + c, 1)] = i;
}

// Members of each cell in index order, and their float32 positions in the
// same order (the screen of the pair kernels); clears the counts for the
// next build.
template <int D>
__global__ void k_cell_sort(int ncell, const double* __restrict__ x,
                            const int* __restrict__ start, int* __restrict__ idx,
                            float* __restrict__ xs, int* __restrict__ count) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int b = start[c], e = start[c + 1];
  for (int p = b + 1; p < e; p++) {
    const int v = idx[p];
    int q = p - 1;
    while (q >= b && idx[q] > v) {
      idx[q + 1] = idx[q];
      q--;
    }
    idx[q + 1] = v;
  }
  for (int p = b; p < e; p++) {
    const int j = idx[p];
#pragma unroll
    for (int k = 0; k < D; k++) xs[(size_t)p * D + k] = (float)x[(size_t)j * D + k];
  }
  count[c] = 0;
}

// Neighbour list of one state (or of R states: the screen distance then
// includes twice the allowed displacement).  TPP lanes per particle i: lane l takes the
// members l, l + TPP, ... of each of the 3^D cells around i's cell (cells in
// a fixed order, members in index order) that pass the float32 distance
// screen and keeps them in its own sub-list nbr[(e * TPP + l) * N + i],
// e < min(count, W); ncnt[l * N + i] = count.  maxcnt receives the largest
// count (the caller enlarges W and repeats when it exceeds W).
template <int D>
__global__ void __launch_bounds__(BLK) k_adj_list(AdjArgs g, const double* __restrict__ x,
                                                  const int* __restrict__ start,
                                                  const int* __restrict__ idx,
                                                  const float* __restrict__ xs, int W,
                                                  int* __restrict__ nbr, int* __restrict__ ncnt,
                                                  int* __restrict__ maxcnt,
                                                  float* __restrict__ xr) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = t % TPP, i = t / TPP;
  int cnt = 0;
  if (i < g.N) {
    int c[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    float xf[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < D; k++) {
      const double xk = x[(size_t)i * D + k];
      xf[k] = (float)xk;
      c[k] = cell_of(g, k, xk);
      if (g.nc[k] >= 3) {
        lo[k] = c[k] - 1;
        hi[k] = c[k] + 1;
      } else {
        lo[k] = 0;
        hi[k] = g.nc[k] - 1;
      }
    }
    for (int cz = lo[2]; cz <= hi[2]; cz++)
      for (int cy = lo[1]; cy <= hi[1]; cy++)
        for (int cx = lo[0]; cx <= hi[0]; cx++) {
          const int cc[3] = {cx, cy, cz};
          int cell = 0, mult = 1;
#pragma unroll
          for (int k = 0; k < D; k++) {
            int ck = cc[k];
            if (ck < 0) ck += g.nc[k];
            else if (ck >= g.nc[k]) ck -= g.nc[k];
            cell += ck * mult;
            mult *= g.nc[k];
          }
          const int e = start[cell + 1];
          for (int p = start[cell] + lane; p < e; p += TPP) {
            float r2f = 0.f;
#pragma unroll
            for (int k = 0; k < D; k++) {
              float v = xs[(size_t)p * D + k] - xf[k];
              v -= g.Lf[k] * rintf(v * g.Linvf[k]);
              r2f += v * v;
            }
            if (r2f > g.cut2f) continue;
            const int j = idx[p];
            if (j == i) continue;
            if (cnt < W) nbr[((size_t)cnt * TPP + lane) * g.N + i] = j;
            cnt++;
          }
        }
    ncnt[(size_t)lane * g.N + i] = cnt;
    if (xr && lane == 0) {  // positions of this list, for the displacement check
#pragma unroll
      for (int k = 0; k < D; k++) xr[(size_t)i * D + k] = xf[k];
    }
  }
  const int m = __reduce_max_sync(0xffffffffu, cnt);
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(maxcnt, m);
}

// Visit, on lane `lane` of the TPP lanes of particle i, the entries of its
// sub-list, with the float64 minimum-image vector d = x_j - x_i.
template <int D, class Fn>
__device__ inline void for_list(const AdjArgs& g, const double* __restrict__ x,
                                const int* __restrict__ nbr, const int* __restrict__ ncnt, int W,
                                int i, const double* xi, int lane, Fn&& fn) {
  const int cnt = min(ncnt[(size_t)lane * g.N + i], W);
  for (int e = 0; e < cnt; e++) {
    const int j = nbr[((size_t)e * TPP + lane) * g.N + i];
    double d[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < D; k++) {
      double v = x[(size_t)j * D + k] - xi[k];
      // minimum image; rint(v / L) is 0 whenever |v| < 0.49 L
      if (!(fabs(v) < 0.49 * g.L[k])) v -= g.L[k] * rint(v / g.L[k]);
      d[k] = v;
    }
    fn(j, d);
  }
}

// Sum over the TPP lanes of one particle (xor tree: the same order on every
// lane, so all lanes hold the same value).
__device__ inline double lane_sum(double v) {
#pragma unroll
  for (int o = 1; o < TPP; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One state: loss terms (F_LOSS, accumulated per particle into lacc) and the
// step to the next state (F_STEP).  TPP lanes per particle.
template <int D, int FL>
__global__ void __launch_bounds__(BLK) k_adj_step(AdjArgs g, const double* __restrict__ x,
                                                  const int* __restrict__ nbr,
                                                  const int* __restrict__ ncnt, int W,
                                                  const int* __restrict__ types,
                                                  const double* __restrict__ noise,
                                                  double* __restrict__ x_out,
                                                  double* __restrict__ lacc,
                                                  const float* __restrict__ xr,
                                                  int* __restrict__ moved) {
  __shared__ Law slaws[MAXL];
  if (threadIdx.x < (unsigned)g.nlaws) slaws[threadIdx.x] = g.laws[threadIdx.x];
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = t % TPP;
  const int i = min(t / TPP, g.N - 1);  // surplus lanes mirror the last particle
  const bool own = t / TPP < g.N;
  const int ti = types[i];
  double xi[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < D; k++) xi[k] = x[(size_t)i * D + k];
  double a[3] = {0.0, 0.0, 0.0};
  double loss = 0.0;
  for_list<D>(g, x, nbr, ncnt, W, i, xi, lane, [&](int j, const double* d) {
    const int tj = types[j];
    const unsigned int m = g.lawmask[ti * MAXT + tj];
    if (!m) return;
    double r2 = 0.0;
#pragma unroll
    for (int k = 0; k < D; k++) r2 += d[k] * d[k];
    if (!(r2 < g.rc2max)) return;  // in the list's skin only
    const double ir = rsqrt(r2), r = r2 * ir;
    // iteration q takes each lane's q-th law: lanes of different type
    // pairs evaluate their first laws together
    for (unsigned int mm = m; mm; mm &= mm - 1) {
      const Law& w = slaws[__ffs(mm) - 1];
      if (!(r < w.rc)) continue;
      const PairEval p = eval_law(w, r, ir);
      const double fi = p.f * ir;
#pragma unroll
      for (int k = 0; k < D; k++) a[k] += fi * d[k];
      // each pair is seen from both ends: half of its loss on each
      if (FL & F_LOSS) loss += 0.5 * (g.wU * (p.U - w.Uc) - g.wW * r * p.f);
    }
  });
#pragma unroll
  for (int k = 0; k < D; k++) a[k] = lane_sum(a[k]);
  if (FL & F_LOSS) loss = lane_sum(loss);
  if (!own || lane != 0) return;
  if (xr) {
    // the list in use dates from an earlier state: it holds every pair in
    // range only while no particle has moved more than the skin allows
    float d2 = 0.f;
#pragma unroll
    for (int k = 0; k < D; k++) {
      float v = (float)xi[k] - xr[(size_t)i * D + k];
      v -= g.Lf[k] * rintf(v * g.Linvf[k]);
      d2 += v * v;
    }
    if (d2 > g.move2f) atomicOr(moved, 1);
  }
  if (FL & F_LOSS) lacc[i] += loss;
  if (FL & F_STEP) {
#pragma unroll
    for (int k = 0; k < D; k++) {
      double v = xi[k];
      v += g.c[ti] * a[k];
      v += g.s[ti] * noise[(size_t)i * D + k];
      v -= g.L[k] * floor(v / g.L[k]);
      x_out[(size_t)i * D + k] = v;
    }
  }
}

// One state of the backward pass (see the file comment).  gpart[block][NG]
// accumulates this CTA's parameter gradients over the steps, in step order.
template <int D, int FL>
__global__ void __launch_bounds__(BLK) k_adj_back(AdjArgs g, const double* __restrict__ x,
                                                  const int* __restrict__ nbr,
                                                  const int* __restrict__ ncnt, int W,
                                                  const int* __restrict__ types,
                                                  const double* __restrict__ lam_next,
                                                  double* __restrict__ lam_out,
                                                  double* __restrict__ gpart) {
  __shared__ Law slaws[MAXL];
  __shared__ double sgp[NG][BLK];  // per-thread parameter gradients
  if (threadIdx.x < (unsigned)g.nlaws) slaws[threadIdx.x] = g.laws[threadIdx.x];
#pragma unroll
  for (int q = 0; q < NG; q++) sgp[q][threadIdx.x] = 0.0;
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = t % TPP;
  const int i = min(t / TPP, g.N - 1);
  const bool own = t / TPP < g.N;
  const int ti = types[i];
  double xi[3] = {0.0, 0.0, 0.0}, wi[3] = {0.0, 0.0, 0.0}, out[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < D; k++) {
    xi[k] = x[(size_t)i * D + k];
    if (FL & F_STEP) wi[k] = g.c[ti] * lam_next[(size_t)i * D + k];
  }
  for_list<D>(g, x, nbr, ncnt, W, i, xi, lane, [&](int j, const double* d) {
    const int tj = types[j];
    const unsigned int m = g.lawmask[ti * MAXT + tj];
    if (!m) return;
    double r2 = 0.0;
#pragma unroll
    for (int k = 0; k < D; k++) r2 += d[k] * d[k];
    if (!(r2 < g.rc2max)) return;  // in the list's skin only
    const double ir = rsqrt(r2), r = r2 * ir;
    double rh[3] = {0.0, 0.0, 0.0}, dw[3] = {0.0, 0.0, 0.0};
    double rdw = 0.0;  // rhat . (w_j - w_i)
#pragma unroll
    for (int k = 0; k < D; k++) {
      rh[k] = d[k] * ir;
      if (FL & F_STEP) {
        dw[k] = g.c[tj] * lam_next[(size_t)j * D + k] - wi[k];
        rdw += rh[k] * dw[k];
      }
    }
    // iteration q takes each lane's q-th law (see k_adj_step)
    for (unsigned int mm = m; mm; mm &= mm - 1) {
      const int l = __ffs(mm) - 1;
      const Law& w = slaws[l];
      if (!(r < w.rc)) continue;
      const PairEval p = eval_law(w, r, ir);
      if (FL & F_STEP) {
        const double fr = p.f * ir;
#pragma unroll
        for (int k = 0; k < D; k++) out[k] += p.fp * rh[k] * rdw + fr * (dw[k] - rh[k] * rdw);
      }
      if (FL & F_LOSS) {
        // d loss_pair / dr times d r / d x_i = -rhat
        const double dl = g.wU * p.f - g.wW * (p.f + r * p.fp);
#pragma unroll
        for (int k = 0; k < D; k++) out[k] -= dl * rh[k];
      }
      if (j > i && own) {
#pragma unroll
        for (int q = 0; q < 2; q++) {
          double v = 0.0;
          if (FL & F_STEP) v -= p.df[q] * rdw;  // df/dtheta rhat . (w_i - w_j)
          if (FL & F_LOSS)
            v += g.wU * (p.dU[q] - (q == 0 ? w.dUc_du0 : w.dUc_dr0)) - g.wW * r * p.df[q];
          sgp[2 * l + q][threadIdx.x] += v;
        }
      }
    }
  });
#pragma unroll
  for (int k = 0; k < D; k++) out[k] = lane_sum(out[k]);
  if (own && lane == 0) {
#pragma unroll
    for (int k = 0; k < D; k++)
      lam_out[(size_t)i * D + k] = out[k] + ((FL & F_STEP) ? lam_next[(size_t)i * D + k] : 0.0);
  }
  // CTA sum of the parameter gradients in thread order, added to this CTA's
  // slot
  __syncthreads();
  if (threadIdx.x < 2 * g.nlaws) {
    double v = 0.0;
    for (int u = 0; u < BLK; u++) v += sgp[threadIdx.x][u];
    gpart[(size_t)blockIdx.x * NG + threadIdx.x] += v;
  }
}

// Sum of n values (or n rows of NG values) in a fixed order: one CTA, thread
// t adds entries t, t + BLK, ..., then a fixed tree.
__global__ void __launch_bounds__(BLK) k_sum_rows(const double* __restrict__ v, int n, int width,
                                                  double* __restrict__ out) {
  __shared__ double sh[BLK];
  for (int col = 0; col < width; col++) {
    double s = 0.0;
    for (int r = threadIdx.x; r < n; r += BLK) s += v[(size_t)r * width + col];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = BLK / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[col] = sh[0];
    __syncthreads();
  }
}

__global__ void k_scale(double* v, size_t n, double f) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] *= f;
}

unsigned nblk(int n) { return (unsigned)((n + BLK - 1) / BLK); }
// CTAs of the pair kernels (TPP lanes per particle)
unsigned pblk(int n) { return nblk(n * TPP); }

}  // namespace

struct rdsim_adjoint {
  int device = 0;
  cudaStream_t stream = nullptr;
  AdjArgs g;
  std::vector<rdsim_interaction> laws;
  int K = 1, E = 32;
  int* types = nullptr;
  // cells of the state being listed (transient)
  int *count = nullptr, *cursor = nullptr, *start = nullptr, *idx = nullptr;
  float* xs = nullptr;             // [N][D] float32 positions in cell order
  // neighbour lists of the segment's states: E + 1 slots of nbr[W][N], ncnt[N]
  int W = 0;
  int *seg_nbr = nullptr, *seg_ncnt = nullptr;
  int* maxcnt = nullptr;
  // list reuse: one list serves R consecutive states (R divides E) when no
  // particle moves more than the skin allows in between
  int R = 1, R_used = 1;
  float cut2f_exact = 0.f, cut2f_skin = 0.f;
  float* xr = nullptr;             // [N][D] float32 positions of the forward list
  int* moved = nullptr;
  double* seg_x = nullptr;         // [E][N][D] states of the current segment
  double* ckpt = nullptr;          // [nckpt][N][D] states 0, E, 2E, ...
  size_t ckpt_cap = 0;
  double* xT = nullptr;            // [N][D] final state
  double* lacc = nullptr;          // [N] per-particle loss
  double* lam[2] = {nullptr, nullptr};
  double* gpart = nullptr;         // [blocks][NG]
  double* red = nullptr;           // [NG] reduction results
  const double* xi = nullptr;      // noise of the last forward (caller's)
  int T = -1;                      // steps of the last forward
};

namespace {

void free_adj(rdsim_adjoint* h) {
  auto F = [](void* p) {
    if (p) cudaFree(p);
  };
  F(h->types); F(h->count); F(h->cursor); F(h->start); F(h->idx); F(h->xs);
  F(h->seg_nbr); F(h->seg_ncnt); F(h->maxcnt); F(h->seg_x); F(h->xr); F(h->moved);
  F(h->ckpt); F(h->xT); F(h->lacc); F(h->lam[0]); F(h->lam[1]); F(h->gpart); F(h->red);
  if (h->stream) cudaStreamDestroy(h->stream);
}

int* slot_nbr(rdsim_adjoint* h, int s) { return h->seg_nbr + (size_t)s * h->W * TPP * h->g.N; }
int* slot_ncnt(rdsim_adjoint* h, int s) { return h->seg_ncnt + (size_t)s * TPP * h->g.N; }

// (Re)allocates the neighbour-list slots for width W.
int alloc_lists(rdsim_adjoint* h, int W) {
  if (h->seg_nbr) cudaFree(h->seg_nbr);
  h->seg_nbr = nullptr;
  h->W = 0;
  const size_t slots = (size_t)h->E + 1;
  if (cudaMalloc(&h->seg_nbr, sizeof(int) * slots * W * TPP * h->g.N) != cudaSuccess)
    return fail(RDSIM_ERR_NOMEM, "neighbour lists");
  h->W = W;
  return 0;
}

template <int D>
void build_list_d(rdsim_adjoint* h, const double* x, int slot, float* xr) {
  const AdjArgs& g = h->g;
  k_bin<D><<<nblk(g.N), BLK, 0, h->stream>>>(g, x, h->count);
  k_scan<<<1, SCAN_T, 0, h->stream>>>(h->count, g.ncell, h->start, h->cursor);
  k_fill<D><<<nblk(g.N), BLK, 0, h->stream>>>(g, x, h->cursor, h->idx);
  k_cell_sort<D><<<nblk(g.ncell), BLK, 0, h->stream>>>(g.ncell, x, h->start, h->idx, h->xs,
                                                        h->count);
  k_adj_list<D><<<pblk(g.N), BLK, 0, h->stream>>>(g, x, h->start, h->idx, h->xs, h->W,
                                                   slot_nbr(h, slot), slot_ncnt(h, slot),
                                                   h->maxcnt, xr);
}

// Cells and neighbour list of state x into list slot `slot` (and its float32
// positions into xr when given).
void build_list(rdsim_adjoint* h, const double* x, int slot, float* xr = nullptr) {
  if (h->g.D == 2) build_list_d<2>(h, x, slot, xr);
  else if (h->g.D == 3) build_list_d<3>(h, x, slot, xr);
  else build_list_d<1>(h, x, slot, xr);
}

template <int D, int FL>
void step_k(rdsim_adjoint* h, const double* x, int slot, const double* noise, double* x_out,
            const float* xr) {
  k_adj_step<D, FL><<<pblk(h->g.N), BLK, 0, h->stream>>>(h->g, x, slot_nbr(h, slot),
                                                          slot_ncnt(h, slot), h->W, h->types,
                                                          noise, x_out, h->lacc, xr, h->moved);
}

template <int D>
void step_d(rdsim_adjoint* h, const double* x, int slot, const double* noise, double* x_out,
            int flags, const float* xr) {
  if (flags == F_STEP) step_k<D, F_STEP>(h, x, slot, noise, x_out, xr);
  else if (flags == F_LOSS) step_k<D, F_LOSS>(h, x, slot, noise, x_out, xr);
  else step_k<D, F_STEP | F_LOSS>(h, x, slot, noise, x_out, xr);
}

// One state's kernel (loss terms and/or the step); with xr the displacement
// since the list was built is checked.
void step(rdsim_adjoint* h, const double* x, int slot, const double* noise, double* x_out,
          int flags, const float* xr = nullptr) {
  if (h->g.D == 2) step_d<2>(h, x, slot, noise, x_out, flags, xr);
  else if (h->g.D == 3) step_d<3>(h, x, slot, noise, x_out, flags, xr);
  else step_d<1>(h, x, slot, noise, x_out, flags, xr);
}

template <int D, int FL>
void back_k(rdsim_adjoint* h, const double* x, int slot, const double* lam_next, double* lam_out) {
  k_adj_back<D, FL><<<pblk(h->g.N), BLK, 0, h->stream>>>(h->g, x, slot_nbr(h, slot),
                                                          slot_ncnt(h, slot), h->W, h->types,
                                                          lam_next, lam_out, h->gpart);
}

template <int D>
void back_d(rdsim_adjoint* h, const double* x, int slot, const double* lam_next, double* lam_out,
            int flags) {
  if (flags == F_STEP) back_k<D, F_STEP>(h, x, slot, lam_next, lam_out);
  else if (flags == F_LOSS) back_k<D, F_LOSS>(h, x, slot, lam_next, lam_out);
  else back_k<D, F_STEP | F_LOSS>(h, x, slot, lam_next, lam_out);
}

void back(rdsim_adjoint* h, const double* x, int slot, const double* lam_next, double* lam_out,
          int flags) {
  if (h->g.D == 2) back_d<2>(h, x, slot, lam_next, lam_out, flags);
  else if (h->g.D == 3) back_d<3>(h, x, slot, lam_next, lam_out, flags);
  else back_d<1>(h, x, slot, lam_next, lam_out, flags);
}

}  // namespace

extern "C" {

int rdsim_adjoint_create(const rdsim_adjoint_system* s, int32_t device, rdsim_adjoint** out) {
  if (!s || !out) return fail(RDSIM_ERR_ARG, "null argument");
  *out = nullptr;
  const int D = s->n_dim, N = s->n_particles;
  if (D < 1 || D > 3) return fail(RDSIM_ERR_ARG, "n_dim must be 1, 2 or 3");
  if (N < 1) return fail(RDSIM_ERR_ARG, "no particles");
  if (s->n_types < 1 || s->n_types > MAXT) return fail(RDSIM_ERR_ARG, "n_types out of range");
  if (s->n_laws < 0 || s->n_laws > MAXL) return fail(RDSIM_ERR_UNSUPPORTED, "at most 8 laws");
  if (s->loss_steps < 1) return fail(RDSIM_ERR_ARG, "loss_steps must be >= 1");
  if (s->checkpoint_every < 1) return fail(RDSIM_ERR_ARG, "checkpoint_every must be >= 1");
  auto* h = new rdsim_adjoint();
  std::memset(&h->g, 0, sizeof h->g);
  AdjArgs& g = h->g;
  g.N = N;
  g.D = D;
  g.nlaws = s->n_laws;
  double rc_max = 0.0, V = 1.0;
  h->E = s->checkpoint_every;
  // list reuse: R states per list (R divides E); the skin covers five
  // standard deviations of R diffusion steps of the most mobile type per
  // dimension (a particle that moves farther makes the forward pass repeat
  // itself with one list per state)
  double sig = 0.0;
  for (int t = 0; t < s->n_types; t++)
    if (s->mobility[t] > 0) sig = std::max(sig, std::sqrt(2.0 * s->dt * s->mobility[t]));
  h->R = h->E % 8 == 0 ? 8 : (h->E % 4 == 0 ? 4 : (h->E % 2 == 0 ? 2 : 1));
  const double skin_half = std::max(0.05, 5.0 * sig * std::sqrt((double)h->R) * std::sqrt((double)D));
  for (int l = 0; l < s->n_laws; l++) {
    const rdsim_interaction& it = s->laws[l];
    if (it.law != RDSIM_LAW_LJ && it.law != RDSIM_LAW_YUKAWA) {
      delete h;
      return fail(RDSIM_ERR_UNSUPPORTED, "the adjoint supports lj and yukawa laws");
    }
    if (it.type_a < 0 || it.type_b < it.type_a || it.type_b >= s->n_types || !(it.rc > 0) ||
        !(it.r0 > 0) || (it.law == RDSIM_LAW_LJ && it.n < 1)) {
      delete h;
      return fail(RDSIM_ERR_ARG, "bad law");
    }
    g.lawmask[it.type_a * MAXT + it.type_b] |= (unsigned char)(1u << l);
    g.lawmask[it.type_b * MAXT + it.type_a] |= (unsigned char)(1u << l);
    rc_max = std::max(rc_max, it.rc);
    h->laws.push_back(it);
  }
  double Lmin = 1e300, Lmax = 0.0;
  for (int k = 0; k < D; k++) {
    Lmin = std::min(Lmin, s->L[k]);
    Lmax = std::max(Lmax, s->L[k]);
  }
  // screen distances: float32 positions and minimum image err by a few
  // 1e-7 L per coordinate
  const double cut_exact = rc_max + 1e-3 + 1e-6 * Lmax;
  const double cut_skin = cut_exact + 2.0 * skin_half;
  if (rc_max <= 0 || 2.0 * cut_skin > Lmin) h->R = 1;
  const double cut_cells = h->R > 1 ? cut_skin : cut_exact;
  g.rc2max = rc_max * rc_max;
  h->cut2f_exact = (float)(cut_exact * cut_exact * (1.0 + 1e-6));
  h->cut2f_skin = (float)(cut_skin * cut_skin * (1.0 + 1e-6));
  {
    const double mv = skin_half - 1e-4 - 1e-6 * Lmax;  // float32 check, conservative
    g.move2f = (float)(mv > 0 ? mv * mv : 0.0);
  }
  for (int k = 0; k < D; k++) {
    if (!(s->L[k] >= 2.0 * rc_max) || !(s->L[k] > 0)) {
      delete h;
      return fail(RDSIM_ERR_ARG, "box length below twice the largest cutoff");
    }
    int nc = rc_max > 0 ? (int)std::floor(s->L[k] / cut_cells) : 1;
    nc = std::min(std::max(nc, 1), 1 << 12);
    if (nc < 3) nc = 1;
    g.nc[k] = nc;
    g.L[k] = s->L[k];
    g.Lf[k] = (float)s->L[k];
    g.Linvf[k] = (float)(1.0 / s->L[k]);
    g.cellinv[k] = nc / s->L[k];
    V *= s->L[k];
  }
  for (int k = D; k < 3; k++) g.nc[k] = 1;
  g.cut2f = h->R > 1 ? h->cut2f_skin : h->cut2f_exact;
  g.ncell = g.nc[0] * g.nc[1] * g.nc[2];
  for (int t = 0; t < s->n_types; t++) {
    const double Dt = s->mobility[t];
    g.c[t] = Dt > 0 ? s->dt * Dt : 0.0;
    g.s[t] = Dt > 0 ? std::sqrt(2.0 * s->dt * Dt) : 0.0;
  }
  h->K = s->loss_steps;
  g.wU = 1.0 / h->K;
  g.wW = 1.0 / (h->K * D * V);
  std::vector<int> types(s->types, s->types + N);
  for (int t : types)
    if (t < 0 || t >= s->n_types) {
      delete h;
      return fail(RDSIM_ERR_ARG, "particle type out of range");
    }
  h->device = device;
  auto bail = [&](int rc) {
    free_adj(h);
    delete h;
    return rc;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bail(fail(RDSIM_ERR_CUDA, "cudaSetDevice"));
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(RDSIM_ERR_CUDA, "cudaStreamCreate"));
  const size_t nd = (size_t)N * D;
  const size_t slots = (size_t)h->E + 1;
  bool ok = cudaMalloc(&h->types, sizeof(int) * N) == cudaSuccess &&
            cudaMalloc(&h->count, sizeof(int) * g.ncell) == cudaSuccess &&
            cudaMalloc(&h->cursor, sizeof(int) * g.ncell) == cudaSuccess &&
            cudaMalloc(&h->start, sizeof(int) * (g.ncell + 1)) == cudaSuccess &&
            cudaMalloc(&h->idx, sizeof(int) * N) == cudaSuccess &&
            cudaMalloc(&h->xs, sizeof(float) * nd) == cudaSuccess &&
            cudaMalloc(&h->seg_ncnt, sizeof(int) * slots * TPP * N) == cudaSuccess &&
            cudaMalloc(&h->maxcnt, sizeof(int)) == cudaSuccess &&
            cudaMalloc(&h->xr, sizeof(float) * nd) == cudaSuccess &&
            cudaMalloc(&h->moved, sizeof(int)) == cudaSuccess &&
            cudaMalloc(&h->seg_x, sizeof(double) * h->E * nd) == cudaSuccess &&
            cudaMalloc(&h->xT, sizeof(double) * nd) == cudaSuccess &&
            cudaMalloc(&h->lacc, sizeof(double) * N) == cudaSuccess &&
            cudaMalloc(&h->lam[0], sizeof(double) * nd) == cudaSuccess &&
            cudaMalloc(&h->lam[1], sizeof(double) * nd) == cudaSuccess &&
            cudaMalloc(&h->gpart, sizeof(double) * pblk(N) * NG) == cudaSuccess &&
            cudaMalloc(&h->red, sizeof(double) * NG) == cudaSuccess;
  if (!ok) return bail(fail(RDSIM_ERR_NOMEM, "device allocation failed"));
  {
    // sub-list width: twice the expected number of particles within the
    // screen distance per lane, plus a margin (a forward pass that finds
    // more widens it)
    const double cut = std::sqrt((double)g.cut2f);
    const double ball = D == 1 ? 2.0 * cut : (D == 2 ? M_PI * cut * cut : 4.0 / 3.0 * M_PI * cut * cut * cut);
    const double expect = std::min((double)N, N / V * ball) / TPP;
    const int W = (int)(2.0 * expect) + 8;
    int rc = alloc_lists(h, std::min(W, N));
    if (rc) return bail(rc);
  }
  if (cudaMemcpyAsync(h->types, types.data(), sizeof(int) * N, cudaMemcpyHostToDevice, h->stream) !=
          cudaSuccess ||
      cudaMemsetAsync(h->count, 0, sizeof(int) * g.ncell, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return bail(fail(RDSIM_ERR_CUDA, "upload"));
  *out = h;
  return 0;
}

int rdsim_adjoint_destroy(rdsim_adjoint* h) {
  if (!h) return 0;
  cudaSetDevice(h->device);
  free_adj(h);
  delete h;
  return 0;
}

int rdsim_adjoint_get_lists(rdsim_adjoint* h, int32_t* states_per_list, int32_t* list_width) {
  if (!h || !states_per_list || !list_width) return fail(RDSIM_ERR_ARG, "null argument");
  *states_per_list = h->R_used;
  *list_width = h->W;
  return 0;
}

int rdsim_adjoint_get_stream(rdsim_adjoint* h, void** stream) {
  if (!h || !stream) return fail(RDSIM_ERR_ARG, "null argument");
  *stream = (void*)h->stream;
  return 0;
}

int rdsim_adjoint_forward(rdsim_adjoint* h, const double* x0, const double* params,
                          const double* xi, int32_t n_steps, double* loss, double* x_final) {
  if (!h || !x0 || !params || !loss || (n_steps > 0 && !xi)) return fail(RDSIM_ERR_ARG, "null argument");
  if (n_steps < 0) return fail(RDSIM_ERR_ARG, "n_steps must be >= 0");
  if (h->K > n_steps + 1) return fail(RDSIM_ERR_ARG, "loss_steps exceeds the number of states");
  CK(cudaSetDevice(h->device));
  AdjArgs& g = h->g;
  for (int l = 0; l < g.nlaws; l++) {
    const rdsim_interaction& it = h->laws[l];
    Law& w = g.laws[l];
    w.law = it.law;
    w.n = it.n;
    w.u0 = params[2 * l];
    w.r0 = params[2 * l + 1];
    w.rc = it.rc;
    if (!(w.r0 > 0)) return fail(RDSIM_ERR_ARG, "r0 must be positive");
    w.ir0 = 1.0 / w.r0;
    const PairEval p = eval_law(w, w.rc, 1.0 / w.rc);
    w.Uc = p.U;
    w.dUc_du0 = p.dU[0];
    w.dUc_dr0 = p.dU[1];
  }
  const int N = g.N, D = g.D, E = h->E;
  const size_t nd = (size_t)N * D;
  const size_t nck = (size_t)n_steps / E + 1;
  if (nck * nd > h->ckpt_cap) {
    if (h->ckpt) cudaFree(h->ckpt);
    h->ckpt = nullptr;
    h->ckpt_cap = 0;
    if (cudaMalloc(&h->ckpt, sizeof(double) * nck * nd) != cudaSuccess)
      return fail(RDSIM_ERR_NOMEM, "checkpoint buffer");
    h->ckpt_cap = nck * nd;
  }
  const double* cur = nullptr;
  int R = h->R;
  for (int attempt = 0;; attempt++) {
    g.cut2f = R > 1 ? h->cut2f_skin : h->cut2f_exact;
    CK(cudaMemsetAsync(h->lacc, 0, sizeof(double) * N, h->stream));
    CK(cudaMemsetAsync(h->maxcnt, 0, sizeof(int), h->stream));
    CK(cudaMemsetAsync(h->moved, 0, sizeof(int), h->stream));
    CK(cudaMemcpyAsync(h->ckpt, x0, sizeof(double) * nd, cudaMemcpyDeviceToDevice, h->stream));
    // states between checkpoints alternate between seg_x[0] and seg_x[1]
    // (the segment buffer is free during the forward pass; E >= 2 there)
    cur = h->ckpt;
    const int slot = E;  // list slot of the forward pass
    for (int n = 0; n <= n_steps; n++) {
      int flags = n >= n_steps - h->K + 1 ? F_LOSS : 0;
      double* nxt = nullptr;
      if (n < n_steps) {
        flags |= F_STEP;
        const int m = n + 1;
        nxt = m % E == 0 ? h->ckpt + (size_t)(m / E) * nd : h->seg_x + (size_t)(m & 1) * nd;
      }
      if (n % R == 0) build_list(h, cur, slot, R > 1 ? h->xr : nullptr);
      step(h, cur, slot, n < n_steps ? xi + (size_t)n * nd : nullptr, nxt, flags,
           R > 1 ? h->xr : nullptr);
      if (nxt) cur = nxt;
    }
    CK(cudaGetLastError());
    int mx = 0, moved = 0;
    CK(cudaMemcpyAsync(&mx, h->maxcnt, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(&moved, h->moved, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (mx <= h->W && !moved) break;
    if (attempt > 2) return fail(RDSIM_ERR_CAPACITY, "neighbour list overflow");
    if (moved) {
      R = 1;  // a particle outran the skin: one list per state
    } else {
      // a list row overflowed: widen the lists and run the pass again
      int rc = alloc_lists(h, std::min(N, mx + mx / 4 + 4));
      if (rc) return rc;
    }
  }
  h->R_used = R;
  if (cur != h->xT) CK(cudaMemcpyAsync(h->xT, cur, sizeof(double) * nd, cudaMemcpyDeviceToDevice, h->stream));
  k_sum_rows<<<1, BLK, 0, h->stream>>>(h->lacc, N, 1, h->red);
  CK(cudaMemcpyAsync(loss, h->red, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (x_final) CK(cudaMemcpyAsync(x_final, h->xT, sizeof(double) * nd, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->xi = xi;
  h->T = n_steps;
  return 0;
}

int rdsim_adjoint_backward(rdsim_adjoint* h, double dloss, double* grad_x0, double* grad_params) {
  if (!h || !grad_x0 || !grad_params) return fail(RDSIM_ERR_ARG, "null argument");
  if (h->T < 0) return fail(RDSIM_ERR_ARG, "no forward pass to differentiate");
  CK(cudaSetDevice(h->device));
  AdjArgs& g = h->g;
  const int N = g.N, D = g.D, E = h->E, T = h->T;
  const size_t nd = (size_t)N * D;
  CK(cudaMemsetAsync(h->gpart, 0, sizeof(double) * pblk(N) * NG, h->stream));
  CK(cudaMemsetAsync(h->lam[0], 0, sizeof(double) * nd, h->stream));
  const int R = h->R_used;
  g.cut2f = R > 1 ? h->cut2f_skin : h->cut2f_exact;
  const int extra = E;  // list slot of the final state when it starts a list
  int cur = 0;     // lam[cur] holds lambda_{n+1}
  int seg = -1;    // base step of the states held in seg_x
  // states b .. b + E - 1 below T recomputed from checkpoint b / E, with the
  // lists of states b, b + R, ... in slots 0, 1, ... (the forward pass used
  // the list of state floor(n / R) R for state n; R divides E)
  auto segment = [&](int b) -> int {
    if (b == seg) return 0;
    CK(cudaMemcpyAsync(h->seg_x, h->ckpt + (size_t)(b / E) * nd, sizeof(double) * nd,
                       cudaMemcpyDeviceToDevice, h->stream));
    const int last = std::min(b + E - 1, T - 1);
    for (int q = 0; q <= last - b; q++) {
      double* xq = h->seg_x + (size_t)q * nd;
      if (q > 0) step(h, xq - nd, (q - 1) / R, h->xi + (size_t)(b + q - 1) * nd, xq, F_STEP);
      if (q % R == 0) build_list(h, xq, q / R);
    }
    seg = b;
    return 0;
  };
  for (int n = T; n >= 0; n--) {
    const double* x;
    int slot;
    if (n == T) {
      x = h->xT;
      const int r0 = (T / R) * R;
      if (r0 == T) {
        slot = extra;
        build_list(h, x, slot);
      } else {
        const int b = ((T - 1) / E) * E;
        int rc = segment(b);
        if (rc) return rc;
        slot = (r0 - b) / R;
      }
    } else {
      const int b = (n / E) * E;
      int rc = segment(b);
      if (rc) return rc;
      x = h->seg_x + (size_t)(n - b) * nd;
      slot = (n - b) / R;
    }
    int flags = n >= T - h->K + 1 ? F_LOSS : 0;
    if (n < T) flags |= F_STEP;
    back(h, x, slot, h->lam[cur], h->lam[1 - cur], flags);
    cur = 1 - cur;
  }
  CK(cudaGetLastError());
  k_sum_rows<<<1, BLK, 0, h->stream>>>(h->gpart, (int)pblk(N), NG, h->red);
  double gsum[NG];
  CK(cudaMemcpyAsync(gsum, h->red, sizeof gsum, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(grad_x0, h->lam[cur], sizeof(double) * nd, cudaMemcpyDeviceToDevice,
                     h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int q = 0; q < 2 * g.nlaws; q++) grad_params[q] = dloss * gsum[q];
  if (dloss != 1.0) {
    k_scale<<<(unsigned)((nd + BLK - 1) / BLK), BLK, 0, h->stream>>>(grad_x0, nd, dloss);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
  }
  return 0;
}

}  // extern "C"
