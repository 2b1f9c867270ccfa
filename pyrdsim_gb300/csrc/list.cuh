// list.cuh -- Verlet-list step kernels.
//
// At every rebuild k_nlist writes, for each particle in sorted order, the
// particles of the 3^D cells around its cell that lie within the list radius
// (range + 2 sqrt(D) delta) and form a listed pair at that rebuild:
// interaction partners (types at the rebuild, pyrdsim.pyx:1448-1587) of
// another molecule, or bonded-list members of its own molecule (flagged with
// LIST_SAME_MOL: they count for reactions, not for pair forces).  The drift
// kernel's displacement check bounds every particle's motion since the
// rebuild by delta per dimension, so every pair that comes within range
// during the rebuild period is in the list, and each step kernel applies the
// same distance tests as the reference to the listed pairs only.
//
// Layout: ELL of width W, interleaved by TPP so that the TPP lanes serving
// one particle read consecutive words: entry e of particle i sits at
//   ((e / TPP) * npad + i) * TPP + e % TPP.
// A particle with more than W entries keeps its full count; the step kernels
// then regenerate its row from the cells, in the same order and on the same
// lanes as the list would have delivered it, so results do not depend on W.
//
// Step kernels run in two phases per CTA of LBLOCK threads and LBLOCK / TPP
// particles.  Phase A: TPP lanes per particle walk its list and combine with
// shuffles into shared memory.  Phase B: one thread per particle runs the
// per-particle tail (walls, bonded terms, Euler-Maruyama update; or the
// reaction draw).  The data phase B needs and the warp's list rows are
// prefetched into L1 at kernel start.
#pragma once

#include "kernels.cuh"

// resident CTAs per SM the step kernels are compiled for (register budget)
#ifndef RD_LIST_MIN_BLOCKS
#define RD_LIST_MIN_BLOCKS 8
#endif
// list entries loaded per lane before their neighbours are gathered
#ifndef RD_LIST_BATCH
#define RD_LIST_BATCH 2
#endif

namespace rd {

constexpr int LBLOCK = 128;                    // threads per CTA
constexpr int LIST_SAME_MOL = (int)0x80000000;
constexpr int BUILD_LANES = 8;                 // lanes per particle in k_nlist

template <int TPP>
__device__ inline int ell_index(int e, int i, int npad) {
  return ((e / TPP) * npad + i) * TPP + (e % TPP);
}

__device__ inline void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

struct ListShared {
  SysDev sys;
  PairLaw laws[MAXI];
  WallLaw walls[MAXW];
  RxDev rx[MAXR];
};

// The CTA's run of particles: from blockIdx for a single system, else from
// the chunk table.
template <int PER>
__device__ inline Chunk chunk_of(const Args& a) {
  if (a.single) {
    Chunk c = a.chunk1;
    c.beg = blockIdx.x * PER;
    c.cnt = min(PER, a.n_total - c.beg);
    return c;
  }
  return a.chunks[blockIdx.x];
}

__device__ inline void list_tables(ListShared& sh, const Args& a, const Chunk& c, bool laws,
                                   bool walls, bool rx) {
  copy_words(reinterpret_cast<int*>(&sh.sys), reinterpret_cast<const int*>(&a.sys[c.sys]),
             (int)(sizeof(SysDev) / 4));
  if (laws)
    copy_words(reinterpret_cast<int*>(sh.laws), reinterpret_cast<const int*>(a.laws + c.law0),
               c.nlaws * (int)(sizeof(PairLaw) / 4));
  if (walls)
    copy_words(reinterpret_cast<int*>(sh.walls), reinterpret_cast<const int*>(a.walls + c.wall0),
               c.nwalls * (int)(sizeof(WallLaw) / 4));
  if (rx)
    copy_words(reinterpret_cast<int*>(sh.rx), reinterpret_cast<const int*>(a.rx + c.rx0),
               c.nrx * (int)(sizeof(RxDev) / 4));
}

// Prefetch into L1 the list words of this warp's particles: column block q
// (entries q*TPP .. q*TPP+TPP-1 of every particle of the warp) on lane q.
// Every lane of the warp calls it.
template <int TPP>
__device__ inline void prefetch_rows(const Args& a, const Chunk& ch, int cnt, bool active) {
  const int warp0 = ch.beg + ((int)(threadIdx.x & ~31u)) / TPP;
  const int wlast = min(warp0 + 32 / TPP, ch.beg + ch.cnt) - 1;
  const unsigned int mc = __reduce_max_sync(0xffffffffu, active ? (unsigned)min(cnt, a.W) : 0u);
  const int q = threadIdx.x & 31;
  if (wlast >= warp0 && q * TPP < (int)mc) {
    prefetch_l1(a.nbr + ell_index<TPP>(q * TPP, warp0, a.npad));
    prefetch_l1(a.nbr + ell_index<TPP>(q * TPP + TPP - 1, wlast, a.npad));
  }
}

// The list row of sorted particle i, generated from the cells and the
// positions at the last rebuild (xr).  Candidates are visited in a fixed
// order (rows of cells in dz, dy order; along x the adjacent cells form one
// or two contiguous runs of the sorted arrays, in dx order).  L lanes test L
// candidates per round; hits are numbered in candidate order and hit e is
// handed to lane e % L, which calls emit(e, entry).  Returns the number of
// entries.  The entry order does not depend on L.  All lanes of the group
// must call it together.
template <int D, int L, class Emit>
__device__ inline int row_scan(const SysDev& s, const Args& a, int i, int lane, Emit&& emit) {
  const unsigned int gshift = (threadIdx.x & 31) & ~(L - 1);
  const unsigned int gmask = (L == 32 ? 0xffffffffu : ((1u << L) - 1u)) << gshift;
  uint32_t xi[3] = {0u, 0u, 0u};
  int c[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < D; k++) {
    xi[k] = a.xr[k][i];
    c[k] = cell_coord(s, k, xi[k]);
  }
  const uint32_t mi = a.meta[i];
  const int moli = a.mol[i];
  const int trbi = (mi >> 8) & 0xff, loci = (mi >> 16) & 0xff, tmi = mi >> 24;
  const unsigned int pmask = s.partner[trbi];
  const uint32_t bmask = tmi != 0xff ? a.tmpl[tmi].bondmask[loci] : 0u;
  const float Rl2 = s.Rl2;
  const int nx = s.nc[0], cx = c[0];
  const int h1 = D > 1 ? s.halo[1] : 0;
  const int h2 = D > 2 ? s.halo[2] : 0;
  int cnt = 0;
  for (int dz = -h2; dz <= h2; dz++)
    for (int dy = -h1; dy <= h1; dy++) {
      // cell index of (x = 0, this row)
      int row = 0;
      bool inside = true;
      if (D > 1) {
        int mult = nx;
#pragma unroll
        for (int k = 1; k < D; k++) {
          int ck = c[k] + (k == 1 ? dy : dz);
          if ((s.periodic >> k) & 1) {
            if (ck < 0) ck += s.nc[k];
            else if (ck >= s.nc[k]) ck -= s.nc[k];
          } else if (ck < 0 || ck >= s.nc[k]) {
            inside = false;
          }
          row += ck * mult;
          mult *= s.nc[k];
        }
      }
      if (!inside) continue;
      // one or two runs of x cells [lo0, hi0], [lo1, hi1]
      int lo0, hi0, lo1 = 0, hi1 = -1;
      if (s.halo[0] == 0) {
        lo0 = hi0 = cx;
      } else if (s.periodic & 1) {  // nx >= 3 here
        if (cx == 0) { lo0 = hi0 = nx - 1; lo1 = 0; hi1 = 1; }
        else if (cx == nx - 1) { lo0 = nx - 2; hi0 = nx - 1; lo1 = hi1 = 0; }
        else { lo0 = cx - 1; hi0 = cx + 1; }
      } else {
        lo0 = max(cx - 1, 0);
        hi0 = min(cx + 1, nx - 1);
      }
      const int* cs = a.cell_start + s.c0 + row;
      const int b0 = cs[lo0], e0 = cs[hi0 + 1];
      const int b1 = hi1 >= lo1 ? cs[lo1] : 0, e1 = hi1 >= lo1 ? cs[hi1 + 1] : 0;
      const int n0 = e0 - b0, ntot = n0 + (e1 - b1);
      for (int base = 0; base < ntot; base += L) {
        const int t = base + lane;
        const int j = t < n0 ? b0 + t : b1 + (t - n0);
        int ent = 0;
        bool hit = false;
        if (t < ntot && j != i) {
          float r2 = 0.f;
#pragma unroll
          for (int k = 0; k < D; k++) {
            const float d = (float)(int)(a.xr[k][j] - xi[k]) * s.unit_hi[k];
            r2 += d * d;
          }
          if (r2 < Rl2) {
            const uint32_t mj = a.meta[j];
            if (a.mol[j] == moli) {
              hit = (bmask >> ((mj >> 16) & 31)) & 1;
              ent = j | LIST_SAME_MOL;
            } else {
              hit = (pmask >> ((mj >> 8) & 0xff)) & 1;
              ent = j;
            }
          }
        }
        const unsigned int m = (__ballot_sync(gmask, hit) & gmask) >> gshift;
        const int nh = __popc(m);
        const int r = (lane - cnt) & (L - 1);  // this lane takes hit cnt + r
        int src = lane;
        if (r < nh) {
          unsigned int mm = m;
          for (int q = 0; q < r; q++) mm &= mm - 1u;
          src = __ffs(mm) - 1;
        }
        const int v = __shfl_sync(gmask, ent, src, L);
        if (r < nh) emit(cnt + r, v);
        cnt += nh;
      }
    }
  return cnt;
}

// A list entry with the neighbour's current high words and meta word.
struct Nb {
  uint32_t x[3];
  uint32_t m;
  int v;  // entry: sorted index | LIST_SAME_MOL
};

template <int D>
__device__ inline Nb gather(const Args& a, int v) {
  Nb n;
  const int j = v & 0x7fffffff;
  n.v = v;
#pragma unroll
  for (int k = 0; k < 3; k++) n.x[k] = k < D ? a.xh[k][j] : 0u;
  n.m = a.meta[j];
  return n;
}

// Visit the list entries of particle i on this lane (entries lane, lane +
// TPP, ...), from the list or, for an overflowing row, from the cells.  List
// rows are read RD_LIST_BATCH entries at a time: all index loads, then all
// neighbour loads, then the arithmetic.
template <int D, int TPP, class Fn>
__device__ inline void for_entries(const SysDev& s, const Args& a, int i, int lane, int cnt,
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
      Nb nb[B];
#pragma unroll
      for (int u = 0; u < B; u++) nb[u] = gather<D>(a, v[u]);
#pragma unroll
      for (int u = 0; u < B; u++)
        if (e0 + u * TPP < cnt) fn(nb[u]);
    }
  } else {
    row_scan<D, TPP>(s, a, i, lane, [&](int, int v) { fn(gather<D>(a, v)); });
  }
}

// Rebuild: every particle's list row and entry count, BUILD_LANES lanes per
// particle (the row order does not depend on the lane count).
template <int D, int TPP>
__global__ void __launch_bounds__(LBLOCK) k_nlist(Args a) {
  constexpr int PER = LBLOCK / TPP;
  constexpr int L = BUILD_LANES;
  __shared__ SysDev sys;
  const Chunk ch = chunk_of<PER>(a);
  copy_words(reinterpret_cast<int*>(&sys), reinterpret_cast<const int*>(&a.sys[ch.sys]),
             (int)(sizeof(SysDev) / 4));
  __syncthreads();
  const int g = threadIdx.x / L, lane = threadIdx.x % L;
  int* nbr = a.nbr_out;
  const int W = a.W, npad = a.npad;
  for (int p = g; p < ch.cnt; p += LBLOCK / L) {
    const int i = ch.beg + p;
    const int cnt = row_scan<D, L>(sys, a, i, lane, [&](int e, int v) {
      if (e < W) nbr[ell_index<TPP>(e, i, npad)] = v;
    });
    if (lane == 0) a.ncnt_out[i] = cnt;
  }
}

// Drift kernel.  Phase A: TPP lanes per particle sum the pair drift over its
// list entries (pyrdsim.pyx:1988-2030).  Phase B: one thread per particle
// adds walls and bonded terms and performs the fused Euler-Maruyama update.
template <int D, int TPP>
__global__ void __launch_bounds__(LBLOCK, RD_LIST_MIN_BLOCKS) k_force_l(Args a) {
  constexpr int PER = LBLOCK / TPP;
  __shared__ ListShared sh;
  __shared__ float sacc[3][PER];
  const Chunk ch = chunk_of<PER>(a);
  const int tid = threadIdx.x, g = tid / TPP, lane = tid % TPP;
  const bool active = g < ch.cnt;
  const int i = ch.beg + (active ? g : 0);
  if (tid < ch.cnt) {  // phase B reads of particle beg + tid
    const int ib = ch.beg + tid;
    prefetch_l1(a.pid + ib);
#pragma unroll
    for (int k = 0; k < D; k++) prefetch_l1(a.xl[k] + ib);
  }
  const int cnt = a.ncnt[i];
  uint32_t xo[3] = {0u, 0u, 0u};
#pragma unroll
  for (int k = 0; k < D; k++) xo[k] = a.xh[k][i];
  const uint32_t mi = a.meta[i];
  prefetch_rows<TPP>(a, ch, cnt, active);
  list_tables(sh, a, ch, true, true, false);
  __syncthreads();
  const SysDev& s = sh.sys;
  float acc[3] = {0.f, 0.f, 0.f};
  if (active && s.R2 > 0.f) {
    const int ti = mi & 0xff;
    const float R2 = s.R2;
    for_entries<D, TPP>(s, a, i, lane, cnt, [&](const Nb& nb) {
      if (nb.v < 0) return;  // same molecule: reactions only
      float dx[3], r2 = 0.f;
#pragma unroll
      for (int k = 0; k < D; k++) {
        dx[k] = (float)(int)(nb.x[k] - xo[k]) * s.unit_hi[k];
        r2 += dx[k] * dx[k];
      }
      if (!(r2 < R2)) return;
      const unsigned int pp = s.ppair[ti * MAXT + (nb.m & 0xff)];
      if (!(pp & 31)) return;
      const float fr = pair_force<D>(s, sh.laws, a, i, nb.v, pp, r2);
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
  if (tid < ch.cnt) {
    const int ib = ch.beg + tid;
    uint32_t xb[3] = {0u, 0u, 0u};
#pragma unroll
    for (int k = 0; k < D; k++) xb[k] = a.xh[k][ib];
    float accb[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < D; k++) accb[k] = sacc[k][tid];
    force_tail<D>(s, sh.walls, a, ib, xb, a.meta[ib], accb);
  }
}

// Reaction kernel.  Phase A: TPP lanes per particle count, for every
// neighbour-dependent reaction, the listed partners of the right type within
// r0 (16-bit counters, two reactions per word).  Phase B: one thread per
// particle forms the propensities, draws and writes the new type
// (pyrdsim.pyx:2070-2223).
template <int D, int TPP>
__global__ void __launch_bounds__(LBLOCK, RD_LIST_MIN_BLOCKS) k_react_l(Args a) {
  constexpr int PER = LBLOCK / TPP;
  __shared__ ListShared sh;
  __shared__ uint32_t scnt[4][PER];
  const Chunk ch = chunk_of<PER>(a);
  const int tid = threadIdx.x, g = tid / TPP, lane = tid % TPP;
  const bool active = g < ch.cnt;
  const int i = ch.beg + (active ? g : 0);
  if (tid < ch.cnt) prefetch_l1(a.pid + ch.beg + tid);
  const int cnt = a.ncnt[i];
  const uint32_t mi = a.meta[i];
  uint32_t xo[3] = {0u, 0u, 0u};
#pragma unroll
  for (int k = 0; k < D; k++) xo[k] = a.xh[k][i];
  prefetch_rows<TPP>(a, ch, cnt, active);
  list_tables(sh, a, ch, false, false, true);
  __syncthreads();
  const SysDev& s = sh.sys;
  uint32_t c0 = 0u, c1 = 0u, c2 = 0u, c3 = 0u;
  const int ti = mi & 0xff;
  if (active && ((s.rx_nb_mask >> ti) & 1)) {
    const float Rrx2 = s.Rrx2;
    for_entries<D, TPP>(s, a, i, lane, cnt, [&](const Nb& nb) {
      float r2 = 0.f;
#pragma unroll
      for (int k = 0; k < D; k++) {
        const float d = (float)(int)(nb.x[k] - xo[k]) * s.unit_hi[k];
        r2 += d * d;
      }
      if (!(r2 < Rrx2)) return;
      const unsigned int rm = s.rxmatch[ti * MAXT + (nb.m & 0xff)];
      double dexact = -1.0;
      for (unsigned int mm = rm; mm; mm &= mm - 1u) {
        const int r = __ffs(mm) - 1;
        const RxDev& R = sh.rx[r];
        bool inside;
        if (r2 < R.r02_lo) inside = true;
        else if (r2 > R.r02_hi) inside = false;
        else {
          if (dexact < 0) dexact = exact_dist<D>(s, a, i, nb.v & 0x7fffffff);
          inside = dexact < R.r0;
        }
        if (inside) {
          const uint32_t inc = 1u << (16 * (r & 1));
          switch (r >> 1) {
            case 0: c0 += inc; break;
            case 1: c1 += inc; break;
            case 2: c2 += inc; break;
            default: c3 += inc; break;
          }
        }
      }
    });
  }
#pragma unroll
  for (int o = TPP >> 1; o > 0; o >>= 1) {
    c0 += __shfl_xor_sync(0xffffffffu, c0, o);
    c1 += __shfl_xor_sync(0xffffffffu, c1, o);
    c2 += __shfl_xor_sync(0xffffffffu, c2, o);
    c3 += __shfl_xor_sync(0xffffffffu, c3, o);
  }
  if (active && lane == 0) {
    scnt[0][g] = c0;
    scnt[1][g] = c1;
    scnt[2][g] = c2;
    scnt[3][g] = c3;
  }
  __syncthreads();
  if (tid < ch.cnt) {
    const int ib = ch.beg + tid;
    const uint32_t cw[4] = {scnt[0][tid], scnt[1][tid], scnt[2][tid], scnt[3][tid]};
    react_tail(s, sh.rx, a, ib, a.meta[ib], cw);
  }
}

}  // namespace rd
