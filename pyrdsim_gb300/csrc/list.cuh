// list.cuh -- Verlet-list step kernels.
//
// At every rebuild k_nlist writes, for each particle in sorted order, the
// particles of the 3^D cells around its cell that lie within the list radius
// (range + 2 delta) and form a listed pair at that rebuild:
// interaction partners (types at the rebuild, pyrdsim.pyx:1448-1587) of
// another molecule, or bonded-list members of its own molecule (flagged with
// LIST_SAME_MOL: they count for reactions, not for pair forces).  The drift
// kernel's displacement check bounds every particle's motion since the
// rebuild by delta (Euclidean), so every pair that comes within range
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

constexpr int LBLOCK = BLOCK;                  // threads per CTA
constexpr int LIST_SAME_MOL = (int)0x80000000;

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

// Run of particles number q (PER per run): computed for a single system,
// else from the chunk table.
template <int PER>
__device__ inline Chunk chunk_at(const Args& a, int q) {
  if (a.single) {
    Chunk c = a.chunk1;
    c.beg = q * PER;
    c.cnt = min(PER, a.n_total - c.beg);
    return c;
  }
  return a.chunks[q];
}

template <int PER>
__device__ inline Chunk chunk_of(const Args& a) {
  return chunk_at<PER>(a, (int)blockIdx.x);
}

// The chunk's system tables into shared memory: one round trip (all loads
// first, then the stores; the caller synchronises).
template <bool LAWS, bool WALLS, bool RX>
__device__ inline void list_tables(ListShared& sh, const Args& a, const Chunk& c) {
  constexpr int NS = (int)(sizeof(SysDev) / 4);
  constexpr int NL = LAWS ? MAXI * (int)(sizeof(PairLaw) / 4) : 0;
  constexpr int NW = WALLS ? MAXW * (int)(sizeof(WallLaw) / 4) : 0;
  constexpr int NR = RX ? MAXR * (int)(sizeof(RxDev) / 4) : 0;
  const int nl = c.nlaws * (int)(sizeof(PairLaw) / 4);
  const int nw = c.nwalls * (int)(sizeof(WallLaw) / 4);
  const int nr = c.nrx * (int)(sizeof(RxDev) / 4);
  WordLoad<NS> ls;
  WordLoad<NL> ll;
  WordLoad<NW> lw;
  WordLoad<NR> lr;
  ls.load(reinterpret_cast<const int*>(&a.sys[c.sys]), NS);
  if (LAWS) ll.load(reinterpret_cast<const int*>(a.laws + c.law0), nl);
  if (WALLS) lw.load(reinterpret_cast<const int*>(a.walls + c.wall0), nw);
  if (RX) lr.load(reinterpret_cast<const int*>(a.rx + c.rx0), nr);
  ls.store(reinterpret_cast<int*>(&sh.sys), NS);
  if (LAWS) ll.store(reinterpret_cast<int*>(sh.laws), nl);
  if (WALLS) lw.store(reinterpret_cast<int*>(sh.walls), nw);
  if (RX) lr.store(reinterpret_cast<int*>(sh.rx), nr);
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

// Cells of one row of particle cell c (offsets dy, dz): the cell index of
// x = 0 in that row and one or two runs of x cells [lo0, hi0], [lo1, hi1]
// (hi1 < lo1: none), in dx order.  False if the row lies outside a
// reflecting box.
template <int D>
__device__ inline bool row_runs(const SysDev& s, const int* c, int dy, int dz, int& row, int& lo0,
                                int& hi0, int& lo1, int& hi1) {
  const int nx = s.nc[0], cx = c[0];
  row = 0;
  if (D > 1) {
    int mult = nx;
#pragma unroll
    for (int k = 1; k < D; k++) {
      int ck = c[k] + (k == 1 ? dy : dz);
      if ((s.periodic >> k) & 1) {
        if (ck < 0) ck += s.nc[k];
        else if (ck >= s.nc[k]) ck -= s.nc[k];
      } else if (ck < 0 || ck >= s.nc[k]) {
        return false;
      }
      row += ck * mult;
      mult *= s.nc[k];
    }
  }
  lo1 = 0;
  hi1 = -1;
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
  return true;
}

// The list row of sorted particle i, generated from the cells and the
// positions at the last rebuild (xr).  Candidates are visited in a fixed
// order (rows of cells in dz, dy order; along x the adjacent cells form one
// or two contiguous runs of the sorted arrays, in dx order).  All run
// boundaries are loaded at once, then the L lanes enumerate the candidates
// of all runs together, L per round, two rounds per batch of loads.  Hits are
// numbered in candidate order and hit e is handed to lane e % L, which calls
// emit(e, entry).  Returns the number of entries.  The entry order does not
// depend on L.  All lanes of the group must call it together.
template <int D, int L, class Emit>
__device__ inline int row_scan(const SysDev& s, const Args& a, int i, int lane, Emit&& emit) {
  constexpr int NROW = D == 3 ? 9 : (D == 2 ? 3 : 1);
  constexpr int NRUN = 2 * NROW;
  constexpr int U = 2;
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
  const int h1 = D > 1 ? s.halo[1] : 0;
  const int h2 = D > 2 ? s.halo[2] : 0;
  // runs [rb, re) of the sorted arrays, in candidate order
  int rb[NRUN], re[NRUN];
#pragma unroll
  for (int q = 0; q < NROW; q++) {
    const int dz = D == 3 ? q / 3 - 1 : 0;
    const int dy = D >= 2 ? q % 3 - 1 : 0;
    int row, lo0, hi0, lo1, hi1;
    const bool ok = dy >= -h1 && dy <= h1 && dz >= -h2 && dz <= h2 &&
                    row_runs<D>(s, c, dy, dz, row, lo0, hi0, lo1, hi1);
    const int* cs = a.cell_start + s.c0 + row;
    rb[2 * q] = ok ? cs[lo0] : 0;
    re[2 * q] = ok ? cs[hi0 + 1] : 0;
    const bool two = ok && hi1 >= lo1;
    rb[2 * q + 1] = two ? cs[lo1] : 0;
    re[2 * q + 1] = two ? cs[hi1 + 1] : 0;
  }
  int total = 0;
#pragma unroll
  for (int q = 0; q < NRUN; q++) total += re[q] - rb[q];
  int cnt = 0;
  for (int base = 0; base < total; base += U * L) {
    int jj[U];
    uint32_t xx[U][3], mj[U];
    int molj[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      // candidate t -> sorted index
      int off = base + u * L + lane, j = -1;
#pragma unroll
      for (int q = 0; q < NRUN; q++) {
        const int len = re[q] - rb[q];
        if (j < 0) {
          if (off < len) j = rb[q] + off;
          else off -= len;
        }
      }
      jj[u] = j;
      const int jl = j < 0 ? i : j;
#pragma unroll
      for (int k = 0; k < 3; k++) xx[u][k] = k < D ? a.xr[k][jl] : 0u;
      mj[u] = a.meta[jl];
      molj[u] = a.mol[jl];
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (base + u * L >= total) break;  // uniform across the group
      const int j = jj[u];
      int ent = 0;
      bool hit = false;
      if (j >= 0 && j != i) {
        float r2 = 0.f;
#pragma unroll
        for (int k = 0; k < D; k++) {
          const float d = (float)(int)(xx[u][k] - xi[k]) * s.unit_hi[k];
          r2 += d * d;
        }
        if (r2 < Rl2) {
          if (molj[u] == moli) {
            hit = (bmask >> ((mj[u] >> 16) & 31)) & 1;
            ent = j | LIST_SAME_MOL;
          } else {
            hit = (pmask >> ((mj[u] >> 8) & 0xff)) & 1;
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

// A list entry with the neighbour's current pair words and meta word.
struct Nb {
  uint32_t x[3];
  uint32_t m;
  int v;  // entry: sorted index | LIST_SAME_MOL
};

// The final type word of sorted particle j whose reaction draw is still
// pending (period kernel): polled until its chunk writes it, for at most
// a.wait_ns; then RDSIM_ERR_SYNC is recorded and the old word is used.
__device__ inline uint32_t wait_final_meta(const Args& a, int j, uint32_t v) {
  const unsigned long long t0 = global_timer();
  while (v & META_PENDING) {
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(a.meta + j) : "memory");
    if ((long long)(global_timer() - t0) > a.wait_ns) {
      record_error(a.err, RDSIM_ERR_SYNC, (long long)j, -2, 0.0, eff_step(a));
      return v & ~META_PENDING;
    }
  }
  return v;
}

// PEND (period kernel): a neighbour whose draw of this step is pending is
// waited for, so that its type is the one after this step's reactions.
template <int D, bool PEND = false>
__device__ inline Nb gather(const Args& a, int v) {
  Nb n;
  const int j = v & 0x7fffffff;
  n.v = v;
#pragma unroll
  for (int k = 0; k < 3; k++) n.x[k] = k < D ? (PEND ? ldw(a, a.xp[k] + j) : a.xp[k][j]) : 0u;
  n.m = PEND ? ldw(a, a.meta + j) : a.meta[j];
  if (PEND && (n.m & META_PENDING)) n.m = wait_final_meta(a, j, n.m);
  return n;
}

// Displacement of an entry from its pair words (the exact integer
// difference rounded once to float32, then scaled by the unit) and the
// squared distance.
template <int D>
__device__ inline float pair_geom(const SysDev& s, const uint32_t* xj, const uint32_t* xi,
                                  float* dx) {
  float r2 = 0.f;
#pragma unroll
  for (int k = 0; k < D; k++) {
    dx[k] = (float)(int)(xj[k] - xi[k]) * s.qf[k];
    r2 = fmaf(dx[k], dx[k], r2);
  }
  return r2;
}

// Visit the list entries of particle i on this lane (entries lane, lane +
// TPP, ...), from the list or, for an overflowing row, from the cells.  List
// rows are read RD_LIST_BATCH entries at a time: all index loads, then all
// neighbour loads, then the arithmetic.
template <int D, int TPP, bool PEND = false, class Fn>
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
      for (int u = 0; u < B; u++) nb[u] = gather<D, PEND>(a, v[u]);
#pragma unroll
      for (int u = 0; u < B; u++)
        if (e0 + u * TPP < cnt) fn(nb[u]);
    }
  } else {
    row_scan<D, TPP>(s, a, i, lane, [&](int, int v) { fn(gather<D, PEND>(a, v)); });
  }
}

// Reaction prefilter of a step (sorted particle gi of type ti): the
// float64 total propensity of that step grows monotonically with every
// neighbour count, so rxA + rxB * (list entries), with a relative margin far
// above the rounding of the reference's repeated additions, bounds it from
// above.  If dt times the bound does not exceed the step's u1 (the same
// counter-based draw the reaction kernel makes), the draw `dt * total > u1`
// (pyrdsim.pyx:2211-2213) cannot succeed and the particle keeps its type.
// The bound and the comparison are float32: rxAf, rxBf and dtf are rounded
// up, the relative margin 1e-5 covers the float32 rounding, and the uniform
// is replaced by the lower bound of its top 24 bits.  Returns true when the
// draw may succeed (cnt: list entries, pid: caller index, w0: the tag-0
// words of the next step).
template <int D>
__device__ inline bool rx_may_react(const SysDev& s, int ti, int cnt, int pid, long long step,
                                    const U4* w0) {
  if (!((s.rx_any_mask >> ti) & 1)) return false;
  uint32_t hi, lo;
  u1_words<D>(s.seed, step, pid, w0, hi, lo);
  float u1lo, u1hi;
  uniform_bounds(hi, u1lo, u1hi);
  const float ub = (s.rxAf[ti] + s.rxBf[ti] * (float)cnt) * (1.0f + 1e-5f);
  return s.dtf * ub > u1lo;
}

// Rebuild: every particle's list row and entry count.  NT threads per
// particle (3 for D >= 2: one per row of cells in 2D, one per three rows in
// 3D) scan their rows' runs in candidate order, four candidates per batch of
// loads, into shared-memory buffers; the buffers are then concatenated in row
// order (the order row_scan uses), so the row does not depend on NT.  A
// thread whose rows hold more than BCAP listed pairs rescans them to write
// the rest.  With F_RX_HERE the first thread of each particle also runs the
// reaction prefilter of its step with the fresh entry count.  With
// F_PERIOD_PREP (CTA = chunk of the period kernel) it also writes the
// chunk's neighbour-chunk bitmap (the chunks of every list entry, of the
// bonded partners and the chunk itself), its candidate mask of the rebuild
// step (their type words carry META_PENDING until resolved, by the period
// kernel or by the listed reaction kernel, which also gets the candidate
// list) and its progress word (0).
template <int D, int TPP>
__global__ void __launch_bounds__((LBLOCK / TPP) * (D == 1 ? 1 : 3)) k_nlist(Args a) {
  constexpr int PER = LBLOCK / TPP;
  constexpr int NT = D == 1 ? 1 : 3;
  constexpr int NTH = PER * NT;
  constexpr int NROW = D == 3 ? 9 : (D == 2 ? 3 : 1);
  constexpr int RPT = NROW / NT;  // rows per thread
  constexpr int NRUN = 2 * RPT;
  constexpr int U = 4;
  constexpr int BCAP = 24;
  __shared__ SysDev sys;
  __shared__ int sbuf[NTH][BCAP];
  __shared__ int scnt[NTH];
  __shared__ uint32_t sbits[PMASK_WORDS];
  __shared__ uint32_t scand[CAND_WORDS];
  pdl_trigger();
  const Chunk ch = chunk_at<PER>(a, (int)blockIdx.x);
  {
    constexpr int NS = (int)(sizeof(SysDev) / 4);
    WordLoad<NS, NTH> ls;
    ls.load(reinterpret_cast<const int*>(&a.sys[ch.sys]), NS);
    ls.store(reinterpret_cast<int*>(&sys), NS);
  }
  const bool prep = (a.flags & F_PERIOD_PREP) != 0;
  if (prep) {
    for (int w = (int)threadIdx.x; w < PMASK_WORDS; w += NTH) sbits[w] = 0u;
    for (int w = (int)threadIdx.x; w < CAND_WORDS; w += NTH) scand[w] = 0u;
  }
  pdl_wait();
  __syncthreads();
  const SysDev& s = sys;
  const int tid = (int)threadIdx.x, pp = tid / NT, t = tid % NT;
  const bool valid = pp < ch.cnt;
  const int i = ch.beg + (valid ? pp : 0);
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
  const int h1 = D > 1 ? s.halo[1] : 0;
  const int h2 = D > 2 ? s.halo[2] : 0;
  int rb[NRUN], re[NRUN];
#pragma unroll
  for (int r = 0; r < RPT; r++) {
    const int q = t * RPT + r;
    const int dz = D == 3 ? q / 3 - 1 : 0;
    const int dy = D >= 2 ? q % 3 - 1 : 0;
    int row, lo0, hi0, lo1, hi1;
    const bool ok = valid && dy >= -h1 && dy <= h1 && dz >= -h2 && dz <= h2 &&
                    row_runs<D>(s, c, dy, dz, row, lo0, hi0, lo1, hi1);
    const int* cs = a.cell_start + s.c0 + row;
    rb[2 * r] = ok ? cs[lo0] : 0;
    re[2 * r] = ok ? cs[hi0 + 1] : 0;
    const bool two = ok && hi1 >= lo1;
    rb[2 * r + 1] = two ? cs[lo1] : 0;
    re[2 * r + 1] = two ? cs[hi1 + 1] : 0;
  }
  // the listed pairs of this thread's rows, in candidate order: emit(k, entry)
  auto scan_rows = [&](auto&& emit) {
    int k = 0;
#pragma unroll
    for (int q = 0; q < NRUN; q++) {
      for (int j0 = rb[q]; j0 < re[q]; j0 += U) {
        uint32_t xx[U][3], mj[U];
        int molj[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int jl = j0 + u < re[q] ? j0 + u : i;
#pragma unroll
          for (int d = 0; d < 3; d++) xx[u][d] = d < D ? a.xr[d][jl] : 0u;
          mj[u] = a.meta[jl];
          molj[u] = a.mol[jl];
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int j = j0 + u;
          if (j >= re[q] || j == i) continue;
          float r2 = 0.f;
#pragma unroll
          for (int d = 0; d < D; d++) {
            const float dd = (float)(int)(xx[u][d] - xi[d]) * s.unit_hi[d];
            r2 += dd * dd;
          }
          if (!(r2 < Rl2)) continue;
          bool hit;
          int ent;
          if (molj[u] == moli) {
            hit = (bmask >> ((mj[u] >> 16) & 31)) & 1;
            ent = j | LIST_SAME_MOL;
          } else {
            hit = (pmask >> ((mj[u] >> 8) & 0xff)) & 1;
            ent = j;
          }
          if (hit) emit(k++, ent);
        }
      }
    }
    return k;
  };
  // period kernel: the chunk of sorted particle j of this system (a
  // system's chunks are consecutive runs of PER particles) into the bitmap;
  // runs of entries fall into one chunk, so only changes are marked
  const int chunk0 = (int)blockIdx.x - (ch.beg - s.p0) / PER;
  int lastc = -1;
  auto mark = [&](int j) {
    const int c = chunk0 + (j - s.p0) / PER;
    if (c != lastc) {
      atomicOr(&sbits[c >> 5], 1u << (c & 31));
      lastc = c;
    }
  };
  const int cnt = scan_rows([&](int k, int ent) {
    if (k < BCAP) sbuf[tid][k] = ent;
    if (prep) mark(ent & 0x7fffffff);
  });
  if (prep && valid) {
    mark(i);
    if (t == 0 && tmi != 0xff) {  // bonded partners: every atom of the molecule
      const int mb = a.pid[i] - loci, na = a.tmpl[tmi].n_atoms;
      for (int b = 0; b < na; b++) mark(a.slot_of[mb + b]);
    }
  }
  scnt[tid] = cnt;
  __syncthreads();
  int off = 0, total = 0;
#pragma unroll
  for (int u = 0; u < NT; u++) {
    const int cu = scnt[pp * NT + u];
    if (u < t) off += cu;
    total += cu;
  }
  int4 rec = make_int4(0, 0, 0, 0);
  bool listed = false;
  if (valid) {
    int* nbr = a.nbr_out;
    const int W = a.W, npad = a.npad;
    const int nb = min(cnt, BCAP);
    for (int k = 0; k < nb; k++)
      if (off + k < W) nbr[ell_index<TPP>(off + k, i, npad)] = sbuf[tid][k];
    if (cnt > BCAP && off + BCAP < W)
      scan_rows([&](int k, int ent) {
        if (k >= BCAP && off + k < W) nbr[ell_index<TPP>(off + k, i, npad)] = ent;
      });
    if (t == 0) {
      a.ncnt_out[i] = total;
      if (a.flags & F_RX_HERE) {  // reaction prefilter of this step (see rx_may_react)
        rec = make_int4(i, (int)mi, total, a.pid[i]);
        listed = rx_may_react<D>(s, (int)(mi & 0xff), total, rec.w, eff_step(a), nullptr);
        a.meta_out[i] = mi | ((prep && listed) ? META_PENDING : 0u);
      }
    }
  }
  if (prep) {
    if (listed) atomicOr(&scand[pp >> 5], 1u << (pp & 31));
    __syncthreads();
    const int c = (int)blockIdx.x;
    for (int w = (int)threadIdx.x; w < PMASK_WORDS; w += NTH)
      a.nbmask[(size_t)c * PMASK_WORDS + w] = sbits[w];
    for (int w = (int)threadIdx.x; w < CAND_WORDS; w += NTH) a.cand0[c * CAND_WORDS + w] = scand[w];
    if (threadIdx.x == 0) a.pflag[c * PFLAG_STRIDE] = 0;
  }
  if (a.flags & F_RX_HERE) {  // the candidate list of the per-step kernels
    const unsigned int bal = __ballot_sync(0xffffffffu, listed);
    if (bal) {
      const int l32 = threadIdx.x & 31, leader = __ffs(bal) - 1;
      const int p = rx_slot(eff_step(a));
      int base = 0;
      if (l32 == leader) base = atomicAdd(a.rx_count + p, __popc(bal));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (listed) a.rx_list[(size_t)p * a.npad + base + __popc(bal & ((1u << l32) - 1u))] = rec;
    }
  }
}

// One listed particle's reaction draw at the kernel's step, by a whole warp
// (pyrdsim.pyx:2070-2223): the lanes count, for every neighbour-dependent
// reaction, its listed partners of the right type within r0 (types before
// this step's reactions, positions of this step), and lane 0 forms the
// propensities and draws.  rec = {sorted index, meta, list entries, pid}.
// Returns the new type on lane 0.
template <int D, int TPP>
__device__ inline int resolve_listed(const SysDev& s, const RxDev* rx, const Args& a, int4 rec,
                                     int lane) {
  const int m = rec.x, cnt = rec.z, pid = rec.w;
  // lane 0's counter-based words of the draw (2D: u1 from the tag-0 words),
  // computed while the neighbour loads below are in flight
  U4 w0 = {0u, 0u, 0u, 0u};
  if (D <= 2 && lane == 0 && !(a.flags & F_INJECT)) w0 = noise_words(s.seed, eff_step(a), pid, 0u);
  const uint32_t mm = (uint32_t)rec.y;
  const int tm = mm & 0xff;
  uint32_t cw[4] = {0u, 0u, 0u, 0u};
  if ((s.rx_nb_mask >> tm) & 1) {
    uint32_t xm[3] = {0u, 0u, 0u};
#pragma unroll
    for (int k = 0; k < D; k++) xm[k] = a.xp[k][m];
    const float Rrx2 = s.Rrx2;
    auto count = [&](const Nb& nb) {
      const int j = nb.v & 0x7fffffff;
      float d[3];
      const float r2 = pair_geom<D>(s, nb.x, xm, d);
      if (!(r2 < Rrx2)) return;
      const unsigned int rmask = s.rxmatch[tm * MAXT + (nb.m & 0xff)];
      double dexact = -1.0;
      for (unsigned int b = rmask; b; b &= b - 1u) {
        const int r = __ffs(b) - 1;
        const RxDev& R = rx[r];
        bool inside;
        if (r2 < R.r02_lo) inside = true;
        else if (r2 > R.r02_hi) inside = false;
        else {
          if (dexact < 0) dexact = exact_dist<D>(s, a, m, j);
          inside = dexact < R.r0;
        }
        if (inside) cw[r >> 1] += 1u << (16 * (r & 1));
      }
    };
    if (cnt <= a.W) {
      for (int e = lane; e < cnt; e += 32) count(gather<D>(a, a.nbr[ell_index<TPP>(e, m, a.npad)]));
    } else {
      row_scan<D, 32>(s, a, m, lane, [&](int, int v) { count(gather<D>(a, v)); });
    }
#pragma unroll
    for (int w = 0; w < 4; w++) cw[w] = __reduce_add_sync(0xffffffffu, cw[w]);
  }
  return lane == 0 ? react_decide<D>(s, rx, a, pid, tm, cw,
                                     (D <= 2 && !(a.flags & F_INJECT)) ? &w0 : nullptr)
                   : tm;
}

// Phase A of the drift kernels: this lane's share of the pair drift of
// sorted particle i (type word mi, pair words xo) over its list entries
// (pyrdsim.pyx:1988-2030), added to acc.
// One list entry's pair drift on particle i (type ti, pair words xo).
template <int D>
__device__ __forceinline__ void pair_term(const ListShared& sh, const Args& a, int i, int ti,
                                          const uint32_t* xo, const Nb& nb, float* acc) {
  const SysDev& s = sh.sys;
  if (nb.v < 0) return;  // same molecule: reactions only
  float d[3];
  const float r2 = pair_geom<D>(s, nb.x, xo, d);
  const int tj = nb.m & 0xff;
  if (!(r2 < s.prc2[ti * MAXT + tj])) return;  // beyond every law of the pair
  const unsigned int pp = s.ppair[ti * MAXT + tj];
  const PairLaw& L0 = sh.laws[(pp >> 5) & 0x3ff];
  float fr;
  if ((pp & 0x8000u) && r2 < L0.rc2_lo) {
    // a single Lennard-Jones n = 6 law, clear of its cutoff: eval_pair's
    // arithmetic inline
    fr = lj6_over_r(L0.c0, L0.c1, r2, recip(r2));
  } else {
    fr = pair_force<D>(s, sh.laws, a, i, nb.v, pp, r2);
  }
#pragma unroll
  for (int k = 0; k < D; k++) acc[k] = fmaf(fr, d[k], acc[k]);
}

template <int D, int TPP, bool PEND = false>
__device__ __forceinline__ void pair_drift(const ListShared& sh, const Args& a, int i, int lane,
                                           int cnt, const uint32_t* xo, uint32_t mi, float* acc) {
  const int ti = mi & 0xff;
  for_entries<D, TPP, PEND>(sh.sys, a, i, lane, cnt,
                            [&](const Nb& nb) { pair_term<D>(sh, a, i, ti, xo, nb, acc); });
}

// Drift kernel.  Phase A: TPP lanes per particle sum the pair drift over its
// list entries (pyrdsim.pyx:1988-2030).  Phase B: one thread per particle
// adds walls and bonded terms and performs the fused Euler-Maruyama update.
template <int D, int TPP>
__global__ void __launch_bounds__(LBLOCK, RD_LIST_MIN_BLOCKS) k_force_l(Args a) {
  constexpr int PER = LBLOCK / TPP;
  __shared__ ListShared sh;
  __shared__ float sacc[3][PER];
  pdl_trigger();
  const Chunk ch = chunk_of<PER>(a);
  const int tid = threadIdx.x, g = tid / TPP, lane = tid % TPP;
  const bool active = g < ch.cnt;
  const int i = ch.beg + (active ? g : 0);
  list_tables<true, true, false>(sh, a, ch);
  pdl_wait();
  if (tid < ch.cnt) {  // phase B reads of particle beg + tid
    const int ib = ch.beg + tid;
    prefetch_l1(a.pid + ib);
#pragma unroll
    for (int k = 0; k < D; k++) prefetch_l1(a.xl[k] + ib);
  }
  const int cnt = a.ncnt[i];
  uint32_t xo[3] = {0u, 0u, 0u};
#pragma unroll
  for (int k = 0; k < D; k++) xo[k] = a.xp[k][i];
  if (a.stamps && threadIdx.x == 0)
    a.stamps[((size_t)(eff_step(a) % a.stamp_ring) * gridDim.x + blockIdx.x) * 2] = global_timer();
  const uint32_t mi = a.meta[i];
  prefetch_rows<TPP>(a, ch, cnt, active);
  __syncthreads();
  const SysDev& s = sh.sys;
  float acc[3] = {0.f, 0.f, 0.f};
  if (active && s.R2 > 0.f) pair_drift<D, TPP>(sh, a, i, lane, cnt, xo, mi, acc);
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
    float accb[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < D; k++) accb[k] = sacc[k][tid];
    const uint32_t mb = a.meta[ib];
    const int pid = a.pid[ib];
    // one Philox call for the next step's noise and reaction uniform
    const bool words = (a.flags & F_RX_NEXT) ||
                       ((a.flags & F_EM) && !(a.flags & (F_NO_NOISE | F_INJECT)));
    U4 w0 = {0u, 0u, 0u, 0u};
    if (words) w0 = noise_words(s.seed, eff_em_step(a), pid, 0u);
    force_tail<D>(s, sh.walls, a, ib, pid, xb, mb, accb, words ? &w0 : nullptr);
    if (a.flags & F_RX_NEXT) {
      a.meta_out[ib] = mb;  // the next step's types, unless its draw succeeds
      rec = make_int4(ib, (int)mb, a.ncnt[ib], pid);
      listed = rx_may_react<D>(s, (int)(mb & 0xff), rec.z, pid, eff_em_step(a), &w0);
    }
  }
  if (a.flags & F_RX_NEXT) {
    // append the particles whose draw may succeed (warp-aggregated)
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
  // the slot of two steps ago was consumed before this kernel: empty it for
  // the drift kernel (or list builder) of the next step that appends to it
  if (blockIdx.x == 0 && threadIdx.x == 0) a.rx_count[rx_slot(eff_step(a) + 2)] = 0;
  // each warp's end: the CTA's end is their maximum (no barrier; the times
  // only grow, so a reused slot's older value never wins)
  if (a.stamps && (threadIdx.x & 31) == 0)
    atomicMax(a.stamps + ((size_t)(eff_step(a) % a.stamp_ring) * gridDim.x + blockIdx.x) * 2 + 1,
              global_timer());
}

// Spans of the stamped drift launches: per ring slot, the last CTA end minus
// the first CTA start (slots never written are skipped), summed.
static __global__ void k_stamp_spans(const unsigned long long* st, int ring, int nctas,
                              unsigned long long* sum, unsigned long long* count) {
  __shared__ unsigned long long lo[32], hi[32];
  const int slot = blockIdx.x;
  unsigned long long a0 = ~0ull, b0 = 0ull;
  for (int c = threadIdx.x; c < nctas; c += blockDim.x) {
    const unsigned long long s0 = st[((size_t)slot * nctas + c) * 2];
    const unsigned long long e0 = st[((size_t)slot * nctas + c) * 2 + 1];
    if (s0 && e0) {
      a0 = min(a0, s0);
      b0 = max(b0, e0);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    a0 = min(a0, __shfl_xor_sync(0xffffffffu, a0, o));
    b0 = max(b0, __shfl_xor_sync(0xffffffffu, b0, o));
  }
  if ((threadIdx.x & 31) == 0) {
    lo[threadIdx.x >> 5] = a0;
    hi[threadIdx.x >> 5] = b0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
      a0 = min(a0, lo[w]);
      b0 = max(b0, hi[w]);
    }
    if (b0 > a0) {
      atomicAdd(sum, b0 - a0);
      atomicAdd(count, 1ull);
    }
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
  pdl_trigger();
  const Chunk ch = chunk_of<PER>(a);
  list_tables<false, false, true>(sh, a, ch);
  pdl_wait();
  const int tid = threadIdx.x, g = tid / TPP, lane = tid % TPP;
  const bool active = g < ch.cnt;
  const int i = ch.beg + (active ? g : 0);
  if (tid < ch.cnt) prefetch_l1(a.pid + ch.beg + tid);
  const int cnt = a.ncnt[i];
  const uint32_t mi = a.meta[i];
  uint32_t xo[3] = {0u, 0u, 0u};
#pragma unroll
  for (int k = 0; k < D; k++) xo[k] = a.xp[k][i];
  prefetch_rows<TPP>(a, ch, cnt, active);
  __syncthreads();
  const SysDev& s = sh.sys;
  uint32_t c0 = 0u, c1 = 0u, c2 = 0u, c3 = 0u;
  const int ti = mi & 0xff;
  if (active && ((s.rx_nb_mask >> ti) & 1)) {
    const float Rrx2 = s.Rrx2;
    for_entries<D, TPP>(s, a, i, lane, cnt, [&](const Nb& nb) {
      float d[3];
      const float r2 = pair_geom<D>(s, nb.x, xo, d);
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
    react_tail<D>(s, sh.rx, a, ib, a.pid[ib], a.meta[ib], cw);
  }
}

// Reaction kernel of the steps the previous drift kernel (or the list
// builder) prefiltered: that kernel copied every type forward and listed the
// particles whose draw may succeed; one warp per listed particle resolves it
// (resolve_listed) and writes its new type (pyrdsim.pyx:2070-2223).  A
// single system's tables are staged in shared memory; a batch's are read
// through L1.
template <int D, int TPP>
__global__ void __launch_bounds__(LBLOCK) k_react_listed(Args a) {
  __shared__ SysDev sys1;
  __shared__ RxDev rx1[MAXR];
  pdl_trigger();
  if (a.single) {
    constexpr int NS = (int)(sizeof(SysDev) / 4), NR = MAXR * (int)(sizeof(RxDev) / 4);
    const int nr = a.chunk1.nrx * (int)(sizeof(RxDev) / 4);
    WordLoad<NS> ls;
    WordLoad<NR> lr;
    ls.load(reinterpret_cast<const int*>(a.sys), NS);
    lr.load(reinterpret_cast<const int*>(a.rx), nr);
    ls.store(reinterpret_cast<int*>(&sys1), NS);
    lr.store(reinterpret_cast<int*>(rx1), nr);
  }
  pdl_wait();
  // the step counter, the three slots' counts and this warp's first record
  // of each slot are loaded together (one round trip instead of three)
  const int w0 = (int)((blockIdx.x * LBLOCK + threadIdx.x) >> 5);
  int nc[3];
  int4 f[3];
  const int4 zero = make_int4(0, 0, 0, 0);
#pragma unroll
  for (int q = 0; q < 3; q++) {
    nc[q] = a.rx_count[q];
    f[q] = w0 < a.npad ? a.rx_list[(size_t)q * a.npad + w0] : zero;
  }
  const int p = rx_slot(eff_step(a));
  const int n = p == 0 ? nc[0] : (p == 1 ? nc[1] : nc[2]);
  const int4 first = p == 0 ? f[0] : (p == 1 ? f[1] : f[2]);
  __syncthreads();
  const int4* list = a.rx_list + (size_t)p * a.npad;
  const int lane = threadIdx.x & 31;
  const int nwarps = (int)(gridDim.x * LBLOCK / 32);
  for (int q = w0; q < n; q += nwarps) {
    const int4 rec = q == w0 ? first : list[q];
    const SysDev& s = a.single ? sys1 : a.sys[a.sid[rec.x]];
    const RxDev* rx = a.single ? rx1 : a.rx + s.rx0;
    const int newt = resolve_listed<D, TPP>(s, rx, a, rec, lane);
    if (lane == 0) a.meta_out[rec.x] = ((uint32_t)rec.y & 0xffffff00u) | (uint32_t)newt;
  }
}

// ---------------------------------------------------------------------------
// Period kernel: every step of one rebuild period (the listed reactions of
// each step, then its drift with the fused update of the next step) in one
// launch, one CTA per chunk, all CTAs resident.  There is no grid-wide
// barrier: after its drift of step n a chunk publishes progress n + 1, and
// a chunk starts step n once every chunk it reads (its list entries' and
// bonded partners' chunks, from the list builder's bitmap) has progress
// >= n: their positions of step n and their types are written.  The list
// relation is symmetric (the same distance and partner tests from both
// ends), so the chunks that read a chunk are among those it waits for,
// which also protects the buffers it overwrites.
// Reactions: the drift of step n - 1 marks the type word of each particle
// whose draw of step n may succeed with META_PENDING; the particle's own
// chunk resolves the draw at the start of step n and writes the final word.
// A neighbour that gathers a pending word waits for that word alone, so
// only the particles next to a pending draw wait for it (and the symmetric
// list again orders the resolution's reads of the old types before the
// neighbour overwrites them).  Every wait ends after wait_ns of the global
// timer, or as soon as any CTA has recorded an error: RDSIM_ERR_SYNC is
// recorded and the CTA returns.  The arithmetic per particle is that of
// k_force_l and k_react_listed (same functions), so the results equal
// theirs bit for bit.

// Polling: relaxed loads (an acquire load invalidates the SM's L1, which
// the other CTAs on the SM use for their list rows).  With RD_PERIOD_CG = 0
// (plain loads of other CTAs' words) one acquire fence follows once every
// word has reached its target; with the default strong loads none does.
#ifndef RD_PERIOD_POLL_ACQUIRE
#define RD_PERIOD_POLL_ACQUIRE 0
#endif
#ifndef RD_PERIOD_SLEEP_NS
#define RD_PERIOD_SLEEP_NS 32
#endif

__device__ inline int ld_poll(const int* p) {
  int v;
#if RD_PERIOD_POLL_ACQUIRE
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
#else
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
#endif
  return v;
}

// With RD_PERIOD_CG the words written by other CTAs are read from L2 and
// the relaxed poll that saw a chunk's progress precedes those reads (they
// issue only after the poll's loop has exited on the value, and the writer
// fenced its words before publishing): no fence here, and the SM's L1 keeps
// the list rows.
__device__ inline void fence_acquire() {
#if !RD_PERIOD_POLL_ACQUIRE && !RD_PERIOD_CG
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
#endif
}

__device__ inline void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Per-particle words of the chunk staged in shared memory by the tail
// threads: static ones once per period (caller index, high words at the
// rebuild), the CTA's own positions and the noise of the coming update
// before each step's wait (they depend on no other chunk).
template <int PER>
struct PeriodStage {
  int pid[PER];
  uint32_t xr[3][PER];
  uint32_t xh[3][PER];
  uint32_t xl[3][PER];
  uint32_t w[4][PER];               // Philox words of the update (tag 0)
  float xi[3][PER];                 // their standard normals
};

// Neighbour staging of a chunk (period kernel).  Built once per period from
// the chunk's static list rows: per chunk that its entries touch (itself
// included), the run [lo, hi] of sorted indices touched, laid out back to
// back (slot -> sorted index in g); every entry of a particle whose row fits
// (at most LS_MAX entries, none regenerated from the cells) is rewritten as
// its slot (bit 15: same molecule).  Each step the pair and type words of
// all slots are loaded once, coalesced, into x / m; the pair loop reads them
// from shared memory in the list's order, so its sums are those of the
// gathers.  A chunk whose runs exceed SMAX slots (six per particle of the
// chunk) or that touches more than STAGE_CH chunks gathers from memory as
// before.
constexpr int STAGE_CH = 64;
constexpr int LS_MAX = 32;

template <int D, int PER>
struct PeriodNbStage {
  static constexpr int SMAX = 6 * PER;
  uint32_t x[D][SMAX];
  uint32_t m[SMAX];
  int g[SMAX];
  unsigned short slot[LS_MAX][PER];
  int lo[STAGE_CH], hi[STAGE_CH], base[STAGE_CH + 1];
  unsigned short ch[STAGE_CH];
  int nch, total, on;
};

struct PeriodShared {
  ListShared sh;
  unsigned short wl[PMAX_CHUNKS];   // chunks waited for (not itself)
  uint32_t cmask[2][CAND_WORDS];    // listed particles of steps of parity 0/1
  long long s0;                     // first step of the period
  int nwl;
  int ok;
};

// All threads: true once every listed chunk has published progress >=
// target; false (after recording the error) if the wait gave up.
__device__ inline bool period_wait(PeriodShared& ps, const int* pflag, int target,
                                   const PeriodArgs& p, ErrDev* err, long long step) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    bool ok = true;
    unsigned long long t0 = 0ull;
    for (int b = 0; b < ps.nwl && ok; b += 32) {
      const int c = b + lane < ps.nwl ? (int)ps.wl[b + lane] : -1;
      for (;;) {
        const int v = c >= 0 ? ld_poll(pflag + c * PFLAG_STRIDE) : target;
        if (__all_sync(0xffffffffu, v - target >= 0)) break;
        bool give_up = false;
        if (lane == 0) {
          const unsigned long long now = global_timer();
          if (t0 == 0ull) t0 = now;
          const int e = *(volatile int*)&err->code;
          give_up = e != 0 || (long long)(now - t0) > p.wait_ns;
          if (give_up && e == 0)
            record_error(err, RDSIM_ERR_SYNC, (long long)blockIdx.x, -1, (double)target, step);
        }
        if (__shfl_sync(0xffffffffu, give_up, 0)) {
          ok = false;
          break;
        }
        if (RD_PERIOD_SLEEP_NS > 0) __nanosleep(RD_PERIOD_SLEEP_NS);
      }
    }
    fence_acquire();
    if (lane == 0) ps.ok = ok;
  }
  __syncthreads();
  return ps.ok != 0;
}

// Publishes progress v of the CTA's chunk; the caller has synchronised the
// CTA after its last write of the phase (the barrier orders the other
// threads' writes before thread 0's release, which is cumulative).
// RD_PERIOD_PUBLISH_FENCE adds a full fence before the release.
#ifndef RD_PERIOD_PUBLISH_FENCE
#define RD_PERIOD_PUBLISH_FENCE 0
#endif
__device__ inline void period_publish(int* pflag, int v, const PeriodArgs& p) {
  if (threadIdx.x == 0 && (int)blockIdx.x != p.withhold) {
    if (RD_PERIOD_PUBLISH_FENCE) __threadfence();
    st_release(pflag + (size_t)blockIdx.x * PFLAG_STRIDE, v);
  }
}

// The reaction draw of listed particle m by the calling warp (out of line:
// rare, and its registers stay out of the drift's budget).
template <int D, int TPP>
__device__ __noinline__ void period_resolve(const ListShared& sh, const Args& r, int m, int lane) {
  const int4 rec = make_int4(m, (int)r.meta[m], r.ncnt[m], r.pid[m]);
  const int newt = resolve_listed<D, TPP>(sh.sys, sh.rx, r, rec, lane);
  if (lane == 0) r.meta_out[m] = ((uint32_t)rec.y & 0xffffff00u) | (uint32_t)newt;
}

// Step n of the period on the CTA's chunk: d / r are the step arguments of
// the drift and of the reactions (buffers of parity P = n & 1).
template <int D, int TPP, int P>
__device__ __forceinline__ bool period_run_step(PeriodShared& ps,
                                                PeriodStage<LBLOCK / TPP>& st,
                                                PeriodNbStage<D, LBLOCK / TPP>& ns,
                                                float (*sacc)[LBLOCK / TPP],
                                                const Args& d, const Args& r,
                                                const PeriodArgs& p, const Chunk& ch, int n) {
  const int tid = threadIdx.x, warp = tid >> 5, l32 = tid & 31;
  const SysDev& s = ps.sh.sys;
  const bool rx_next = p.rx && n + 1 < p.nsteps;
  const bool words = rx_next || !(d.flags & F_NO_NOISE);
  // the tail thread's own words and noise, while other chunks finish
  if (tid < ch.cnt) {
    const int ib = ch.beg + tid;
#pragma unroll
    for (int k = 0; k < D; k++) {
      st.xh[k][tid] = d.xh[k][ib];
      st.xl[k][tid] = d.xl[k][ib];
    }
    if (words) {
      const U4 w0 = noise_words(s.seed, ps.s0 + n + 1, st.pid[tid], 0u);
      st.w[0][tid] = w0.x;
      st.w[1][tid] = w0.y;
      st.w[2][tid] = w0.z;
      st.w[3][tid] = w0.w;
      if (!(d.flags & F_NO_NOISE)) {
        float xi[3];
        gaussians<D>(w0, xi);
#pragma unroll
        for (int k = 0; k < D; k++) st.xi[k][tid] = xi[k];
      }
    }
  }
  if (tid == 0) period_step = ps.s0 + n;
  if (!period_wait(ps, d.pflag, n, p, d.err, ps.s0 + n)) return false;
  // reactions of step n: the chunk's listed particles, a warp each
  // (k_react_listed's resolution); their neighbours wait for the words
  if (p.rx) {
    uint32_t pend = 0u;
#pragma unroll
    for (int w = 0; w < CAND_WORDS; w++) pend |= ps.cmask[P][w];
    if (pend) {
      int k = 0;
#pragma unroll 1
      for (int w = 0; w < CAND_WORDS; w++) {
        for (uint32_t b = ps.cmask[P][w]; b; b &= b - 1u, k++) {
          if ((k & (LBLOCK / 32 - 1)) != warp) continue;
          period_resolve<D, TPP>(ps.sh, r, ch.beg + w * 32 + __ffs(b) - 1, l32);
        }
      }
      __syncthreads();
    }
  }
  // drift of step n and the update of step n + 1 (k_force_l)
  const int g = tid / TPP, lane = tid % TPP;
  const bool active = g < ch.cnt;
  const int i = ch.beg + (active ? g : 0);
  const int cnt = d.ncnt[i];
  uint32_t xo[3] = {0u, 0u, 0u};
#pragma unroll
  for (int k = 0; k < D; k++) xo[k] = d.xp[k][i];
  const uint32_t mi = d.meta[i];
  // the staged neighbours' words of this step, one coalesced pass
  if (ns.on) {
    for (int sl = tid; sl < ns.total; sl += LBLOCK) {
      const int j = ns.g[sl];
#pragma unroll
      for (int k = 0; k < D; k++) ns.x[k][sl] = ldw(d, d.xp[k] + j);
      ns.m[sl] = ldw(d, d.meta + j);
    }
    __syncthreads();
  }
  const bool staged = ns.on && active && cnt <= min(d.W, LS_MAX);
  prefetch_rows<TPP>(d, ch, cnt, active && !staged);
  float acc[3] = {0.f, 0.f, 0.f};
  if (active && s.R2 > 0.f) {
    if (staged) {
      const int ti = mi & 0xff;
      for (int e = lane; e < cnt; e += TPP) {
        const unsigned int code = ns.slot[e][g];
        const int sl = (int)(code & 0x7fffu);
        Nb nb;
#pragma unroll
        for (int k = 0; k < 3; k++) nb.x[k] = k < D ? ns.x[k][sl] : 0u;
        nb.m = ns.m[sl];
        const int j = ns.g[sl];
        if (nb.m & META_PENDING) nb.m = wait_final_meta(d, j, nb.m);
        nb.v = (code & 0x8000u) ? (j | LIST_SAME_MOL) : j;
        pair_term<D>(ps.sh, d, i, ti, xo, nb, acc);
      }
    } else {
      pair_drift<D, TPP, true>(ps.sh, d, i, lane, cnt, xo, mi, acc);
    }
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
  if (tid < ch.cnt) {
    TailIn t;
    float xi[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      t.xh[k] = k < D ? st.xh[k][tid] : 0u;
      t.xl[k] = k < D ? st.xl[k][tid] : 0u;
      t.xr[k] = k < D ? st.xr[k][tid] : 0u;
      if (k < D && !(d.flags & F_NO_NOISE)) xi[k] = st.xi[k][tid];
    }
    t.xi = xi;
    float accb[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < D; k++) accb[k] = sacc[k][tid];
    const uint32_t mb = d.meta[ib];
    const int pid = st.pid[tid];
    U4 w0 = {0u, 0u, 0u, 0u};
    if (words) w0 = U4{st.w[0][tid], st.w[1][tid], st.w[2][tid], st.w[3][tid]};
    force_tail_in<D>(s, ps.sh.walls, d, ib, pid, t, mb, accb, words ? &w0 : nullptr);
    if (rx_next) {
      listed = rx_may_react<D>(s, (int)(mb & 0xff), d.ncnt[ib], pid, ps.s0 + n + 1, &w0);
      // the next step's type word, marked while its draw is pending
      d.meta_out[ib] = mb | (listed ? META_PENDING : 0u);
    }
  }
  // the particles whose draw of step n + 1 may succeed: one word per warp
  const unsigned int bal = __ballot_sync(0xffffffffu, listed);
  if (l32 == 0 && warp < CAND_WORDS) ps.cmask[P ^ 1][warp] = rx_next ? bal : 0u;
  __syncthreads();
  period_publish(d.pflag, n + 1, p);
  return true;
}

// Clears the pending marks that a period kernel stopped by an error leaves.
static __global__ void k_clear_pending(uint32_t* m0, uint32_t* m1, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    m0[i] &= ~META_PENDING;
    m1[i] &= ~META_PENDING;
  }
}

// Resident CTAs per SM the period kernel is compiled for: 7 x 152 SMs hold
// the 1,024 chunks of 65,536 particles with 72 registers per thread.
#ifndef RD_PERIOD_MIN_BLOCKS
#define RD_PERIOD_MIN_BLOCKS 7
#endif

template <int D, int TPP>
__global__ void __launch_bounds__(LBLOCK, RD_PERIOD_MIN_BLOCKS)
    k_period(const __grid_constant__ Args d0, const __grid_constant__ Args d1,
             const __grid_constant__ Args r0, const __grid_constant__ Args r1, PeriodArgs p) {
  constexpr int PER = LBLOCK / TPP;
  __shared__ PeriodShared ps;
  __shared__ PeriodStage<PER> st;
  __shared__ PeriodNbStage<D, PER> ns;
  __shared__ float sacc[3][PER];
  // No early launch of the next kernel: its CTAs must not take the SM slots
  // that CTAs of this kernel still wait for.
  const Chunk ch = chunk_at<PER>(d0, (int)blockIdx.x);
  list_tables<true, true, true>(ps.sh, d0, ch);
  pdl_wait();
  const int tid = threadIdx.x;
  const int g = tid / TPP, lane = tid % TPP;
  const int i = ch.beg + (g < ch.cnt ? g : 0);
  // every word the set-up reads (written by the list builder), issued
  // together: one round trip instead of a chain
  long long s0v = 0;
  if (tid == 0) s0v = d0.step_base ? *d0.step_base + d0.step : d0.step;
  uint32_t cw = 0u;
  if (tid < CAND_WORDS && p.rx && p.first_rx) cw = d0.cand0[blockIdx.x * CAND_WORDS + tid];
  int pidv = 0;
  uint32_t xrv[3] = {0u, 0u, 0u};
  if (tid < ch.cnt) {
    pidv = d0.pid[ch.beg + tid];
#pragma unroll
    for (int k = 0; k < D; k++) xrv[k] = d0.xr[k][ch.beg + tid];
  }
  uint32_t bits[2] = {0u, 0u};
  if (tid < 32) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int w = h * 32 + tid;
      if (w < PMASK_WORDS) bits[h] = d0.nbmask[(size_t)blockIdx.x * PMASK_WORDS + w];
    }
  }
  const int cnt = g < ch.cnt ? d0.ncnt[i] : 0;
  // this lane's entries of the row (up to the staging width, whatever the
  // count: the ELL array holds W entries per particle)
  constexpr int EPL = (LS_MAX + TPP - 1) / TPP;
  const int wmax = min(d0.W, LS_MAX);
  int ent[EPL];
#pragma unroll
  for (int u = 0; u < EPL; u++) {
    const int e = lane + u * TPP;
    ent[u] = (g < ch.cnt && e < wmax) ? d0.nbr[ell_index<TPP>(e, i, d0.npad)] : 0;
  }
  if (tid == 0) {
    ps.s0 = s0v;
    if (blockIdx.x == 0) {
      // the candidate lists of the per-step kernels stay empty
      d0.rx_count[0] = 0;
      d0.rx_count[1] = 0;
      d0.rx_count[2] = 0;
    }
  }
  if (tid < CAND_WORDS) {
    ps.cmask[0][tid] = cw;
    ps.cmask[1][tid] = 0u;
  }
  if (tid < ch.cnt) {  // static for the period
    st.pid[tid] = pidv;
#pragma unroll
    for (int k = 0; k < D; k++) st.xr[k][tid] = xrv[k];
  }
  // the wait list: the bitmap's chunks other than this one, in order
  if (tid < 32) {
    int base = 0;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int w = h * 32 + tid;
      uint32_t bw = bits[h];
      if (w == (int)(blockIdx.x >> 5)) bw &= ~(1u << (blockIdx.x & 31));
      const int cntw = __popc(bw);
      int incl = cntw;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (tid >= o) incl += v;
      }
      int pos = base + incl - cntw;
      for (uint32_t b = bw; b; b &= b - 1u) ps.wl[pos++] = (unsigned short)(w * 32 + __ffs(b) - 1);
      base += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (tid == 0) ps.nwl = base;
  }
  __syncthreads();
  // the neighbour staging table (PeriodNbStage)
  {
    const int self = (int)blockIdx.x;
    const int nwl = ps.nwl;
    const int on0 = nwl + 1 <= STAGE_CH ? 1 : 0;
    // the waited chunks and this one, in order (warp 0; ps.wl is sorted)
    if (tid < 32) {
      if (on0) {
        int below = 0;
        for (int q = tid; q < nwl; q += 32) {
          const int c = ps.wl[q];
          below += c < self ? 1 : 0;
          ns.ch[q + (c > self ? 1 : 0)] = (unsigned short)c;
        }
        below = __reduce_add_sync(0xffffffffu, below);
        if (tid == 0) ns.ch[below] = (unsigned short)self;
      }
      if (tid == 0) {
        ns.on = on0;
        ns.nch = on0 ? nwl + 1 : 0;
        ns.total = 0;
      }
    }
    for (int q = tid; q < STAGE_CH; q += LBLOCK) {
      ns.lo[q] = 0x7fffffff;
      ns.hi[q] = -1;
    }
    const SysDev& s = ps.sh.sys;
    const int chunk0 = (int)blockIdx.x - (ch.beg - s.p0) / PER;
    const bool mine = on0 && g < ch.cnt && cnt <= wmax;
    __syncthreads();
    // position of the chunk of sorted particle j in ns.ch (-1: absent)
    auto pos_of = [&](int j) {
      const int h = chunk0 + (j - s.p0) / PER;
      int lo = 0, hi = ns.nch - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int)ns.ch[mid] < h) lo = mid + 1;
        else hi = mid;
      }
      return (int)ns.ch[lo] == h ? lo : -1;
    };
    if (mine) {
#pragma unroll
      for (int u = 0; u < EPL; u++) {
        if (lane + u * TPP >= cnt) break;
        const int j = ent[u] & 0x7fffffff;
        const int q = pos_of(j);
        if (q < 0) {
          ns.on = 0;
          continue;
        }
        atomicMin(&ns.lo[q], j);
        atomicMax(&ns.hi[q], j);
      }
    }
    __syncthreads();
    // run lengths -> bases (warp 0, shuffle scan over at most STAGE_CH runs)
    if (tid < 32 && ns.on) {
      const int n = ns.nch;
      int carry = 0;
      for (int q0 = 0; q0 < n; q0 += 32) {
        const int q = q0 + tid;
        const int len = (q < n && ns.hi[q] >= ns.lo[q]) ? ns.hi[q] - ns.lo[q] + 1 : 0;
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (tid >= o) incl += v;
        }
        if (q < n) ns.base[q] = carry + incl - len;
        carry += __shfl_sync(0xffffffffu, incl, 31);
      }
      if (tid == 0) {
        ns.base[n] = carry;
        ns.total = carry;
        if (carry > PeriodNbStage<D, PER>::SMAX) ns.on = 0;
      }
    }
    __syncthreads();
    if (ns.on) {
      for (int sl = tid; sl < ns.total; sl += LBLOCK) {
        int lo = 0, hi = ns.nch - 1;  // the last run starting at or before sl
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (ns.base[mid] <= sl) lo = mid;
          else hi = mid - 1;
        }
        ns.g[sl] = ns.lo[lo] + (sl - ns.base[lo]);
      }
      if (mine) {
#pragma unroll
        for (int u = 0; u < EPL; u++) {
          const int e = lane + u * TPP;
          if (e >= cnt) break;
          const int v = ent[u];
          const int j = v & 0x7fffffff;
          const int q = pos_of(j);
          const int sl = ns.base[q] + (j - ns.lo[q]);
          ns.slot[e][g] = (unsigned short)(sl | (v < 0 ? 0x8000 : 0));
        }
      }
    }
    __syncthreads();
  }
  const long long slot = d0.stamps ? (ps.s0 / p.nsteps) % d0.stamp_ring : 0;
  if (d0.stamps && tid == 0)
    d0.stamps[((size_t)slot * gridDim.x + blockIdx.x) * 2] = global_timer();
  for (int n = 0; n < p.nsteps; n += 2) {
    if (!period_run_step<D, TPP, 0>(ps, st, ns, sacc, d0, r0, p, ch, n)) return;
    if (n + 1 < p.nsteps && !period_run_step<D, TPP, 1>(ps, st, ns, sacc, d1, r1, p, ch, n + 1))
      return;
  }
  if (d0.stamps && (tid & 31) == 0)
    atomicMax(d0.stamps + ((size_t)slot * gridDim.x + blockIdx.x) * 2 + 1, global_timer());
}

}  // namespace rd
