// device.cuh -- data layout and device helpers of the GB300 step engine.
//
// Layout in HBM (all per-particle arrays in *cell-sorted* order, systems
// concatenated; re-sorted at every neighbour-list rebuild):
//   xh[buf][k][i]  u32  high word of the 64-bit fixed-point coordinate k
//   xl[buf][k][i]  u32  low word
//   xp[buf][k][i]  u32  pair word: bits ps_k .. ps_k + 31 of the coordinate
//   meta[buf][i]   u32  type | type_at_rebuild << 8 | local atom << 16 |
//                       template << 24 (0xff = no bonded terms)
//   mol[buf][i]    i32  molecule number (initial-condition column 0)
//   pid[buf][i]    i32  particle index in the caller's order
// Fixed point per dimension k of a system with box length L:
//   periodic   : X in [0, 2^64) represents X * L / 2^64 (wraps exactly)
//   reflecting : X in [0, S], S = 2^62, represents X * L / S
// The pair kernels read only the pair words: (int32)(pj - pi) is the
// displacement in units of q_k = (length per fixed unit) * 2^ps_k, the
// minimum image in periodic dimensions (the wrap of X at 2^64 carries over
// to the 32-bit difference) and the plain displacement in reflecting ones.
// ps_k is the smallest shift whose range (2^31 q_k) holds twice the largest
// per-dimension separation of listed pairs, so q_k is about 1e-9 to 1e-8
// length units whatever the box length (the high words alone resolve L/2^32).
// Each difference is rounded once to float32 and scaled by q_k.  The
// cell-list rebuild uses the high words (bits 32..63).
#pragma once

#include <cstdint>

#include "../../include/rdsim.h"

namespace rd {

constexpr int MAXT = RDSIM_MAX_TYPES;
constexpr int MAXI = RDSIM_MAX_INTERACTIONS;
constexpr int MAXR = RDSIM_MAX_REACTIONS;
constexpr int MAXA = RDSIM_MAX_ATOMS;
constexpr int MAXW = 8;          // wall interactions per system
constexpr int BLOCK = 128;       // threads per CTA of the step kernels

// One nonbonded pair law in evaluation form (pyrdsim.pyx:1068-1130).
struct PairLaw {
  int law, n;
  float c0, c1, c2, c3;           // law constants, see eval_pair()
  float rc2_lo, rc2_hi;           // guard band around rc^2 (exact check inside)
  float in2_lo, in2_hi;           // piecewise_linear: guard band around (r0-dr)^2
  double rc, rin;                 // exact thresholds
};

// One wall law (pyrdsim.pyx:1132-1145; 9-3 wall extension).
struct WallLaw {
  int law, type, dim, pad;
  float c0, c1, c2, c3;
  float rc_lo, rc_hi;             // 9-3 wall: guard band around rc (length units)
  double r0, rc;
  long long hr0;                  // fixed-point value of r0 (tanh wall)
};

// One reaction (pyrdsim.pyx:2070-2223).
struct RxDev {
  int kind, reactant, product, catalyst, inh, inh2;
  float ratef;                    // rate as float32, rounded up
  int pad1;
  double rate, r0, dec;
  float r02_lo, r02_hi;           // guard band around r0^2
};

struct TermDev {                  // bonded term; angles in radians
  int kind, i, j, k;
  float p0, k0, thr;
  float pi;                       // angle: +1 if its theta0 == pi, else -1
  unsigned long long r0q_lo, r0q_hi;  // bond: r0^2 in fixed units^2 (128 bits)
};

struct TmplDev {
  int n_atoms, n_terms, term0, atom0;  // atom0: offset into atom-term CSR
  uint32_t bondmask[MAXA];        // bit b of [a]: (a,b) is a bonded-list pair
};

struct SysDev {
  int p0, n;                      // particle range in the sorted arrays
  int c0;                         // first global cell
  int nc[3];                      // cells per dimension
  int halo[3];                    // 1, or 0 where nc == 1 and periodic
  int ntypes;
  int periodic;                   // bit k set: dimension k periodic
  int nlaws, nwalls, nrx;
  int law0, wall0, rx0;
  int angle_is_pi;
  int has_terms;
  int rx_any_mask;                // types that are reactant of any reaction
  int rx_nb_mask;                 // ... of a neighbour-dependent reaction
  double L[3];
  double unit_d[3];               // length per fixed unit
  double inv_unit_d[3];           // fixed units per length
  double S[3];                    // reflecting: fixed value of L (as double)
  long long Si[3];                // reflecting: fixed value of L
  float unit_hi[3];               // length per high-word unit
  float inv_unit_hi[3];
  float unitf[3];                 // length per fixed unit (float32)
  int ps[3];                      // pair-word shift
  float qf[3];                    // length per pair-word unit

  // Bonds: with one fixed unit in every dimension, squared bond lengths are
  // exact 128-bit integers in units of unit^2 (bonded_terms).
  int bond128;                    // 1: every dimension has the same unit
  float unit2f;                   // unit^2 as float32
  float delta;                    // allowed displacement since the last
                                  // rebuild (Euclidean, length units)
  int hshift[3];                  // cell of high word h: (h * nc) >> hshift
                                  // (32 periodic, 30 reflecting: h <= 2^30)
  float R2;                       // candidate radius^2 (forces + reactions)
  float Rrx2;                     // reaction radius^2 (guarded)
  float Rl2;                      // Verlet-list radius^2: range + 2 delta
  double dt;
  unsigned long long seed;
  float fp[MAXT], npf[MAXT];      // dt*D and sqrt(2 dt D) per type
  unsigned int partner[MAXT];     // bit j of [i]: types i, j are partners
  unsigned short ppair[MAXT * MAXT];  // first law << 5 | count, symmetric;
                                      // bit 15: one Lennard-Jones n = 6 law
  float prc2[MAXT * MAXT];        // largest guarded rc^2 of the pair's laws
  unsigned char rxmatch[MAXT * MAXT]; // bit r of [ti * MAXT + tj]: neighbour
                                      // reaction r has reactant ti and counts tj
  // Upper bound of a particle's total propensity for the reaction prefilter:
  // rxA[t] + rxB[t] * (listed neighbours) >= the float64 total of a type-t
  // particle (linear and inhibited rates in rxA, catalysed rates in rxB).
  double rxA[MAXT], rxB[MAXT];
  float rxAf[MAXT], rxBf[MAXT];   // the same as float32, rounded up
  float dtf;                      // dt as float32, rounded up
  int rx_screen_mask;             // types whose reactions are all linear or
                                  // catalysed (float32 screening of draws)
};

// A run of consecutive particles (sorted order) of one system, handled by one
// CTA of the list kernels; the system's table offsets are copied in.
struct Chunk {
  int sys, beg, cnt;
  int law0, nlaws, wall0, nwalls, rx0, nrx;
  int pad[3];
};

struct ErrDev {
  int code, dim;
  long long particle, step;
  double value;
};

// Kernel arguments shared by the step kernels (passed by value).
struct Args {
  const SysDev* sys;
  const PairLaw* laws;
  const WallLaw* walls;
  const RxDev* rx;
  const TmplDev* tmpl;
  const TermDev* terms;
  const int* atomterm;            // term index * 4 + role, per template atom
  const int* cell_start;
  const uint32_t* xh[3];
  const uint32_t* xl[3];
  const uint32_t* xp[3];          // pair words
  const uint32_t* meta;
  const int* mol;
  const int* pid;
  const int* slot_of;             // caller index -> sorted slot
  const uint32_t* xr[3];          // high words at the last rebuild
  uint32_t* xh_out[3];
  uint32_t* xl_out[3];
  uint32_t* xp_out[3];
  uint32_t* meta_out;
  float* drift[3];
  // float64 force mode (force64.cuh): drift, the laws, walls and bonded
  // terms with their float64 deck parameters (same order as laws / walls /
  // terms), and per system [2][MAXT]: dt D and sqrt(2 dt D) per type
  double* drift_d[3];
  const rdsim_interaction* olaws;
  const rdsim_interaction* owalls;
  const rdsim_term* oterms;
  const double* typed;
  double* rates_out;              // reaction-rate hook (sorted order)
  ErrDev* err;
  const double* xi;               // injected normals for the EM step
  const double* u1;               // injected uniforms for this step
  const double* u2;
  long long step;                 // step number of this kernel's work
  long long em_step;              // step number of the fused EM update
  const long long* step_base;     // graph replays: step numbers are offsets
                                  // from this device counter
  const Chunk* chunks;            // list kernels: CTA -> particle run
  const int* nbr;                 // Verlet list (ELL, see list.cuh)
  const int* ncnt;                // entries per particle (may exceed W)
  int* nbr_out;
  int* ncnt_out;
  int W, npad;                    // list width and particle stride
  int4* rx_list;                  // [3][npad]: particles whose reaction draw
                                  // may succeed at a step, in slot step % 3,
                                  // as {sorted index, meta, list entries, pid}
  int* rx_count;                  // [3]
  const int* sid;                 // system of each particle
  int single;                     // one system: chunks follow from blockIdx
  Chunk chunk1;                   // ... with these table offsets
  int n_total;
  int flags;
  // drift-kernel timestamps (measurement): [ring][CTAs][2] global-timer
  // values of each CTA's start and end, slot = step mod ring
  unsigned long long* stamps;
  int stamp_ring;
  // period kernel (list.cuh: k_period), written by the list builder with
  // F_PERIOD_PREP: per chunk, the bitmap of the chunks its particles read
  // (list entries and bonded partners, itself included; PMASK_WORDS words),
  // the particles whose reaction draw of the rebuild step may succeed
  // (CAND_WORDS words, bit = particle within the chunk) and the progress word
  uint32_t* nbmask;
  uint32_t* cand0;
  int* pflag;
  long long wait_ns;              // period kernel: limit of one wait (ns)
};

// Period kernel: a particle whose reaction draw of the next step is pending
// carries this bit in that step's type word (bits 21-23 of the atom-index
// byte are otherwise zero: at most 32 atoms per molecule) until its chunk
// has resolved the draw and written the final word.
constexpr uint32_t META_PENDING = 1u << 23;

// Period kernel limits: chunks of one launch (bitmap width) and particles
// per chunk (candidate mask width).
constexpr int PMASK_WORDS = 40;
constexpr int PMAX_CHUNKS = PMASK_WORDS * 32;
constexpr int CAND_WORDS = 4;
// Ints per progress word of the period kernel (32: one 128-byte line each,
// so that the ~20 CTAs polling a chunk do not share a line with others).
#ifndef RD_PERIOD_FLAG_STRIDE
#define RD_PERIOD_FLAG_STRIDE 32
#endif
constexpr int PFLAG_STRIDE = RD_PERIOD_FLAG_STRIDE;

// Arguments of the period kernel besides its four step-argument blocks.
struct PeriodArgs {
  int nsteps;                     // steps of the rebuild period
  int nchunks;                    // chunks = CTAs (all resident)
  int rx;                         // prefiltered reaction phases run
  int first_rx;                   // the first step's reactions run here (its
                                  // candidates from the list builder); 0: done
                                  // before the launch
  int withhold;                   // test hook: this chunk never publishes
                                  // its progress (-1: none)
  long long wait_ns;              // limit of one wait (global timer, ns)
};

__device__ inline unsigned long long global_timer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

enum : int {
  F_STORE_DRIFT = 1,              // write the drift (sorted order)
  F_EM = 2,                       // fuse the Euler-Maruyama update
  F_NO_NOISE = 4,                 // random_force = False
  F_INJECT = 8,                   // xi / u1 / u2 come from buffers
  F_RATES_ONLY = 16,              // reaction kernel: write total rates, no draw
  F_CHECK_SKIN = 32,
  F_RX_NEXT = 64,                 // drift kernel: copy the types forward and
                                  // list the particles whose reaction draw of
                                  // the next step may succeed
  F_RX_HERE = 128,                // list builder: the same for its own step
  F_PERIOD = 256,                 // step kernels inside k_period: the step
                                  // number is the CTA's current step
  F_PERIOD_PREP = 512             // list builder: write the period kernel's
                                  // neighbour-chunk bitmaps, progress words
                                  // and (with F_RX_HERE) candidate masks
};

// Slot of the candidate list of a step: three slots, so that a drift kernel
// appends to the next step's slot and clears the one consumed two steps
// earlier, never the slot that the kernels around it read.
__host__ __device__ inline int rx_slot(long long step) {
  return (int)(((step % 3) + 3) % 3);
}

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) -------------------
struct U4 {
  uint32_t x, y, z, w;
};

__host__ __device__ inline U4 philox(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)M0 * c.x;
    uint64_t p1 = (uint64_t)M1 * c.z;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    U4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// Noise streams: tag 0 = Gaussian increments, tag 1 = reaction uniforms,
// tag 2 = second Gaussian block (3D).
__host__ __device__ inline U4 noise_words(unsigned long long seed, long long step,
                                          int pid, uint32_t tag) {
  U4 c{(uint32_t)step, (uint32_t)((unsigned long long)step >> 32), (uint32_t)pid, tag};
  return philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

}  // namespace rd
