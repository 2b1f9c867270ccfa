// engine.cu -- host side of the GB300 step engine: the C ABI of rdsim.h.
//
// One handle = one CUDA stream + device buffers for a batch of independent
// systems.  Set-up builds the flat tables (pair laws, walls, reactions,
// bonded templates), the cell grid and the CTA chunks of the list kernels;
// each rdsim_step launches, per step: [EM] -> [rebuild (cells + Verlet list)
// every freq steps] -> [reactions] -> drift (with the next step's EM fused in).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rdsim.h"
#include "device.cuh"
#include "kernels.cuh"
#include "force64.h"
#include "launch.cuh"
#include "list.cuh"
#include "observe.cuh"

using namespace rd;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

// A failing runtime call also sets the thread's last-error state; it is
// cleared here so that a later launch check does not report it again.
#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      cudaGetLastError();                                                         \
      return fail(RDSIM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    }                                                                             \
  } while (0)

constexpr double TWO32 = 4294967296.0;
constexpr double TWO64 = 18446744073709551616.0;
// Reflecting dimensions map [0, L] to [0, 2^62]: positions down to -L (an
// initial condition may lie below 0) still fit a signed 64-bit word, and the
// fixed unit L / 2^62 is a power-of-two multiple of a periodic dimension's
// L / 2^64 (square boxes get one pair-word unit in every dimension).
const long long S_REFLECT = (long long)(1ULL << 62);

struct HostSys {
  int p0, n, pid0;
  double cl_ref[3];
  double rs;
  int freq;
  double L[3];
  int periodic_mask;
  long long Si[3];
};

template <class T>
int dalloc(T** p, size_t n, int64_t* acc) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear the non-sticky allocation error
    return fail(RDSIM_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  *acc += (int64_t)(n * sizeof(T));
  return 0;
}

}  // namespace

struct rdsim_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  int D = 2, nsys = 0, N = 0;
  int64_t step = 0;
  int freq = 10;
  bool has_rx = false;
  double skin = 0, cell_min = 0, range = 0;
  int64_t device_bytes = 0;
  std::vector<HostSys> hs;
  std::vector<SysDev> sys_h;
  SysDev* sys_d = nullptr;
  PairLaw* laws_d = nullptr;
  WallLaw* walls_d = nullptr;
  RxDev* rx_d = nullptr;
  TmplDev* tmpl_d = nullptr;
  TermDev* terms_d = nullptr;
  int* atomterm_d = nullptr;
  // float64 parameters of the same tables (observables)
  rdsim_interaction* olaws_d = nullptr;
  rdsim_interaction* owalls_d = nullptr;
  rdsim_term* oterms_d = nullptr;
  // observables scratch, allocated by the first call that needs it
  double* obs_part = nullptr;          // [obs_cap][OBS_NSUM] CTA partials, then sums
  unsigned long long* obs_counts = nullptr;  // [1 + MAXT]
  int obs_cap = 0;
  unsigned long long* rdf_counts = nullptr;  // [RDF_MAX_BINS]
  int ncells = 0, nscan = 0;
  int *cell_count = nullptr, *cell_start = nullptr, *bsum = nullptr;
  // Verlet-list kernels
  int ltpp = 2;                      // lanes per particle
  bool rx_pre = true;                // reaction prefilter (see rx_may_react)
  int4* rx_list = nullptr;           // [3][npad] prefiltered particles
  int* rx_count = nullptr;           // [3]
  int W = 0;                         // list width (entries per particle)
  int npad = 0;                      // particle stride of the list
  // period kernel (list.cuh: k_period): one launch per graph-replayed period
  bool period_on = false;
  uint32_t* nbmask = nullptr;        // [chunks][PMASK_WORDS]
  uint32_t* cand0 = nullptr;         // [chunks][CAND_WORDS]
  int* pflag = nullptr;              // [chunks] progress words
  int withhold = -1;                 // test hook (rdsim_test_withhold)
  long long wait_ns = 1000000000LL;
  std::vector<Chunk> chunks_h;
  Chunk* chunks_d = nullptr;
  int* nbr = nullptr;
  int* ncnt = nullptr;
  int *cell_of = nullptr, *rank_of = nullptr, *tmp = nullptr, *sid = nullptr, *slot_of = nullptr;
  uint32_t* xh[2][3] = {};
  uint32_t* xl[2][3] = {};
  uint32_t* xp[2][3] = {};          // pair words (see device.cuh)
  uint32_t* xr[3] = {};
  uint32_t* meta[2] = {};
  int* mol[2] = {};
  int* pid[2] = {};
  float* drift[3] = {};
  // float64 force mode (force64.cuh)
  bool f64 = false;
  double* drift_d[3] = {};
  double* typed_d = nullptr;           // [nsys][2][MAXT]: dt D, sqrt(2 dt D)
  double* rates = nullptr;
  double* xbuf = nullptr;  // float64 positions in caller order (hooks)
  int* tbuf = nullptr;
  ErrDev* err = nullptr;
  double* cl_d = nullptr;
  int cx = 0, cm = 0, co = 0;
  // static per-particle data (caller order): host copies and device copies
  std::vector<uint32_t> meta_static;  // local << 16 | template << 24
  std::vector<int> mol_h;
  uint32_t* meta_static_d = nullptr;
  int* mol_static_d = nullptr;
  int* flag_d = nullptr;              // first problem of a state upload
  // injected noise staging
  double *inj_xi = nullptr, *inj_u1 = nullptr, *inj_u2 = nullptr;
  size_t inj_steps = 0;
  // trajectory ring
  int traj_stride = 0, traj_frames = 0;
  double* traj_x = nullptr;
  int* traj_t = nullptr;
  // CUDA graphs of whole rebuild periods (Philox noise only)
  bool graphs = true;
  long long* step_dev = nullptr;       // device step counter read by replays
  long long step_dev_value = -1;       // its value once queued work has run
  struct GraphEntry {
    cudaGraphExec_t exec;
    int64_t launches[RDSIM_PROFILE_CLASSES];
  };
  std::map<int, GraphEntry> graph_cache;
  // kernel accounting
  int64_t nlaunch[RDSIM_PROFILE_CLASSES] = {};
  bool prof = false;
  struct Pend {
    int cls;
    cudaEvent_t a, b;
  };
  std::vector<Pend> pending;
  std::vector<cudaEvent_t> ev_pool;
  double prof_ms[RDSIM_PROFILE_CLASSES] = {};
  // drift-kernel timestamps (rdsim_set_profiling bit 1)
  bool stamp_on = false;
  unsigned long long* stamps = nullptr;   // [ring][CTAs][2]
  unsigned long long* stamp_sum = nullptr;  // [2]: span sum (ns), launches
  int stamp_ring = 0;
  int64_t prof_n[RDSIM_PROFILE_CLASSES] = {};
};

namespace {

enum { P_FORCE = 0, P_REACT = 1, P_EM = 2, P_REBUILD = 3, P_HOOK = 4 };

cudaEvent_t take_event(rdsim_handle* h) {
  if (!h->ev_pool.empty()) {
    cudaEvent_t e = h->ev_pool.back();
    h->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Brackets the launches of one class with events when profiling is on.
struct ProfScope {
  rdsim_handle* h;
  int cls;
  cudaEvent_t a = nullptr;
  ProfScope(rdsim_handle* h_, int c, int nkernels) : h(h_), cls(c) {
    h->nlaunch[c] += nkernels;
    if (h->prof) {
      a = take_event(h);
      cudaEventRecord(a, h->stream);
    }
  }
  ~ProfScope() {
    if (a) {
      cudaEvent_t b = take_event(h);
      cudaEventRecord(b, h->stream);
      h->pending.push_back({cls, a, b});
    }
  }
};

void resolve_profile(rdsim_handle* h) {
  for (auto& p : h->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      h->prof_ms[p.cls] += ms;
      h->prof_n[p.cls] += 1;
    }
    h->ev_pool.push_back(p.a);
    h->ev_pool.push_back(p.b);
  }
  h->pending.clear();
}

Args make_args(rdsim_handle* h) {
  Args a;
  std::memset(&a, 0, sizeof a);
  a.sys = h->sys_d;
  a.laws = h->laws_d;
  a.walls = h->walls_d;
  a.rx = h->rx_d;
  a.tmpl = h->tmpl_d;
  a.terms = h->terms_d;
  a.atomterm = h->atomterm_d;
  a.cell_start = h->cell_start;
  for (int k = 0; k < 3; k++) {
    a.xh[k] = h->xh[h->cx][k];
    a.xl[k] = h->xl[h->cx][k];
    a.xp[k] = h->xp[h->cx][k];
    a.xh_out[k] = h->xh[1 - h->cx][k];
    a.xl_out[k] = h->xl[1 - h->cx][k];
    a.xp_out[k] = h->xp[1 - h->cx][k];
    a.xr[k] = h->xr[k];
    a.drift[k] = h->drift[k];
    a.drift_d[k] = h->drift_d[k];
  }
  a.olaws = h->olaws_d;
  a.owalls = h->owalls_d;
  a.oterms = h->oterms_d;
  a.typed = h->typed_d;
  a.meta = h->meta[h->cm];
  a.meta_out = h->meta[1 - h->cm];
  a.mol = h->mol[h->co];
  a.pid = h->pid[h->co];
  a.slot_of = h->slot_of;
  a.rates_out = h->rates;
  a.err = h->err;
  a.n_total = h->N;
  a.chunks = h->chunks_d;
  a.nbr = h->nbr;
  a.ncnt = h->ncnt;
  a.nbr_out = h->nbr;
  a.ncnt_out = h->ncnt;
  a.W = h->W;
  a.rx_list = h->rx_list;
  a.rx_count = h->rx_count;
  a.sid = h->sid;
  a.npad = h->npad;
  a.single = h->nsys == 1 ? 1 : 0;
  if (h->stamp_on) {
    a.stamps = h->stamps;
    a.stamp_ring = h->stamp_ring;
  }
  if (!h->chunks_h.empty()) a.chunk1 = h->chunks_h[0];
  a.nbmask = h->nbmask;
  a.cand0 = h->cand0;
  a.pflag = h->pflag;
  return a;
}

template <int D, int TPP>
void launch_list(rdsim_handle* h, bool react, const Args& a) {
  const dim3 grid((unsigned)h->chunks_h.size());
  if (react) launch(k_react_l<D, TPP>, grid, LBLOCK, h->stream, a);
  else launch(k_force_l<D, TPP>, grid, LBLOCK, h->stream, a);
}

template <int D>
void launch_list_d(rdsim_handle* h, bool react, const Args& a) {
  if (h->ltpp == 1) launch_list<D, 1>(h, react, a);
  else if (h->ltpp == 2) launch_list<D, 2>(h, react, a);
  else if (h->ltpp == 8) launch_list<D, 8>(h, react, a);
  else launch_list<D, 4>(h, react, a);
}

template <int D>
void launch_listed(rdsim_handle* h, unsigned g, const Args& a) {
  if (h->ltpp == 1) launch(k_react_listed<D, 1>, g, LBLOCK, h->stream, a);
  else if (h->ltpp == 2) launch(k_react_listed<D, 2>, g, LBLOCK, h->stream, a);
  else if (h->ltpp == 8) launch(k_react_listed<D, 8>, g, LBLOCK, h->stream, a);
  else launch(k_react_listed<D, 4>, g, LBLOCK, h->stream, a);
}

template <int D>
void launch_nlist(rdsim_handle* h, const Args& a) {
  const dim3 grid((unsigned)h->chunks_h.size());
  const unsigned per = (unsigned)(LBLOCK / h->ltpp * (D == 1 ? 1 : 3));
  if (h->ltpp == 1) launch(k_nlist<D, 1>, grid, per, h->stream, a);
  else if (h->ltpp == 2) launch(k_nlist<D, 2>, grid, per, h->stream, a);
  else if (h->ltpp == 8) launch(k_nlist<D, 8>, grid, per, h->stream, a);
  else launch(k_nlist<D, 4>, grid, per, h->stream, a);
}

void launch_step_kernel(rdsim_handle* h, bool react, const Args& a) {
  if (h->D == 2) launch_list_d<2>(h, react, a);
  else if (h->D == 3) launch_list_d<3>(h, react, a);
  else launch_list_d<1>(h, react, a);
}

unsigned nblk(int n, int b = 256) { return (unsigned)((n + b - 1) / b); }

// `prefilter`: the list builder also runs the reaction prefilter of `step`
// (then the reaction kernel of that step visits the listed particles only);
// `rel`: step numbers are offsets from the device counter (graph capture).
int rebuild(rdsim_handle* h, long long step = 0, bool prefilter = false, bool rel = false,
            bool period_prep = false) {
  const int n = h->N;
  ProfScope ps(h, P_REBUILD, h->ncells <= SCAN1_T * SCAN1_I ? 5 : 6);
  uint32_t* const* x = h->xh[h->cx];
  // a captured period advances the step counter by one period in k_bin
  long long* ctr = rel ? h->step_dev : nullptr;
  const long long add = h->freq;
  if (h->D == 2)
    launch(k_bin<2>, nblk(n), 256, h->stream, h->sys_d, h->sid, x[0], x[1], x[2], n, h->cell_of, h->rank_of, h->cell_count, ctr, add);
  else if (h->D == 3)
    launch(k_bin<3>, nblk(n), 256, h->stream, h->sys_d, h->sid, x[0], x[1], x[2], n, h->cell_of, h->rank_of, h->cell_count, ctr, add);
  else
    launch(k_bin<1>, nblk(n), 256, h->stream, h->sys_d, h->sid, x[0], x[1], x[2], n, h->cell_of, h->rank_of, h->cell_count, ctr, add);
  if (h->ncells <= SCAN1_T * SCAN1_I) {
    launch(k_scan_one, 1, SCAN1_T, h->stream, h->cell_count, h->ncells, h->cell_start);
  } else {
    launch(k_scan_partial, h->nscan, 256, h->stream, h->cell_count, h->ncells, h->bsum);
    launch(k_scan_final, h->nscan, 256, h->stream, h->cell_count, h->ncells, h->bsum, h->cell_start);
  }
  launch(k_scatter, nblk(n), 256, h->stream, h->cell_of, h->rank_of, h->cell_start, n, h->tmp,
         h->cell_count, h->ncells);
  Args a = make_args(h);
  OrderOut o;
  o.mol = h->mol[1 - h->co];
  o.pid = h->pid[1 - h->co];
  for (int k = 0; k < 3; k++) o.xr[k] = h->xr[k];
  o.slot_of = h->slot_of;
  if (h->D == 2) launch(k_order<2>, nblk(n), 256, h->stream, a, o, h->tmp, h->cell_of, h->cell_start, n);
  else if (h->D == 3) launch(k_order<3>, nblk(n), 256, h->stream, a, o, h->tmp, h->cell_of, h->cell_start, n);
  else launch(k_order<1>, nblk(n), 256, h->stream, a, o, h->tmp, h->cell_of, h->cell_start, n);
  h->cx = 1 - h->cx;
  h->cm = 1 - h->cm;
  h->co = 1 - h->co;
  Args b = make_args(h);
  b.step = step;
  b.step_base = rel ? h->step_dev : nullptr;
  b.flags = (prefilter ? F_RX_HERE : 0) | (period_prep ? F_PERIOD_PREP : 0);
  if (h->D == 2) launch_nlist<2>(h, b);
  else if (h->D == 3) launch_nlist<3>(h, b);
  else launch_nlist<1>(h, b);
  CK(cudaGetLastError());
  return 0;
}

// `rel`: step numbers are offsets from the device counter (graph capture)
int force(rdsim_handle* h, long long step, int flags, const double* xi_next, bool rel = false) {
  Args a = make_args(h);
  // with the period kernel on, only its launches record timestamps (one
  // span per list period; the per-step drift launches at call boundaries
  // would mix one-step spans into the average)
  if (h->period_on) a.stamps = nullptr;
  a.step_base = rel ? h->step_dev : nullptr;
  a.step = step;
  a.em_step = step + 1;
  a.flags = flags | F_CHECK_SKIN;
  a.xi = xi_next;
  {
    ProfScope ps(h, P_FORCE, 1);
    if (h->f64) CK(launch_force64(h->D, h->ltpp, (unsigned)h->chunks_h.size(), h->stream, a));
    else launch_step_kernel(h, false, a);
  }
  CK(cudaGetLastError());
  if (flags & F_EM) h->cx = 1 - h->cx;
  return 0;
}

// `listed`: the previous drift kernel copied the types forward and listed
// the particles whose draw may succeed; only those are processed.
int react(rdsim_handle* h, long long step, int flags, const double* u1, const double* u2,
          bool rel = false, bool listed = false) {
  Args a = make_args(h);
  a.step_base = rel ? h->step_dev : nullptr;
  a.step = step;
  a.flags = flags;
  a.u1 = u1;
  a.u2 = u2;
  {
    ProfScope ps(h, (flags & F_RATES_ONLY) ? P_HOOK : P_REACT, 1);
    if (listed) {
      const unsigned g = (unsigned)std::min(2 * 152, (h->N + 3) / 4);
      if (h->D == 2) launch_listed<2>(h, g, a);
      else if (h->D == 3) launch_listed<3>(h, g, a);
      else launch_listed<1>(h, g, a);
    } else {
      launch_step_kernel(h, true, a);
    }
  }
  CK(cudaGetLastError());
  if (!(flags & F_RATES_ONLY)) h->cm = 1 - h->cm;
  return 0;
}

int em(rdsim_handle* h, long long step, int flags, const double* xi) {
  Args a = make_args(h);
  a.em_step = step;
  a.flags = flags;
  a.xi = xi;
  unsigned g = nblk(h->N);
  ProfScope ps(h, P_EM, 1);
  if (h->f64) CK(launch_em64(h->D, g, h->stream, a, h->sid));
  else if (h->D == 2) launch(k_em<2>, g, 256, h->stream, a, h->sid);
  else if (h->D == 3) launch(k_em<3>, g, 256, h->stream, a, h->sid);
  else launch(k_em<1>, g, 256, h->stream, a, h->sid);
  CK(cudaGetLastError());
  h->cx = 1 - h->cx;
  return 0;
}

int snapshot(rdsim_handle* h, double* fx, int* ft) {
  Args a = make_args(h);
  unsigned g = nblk(h->N);
  if (h->D == 2) launch(k_snapshot<2>, g, 256, h->stream, h->sys_d, h->sid, a, fx, ft);
  else if (h->D == 3) launch(k_snapshot<3>, g, 256, h->stream, h->sys_d, h->sid, a, fx, ft);
  else launch(k_snapshot<1>, g, 256, h->stream, h->sys_d, h->sid, a, fx, ft);
  CK(cudaGetLastError());
  return 0;
}

int check_device_error(rdsim_handle* h) {
  ErrDev e;
  CK(cudaMemcpyAsync(&e, h->err, sizeof e, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (e.code == 0) return 0;
  CK(cudaMemsetAsync(h->err, 0, sizeof(ErrDev), h->stream));
  if (h->period_on) {
    // a period kernel that stopped early may leave draws marked pending
    k_clear_pending<<<nblk(h->N), 256, 0, h->stream>>>(h->meta[0], h->meta[1], h->N);
    CK(cudaGetLastError());
  }
  char buf[256];
  if (e.code == RDSIM_ERR_OUT_OF_BOUNDS) {
    snprintf(buf, sizeof buf,
             "x[%lld,%d] = %.17g out of bounds. Maybe the timestep is too large for the "
             "given the interaction parameters?", e.particle, e.dim, e.value);
  } else if (e.code == RDSIM_ERR_SKIN) {
    snprintf(buf, sizeof buf,
             "particle %lld moved %.6g along dimension %d since the last neighbour-list "
             "rebuild (step %lld), more than the skin allows; increase gpu_skin or "
             "rebuild more often", e.particle, e.value, e.dim, e.step);
  } else if (e.code == RDSIM_ERR_NONFINITE) {
    snprintf(buf, sizeof buf,
             "non-finite or larger-than-box update of particle %lld, dimension %d "
             "(value %.6g) at step %lld", e.particle, e.dim, e.value, e.step);
  } else if (e.code == RDSIM_ERR_SYNC) {
    snprintf(buf, sizeof buf,
             "period kernel: chunk %lld waited longer than the limit for the progress of "
             "its neighbouring chunks (step %lld); the state of this call is not valid",
             e.particle, e.step);
  } else {
    snprintf(buf, sizeof buf, "device error %d at step %lld", e.code, e.step);
  }
  return fail(e.code, buf);
}

// Caller-order float64 positions and types in xbuf / tbuf (device) -> the
// engine's state (fixed point, slot = caller index), converted exactly on
// the device (fixed_from_double).
int upload_state(rdsim_handle* h) {
  const int N = h->N;
  h->cx = h->cm = h->co = 0;
  CK(cudaMemsetAsync(h->flag_d, 0, sizeof(int), h->stream));
  StateOut a;
  std::memset(&a, 0, sizeof a);
  for (int k = 0; k < 3; k++) {
    a.xh[k] = h->xh[0][k];
    a.xl[k] = h->xl[0][k];
    a.xp[k] = h->xp[0][k];
  }
  a.meta = h->meta[0];
  a.mol = h->mol[0];
  a.pid = h->pid[0];
  a.n = N;
  const unsigned g = nblk(N);
  if (h->D == 2)
    k_from_double<2><<<g, 256, 0, h->stream>>>(h->sys_d, h->sid, h->xbuf, h->tbuf, h->meta_static_d,
                                               h->mol_static_d, a, h->flag_d);
  else if (h->D == 3)
    k_from_double<3><<<g, 256, 0, h->stream>>>(h->sys_d, h->sid, h->xbuf, h->tbuf, h->meta_static_d,
                                               h->mol_static_d, a, h->flag_d);
  else
    k_from_double<1><<<g, 256, 0, h->stream>>>(h->sys_d, h->sid, h->xbuf, h->tbuf, h->meta_static_d,
                                               h->mol_static_d, a, h->flag_d);
  CK(cudaGetLastError());
  int bad = 0;
  CK(cudaMemcpyAsync(&bad, h->flag_d, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (bad == 1) return fail(RDSIM_ERR_ARG, "initial position outside the reflecting box");
  if (bad == 2) return fail(RDSIM_ERR_ARG, "non-finite initial position");
  if (bad == 3) return fail(RDSIM_ERR_ARG, "particle type without tau_by_tauD entry");
  return 0;
}

int initial_drift(rdsim_handle* h) {
  CK(cudaMemsetAsync(h->rx_count, 0, 3 * sizeof(int), h->stream));
  int rc = rebuild(h, 0, false, false, h->period_on);
  if (rc) return rc;
  rc = force(h, h->step, F_STORE_DRIFT, nullptr);
  if (rc) return rc;
  return check_device_error(h);
}

// True if a trajectory frame falls on a step in [a, b].
bool snapshot_in(rdsim_handle* h, long long a, long long b) {
  if (h->traj_frames <= 0) return false;
  const long long first = ((a + h->traj_stride - 1) / h->traj_stride) * h->traj_stride;
  return first <= b;
}

template <int D>
void launch_period_d(rdsim_handle* h, const Args* A, const PeriodArgs& p) {
  const dim3 g((unsigned)p.nchunks);
  if (h->ltpp == 1) launch(k_period<D, 1>, g, LBLOCK, h->stream, A[0], A[1], A[2], A[3], p);
  else if (h->ltpp == 2) launch(k_period<D, 2>, g, LBLOCK, h->stream, A[0], A[1], A[2], A[3], p);
  else if (h->ltpp == 8) launch(k_period<D, 8>, g, LBLOCK, h->stream, A[0], A[1], A[2], A[3], p);
  else launch(k_period<D, 4>, g, LBLOCK, h->stream, A[0], A[1], A[2], A[3], p);
}

// Steps of one list period as one launch of the period kernel (the list's
// last rebuild ran with period_prep): the drift arguments of steps of parity
// P read positions xh[cx ^ P] and the types after the step's reactions; the
// reaction arguments read the types before them.  rel: a whole period in a
// graph capture, step numbers offsets from the device counter, the first
// step's reactions in the kernel.  Otherwise (the rest of a period after a
// call started inside it): `nsteps` steps from step `step0`, whose reactions
// already ran on the reaction kernels.
int period_launch(rdsim_handle* h, int kf, bool pre, bool rel = true, long long step0 = 0,
                  int nsteps = 0) {
  const int cx0 = h->cx;
  const int cm0 = (!rel && h->has_rx) ? h->cm ^ 1 : h->cm;
  Args A[4];
  for (int P = 0; P < 2; P++) {
    h->cx = cx0 ^ P;
    h->cm = cm0 ^ P;
    Args r = make_args(h);
    h->cm = h->has_rx ? (cm0 ^ P ^ 1) : cm0;
    Args d = make_args(h);
    d.flags = F_EM | F_CHECK_SKIN | F_PERIOD | kf;
    r.flags = F_PERIOD | kf;
    d.step_base = r.step_base = rel ? h->step_dev : nullptr;
    d.step = r.step = rel ? 0 : step0;
    d.wait_ns = r.wait_ns = h->wait_ns;
    if (!rel) d.stamps = r.stamps = nullptr;  // the timestamps cover whole periods
    A[P] = d;
    A[2 + P] = r;
  }
  h->cx = cx0;
  h->cm = (!rel && h->has_rx) ? cm0 ^ 1 : cm0;
  PeriodArgs p;
  std::memset(&p, 0, sizeof p);
  p.nsteps = rel ? h->freq : nsteps;
  p.nchunks = (int)h->chunks_h.size();
  p.rx = pre ? 1 : 0;
  p.first_rx = rel ? 1 : 0;
  if (!rel)  // progress words of a launch without the list builder before it
    CK(cudaMemsetAsync(h->pflag, 0, sizeof(int) * (size_t)p.nchunks * PFLAG_STRIDE, h->stream));
  p.withhold = h->withhold;
  p.wait_ns = h->wait_ns;
  {
    ProfScope ps(h, P_FORCE, 1);
    if (h->D == 2) launch_period_d<2>(h, A, p);
    else if (h->D == 3) launch_period_d<3>(h, A, p);
    else launch_period_d<1>(h, A, p);
  }
  CK(cudaGetLastError());
  return 0;
}

// Resident CTAs of the period kernel on the handle's device (0 if unknown).
template <int D>
int period_capacity_d(int tpp) {
  int nb = 0;
  cudaError_t e;
  if (tpp == 1) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_period<D, 1>, LBLOCK, 0);
  else if (tpp == 2) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_period<D, 2>, LBLOCK, 0);
  else if (tpp == 8) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_period<D, 8>, LBLOCK, 0);
  else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_period<D, 4>, LBLOCK, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return nb;
}

int period_capacity(rdsim_handle* h) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const int nb = h->D == 2 ? period_capacity_d<2>(h->ltpp)
                           : (h->D == 3 ? period_capacity_d<3>(h->ltpp) : period_capacity_d<1>(h->ltpp));
  return nb * sms;
}

// One rebuild period (steps s .. s+freq-1, each ending with the fused EM
// update of the next step) as a CUDA graph.  Graphs are cached per buffer
// parity state; kernel step numbers are offsets from a device counter that
// the graph's first kernel (k_bin) advances by freq: before a replay of the
// period starting at s it holds s - freq.
int run_period_graph(rdsim_handle* h, long long s, int kf, bool pre) {
  const int key = h->cx | (h->cm << 1) | (h->co << 2) | ((kf & F_NO_NOISE) ? 8 : 0);
  auto it = h->graph_cache.find(key);
  const int cx0 = h->cx, cm0 = h->cm, co0 = h->co;
  if (it == h->graph_cache.end()) {
    int64_t before[RDSIM_PROFILE_CLASSES];
    std::memcpy(before, h->nlaunch, sizeof before);
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const bool one_launch = h->period_on && (pre || !h->has_rx);
    int rc = rebuild(h, 0, pre, true, one_launch);
    if (one_launch) {
      if (!rc) rc = period_launch(h, kf, pre);
    } else {
      for (int i = 0; i < h->freq && !rc; i++) {
        // the prefiltered particles of step i are listed by the list builder
        // (i = 0) or by the drift kernel of step i - 1
        const bool flagged = pre, flag_next = pre && i + 1 < h->freq;
        if (h->has_rx) rc = react(h, i, kf, nullptr, nullptr, true, flagged);
        if (!rc) rc = force(h, i, F_EM | kf | (flag_next ? F_RX_NEXT : 0), nullptr, true);
      }
    }
    cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ec != cudaSuccess) return fail(RDSIM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
    rdsim_handle::GraphEntry e;
    ec = cudaGraphInstantiate(&e.exec, g, 0);
    cudaGraphDestroy(g);
    if (ec != cudaSuccess) return fail(RDSIM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ec));
    for (int c = 0; c < RDSIM_PROFILE_CLASSES; c++) {
      e.launches[c] = h->nlaunch[c] - before[c];  // counted when replayed
      h->nlaunch[c] = before[c];
    }
    it = h->graph_cache.emplace(key, e).first;
    h->cx = cx0;
    h->cm = cm0;
    h->co = co0;
  }
  if (h->step_dev_value != s - h->freq)
    launch(k_set_counter, 1, 1, h->stream, h->step_dev, s - h->freq, 0);
  CK(cudaGetLastError());
  CK(cudaGraphLaunch(it->second.exec, h->stream));
  h->step_dev_value = s;
  for (int c = 0; c < RDSIM_PROFILE_CLASSES; c++) h->nlaunch[c] += it->second.launches[c];
  const int flips = (1 + h->freq) & 1;  // rebuild + freq updates / reactions
  h->cx ^= flips;
  if (h->has_rx) h->cm ^= flips;
  else h->cm ^= 1;
  h->co ^= 1;
  return 0;
}

void free_all(rdsim_handle* h) {
  auto F = [](void* p) {
    if (p) cudaFree(p);
  };
  F(h->sys_d); F(h->laws_d); F(h->walls_d); F(h->rx_d); F(h->tmpl_d);
  F(h->terms_d); F(h->atomterm_d); F(h->cell_count); F(h->cell_start); F(h->bsum);
  F(h->cell_of); F(h->rank_of); F(h->tmp); F(h->sid); F(h->slot_of);
  F(h->chunks_d); F(h->nbr); F(h->ncnt); F(h->rx_list); F(h->rx_count);
  F(h->nbmask); F(h->cand0); F(h->pflag);
  for (int b = 0; b < 2; b++) {
    for (int k = 0; k < 3; k++) { F(h->xh[b][k]); F(h->xl[b][k]); F(h->xp[b][k]); }
    F(h->meta[b]); F(h->mol[b]); F(h->pid[b]);
  }
  for (int k = 0; k < 3; k++) { F(h->xr[k]); F(h->drift[k]); F(h->drift_d[k]); }
  F(h->typed_d);
  F(h->rates); F(h->xbuf); F(h->tbuf); F(h->err); F(h->cl_d);
  F(h->meta_static_d); F(h->mol_static_d); F(h->flag_d);
  F(h->inj_xi); F(h->inj_u1); F(h->inj_u2); F(h->traj_x); F(h->traj_t);
  F(h->olaws_d); F(h->owalls_d); F(h->oterms_d); F(h->obs_part); F(h->obs_counts);
  F(h->rdf_counts);
  F(h->stamps);
  F(h->stamp_sum);
  for (auto& p : h->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : h->ev_pool) cudaEventDestroy(e);
  for (auto& g : h->graph_cache) cudaGraphExecDestroy(g.second.exec);
  h->graph_cache.clear();
  F(h->step_dev);
  if (h->stream) cudaStreamDestroy(h->stream);
}

// Half-width of the guard band around r^2 inside which the float64 distance
// decides.  The kernels' float32 r^2 from pair words errs by less than
// 5e-7 r^2 (rounding of the squares, the unit and the sum) plus 2 r sqrt(3)
// unit (truncation of both coordinates to the word's unit); the band is
// four times wider.
// The smallest float32 not below v (v >= 0).
float float_up(double v) {
  float f = (float)v;
  if ((double)f < v) f = std::nextafter(f, 3.0e38f);
  return f;
}

float guard2(double r, double unit) {
  return (float)(r * r * 2e-6 + 2.0 * r * 4.0 * unit + 1e-12);
}

}  // namespace

extern "C" {

const char* rdsim_last_error(void) { return g_err.c_str(); }

int rdsim_create(const rdsim_system* systems, int32_t n_systems, const rdsim_options* options,
                 rdsim_handle** out) {
  if (!systems || n_systems <= 0 || !out) return fail(RDSIM_ERR_ARG, "no systems");
  rdsim_options opt;
  std::memset(&opt, 0, sizeof opt);
  if (options) opt = *options;
  auto* h = new rdsim_handle();
  h->device = opt.device;
  h->D = systems[0].n_dim;
  if (opt.force_precision != 0 && opt.force_precision != 1) {
    delete h;
    return fail(RDSIM_ERR_ARG, "force_precision must be 0 (float32) or 1 (float64)");
  }
  h->f64 = opt.force_precision == 1;
  h->nsys = n_systems;
  int rc = 0;
  auto bail = [&](int code) {
    free_all(h);
    delete h;
    return code;
  };
  if (cudaSetDevice(h->device) != cudaSuccess) return bail(fail(RDSIM_ERR_CUDA, "cudaSetDevice failed"));
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(RDSIM_ERR_CUDA, "cudaStreamCreate failed"));
  const int D = h->D;
  if (D < 1 || D > 3) return bail(fail(RDSIM_ERR_ARG, "n_dim must be 1, 2 or 3"));

  std::vector<PairLaw> laws;
  std::vector<WallLaw> walls;
  std::vector<RxDev> rxs;
  std::vector<TmplDev> tmpls;
  std::vector<TermDev> terms;
  std::vector<rdsim_interaction> olaws, owalls;  // float64 copies, same order
  std::vector<rdsim_term> oterms;
  std::vector<double> typed;  // per system: dt D and sqrt(2 dt D) per type
  std::vector<int> atomterm;
  std::vector<double> x_all;
  std::vector<int> t_all;
  std::vector<int> sid_h;
  int total_cells = 0;
  double skin_report = 0, cell_report = 1e300, range_report = 0;
  bool rx_pre_worth = true;  // few draws expected to pass the bound
  if (opt.threads_per_particle == 1 || opt.threads_per_particle == 2 ||
      opt.threads_per_particle == 4 || opt.threads_per_particle == 8)
    h->ltpp = opt.threads_per_particle;
  double list_expect = 0;  // expected list entries per particle (densest system)

  for (int si = 0; si < n_systems; si++) {
    const rdsim_system& S = systems[si];
    if (S.n_dim != D) return bail(fail(RDSIM_ERR_ARG, "all systems of a batch must share n_dim"));
    if (S.n_particles <= 0) return bail(fail(RDSIM_ERR_ARG, "system without particles"));
    if (S.n_types <= 0 || S.n_types > MAXT) return bail(fail(RDSIM_ERR_UNSUPPORTED, "1..16 particle types supported"));
    if (S.n_interactions > MAXI) return bail(fail(RDSIM_ERR_UNSUPPORTED, "at most 32 interactions per system"));
    if (S.n_reactions > MAXR) return bail(fail(RDSIM_ERR_UNSUPPORTED, "at most 8 reactions per system"));
    if (S.neighbor_list_update_frequency <= 0) return bail(fail(RDSIM_ERR_ARG, "neighbor_list_update_frequency must be positive"));
    if (si == 0) h->freq = opt.list_period > 0 ? opt.list_period : S.neighbor_list_update_frequency;
    else if (S.neighbor_list_update_frequency != systems[0].neighbor_list_update_frequency)
      return bail(fail(RDSIM_ERR_UNSUPPORTED, "batched systems must share neighbor_list_update_frequency"));
    SysDev sd;
    std::memset(&sd, 0, sizeof sd);
    HostSys hsys;
    std::memset(&hsys, 0, sizeof hsys);
    sd.p0 = h->N;
    sd.n = S.n_particles;
    sd.ntypes = S.n_types;
    sd.dt = S.dt;
    sd.dtf = float_up(S.dt);
    sd.seed = S.seed ^ (0x9E3779B97F4A7C15ULL * (unsigned long long)si);
    sd.angle_is_pi = S.angle_is_pi;
    hsys.p0 = h->N;
    hsys.n = S.n_particles;
    hsys.pid0 = h->N;
    hsys.rs = S.rs;
    hsys.freq = S.neighbor_list_update_frequency;
    double max_unit = 0;
    for (int k = 0; k < D; k++) {
      if (!(S.L[k] > 0)) return bail(fail(RDSIM_ERR_ARG, "box lengths must be positive"));
      sd.L[k] = S.L[k];
      hsys.L[k] = S.L[k];
      // pyrdsim.pyx:2266 wraps for periodic >= 0 but applies the minimum image
      // only for periodic > 0 (1540-1564, 1629); the mixed case 0 is rejected
      if (S.periodic[k] == 0)
        return bail(fail(RDSIM_ERR_UNSUPPORTED, "periodic must be > 0 (periodic) or < 0 (reflecting)"));
      const bool per = S.periodic[k] > 0;
      if (per) {
        sd.periodic |= 1 << k;
        hsys.periodic_mask |= 1 << k;
        sd.unit_d[k] = S.L[k] / TWO64;
        sd.inv_unit_d[k] = TWO64 / S.L[k];
        sd.unit_hi[k] = (float)(S.L[k] / TWO32);
        sd.inv_unit_hi[k] = (float)(TWO32 / S.L[k]);
        sd.hshift[k] = 32;
      } else {
        sd.Si[k] = S_REFLECT;
        hsys.Si[k] = S_REFLECT;
        sd.S[k] = (double)S_REFLECT;
        sd.unit_d[k] = S.L[k] / (double)S_REFLECT;
        sd.inv_unit_d[k] = (double)S_REFLECT / S.L[k];
        sd.unit_hi[k] = (float)(S.L[k] * TWO32 / (double)S_REFLECT);
        sd.inv_unit_hi[k] = (float)((double)S_REFLECT / (S.L[k] * TWO32));
        sd.hshift[k] = 30;  // high words of [0, 2^62] span [0, 2^30]
      }
      max_unit = std::max(max_unit, (double)sd.unit_hi[k]);
    }
    // Pair words (device.cuh): listed pairs are at most (list radius + 2
    // delta) <= 2 rs apart at any step of a rebuild period (rs bounds the
    // list radius, rebuilt every freq steps, and the displacement check
    // stops a call before a particle exceeds delta); the shift is the
    // smallest whose range 2^31 q holds twice that.
    double max_q = 0;
    {
      const double sep = 2.0 * std::max(S.rs, 1e-3) + 8.0 * max_unit;
      for (int k = 0; k < D; k++) {
        int ps = 0;
        while (ps < 32 && std::ldexp(sd.unit_d[k], ps + 31) < 2.0 * sep) ps++;
        sd.ps[k] = ps;
        const double q = std::ldexp(sd.unit_d[k], ps);
        sd.qf[k] = (float)q;
        sd.unitf[k] = (float)sd.unit_d[k];
        max_q = std::max(max_q, q);
      }
      sd.bond128 = 1;
      for (int k = 1; k < D; k++)
        if (sd.unit_d[k] != sd.unit_d[0]) sd.bond128 = 0;
      sd.unit2f = (float)(sd.unit_d[0] * sd.unit_d[0]);
    }
    // reference cell geometry for the cell-id hook (pyrdsim.pyx:1436-1444)
    if (S.rs > 0 && S.cell_length_ratio > 0) {
      for (int k = 0; k < D; k++) {
        int l = 1;
        while (S.L[k] / (double)(l + 1) >= S.rs / (double)S.cell_length_ratio && l < (1 << 28)) l += 1;
        hsys.cl_ref[k] = S.L[k] / (double)l;
      }
    }
    // per-type prefactors (pyrdsim.pyx:488-496) and partners (1157-1263)
    typed.resize(typed.size() + 2 * MAXT, 0.0);
    double* td = typed.data() + typed.size() - 2 * MAXT;
    for (int t = 0; t < S.n_types; t++) {
      double tau = S.tau_by_tauD[t];
      if (tau < 0) {
        sd.fp[t] = 0.f;
        sd.npf[t] = 0.f;
      } else {
        sd.fp[t] = (float)(S.dt * tau);
        sd.npf[t] = (float)std::sqrt(2.0 * S.dt * tau);
        td[t] = S.dt * tau;
        td[MAXT + t] = std::sqrt(2.0 * S.dt * tau);
      }
    }
    auto add_partner = [&](int a, int b) -> bool {
      if (a < 0 || b < 0 || a >= MAXT || b >= MAXT) return false;
      sd.partner[a] |= 1u << b;
      sd.partner[b] |= 1u << a;
      return true;
    };
    // pair laws grouped by sorted type pair, file order within a pair
    sd.law0 = (int)laws.size();
    sd.wall0 = (int)walls.size();
    double R = 0;
    std::vector<std::vector<PairLaw>> by_pair(MAXT * MAXT);
    std::vector<std::vector<rdsim_interaction>> by_pair_o(MAXT * MAXT);
    for (int q = 0; q < S.n_interactions; q++) {
      const rdsim_interaction& it = S.interactions[q];
      if (it.law == RDSIM_LAW_WALL || it.law == RDSIM_LAW_WALL93) {
        if (it.type_b < 0 || it.type_b >= D) return bail(fail(RDSIM_ERR_ARG, "wall direction out of range"));
        if ((int)walls.size() - sd.wall0 >= MAXW) return bail(fail(RDSIM_ERR_UNSUPPORTED, "at most 8 walls per system"));
        WallLaw w;
        std::memset(&w, 0, sizeof w);
        w.law = it.law;
        w.type = it.type_a;
        w.dim = it.type_b;
        w.r0 = it.r0;
        w.rc = it.rc;
        if (it.law == RDSIM_LAW_WALL) {
          if (it.a == 0) return bail(fail(RDSIM_ERR_ARG, "wall with a = 0"));
          w.c0 = (float)(it.u0 * (1.0 / it.a) / 2.0);
          w.c2 = (float)(1.0 / it.a);
          w.hr0 = (long long)std::llround(it.r0 / (double)sd.unit_hi[w.dim]);
        } else {
          w.c0 = (float)it.u0;
          w.c1 = (float)it.r0;
          w.rc_lo = (float)(it.rc * (1 - 1e-5) - 4 * sd.unit_hi[w.dim]);
          w.rc_hi = (float)(it.rc * (1 + 1e-5) + 4 * sd.unit_hi[w.dim]);
        }
        walls.push_back(w);
        owalls.push_back(it);
        continue;
      }
      if (it.law < RDSIM_LAW_LJ || it.law > RDSIM_LAW_PIECEWISE_LINEAR)
        return bail(fail(RDSIM_ERR_ARG, "unknown interaction law"));
      if (!add_partner(it.type_a, it.type_b)) return bail(fail(RDSIM_ERR_UNSUPPORTED, "interaction type out of range"));
      // pyrdsim.pyx:1999-2007: only a pair listed as (small, large) ever matches
      if (it.type_a > it.type_b) continue;
      PairLaw L;
      std::memset(&L, 0, sizeof L);
      L.law = it.law;
      L.n = it.n;
      double rc = it.law == RDSIM_LAW_PIECEWISE_LINEAR ? it.r0 : it.rc;
      L.rc = rc;
      switch (it.law) {
        case RDSIM_LAW_LJ:
          L.c0 = (float)(-2.0 * it.n * it.u0);
          L.c1 = (float)(it.r0 * it.r0);
          break;
        case RDSIM_LAW_TANH:
          if (it.a == 0) return bail(fail(RDSIM_ERR_ARG, "tanh interaction with a = 0"));
          L.c0 = (float)(it.u0 * (1.0 / it.a) / 2.0);
          L.c1 = (float)it.r0;
          L.c2 = (float)(1.0 / it.a);
          break;
        case RDSIM_LAW_YUKAWA:
          L.c0 = (float)(-it.u0 / it.r0);
          L.c1 = (float)it.r0;
          L.c2 = (float)(1.0 / it.r0);
          break;
        case RDSIM_LAW_HARMONIC:
          L.c0 = (float)it.u0;
          break;
        case RDSIM_LAW_PIECEWISE_LINEAR:
          L.c0 = (float)(it.u0 / it.dr);
          L.rin = it.r0 - it.dr;
          break;
      }
      float g = guard2(rc, max_q);
      L.rc2_lo = (float)(rc * rc) - g;
      L.rc2_hi = (float)(rc * rc) + g;
      if (it.law == RDSIM_LAW_PIECEWISE_LINEAR) {
        double ri = std::max(0.0, L.rin);
        float gi2 = guard2(ri, max_q);
        L.in2_lo = (float)(ri * ri) - gi2;
        L.in2_hi = (float)(ri * ri) + gi2;
      }
      if (rc > 0) R = std::max(R, rc);
      by_pair[it.type_a * MAXT + it.type_b].push_back(L);
      by_pair_o[it.type_a * MAXT + it.type_b].push_back(it);
    }
    float R2 = 0.f;
    for (int a = 0; a < MAXT; a++)
      for (int b = a; b < MAXT; b++) {
        auto& v = by_pair[a * MAXT + b];
        if (v.empty()) continue;
        int first = (int)laws.size() - sd.law0;
        if (first + (int)v.size() > 1023) return bail(fail(RDSIM_ERR_UNSUPPORTED, "too many pair laws"));
        for (const rdsim_interaction& it : by_pair_o[a * MAXT + b]) olaws.push_back(it);
        for (auto& L : v) {
          laws.push_back(L);
          R2 = std::max(R2, L.rc2_hi);
          sd.prc2[a * MAXT + b] = std::max(sd.prc2[a * MAXT + b], L.rc2_hi);
        }
        sd.prc2[b * MAXT + a] = sd.prc2[a * MAXT + b];
        // bit 15: the pair has a single Lennard-Jones law with n = 6 (the
        // drift kernel evaluates it inline)
        const bool lj6 = v.size() == 1 && v[0].law == RDSIM_LAW_LJ && v[0].n == 6;
        unsigned short code = (unsigned short)((first << 5) | (int)v.size() | (lj6 ? 0x8000 : 0));
        sd.ppair[a * MAXT + b] = code;
        sd.ppair[b * MAXT + a] = code;
      }
    sd.nlaws = (int)laws.size() - sd.law0;
    sd.nwalls = (int)walls.size() - sd.wall0;
    if (sd.nlaws > MAXI) return bail(fail(RDSIM_ERR_UNSUPPORTED, "too many pair laws"));
    // reactions
    sd.rx0 = (int)rxs.size();
    sd.rx_screen_mask = (1 << MAXT) - 1;
    float Rrx2 = 0.f;
    for (int q = 0; q < S.n_reactions; q++) {
      const rdsim_reaction& r = S.reactions[q];
      RxDev x;
      std::memset(&x, 0, sizeof x);
      x.kind = r.kind;
      x.reactant = r.reactant;
      x.product = r.product;
      x.catalyst = r.catalyst;
      x.inh = r.inhibitor;
      x.inh2 = r.inhibitor2;
      x.rate = r.rate;
      x.r0 = r.r0;
      x.dec = r.rate_decrease;
      x.ratef = float_up(r.rate);
      if (r.product < 0 || r.product >= S.n_types || r.reactant < 0 || r.reactant >= MAXT)
        return bail(fail(RDSIM_ERR_UNSUPPORTED, "reaction types out of range"));
      if (r.kind != RDSIM_RX_LINEAR) {
        if (r.kind == RDSIM_RX_CATALYZED) {
          if (!add_partner(r.reactant, r.catalyst)) return bail(fail(RDSIM_ERR_UNSUPPORTED, "reaction type out of range"));
        } else if (r.kind == RDSIM_RX_INHIBITED) {
          if (!add_partner(r.reactant, r.inhibitor)) return bail(fail(RDSIM_ERR_UNSUPPORTED, "reaction type out of range"));
          if (r.inhibitor2 >= 0) add_partner(r.reactant, r.inhibitor2);
        } else {
          return bail(fail(RDSIM_ERR_ARG, "unknown reaction kind"));
        }
        float g = guard2(r.r0, max_q);
        x.r02_lo = (float)(r.r0 * r.r0) - g;
        x.r02_hi = (float)(r.r0 * r.r0) + g;
        Rrx2 = std::max(Rrx2, x.r02_hi);
        R = std::max(R, r.r0);
        sd.rx_nb_mask |= 1 << r.reactant;
        for (int tj = 0; tj < MAXT; tj++) {
          const bool m = (r.kind == RDSIM_RX_CATALYZED && tj == r.catalyst) ||
                         (r.kind == RDSIM_RX_INHIBITED && (tj == r.inhibitor || tj == r.inhibitor2));
          if (m) sd.rxmatch[r.reactant * MAXT + tj] |= (unsigned char)(1u << q);
        }
      }
      sd.rx_any_mask |= 1 << r.reactant;
      if (r.kind == RDSIM_RX_CATALYZED) sd.rxB[r.reactant] += r.rate;
      else sd.rxA[r.reactant] += r.rate;  // linear; inhibited at most its rate
      if (r.kind == RDSIM_RX_INHIBITED) sd.rx_screen_mask &= ~(1 << r.reactant);
      if (!(r.rate >= 0.0 && std::isfinite(r.rate)) ||
          (r.kind == RDSIM_RX_INHIBITED && !(r.rate_decrease >= 0.0)))
        h->rx_pre = false;  // the bound needs non-negative rates
      rxs.push_back(x);
    }
    sd.nrx = S.n_reactions;
    for (int t = 0; t < MAXT; t++) {  // bounds above the float64 sums
      sd.rxAf[t] = float_up(sd.rxA[t] * (1.0 + 1e-12));
      sd.rxBf[t] = float_up(sd.rxB[t] * (1.0 + 1e-12));
    }
    if (S.n_reactions > 0) h->has_rx = true;
    sd.R2 = R2;
    sd.Rrx2 = Rrx2;
    // skin: diffusion over one rebuild period plus margin, within rs; at
    // least 15 standard deviations of the period's diffusion per dimension
    // (the allowed displacement, half the skin, then exceeds 7.5 of them: a
    // chance below 1e-12 per particle and period)
    double sig = 0;
    for (int t = 0; t < S.n_types; t++)
      if (S.tau_by_tauD[t] > 0) sig = std::max(sig, std::sqrt(2.0 * S.dt * S.tau_by_tauD[t]));
    const double diff = sig * std::sqrt((double)h->freq);
    double skin = opt.skin > 0 ? opt.skin : std::max(10.0 * diff + 0.05 * R + 0.1, 15.0 * diff);
    double delta = skin / 2;
    if (R > 0) {
      double room = (S.rs - R) / 2.0;
      if (room <= 1e-6 * R)
        return bail(fail(RDSIM_ERR_UNSUPPORTED,
                         "rs must exceed the largest interaction / reaction range"));
      delta = std::min(delta, room);
    }
    double cmin = R > 0 ? R + 2 * delta : 0;
    skin_report = std::max(skin_report, 2 * delta);
    range_report = std::max(range_report, R);
    // with no pair work the displacement check is off
    sd.delta = R > 0 ? (float)delta : 1e30f;
    // Verlet-list radius: a pair within range at some step of a rebuild period
    // was within range + 2 delta at its start (plus float margin)
    if (R > 0) {
      const double rr = std::sqrt((double)std::max(R2, Rrx2)) + 2.0 * delta;
      const double rl = rr * (1.0 + 1e-6) + 8.0 * max_unit;
      sd.Rl2 = (float)(rl * rl);
      double vol = 1.0, ball = D == 1 ? 2.0 * rl : (D == 2 ? M_PI * rl * rl : 4.0 / 3.0 * M_PI * rl * rl * rl);
      for (int k = 0; k < D; k++) vol *= S.L[k];
      const double expect = std::min((double)S.n_particles, S.n_particles / vol * ball);
      list_expect = std::max(list_expect, expect);
      // the prefilter pays when few draws can succeed
      for (int t = 0; t < MAXT; t++)
        if (S.dt * (sd.rxA[t] + sd.rxB[t] * expect) > 0.02) rx_pre_worth = false;
    }
    // cells
    int ncs = 1;
    for (int k = 0; k < D; k++) {
      int nc;
      if (cmin <= 0) nc = std::max(1, (int)std::min(64.0, S.L[k]));
      else nc = (int)std::floor(S.L[k] / cmin);
      if (nc < 1) nc = 1;
      if ((sd.periodic >> k) & 1) {
        if (nc < 3) nc = 1;
      }
      nc = std::min(nc, 1 << 16);
      sd.nc[k] = nc;
      sd.halo[k] = (((sd.periodic >> k) & 1) && nc == 1) ? 0 : 1;
      if (nc == 1 && !((sd.periodic >> k) & 1)) sd.halo[k] = 0;
      ncs *= nc;
      cell_report = std::min(cell_report, S.L[k] / nc);
    }
    sd.c0 = total_cells;
    total_cells += ncs;
    if (total_cells < 0 || total_cells > (1 << 28)) return bail(fail(RDSIM_ERR_UNSUPPORTED, "too many cells"));
    // bonded templates
    std::map<int, int> tmpl_index;  // molecule_id -> device template
    std::vector<int> tmpl_of_mol(S.n_molecules, 0xff);
    for (int m = 0; m < S.n_molecules; m++) {
      int j = S.first_index_of_molecule[m];
      if (j < 0 || j >= S.n_particles) return bail(fail(RDSIM_ERR_ARG, "first_index_of_molecule out of range"));
      int mid = S.molecule_ids[3 * j + 2];
      int tq = -1;
      for (int q = 0; q < S.n_templates; q++)
        if (S.templates[q].molecule_id == mid) tq = q;
      if (tq < 0) return bail(fail(RDSIM_ERR_ARG, "molecule id " + std::to_string(mid) + " has no definition"));
      const rdsim_template& T = S.templates[tq];
      if (T.n_terms == 0) continue;
      auto it = tmpl_index.find(mid);
      if (it == tmpl_index.end()) {
        TmplDev td;
        std::memset(&td, 0, sizeof td);
        int maxatom = 0;
        for (int e = 0; e < T.n_terms; e++) {
          const rdsim_term& tr = S.terms[T.first_term + e];
          maxatom = std::max(maxatom, std::max(tr.i, tr.j));
          if (tr.kind == RDSIM_TERM_ANGLE) maxatom = std::max(maxatom, tr.k);
          if (tr.i < 0 || tr.j < 0 || (tr.kind == RDSIM_TERM_ANGLE && tr.k < 0))
            return bail(fail(RDSIM_ERR_ARG, "negative atom index in bonded term"));
        }
        if (maxatom >= MAXA) return bail(fail(RDSIM_ERR_UNSUPPORTED, "molecules with bonded terms are limited to 32 atoms"));
        td.n_atoms = maxatom + 1;
        td.n_terms = T.n_terms;
        td.term0 = (int)terms.size();
        std::vector<std::vector<int>> per_atom(td.n_atoms);
        for (int e = 0; e < T.n_terms; e++) {
          const rdsim_term& tr = S.terms[T.first_term + e];
          TermDev d;
          std::memset(&d, 0, sizeof d);
          d.kind = tr.kind;
          d.i = tr.i;
          d.j = tr.j;
          d.k = tr.k;
          d.p0 = (float)tr.p0;
          d.k0 = (float)tr.k0;
          d.thr = (float)(tr.p0 - 0.1);
          d.pi = std::fabs(tr.p0 - M_PI) <= 1e-5 + 1e-5 * M_PI ? 1.f : -1.f;  // np.isclose
          if (tr.kind == RDSIM_TERM_BOND && sd.bond128) {
            // r0^2 in units of unit^2 as a 128-bit integer: (r0 / unit)
            // rounded to an integer, squared exactly (its rounding moves
            // r0 by under one fixed unit)
            const double v = std::min(std::fabs(tr.p0) / sd.unit_d[0], 1.8e19);
            if (!(v < 9.2e18)) sd.bond128 = 0;  // a rest length beyond the box
            const unsigned __int128 r = (unsigned __int128)(unsigned long long)std::llround(std::min(v, 9.2e18));
            const unsigned __int128 r2 = v < 9.2e18 ? r * r : ~(unsigned __int128)0;
            d.r0q_lo = (unsigned long long)r2;
            d.r0q_hi = (unsigned long long)(r2 >> 64);
          }
          int ti = (int)terms.size();
          terms.push_back(d);
          oterms.push_back(tr);
          per_atom[tr.i].push_back(ti * 4 + 0);
          per_atom[tr.j].push_back(ti * 4 + 1);
          td.bondmask[tr.i] |= 1u << tr.j;
          td.bondmask[tr.j] |= 1u << tr.i;
          if (tr.kind == RDSIM_TERM_ANGLE) {
            per_atom[tr.k].push_back(ti * 4 + 2);
            td.bondmask[tr.j] |= 1u << tr.k;
            td.bondmask[tr.k] |= 1u << tr.j;
          }
        }
        // CSR: atomterm[atom0 + a] .. atomterm[atom0 + a + 1] index the entry list
        td.atom0 = (int)atomterm.size();
        atomterm.resize(atomterm.size() + td.n_atoms + 1);
        for (int a = 0; a <= td.n_atoms; a++) atomterm[td.atom0 + a] = 0;
        int idx = (int)tmpls.size();
        tmpls.push_back(td);
        tmpl_index[mid] = idx;
        // entries appended after the offsets; offsets are absolute
        TmplDev& tt = tmpls.back();
        for (int a = 0; a < tt.n_atoms; a++) {
          atomterm[tt.atom0 + a] = (int)atomterm.size();
          for (int v : per_atom[a]) atomterm.push_back(v);
        }
        atomterm[tt.atom0 + tt.n_atoms] = (int)atomterm.size();
        if ((int)tmpls.size() > 0xfe) return bail(fail(RDSIM_ERR_UNSUPPORTED, "too many molecule templates"));
        it = tmpl_index.find(mid);
      }
      tmpl_of_mol[m] = it->second;
      sd.has_terms = 1;
    }
    // static per-particle metadata (caller order)
    std::vector<int> mol_range_start(S.n_particles, -1), mol_of(S.n_particles, -1);
    for (int m = 0; m < S.n_molecules; m++) {
      int b = S.first_index_of_molecule[m];
      int e = (m + 1 < S.n_molecules) ? S.first_index_of_molecule[m + 1] : S.n_particles;
      for (int i = b; i < e && i < S.n_particles; i++) {
        mol_range_start[i] = b;
        mol_of[i] = m;
      }
    }
    for (int i = 0; i < S.n_particles; i++) {
      uint32_t ms = 0xffu << 24;
      int m = mol_of[i];
      if (m >= 0 && tmpl_of_mol[m] != 0xff) {
        int loc = i - mol_range_start[i];
        const TmplDev& td = tmpls[tmpl_of_mol[m]];
        int msize = ((m + 1 < S.n_molecules) ? S.first_index_of_molecule[m + 1] : S.n_particles) - mol_range_start[i];
        if (td.n_atoms > msize)
          return bail(fail(RDSIM_ERR_UNSUPPORTED, "bonded term references an atom beyond its molecule"));
        if (loc < td.n_atoms) ms = ((uint32_t)tmpl_of_mol[m] << 24) | ((uint32_t)loc << 16);
      }
      h->meta_static.push_back(ms);
      h->mol_h.push_back(S.molecule_ids[3 * i]);
      x_all.insert(x_all.end(), S.x + (size_t)i * D, S.x + (size_t)(i + 1) * D);
      t_all.push_back(S.particle_types[i]);
      sid_h.push_back(si);
    }
    // molecule labels must identify molecules for the same-molecule tests
    {
      std::map<int, int> label_mol;
      for (int i = 0; i < S.n_particles; i++) {
        if (mol_of[i] < 0) continue;
        auto it = label_mol.find(S.molecule_ids[3 * i]);
        if (it == label_mol.end()) label_mol[S.molecule_ids[3 * i]] = mol_of[i];
        else if (it->second != mol_of[i] && tmpl_of_mol[mol_of[i]] != 0xff)
          return bail(fail(RDSIM_ERR_UNSUPPORTED, "molecule numbers (column 0) must differ between bonded molecules"));
      }
    }
    h->N += S.n_particles;
    h->sys_h.push_back(sd);
    h->hs.push_back(hsys);
  }
  h->skin = skin_report;
  h->cell_min = cell_report;
  h->range = range_report;
  h->ncells = total_cells;
  h->nscan = std::max(1, (total_cells + SCAN_TILE - 1) / SCAN_TILE);
  if (opt.reaction_prefilter < 0 || (opt.reaction_prefilter == 0 && !rx_pre_worth)) h->rx_pre = false;
  // list kernels: CTA chunks per system; list width from the expected
  // population (rows beyond it are regenerated from the cells)
  {
    const int per = LBLOCK / h->ltpp;
    for (int si = 0; si < (int)h->sys_h.size(); si++) {
      const SysDev& sd = h->sys_h[si];
      for (int b = 0; b < sd.n; b += per) {
        Chunk c;
        std::memset(&c, 0, sizeof c);
        c.sys = si;
        c.beg = sd.p0 + b;
        c.cnt = std::min(per, sd.n - b);
        c.law0 = sd.law0;
        c.nlaws = sd.nlaws;
        c.wall0 = sd.wall0;
        c.nwalls = sd.nwalls;
        c.rx0 = sd.rx0;
        c.nrx = sd.nrx;
        h->chunks_h.push_back(c);
      }
    }
    int W = (int)std::ceil(2.0 * list_expect + 16.0);
    W = std::max(16, std::min(W, 2048));
    h->npad = (h->N + 31) / 32 * 32;
    const double limit = (double)(1 << 30);  // entries (32-bit list indices)
    while (W > 16 && (double)W * h->npad > limit) W /= 2;
    if (opt.list_width > 0) W = std::min(opt.list_width, 2048);
    h->W = (W + 7) / 8 * 8;
    if ((double)h->W * h->npad > limit)
      return bail(fail(RDSIM_ERR_UNSUPPORTED, "too many particles for the list kernels"));
  }
  // device memory
  int64_t& B = h->device_bytes;
  const int N = h->N;
  if ((rc = dalloc(&h->sys_d, h->sys_h.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->laws_d, laws.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->walls_d, walls.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->rx_d, rxs.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->tmpl_d, tmpls.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->terms_d, terms.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->atomterm_d, atomterm.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->olaws_d, olaws.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->owalls_d, owalls.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->oterms_d, oterms.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->cell_count, (size_t)h->ncells, &B))) return bail(rc);
  // zero once; every rebuild leaves them zero for the next (k_scatter)
  if (cudaMemsetAsync(h->cell_count, 0, sizeof(int) * (size_t)h->ncells, h->stream) != cudaSuccess)
    return bail(fail(RDSIM_ERR_CUDA, "memset"));
  if ((rc = dalloc(&h->cell_start, (size_t)h->ncells + 1, &B))) return bail(rc);
  if ((rc = dalloc(&h->bsum, (size_t)h->nscan, &B))) return bail(rc);
  if ((rc = dalloc(&h->cell_of, N, &B))) return bail(rc);
  if ((rc = dalloc(&h->rank_of, N, &B))) return bail(rc);
  if ((rc = dalloc(&h->tmp, N, &B))) return bail(rc);
  if ((rc = dalloc(&h->sid, N, &B))) return bail(rc);
  if ((rc = dalloc(&h->slot_of, N, &B))) return bail(rc);
  for (int b = 0; b < 2; b++) {
    for (int k = 0; k < D; k++) {
      if ((rc = dalloc(&h->xh[b][k], N, &B))) return bail(rc);
      if ((rc = dalloc(&h->xl[b][k], N, &B))) return bail(rc);
      if ((rc = dalloc(&h->xp[b][k], N, &B))) return bail(rc);
    }
    if ((rc = dalloc(&h->meta[b], N, &B))) return bail(rc);
    if ((rc = dalloc(&h->mol[b], N, &B))) return bail(rc);
    if ((rc = dalloc(&h->pid[b], N, &B))) return bail(rc);
  }
  for (int k = 0; k < D; k++) {
    if ((rc = dalloc(&h->xr[k], N, &B))) return bail(rc);
    if ((rc = dalloc(&h->drift[k], N, &B))) return bail(rc);
    if (h->f64 && (rc = dalloc(&h->drift_d[k], N, &B))) return bail(rc);
  }
  if ((rc = dalloc(&h->typed_d, typed.size(), &B))) return bail(rc);
  if ((rc = dalloc(&h->rates, N, &B))) return bail(rc);
  if ((rc = dalloc(&h->xbuf, (size_t)N * D, &B))) return bail(rc);
  if ((rc = dalloc(&h->tbuf, N, &B))) return bail(rc);
  if ((rc = dalloc(&h->meta_static_d, N, &B))) return bail(rc);
  if ((rc = dalloc(&h->mol_static_d, N, &B))) return bail(rc);
  if ((rc = dalloc(&h->flag_d, 1, &B))) return bail(rc);
  if ((rc = dalloc(&h->err, 1, &B))) return bail(rc);
  if ((rc = dalloc(&h->step_dev, 1, &B))) return bail(rc);
  {
    if ((rc = dalloc(&h->chunks_d, h->chunks_h.size(), &B))) return bail(rc);
    if ((rc = dalloc(&h->nbr, (size_t)h->W * h->npad, &B))) return bail(rc);
    if ((rc = dalloc(&h->ncnt, N, &B))) return bail(rc);
    if ((rc = dalloc(&h->rx_list, 3 * (size_t)h->npad, &B))) return bail(rc);
    if ((rc = dalloc(&h->rx_count, 3, &B))) return bail(rc);
    if (cudaMemsetAsync(h->rx_count, 0, 3 * sizeof(int), h->stream) != cudaSuccess)
      return bail(fail(RDSIM_ERR_CUDA, "memset"));
  }
  h->graphs = opt.use_graphs >= 0;
  // period kernel: float32 forces, every chunk resident at once (its CTAs
  // wait for each other) and within the neighbour-chunk bitmap
  if (opt.sync_wait_ms > 0) h->wait_ns = (long long)opt.sync_wait_ms * 1000000LL;
  {
    const int nch = (int)h->chunks_h.size();
    if (opt.period_kernel >= 0 && !h->f64 && nch <= PMAX_CHUNKS && nch <= period_capacity(h)) {
      if ((rc = dalloc(&h->nbmask, (size_t)nch * PMASK_WORDS, &B))) return bail(rc);
      if ((rc = dalloc(&h->cand0, (size_t)nch * CAND_WORDS, &B))) return bail(rc);
      if ((rc = dalloc(&h->pflag, (size_t)nch * PFLAG_STRIDE, &B))) return bail(rc);
      h->period_on = true;
    }
  }
  if ((rc = dalloc(&h->cl_d, (size_t)3 * h->nsys, &B))) return bail(rc);
  auto up = [&](void* d, const void* s, size_t bytes) -> int {
    if (bytes == 0) return 0;
    CK(cudaMemcpyAsync(d, s, bytes, cudaMemcpyHostToDevice, h->stream));
    return 0;
  };
  std::vector<double> cl(3 * h->nsys, 1.0);
  for (int s = 0; s < h->nsys; s++)
    for (int k = 0; k < D; k++) cl[3 * s + k] = h->hs[s].cl_ref[k];
  if ((rc = up(h->sys_d, h->sys_h.data(), sizeof(SysDev) * h->sys_h.size()))) return bail(rc);
  if ((rc = up(h->chunks_d, h->chunks_h.data(), sizeof(Chunk) * h->chunks_h.size())))
    return bail(rc);
  if ((rc = up(h->laws_d, laws.data(), sizeof(PairLaw) * laws.size()))) return bail(rc);
  if ((rc = up(h->walls_d, walls.data(), sizeof(WallLaw) * walls.size()))) return bail(rc);
  if ((rc = up(h->rx_d, rxs.data(), sizeof(RxDev) * rxs.size()))) return bail(rc);
  if ((rc = up(h->tmpl_d, tmpls.data(), sizeof(TmplDev) * tmpls.size()))) return bail(rc);
  if ((rc = up(h->terms_d, terms.data(), sizeof(TermDev) * terms.size()))) return bail(rc);
  if ((rc = up(h->atomterm_d, atomterm.data(), sizeof(int) * atomterm.size()))) return bail(rc);
  if ((rc = up(h->olaws_d, olaws.data(), sizeof(rdsim_interaction) * olaws.size()))) return bail(rc);
  if ((rc = up(h->owalls_d, owalls.data(), sizeof(rdsim_interaction) * owalls.size()))) return bail(rc);
  if ((rc = up(h->oterms_d, oterms.data(), sizeof(rdsim_term) * oterms.size()))) return bail(rc);
  if ((rc = up(h->sid, sid_h.data(), sizeof(int) * sid_h.size()))) return bail(rc);
  if ((rc = up(h->cl_d, cl.data(), sizeof(double) * cl.size()))) return bail(rc);
  if ((rc = up(h->typed_d, typed.data(), sizeof(double) * typed.size()))) return bail(rc);
  if (cudaMemsetAsync(h->err, 0, sizeof(ErrDev), h->stream) != cudaSuccess)
    return bail(fail(RDSIM_ERR_CUDA, "memset"));
  for (int k = 0; k < D; k++) {
    if (cudaMemsetAsync(h->drift[k], 0, sizeof(float) * N, h->stream) != cudaSuccess)
      return bail(fail(RDSIM_ERR_CUDA, "memset"));
    if (h->f64 && cudaMemsetAsync(h->drift_d[k], 0, sizeof(double) * N, h->stream) != cudaSuccess)
      return bail(fail(RDSIM_ERR_CUDA, "memset"));
  }
  if ((rc = up(h->meta_static_d, h->meta_static.data(), sizeof(uint32_t) * (size_t)N))) return bail(rc);
  if ((rc = up(h->mol_static_d, h->mol_h.data(), sizeof(int) * (size_t)N))) return bail(rc);
  if ((rc = up(h->xbuf, x_all.data(), sizeof(double) * x_all.size()))) return bail(rc);
  if ((rc = up(h->tbuf, t_all.data(), sizeof(int) * t_all.size()))) return bail(rc);
  if ((rc = upload_state(h))) return bail(rc);
  if ((rc = initial_drift(h))) return bail(rc);
  *out = h;
  return 0;
}

int rdsim_destroy(rdsim_handle* h) {
  if (!h) return 0;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
  return 0;
}

int rdsim_step(rdsim_handle* h, int32_t n_steps, int32_t flags, const double* xi,
               const double* u1, const double* u2) {
  if (!h) return fail(RDSIM_ERR_ARG, "null handle");
  if (n_steps <= 0) return 0;
  CK(cudaSetDevice(h->device));
  const int N = h->N, D = h->D;
  int kf = 0;
  if (flags & RDSIM_STEP_NO_NOISE) kf |= F_NO_NOISE;
  const bool inj = (flags & (RDSIM_STEP_INJECT_HOST | RDSIM_STEP_INJECT_DEVICE)) != 0;
  const double *dxi = nullptr, *du1 = nullptr, *du2 = nullptr;
  if (inj) {
    kf |= F_INJECT;
    if (flags & RDSIM_STEP_INJECT_HOST) {
      if ((size_t)n_steps > h->inj_steps) {
        if (h->inj_xi) cudaFree(h->inj_xi);
        if (h->inj_u1) cudaFree(h->inj_u1);
        if (h->inj_u2) cudaFree(h->inj_u2);
        h->inj_xi = h->inj_u1 = h->inj_u2 = nullptr;
        int64_t dummy = 0;
        int rc;
        if ((rc = dalloc(&h->inj_xi, (size_t)n_steps * N * D, &dummy))) return rc;
        if ((rc = dalloc(&h->inj_u1, (size_t)n_steps * N, &dummy))) return rc;
        if ((rc = dalloc(&h->inj_u2, (size_t)n_steps * N, &dummy))) return rc;
        h->inj_steps = n_steps;
      }
      if (xi) CK(cudaMemcpyAsync(h->inj_xi, xi, sizeof(double) * n_steps * N * D, cudaMemcpyHostToDevice, h->stream));
      else CK(cudaMemsetAsync(h->inj_xi, 0, sizeof(double) * n_steps * N * D, h->stream));
      if (u1) CK(cudaMemcpyAsync(h->inj_u1, u1, sizeof(double) * n_steps * N, cudaMemcpyHostToDevice, h->stream));
      else CK(cudaMemsetAsync(h->inj_u1, 0x7f, sizeof(double) * n_steps * N, h->stream));
      if (u2) CK(cudaMemcpyAsync(h->inj_u2, u2, sizeof(double) * n_steps * N, cudaMemcpyHostToDevice, h->stream));
      else CK(cudaMemsetAsync(h->inj_u2, 0x7f, sizeof(double) * n_steps * N, h->stream));
      dxi = h->inj_xi;
      du1 = h->inj_u1;
      du2 = h->inj_u2;
    } else {
      dxi = xi;
      du1 = u1;
      du2 = u2;
      if (!xi && !(flags & RDSIM_STEP_NO_NOISE)) return fail(RDSIM_ERR_ARG, "injected noise missing");
      if (h->has_rx && (!u1 || !u2)) return fail(RDSIM_ERR_ARG, "injected uniforms missing");
    }
  }
  int rc;
  // first step: the stand-alone update with the drift left by the last call
  if ((rc = em(h, h->step + 1, kf, dxi))) return rc;
  const bool graphable = h->graphs && !inj && !h->prof;
  // reaction prefilter: needs the counter-based draws (not injected ones)
  const bool pre = h->rx_pre && h->has_rx && !inj;
  bool flagged = false;  // the last drift kernel flagged this step's draws
  for (int q = 0; q < n_steps;) {
    const long long s = h->step + 1;
    const int left = n_steps - q;
    if (graphable && s % h->freq == 0 && left > h->freq && !snapshot_in(h, s, s + h->freq - 1)) {
      if ((rc = run_period_graph(h, s, kf, pre))) return rc;
      h->step = s + h->freq - 1;
      q += h->freq;
      flagged = false;
      continue;
    }
    // a call that starts inside a list period: the step's reactions on the
    // reaction kernels, then the rest of the period in one period-kernel
    // launch (not when a trajectory frame or the call's last step falls in it)
    const long long e = (s / h->freq + 1) * h->freq - 1;
    const int m = (int)(e - s + 1);
    if (graphable && h->period_on && (pre || !h->has_rx) && s % h->freq != 0 && left > m &&
        !snapshot_in(h, s, e)) {
      if (h->has_rx &&
          (rc = react(h, s, kf, nullptr, nullptr, false, flagged)))
        return rc;
      if ((rc = period_launch(h, kf, pre, false, s, m))) return rc;
      h->cx ^= m & 1;
      if (h->has_rx) h->cm ^= (m - 1) & 1;
      h->step = e;
      q += m;
      flagged = false;
      continue;
    }
    if (s % h->freq == 0) {
      if ((rc = rebuild(h, s, pre, false, h->period_on))) return rc;
      flagged = pre;  // the builder listed this step's candidates
    }
    if (h->has_rx) {
      if ((rc = react(h, s, kf, du1 ? du1 + (size_t)q * N : nullptr,
                      du2 ? du2 + (size_t)q * N : nullptr, false, flagged)))
        return rc;
    }
    if (h->traj_frames > 0 && s % h->traj_stride == 0) {
      long long m = (s / h->traj_stride - 1) % h->traj_frames;
      if ((rc = snapshot(h, h->traj_x + (size_t)m * N * D, h->traj_t + (size_t)m * N))) return rc;
    }
    const bool last = q == n_steps - 1;
    const double* xn = (dxi && !last) ? dxi + (size_t)(q + 1) * N * D : nullptr;
    flagged = pre && !last && (s + 1) % h->freq != 0;
    if ((rc = force(h, s, (last ? F_STORE_DRIFT : F_EM) | kf | (flagged ? F_RX_NEXT : 0), xn)))
      return rc;
    h->step = s;
    q++;
  }
  return check_device_error(h);
}

int rdsim_set_state(rdsim_handle* h, const double* x, const int32_t* types) {
  if (!h) return fail(RDSIM_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  const int N = h->N, D = h->D;
  if (!x || !types) {
    // the part not given: the current state, in caller order, on the device
    Args a = make_args(h);
    const unsigned g = nblk(N);
    if (D == 2) k_to_double<2><<<g, 256, 0, h->stream>>>(h->sys_d, h->sid, a, h->xbuf, h->tbuf);
    else if (D == 3) k_to_double<3><<<g, 256, 0, h->stream>>>(h->sys_d, h->sid, a, h->xbuf, h->tbuf);
    else k_to_double<1><<<g, 256, 0, h->stream>>>(h->sys_d, h->sid, a, h->xbuf, h->tbuf);
    CK(cudaGetLastError());
  }
  if (x) CK(cudaMemcpyAsync(h->xbuf, x, sizeof(double) * (size_t)N * D, cudaMemcpyHostToDevice, h->stream));
  if (types) CK(cudaMemcpyAsync(h->tbuf, types, sizeof(int) * (size_t)N, cudaMemcpyHostToDevice, h->stream));
  int rc = upload_state(h);
  if (rc) return rc;
  return initial_drift(h);
}

int rdsim_get_state(rdsim_handle* h, double* x, int32_t* types) {
  if (!h) return fail(RDSIM_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  Args a = make_args(h);
  unsigned g = nblk(h->N);
  if (h->D == 2) k_to_double<2><<<g, 256, 0, h->stream>>>(h->sys_d, h->sid, a, h->xbuf, h->tbuf);
  else if (h->D == 3) k_to_double<3><<<g, 256, 0, h->stream>>>(h->sys_d, h->sid, a, h->xbuf, h->tbuf);
  else k_to_double<1><<<g, 256, 0, h->stream>>>(h->sys_d, h->sid, a, h->xbuf, h->tbuf);
  CK(cudaGetLastError());
  if (x) CK(cudaMemcpyAsync(x, h->xbuf, sizeof(double) * (size_t)h->N * h->D, cudaMemcpyDeviceToHost, h->stream));
  if (types) CK(cudaMemcpyAsync(types, h->tbuf, sizeof(int) * (size_t)h->N, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int rdsim_get_drift(rdsim_handle* h, double* a) {
  if (!h || !a) return fail(RDSIM_ERR_ARG, "null argument");
  CK(cudaSetDevice(h->device));
  const int N = h->N, D = h->D;
  std::vector<float> d[3];
  std::vector<double> dd[3];
  std::vector<int> pid(N);
  for (int k = 0; k < D; k++) {
    if (h->f64) {
      dd[k].resize(N);
      CK(cudaMemcpyAsync(dd[k].data(), h->drift_d[k], 8 * (size_t)N, cudaMemcpyDeviceToHost, h->stream));
    } else {
      d[k].resize(N);
      CK(cudaMemcpyAsync(d[k].data(), h->drift[k], 4 * (size_t)N, cudaMemcpyDeviceToHost, h->stream));
    }
  }
  CK(cudaMemcpyAsync(pid.data(), h->pid[h->co], 4 * (size_t)N, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int i = 0; i < N; i++)
    for (int k = 0; k < D; k++)
      a[(size_t)pid[i] * D + k] = h->f64 ? dd[k][i] : (double)d[k][i];
  return 0;
}

int rdsim_get_reaction_rates(rdsim_handle* h, double* total) {
  if (!h || !total) return fail(RDSIM_ERR_ARG, "null argument");
  CK(cudaSetDevice(h->device));
  CK(cudaMemsetAsync(h->rates, 0, sizeof(double) * h->N, h->stream));
  if (h->has_rx) {
    int rc = react(h, h->step, F_RATES_ONLY, nullptr, nullptr);
    if (rc) return rc;
  }
  CK(cudaMemcpyAsync(total, h->rates, sizeof(double) * h->N, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int rdsim_get_pairs(rdsim_handle* h, int32_t sys, int32_t* pairs, int64_t cap, int64_t* n_pairs) {
  if (!h || sys < 0 || sys >= h->nsys || !n_pairs) return fail(RDSIM_ERR_ARG, "bad argument");
  CK(cudaSetDevice(h->device));
  const HostSys& q = h->hs[sys];
  const SysDev& sd = h->sys_h[sys];
  unsigned long long* cnt = nullptr;
  int* buf = nullptr;
  size_t bcap = (size_t)std::max<int64_t>(cap, 1);
  if (cudaMalloc(&cnt, sizeof(unsigned long long)) != cudaSuccess) {
    cudaGetLastError();
    return fail(RDSIM_ERR_NOMEM, "pair counter");
  }
  if (cudaMalloc(&buf, sizeof(int) * 2 * bcap) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(cnt);
    return fail(RDSIM_ERR_NOMEM, "pair buffer");
  }
  cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), h->stream);
  double maxu = 0;
  for (int k = 0; k < h->D; k++) maxu = std::max(maxu, (double)sd.unit_hi[k]);
  float rs2_hi = (float)(q.rs * q.rs) + guard2(q.rs, maxu);
  Args a = make_args(h);
  unsigned g = nblk(q.n);
  if (h->D == 2) k_pairs<2><<<g, 256, 0, h->stream>>>(h->sys_d, sys, a, h->tmpl_d, q.rs, rs2_hi, q.p0, q.n, q.pid0, buf, (unsigned long long)cap, cnt);
  else if (h->D == 3) k_pairs<3><<<g, 256, 0, h->stream>>>(h->sys_d, sys, a, h->tmpl_d, q.rs, rs2_hi, q.p0, q.n, q.pid0, buf, (unsigned long long)cap, cnt);
  else k_pairs<1><<<g, 256, 0, h->stream>>>(h->sys_d, sys, a, h->tmpl_d, q.rs, rs2_hi, q.p0, q.n, q.pid0, buf, (unsigned long long)cap, cnt);
  unsigned long long n = 0;
  cudaError_t e1 = cudaGetLastError();
  cudaMemcpyAsync(&n, cnt, sizeof n, cudaMemcpyDeviceToHost, h->stream);
  cudaStreamSynchronize(h->stream);
  *n_pairs = (int64_t)n;
  int rc = 0;
  if (e1 != cudaSuccess) rc = fail(RDSIM_ERR_CUDA, cudaGetErrorString(e1));
  else if ((int64_t)n > cap) rc = fail(RDSIM_ERR_CAPACITY, "pair buffer too small");
  else if (n > 0 && pairs) {
    std::vector<int> tmp(2 * n);
    cudaMemcpy(tmp.data(), buf, sizeof(int) * 2 * n, cudaMemcpyDeviceToHost);
    std::vector<std::pair<int, int>> v(n);
    for (size_t p = 0; p < n; p++) v[p] = {tmp[2 * p], tmp[2 * p + 1]};
    std::sort(v.begin(), v.end());
    for (size_t p = 0; p < n; p++) {
      pairs[2 * p] = v[p].first;
      pairs[2 * p + 1] = v[p].second;
    }
  }
  cudaFree(cnt);
  cudaFree(buf);
  return rc;
}

int rdsim_get_cell_ids(rdsim_handle* h, int32_t sys, int32_t* cell_ids) {
  if (!h || sys < 0 || sys >= h->nsys || !cell_ids) return fail(RDSIM_ERR_ARG, "bad argument");
  CK(cudaSetDevice(h->device));
  const HostSys& q = h->hs[sys];
  int* buf = nullptr;
  CK(cudaMalloc(&buf, sizeof(int) * (size_t)q.n * h->D));
  Args a = make_args(h);
  unsigned g = nblk(q.n);
  const double* cl = h->cl_d + 3 * sys;
  if (h->D == 2) k_ref_cells<2><<<g, 256, 0, h->stream>>>(h->sys_d, sys, a, cl, q.p0, q.n, q.pid0, buf);
  else if (h->D == 3) k_ref_cells<3><<<g, 256, 0, h->stream>>>(h->sys_d, sys, a, cl, q.p0, q.n, q.pid0, buf);
  else k_ref_cells<1><<<g, 256, 0, h->stream>>>(h->sys_d, sys, a, cl, q.p0, q.n, q.pid0, buf);
  cudaError_t e1 = cudaGetLastError();
  cudaMemcpyAsync(cell_ids, buf, sizeof(int) * (size_t)q.n * h->D, cudaMemcpyDeviceToHost, h->stream);
  cudaStreamSynchronize(h->stream);
  cudaFree(buf);
  if (e1 != cudaSuccess) return fail(RDSIM_ERR_CUDA, cudaGetErrorString(e1));
  return 0;
}

int rdsim_get_observables(rdsim_handle* h, int32_t sys, rdsim_observables* out) {
  if (!h || !out || sys < 0 || sys >= h->nsys) return fail(RDSIM_ERR_ARG, "bad argument");
  CK(cudaSetDevice(h->device));
  const HostSys& q = h->hs[sys];
  const int nb = std::max(1, (q.n + OBS_BLOCK - 1) / OBS_BLOCK);
  if (nb > h->obs_cap) {
    if (h->obs_part) cudaFree(h->obs_part);
    h->obs_part = nullptr;
    h->obs_cap = 0;
    if (cudaMalloc(&h->obs_part, sizeof(double) * ((size_t)nb + 1) * OBS_NSUM) != cudaSuccess) {
      cudaGetLastError();
      return fail(RDSIM_ERR_NOMEM, "observables scratch");
    }
    h->obs_cap = nb;
  }
  if (!h->obs_counts && cudaMalloc(&h->obs_counts, sizeof(unsigned long long) * (1 + MAXT)) != cudaSuccess) {
    cudaGetLastError();
    return fail(RDSIM_ERR_NOMEM, "observables scratch");
  }
  ObsArgs o;
  std::memset(&o, 0, sizeof o);
  o.laws = h->olaws_d;
  o.walls = h->owalls_d;
  o.terms = h->oterms_d;
  o.part = h->obs_part;
  o.sums = h->obs_part + (size_t)nb * OBS_NSUM;
  o.counts = h->obs_counts;
  o.sys = sys;
  o.tpp = h->ltpp;
  o.nblocks = nb;
  CK(cudaMemsetAsync(h->obs_counts, 0, sizeof(unsigned long long) * (1 + MAXT), h->stream));
  Args a = make_args(h);
  {
    ProfScope ps(h, 4, 2);
    if (h->D == 2) k_observe<2><<<nb, OBS_BLOCK, 0, h->stream>>>(a, o);
    else if (h->D == 3) k_observe<3><<<nb, OBS_BLOCK, 0, h->stream>>>(a, o);
    else k_observe<1><<<nb, OBS_BLOCK, 0, h->stream>>>(a, o);
    k_observe_sum<<<1, OBS_BLOCK, 0, h->stream>>>(o);
  }
  CK(cudaGetLastError());
  double sums[OBS_NSUM];
  unsigned long long counts[1 + MAXT];
  CK(cudaMemcpyAsync(sums, o.sums, sizeof sums, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(counts, h->obs_counts, sizeof counts, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  std::memset(out, 0, sizeof *out);
  out->pair_energy = sums[0];
  out->wall_energy = sums[1];
  out->bond_energy = sums[2];
  out->angle_energy = sums[3];
  out->virial = sums[4];
  out->min_distance = sums[5];
  out->n_pairs = (int64_t)counts[0];
  out->n_particles = q.n;
  for (int t = 0; t < MAXT; t++) out->type_counts[t] = (int64_t)counts[1 + t];
  return 0;
}

int rdsim_get_rdf(rdsim_handle* h, int32_t sys, int32_t type_a, int32_t type_b, double r_max,
                  int32_t n_bins, int32_t flags, int64_t* counts) {
  if (!h || !counts || sys < 0 || sys >= h->nsys) return fail(RDSIM_ERR_ARG, "bad argument");
  if (n_bins < 1 || n_bins > RDF_MAX_BINS) return fail(RDSIM_ERR_ARG, "n_bins must be in [1, 8192]");
  if (!(r_max > 0) || !std::isfinite(r_max)) return fail(RDSIM_ERR_ARG, "r_max must be positive");
  if (type_a >= MAXT || type_b >= MAXT) return fail(RDSIM_ERR_ARG, "type out of range");
  const HostSys& q = h->hs[sys];
  const SysDev& sd = h->sys_h[sys];
  RdfArgs o;
  std::memset(&o, 0, sizeof o);
  double maxu = 0;
  for (int k = 0; k < h->D; k++) {
    if (((sd.periodic >> k) & 1) && r_max > 0.5 * q.L[k])
      return fail(RDSIM_ERR_ARG, "r_max exceeds half of a periodic box length");
    maxu = std::max(maxu, (double)sd.unit_hi[k]);
    // pairs closer than r_max now were within r_max + 2 delta at the rebuild
    const double cell = q.L[k] / sd.nc[k];
    const double reach = r_max + 2.0 * (double)sd.delta * 1.01 + 8.0 * maxu;
    o.h[k] = (int)std::min<double>(sd.nc[k], std::floor(reach / cell) + 1.0);
  }
  CK(cudaSetDevice(h->device));
  if (!h->rdf_counts && cudaMalloc(&h->rdf_counts, sizeof(unsigned long long) * RDF_MAX_BINS) != cudaSuccess) {
    cudaGetLastError();
    return fail(RDSIM_ERR_NOMEM, "histogram scratch");
  }
  o.counts = h->rdf_counts;
  o.r_max = r_max;
  o.width = r_max / n_bins;
  o.r2_hi = (float)(r_max * r_max) + guard2(r_max, maxu);
  o.sys = sys;
  o.type_a = type_a;
  o.type_b = type_b;
  o.nbins = n_bins;
  o.flags = flags;
  CK(cudaMemsetAsync(h->rdf_counts, 0, sizeof(unsigned long long) * n_bins, h->stream));
  Args a = make_args(h);
  const unsigned nb = (unsigned)std::max(1, (q.n + OBS_BLOCK - 1) / OBS_BLOCK);
  {
    ProfScope ps(h, 4, 1);
    if (h->D == 2) k_rdf<2><<<nb, OBS_BLOCK, 0, h->stream>>>(a, o);
    else if (h->D == 3) k_rdf<3><<<nb, OBS_BLOCK, 0, h->stream>>>(a, o);
    else k_rdf<1><<<nb, OBS_BLOCK, 0, h->stream>>>(a, o);
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(counts, h->rdf_counts, sizeof(int64_t) * n_bins, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int rdsim_get_step(rdsim_handle* h, int64_t* step) {
  if (!h || !step) return fail(RDSIM_ERR_ARG, "null argument");
  *step = h->step;
  return 0;
}

int rdsim_set_step(rdsim_handle* h, int64_t step) {
  if (!h) return fail(RDSIM_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  h->step = step;
  // candidate-list slots follow the step number: start them empty
  CK(cudaMemsetAsync(h->rx_count, 0, 3 * sizeof(int), h->stream));
  return 0;
}

int rdsim_set_trajectory(rdsim_handle* h, int32_t stride, int32_t n_frames) {
  if (!h || stride <= 0 || n_frames < 0) return fail(RDSIM_ERR_ARG, "bad trajectory arguments");
  CK(cudaSetDevice(h->device));
  if (h->traj_x) cudaFree(h->traj_x);
  if (h->traj_t) cudaFree(h->traj_t);
  h->traj_x = nullptr;
  h->traj_t = nullptr;
  h->traj_stride = stride;
  h->traj_frames = n_frames;
  if (n_frames == 0) return 0;
  int64_t dummy = 0;
  int rc;
  if ((rc = dalloc(&h->traj_x, (size_t)n_frames * h->N * h->D, &dummy))) return rc;
  if ((rc = dalloc(&h->traj_t, (size_t)n_frames * h->N, &dummy))) return rc;
  CK(cudaMemsetAsync(h->traj_x, 0, sizeof(double) * (size_t)n_frames * h->N * h->D, h->stream));
  CK(cudaMemsetAsync(h->traj_t, 0, sizeof(int) * (size_t)n_frames * h->N, h->stream));
  return 0;
}

int rdsim_get_trajectory(rdsim_handle* h, double* x, int32_t* types) {
  if (!h) return fail(RDSIM_ERR_ARG, "null handle");
  if (h->traj_frames == 0) return 0;
  CK(cudaSetDevice(h->device));
  size_t nx = (size_t)h->traj_frames * h->N * h->D, nt = (size_t)h->traj_frames * h->N;
  if (x) CK(cudaMemcpyAsync(x, h->traj_x, sizeof(double) * nx, cudaMemcpyDeviceToHost, h->stream));
  if (types) CK(cudaMemcpyAsync(types, h->traj_t, sizeof(int) * nt, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int rdsim_get_error(rdsim_handle* h, int32_t* code, int64_t* particle, int32_t* dim,
                    double* value, int64_t* step) {
  if (!h) return fail(RDSIM_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  ErrDev e;
  CK(cudaMemcpyAsync(&e, h->err, sizeof e, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemsetAsync(h->err, 0, sizeof e, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (code) *code = e.code;
  if (particle) *particle = e.particle;
  if (dim) *dim = e.dim;
  if (value) *value = e.value;
  if (step) *step = e.step;
  return 0;
}

int rdsim_get_stream(rdsim_handle* h, void** stream) {
  if (!h || !stream) return fail(RDSIM_ERR_ARG, "null argument");
  *stream = (void*)h->stream;
  return 0;
}

int rdsim_set_profiling(rdsim_handle* h, int32_t enable) {
  if (!h) return fail(RDSIM_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  h->prof = (enable & 1) != 0;
  const bool stamp = (enable & 2) != 0;
  if (stamp != h->stamp_on) {
    // captured graphs hold the kernels' arguments: capture them again
    CK(cudaStreamSynchronize(h->stream));
    for (auto& g : h->graph_cache) cudaGraphExecDestroy(g.second.exec);
    h->graph_cache.clear();
    h->stamp_on = stamp;
  }
  if (stamp && !h->stamps) {
    const size_t nctas = std::max<size_t>(1, h->chunks_h.size());
    const size_t ring = std::min<size_t>(32768, std::max<size_t>(64, (512u << 20) / (16 * nctas)));
    int64_t dummy = 0;
    int rc;
    if ((rc = dalloc(&h->stamps, ring * nctas * 2, &dummy))) return rc;
    if ((rc = dalloc(&h->stamp_sum, 2, &dummy))) return rc;
    h->stamp_ring = (int)ring;
    CK(cudaMemsetAsync(h->stamps, 0, sizeof(unsigned long long) * ring * nctas * 2, h->stream));
  }
  return 0;
}

int rdsim_get_profile(rdsim_handle* h, rdsim_profile* p) {
  if (!h || !p) return fail(RDSIM_ERR_ARG, "null argument");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  resolve_profile(h);
  p->drift_span_ms = 0.0;
  p->drift_spans = 0;
  if (h->stamps) {
    const int nctas = (int)std::max<size_t>(1, h->chunks_h.size());
    CK(cudaMemsetAsync(h->stamp_sum, 0, 2 * sizeof(unsigned long long), h->stream));
    k_stamp_spans<<<h->stamp_ring, 256, 0, h->stream>>>(h->stamps, h->stamp_ring, nctas,
                                                        h->stamp_sum, h->stamp_sum + 1);
    CK(cudaGetLastError());
    unsigned long long r[2] = {0ull, 0ull};
    CK(cudaMemcpyAsync(r, h->stamp_sum, sizeof r, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemsetAsync(h->stamps, 0,
                       sizeof(unsigned long long) * (size_t)h->stamp_ring * nctas * 2, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    p->drift_span_ms = (double)r[0] * 1e-6;
    p->drift_spans = (int64_t)r[1];
  }
  for (int c = 0; c < RDSIM_PROFILE_CLASSES; c++) {
    p->launches[c] = h->nlaunch[c];
    p->ms[c] = h->prof_ms[c];
    p->timed[c] = h->prof_n[c];
    h->nlaunch[c] = 0;
    h->prof_ms[c] = 0;
    h->prof_n[c] = 0;
  }
  return 0;
}

int rdsim_get_info(rdsim_handle* h, rdsim_info* info) {
  if (!h || !info) return fail(RDSIM_ERR_ARG, "null argument");
  std::memset(info, 0, sizeof *info);
  info->n_particles = h->N;
  info->n_cells = h->ncells;
  info->n_blocks = (int64_t)h->chunks_h.size();
  info->threads_per_particle = h->ltpp;
  info->list_width = h->W;
  info->skin = h->skin;
  info->cell_size_min = h->cell_min;
  info->interaction_range = h->range;
  info->device_bytes = h->device_bytes;
  info->reaction_prefilter = (h->rx_pre && h->has_rx) ? 1 : 0;
  info->force_precision = h->f64 ? 1 : 0;
  info->period_kernel = h->period_on ? 1 : 0;
  info->list_period = h->freq;
  return 0;
}

int rdsim_test_withhold(rdsim_handle* h, int32_t chunk) {
  if (!h) return fail(RDSIM_ERR_ARG, "null handle");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  h->withhold = chunk;
  // periods are captured with the hook's value: recapture
  for (auto& g : h->graph_cache) cudaGraphExecDestroy(g.second.exec);
  h->graph_cache.clear();
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Neighbour pairs without allocation.
//
// rdsim_get_pairs allocates its device scratch (a pair counter and a pair
// buffer) with cudaMalloc and releases it with cudaFree on every call.  Some
// callers cannot do that: processes whose device memory is fully committed
// (a preallocated pool, another framework's cache), where cudaMalloc fails,
// and loops that must not pay the device-wide synchronisation of cudaFree.
// rdsim_get_pairs_static computes the same sorted pair list into the
// caller's host buffer with its scratch in the static device array below
// instead.
//
// The array is RDSIM_STATIC_PAIRS_MAX pairs (8 MiB) plus a counter; every GPU
// that loads the library holds it until the process exits.  Its device
// address belongs to the CUDA context that loaded the module: it is looked up
// (cudaGetSymbolAddress, with that device current) by the first call in each
// context on a device and again after the context changes (a cudaDeviceReset
// makes a new primary context, and with it a new array), under a lock.  The
// same set-up also loads k_pairs for every dimension, so that under lazy
// module loading no later call loads code.  All calls share the array: the
// counter is cleared at the start of every call, and calls that overlap on
// the GPU (from several threads or handles at once) race on it.
namespace {

constexpr long long kStaticPairsMax = RDSIM_STATIC_PAIRS_MAX;
// [0]: pair counter; [1 + p]: pair p as two int32 (i, j)
static __device__ __align__(256) unsigned long long g_pairs_scratch[1 + kStaticPairsMax];

constexpr int kMaxDevices = 64;
struct ScratchSlot {
  unsigned long long ctx_id = 0;   // context the address belongs to
  bool valid = false;
  unsigned long long* ptr = nullptr;
};
ScratchSlot g_pairs_slot[kMaxDevices];
std::mutex g_pairs_mutex;

// Current context's unique id (cuCtxGetId, through the runtime's driver entry
// points: the library does not link the driver directly).  False if the
// driver offers no such call; the address is then looked up on every call.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);
bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {  // under g_pairs_mutex
    looked_up = true;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
      get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
      get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    cudaGetLastError();
  }
  if (!get_current || !get_id) return false;
  void* ctx = nullptr;
  if (get_current(&ctx) != 0 || !ctx) return false;
  return get_id(ctx, id) == 0;
}

// Device address of g_pairs_scratch in the current context of `device` (the
// caller has made it current).
int static_scratch(int device, unsigned long long** out) {
  if (device < 0 || device >= kMaxDevices) return fail(RDSIM_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_pairs_mutex);
  unsigned long long id = 0;
  const bool have_id = current_context_id(&id);
  ScratchSlot& slot = g_pairs_slot[device];
  if (!have_id || !slot.valid || slot.ctx_id != id) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_pairs_scratch);
    if (e != cudaSuccess)
      return fail(RDSIM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    // load the pair kernels of every dimension now (lazy loading would
    // otherwise load each on its first launch)
    cudaFuncAttributes fa;
    const cudaError_t e1 = cudaFuncGetAttributes(&fa, k_pairs<1>);
    const cudaError_t e2 = cudaFuncGetAttributes(&fa, k_pairs<2>);
    const cudaError_t e3 = cudaFuncGetAttributes(&fa, k_pairs<3>);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
      return fail(RDSIM_ERR_CUDA, "loading the pair kernels failed");
    slot.ptr = static_cast<unsigned long long*>(p);
    slot.ctx_id = id;
    slot.valid = have_id;
  }
  *out = slot.ptr;
  return 0;
}

}  // namespace

extern "C" int rdsim_get_pairs_static(rdsim_handle* h, int32_t sys, int32_t* pairs,
                                      int64_t cap, int64_t* n_pairs) {
  if (!h || sys < 0 || sys >= h->nsys || !n_pairs) return fail(RDSIM_ERR_ARG, "bad argument");
  CK(cudaSetDevice(h->device));
  unsigned long long* scratch = nullptr;
  int rc = static_scratch(h->device, &scratch);
  if (rc) return rc;
  const HostSys& q = h->hs[sys];
  const SysDev& sd = h->sys_h[sys];
  CK(cudaMemsetAsync(scratch, 0, sizeof(unsigned long long), h->stream));
  double maxu = 0;
  for (int k = 0; k < h->D; k++) maxu = std::max(maxu, (double)sd.unit_hi[k]);
  const float rs2_hi = (float)(q.rs * q.rs) + guard2(q.rs, maxu);
  Args a = make_args(h);
  const unsigned g = nblk(q.n);
  int* buf = reinterpret_cast<int*>(scratch + 1);
  unsigned long long* cnt = scratch;
  const unsigned long long lim = (unsigned long long)kStaticPairsMax;
  if (h->D == 2) k_pairs<2><<<g, 256, 0, h->stream>>>(h->sys_d, sys, a, h->tmpl_d, q.rs, rs2_hi, q.p0, q.n, q.pid0, buf, lim, cnt);
  else if (h->D == 3) k_pairs<3><<<g, 256, 0, h->stream>>>(h->sys_d, sys, a, h->tmpl_d, q.rs, rs2_hi, q.p0, q.n, q.pid0, buf, lim, cnt);
  else k_pairs<1><<<g, 256, 0, h->stream>>>(h->sys_d, sys, a, h->tmpl_d, q.rs, rs2_hi, q.p0, q.n, q.pid0, buf, lim, cnt);
  CK(cudaGetLastError());
  unsigned long long n = 0;
  CK(cudaMemcpyAsync(&n, cnt, sizeof n, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  *n_pairs = (int64_t)n;
  if ((long long)n > kStaticPairsMax)
    return fail(RDSIM_ERR_CAPACITY,
                "rdsim_get_pairs_static: " + std::to_string(n) + " pairs exceed its static scratch of " +
                    std::to_string(kStaticPairsMax) + " pairs; use rdsim_get_pairs");
  if ((int64_t)n > cap) return fail(RDSIM_ERR_CAPACITY, "pair buffer too small");
  if (n == 0 || !pairs) return 0;
  CK(cudaMemcpyAsync(pairs, buf, sizeof(int) * 2 * n, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  // sort in the caller's buffer: (i, j) pairs of int32 viewed as one key each
  struct P {
    int32_t i, j;
  };
  P* v = reinterpret_cast<P*>(pairs);
  std::sort(v, v + n, [](const P& x, const P& y) { return x.i != y.i ? x.i < y.i : x.j < y.j; });
  return 0;
}
