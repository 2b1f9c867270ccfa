/*
 * rdsim_adjoint.h -- gradients of trajectory losses of the reaction-free
 * step (no reference counterpart: PyRDSim has no derivatives).
 *
 * The differentiated map is the reaction-free integration step of
 * pyrdsim.pyx:2296-2322 with injected noise and periodic boundaries:
 *   x_{n+1} = wrap(x_n + c * a(x_n) + s * xi_n),  c = dt D_t, s = sqrt(2 dt D_t)
 * (pyrdsim.pyx:2225-2250, 2253-2292), a = the pair drift of
 * pyrdsim.pyx:1941-2067 for Lennard-Jones and Yukawa laws
 * (pyrdsim.pyx:1068-1130), everything in float64.  The loss is
 *   L = (1/K) sum_{n = T-K+1}^{T} [ U(x_n) + W(x_n) / (d V) ]
 * with U the pair energy truncated and shifted at each law's rc (so that U
 * is continuous), W = sum over pairs of -r dU/dr (the virial), d the
 * dimension and V the box volume: the time-averaged potential energy plus
 * the virial part of the pressure over the last K of T steps.
 * rdsim_adjoint_backward returns dL/dx_0 and dL/d(u0, r0) of every law by
 * the discrete adjoint of the same float64 steps (Hessian-vector products
 * of the pair potential), recomputing states from checkpoints kept every
 * checkpoint_every steps.
 *
 * Pair set: all pairs of the box (any molecules; this path has no bonded
 * terms) whose sorted type pair matches a law, r < rc, minimum image.
 */
#ifndef RDSIM_ADJOINT_H
#define RDSIM_ADJOINT_H

#include <stdint.h>

#include "rdsim.h"

#ifdef __cplusplus
extern "C" {
#endif

#define RDSIM_ADJ_MAX_LAWS 8

typedef struct {
  int32_t n_dim;              /* 2 or 3                                      */
  int32_t n_particles;
  int32_t n_types;
  int32_t n_laws;             /* <= RDSIM_ADJ_MAX_LAWS                       */
  double L[RDSIM_MAX_DIM];    /* periodic box, L >= 2 rc of every law        */
  double dt;
  const double* mobility;     /* [n_types] tau_by_tauD (D of each type)      */
  const int32_t* types;       /* [n_particles]                               */
  const rdsim_interaction* laws; /* RDSIM_LAW_LJ or RDSIM_LAW_YUKAWA, pair
                                    (type_a <= type_b); u0, r0 are the
                                    differentiated parameters, rc fixed      */
  int32_t loss_steps;         /* K                                           */
  int32_t checkpoint_every;   /* states kept every this many steps (>= 1)    */
} rdsim_adjoint_system;

typedef struct rdsim_adjoint rdsim_adjoint;

int rdsim_adjoint_create(const rdsim_adjoint_system* sys, int32_t device,
                         rdsim_adjoint** out);
int rdsim_adjoint_destroy(rdsim_adjoint* h);

/* T = n_steps steps from x0 with noise xi.  x0 [N][n_dim] and xi
 * [n_steps][N][n_dim] are DEVICE pointers (float64); params [n_laws][2]
 * (u0, r0 per law) is a host array.  *loss receives L; x_final (device,
 * may be NULL) receives x_T.  Keeps the checkpoints for the backward pass;
 * xi must stay valid until then. */
int rdsim_adjoint_forward(rdsim_adjoint* h, const double* x0, const double* params,
                          const double* xi, int32_t n_steps, double* loss,
                          double* x_final);

/* Gradients of dloss * L of the last forward: grad_x0 [N][n_dim] (DEVICE)
 * and grad_params [n_laws][2] (host: dL/du0, dL/dr0 per law). */
int rdsim_adjoint_backward(rdsim_adjoint* h, double dloss, double* grad_x0,
                           double* grad_params);

/* Neighbour lists of the last forward pass: each served *states_per_list
 * consecutive states (8, 4 or 2 when checkpoint_every allows it and no
 * particle outran the skin, else 1); *list_width entries per lane. */
int rdsim_adjoint_get_lists(rdsim_adjoint* h, int32_t* states_per_list, int32_t* list_width);

/* CUDA stream of the handle (cudaStream_t). */
int rdsim_adjoint_get_stream(rdsim_adjoint* h, void** stream);

#ifdef __cplusplus
}
#endif
#endif
