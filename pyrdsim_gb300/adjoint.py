"""Gradients of trajectory losses of the reaction-free step on the GPU.

:class:`Adjoint` binds ``include/rdsim_adjoint.h``: a float64 forward run of
T reaction-free Euler-Maruyama steps (pyrdsim.pyx:2225-2292 with the pair
drift of pyrdsim.pyx:1941-2067, Lennard-Jones and Yukawa laws) under fixed,
injected noise, the loss

    L = (1/K) sum over the last K states of [U(x_n) + W(x_n) / (d V)]

(U truncated and shifted at each law's rc, W the pair virial), and its
discrete adjoint for dL/dx_0 and dL/d(u0, r0) of every law.
:func:`trajectory_loss` wraps it as a ``torch.autograd.Function``: tensors in,
a scalar loss out, gradients through ``loss.backward()``.  PyTorch provides
device memory and the autograd graph; the steps and their adjoint are the
hand-written kernels of ``csrc/adjoint.cu``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .engine import EngineError, load_library

EXPORTS = ["rdsim_adjoint_create", "rdsim_adjoint_destroy", "rdsim_adjoint_forward",
           "rdsim_adjoint_backward", "rdsim_adjoint_get_lists", "rdsim_adjoint_get_stream"]

MAX_LAWS = 8


class AdjointSystemStruct(C.Structure):
    _fields_ = [("n_dim", C.c_int32), ("n_particles", C.c_int32), ("n_types", C.c_int32),
                ("n_laws", C.c_int32), ("L", C.c_double * abi.MAX_DIM), ("dt", C.c_double),
                ("mobility", C.POINTER(C.c_double)), ("types", C.POINTER(C.c_int32)),
                ("laws", C.POINTER(abi.Interaction)), ("loss_steps", C.c_int32),
                ("checkpoint_every", C.c_int32)]


def _lib():
    L = load_library()
    if not getattr(L, "_adjoint_declared", False):
        vp = C.c_void_p
        dp = C.POINTER(C.c_double)
        L.rdsim_adjoint_create.argtypes = [C.POINTER(AdjointSystemStruct), C.c_int32,
                                           C.POINTER(vp)]
        L.rdsim_adjoint_destroy.argtypes = [vp]
        L.rdsim_adjoint_forward.argtypes = [vp, vp, dp, vp, C.c_int32, dp, vp]
        L.rdsim_adjoint_backward.argtypes = [vp, C.c_double, vp, dp]
        L.rdsim_adjoint_get_stream.argtypes = [vp, C.POINTER(vp)]
        L.rdsim_adjoint_get_lists.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L._adjoint_declared = True
    return L


def _check(rc):
    if rc != 0:
        raise EngineError(rc, _lib().rdsim_last_error().decode())


def law(kind, pair, u0, r0, rc, n=6):
    """One pair law: ``kind`` "lj" (U = u0[(r0/r)^2n - 2(r0/r)^n]) or "yukawa"
    (U = u0 exp(-r/r0)/r), types ``pair`` (a <= b), cutoff ``rc``."""
    it = abi.Interaction()
    it.law = abi.LAW_LJ if kind == "lj" else abi.LAW_YUKAWA
    it.type_a, it.type_b = int(min(pair)), int(max(pair))
    it.n = int(n)
    it.u0, it.r0, it.rc = float(u0), float(r0), float(rc)
    return it


class Adjoint:
    """One reaction-free system (periodic box) with a trajectory loss over the
    last ``loss_steps`` states, checkpoints every ``checkpoint_every`` steps."""

    def __init__(self, n_dim, L, dt, mobility, types, laws, loss_steps, checkpoint_every=32,
                 device=0):
        self.lib = _lib()
        self.D = int(n_dim)
        self.types = np.ascontiguousarray(types, dtype=np.int32)
        self.N = int(self.types.size)
        self.mobility = np.ascontiguousarray(mobility, dtype=np.float64)
        self.laws = (abi.Interaction * max(1, len(laws)))(*laws)
        self.n_laws = len(laws)
        self.loss_steps = int(loss_steps)
        self.device = int(device)
        s = AdjointSystemStruct()
        s.n_dim = self.D
        s.n_particles = self.N
        s.n_types = int(self.mobility.size)
        s.n_laws = self.n_laws
        for k in range(self.D):
            s.L[k] = float(L[k])
        s.dt = float(dt)
        s.mobility = self.mobility.ctypes.data_as(C.POINTER(C.c_double))
        s.types = self.types.ctypes.data_as(C.POINTER(C.c_int32))
        s.laws = C.cast(self.laws, C.POINTER(abi.Interaction))
        s.loss_steps = self.loss_steps
        s.checkpoint_every = int(checkpoint_every)
        h = C.c_void_p()
        _check(self.lib.rdsim_adjoint_create(C.byref(s), self.device, C.byref(h)))
        self.h = h
        self.generation = 0  # forward passes so far (the backward differentiates the last)
        st = C.c_void_p()
        _check(self.lib.rdsim_adjoint_get_stream(self.h, C.byref(st)))
        self.stream_ptr = st.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.rdsim_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def states_per_list(self):
        """States each neighbour list served in the last forward pass."""
        r, w = C.c_int32(), C.c_int32()
        _check(self.lib.rdsim_adjoint_get_lists(self.h, C.byref(r), C.byref(w)))
        return r.value

    def initial_params(self):
        """(u0, r0) of every law as given at construction, [n_laws, 2]."""
        return np.array([[w.u0, w.r0] for w in self.laws[: self.n_laws]], dtype=np.float64)

    def _order_after_torch(self):
        import torch
        ext = torch.cuda.ExternalStream(self.stream_ptr, device=self.device)
        ext.wait_stream(torch.cuda.current_stream(self.device))

    def forward(self, x0, params, xi):
        """x0 [N, D] and xi [T, N, D]: float64 CUDA tensors; params [n_laws, 2].
        Returns (loss, x_T)."""
        import torch
        x0 = x0.detach().contiguous()
        xi = xi.detach().contiguous()
        if x0.dtype != torch.float64 or xi.dtype != torch.float64 or not x0.is_cuda or not xi.is_cuda:
            raise TypeError("x0 and xi must be float64 CUDA tensors")
        if tuple(x0.shape) != (self.N, self.D) or xi.dim() != 3 or tuple(xi.shape[1:]) != (self.N, self.D):
            raise ValueError("x0 must be [N, D] and xi [T, N, D]")
        p = np.ascontiguousarray(np.asarray(params.detach().cpu() if hasattr(params, "detach")
                                            else params, dtype=np.float64).reshape(-1))
        if p.size != 2 * self.n_laws:
            raise ValueError("params must be [n_laws, 2]")
        xT = torch.empty_like(x0)
        self._order_after_torch()
        loss = C.c_double()
        _check(self.lib.rdsim_adjoint_forward(self.h, x0.data_ptr(),
                                              p.ctypes.data_as(C.POINTER(C.c_double)),
                                              xi.data_ptr(), int(xi.shape[0]), C.byref(loss),
                                              xT.data_ptr()))
        self.generation += 1
        self._keep = (x0, xi)  # the backward pass re-reads the noise
        return loss.value, xT

    def backward(self, dloss=1.0):
        """Gradients of dloss * L of the last forward pass: (dL/dx0 [N, D] on the
        device, dL/d(u0, r0) [n_laws, 2] on the host)."""
        import torch
        gx = torch.empty((self.N, self.D), dtype=torch.float64, device=f"cuda:{self.device}")
        gp = np.zeros(2 * max(1, self.n_laws), dtype=np.float64)
        self._order_after_torch()
        _check(self.lib.rdsim_adjoint_backward(self.h, float(dloss), gx.data_ptr(),
                                               gp.ctypes.data_as(C.POINTER(C.c_double))))
        return gx, torch.from_numpy(gp[: 2 * self.n_laws].reshape(self.n_laws, 2).copy())


def _function():
    import torch

    class TrajectoryLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x0, params, xi, adj):
            loss, _ = adj.forward(x0, params, xi)
            ctx.adj = adj
            ctx.generation = adj.generation
            ctx.params_device = params.device
            ctx.save_for_backward(xi)
            return torch.tensor(loss, dtype=torch.float64, device=x0.device)

        @staticmethod
        def backward(ctx, gout):
            adj = ctx.adj
            if adj.generation != ctx.generation:
                raise RuntimeError("another forward pass ran on this Adjoint handle since; "
                                   "use one handle per loss that is differentiated")
            gx, gp = adj.backward(float(gout))
            return gx, gp.to(ctx.params_device), None, None

    return TrajectoryLoss


_FN = None


def trajectory_loss(x0, params, xi, adj):
    """Differentiable L(x0, params) for fixed noise xi (see the module doc)."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(x0, params, xi, adj)


def _main(argv=None):
    """Loss and gradients of the mixed Lennard-Jones + Yukawa workload:
    ``python -m pyrdsim_gb300.adjoint --n 16384 --steps 1000``."""
    import argparse
    import time

    import torch

    from . import workloads
    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, default=16384)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--loss-steps", type=int, default=0, help="default: half the steps")
    p.add_argument("--checkpoint-every", type=int, default=32)
    p.add_argument("--repeat", type=int, default=2)
    a = p.parse_args(argv)
    w = workloads.mixed_lj_yukawa(n=a.n)
    K = a.loss_steps or max(1, a.steps // 2)
    adj = Adjoint(2, w["L"], w["dt"], w["mobility"], w["types"], workloads.mixed_lj_yukawa_laws(w),
                  loss_steps=K, checkpoint_every=a.checkpoint_every)
    gen = torch.Generator(device="cuda").manual_seed(5)
    xi = torch.randn((a.steps, a.n, 2), dtype=torch.float64, device="cuda", generator=gen)
    x0 = torch.tensor(w["x0"], dtype=torch.float64, device="cuda")
    params = workloads.mixed_lj_yukawa_params(w["theta"])
    for _ in range(a.repeat):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss, _ = adj.forward(x0, params, xi)
        t1 = time.perf_counter()
        gx, gp = adj.backward()
        t2 = time.perf_counter()
    print(f"N={a.n} T={a.steps} K={K} E={a.checkpoint_every}: loss {loss:.10g}, "
          f"forward {1e6 * (t1 - t0) / a.steps:.1f} us/step, "
          f"backward {1e6 * (t2 - t1) / a.steps:.1f} us/step, |dL/dx0| {float(gx.norm()):.6g}")


if __name__ == "__main__":
    _main()
