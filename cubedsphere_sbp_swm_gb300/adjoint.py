"""Tangent-linear and adjoint of the FP64 model, binomially checkpointed
gradients of RK4 trajectories, and a torch.autograd.Function over them.

No counterpart in the reference.  Every product runs in the CUDA library
(include/swm_gpu.h: swm_apply_tl/ad, swm_rk4_tl/ad, swm_adjoint_*); torch
is used only to hand device tensors to it and to take part in autograd.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from . import OperatorSWM, StvecSWM


def apply_tl(op: OperatorSWM, y: StvecSWM, dx: StvecSWM, dk: StvecSWM):
    """dk = F'(y) dx (F: the model operator of OperatorSWM.apply)."""
    op._check(op._L.swm_apply_tl(op._h, y._h, dx._h, dk._h))


def apply_ad(op: OperatorSWM, y: StvecSWM, lk: StvecSWM, lx: StvecSWM):
    """lx = F'(y)^T lk."""
    op._check(op._L.swm_apply_ad(op._h, y._h, lk._h, lx._h))


def rk4_tl(op: OperatorSWM, x: StvecSWM, dx: StvecSWM, dt: float):
    """dx <- Phi'(x) dx for one RK4 step Phi."""
    op._check(op._L.swm_rk4_tl(op._h, x._h, dx._h, float(dt)))


def rk4_ad(op: OperatorSWM, x: StvecSWM, lx: StvecSWM, dt: float):
    """lx <- Phi'(x)^T lx."""
    op._check(op._L.swm_rk4_ad(op._h, x._h, lx._h, float(dt)))


def quadrature_weights(op: OperatorSWM) -> np.ndarray:
    """SBP quadrature weight of every node (J hx^2 A_i A_j), shape (6, N+1, N+1)."""
    w = np.empty(op.shape)
    op._check(op._L.swm_quadrature_weights(op._h, w.ctypes.data_as(_abi._D)))
    return w


class CheckpointedRK4:
    """nsteps RK4 steps of dt with binomial checkpointing (nsnap stored
    states, x0 included): forward() runs the trajectory and keeps the first
    snapshots, backward() turns dJ/dx_T into dJ/dx0, recomputing from the
    snapshots as the revolve recursion plans."""

    def __init__(self, op: OperatorSWM, dt: float, nsteps: int, nsnap: int = 16):
        self.op, self.dt, self.nsteps, self.nsnap = op, float(dt), int(nsteps), int(nsnap)
        h = ctypes.c_void_p()
        op._check(op._L.swm_adjoint_create(op._h, self.nsteps, self.nsnap, self.dt, ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.op._L.swm_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, x0: StvecSWM, xT: StvecSWM):
        self.op._check(self.op._L.swm_adjoint_forward(self._h, x0._h, xT._h))

    def backward(self, lam: StvecSWM):
        self.op._check(self.op._L.swm_adjoint_backward(self._h, lam._h))

    def counts(self) -> dict:
        f, a, p = ctypes.c_long(), ctypes.c_long(), ctypes.c_long()
        self.op._check(self.op._L.swm_adjoint_counts(self._h, ctypes.byref(f), ctypes.byref(a),
                                                     ctypes.byref(p)))
        return {"forward_steps": f.value, "adjoint_steps": a.value, "planned_forward_steps": p.value}


def _torch_trajectory_function():
    import torch

    def upload(op, s, t):
        t = t.detach().to(dtype=torch.float64).contiguous()
        torch.cuda.current_stream(t.device).synchronize()
        op._check(op._L.swm_state_upload_device(op._h, s._h, t[0].data_ptr(), t[1].data_ptr(),
                                                t[2].data_ptr()))
        return t

    def download(op, s, like):
        out = torch.empty_like(like)
        op._check(op._L.swm_state_download_device(op._h, s._h, out[0].data_ptr(), out[1].data_ptr(),
                                                  out[2].data_ptr()))
        op.synchronize()
        return out

    class RK4Trajectory(torch.autograd.Function):
        """x_T = Phi^nsteps(x0) on the GPU; backward through the discrete
        adjoint with binomial checkpointing.  x0: float64 CUDA tensor of
        shape (3, 6, N+1, N+1) holding (h, u, v)."""

        @staticmethod
        def forward(ctx, x0, runner: CheckpointedRK4):
            op = runner.op
            s0, sT = op.create_stvec(), op.create_stvec()
            x0c = upload(op, s0, x0)
            runner.forward(s0, sT)
            xT = download(op, sT, x0c)
            ctx.runner = runner
            ctx.like = x0c
            return xT

        @staticmethod
        def backward(ctx, g):
            runner = ctx.runner
            op = runner.op
            lam = op.create_stvec()
            upload(op, lam, g)
            runner.backward(lam)
            return download(op, lam, ctx.like), None

    return RK4Trajectory


_RK4Trajectory = None


def trajectory(x0, runner: CheckpointedRK4):
    """Differentiable x_T = Phi^nsteps(x0) for a float64 CUDA tensor x0 of
    shape (3, 6, N+1, N+1)."""
    global _RK4Trajectory
    if _RK4Trajectory is None:
        _RK4Trajectory = _torch_trajectory_function()
    return _RK4Trajectory.apply(x0, runner)
