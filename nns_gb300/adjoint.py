"""Trajectory gradients through the Barnes-Hut pipeline (libnbx adjoint kernels).

``Adjoint`` drives the C ABI (include/nbx.h, nbx_adjoint_*): T kick-drift steps
with checkpoints every C steps, then the reverse pass over recomputed,
recorded interaction lists.  ``TrajectoryLoss`` wraps it in a
``torch.autograd.Function`` -- only so that gradient checks can be written
against torch's API; the forward and backward are the library's kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import check, lib
from .barnes_hut import Context, State, _stream_ptr


class Adjoint:
    def __init__(self, ctx: Context, nsteps: int, checkpoint_every: int = 10,
                 list_capacity: int = 8192, tape_steps: int | None = None):
        self.ctx = ctx
        self.nsteps = nsteps
        self.checkpoint_every = checkpoint_every
        h = C.c_void_p()
        check(lib().nbx_adjoint_create(ctx.h, nsteps, checkpoint_every, list_capacity,
                                       tape_steps or checkpoint_every, C.byref(h)),
              "nbx_adjoint_create", ctx.h)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().nbx_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 -- interpreter shutdown
            pass

    def forward(self, s: State, target: torch.Tensor, stream=None) -> float:
        """T steps from s (advanced in place); loss against target (3, n) on the device.

        The steps run on the adjoint's own copy of the state, as replayed CUDA
        graphs on the adjoint's stream (ordered after ``stream``); the call
        returns when the loss is known.  The context needs a new build before
        its next walk."""
        t = target.contiguous()
        loss = C.c_double()
        check(lib().nbx_adjoint_forward(self.ctx.h, self.h, C.byref(s.c), t[0].data_ptr(),
                                        t[1].data_ptr(), t[2].data_ptr(), C.byref(loss),
                                        _stream_ptr(stream)),
              "nbx_adjoint_forward", self.ctx.h)
        return loss.value

    def backward(self, s: State, stream=None):
        """(dL/dx0 (3,n), dL/dv0 (3,n), dL/dm (n,)) of the last forward, as device tensors."""
        n = s.x.numel()
        g = torch.empty(7, n, dtype=torch.float32, device=s.x.device)
        check(lib().nbx_adjoint_backward(self.ctx.h, self.h, C.byref(s.c),
                                         *[g[k].data_ptr() for k in range(7)], _stream_ptr(stream)),
              "nbx_adjoint_backward", self.ctx.h)
        return g[0:3], g[3:6], g[6]

    def record(self, s: State, stream=None):
        check(lib().nbx_adjoint_record(self.ctx.h, self.h, C.byref(s.c), _stream_ptr(stream)),
              "nbx_adjoint_record", self.ctx.h)

    def replay_fp64(self, state0: torch.Tensor, stream=None) -> float:
        """FP64 loss of the recorded trajectory from state0 (7, n) float64 on the device."""
        loss = C.c_double()
        check(lib().nbx_adjoint_replay_fp64(self.ctx.h, self.h, state0.contiguous().data_ptr(),
                                            C.byref(loss), _stream_ptr(stream)),
              "nbx_adjoint_replay_fp64", self.ctx.h)
        return loss.value

    def stats(self) -> dict:
        b = C.c_int64()
        f, w = C.c_float(), C.c_float()
        check(lib().nbx_adjoint_stats(self.h, C.byref(b), C.byref(f), C.byref(w)),
              "nbx_adjoint_stats")
        return {"bytes": b.value, "forward_ms": f.value, "backward_ms": w.value}


class TrajectoryLoss(torch.autograd.Function):
    """L(x0, v0, m) = sum |x(T) - x*|^2 through the Barnes-Hut steps of `adj`.

    x0, v0: (3, n) float32 CUDA tensors; m: (n,) float32; target: (3, n)."""

    @staticmethod
    def forward(fctx, x0, v0, m, target, adj: Adjoint):
        n = m.numel()
        z = lambda: torch.zeros(n, dtype=torch.float32, device=m.device)  # noqa: E731
        s = State(x0[0].clone(), x0[1].clone(), x0[2].clone(), v0[0].clone(), v0[1].clone(),
                  v0[2].clone(), z(), z(), z(), m.clone())
        loss = adj.forward(s, target)
        fctx.adj = adj
        fctx.state = s
        return torch.tensor(loss, dtype=torch.float64, device=m.device)

    @staticmethod
    def backward(fctx, gout):
        gx, gv, gm = fctx.adj.backward(fctx.state)
        sc = gout.to(torch.float32)
        return gx * sc, gv * sc, gm * sc, None, None


def random_directions(n: int, k: int, seed: int = 7) -> np.ndarray:
    """k random unit vectors over the 7n parameters (x0, v0, m)."""
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((k, 7, n))
    u /= np.linalg.norm(u.reshape(k, -1), axis=1)[:, None, None]
    return u
