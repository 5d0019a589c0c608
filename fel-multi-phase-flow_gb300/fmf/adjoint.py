"""The adjoint of the K-step rollout (``fmf_adj_*`` of include/fmf_capi.h part 4).

``Adjoint.rollout`` returns the contact-line objective J (the reference's
find_interface_positions_lower of phi after K steps) and its gradients with
respect to the per-wall-cell static angle theta0, the GNBC coefficient zeta, the
slip lengths l1, l2 and the initial phi.  ``RolloutJ`` wraps it as a
``torch.autograd.Function`` of (theta0, zeta, l1, l2, phi): the forward pass runs
the GPU solver, the backward pass returns the adjoint gradients.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import config as fcfg
from .capi import FmfError, P, _ptr_array, check, lib, params

_bound = False


def _bind():
    global _bound
    if _bound:
        return
    L = lib()
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.fmf_adj_create.argtypes = [vp, ctypes.POINTER(vp)]
    L.fmf_adj_destroy.argtypes = [vp]
    L.fmf_adj_set_solver.argtypes = [vp, dp, ip, dp, ip]
    L.fmf_adj_forward.argtypes = [vp, ip, vp, vp, vp, vp, vp, ctypes.POINTER(dp), vp]
    L.fmf_adj_rollout.argtypes = [vp, ip, ip, vp, vp, vp, vp, vp, ctypes.POINTER(dp), vp, vp, vp, vp, vp]
    L.fmf_adj_iterations.argtypes = [vp, ctypes.POINTER(ip), ctypes.POINTER(ip)]
    L.fmf_adj_phase_seconds.argtypes = [vp, ctypes.POINTER(dp)]
    L.fmf_adj_device_bytes.argtypes = [vp]
    L.fmf_adj_device_bytes.restype = ctypes.c_longlong
    _bound = True


class Adjoint:
    """One GPU adjoint context for a configuration."""

    def __init__(self, cfg: fcfg.Config, sor_tol: float = 1e-3, sor_max: int = 21, adj_tol: float = 1e-12,
                 adj_max: int = 200, precision: int = 0):
        """precision: 0 (FMF_FP64) or 1 (FMF_MIXED: the forward and recomputed steps
        run the mixed-precision step; the reverse stays FP64)."""
        _bind()
        self.cfg = cfg
        self._prm = params(cfg, precision)
        h = ctypes.c_void_p()
        check(lib().fmf_adj_create(ctypes.byref(self._prm), ctypes.byref(h)), "fmf_adj_create")
        self.h = h
        check(lib().fmf_adj_set_solver(self.h, sor_tol, int(sor_max), adj_tol, int(adj_max)), "set_solver")

    def close(self):
        if getattr(self, "h", None):
            lib().fmf_adj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, K: int, state0: np.ndarray, walls, want_state: bool = False):
        th, ze, l1, l2 = [np.ascontiguousarray(w, dtype=np.float64) for w in walls]
        st = np.ascontiguousarray(state0, dtype=np.float64)
        J = ctypes.c_double()
        out = np.zeros_like(st) if want_state else None
        check(lib().fmf_adj_forward(self.h, int(K), _ptr_array(list(st)), P(th), P(ze), P(l1), P(l2),
                                    ctypes.byref(J), _ptr_array(list(out)) if want_state else None),
              "fmf_adj_forward")
        return (J.value, out) if want_state else J.value

    def rollout(self, K: int, state0: np.ndarray, walls, every: int = 0):
        """J and the gradients (theta0, zeta, l1, l2, phi1_initial) as full arrays."""
        th, ze, l1, l2 = [np.ascontiguousarray(w, dtype=np.float64) for w in walls]
        st = np.ascontiguousarray(state0, dtype=np.float64)
        grads = [np.zeros(self.cfg.shape) for _ in range(5)]
        J = ctypes.c_double()
        check(lib().fmf_adj_rollout(self.h, int(K), int(every), _ptr_array(list(st)), P(th), P(ze), P(l1),
                                    P(l2), ctypes.byref(J), *[P(gr) for gr in grads]), "fmf_adj_rollout")
        return J.value, grads

    def iterations(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        check(lib().fmf_adj_iterations(self.h, ctypes.byref(a), ctypes.byref(b)), "iterations")
        return a.value, b.value

    def phase_seconds(self):
        """(forward, segment recomputation, reverse) seconds of the last rollout."""
        out = (ctypes.c_double * 3)()
        check(lib().fmf_adj_phase_seconds(self.h, out), "phase_seconds")
        return tuple(out)

    def device_bytes(self) -> int:
        """Device bytes the handle (and its recomputing second handle) holds."""
        return int(lib().fmf_adj_device_bytes(self.h))


def rollout_function(adj: Adjoint, K: int, state0: np.ndarray, every: int = 0):
    """A torch.autograd.Function J(theta0, zeta, l1, l2, phi1) of the K-step rollout
    (phi1: the initial slice-1 volume fraction; the rest of state0 is held fixed)."""
    import torch

    class RolloutJ(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta0, zeta, l1, l2, phi1):
            st = np.array(state0, dtype=np.float64, copy=True)
            st[fcfg.STATE_FIELDS.index("phi1")] = phi1.detach().cpu().numpy()
            walls = [t.detach().cpu().numpy() for t in (theta0, zeta, l1, l2)]
            J, grads = adj.rollout(K, st, walls, every)
            ctx.grads = [torch.from_numpy(gr) for gr in grads]
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            return tuple(gJ * gr for gr in ctx.grads)

    return RolloutJ.apply


__all__ = ["Adjoint", "rollout_function", "FmfError"]
