"""ctypes binding of libfmf.so (the CUDA product).

``load()`` raises when the library is missing: there is no CPU fallback.
``Stepper`` drives the fused device-resident time step (``fmf_ctx_*``); the
drop-in subroutines (``<name>_``) are reached through ``lib()`` with the same
arguments the Fortran caller passes (every argument by reference).
"""
from __future__ import annotations

import ctypes
import os
import warnings

import numpy as np

from . import config as fcfg
from .build import LIB

_lib = None

FMF_FP64, FMF_MIXED, FMF_FP64E = 0, 1, 2
FMF_RESIDENT, FMF_COHERENT = 0, 1
FMF_ERR_ITER_CAP = 4


class SorCapWarning(UserWarning):
    """A viscous solve ended at its iteration cap without meeting its stop rule (the
    step carried on with the last iterate, as the reference's does)."""


class FmfError(RuntimeError):
    pass


class Params(ctypes.Structure):
    _fields_ = [("ni", ctypes.c_int), ("nj", ctypes.c_int), ("nk", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("dt", ctypes.c_double), ("rhol", ctypes.c_double), ("rhog", ctypes.c_double),
                ("rmul", ctypes.c_double), ("rmug", ctypes.c_double), ("sigma", ctypes.c_double),
                ("uwall", ctypes.c_double), ("grvb", ctypes.c_double), ("grvp", ctypes.c_double),
                ("bet_mthinc", ctypes.c_double), ("harmonic", ctypes.c_int), ("precision", ctypes.c_int)]


def params(cfg: fcfg.Config, precision: int = FMF_FP64) -> Params:
    return Params(cfg.ni, cfg.nj, cfg.nk, cfg.dx, cfg.dy, cfg.dz, cfg.dt, cfg.rhol, cfg.rhog,
                  cfg.rmul, cfg.rmug, cfg.sigma, cfg.uwall, cfg.grvb, cfg.grvp, cfg.bet_mthinc,
                  cfg.harmonic, precision)


def load(path: str | None = None):
    """Load libfmf.so; raise FmfError if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB
    if not os.path.exists(path):
        raise FmfError(f"{path} is missing: build it with fmf.build.build() (nvcc, sm_103a)")
    L = ctypes.CDLL(path)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.fmf_ctx_create.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(vp)]
    L.fmf_ctx_create.restype = ip
    for name in ("fmf_ctx_destroy", "fmf_ctx_init_bc", "fmf_ctx_synchronize"):
        getattr(L, name).argtypes = [vp]
        getattr(L, name).restype = ip
    L.fmf_ctx_step.argtypes = [vp, ip]
    L.fmf_ctx_step.restype = ip
    L.fmf_ctx_set_sor.argtypes = [vp, dp, ip]
    L.fmf_ctx_set_sor.restype = ip
    L.fmf_ctx_check_sor.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    L.fmf_ctx_check_sor.restype = ip
    L.fmf_set_sor.argtypes = [dp, ip]
    L.fmf_set_sor.restype = ip
    L.fmf_last_solp_residual.argtypes = [ctypes.POINTER(dp), ctypes.POINTER(dp)]
    L.fmf_last_solp_residual.restype = ip
    L.fmf_ctx_set_stream.argtypes = [vp, vp]
    L.fmf_ctx_set_walls.argtypes = [vp, vp, vp, vp, vp]
    L.fmf_ctx_upload.argtypes = [vp, ctypes.POINTER(vp)]
    L.fmf_ctx_download.argtypes = [vp, ctypes.POINTER(vp)]
    L.fmf_ctx_step_host.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.fmf_ctx_sor_iterations.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ip]
    L.fmf_ctx_sor_iterations.restype = ip
    L.fmf_ctx_state_device_ptr.argtypes = [vp, ip, ctypes.POINTER(vp)]
    L.fmf_ctx_device_bytes.argtypes = [vp]
    L.fmf_ctx_device_bytes.restype = ctypes.c_longlong
    L.fmf_kernel_launches.restype = ctypes.c_longlong
    L.fmf_error_string.restype = ctypes.c_char_p
    L.fmf_last_sor_ratio.restype = dp
    L.fmf_interface_lower.restype = dp
    L.fmf_interface_lower.argtypes = [ip, ip, ip, vp, dp, dp]
    L.fmf_set_stream.argtypes = [vp]
    L.fmf_dev_weno5_fused.argtypes = [ip, ip, ip, ip, dp, dp, dp, vp, vp, vp, vp, vp, vp]
    L.fmf_dev_weno5_fused.restype = ip
    L.fmf_dev_csf_fused.argtypes = [ip, ip, ip, ip, dp, dp, dp, dp, dp, dp, vp, vp, vp, vp]
    L.fmf_dev_csf_fused.restype = ip
    for name in ("fmf_sync_to_host", "fmf_sync_to_device", "fmf_forget"):
        getattr(L, name).argtypes = [vp]
    _lib = L
    return L


def lib():
    return load()


def check(code: int, what: str = "") -> None:
    """Raise FmfError for a nonzero status; the iteration-cap status (not fatal:
    the step carried on) is a SorCapWarning instead."""
    if code == FMF_ERR_ITER_CAP:
        warnings.warn(f"{what}: {lib().fmf_error_string(code).decode()}", SorCapWarning, stacklevel=2)
    elif code:
        msg = lib().fmf_error_string(code).decode()
        raise FmfError(f"{what}: {msg} ({code})")


# ---- Fortran-style argument helpers -----------------------------------------
def I(x: int):
    return ctypes.byref(ctypes.c_int(int(x)))


def D(x: float):
    return ctypes.byref(ctypes.c_double(float(x)))


def P(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return ctypes.c_void_p(a.ctypes.data)


def IA(vals):
    return (ctypes.c_int * len(vals))(*vals)


def _ptr_array(arrs):
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


class Stepper:
    """The fused device-resident time step on one GPU."""

    def __init__(self, cfg: fcfg.Config, precision: int = FMF_FP64, stream=None):
        self.cfg = cfg
        self._prm = params(cfg, precision)
        h = ctypes.c_void_p()
        check(lib().fmf_ctx_create(ctypes.byref(self._prm), ctypes.byref(h)), "fmf_ctx_create")
        self.h = h
        if stream is not None:
            check(lib().fmf_ctx_set_stream(self.h, ctypes.c_void_p(stream)), "set_stream")
        self.walls = fcfg.wall_arrays(cfg)
        th, ze, l1, l2 = self.walls
        check(lib().fmf_ctx_set_walls(self.h, P(th), P(ze), P(l1), P(l2)), "set_walls")

    def close(self):
        if getattr(self, "h", None):
            lib().fmf_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, st: np.ndarray):
        self._up = st  # keep the host buffer alive while the copy is in flight
        check(lib().fmf_ctx_upload(self.h, _ptr_array(list(st))), "upload")

    def download(self, st: np.ndarray):
        check(lib().fmf_ctx_download(self.h, _ptr_array(list(st))), "download")

    def init_bc(self):
        check(lib().fmf_ctx_init_bc(self.h), "init_bc")

    def step(self, n: int = 1):
        check(lib().fmf_ctx_step(self.h, int(n)), "step")

    def set_sor(self, tol: float = 1e-3, max_iter: int = 21):
        """The viscous solve's stop rule (default: the reference's)."""
        check(lib().fmf_ctx_set_sor(self.h, float(tol), int(max_iter)), "set_sor")

    def check_sor(self) -> dict:
        """The next step's viscous solve against the FP64 stop rule, on the current
        state (not advanced): its outer iterations, the ratio its own rule stopped
        on, the FP64 ratio of one more FP64 iteration from its result and from an
        FP64 solve's result, and its result's distance from the FP64 solve's
        relative to the step's velocity change (fmf_ctx_check_sor)."""
        out = (ctypes.c_double * 5)()
        check(lib().fmf_ctx_check_sor(self.h, out), "check_sor")
        return {"iterations": int(out[0]), "own_ratio": out[1], "fp64_ratio": out[2],
                "fp64_ratio_of_fp64_solve": out[3], "rel_diff_vs_fp64_solve": out[4]}

    def step_host(self, st_in: np.ndarray, st_out: np.ndarray):
        """One step from host state st_in to host state st_out (fmf_ctx_step_host;
        synchronous, the early result fields copied back while the step runs)."""
        check(lib().fmf_ctx_step_host(self.h, _ptr_array(list(st_in)), _ptr_array(list(st_out))), "step_host")

    def sync(self):
        check(lib().fmf_ctx_synchronize(self.h), "synchronize")

    def sor_iterations(self):
        buf = (ctypes.c_int * 100000)()
        n = lib().fmf_ctx_sor_iterations(self.h, buf, 100000)
        return list(buf[:n])

    def device_bytes(self) -> int:
        return int(lib().fmf_ctx_device_bytes(self.h))

    def initial_state(self) -> np.ndarray:
        st = fcfg.raw_state(self.cfg)
        self.upload(st)
        self.init_bc()
        self.download(st)
        self.sync()
        return st

    def get_state(self) -> np.ndarray:
        st = np.zeros((12,) + self.cfg.shape)
        self.download(st)
        self.sync()
        return st
