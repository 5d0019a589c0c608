"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module; the CUDA product never does.  ``build()`` compiles
``fmf_oracle.cpp`` into ``oracle/_build/libfmf_oracle.so``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libfmf_oracle.so")
SRC = os.path.join(HERE, "fmf_oracle.cpp")

_REPO = os.path.dirname(HERE)
_PKG = os.path.join(_REPO, "fel-multi-phase-flow_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)
from fmf import config as fcfg  # noqa: E402

_lib = None


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "fmf_oracle.h"))):
        cmd = ["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               "-std=c++17", "-o", LIB + ".tmp", SRC]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _lib.orc_step.restype = ctypes.c_int
        _lib.orc_solu_sor4_v.restype = ctypes.c_int
        _lib.orc_interface_lower.restype = ctypes.c_double
        _lib.orc_ws_create.restype = ctypes.c_void_p
        _lib.orc_ws_destroy.argtypes = [ctypes.c_void_p]
    return _lib


# ---- argument helpers -------------------------------------------------------
def I(x: int):
    return ctypes.byref(ctypes.c_int(int(x)))


def D(x: float):
    return ctypes.byref(ctypes.c_double(float(x)))


def P(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def IA(vals):
    arr = (ctypes.c_int * len(vals))(*vals)
    return arr


NID = (-1, -1, -1, -1, -1, -1)


class OrcParams(ctypes.Structure):
    _fields_ = [("ni", ctypes.c_int), ("nj", ctypes.c_int), ("nk", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("dt", ctypes.c_double), ("rhol", ctypes.c_double), ("rhog", ctypes.c_double),
                ("rmul", ctypes.c_double), ("rmug", ctypes.c_double), ("sigma", ctypes.c_double),
                ("uwall", ctypes.c_double), ("grvb", ctypes.c_double), ("grvp", ctypes.c_double),
                ("bet_mthinc", ctypes.c_double), ("harmonic", ctypes.c_int)]


def params(cfg: fcfg.Config) -> OrcParams:
    return OrcParams(cfg.ni, cfg.nj, cfg.nk, cfg.dx, cfg.dy, cfg.dz, cfg.dt, cfg.rhol, cfg.rhog,
                     cfg.rmul, cfg.rmug, cfg.sigma, cfg.uwall, cfg.grvb, cfg.grvp, cfg.bet_mthinc,
                     cfg.harmonic)


class Solver:
    """Runs the oracle's restatement of main.f90's time loop on a numpy state stack."""

    def __init__(self, cfg: fcfg.Config):
        self.cfg = cfg
        self._prm = params(cfg)
        self.ws = ctypes.c_void_p(lib().orc_ws_create(ctypes.byref(self._prm)))
        self.walls = fcfg.wall_arrays(cfg)
        self.sor_iters = []
        self.diag = []

    def close(self):
        if self.ws:
            lib().orc_ws_destroy(self.ws)
            self.ws = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ptrs(self, st):
        arr = (ctypes.POINTER(ctypes.c_double) * 12)(*[P(st[n]) for n in range(12)])
        return arr

    def initial_state(self) -> np.ndarray:
        st = fcfg.raw_state(self.cfg)
        th, ze, l1, l2 = self.walls
        lib().orc_init_bc(self.ws, self._ptrs(st), P(th), P(ze), P(l1), P(l2))
        return st

    def step(self, st: np.ndarray, n: int = 1) -> np.ndarray:
        th, ze, l1, l2 = self.walls
        ptrs = self._ptrs(st)
        diag = (ctypes.c_double * 2)()
        for _ in range(n):
            it = lib().orc_step(self.ws, ptrs, P(th), P(ze), P(l1), P(l2), diag)
            self.sor_iters.append(it)
            self.diag.append((diag[0], diag[1]))
        return st
