"""Pins of the CPU oracle (no GPU): golden FFT vectors from numpy, analytic
known answers, and the invariants the reference monitors at run time
(AV_PHI main.f90:519-524, Err_div main.f90:675-684, Err_solp
solp_fft_tdma4.f:28-93, Err_solu solu_sor4.f:298-305)."""
import ctypes
import os

import numpy as np
import pytest

from fmf import config as C

GOLD = os.path.join(os.path.dirname(__file__), "golden", "fft2_golden.npz")


def _fft2(orc, x, sign):
    n2, n1 = x.shape
    buf = np.empty(2 * x.size)
    buf[0::2] = x.real.ravel()
    buf[1::2] = x.imag.ravel()
    orc.lib().orc_fft2d(orc.P(buf), ctypes.c_int(n1), ctypes.c_int(n2), ctypes.c_int(sign))
    return (buf[0::2] + 1j * buf[1::2]).reshape(n2, n1)


def test_fft_golden(orc):
    g = np.load(GOLD)
    for key in g.files:
        if not key.startswith("x_"):
            continue
        tag = key[2:]
        x = g[key]
        f = _fft2(orc, x, -1)
        b = _fft2(orc, x, +1)
        scale = np.abs(g["fwd_" + tag]).max()
        assert np.abs(f - g["fwd_" + tag]).max() <= 1e-13 * scale, tag
        assert np.abs(b - g["inv_" + tag]).max() <= 1e-13 * scale, tag


def test_weno5_linear_is_exact(orc):
    """weno5.h: on a linear field every smoothness indicator is 0, the weights
    collapse to the central candidate and the scheme returns vel*du/dx exactly."""
    cfg = C.Config("t", 16, 8, 8, 1.0, 1.0, 1.0, dt=1e-3, steps=1)
    sh = cfg.shape
    ii = np.arange(-2, cfg.ni + 4, dtype=np.float64)
    u = np.broadcast_to(0.3 + 0.7 * ii[None, None, :], sh).copy()
    v = np.zeros(sh)
    w = np.zeros(sh)
    out = [np.zeros(sh) for _ in range(3)]
    dxi = 1.0 / cfg.dx
    orc.lib().orc_cal_advu_weno5(orc.I(cfg.ni), orc.I(cfg.nj), orc.I(cfg.nk), orc.D(dxi), orc.D(dxi), orc.D(dxi),
                                 orc.P(u), orc.P(v), orc.P(w), *[orc.P(a) for a in out])
    # u(i) = 0.3 + 0.7 i at staggered x-faces; the advecting velocity is u itself there
    ui = C.interior(u)
    want = ui * 0.7 * dxi
    np.testing.assert_allclose(C.interior(out[0]), want, rtol=1e-14, atol=1e-14)
    assert np.all(C.interior(out[1]) == 0) and np.all(C.interior(out[2]) == 0)


def _run(orc, cfg, steps):
    s = orc.Solver(cfg)
    st = s.initial_state()
    s.step(st, steps)
    return s, st


def test_volume_conservation(orc):
    cfg = C.get("couette32")
    s = orc.Solver(cfg)
    st = s.initial_state()
    v0 = C.interior(st[9]).sum()
    s.step(st, 20)
    v1 = C.interior(st[9]).sum()
    assert abs(v1 - v0) <= 1e-12 * v0
    assert all(2 <= n <= 21 for n in s.sor_iters)


def _div(cfg, u, v, w):
    dxi, dyi, dzi = 1 / cfg.dx, 1 / cfg.dy, 1 / cfg.dz
    ui, vi, wi = (a[3:-3, 3:-3, 3:-3] for a in (u, v, w))
    um = u[3:-3, 3:-3, 2:-4]
    vm = v[3:-3, 2:-4, 3:-3]
    wm = w[2:-4, 3:-3, 3:-3]
    return (ui - um) * dxi + (vi - vm) * dyi + (wi - wm) * dzi


def test_projection_removes_divergence(orc):
    """After corunp_explicit the discrete divergence (caldiv.f:30-41 stencil) of the
    new velocity is at round-off, while the predictor's (err_div0) is not."""
    cfg = C.get("couette32")
    s, st = _run(orc, cfg, 5)
    d = _div(cfg, st[0], st[1], st[2])
    umax = np.abs(C.interior(st[0])).max()
    assert np.abs(d).max() <= 1e-9 * umax / cfg.dx
    assert s.diag[-1][0] > 1e3 * np.abs(d).max() * cfg.dt ** -1 * cfg.dt


def test_single_phase_slip_couette_is_steady(orc):
    """Single fluid (phi=0), Navier-slip walls moving at -/+uwall: the linear profile
    u = A + B y with u - ls du/dy = -uwall at y=0 and u + ls du/dy = uwall at y=yl is an
    exact discrete steady state of the step (bndu.f:39-57 ghosts, WENO5 and the
    viscous operator are exact on it)."""
    cfg = C.Config("couette_sp", 16, 16, 8, 1.0, 1.0, 1.0, dt=1e-3, steps=1, uwall=0.5, slip=0.05,
                   init="stripe")
    s = orc.Solver(cfg)
    st = C.raw_state(cfg)
    st[8:] = 0.0
    ls = cfg.slip
    B = 2 * cfg.uwall / (cfg.yl + 2 * ls)
    A = -cfg.uwall + ls * B
    y = (np.arange(-2, cfg.nj + 4) - 0.5) * cfg.dy
    prof = (A + B * y)[None, :, None]
    st[0][:] = prof
    st[3][:] = prof
    th, ze, l1, l2 = s.walls
    lib = orc.lib()
    lib.orc_init_bc(s.ws, s._ptrs(st), orc.P(th), orc.P(ze), orc.P(l1), orc.P(l2))
    u0 = st[0].copy()
    s.step(st, 3)
    assert np.abs(C.interior(st[0]) - C.interior(u0)).max() <= 1e-12
    assert np.abs(C.interior(st[1])).max() <= 1e-12
    assert np.abs(C.interior(st[2])).max() <= 1e-12


def test_poisson_residual_roundoff(orc):
    """solp_fft_tdma4: the FFT+TDMA solution satisfies the 7-point Poisson equation."""
    cfg = C.Config("p", 32, 16, 16, 2.0, 1.0, 1.0, dt=1e-3, steps=1)
    lib = orc.lib()
    rng = np.random.default_rng(5)
    n = cfg.ni * cfg.nj * cfg.nk
    div = np.zeros(cfg.shape)
    d = rng.normal(size=(cfg.nk, cfg.nj, cfg.ni))
    d -= d.mean()
    div[3:-3, 3:-3, 3:-3] = d
    pr, pi = np.zeros(n), np.zeros(n)
    fft = np.zeros(2 * n)
    I, D, P = orc.I, orc.D, orc.P
    lib.orc_solp_fft_tdma1(I(cfg.ni), I(cfg.nj), I(cfg.nk), P(fft), P(div), P(pr), P(pi))
    nj6 = cfg.nj + 6
    arr = [np.zeros(nj6) for _ in range(7)]
    f3 = [np.zeros(nj6) for _ in range(3)]
    rho = 1.0
    lib.orc_cal_coef_prs(I(cfg.nj), D(rho), D(1 / cfg.dx), D(1 / cfg.dy), D(1 / cfg.dz), *[P(a) for a in arr])
    lib.orc_cal_coef_solp_fft(I(cfg.nj), P(arr[2]), P(arr[3]), *[P(a) for a in f3])
    sv = orc.IA([cfg.ni, cfg.nj, cfg.nk])
    lib.orc_solp_fft_tdma2(I(0), I(1), sv, D(rho), D(1 / cfg.dx), D(1 / cfg.dz), *[P(a) for a in f3], None, None,
                           None, P(pr), P(pi))
    dp = np.zeros(cfg.shape)
    lib.orc_solp_fft_tdma3(I(cfg.ni), I(cfg.nj), I(cfg.nk), P(fft), P(pr), P(pi), P(dp))
    nid = orc.IA(orc.NID)
    lib.orc_bnd_avzero(I(0), I(1), I(cfg.ni), I(cfg.nj), I(cfg.nk), P(dp))
    lib.orc_bnd_neumann(nid, I(cfg.ni), I(cfg.nj), I(cfg.nk), P(dp))
    lib.orc_bnd_periodic(I(cfg.ni), I(cfg.nj), I(cfg.nk), P(dp))
    e = (ctypes.c_double * 1)()
    e0 = (ctypes.c_double * 1)()
    lib.orc_solp_fft_tdma4_v(I(cfg.ni), I(cfg.nj), I(cfg.nk), D(rho), D(1 / cfg.dx), D(1 / cfg.dy), D(1 / cfg.dz),
                             P(div), P(dp), e, e0)
    assert e[0] / e0[0] < 1e-12
