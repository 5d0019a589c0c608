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
    """The FFT+TDMA solution (solp_fft_tdma1-3 with cal_coef_prs/cal_coef_solp_fft)
    satisfies the 7-point Poisson equation: by the reference's own monitor
    (solp_fft_tdma4), and by the operator written here in numpy (periodic in x and z,
    closed wall faces at j = 1 and nj), to 1e-11 of the right-hand side (measured
    8e-16; a periodic y operator misses by 0.57)."""
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
    # the same equation written here: the 7-point operator over rho, periodic in x
    # and z, the wall faces closed at j = 1 and j = nj (cal_coef_prs.f's fold), on the
    # interior of dp, against the right-hand side
    q = dp[3:-3, 3:-3, 3:-3]
    lap = (np.roll(q, -1, 2) - 2 * q + np.roll(q, 1, 2)) / cfg.dx ** 2
    lap += (np.roll(q, -1, 0) - 2 * q + np.roll(q, 1, 0)) / cfg.dz ** 2
    up = np.zeros_like(q)
    up[:, :-1, :] = q[:, 1:, :] - q[:, :-1, :]  # (j+1) - j, closed at j = nj
    dn = np.zeros_like(q)
    dn[:, 1:, :] = q[:, 1:, :] - q[:, :-1, :]  # j - (j-1), closed at j = 1
    lap += (up - dn) / cfg.dy ** 2
    assert np.abs(lap / rho - d).max() <= 1e-11 * np.abs(d).max()


def _grads_p2a(orc, cfg, phi):
    I, D, P = orc.I, orc.D, orc.P
    g = [np.zeros(cfg.shape) for _ in range(3)]
    dya = np.full(cfg.nj + 6, 1.0 / cfg.dy)
    orc.lib().orc_cal_grad_p2a(I(0), I(cfg.nj), I(cfg.ni), I(cfg.nj), I(cfg.nk), D(1 / cfg.dx), P(dya),
                               D(1 / cfg.dz), P(phi), *[P(a) for a in g])
    return g


def test_mthinc_planar_interface_flux(orc):
    """solphi_mthinc1.f:56-282 on a planar interface normal to x (phi a function of x
    only) advected at a constant u > 0.  The vertex gradients have no y or z part,
    so the unit normal is (s, 0, 0), s = +-1, and the 8 Gauss points of the
    reconstruction H(t) = 1/(1 + exp(-2 beta t)), t = n.x + d, fall on 2 along x:
    the offset d solves (H(s x1 + d) + H(s x2 + d))/2 = phi_cell with x1,2 = -+1/(2
    sqrt 3) (found here by bisection, independently of the oracle's Newton
    iteration), and the flux through the east face is c (H(s g1 + d) + H(s g2 + d))/2
    with c = u dt/dx and g1,2 the 2-point Gauss nodes of [1/2 - c, 1/2].  Outside the
    band (mean gradient <= eps dcellinv) it is c phi with phi snapped to 0/1 within
    eps_trunc of them."""
    cfg = C.Config("planar", 32, 8, 8, 1.0, 0.25, 0.25, dt=1e-3, steps=1)
    sh = cfg.shape
    bet, u0 = 2.0, 0.4
    dt = 0.2 * cfg.dx / u0
    c = u0 * dt / cfg.dx
    xc = (np.arange(-2, cfg.ni + 4) - 0.5) * cfg.dx
    prof = 0.5 * (1.0 + np.tanh((xc - 0.503) / (1.5 * cfg.dx)))
    phi = np.broadcast_to(prof[None, None, :], sh).copy()
    gx, gy, gz = _grads_p2a(orc, cfg, phi)
    # rounding-level y, z parts (the reference sums differences in its own order)
    assert np.abs(gy).max() <= 1e-12 * np.abs(gx).max() and np.abs(gz).max() <= 1e-12 * np.abs(gx).max()
    u = np.full(sh, u0)
    v = np.zeros(sh)
    w = np.zeros(sh)
    fl = [np.zeros(sh) for _ in range(3)]
    I, D, P = orc.I, orc.D, orc.P
    orc.lib().orc_solphi_mthinc1(I(cfg.ni), I(cfg.nj), I(cfg.nk), D(1 / cfg.dx), D(1 / cfg.dy), D(1 / cfg.dz),
                                 D(dt), D(bet), P(phi), P(gx), P(gy), P(gz), P(u), P(v), P(w), *[P(a) for a in fl])
    H = lambda t: 1.0 / (1.0 + np.exp(-2.0 * bet * t))
    gp = 0.5 / np.sqrt(3.0)
    dx, dy, dz = cfg.dx, cfg.dy, cfg.dz
    dcellinv = 1.0 / np.sqrt((dx * dx + dy * dy + dz * dz) / 3.0)
    eps = bet / (2.0 * np.cosh(-bet * 1.5) ** 2)
    eps_trunc = 0.5 * (np.tanh(-bet * 2.5) + 1.0)
    k0, j0 = 4 + 2, 3 + 2
    nband = 0
    for i in range(0, cfg.ni + 2):
        ix = i + 2
        # mean of the 8 vertex gradients around the cell (all equal in y and z)
        rn = 0.5 * (gx[k0, j0, ix - 1] + gx[k0, j0, ix])
        p0 = phi[k0, j0, ix]
        got = fl[0][k0, j0, ix]
        if abs(rn) <= eps * dcellinv:
            ph = 0.0 if p0 <= eps_trunc else (1.0 if 1.0 - p0 <= eps_trunc else p0)
            want = u0 * ph * dt / dx
        else:
            nband += 1
            s = np.sign(rn)
            lo, hi = -50.0, 50.0
            for _ in range(200):
                mid = 0.5 * (lo + hi)
                if 0.5 * (H(-s * gp + mid) + H(s * gp + mid)) < p0:
                    lo = mid
                else:
                    hi = mid
            d = 0.5 * (lo + hi)
            a, b = 0.5 - c, 0.5
            g1, g2 = 0.5 * (a + b) - (b - a) * gp, 0.5 * (a + b) + (b - a) * gp
            want = 0.5 * c * (H(s * g1 + d) + H(s * g2 + d))
        assert abs(got - want) <= 1e-12 * max(abs(want), 1e-3), (i, got, want)
    assert nband >= 4


def test_gnbc_known_answers(orc):
    """gnbc.f90:24-97: with the fluid at rest on resting walls the dynamic angle is
    the static one, up to the law's regularisation (|u_cl| = sqrt(0 + 1e-12)); with
    a uniform x-velocity U it is acos(cos theta0 -+ zeta sqrt(U^2 + 1e-12)/sigma),
    the sign flipped for i <= ni/2, clamped to [-1, 1]."""
    cfg = C.get("couette32", ni=16, nj=8, nk=8, theta_lo=60.0, theta_hi=110.0)
    th0, ze, l1, l2 = C.wall_arrays(cfg)
    sh = cfg.shape
    sigma, zeta = 0.7, ze[3, 3, 3]
    I, D, P = orc.I, orc.D, orc.P
    ii = np.arange(-2, cfg.ni + 4)
    for U in (0.0, 0.35, 30.0):  # at rest, a moderate speed, a speed that saturates the clamp
        u = np.full(sh, U)
        w = np.zeros(sh)
        theta = np.zeros(sh)
        orc.lib().orc_gnbc(orc.IA([-1] * 6), I(cfg.ni), I(cfg.nj), I(cfg.nk), P(u), P(w), D(0.0), P(th0),
                           D(sigma), P(ze), P(theta))
        for jw, sgn_wall in ((1, 1.0), (cfg.nj, 1.0)):
            ucl = np.sqrt(U * U + 1e-12) * sgn_wall * np.where(ii <= cfg.ni // 2, -1.0, 1.0)
            cos_t = np.clip(np.cos(np.radians(th0[:, jw + 2, :])) - zeta * ucl[None, :] / sigma, -1.0, 1.0)
            want = np.degrees(np.arccos(cos_t))
            np.testing.assert_allclose(theta[:, jw + 2, :], want, rtol=0, atol=1e-10)
        if U == 0.0:
            np.testing.assert_allclose(theta[:, 3, :], th0[:, 3, :], rtol=0, atol=1e-4)


def test_bnd_contact_angle_known_answers(orc):
    """bnd_contact_angle.f90:25-85 on fields with closed-form ghosts, unequal
    spacings and a different static angle in every wall cell:
    * a field linear in i and k, q = q0 + a i + b j + c k: the wall normal
      (sg sin(theta) dy/dx, cos(theta), sg sin(theta) dy/dz) (sg = +1 for
      i >= ni/2, else -1) turns the centred x and z differences into the ghost
      q(j=0) = q(j=1) - sg cot(theta) (a + c) (and q(nj+1) = q(nj) - ... at the upper
      wall), and the two outer ghosts continue linearly;
    * theta = 90 deg: every ghost is the first interior value, for any field;
    * a field that varies in j only: the same, for any angle;
    * the columns i = -2, ni+3 and planes k = -2, nk+3, which the reference's
      stencil would read out of bounds, are left as they were (every call site
      refills them with bnd_periodic)."""
    ni, nj, nk = 16, 8, 8
    dx, dy, dz = 0.1, 0.05, 0.2
    sh = (nk + 6, nj + 6, ni + 6)
    rng = np.random.default_rng(5)
    kk, jj, ii = np.meshgrid(np.arange(-2, nk + 4), np.arange(-2, nj + 4), np.arange(-2, ni + 4), indexing="ij")
    theta = rng.uniform(35.0, 145.0, sh)
    sg = np.where(np.arange(-1, ni + 3) - ni // 2 >= 0, 1.0, -1.0)[None, :]
    I, D, P = orc.I, orc.D, orc.P

    def run(q, th):
        q = np.ascontiguousarray(q.copy())
        orc.lib().orc_bnd_contact_angle(orc.IA([-1] * 6), I(ni), I(nj), I(nk), P(q), P(th), D(dx), D(dy), D(dz))
        return q

    a, b, c = 0.3, 0.11, -0.7
    q = 0.5 + a * ii + b * jj + c * kk
    got = run(q, theta)
    inner = (slice(1, nk + 5), slice(1, ni + 5))  # k, i in -1 .. n+2
    for jw, ghosts in ((1, (0, -1, -2)), (nj, (nj + 1, nj + 2, nj + 3))):
        cot = 1.0 / np.tan(np.radians(theta[:, jw + 2, :][inner]))
        step = -sg * cot * (a + c)  # q(ghost 1) - q(wall row)
        q1 = q[:, jw + 2, :][inner]
        for m, jg in enumerate(ghosts, start=1):
            np.testing.assert_allclose(got[:, jg + 2, :][inner], q1 + m * step, rtol=0, atol=1e-12)
    # D2: the outermost columns and planes keep their values
    for jg in (0, -1, -2, nj + 1, nj + 2, nj + 3):
        assert np.array_equal(got[:, jg + 2, 0], q[:, jg + 2, 0]) and np.array_equal(got[:, jg + 2, -1], q[:, jg + 2, -1])
        assert np.array_equal(got[0, jg + 2, :], q[0, jg + 2, :]) and np.array_equal(got[-1, jg + 2, :], q[-1, jg + 2, :])
    # 90 degrees, any field; a field that varies in j only, any angle
    for field, th in ((rng.standard_normal(sh), np.full(sh, 90.0)), (np.sin(0.7 * jj) + 0.0 * ii, theta)):
        got = run(field, th)
        for jw, ghosts in ((1, (0, -1, -2)), (nj, (nj + 1, nj + 2, nj + 3))):
            for jg in ghosts:
                np.testing.assert_allclose(got[:, jg + 2, :][inner], field[:, jw + 2, :][inner], rtol=0, atol=1e-13)


def test_bndu_navier_slip_law(orc):
    """bndu.f:29-97: at both walls the first ghost of u satisfies the discrete
    Navier-slip law at the wall face, (u_ghost + u_wall_row)/2 - U = ls (du/dn)
    with du/dn the one-cell difference into the fluid, U = -uwall at the lower and
    +uwall at the upper wall, and ls = 1/(phi_bar/l1 + (1 - phi_bar)/l2), phi_bar
    the mean of phi over the two cells beside the u point; w the same law with U = 0
    (and the u point's slip length, as the reference has it); v vanishes on the wall
    face and is odd about it; the outer ghosts of u and w continue linearly.
    Checked on the interior columns (the x and z halos are refilled afterwards) with
    random fields, phi in [0, 1] and l1 != l2."""
    ni, nj, nk = 16, 8, 8
    dy, uwall = 0.05, 0.8
    sh = (nk + 6, nj + 6, ni + 6)
    rng = np.random.default_rng(9)
    u, v, w = (rng.standard_normal(sh) for _ in range(3))
    phi = rng.uniform(0.0, 1.0, sh)
    l1, l2 = rng.uniform(0.01, 0.2, sh), rng.uniform(0.3, 2.0, sh)
    u0, v0, w0 = u.copy(), v.copy(), w.copy()
    I, D, P = orc.I, orc.D, orc.P
    orc.lib().orc_bndu(orc.IA([-1] * 6), I(ni), I(nj), I(nk), P(u), P(v), P(w), D(uwall), D(dy), P(l1), P(l2),
                       P(phi))
    K, Ii = slice(3, nk + 3), slice(3, ni + 3)  # k, i in 1 .. n
    for jw, jg, sgn, U in ((1, 0, 1.0, -uwall), (nj, nj + 1, -1.0, uwall)):
        pb = 0.5 * (phi[K, jw + 2, Ii] + phi[K, jw + 2, 4:ni + 4])
        ls = 1.0 / (pb / l1[K, jw + 2, Ii] + (1.0 - pb) / l2[K, jw + 2, Ii])
        for q, Uw in ((u, U), (w, 0.0)):
            qw, qg = q[K, jw + 2, Ii], q[K, jg + 2, Ii]
            lhs = 0.5 * (qg + qw) - Uw
            rhs = ls * (qw - qg) / dy  # into the fluid: (wall row - ghost) / dy at either wall
            np.testing.assert_allclose(lhs, rhs, rtol=0, atol=1e-12 * (1 + np.abs(rhs).max()))
            # outer ghosts linear
            step = qg - qw
            for m in (2, 3):
                jo = jw - sgn * m  # j = -1, -2 below, nj + 2, nj + 3 above
                np.testing.assert_allclose(q[K, int(jo) + 2, Ii], qw + m * step, rtol=0, atol=1e-12)
    # v: zero on the wall face, odd about it
    assert np.all(v[K, 2, Ii] == 0.0) and np.all(v[K, nj + 2, Ii] == 0.0)
    for m in (1, 2):
        np.testing.assert_array_equal(v[K, 2 - m, Ii], -v0[K, 2 + m, Ii])
    for m in (1, 2, 3):
        np.testing.assert_array_equal(v[K, nj + 2 + m, Ii], -v0[K, nj + 2 - m, Ii])
    # the interior is untouched
    sl = (K, slice(3, nj + 2), Ii)
    assert np.array_equal(u[sl], u0[sl]) and np.array_equal(w[sl], w0[sl]) and np.array_equal(v[sl], v0[sl])


def test_explicit_viscous_term_known_answers(orc):
    """calsij.f:28-139, cal_arith_tau.f:21-117 and cal_div_tensor.f:20-86 chained
    (the explicit term div(2 mu S) of main.f90:538-541) on fields where the
    staggered second-order differences are exact, with unequal spacings:
    * constant mu, quadratic u, v, w: div(2 mu S) = mu (lap u + grad div u), a
      constant per component (u: mu (2 Axx + 2 Ayy + 2 Azz + 2 Axx + Bxy + Cxz) for
      u = ... + Axx x^2 + Axy x y + ..., v and w with coefficients B and C);
    * linear mu, linear u, v, w (S constant): div(2 mu S) = 2 S grad mu, a constant
      (the four-cell edge means of a linear mu are its values on the edges).
    Checked at the interior u, v, w points to 1e-9 of the largest term."""
    ni, nj, nk = 16, 8, 12
    dx, dy, dz = 0.11, 0.07, 0.23
    sh = (nk + 6, nj + 6, ni + 6)
    kk, jj, ii = np.meshgrid(np.arange(-2, nk + 4), np.arange(-2, nj + 4), np.arange(-2, ni + 4), indexing="ij")
    x, y, z = ii * dx, jj * dy, kk * dz
    I, D, P = orc.I, orc.D, orc.P
    inner = (slice(3, nk + 3), slice(3, nj + 3), slice(3, ni + 3))

    def chain(u, v, w, mu):
        sk = np.zeros((6,) + sh)
        tau = np.zeros((6,) + sh)
        out = [np.zeros(sh) for _ in range(3)]
        orc.lib().orc_calsij(I(ni), I(nj), I(nk), D(1 / dx), D(1 / dy), D(1 / dz), P(u), P(v), P(w), P(sk))
        orc.lib().orc_cal_arith_tau(I(ni), I(nj), I(nk), P(sk), P(mu), P(tau))
        orc.lib().orc_cal_div_tensor(I(ni), I(nj), I(nk), D(1 / dx), D(1 / dy), D(1 / dz), P(tau), *[P(o) for o in out])
        return out

    rng = np.random.default_rng(13)
    keys = ("xx", "yy", "zz", "xy", "xz", "yz", "x", "y", "z", "c")
    A, B, C = ({k: rng.uniform(-1, 1) for k in keys} for _ in range(3))

    def quad(c):
        return (c["xx"] * x * x + c["yy"] * y * y + c["zz"] * z * z + c["xy"] * x * y + c["xz"] * x * z
                + c["yz"] * y * z + c["x"] * x + c["y"] * y + c["z"] * z + c["c"])

    mu0 = 0.37
    got = chain(quad(A), quad(B), quad(C), np.full(sh, mu0))
    want = (mu0 * (4 * A["xx"] + 2 * A["yy"] + 2 * A["zz"] + B["xy"] + C["xz"]),
            mu0 * (2 * B["xx"] + 4 * B["yy"] + 2 * B["zz"] + A["xy"] + C["yz"]),
            mu0 * (2 * C["xx"] + 2 * C["yy"] + 4 * C["zz"] + A["xz"] + B["yz"]))
    for g, w_ in zip(got, want):
        np.testing.assert_allclose(g[inner], w_, rtol=0, atol=1e-9 * max(abs(x) for x in want))

    # linear mu and velocities
    m = {"x": 0.3, "y": -0.2, "z": 0.45}
    mu = 2.0 + m["x"] * x + m["y"] * y + m["z"] * z
    lin = [{k: rng.uniform(-1, 1) for k in ("x", "y", "z", "c")} for _ in range(3)]
    vel = [L["x"] * x + L["y"] * y + L["z"] * z + L["c"] for L in lin]
    got = chain(*vel, mu)
    grad = [[lin[a][b] for b in ("x", "y", "z")] for a in range(3)]  # grad[a][b] = d u_a / d x_b
    gm = (m["x"], m["y"], m["z"])
    want = [sum((grad[a][b] + grad[b][a]) * gm[b] for b in range(3)) for a in range(3)]
    for g, w_ in zip(got, want):
        np.testing.assert_allclose(g[inner], w_, rtol=0, atol=1e-9 * max(abs(x) for x in want))


@pytest.mark.parametrize("N", [32, 64])
def test_csf_curvature_of_a_sphere(orc, N):
    """calrn.f + calrkap.f on a resolved sphere of radius R = 0.25 (phi = 1 inside,
    a tanh profile of width 1.5 cells): the curvature at the u points, weighted by
    the face gradient |phi(i+1) - phi(i)| that multiplies it in calfst.f, is the
    sphere's -2/R (normals point into the phi = 1 fluid) to within the
    discretisation error, and that error falls as the grid is refined."""
    cfg = C.Config("sphere", N, N, N, 1.0, 1.0, 1.0, dt=1e-3, steps=1)
    sh = cfg.shape
    x = (np.arange(-2, N + 4) - 0.5) / N
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    R = 0.25
    r = np.sqrt((X - 0.501) ** 2 + (Y - 0.497) ** 2 + (Z - 0.5) ** 2)
    phi = 0.5 * (1.0 + np.tanh((R - r) / (1.5 / N)))
    gx, gy, gz = _grads_p2a(orc, cfg, phi)
    I, D, P = orc.I, orc.D, orc.P
    dxi = float(N)
    rns = []
    for ip, jp, kp in ((1, 1, 1), (0, 0, 1), (0, 1, 0), (1, 0, 0)):
        rn = np.zeros((3,) + sh)
        orc.lib().orc_calrn(I(N), I(N), I(N), D(dxi), D(dxi), D(dxi), I(ip), I(jp), I(kp), P(gx), P(gy), P(gz), P(rn))
        rns.append(rn)
    kap = np.zeros((3,) + sh)
    orc.lib().orc_calrkap(I(N), I(N), I(N), D(dxi), D(dxi), D(dxi), *[P(a) for a in rns], P(kap))
    ku = C.interior(kap[0])
    wgt = np.abs(C.interior(np.roll(phi, -1, axis=2) - phi))
    mean = float((ku * wgt).sum() / wgt.sum())
    err = abs(mean * R / 2.0 + 1.0)
    test_csf_curvature_of_a_sphere.errs[N] = err
    assert err <= 0.05, (N, mean, -2.0 / R)
    if 32 in test_csf_curvature_of_a_sphere.errs and 64 in test_csf_curvature_of_a_sphere.errs:
        assert test_csf_curvature_of_a_sphere.errs[64] < test_csf_curvature_of_a_sphere.errs[32]


test_csf_curvature_of_a_sphere.errs = {}


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_weno5_fifth_order_on_a_smooth_field(orc, axis, sign):
    """weno5.h on a smooth monotone field q = sign * exp(x/2) along one axis (the
    component of that axis, the others zero; every halo point filled with the exact
    function): the advection term divided by the discrete advecting velocity of
    cal_advu_weno5.f ((q(i-1) + 2 q(i) + q(i+1))/4) is the upwind-biased WENO5
    derivative, which converges to dq/dx at fifth order where the field has no
    critical point.  Checked on 16, 32 and 64 cells (each halving the error about
    32-fold) on both upwind sides and every axis."""
    errs = []
    for n in (16, 32, 64):
        dims = [8, 8, 8]
        dims[axis] = n
        ni, nj, nk = dims
        h = 1.0 / n
        sh = (nk + 6, nj + 6, ni + 6)
        x = (np.arange(-2, n + 4, dtype=np.float64)) * h
        f = sign * np.exp(0.5 * x)
        bshape = [1, 1, 1]
        bshape[2 - axis] = n + 6
        fields = [np.zeros(sh) for _ in range(3)]
        fields[axis] = np.broadcast_to(f.reshape(bshape), sh).copy()
        out = [np.zeros(sh) for _ in range(3)]
        d = [1.0, 1.0, 1.0]
        d[axis] = 1.0 / h
        orc.lib().orc_cal_advu_weno5(orc.I(ni), orc.I(nj), orc.I(nk), orc.D(d[0]), orc.D(d[1]), orc.D(d[2]),
                                     *[orc.P(a) for a in fields], *[orc.P(a) for a in out])
        line = [slice(3, 4)] * 3
        line[2 - axis] = slice(3, n + 3)
        adv = out[axis][tuple(line)].ravel()
        fi = f[3:n + 3]
        vel = ((f[2:n + 2] + fi) * 0.5 + (fi + f[4:n + 4]) * 0.5) * 0.5
        exact = 0.5 * fi
        errs.append(np.abs(adv / vel - exact).max())
        for q in range(3):
            if q != axis:
                assert np.all(out[q] == 0.0)
    orders = [np.log2(errs[t] / errs[t + 1]) for t in range(2)]
    assert min(orders) >= 4.5, (errs, orders)
    assert errs[-1] <= 1e-9, errs


def test_viscous_solve_fixed_point_is_the_staggered_stress_divergence(orc):
    """cal_arith_coef_vis + solu_sor4, run to round-off (stop rule 1e-300, 200 outer
    iterations), solve  q/dt - (0.5/rho) div(tau)_h(q) = src  for (u, v, w), with
    div(tau)_h the staggered-grid stress divergence written here from its
    definition: normal stresses 2 mu dq_i/dx_i at cell centres, shear stresses
    mu_e (du_i/dx_j + du_j/dx_i) on the cell edges with mu_e the mean of the four
    cells around the edge.  Smoothly varying viscosity, uniform density, unequal dx,
    dy, dz; checked at every point whose stencil stays off the wall ghosts (x and
    z periodic), to 1e-12 of the largest source."""
    import ctypes

    ni, nj, nk = 16, 16, 8
    lx, ly, lz = 2.0, 1.0, 0.75
    dx, dy, dz = lx / ni, ly / nj, lz / nk
    dt, rho0 = 2e-3, 2.0
    sh = (nk + 6, nj + 6, ni + 6)
    k3, j3, i3 = np.meshgrid(np.arange(-2, nk + 4), np.arange(-2, nj + 4), np.arange(-2, ni + 4), indexing="ij")
    xc, yc, zc = (i3 - 0.5) * dx, (j3 - 0.5) * dy, (k3 - 0.5) * dz
    mu = 0.05 * (1.0 + 0.3 * np.sin(2 * np.pi * xc / lx) * np.cos(2 * np.pi * zc / lz) + 0.2 * yc)
    rho = np.full(sh, rho0)
    src = [np.sin(2 * np.pi * xc / lx + 0.3 * q) * np.cos(2 * np.pi * zc / lz) * (1.0 + yc) for q in range(3)]
    u, v, w = np.zeros(sh), np.zeros(sh), np.zeros(sh)
    l1, l2, phi = np.full(sh, 0.1), np.full(sh, 0.1), np.zeros(sh)
    I, D, P = orc.I, orc.D, orc.P
    coef = [np.zeros(sh) for _ in range(45)]
    parr = (ctypes.POINTER(ctypes.c_double) * 45)(*[P(c) for c in coef])
    L = orc.lib()
    L.orc_cal_arith_coef_vis_v(I(ni), I(nj), I(nk), D(1 / dx), D(1 / dy), D(1 / dz), P(mu), parr, ctypes.c_int(0))
    L.orc_set_sor.argtypes = [ctypes.c_double, ctypes.c_int]
    L.orc_set_sor(1e-300, 200)
    try:
        err = ctypes.c_double()
        L.orc_solu_sor4_v(orc.IA(orc.NID), I(ni), I(nj), I(nk), D(dt), P(rho), P(rho), parr, P(src[0]), P(src[1]),
                          P(src[2]), P(u), P(v), P(w), D(0.0), D(dy), P(l1), P(l2), P(phi), ctypes.byref(err))
    finally:
        L.orc_set_sor(1e-3, 21)

    def at(a, di=0, dj=0, dk=0):  # a[i+di, j+dj, k+dk] over i, j, k = 1..n (the interior block)
        return a[3 + dk:3 + dk + nk, 3 + dj:3 + dj + nj, 3 + di:3 + di + ni]

    m = lambda di=0, dj=0, dk=0: at(mu, di, dj, dk)
    exy = lambda di=0, dj=0: (m(di, dj) + m(di + 1, dj) + m(di, dj + 1) + m(di + 1, dj + 1)) / 4
    exz = lambda di=0, dk=0: (m(di, 0, dk) + m(di + 1, 0, dk) + m(di, 0, dk + 1) + m(di + 1, 0, dk + 1)) / 4
    eyz = lambda dj=0, dk=0: (m(0, dj, dk) + m(0, dj + 1, dk) + m(0, dj, dk + 1) + m(0, dj + 1, dk + 1)) / 4
    # shear stresses on the edges (i+1/2, j+1/2), (i+1/2, k+1/2), (j+1/2, k+1/2) of cell (i, j, k)
    txy = lambda di=0, dj=0: exy(di, dj) * ((at(u, di, dj + 1) - at(u, di, dj)) / dy +
                                            (at(v, di + 1, dj) - at(v, di, dj)) / dx)
    txz = lambda di=0, dk=0: exz(di, dk) * ((at(u, di, 0, dk + 1) - at(u, di, 0, dk)) / dz +
                                            (at(w, di + 1, 0, dk) - at(w, di, 0, dk)) / dx)
    tyz = lambda dj=0, dk=0: eyz(dj, dk) * ((at(v, 0, dj, dk + 1) - at(v, 0, dj, dk)) / dz +
                                            (at(w, 0, dj + 1, dk) - at(w, 0, dj, dk)) / dy)
    # normal stresses at cell centres
    txx = lambda di=0: 2 * m(di) * (at(u, di) - at(u, di - 1)) / dx
    tyy = lambda dj=0: 2 * m(0, dj) * (at(v, 0, dj) - at(v, 0, dj - 1)) / dy
    tzz = lambda dk=0: 2 * m(0, 0, dk) * (at(w, 0, 0, dk) - at(w, 0, 0, dk - 1)) / dz
    div = [(txx(1) - txx(0)) / dx + (txy(0, 0) - txy(0, -1)) / dy + (txz(0, 0) - txz(0, -1)) / dz,
           (txy(0, 0) - txy(-1, 0)) / dx + (tyy(1) - tyy(0)) / dy + (tyz(0, 0) - tyz(0, -1)) / dz,
           (txz(0, 0) - txz(-1, 0)) / dx + (tyz(0, 0) - tyz(-1, 0)) / dy + (tzz(1) - tzz(0)) / dz]
    scale = max(np.abs(at(s)).max() for s in src)
    # points whose stencils stay off the wall ghosts (j = 0, nj + 1) and the walls'
    # v, and off the x and z halos: bndu.f refreshes every component's halos
    # shifted by one cell before the periodic copy of the swept one only, so the
    # other components' halos differ between the sweeps that read them and the end
    # of the solve
    rows = {0: slice(1, nj - 1), 1: slice(1, nj - 2), 2: slice(1, nj - 1)}
    for q, fld in enumerate((u, v, w)):
        res = at(fld) / dt - 0.5 / rho0 * div[q] - at(src[q])
        r = np.abs(res[1:nk - 1, rows[q], 1:ni - 1]).max()
        assert r <= 1e-12 * scale, (q, r, scale)
    assert np.abs(at(v)).max() > 0.0 and np.abs(at(w)).max() > 0.0  # the coupling is exercised
