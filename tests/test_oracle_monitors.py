"""Pins of the oracle's run-time monitors (no GPU): cal_vel.f, cal_center.f and
find_interface_positions_upper.f90 against numpy restatements and known answers
(a uniform velocity, a box of phi with a known centre, a blob carried across the
periodic x boundary), and the adjoint's objective find_interface_positions_lower
on wall rows whose contact-line positions are known exactly."""
import ctypes

import numpy as np

NI, NJ, NK = 16, 8, 8
SH = (NK + 6, NJ + 6, NI + 6)
INT = (slice(3, NK + 3), slice(3, NJ + 3), slice(3, NI + 3))


def _vel(orc, u, v, w, phi, radius=0.25, rhol=2.0, rmul=0.1):
    I, D, P = orc.I, orc.D, orc.P
    vel, re = np.zeros(3), np.zeros(3)
    orc.lib().orc_cal_vel(I(0), I(NI), I(NJ), I(NK), D(radius), D(rhol), D(rmul), P(u), P(v), P(w), P(phi),
                          P(vel), P(re))
    return vel, re


def test_cal_vel_matches_numpy(orc):
    rng = np.random.default_rng(3)
    u, v, w = (rng.normal(size=SH) for _ in range(3))
    phi = rng.random(SH)
    vel, re = _vel(orc, u, v, w, phi)
    p = phi[INT]
    ref = np.array([(p * q[INT]).sum() / p.sum() for q in (u, v, w)])
    assert np.allclose(vel, ref, rtol=1e-13, atol=0)
    assert np.allclose(re, 2.0 * ref * 0.5 / 0.1, rtol=1e-13, atol=0)


def test_cal_vel_uniform_velocity(orc):
    rng = np.random.default_rng(4)
    phi = rng.random(SH)
    vel, _ = _vel(orc, np.full(SH, 0.3), np.full(SH, -0.2), np.full(SH, 0.0), phi)
    assert np.allclose(vel, [0.3, -0.2, 0.0], rtol=1e-14, atol=1e-16)


class Center:
    """The cal_center state of one caller, advanced through the oracle."""

    def __init__(self, orc, xl, yl, svall=NJ):
        self.orc, self.xl, self.yl, self.svall = orc, xl, yl, svall
        self.pre1, self.pre2 = ctypes.c_double(0.0), ctypes.c_double(0.0)
        self.a1, self.a2, self.lap = ctypes.c_int(2), ctypes.c_int(2), ctypes.c_int(0)

    def __call__(self, phi, dt=0.1):
        I, D, P = self.orc.I, self.orc.D, self.orc.P
        c, vel = np.zeros(3), ctypes.c_double()
        self.orc.lib().orc_cal_center(I(0), I(0), I(self.svall), I(NI), I(NJ), I(NK), D(self.xl), D(self.yl),
                                      D(1.0), D(dt), D(1.0), P(phi), P(c), ctypes.byref(self.pre1),
                                      ctypes.byref(self.pre2), ctypes.byref(self.a1), ctypes.byref(self.a2),
                                      ctypes.byref(self.lap), ctypes.byref(vel))
        return c, vel.value


def box(i0, i1, j0, j1, k0, k1):
    """phi = 1 on the interior cells i0..i1 (periodic in i), j0..j1, k0..k1."""
    phi = np.zeros(SH)
    for i in range(i0, i1 + 1):
        ii = (i - 1) % NI + 1
        phi[k0 + 2:k1 + 3, j0 + 2:j1 + 3, ii + 2] = 1.0
    return phi


def test_cal_center_box(orc):
    delta = 1.0 / NJ  # yl = 1, svall = nj: cubic cells of 1/8
    xl = NI * delta
    st = Center(orc, xl, 1.0)
    c, _ = st(box(5, 8, 2, 5, 3, 6))  # cell centres (i - 0.5) delta: means 6, 3, 4 cells
    assert np.allclose(c, [6.0 * delta, 3.0 * delta, 4.0 * delta], rtol=1e-14)
    assert st.a1.value == 2  # 0.8125 between xl/4 and 3xl/4


def test_cal_center_unwraps_across_the_periodic_boundary(orc):
    """A box moving in +x one cell per call: the centre grows monotonically through
    xl (unwrapped with area 3 -> 1 and lap), the velocity stays one cell per dt."""
    delta = 1.0 / NJ
    xl = NI * delta
    st = Center(orc, xl, 1.0)
    dt = 0.1
    prev = None
    for step in range(2 * NI):
        i0 = 3 + step
        c, vel = st(box(i0, i0 + 3, 2, 5, 3, 6), dt)
        expect = (i0 + 1.5 - 0.5) * delta  # mean of cell centres i0..i0+3, unwrapped
        assert abs(c[0] - expect) < 1e-12, (step, c[0], expect)
        if prev is not None:
            assert abs(vel - delta / dt) < 1e-10
        prev = c[0]
    assert st.lap.value >= 1


def _upper_numpy(phi, dx, dz, xl):
    out = []
    for k in range(1, NK + 1):
        for i in range(1, NI + 1):
            p1, p2 = phi[k + 2, NJ + 2, i + 2], phi[k + 2, NJ + 2, i + 3]
            if p1 > 0.5 and p2 < 0.5:
                out.append(((i - 0.5) * dx + (0.5 - p1) * dx / (p2 - p1) - xl * 0.75, (k - 0.5) * dz))
    return np.array(out).reshape(-1, 2)


def test_interface_upper_matches_numpy(orc):
    rng = np.random.default_rng(5)
    phi = rng.random(SH)
    I, D, P = orc.I, orc.D, orc.P
    cap = NI * NK
    xz = np.zeros(2 * cap)
    n = orc.lib().orc_interface_upper(I(NI), I(NJ), I(NK), P(phi), D(0.1), D(0.2), D(1.6), P(xz), ctypes.c_int(cap))
    ref = _upper_numpy(phi, 0.1, 0.2, 1.6)
    assert n == len(ref) > 0
    assert np.array_equal(xz[:2 * n].reshape(-1, 2), ref)
    # a short output buffer still gets the count
    assert orc.lib().orc_interface_upper(I(NI), I(NJ), I(NK), P(phi), D(0.1), D(0.2), D(1.6), P(xz),
                                         ctypes.c_int(1)) == n


def test_interface_lower_known_positions(orc):
    """find_interface_positions_lower.f90:15-32 (the adjoint's objective): on each
    wall row k of phi slice 0 (j = 1) a profile falling linearly through 0.5 at a
    chosen x0_k (cell centres at (i - 1/2) dx, clipped to [0, 1]) is found at x0_k
    exactly by the linear interpolation between the first pair of cells that
    brackets 0.5, less the reference's 0.75 xl shift; a row that never crosses
    counts as 0; J = -(mean over the rows).  Rows of the other j and the other
    slices do not enter."""
    dx, xl = 0.125, NI * 0.125
    rng = np.random.default_rng(21)
    phi = rng.random(SH)  # noise everywhere but the wall row
    x0 = 0.3 * xl + rng.uniform(-0.4, 0.4, NK) * dx * 3
    xc = (np.arange(-2, NI + 4) - 0.5) * dx
    want = []
    for k in range(NK):
        if k == 2:
            phi[k + 3, 3, :] = 1.0  # no crossing on this row
            want.append(0.0)
            continue
        slope = rng.uniform(0.1, 0.45) / dx  # the two bracketing cells stay inside [0, 1]
        phi[k + 3, 3, :] = np.clip(0.5 - slope * (xc - x0[k]), 0.0, 1.0)
        want.append(x0[k] - 0.75 * xl)
    J = orc.lib().orc_interface_lower(orc.I(NI), orc.I(NJ), orc.I(NK), orc.P(phi), orc.D(dx), orc.D(xl))
    assert abs(J - (-np.mean(want))) <= 1e-14, (J, -np.mean(want))
