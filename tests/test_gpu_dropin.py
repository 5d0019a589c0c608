"""Parity of every drop-in C-ABI routine (Fortran name, Fortran argument list,
host arrays) against the CPU oracle on identical seeded inputs.

The drop-in kernels are built without multiply-add contraction and follow the
reference's operation order, so arithmetic-only routines must agree to the last
bit up to reduction order; routines that call exp/cosh/tanh/cos/acos/sin agree
to a few ulp.  Tolerances (relative to the largest magnitude of the output):
EXACT = 1e-14, TRANSC = 1e-12.
"""
import ctypes

import numpy as np
import pytest

from fmf import config as C

pytestmark = pytest.mark.gpu

EXACT = 1e-14
TRANSC = 1e-12
NI, NJ, NK = 32, 16, 16


@pytest.fixture(scope="module")
def L(fmf_lib):
    from fmf import capi
    fmf_lib.fmf_set_mode(capi.FMF_COHERENT)
    fmf_lib.fmf_reset()
    yield fmf_lib
    fmf_lib.fmf_reset()
    fmf_lib.fmf_set_mode(capi.FMF_RESIDENT)


CFG = C.Config("dropin", NI, NJ, NK, 2.0, 1.0, 1.0, dt=1e-3, steps=1)
SH = CFG.shape
RNG = np.random.default_rng(42)


def field(scale=1.0, smooth=False):
    if smooth:
        z, y, x = np.meshgrid(*[np.linspace(0, 2 * np.pi, n) for n in SH], indexing="ij")
        return scale * (0.5 + 0.5 * np.tanh(2 * np.sin(x + 0.3) * np.cos(y) + np.sin(z)))
    return scale * RNG.normal(size=SH)


def phi_field():
    x = (np.arange(-2, NI + 4) - 0.5) * CFG.dx
    z, y, xx = np.meshgrid(np.arange(SH[0]), np.arange(SH[1]), x, indexing="ij")
    d = 0.5 - np.abs(xx - 1.0 - 0.05 * np.sin(0.4 * y + 0.3 * z))
    return 0.5 * (1 + np.tanh(d / (1.5 * CFG.dx))) + 1e-3 * RNG.normal(size=SH) * (np.abs(d) < 0.1)


def rel(a, b):
    m = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / m


def both(orc, L, name, args, outs, orc_name=None):
    """Call orc_<name> and <name>_ with the same argument recipe.
    args: list of ('i',v) | ('d',v) | ('a',ndarray) | ('ia',list) | ('none',None)
    Returns (oracle outputs, gpu outputs) for the array indices in outs."""
    def build(lib_mod, copies):
        out = []
        for kind, v in args:
            if kind == "i":
                out.append(ctypes.byref(ctypes.c_int(v)))
            elif kind == "d":
                out.append(ctypes.byref(ctypes.c_double(v)))
            elif kind == "ia":
                out.append((ctypes.c_int * len(v))(*v))
            elif kind == "none":
                out.append(None)
            else:
                arr = v.copy()
                copies.append(arr)
                out.append(ctypes.c_void_p(arr.ctypes.data))
        return out
    co, cg = [], []
    ao = build(orc, co)
    ag = build(L, cg)
    getattr(orc.lib(), orc_name or ("orc_" + name))(*ao)
    getattr(L, name + "_")(*ag)
    assert L.fmf_last_error() == 0
    return [co[t] for t in outs], [cg[t] for t in outs]


def dims():
    return [("i", NI), ("i", NJ), ("i", NK)]


def inv():
    return [("d", 1 / CFG.dx), ("d", 1 / CFG.dy), ("d", 1 / CFG.dz)]


NID = [-1] * 6
DYA = np.full(NJ + 6, 1 / CFG.dy)


def check(o, g, tol):
    for a, b in zip(o, g):
        assert rel(b, a) <= tol, rel(b, a)


def test_cal_grad_p2a(orc, L):
    args = [("i", 0), ("i", NJ)] + dims() + [("d", 1 / CFG.dx), ("a", DYA), ("d", 1 / CFG.dz), ("a", phi_field())] + \
        [("a", np.zeros(SH))] * 3
    o, g = both(orc, L, "cal_grad_p2a", args, [1, 2, 3, 4])
    check(o, g, EXACT)


def _grads(orc, phi):
    gx, gy, gz = np.zeros(SH), np.zeros(SH), np.zeros(SH)
    I, D, P = orc.I, orc.D, orc.P
    orc.lib().orc_cal_grad_p2a(I(0), I(NJ), I(NI), I(NJ), I(NK), D(1 / CFG.dx), P(DYA), D(1 / CFG.dz), P(phi),
                               P(gx), P(gy), P(gz))
    return gx, gy, gz


def test_solphi_mthinc1_2_3(orc, L):
    phi = phi_field().clip(0, 1)
    gx, gy, gz = _grads(orc, phi)
    u, v, w = field(0.7), field(0.5), field(0.6)
    dt = 2e-3
    fl = [np.zeros(SH) for _ in range(3)]
    args = dims() + inv() + [("d", dt), ("d", 2.0), ("a", phi), ("a", gx), ("a", gy), ("a", gz), ("a", u), ("a", v),
                             ("a", w)] + [("a", f) for f in fl]
    o, g = both(orc, L, "solphi_mthinc1", args, [7, 8, 9])
    check(o, g, TRANSC)
    args2 = dims() + inv() + [("d", dt), ("a", u), ("a", v), ("a", w)] + [("a", f) for f in o] + \
        [("a", phi), ("a", phi.copy())]
    o2, g2 = both(orc, L, "solphi_mthinc2", args2, [7])
    check(o2, g2, EXACT)
    phin = o2[0]
    hx, hy, hz = _grads(orc, phin)
    args3 = [("i", 0)] + dims() + inv() + [("d", 2.0), ("a", hx), ("a", hy), ("a", hz), ("a", phi), ("a", phin)]
    o3, g3 = both(orc, L, "solphi_mthinc3", args3, [4])
    check(o3, g3, 1e-13)


def test_summation(orc, L):
    q = np.stack([field(), phi_field() * 1.2 - 0.1])
    o, g = both(orc, L, "summation", dims() + [("a", q), ("i", 1)], [0])
    check(o, g, 0.0)


def test_gnbc_contact_angle_bndu(orc, L):
    th0, ze, l1, l2 = C.wall_arrays(C.get("couette32", ni=NI, nj=NJ, nk=NK, theta_lo=70.0, theta_hi=110.0))
    u, w = field(0.4), field(0.2)
    theta = np.zeros(SH)
    args = [("ia", NID)] + dims() + [("a", u), ("a", w), ("d", -1.0), ("a", th0), ("d", 1.0), ("a", ze),
                                     ("a", theta)]
    o, g = both(orc, L, "gnbc", args, [4])
    check(o, g, TRANSC)
    args = [("ia", NID)] + dims() + [("a", phi_field()), ("a", o[0]), ("d", CFG.dx), ("d", CFG.dy), ("d", CFG.dz)]
    o2, g2 = both(orc, L, "bnd_contact_angle", args, [0])
    check(o2, g2, TRANSC)
    args = [("ia", NID)] + dims() + [("a", field()), ("a", field()), ("a", field()), ("d", -1.0), ("d", CFG.dy),
                                     ("a", l1), ("a", l2), ("a", phi_field())]
    o3, g3 = both(orc, L, "bndu", args, [0, 1, 2])
    check(o3, g3, EXACT)


def test_periodic_neumann(orc, L):
    o, g = both(orc, L, "bnd_periodic", dims() + [("a", field())], [0])
    check(o, g, 0.0)
    o, g = both(orc, L, "bnd_neumann", [("ia", NID)] + dims() + [("a", field())], [0])
    check(o, g, 0.0)


def test_weno5(orc, L):
    args = dims() + inv() + [("a", field(smooth=True)), ("a", field(0.5)), ("a", field(0.3))] + \
        [("a", np.zeros(SH))] * 3
    o, g = both(orc, L, "cal_advu_weno5", args, [3, 4, 5])
    check(o, g, 1e-13)


def test_glue(orc, L):
    phi = phi_field()
    o, g = both(orc, L, "cal_arith_mean", dims() + [("a", phi), ("d", 3.0), ("d", 1.0), ("a", np.zeros(SH))], [1])
    check(o, g, EXACT)
    o, g = both(orc, L, "cal_harm_mean", dims() + [("a", phi.clip(0, 1)), ("d", 3.0), ("d", 1.0),
                                                   ("a", np.zeros(SH))], [1])
    check(o, g, EXACT)
    o, g = both(orc, L, "calphat", dims() + [("a", field()), ("a", field()), ("a", field())], [2])
    check(o, g, EXACT)
    o, g = both(orc, L, "cal_grad_prs", dims() + inv() + [("a", field())] + [("a", field())] * 3, [1, 2, 3])
    check(o, g, EXACT)
    s6 = RNG.normal(size=(6,) + SH)
    o, g = both(orc, L, "calsij", dims() + inv() + [("a", field()), ("a", field()), ("a", field()), ("a", s6)], [3])
    check(o, g, EXACT)
    rmu = 0.05 + 0.45 * phi.clip(0, 1)
    for nm in ("cal_arith_tau", "cal_harm_tau"):
        o, g = both(orc, L, nm, dims() + [("a", s6), ("a", rmu), ("a", RNG.normal(size=(6,) + SH))], [2])
        check(o, g, EXACT)
    o, g = both(orc, L, "cal_div_tensor", dims() + inv() + [("a", s6)] + [("a", field())] * 3, [1, 2, 3])
    check(o, g, EXACT)


def test_surface_tension(orc, L):
    phi = phi_field()
    gx, gy, gz = _grads(orc, phi)
    rns = []
    for ip, jp, kp in ((1, 1, 1), (0, 0, 1), (0, 1, 0), (1, 0, 0)):
        args = dims() + inv() + [("i", ip), ("i", jp), ("i", kp), ("a", gx), ("a", gy), ("a", gz),
                                 ("a", RNG.normal(size=(3,) + SH))]
        o, g = both(orc, L, "calrn", args, [3])
        check(o, g, EXACT)
        rns.append(o[0])
    o, g = both(orc, L, "calrkap", dims() + inv() + [("a", r) for r in rns] + [("a", np.zeros((3,) + SH))], [4])
    check(o, g, EXACT)
    rk = o[0]
    args = dims() + [("d", 2.0), ("d", 1.0), ("d", 0.7), ("a", gx), ("a", gy), ("a", gz), ("a", rk)] + \
        [("a", np.zeros(SH))] * 3
    o, g = both(orc, L, "calfst", args, [4, 5, 6])
    check(o, g, EXACT)
    args = dims() + [("a", o[0]), ("a", o[1]), ("a", o[2])] + [("a", field())] * 3
    o2, g2 = both(orc, L, "sum_fst", args, [3, 4, 5])
    check(o2, g2, EXACT)


def test_srcu_coef_sor(orc, L):
    phi = phi_field().clip(0, 1)
    rho = 1.0 + 9.0 * (1 - phi)
    rmu = 0.05 + 0.45 * (1 - phi)
    arr = [field(0.1) for _ in range(18)]
    u, v, w = field(0.5), field(0.2), field(0.3)
    src = [np.zeros(SH) for _ in range(3)]
    args = [("ia", NID)] + dims() + [("d", 1.0), ("d", 1e-3), ("d", 0.0), ("d", 0.0), ("a", u), ("a", v), ("a", w),
                                     ("a", rho), ("a", rho * 1.01)] + [("a", a) for a in arr] + [("a", s) for s in src]
    o, g = both(orc, L, "cal_srcu", args, [23, 24, 25])
    check(o, g, EXACT)
    srcs = o
    coefs = [np.zeros(SH) for _ in range(45)]
    # oracle takes coef as an array of 45 pointers plus a harmonic flag
    for harmonic, nm in ((0, "cal_arith_coef_vis"), (1, "cal_harm_coef_vis")):
        co = [c.copy() for c in coefs]
        cg = [c.copy() for c in coefs]
        I, D, P = orc.I, orc.D, orc.P
        parr = (ctypes.POINTER(ctypes.c_double) * 45)(*[P(c) for c in co])
        orc.lib().orc_cal_arith_coef_vis_v(I(NI), I(NJ), I(NK), D(1 / CFG.dx), D(1 / CFG.dy), D(1 / CFG.dz), P(rmu),
                                           parr, ctypes.c_int(harmonic))
        getattr(L, nm + "_")(I(NI), I(NJ), I(NK), D(1 / CFG.dx), D(1 / CFG.dy), D(1 / CFG.dz),
                             ctypes.c_void_p(rmu.ctypes.data), *[ctypes.c_void_p(c.ctypes.data) for c in cg])
        assert L.fmf_last_error() == 0
        check(co, cg, EXACT)
        if harmonic == 0:
            coef_arith = co
    # SOR: oracle variant returns the iteration count
    th0, ze, l1, l2 = C.wall_arrays(C.get("couette32", ni=NI, nj=NJ, nk=NK))
    uo, vo, wo = u.copy(), v.copy(), w.copy()
    ug, vg, wg = u.copy(), v.copy(), w.copy()
    I, D, P = orc.I, orc.D, orc.P
    parr = (ctypes.POINTER(ctypes.c_double) * 45)(*[P(c) for c in coef_arith])
    err = ctypes.c_double()
    nit = orc.lib().orc_solu_sor4_v(orc.IA(NID), I(NI), I(NJ), I(NK), D(1e-3), P(rho), P(rho * 1.01), parr,
                                    P(srcs[0]), P(srcs[1]), P(srcs[2]), P(uo), P(vo), P(wo), D(-1.0), D(CFG.dy),
                                    P(l1), P(l2), P(phi), ctypes.byref(err))
    rho2 = rho * 1.01
    vp = lambda a: ctypes.c_void_p(a.ctypes.data)
    L.solu_sor4_(I(0), I(0), orc.IA(NID), I(1), I(NI), I(NJ), I(NK), None, None, None, I(1), I(0), D(1e-3), vp(rho),
                 vp(rho2), *[vp(c) for c in coef_arith], vp(srcs[0]), vp(srcs[1]), vp(srcs[2]), vp(ug), vp(vg),
                 vp(wg), D(-1.0), D(CFG.dy), vp(l1), vp(l2), vp(phi))
    assert L.fmf_last_error() == 0
    assert L.fmf_last_sor_iterations() == nit
    check([uo, vo, wo], [ug, vg, wg], 1e-13)


def test_pressure(orc, L):
    n = NI * NJ * NK
    div = np.zeros(SH)
    d = RNG.normal(size=(NK, NJ, NI))
    div[3:-3, 3:-3, 3:-3] = d - d.mean()
    args = dims() + [("a", np.zeros(2 * n)), ("a", div), ("a", np.zeros(n)), ("a", np.zeros(n))]
    o, g = both(orc, L, "solp_fft_tdma1", args, [2, 3])
    check(o, g, 1e-13)
    nj6 = NJ + 6
    as_f = np.zeros(nj6)
    an_f = np.zeros(nj6)
    ap_f = np.zeros(nj6)
    for j in range(1, NJ + 1):
        as_f[j + 2] = an_f[j + 2] = CFG.dy ** -2
        ap_f[j + 2] = 2 * CFG.dy ** -2
    ap_f[3] -= as_f[3]
    as_f[3] = 0
    ap_f[NJ + 2] -= an_f[NJ + 2]
    an_f[NJ + 2] = 0
    args = [("i", 0), ("i", 1), ("ia", [NI, NJ, NK]), ("d", 1.0), ("d", 1 / CFG.dx), ("d", 1 / CFG.dz),
            ("a", as_f), ("a", an_f), ("a", ap_f), ("none", None), ("none", None), ("none", None),
            ("a", o[0]), ("a", o[1])]
    o2, g2 = both(orc, L, "solp_fft_tdma2", args, [3, 4])
    check(o2, g2, 1e-12)
    args = dims() + [("a", np.zeros(2 * n)), ("a", o2[0]), ("a", o2[1]), ("a", np.zeros(SH))]
    o3, g3 = both(orc, L, "solp_fft_tdma3", args, [3])
    check(o3, g3, 1e-12)
    o4, g4 = both(orc, L, "bnd_avzero", [("i", 0), ("i", 1)] + dims() + [("a", o3[0])], [0])
    check(o4, g4, 1e-12)
    u, v, w = field(), field(), field()
    args = [("i", 0), ("i", 1)] + dims() + inv() + [("d", 1e-3), ("a", u), ("a", v), ("a", w), ("a", np.zeros(SH)),
                                                    ("d", 0.0)]
    # caldiv: compare div array (err_div is a scalar output checked separately)
    o5, g5 = both(orc, L, "caldiv", args, [3])
    check(o5, g5, EXACT)
    args = [("ia", NID)] + dims() + [("d", 1.0)] + inv() + [("d", 1e-3), ("a", o4[0]), ("a", field()), ("a", u),
                                                            ("a", v), ("a", w), ("a", np.zeros(SH))]
    o6, g6 = both(orc, L, "corunp_explicit", args, [2, 3, 4, 5])
    check(o6, g6, 1e-13)


def test_cal_av_and_errors(orc, L):
    q = field()
    av = ctypes.c_double()
    I = orc.I
    L.cal_av_(I(0), I(1), I(NI), I(NJ), I(NK), ctypes.c_void_p(q.ctypes.data), ctypes.byref(av))
    assert L.fmf_last_error() == 0
    assert abs(av.value - C.interior(q).mean()) <= 1e-15 * np.abs(q).max()
    # a non-power-of-two grid is rejected with FMF_ERR_ARG and nothing launches
    L.bnd_periodic_(I(30), I(NJ), I(NK), ctypes.c_void_p(q.ctypes.data))
    assert L.fmf_last_error() == 2
    # multi-rank arguments are reported as unsupported on one GPU
    L.cal_av_(I(1), I(2), I(NI), I(NJ), I(NK), ctypes.c_void_p(q.ctypes.data), ctypes.byref(av))
    assert L.fmf_last_error() == 6
    # NaN in a reduction is reported
    q[10, 10, 10] = np.nan
    L.cal_av_(I(0), I(1), I(NI), I(NJ), I(NK), ctypes.c_void_p(q.ctypes.data), ctypes.byref(av))
    assert L.fmf_last_error() == 3


def test_solp_fft_tdma4_monitor(orc, L):
    """The Err_solp monitor (solp_fft_tdma4.f:28-95): RMS of the 7-point Poisson
    residual of dp against div, and RMS of div, as the oracle computes them; on a
    step that is not a monitor step nothing is computed."""
    div = np.zeros(SH)
    d = RNG.normal(size=(NK, NJ, NI))
    div[3:-3, 3:-3, 3:-3] = d - d.mean()
    dp = field(0.01)
    rho, dxi, dyi, dzi = 1.0, 1 / CFG.dx, 1 / CFG.dy, 1 / CFG.dz
    eo, e0o = ctypes.c_double(), ctypes.c_double()
    I, D, P = orc.I, orc.D, orc.P
    orc.lib().orc_solp_fft_tdma4_v(I(NI), I(NJ), I(NK), D(rho), D(dxi), D(dyi), D(dzi), P(div), P(dp),
                                   ctypes.byref(eo), ctypes.byref(e0o))
    vp = lambda a: ctypes.c_void_p(a.ctypes.data)
    L.solp_fft_tdma4_(I(0), I(0), I(1), I(NI), I(NJ), I(NK), I(10), I(5), D(rho), D(dxi), D(dyi), D(dzi), vp(div),
                      vp(dp))
    assert L.fmf_last_error() == 0
    eg, e0g = ctypes.c_double(), ctypes.c_double()
    assert L.fmf_last_solp_residual(ctypes.byref(eg), ctypes.byref(e0g)) == 0
    assert abs(eg.value - eo.value) <= 1e-12 * eo.value, (eg.value, eo.value)
    assert abs(e0g.value - e0o.value) <= 1e-12 * e0o.value, (e0g.value, e0o.value)
    # nstep not a multiple of imon_t: the monitor is skipped, its last values stay
    L.solp_fft_tdma4_(I(0), I(0), I(1), I(NI), I(NJ), I(NK), I(11), I(5), D(rho), D(dxi), D(dyi), D(dzi),
                      vp(field()), vp(dp))
    eg2, e0g2 = ctypes.c_double(), ctypes.c_double()
    L.fmf_last_solp_residual(ctypes.byref(eg2), ctypes.byref(e0g2))
    assert (eg2.value, e0g2.value) == (eg.value, e0g.value)


def test_trans_r2w_w2r(orc, L):
    """trans_r2w / trans_w2r on one rank (trans_r2w.f:23-38): the spectra's storage
    is shared, so both are copies; w2r after r2w returns the input bit for bit."""
    n = NI * NJ * NK
    svall = [NI, NJ, NK]
    r = RNG.normal(size=n)
    args = [("i", 0), ("i", 0), ("i", 1), ("ia", svall), ("i", 0), ("none", None), ("none", None), ("a", r),
            ("a", np.zeros(n))]
    o, g = both(orc, L, "trans_r2w", args, [1])
    check(o, g, 0.0)
    args = [("i", 0), ("i", 0), ("i", 1), ("ia", svall), ("i", 0), ("none", None), ("none", None), ("a", g[0]),
            ("a", np.zeros(n))]
    o2, g2 = both(orc, L, "trans_w2r", args, [1])
    check(o2, g2, 0.0)
    assert np.array_equal(g2[0], r)


def test_cal_grad_p2uvw(orc, L):
    """Face gradients of q at the u, v, w points (cal_grad_p2uvw.f:25-44)."""
    args = [("i", 0), ("i", NJ)] + dims() + [("d", 1 / CFG.dx), ("a", DYA), ("d", 1 / CFG.dz), ("a", field())] + \
        [("a", np.zeros(SH))] * 3
    o, g = both(orc, L, "cal_grad_p2uvw", args, [2, 3, 4])
    check(o, g, EXACT)


def test_cpy_init_q(orc, L):
    """cpy (q2 = q1 over the whole array) and init_q (three arrays to zero)."""
    o, g = both(orc, L, "cpy", dims() + [("a", field()), ("a", field())], [0, 1])
    check(o, g, 0.0)
    assert np.array_equal(g[0], g[1])
    o, g = both(orc, L, "init_q", dims() + [("a", field()), ("a", field()), ("a", field())], [0, 1, 2])
    for a, b in zip(o, g):
        assert not a.any() and not b.any()


def test_bnd_comm_one_rank(orc, L):
    """bnd_comm (bnd_comm.f:18) exchanges nothing on one rank: the field is unchanged;
    a multi-rank call (ipara = 1) is reported as unsupported."""
    q = field()
    args = [("i", 0), ("ia", NID)] + dims() + [("i", 0), ("none", None), ("none", None), ("a", q)]
    o, g = both(orc, L, "bnd_comm", args, [0])
    assert np.array_equal(o[0], q) and np.array_equal(g[0], q)
    I = orc.I
    L.bnd_comm_(I(1), orc.IA(NID), I(NI), I(NJ), I(NK), I(0), None, None, ctypes.c_void_p(q.ctypes.data))
    assert L.fmf_last_error() == 6


def test_solu_sor4_iteration_cap(orc, L):
    """A stop rule the solve cannot meet: after max_iter outer iterations solu_sor4_
    keeps the last iterate, as the reference does (solu_sor4.f:130,291-293), and
    reports FMF_ERR_ITER_CAP; the iterate equals the oracle's after as many
    iterations."""
    phi = phi_field().clip(0, 1)
    rho = 1.0 + 9.0 * (1 - phi)
    rmu = 0.05 + 0.45 * (1 - phi)
    I, D, P = orc.I, orc.D, orc.P
    coef = [np.zeros(SH) for _ in range(45)]
    parr = (ctypes.POINTER(ctypes.c_double) * 45)(*[P(c) for c in coef])
    orc.lib().orc_cal_arith_coef_vis_v(I(NI), I(NJ), I(NK), D(1 / CFG.dx), D(1 / CFG.dy), D(1 / CFG.dz), P(rmu),
                                       parr, ctypes.c_int(0))
    srcs = [field(0.1) for _ in range(3)]
    u, v, w = field(0.5), field(0.2), field(0.3)
    th0, ze, l1, l2 = C.wall_arrays(C.get("couette32", ni=NI, nj=NJ, nk=NK))
    uo, vo, wo = u.copy(), v.copy(), w.copy()
    ug, vg, wg = u.copy(), v.copy(), w.copy()
    rho2 = rho * 1.01
    orc.lib().orc_set_sor.argtypes = [ctypes.c_double, ctypes.c_int]
    L.fmf_set_sor.argtypes = [ctypes.c_double, ctypes.c_int]
    # 1e-300: below what even an exactly converged sweep reaches (err carries +1e-99)
    orc.lib().orc_set_sor(1e-300, 21)
    assert L.fmf_set_sor(1e-300, 21) == 0
    try:
        err = ctypes.c_double()
        nit = orc.lib().orc_solu_sor4_v(orc.IA(NID), I(NI), I(NJ), I(NK), D(1e-3), P(rho), P(rho2), parr,
                                        P(srcs[0]), P(srcs[1]), P(srcs[2]), P(uo), P(vo), P(wo), D(-1.0),
                                        D(CFG.dy), P(l1), P(l2), P(phi), ctypes.byref(err))
        vp = lambda a: ctypes.c_void_p(a.ctypes.data)
        L.solu_sor4_(I(0), I(0), orc.IA(NID), I(1), I(NI), I(NJ), I(NK), None, None, None, I(1), I(0), D(1e-3),
                     vp(rho), vp(rho2), *[vp(c) for c in coef], vp(srcs[0]), vp(srcs[1]), vp(srcs[2]), vp(ug),
                     vp(vg), vp(wg), D(-1.0), D(CFG.dy), vp(l1), vp(l2), vp(phi))
        assert L.fmf_last_error() == 4
        assert nit == 21 and L.fmf_last_sor_iterations() == 21
        check([uo, vo, wo], [ug, vg, wg], 1e-13)
    finally:
        orc.lib().orc_set_sor(1e-3, 21)
        L.fmf_set_sor(1e-3, 21)
