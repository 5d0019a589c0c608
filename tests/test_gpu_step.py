"""Parity of the fused device-resident step (fmf_ctx_step) against the oracle's
restatement of main.f90:473-697: phi, u, v, w, p after 1 and N steps within a
relative tolerance of 1e-10 (FP64 path), identical SOR iteration counts per step,
and at full workload size the invariants (volume conservation, post-projection
divergence) checked on the GPU result alone."""
import numpy as np
import pytest

from fmf import capi
from fmf import config as C

pytestmark = pytest.mark.gpu

TOL = 1e-10
FIELDS = {"u": 0, "v": 1, "w": 2, "p": 6, "phi": 9, "phi0": 8}


def relerr(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def _compare(orc, cfg, steps, tol=TOL):
    s = orc.Solver(cfg)
    st_o = s.initial_state()
    g = capi.Stepper(cfg)
    st_g = g.initial_state()
    # start-up pass parity (main.f90:322-366)
    for name, f in FIELDS.items():
        assert relerr(st_g[f], st_o[f]) <= 1e-13, ("init", name)
    g.upload(st_o)
    gpu_iters = []
    for n in range(steps):
        s.step(st_o, 1)
        g.step(1)
        gpu_iters += g.sor_iterations()
    out = g.get_state()
    errs = {name: relerr(C.interior(out[f]), C.interior(st_o[f])) for name, f in FIELDS.items()}
    full = {name: relerr(out[f], st_o[f]) for name, f in FIELDS.items()}
    g.close()
    assert gpu_iters == s.sor_iters, (gpu_iters, s.sor_iters)
    return errs, full, s.sor_iters


@pytest.mark.parametrize("steps", [1, 100])
def test_step_parity_couette32(orc, fmf_lib, steps):
    """The 32x32x16 Couette workload after 1 step and after its full 100 steps."""
    cfg = C.get("couette32")
    errs, full, _ = _compare(orc, cfg, steps)
    for name in FIELDS:
        assert errs[name] <= TOL, (name, errs)
        assert full[name] <= TOL, (name, full)


def test_step_parity_harmonic_and_walls(orc, fmf_lib):
    """cal_harm_coef_vis path, unequal properties and asymmetric wall angles."""
    cfg = C.get("couette32", harmonic=1, rhol=4.0, rhog=1.0, rmul=0.2, rmug=0.05, theta_lo=60.0,
                theta_hi=110.0, ni=32, nj=16, nk=16)
    errs, full, _ = _compare(orc, cfg, 5)
    for name in FIELDS:
        assert full[name] <= TOL, (name, full)


def test_sor_iterations_match(orc, fmf_lib):
    cfg = C.get("couette32")
    s = orc.Solver(cfg)
    st = s.initial_state()
    g = capi.Stepper(cfg)
    g.upload(st)
    s.step(st, 8)
    g.step(8)
    g.sync()
    assert g.sor_iterations() == s.sor_iters
    g.close()


def test_step_parity_couette256_ten_steps(orc, fmf_lib):
    """The 256x128x128 workload (density and viscosity ratio 10, perturbed interface)
    for 10 steps, with equal viscous iteration counts."""
    cfg = C.get("couette256")
    errs, full, iters = _compare(orc, cfg, 10)
    for name in FIELDS:
        assert full[name] <= TOL, (name, full)


def test_step_parity_droplet(orc, fmf_lib):
    """The sessile drop of the 512x256x256 and 256x128x128 workloads at 64x32x32
    (density ratio 1000, viscosity ratio 100, resting walls, 60/120 deg checkerboard
    lower wall in 0.125 squares) for 20 steps: the GNBC on mixed angles and the large
    density jumps of the momentum factors and the projection against the oracle."""
    cfg = C.get("droplet256", ni=64, nj=32, nk=32, checker_cells=4)
    s = orc.Solver(cfg)
    st_o = s.initial_state()
    g = capi.Stepper(cfg)
    g.upload(st_o)
    s.step(st_o, 20)
    g.step(20)
    out = g.get_state()
    assert g.sor_iterations() == s.sor_iters[-20:]
    for name, f in FIELDS.items():
        assert relerr(out[f], st_o[f]) <= TOL, (name, relerr(out[f], st_o[f]))
    g.close()
    s.close()


def test_iteration_cap_fused_step(orc, fmf_lib):
    """A viscous stop rule the solve cannot meet: each step runs max_iter outer
    iterations, carries on with the last iterate (solu_sor4.f:130,291-293) and the
    call reports FMF_ERR_ITER_CAP (a warning in the binding); the state matches the
    oracle run with the same stop rule."""
    import ctypes

    cfg = C.get("couette32")
    s = orc.Solver(cfg)
    st_o = s.initial_state()
    g = capi.Stepper(cfg)
    g.upload(st_o)
    g.set_sor(1e-300, 6)
    L = orc.lib()
    L.orc_set_sor.argtypes = [ctypes.c_double, ctypes.c_int]
    L.orc_set_sor(1e-300, 6)
    try:
        s.step(st_o, 3)
    finally:
        L.orc_set_sor(1e-3, 21)
    assert capi.lib().fmf_ctx_step(g.h, 3) == capi.FMF_ERR_ITER_CAP
    assert g.sor_iterations() == [6, 6, 6]
    out = g.get_state()
    for name, f in FIELDS.items():
        assert relerr(out[f], st_o[f]) <= TOL, (name, relerr(out[f], st_o[f]))
    with pytest.warns(capi.SorCapWarning):
        g.step(1)
    g.set_sor(1e-3, 21)
    g.step(1)
    assert g.sor_iterations()[0] < 21
    g.close()
    s.close()


def test_invariants_full_size(fmf_lib):
    """couette256 for 20 steps on the GPU alone: phi volume conserved to round-off and
    the post-projection divergence (caldiv.f stencil) at round-off."""
    cfg = C.get("couette256")
    g = capi.Stepper(cfg)
    st = g.initial_state()
    v0 = C.interior(st[9]).sum()
    g.step(20)
    out = g.get_state()
    v1 = C.interior(out[9]).sum()
    assert abs(v1 - v0) <= 1e-11 * v0
    u, v, w = out[0], out[1], out[2]
    d = ((u[3:-3, 3:-3, 3:-3] - u[3:-3, 3:-3, 2:-4]) / cfg.dx + (v[3:-3, 3:-3, 3:-3] - v[3:-3, 2:-4, 3:-3]) / cfg.dy +
         (w[3:-3, 3:-3, 3:-3] - w[2:-4, 3:-3, 3:-3]) / cfg.dz)
    assert np.abs(d).max() <= 1e-8 * np.abs(C.interior(u)).max() / cfg.dx
    assert np.isfinite(out).all()
    g.close()


def test_division_free_reciprocal(fmf_lib):
    """The WENO5 kernel's Newton-Raphson reciprocal against the IEEE quotient over
    2^-1000 .. 2^1000: within two units in the last place."""
    import ctypes

    L = fmf_lib
    L.fmf_check_reciprocal.argtypes = [ctypes.c_longlong, ctypes.POINTER(ctypes.c_double)]
    err = ctypes.c_double(-1.0)
    assert L.fmf_check_reciprocal(1 << 22, ctypes.byref(err)) == 0
    assert 0.0 <= err.value <= 2 * 2.0 ** -52, err.value


def test_division_free_rsqrt(fmf_lib):
    """The CSF kernel's Newton-Raphson reciprocal square root against
    1.0 / sqrt(x) over 2^-1000 .. 2^1000: within two units in the last place."""
    import ctypes

    L = fmf_lib
    L.fmf_check_rsqrt.argtypes = [ctypes.c_longlong, ctypes.POINTER(ctypes.c_double)]
    err = ctypes.c_double(-1.0)
    assert L.fmf_check_rsqrt(1 << 22, ctypes.byref(err)) == 0
    assert 0.0 <= err.value <= 2 * 2.0 ** -52, err.value


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_step_host_matches_upload_step_download(fmf_lib, prec):
    """fmf_ctx_step_host (copies overlapping the step, phin not uploaded) gives bit for
    bit the state of upload + step + download, step after step, in both precisions,
    whether the caller passes back the previous result or a changed state."""
    import torch

    cfg = C.get("couette32")
    p = capi.FMF_FP64 if prec == "fp64" else capi.FMF_MIXED
    a = capi.Stepper(cfg, precision=p)
    st = a.initial_state()
    b = capi.Stepper(cfg, precision=p)
    pin = torch.empty((12,) + cfg.shape, dtype=torch.float64, pin_memory=True).numpy()
    pin[:] = st
    ref = st.copy()
    # from the second call on the inputs are the previous result: the carried
    # advection of (uo, vo, wo) and surface tension of phi(1) are kept after the
    # device compares them; calls 3 and 4 pass a changed uo and phi(1), which the
    # compare must catch (the terms are then recomputed)
    for it in range(5):
        if it == 2:
            pin[3, 5, 6, 7] += 1e-3
        if it == 3:
            pin[9, 6, 7, 8] -= 1e-3
        ref[:] = pin
        b.step_host(pin, pin)
        a.upload(ref)
        a.step(1)
        a.download(ref)
        a.sync()
        assert np.array_equal(pin, ref), it
    a.close()
    b.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("grid", ["fused_csf", "dropin_csf"])
def test_carried_terms_bitwise(fmf_lib, monkeypatch, prec, grid):
    """A step that continues from the previous one takes that step's advection of
    (u, v, w) as its advection of (uo, vo, wo) and its surface tension of phin(1)
    as that of phi(1) (main.f90:686-697 makes them the same fields).  Ten steps
    that way give bit for bit the state of ten steps that recompute both terms
    (FMF_STEP_CACHE=0), including across an upload that restarts the carry.  Two
    grids: one the fused CSF kernel tiles (64x32x32, density and viscosity ratio
    10) and one it does not (16x16x16: the drop-in CSF chain)."""
    if grid == "fused_csf":
        cfg = C.get("couette256", ni=64, nj=32, nk=32)
    else:
        cfg = C.get("couette32", ni=16, nj=16, nk=16, rhol=4.0, rmul=0.2)
    p = capi.FMF_FP64 if prec == "fp64" else capi.FMF_MIXED
    a = capi.Stepper(cfg, precision=p)
    st0 = a.initial_state()
    monkeypatch.setenv("FMF_STEP_CACHE", "0")
    b = capi.Stepper(cfg, precision=p)
    monkeypatch.delenv("FMF_STEP_CACHE")
    b.upload(st0)
    a.step(6)
    b.step(6)
    sa, sb = a.get_state(), b.get_state()
    assert np.array_equal(sa, sb)
    assert a.sor_iterations() == b.sor_iterations()
    # an upload of the same state ends the carry; the next step recomputes both
    a.upload(sa)
    a.step(4)
    b.step(4)
    sa, sb = a.get_state(), b.get_state()
    for f in range(12):
        assert np.array_equal(sa[f], sb[f]), C.STATE_FIELDS[f]
    a.close()
    b.close()


def test_split_pair_precision(fmf_lib):
    """The (hi, lo) float pairs of the mixed WENO5 hold each double to about 2^-48
    of itself over 2^-96 .. 2^127, small magnitudes included (where the low part
    needs a two-factor scale to stay a normal float)."""
    import ctypes

    L = fmf_lib
    L.fmf_check_split_pair.argtypes = [ctypes.c_longlong, ctypes.POINTER(ctypes.c_double)]
    err = ctypes.c_double(-1.0)
    assert L.fmf_check_split_pair(1 << 22, ctypes.byref(err)) == 0
    assert 0.0 <= err.value <= 2.0 ** -47, err.value


@pytest.mark.parametrize("precision", [capi.FMF_FP64, capi.FMF_MIXED])
def test_device_stop_rule_matches_host(fmf_lib, monkeypatch, precision):
    """Graph-replayed steps run the viscous solve's stop rule on the device (a WHILE
    conditional node; no host round trip per outer iteration).  Against a context
    whose host applies the rule after every iteration (FMF_DEVICE_LOOP=0 at
    creation): the same state bit for bit and the same iteration counts after 12
    steps in one call, then after a stop rule the solve cannot meet (the cap) and
    back."""
    cfg = C.get("couette256", ni=64, nj=32, nk=32)
    g0 = capi.Stepper(cfg)
    st0 = g0.initial_state()
    g0.close()
    res = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("FMF_DEVICE_LOOP", mode)
        S = capi.Stepper(cfg, precision=precision)
        monkeypatch.delenv("FMF_DEVICE_LOOP")
        try:
            S.upload(st0)
            S.step(12)
            its = list(S.sor_iterations())
            S.set_sor(1e-300, 5)
            assert capi.lib().fmf_ctx_step(S.h, 3) == capi.FMF_ERR_ITER_CAP
            its += list(S.sor_iterations())
            S.set_sor(1e-3, 21)
            S.step(2)
            its += list(S.sor_iterations())
            res[mode] = (S.get_state(), its)
        finally:
            S.close()
    (a, ia), (b, ib) = res["0"], res["1"]
    assert ia == ib
    assert ia[12:15] == [5, 5, 5] and all(1 <= k < 21 for k in ia[:12] + ia[15:])
    assert np.array_equal(a, b)
