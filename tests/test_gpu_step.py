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
    for n in range(steps):
        s.step(st_o, 1)
        g.step(1)
    out = g.get_state()
    errs = {name: relerr(C.interior(out[f]), C.interior(st_o[f])) for name, f in FIELDS.items()}
    full = {name: relerr(out[f], st_o[f]) for name, f in FIELDS.items()}
    g.close()
    return errs, full, s.sor_iters


@pytest.mark.parametrize("steps", [1, 10])
def test_step_parity_couette32(orc, fmf_lib, steps):
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


def test_step_parity_couette256_two_steps(orc, fmf_lib):
    """The 256x128x128 workload (density and viscosity ratio 10, perturbed interface)."""
    cfg = C.get("couette256")
    errs, full, iters = _compare(orc, cfg, 2)
    for name in FIELDS:
        assert full[name] <= TOL, (name, full)


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
    bit the state of upload + step + download, step after step, in both precisions."""
    import torch

    cfg = C.get("couette32")
    p = capi.FMF_FP64 if prec == "fp64" else capi.FMF_MIXED
    a = capi.Stepper(cfg, precision=p)
    st = a.initial_state()
    b = capi.Stepper(cfg, precision=p)
    pin = torch.empty((12,) + cfg.shape, dtype=torch.float64, pin_memory=True).numpy()
    pin[:] = st
    ref = st.copy()
    for _ in range(3):
        b.step_host(pin, pin)
        a.upload(ref)
        a.step(1)
        a.download(ref)
        a.sync()
        assert np.array_equal(pin, ref)
    a.close()
    b.close()
