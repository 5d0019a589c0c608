"""The FP64-accurate step (precision FMF_FP64E: the FP64 step with its WENO5
advection, CSF force, viscous momentum factors and explicit viscous term in
FP32-pair arithmetic on GB300's FP32 pipe) against the oracle's
restatement of main.f90:473-697 at the FP64 step's bar: phi, u, v, w, p within a
relative tolerance of 1e-10 (largest difference over the oracle field's largest
magnitude) with identical viscous iteration counts per step; and its WENO5 kernel
against the FP64 kernel on fields of many magnitudes (cal_advu_weno5.f:1-258,
weno5.h:2-70)."""
import numpy as np
import pytest

from fmf import capi
from fmf import config as C

pytestmark = pytest.mark.gpu

TOL = 1e-10
FIELDS = {"u": 0, "v": 1, "w": 2, "p": 6, "phi": 9, "phi0": 8}


def relerr(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def _compare(orc, cfg, steps):
    s = orc.Solver(cfg)
    st_o = s.initial_state()
    g = capi.Stepper(cfg, precision=capi.FMF_FP64E)
    g.upload(st_o)
    s.step(st_o, steps)
    g.step(steps)
    out = g.get_state()
    iters = g.sor_iterations()
    g.close()
    s.close()
    assert iters == s.sor_iters[-steps:], (iters, s.sor_iters)
    return {name: relerr(out[f], st_o[f]) for name, f in FIELDS.items()}


@pytest.mark.parametrize("name,kw,steps", [
    ("couette32", {}, 100),
    ("couette32", dict(harmonic=1, rhol=4.0, rhog=1.0, rmul=0.2, rmug=0.05, theta_lo=60.0, theta_hi=110.0,
                       ni=32, nj=16, nk=16), 5),
    ("droplet256", dict(ni=64, nj=32, nk=32, checker_cells=4), 20),
    ("couette256", {}, 10),
])
def test_fp64e_step_parity(orc, fmf_lib, name, kw, steps):
    """The 32x16x32 Couette workload for its 100 steps; the harmonic-coefficient path
    with unequal properties and wall angles; the sessile drop (density ratio 1000,
    checkerboard lower wall) at 64x32x32 for 20 steps; the 256x128x128 Couette
    workload for 10 steps."""
    errs = _compare(orc, C.get(name, **kw), steps)
    for k, e in errs.items():
        assert e <= TOL, (k, errs)


@pytest.mark.parametrize("scale", [1e-15, 1e-6, 1.0, 1e6, 1e15])
def test_weno5_pairs_against_fp64(fmf_lib, scale):
    """fmf_dev_weno5_fused in FP32 pairs against FP64 on one level of (u, v, w) at
    64x32x32: smooth waves, a jump, an exactly linear (Couette-like) region, a
    constant region, zeros and random noise, all times `scale` (the weights scale
    like the 8th power of the differences, so the reference's additive 1e-80
    dominates at the small scales and is negligible at the large ones).  Each
    component within 1e-12 of the FP64 component's largest magnitude."""
    import torch

    ni, nj, nk = 64, 32, 32
    shape = (nk + 6, nj + 6, ni + 6)
    rng = np.random.default_rng(11)
    z, y, x = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), np.arange(shape[2]), indexing="ij")
    fields = []
    for c in range(3):
        f = np.sin(0.3 * x + c) * np.cos(0.2 * y) + 0.5 * np.sin(0.17 * z + 2 * c)
        f = f + np.where(x > 30 + c, 0.7, 0.0)                          # a jump
        lin = (z < 10)
        f = np.where(lin, 0.05 * y - 0.8, f)                            # exactly linear in y
        f = np.where((z >= 10) & (z < 14), 0.25, f)                     # constant
        f = np.where((z >= 14) & (z < 16), 0.0, f)                      # zeros
        f = np.where(z > nk, rng.standard_normal(shape), f)             # noise
        fields.append(np.ascontiguousarray(f * scale))
    dev = [torch.from_numpy(f).cuda() for f in fields]
    outs = {}
    for prec in (capi.FMF_FP64, capi.FMF_FP64E):
        a = [torch.zeros(shape, dtype=torch.float64, device="cuda") for _ in range(3)]
        torch.cuda.synchronize()  # the library runs on its own stream
        st = capi.lib().fmf_dev_weno5_fused(prec, ni, nj, nk, 64.0, 32.0, 32.0, *[d.data_ptr() for d in dev],
                                            *[t.data_ptr() for t in a])
        assert st == 0, st
        assert capi.lib().fmf_device_synchronize() == 0
        outs[prec] = [t.cpu().numpy() for t in a]
    for c in range(3):
        ref, got = outs[capi.FMF_FP64][c], outs[capi.FMF_FP64E][c]
        m = np.abs(ref).max()
        assert m > 0
        err = np.abs(got - ref).max() / m
        assert err <= 1e-12, (c, scale, err)


@pytest.mark.parametrize("shape", [(64, 32, 32), (256, 128, 128)])
def test_csf_pairs_against_fp64(fmf_lib, shape):
    """fmf_dev_csf_fused in FP32 pairs against FP64: the force of a tanh-profiled
    sphere (radius a quarter of the domain height, 1.5-cell width, as the sessile
    drop's initial phi) and of a tilted planar front, whose far field carries
    gradients down to the end of double's range.  Pairs hold phi to 2^-48, so a
    vertex gradient g carries an error of about 2^-48 dxi, its normal 2^-48 dxi / g,
    the curvature dxi times that, and the force C kappa (phi(i+1) - phi(i)) dxi,
    with C = 2 sigma/(rho_l + rho_g) and a phi difference of about g dx, an error of
    about 2^-48 C dxi^2 wherever the interface is: each component within 1e-12 of
    C dxi^2 (the force of a grid-scale curvature on a unit jump), and the sphere's
    within 1e-11 of its own largest force."""
    import torch

    ni, nj, nk = shape
    dx = 1.0 / nj
    rhol, rhog, sigma = 1000.0, 1.0, 1.0
    scale = 2.0 * sigma / (rhol + rhog) / dx ** 2
    pad = (nk + 6, nj + 6, ni + 6)
    z, y, x = np.meshgrid(np.arange(pad[0]) - 2.5, np.arange(pad[1]) - 2.5, np.arange(pad[2]) - 2.5, indexing="ij")
    X, Y, Z = x * dx, y * dx, z * dx
    r = np.sqrt((X - ni * dx / 2) ** 2 + (Y - 0.1) ** 2 + (Z - nk * dx / 2) ** 2)
    w = 1.5 * dx
    phis = {"sphere": 0.5 * (1 - np.tanh((r - 0.25) / w)),
            "front": 0.5 * (1 + np.tanh((0.3 * X + 0.9 * Y - 0.2 * Z - 0.4) / w))}
    errs = {}
    for name, phi in phis.items():
        d = torch.from_numpy(np.ascontiguousarray(phi)).cuda()
        outs = {}
        for prec in (capi.FMF_FP64, capi.FMF_FP64E):
            f = [torch.zeros(pad, dtype=torch.float64, device="cuda") for _ in range(3)]
            torch.cuda.synchronize()
            st = capi.lib().fmf_dev_csf_fused(prec, ni, nj, nk, dx, dx, dx, rhol, rhog, sigma, d.data_ptr(),
                                              *[t.data_ptr() for t in f])
            assert st == 0, st
            assert capi.lib().fmf_device_synchronize() == 0
            outs[prec] = [t.cpu().numpy() for t in f]
        for c in range(3):
            ref, got = outs[capi.FMF_FP64][c], outs[capi.FMF_FP64E][c]
            assert np.isfinite(got).all()
            e = np.abs(got - ref).max()
            errs[(name, c)] = (e / scale, e / np.abs(ref).max())
    for (name, c), (e_scale, e_own) in errs.items():
        assert e_scale <= 1e-12, errs
        if name == "sphere":
            assert e_own <= 1e-11, errs
