"""The adjoint of the rollout with a mixed-precision forward (FP32 WENO5, MTHINC
Newton and fluxes, CSF and viscous corrections in the forward and recomputed
steps; FP64 reverse) against the FP64 adjoint, on the sessile drop of the
256x128x128 workload at 64x32x32 (density ratio 1000, 60/120 deg checkerboard
lower wall), K = 20, checkpoints every ceil(sqrt(K)) steps.  The gradients with
respect to theta0, zeta, l1, l2 and the initial phi agree with the FP64 adjoint's
within 1e-5 of their largest magnitude, and J within 1e-6."""
import numpy as np
import pytest

from fmf import config as C

pytestmark = pytest.mark.gpu

K = 20


def test_mixed_forward_adjoint_matches_fp64(fmf_lib):
    from fmf import capi
    from fmf.adjoint import Adjoint

    cfg = C.get("droplet256", ni=64, nj=32, nk=32, checker_cells=4)
    st0 = C.raw_state(cfg)
    walls = [w.copy() for w in C.wall_arrays(cfg)]
    out = {}
    for prec in (capi.FMF_FP64, capi.FMF_MIXED):
        A = Adjoint(cfg, sor_tol=1e-3, sor_max=21, adj_tol=1e-10, adj_max=400, precision=prec)
        try:
            J, g = A.rollout(K, st0, walls)
            Jf = A.forward(K, st0, walls)
            assert Jf == J
            assert A.device_bytes() > 0
        finally:
            A.close()
        out[prec] = (J, g)
    J64, g64 = out[capi.FMF_FP64]
    Jm, gm = out[capi.FMF_MIXED]
    assert J64 != 0.0
    assert abs(Jm - J64) <= 1e-6 * abs(J64), (Jm, J64)
    for name, a, b in zip(("theta0", "zeta", "l1", "l2", "phi"), gm, g64):
        scale = np.abs(b).max()
        assert scale > 0.0, name
        assert np.isfinite(a).all(), name
        assert np.abs(a - b).max() <= 1e-5 * scale, (name, np.abs(a - b).max() / scale)


def test_fp32_weno_reverse_matches_fp64_reverse(fmf_lib, monkeypatch):
    """With a mixed-precision forward the reverse of its FP32 WENO5 runs in FP32 (on
    the split pairs of the velocity, with the forward kernel's scaling).  Against
    the same handle with that reverse in FP64 (FMF_ADJ_F32_REVERSE=0 at creation):
    the same J, gradients within 1e-6 of their largest magnitude."""
    from fmf import capi
    from fmf.adjoint import Adjoint

    cfg = C.get("droplet256", ni=64, nj=32, nk=32, checker_cells=4)
    st0 = C.raw_state(cfg)
    walls = [w.copy() for w in C.wall_arrays(cfg)]
    out = {}
    for f32 in ("0", "1"):
        monkeypatch.setenv("FMF_ADJ_F32_REVERSE", f32)
        A = Adjoint(cfg, sor_tol=1e-3, sor_max=21, adj_tol=1e-10, adj_max=400, precision=capi.FMF_MIXED)
        monkeypatch.delenv("FMF_ADJ_F32_REVERSE")
        try:
            out[f32] = A.rollout(K, st0, walls)
        finally:
            A.close()
    (J64, g64), (J32, g32) = out["0"], out["1"]
    assert J32 == J64
    for name, a, b in zip(("theta0", "zeta", "l1", "l2", "phi"), g32, g64):
        scale = np.abs(b).max()
        assert scale > 0.0, name
        assert np.abs(a - b).max() <= 1e-6 * scale, (name, np.abs(a - b).max() / scale)
