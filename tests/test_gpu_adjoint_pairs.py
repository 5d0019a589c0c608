"""The adjoint of the rollout with an FP64 forward runs its WENO5 reverse
(cal_advu_weno5.f:44-255, weno5.h:2-70 transposed) in FP32-pair arithmetic: the
walk's five differences taken in FP64 and split into pairs, R and dR/de of the FP64
walk formed in pairs (csrc/weno5_df.cuh's wrev_core, checked on the host against
long double in tests/test_df64_host.py).  Against the same handle with that reverse
in FP64 (FMF_ADJ_PAIR_REVERSE=0 at creation), on the sessile drop at 64x32x32
(density ratio 1000, checkerboard lower wall, fluid at rest at the start, so the
reverse meets flat stencils where the reference's 1e-80 alone weighs in) and on the
128x64x64 Couette workload scaled to 32x16x16 (per-wall-cell angles, moving walls):
the same J, bit for
bit (the forward is unchanged), and gradients within 1e-8 of their largest
magnitude (the transposed viscous solves stop at 1e-10 of their right-hand side, so
rounding-level changes to that side move the result by about that much)."""
import numpy as np
import pytest

from fmf import config as C

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,kw,K", [
    ("droplet256", dict(ni=64, nj=32, nk=32, checker_cells=4), 20),
    ("couette128", dict(ni=32, nj=16, nk=16), 8),
])
def test_pair_weno_reverse_matches_fp64_reverse(fmf_lib, monkeypatch, name, kw, K):
    from fmf import capi
    from fmf.adjoint import Adjoint

    cfg = C.get(name, **kw)
    st0 = C.raw_state(cfg)
    walls = [w.copy() for w in C.wall_arrays(cfg)]
    out = {}
    for pairs in ("0", "1"):
        monkeypatch.setenv("FMF_ADJ_PAIR_REVERSE", pairs)
        A = Adjoint(cfg, sor_tol=1e-3, sor_max=21, adj_tol=1e-10, adj_max=400, precision=capi.FMF_FP64)
        monkeypatch.delenv("FMF_ADJ_PAIR_REVERSE")
        try:
            out[pairs] = A.rollout(K, st0, walls)
        finally:
            A.close()
    (J64, g64), (Jp, gp) = out["0"], out["1"]
    assert Jp == J64
    for gname, a, b in zip(("theta0", "zeta", "l1", "l2", "phi"), gp, g64):
        scale = np.abs(b).max()
        assert scale > 0.0, gname
        assert np.isfinite(a).all(), gname
        assert np.abs(a - b).max() <= 1e-8 * scale, (gname, np.abs(a - b).max() / scale)
