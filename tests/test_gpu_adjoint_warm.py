"""The transposed viscous solve of each reverse step starts from the previous
one's feedback term (lam = lout + G^T lam_prev) and scales its stop rule by that
term's norm.  Against handles whose solves all start cold (FMF_ADJ_WARM=0 at
creation), on the 128x64x64 Couette workload at 64x32x32 (angle 75 +- 5 deg), K =
24 steps, checkpoints every 5: the gradients agree within 20x the solve tolerance
of their largest magnitude (1e-6: the tolerance the cost measurement uses; 1e-10),
J is the same, and the warm start takes no more transposed iterations in total."""
import numpy as np
import pytest

from fmf import config as C

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("adj_tol", [1e-6, 1e-10])
def test_warm_started_transposed_solve(fmf_lib, monkeypatch, adj_tol):
    from fmf.adjoint import Adjoint

    cfg = C.get("couette128", ni=64, nj=32, nk=32)
    st0 = C.raw_state(cfg)
    walls = [w.copy() for w in C.wall_arrays(cfg)]
    K, every = 24, 5
    out = {}
    for warm in ("0", "1"):
        monkeypatch.setenv("FMF_ADJ_WARM", warm)
        A = Adjoint(cfg, sor_tol=1e-3, sor_max=21, adj_tol=adj_tol, adj_max=400)
        monkeypatch.delenv("FMF_ADJ_WARM")
        try:
            J, g = A.rollout(K, st0, walls, every)
            out[warm] = (J, g, A.iterations()[1])
        finally:
            A.close()
    (Jc, gc, itc), (Jw, gw, itw) = out["0"], out["1"]
    assert Jc == Jw
    assert itw <= itc, (itw, itc)
    for name, a, b in zip(("theta0", "zeta", "l1", "l2", "phi"), gw, gc):
        scale = np.abs(b).max()
        assert scale > 0.0, name
        assert np.abs(a - b).max() <= 20 * adj_tol * scale, (name, np.abs(a - b).max() / scale)
