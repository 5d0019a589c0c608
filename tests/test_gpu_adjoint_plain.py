"""The adjoint's forward steps that no reverse step reads (all steps of
fmf_adj_forward, the rollout's steps before its last checkpoint segment) run on the
product step (fmf_ctx: graph-replayed, pointer rotation, no record copies).  It runs
the same kernels in the same order as the recording step, so a handle that records
every step (FMF_ADJ_RECORD_ALL set when it is created) must give the same final
state and J bit for bit, the same viscous iteration counts, and the same gradients
up to the rounding of their atomic sums (1e-12 of each gradient's largest
magnitude), in both precisions."""
import numpy as np
import pytest

from fmf import config as C

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_plain_forward_steps_match_recorded(fmf_lib, monkeypatch, precision):
    from fmf.adjoint import Adjoint

    if precision == 0:
        cfg = C.get("couette128", ni=32, nj=16, nk=16)
    else:
        cfg = C.get("droplet256", ni=64, nj=32, nk=32, checker_cells=4)
    st0 = C.raw_state(cfg)
    walls = [w.copy() for w in C.wall_arrays(cfg)]
    K, every = 12, 4
    monkeypatch.setenv("FMF_ADJ_RECORD_ALL", "1")
    rec = Adjoint(cfg, sor_tol=1e-3, sor_max=21, adj_tol=1e-10, adj_max=400, precision=precision)
    monkeypatch.delenv("FMF_ADJ_RECORD_ALL")
    plain = Adjoint(cfg, sor_tol=1e-3, sor_max=21, adj_tol=1e-10, adj_max=400, precision=precision)
    try:
        Jr, sr = rec.forward(K, st0, walls, want_state=True)
        Jp, sp = plain.forward(K, st0, walls, want_state=True)
        assert Jr == Jp
        for f, (a, b) in enumerate(zip(sr, sp)):
            assert np.array_equal(a, b), C.STATE_FIELDS[f]
        assert rec.iterations()[0] == plain.iterations()[0]
        Jr2, gr = rec.rollout(K, st0, walls, every)
        Jp2, gp = plain.rollout(K, st0, walls, every)
        assert Jr2 == Jr and Jp2 == Jr
        assert rec.iterations()[0] == plain.iterations()[0]
        for name, a, b in zip(("theta0", "zeta", "l1", "l2", "phi"), gr, gp):
            scale = np.abs(a).max()
            assert scale > 0.0, name
            assert np.abs(a - b).max() <= 1e-12 * scale, (name, np.abs(a - b).max() / scale)
        # the product step's buffers are part of the handle's device bytes
        assert plain.device_bytes() > rec.device_bytes()
    finally:
        rec.close()
        plain.close()
