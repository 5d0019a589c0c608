"""Mixed-precision step (FP32 WENO5, MTHINC Newton/fluxes and SOR sweeps; FP64
pressure solve, projection, divergence, volume sums and state storage) against
the FP64 GPU step from the same initial state: phi, u, v, w, p within 1e-5
relative after N steps, identical SOR iteration counts, phi volume conserved."""
import numpy as np
import pytest

from fmf import capi
from fmf import config as C

pytestmark = pytest.mark.gpu

TOL = 1e-5
FIELDS = {"u": 0, "v": 1, "w": 2, "p": 6, "phi": 9}


def _run(cfg, precision, steps, st0):
    g = capi.Stepper(cfg, precision=precision)
    g.upload(st0)
    g.step(steps)
    out = g.get_state()
    it = g.sor_iterations()
    g.close()
    return out, it


def _relerr(a, b):
    return np.abs(C.interior(a) - C.interior(b)).max() / max(np.abs(C.interior(b)).max(), 1e-30)


# the full 256x128x128 Couette case for 30 steps: its linear velocity profile makes
# all three FP32 smoothness indicators of some lines exactly 0 (first at step 15)
@pytest.mark.parametrize("name,shape,steps", [("couette256", (128, 64, 64), 20), ("couette256", (256, 128, 128), 30),
                                              ("droplet256", (64, 32, 32), 10)])
def test_mixed_matches_fp64(fmf_lib, name, shape, steps):
    cfg = C.get(name, ni=shape[0], nj=shape[1], nk=shape[2])
    g = capi.Stepper(cfg)
    st0 = g.initial_state()
    g.close()
    ref, it_ref = _run(cfg, capi.FMF_FP64, steps, st0)
    mix, it_mix = _run(cfg, capi.FMF_MIXED, steps, st0)
    assert np.isfinite(mix).all()
    errs = {k: _relerr(mix[f], ref[f]) for k, f in FIELDS.items()}
    for k, e in errs.items():
        assert e <= TOL, (k, errs)
    assert it_mix == it_ref
    v0 = C.interior(st0[9]).sum()
    assert abs(C.interior(mix[9]).sum() - v0) <= 1e-11 * v0
