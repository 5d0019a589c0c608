"""The adjoint gradient at the 128x64x64 Couette workload's size (per-wall-cell angle
75 +- 5 deg) against central finite differences of the GPU forward.

K = 50 steps, checkpoints every ceil(sqrt(50)) = 8, four seeded directions: theta0
(per wall cell), zeta and l1 (wall planes) and the initial phi (interface band),
each scaled to a largest entry of 1.  Every viscous solve runs a fixed 60 outer
iterations, so that each evaluation of J is the same map, the exactly solved one
the adjoint differentiates (a relative stopping rule can stop J(p + h d) and
J(p - h d) after different iteration counts).

Criterion (absolute, as differences allow at this size): for every direction
|<grad J, d> - FD(h)| <= max(1e-6 |FD(h)|, 2 r), with FD(h) = (J(p + h d) -
J(p - h d)) / 2h at h = 1e-6 and r = the largest |FD(1e-6) - FD(2e-6)| over the
directions.  r is the differences' own resolution: J carries rounding noise from
switches at the rounding level (the MTHINC Newton exit, the snaps and clips of
phi), about 1e-16 relative after these steps, which a central difference divides
by 2h, so on the smaller directional derivatives 1e-6 relative lies below what the
differences can resolve (the truncation error at these steps is far smaller).  The
reduced grid of test_gpu_adjoint.py holds the 1e-6 relative bar outright.
"""
import math

import numpy as np
import pytest

from fmf import config as C

pytestmark = pytest.mark.gpu

K = 50
H1, H2 = 1e-6, 2e-6


def test_gradient_c4_size(fmf_lib):
    from fmf.adjoint import Adjoint
    from fmf.validate_adjoint import KINDS, directions, perturbed

    cfg = C.get("couette128")
    st0 = C.raw_state(cfg)
    walls = [w.copy() for w in C.wall_arrays(cfg)]
    A = Adjoint(cfg, sor_tol=1e-300, sor_max=60, adj_tol=1e-13, adj_max=4000)
    try:
        J, grads = A.rollout(K, st0, walls, every=int(math.ceil(math.sqrt(K))))
        assert np.isfinite(J)
        picks = [d for d in directions(cfg, st0, 5) if d[0] in ("theta0", "zeta", "l1", "phi")]
        rows = []
        for kind, d in picks:
            g = float((grads[KINDS.index(kind)] * d).sum())
            fd = {}
            for h in (H1, H2):
                jp = A.forward(K, *perturbed(st0, walls, kind, d, h))
                jm = A.forward(K, *perturbed(st0, walls, kind, d, -h))
                fd[h] = (jp - jm) / (2 * h)
            rows.append((kind, g, fd[H1], abs(fd[H1] - fd[H2])))
    finally:
        A.close()
    res = max(r[3] for r in rows)
    for kind, g, fd, _ in rows:
        assert abs(g - fd) <= max(1e-6 * abs(fd), 2 * res), (kind, g, fd, res, rows)
    # the derivatives are resolved: the largest is far above the resolution
    assert max(abs(r[2]) for r in rows) > 100 * res, rows
