"""The adjoint gradient of the K-step rollout against central finite differences of
the GPU forward at a workload's full size (the test suite checks a reduced grid,
where differences resolve the derivative to 1e-9):

    python -m fmf.validate_adjoint couette128 200 16 16

arguments: workload, K, checkpoint interval, number of directions.  Directions are
seeded and cycle over theta0 (per wall cell), zeta, l1, l2 (wall planes) and the
initial phi (interface band), each scaled to a largest entry of 1.  For each the
adjoint's directional derivative <grad J, d> is compared with the central
difference (J(p + h d) - J(p - h d)) / 2h at h = 1e-6.  Every viscous solve runs a
fixed 60 outer iterations (about three times what a relative tolerance of 1e-13
takes here), so that every evaluation of J is the same map, the exactly solved one
the adjoint differentiates (with a relative stopping rule the iteration count can
differ between J(p + h d) and J(p - h d)).  After 200 steps J still carries
rounding noise of order 1e-14 relative (switches at the rounding level: the Newton
exit, snaps and clips of phi), which the difference divides by 2h; its size is
estimated per direction as |FD(1e-6) - FD(2e-6)| (the truncation error at these
steps is far below it); the resolution of the differences is the largest such
estimate over the directions, in absolute terms (J's noise does not depend on the
direction, but one pair of differences can undershoot it).  Larger steps cross the
map's discrete switches within 200 steps.  Prints one line per direction; exits
non-zero when a direction's adjoint differs from FD(1e-6) by more than 1e-6
relative and more than twice that resolution.  Needs a GPU.
"""
import sys
import time

import numpy as np

from . import build
from . import config as C
from .adjoint import Adjoint

KINDS = ("theta0", "zeta", "l1", "l2", "phi")
H1, H2 = 1e-6, 2e-6


def directions(cfg, st0, ndir, seed=2024):
    rng = np.random.default_rng(seed)
    jl, jh = 3, cfg.nj + 2  # j = 1 and j = nj in the halo'd arrays
    phi1 = st0[C.STATE_FIELDS.index("phi1")]
    band = (phi1 > 0.02) & (phi1 < 0.98)
    for ax in range(3):
        sl = [slice(None)] * 3
        sl[ax] = slice(0, 3)
        band[tuple(sl)] = False
        sl[ax] = slice(-3, None)
        band[tuple(sl)] = False
    out = []
    for t in range(ndir):
        kind = KINDS[t % len(KINDS)]
        d = np.zeros(cfg.shape)
        if kind == "phi":
            d = np.where(band, rng.normal(size=cfg.shape), 0.0)
        else:
            for jw in (jl, jh):
                d[3:-3, jw, 3:-3] = rng.normal(size=(cfg.nk, cfg.ni))
        d /= np.abs(d).max()
        out.append((kind, d))
    return out


def perturbed(st0, walls, kind, d, h):
    w2 = [w.copy() for w in walls]
    s2 = st0.copy()
    if kind == "phi":
        s2[C.STATE_FIELDS.index("phi1")] += h * d
    else:
        w2[KINDS.index(kind)] = w2[KINDS.index(kind)] + h * d
    return s2, w2


def run(name, K, every, ndir):
    build.build()
    cfg = C.get(name)
    st0 = C.raw_state(cfg)
    walls = [w.copy() for w in C.wall_arrays(cfg)]
    A = Adjoint(cfg, sor_tol=1e-300, sor_max=60, adj_tol=1e-13, adj_max=4000)
    t0 = time.perf_counter()
    J, grads = A.rollout(K, st0, walls, every=every)
    print(f"{name} {cfg.ni}x{cfg.nj}x{cfg.nk} K={K} every={every}: J = {J:.15e} "
          f"(rollout {time.perf_counter() - t0:.1f} s, iterations {A.iterations()})", flush=True)
    rows = []
    for t, (kind, d) in enumerate(directions(cfg, st0, ndir)):
        g = float((grads[KINDS.index(kind)] * d).sum())
        fd = {}
        for h in (H1, H2):
            jp = A.forward(K, *perturbed(st0, walls, kind, d, h))
            jm = A.forward(K, *perturbed(st0, walls, kind, d, -h))
            fd[h] = (jp - jm) / (2 * h)
        rows.append((t, kind, g, fd[H1], abs(fd[H1] - fd[H2])))
        print(f"direction {t:2d} {kind:6s}: adjoint {g:+.12e}  FD(h=1e-6) {fd[H1]:+.12e}  "
              f"|diff| {abs(g - fd[H1]):.1e} (rel {abs(g - fd[H1]) / max(abs(fd[H1]), 1e-300):.1e})  "
              f"|FD(1e-6) - FD(2e-6)| {abs(fd[H1] - fd[H2]):.1e}", flush=True)
    A.close()
    res = max(r[4] for r in rows)
    bad = [r[0] for r in rows if abs(r[2] - r[3]) > max(1e-6 * abs(r[3]), 2 * res)]
    big = max(abs(r[3]) for r in rows)
    worst = max(abs(r[2] - r[3]) for r in rows)
    print(f"FD resolution {res:.1e}; largest |adjoint - FD| {worst:.1e} ({worst / big:.1e} of the largest "
          f"directional derivative); directions outside max(1e-6 relative, 2 x resolution): {bad or 'none'}")
    return len(bad)

if __name__ == "__main__":
    name = sys.argv[1] if len(sys.argv) > 1 else "couette128"
    K = int(sys.argv[2]) if len(sys.argv) > 2 else 200
    every = int(sys.argv[3]) if len(sys.argv) > 3 else 16
    ndir = int(sys.argv[4]) if len(sys.argv) > 4 else 16
    sys.exit(1 if run(name, K, every, ndir) else 0)
