"""Adjoint of the K-step rollout (fmf_adj_*) against central finite differences.

The objective is the reference's find_interface_positions_lower of phi after K
steps; the parameters are the per-wall-cell static angle theta0, the GNBC
coefficient zeta, the slip lengths l1, l2 and the initial phi.  The viscous solve
runs to 1e-13 so that the forward map is the exactly solved one the adjoint
differentiates.  Finite differences (central, Richardson-extrapolated from h and
h/2): of the GPU forward (tolerance 1e-6 relative) and of the CPU oracle, the
reference restated (tolerance 2e-6: the oracle's parity with the GPU, ~1e-10 in
J, limits its difference quotients).
"""
import ctypes

import numpy as np
import pytest

from fmf import config as C

pytestmark = pytest.mark.gpu

K = 8
SOR_TOL = 1e-13


@pytest.fixture(scope="module")
def setup(fmf_lib):
    from fmf.adjoint import Adjoint

    cfg = C.get("couette128", ni=32, nj=16, nk=16)
    adj = Adjoint(cfg, sor_tol=SOR_TOL, sor_max=300, adj_tol=1e-13, adj_max=400)
    st0 = C.raw_state(cfg)
    walls = [w.copy() for w in C.wall_arrays(cfg)]
    J, grads = adj.rollout(K, st0, walls)
    yield cfg, adj, st0, walls, J, grads
    adj.close()


def _directions(cfg, st0):
    rng = np.random.default_rng(11)
    jl, jh = 3, cfg.nj + 2
    out = []
    d = np.zeros(cfg.shape)
    d[3:-3, jl, 3:-3] = rng.normal(size=(cfg.nk, cfg.ni))
    out.append(("theta0", 0, d, 0.05))
    d = np.zeros(cfg.shape)
    d[:, jl, :] = 1.0
    d[:, jh, :] = 1.0
    out.append(("zeta", 1, d, 1e-3))
    out.append(("l1", 2, d.copy(), 1e-3))
    out.append(("l2", 3, d.copy(), 1e-3))
    phi1 = st0[C.STATE_FIELDS.index("phi1")]
    band = (phi1 > 0.02) & (phi1 < 0.98)
    for ax in range(3):
        sl = [slice(None)] * 3
        sl[ax] = slice(0, 3)
        band[tuple(sl)] = False
        sl[ax] = slice(-3, None)
        band[tuple(sl)] = False
    out.append(("phi", 4, np.where(band, rng.normal(size=cfg.shape), 0.0), 1e-4))
    return out


def _perturbed(st0, walls, which, d, h):
    w2 = [w.copy() for w in walls]
    s2 = st0.copy()
    if which < 4:
        w2[which] = w2[which] + h * d
    else:
        s2[C.STATE_FIELDS.index("phi1")] += h * d
    return s2, w2


def test_forward_matches_oracle(setup, orc):
    cfg, adj, st0, walls, J, _ = setup
    Jo = _oracle_J(orc, cfg, st0, walls)
    assert abs(adj.forward(K, st0, walls) - J) <= 1e-14 * max(abs(J), 1e-300) + 1e-22
    assert abs(J - Jo) <= 1e-10 * abs(Jo), (J, Jo)


def _oracle_J(orc, cfg, st0, walls):
    L = orc.lib()
    L.orc_set_sor.argtypes = [ctypes.c_double, ctypes.c_int]
    L.orc_set_sor(SOR_TOL, 300)
    try:
        s = orc.Solver(cfg)
        st = st0.copy()
        th, ze, l1, l2 = walls
        L.orc_init_bc(s.ws, s._ptrs(st), orc.P(th), orc.P(ze), orc.P(l1), orc.P(l2))
        s.walls = walls
        s.step(st, K)
        v = L.orc_interface_lower(orc.I(cfg.ni), orc.I(cfg.nj), orc.I(cfg.nk), orc.P(st[8]), orc.D(cfg.dx),
                                  orc.D(cfg.dx * cfg.ni))
        s.close()
        return v
    finally:
        L.orc_set_sor(1e-3, 21)


@pytest.mark.parametrize("idx", range(5))
def test_gradient_vs_gpu_finite_differences(setup, idx):
    cfg, adj, st0, walls, J, grads = setup
    label, which, d, h = _directions(cfg, st0)[idx]
    ga = float((grads[which] * d).sum())
    fd = []
    for hh in (h, h / 2):
        jp = adj.forward(K, *_perturbed(st0, walls, which, d, hh))
        jm = adj.forward(K, *_perturbed(st0, walls, which, d, -hh))
        fd.append((jp - jm) / (2 * hh))
    rich = (4 * fd[1] - fd[0]) / 3
    assert abs(ga - rich) <= 1e-6 * abs(rich), (label, ga, rich, fd)


@pytest.mark.parametrize("idx", [0, 1, 4])
def test_gradient_vs_oracle_finite_differences(setup, orc, idx):
    cfg, adj, st0, walls, J, grads = setup
    label, which, d, h = _directions(cfg, st0)[idx]
    h = 4.0 * h  # the oracle's J carries ~1e-16 of solver noise: a wider step
    ga = float((grads[which] * d).sum())
    fd = []
    for hh in (h, h / 2):
        jp = _oracle_J(orc, cfg, *_perturbed(st0, walls, which, d, hh))
        jm = _oracle_J(orc, cfg, *_perturbed(st0, walls, which, d, -hh))
        fd.append((jp - jm) / (2 * hh))
    rich = (4 * fd[1] - fd[0]) / 3
    assert abs(ga - rich) <= 2e-6 * abs(rich), (label, ga, rich, fd)


def test_checkpoint_interval_does_not_change_gradient(setup):
    cfg, adj, st0, walls, J, grads = setup
    J1, g1 = adj.rollout(K, st0, walls, every=1)
    J3, g3 = adj.rollout(K, st0, walls, every=3)
    assert J1 == J and J3 == J
    for a, b, c in zip(grads, g1, g3):
        scale = max(np.abs(a).max(), 1e-300)
        # the reverse kernels scatter with atomic adds: equal up to the order of additions
        assert np.abs(a - b).max() <= 1e-10 * scale
        assert np.abs(a - c).max() <= 1e-10 * scale


def test_overlapped_recomputation_matches_serial(setup, monkeypatch):
    """Segments recomputed by the second handle beside the reverse steps (the default)
    and recomputed in line (FMF_ADJ_SERIAL) give the same J and gradients."""
    cfg, adj, st0, walls, J, grads = setup
    Jo, go = adj.rollout(K, st0, walls, every=2)
    monkeypatch.setenv("FMF_ADJ_SERIAL", "1")
    Js, gs = adj.rollout(K, st0, walls, every=2)
    monkeypatch.delenv("FMF_ADJ_SERIAL")
    assert Jo == J and Js == J
    for a, b, c in zip(grads, go, gs):
        scale = max(np.abs(a).max(), 1e-300)
        assert np.abs(b - c).max() <= 1e-10 * scale
        assert np.abs(a - b).max() <= 1e-10 * scale


def test_torch_autograd_function(setup):
    torch = pytest.importorskip("torch")
    from fmf.adjoint import rollout_function

    cfg, adj, st0, walls, J, grads = setup
    fn = rollout_function(adj, K, st0)
    ts = [torch.tensor(w, requires_grad=True) for w in walls]
    phi = torch.tensor(st0[C.STATE_FIELDS.index("phi1")], requires_grad=True)
    out = fn(*ts, phi)
    out.backward()
    assert abs(out.item() - J) <= 1e-15 * max(abs(J), 1e-300)
    for t, g in zip(ts + [phi], grads):
        assert np.abs(t.grad.numpy() - g).max() <= 1e-10 * max(np.abs(g).max(), 1e-300)


def test_carried_terms_in_forward_and_reverse(setup, monkeypatch):
    """The adjoint's forward steps take the previous step's advection of (u, v, w)
    and surface tension of phin(1) for (uo, vo, wo) and phi(1), as the product step
    does.  A handle that recomputes both every step (FMF_STEP_CACHE=0) gives the
    same J bit for bit and the same gradients up to the order of the reverse's
    atomic additions."""
    from fmf.adjoint import Adjoint

    cfg, adj, st0, walls, J, grads = setup
    monkeypatch.setenv("FMF_STEP_CACHE", "0")
    b = Adjoint(cfg, sor_tol=SOR_TOL, sor_max=300, adj_tol=1e-13, adj_max=400)
    monkeypatch.delenv("FMF_STEP_CACHE")
    try:
        assert b.forward(K, st0, walls) == adj.forward(K, st0, walls)
        Jb, gb = b.rollout(K, st0, walls, every=3)
    finally:
        b.close()
    assert Jb == J
    for a_, b_ in zip(grads, gb):
        scale = max(np.abs(a_).max(), 1e-300)
        assert np.abs(a_ - b_).max() <= 1e-10 * scale
