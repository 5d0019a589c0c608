"""The reference's run-time monitors on the GPU (cal_vel.f, cal_center.f,
find_interface_positions_upper.f90 / _lower.f90): the drop-ins (host arrays,
Fortran argument lists) and the fmf_dev_* variants (device arrays, results left
in device memory) against the CPU oracle on the same seeded inputs.

The sums are reduced in a different order on the GPU, so the tolerance is
REL = 1e-12 relative; the crossing positions are computed operation by operation
as the oracle computes them and must agree to REL as well; counts, print order
and the integer state of cal_center must match exactly."""
import ctypes

import numpy as np
import pytest

from fmf import config as C

pytestmark = pytest.mark.gpu

REL = 1e-12
NI, NJ, NK = 32, 16, 16
SH = (NK + 6, NJ + 6, NI + 6)
DX = 2.0 / NI
VP, IP, DP = ctypes.c_void_p, ctypes.c_int, ctypes.c_double


@pytest.fixture(scope="module")
def L(fmf_lib):
    from fmf import capi
    fmf_lib.fmf_set_mode(capi.FMF_COHERENT)
    fmf_lib.fmf_reset()
    fmf_lib.fmf_dev_cal_vel.argtypes = [IP, IP, IP, DP, DP, DP, VP, VP, VP, VP, VP]
    fmf_lib.fmf_dev_cal_center_sums.argtypes = [IP, IP, IP, IP, DP, DP, IP, IP, VP, VP]
    fmf_lib.fmf_dev_interface_upper.argtypes = [IP, IP, IP, VP, DP, DP, DP, VP, VP, IP]
    fmf_lib.fmf_dev_interface_lower.argtypes = [IP, IP, IP, VP, DP, DP, VP]
    yield fmf_lib
    fmf_lib.fmf_reset()
    fmf_lib.fmf_set_mode(capi.FMF_RESIDENT)


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def stripes(seed):
    """phi with three liquid stripes along x (several crossings per row), tilted in
    z, plus noise away from 0.5."""
    rng = np.random.default_rng(seed)
    x = (np.arange(-2, NI + 4) - 0.5) * DX
    z, y, xx = np.meshgrid(np.arange(SH[0]), np.arange(SH[1]), x, indexing="ij")
    s = np.sin(2 * np.pi * (3 * xx / 2.0 + 0.05 * z + 0.02 * y))
    return 0.5 * (1 + np.tanh(4 * s)) + 0.01 * rng.normal(size=SH)


def blob(x0, x_len=2.0):
    """A smooth drop of phi centred at x0 (periodic in x)."""
    x = (np.arange(-2, NI + 4) - 0.5) * DX
    yc = (np.arange(-2, NJ + 4) - 0.5) * (1.0 / NJ)
    zc = (np.arange(-2, NK + 4) - 0.5) * (1.0 / NK)
    z, y, xx = np.meshgrid(zc, yc, x, indexing="ij")
    dxp = (xx - x0 + x_len / 2) % x_len - x_len / 2
    r = np.sqrt(dxp ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2)
    return 0.5 * (1 + np.tanh((0.3 - r) / 0.05))


def test_cal_vel_dropin(orc, L):
    rng = np.random.default_rng(11)
    u, v, w = (rng.normal(size=SH) for _ in range(3))
    phi = stripes(1)
    I, D, P = orc.I, orc.D, orc.P
    vo, ro = np.zeros(3), np.zeros(3)
    orc.lib().orc_cal_vel(I(0), I(NI), I(NJ), I(NK), D(0.25), D(2.0), D(0.1), P(u), P(v), P(w), P(phi), P(vo), P(ro))
    vg, rg = np.zeros(3), np.zeros(3)
    L.cal_vel_(I(0), I(NI), I(NJ), I(NK), D(0.25), D(2.0), D(0.1), P(u), P(v), P(w), P(phi), P(vg), P(rg))
    assert L.fmf_last_error() == 0
    assert rel(vg, vo) <= REL and rel(rg, ro) <= REL


class State:
    def __init__(self):
        self.pre1, self.pre2, self.vel = DP(0.0), DP(0.0), DP(0.0)
        self.a1, self.a2, self.lap = IP(2), IP(2), IP(0)

    def args(self, center):
        return [center.ctypes.data_as(VP), ctypes.byref(self.pre1), ctypes.byref(self.pre2), ctypes.byref(self.a1),
                ctypes.byref(self.a2), ctypes.byref(self.lap), ctypes.byref(self.vel)]

    def ints(self):
        return self.a1.value, self.a2.value, self.lap.value


def test_cal_center_dropin_sequence(orc, L):
    """A drop carried in +x over 1.5 periods: the oracle and the drop-in advance
    their own (center_pre, area_pre, lap) state and must agree at every call."""
    xl, yl, dt = 2.0, 1.0, 0.05
    I, D, P = orc.I, orc.D, orc.P
    so, sg = State(), State()
    for step in range(40):
        phi = blob(0.3 + 0.075 * step)
        co, cg = np.zeros(3), np.zeros(3)
        common = [I(0), I(0), I(NJ), I(NI), I(NJ), I(NK), D(xl), D(yl), D(1.0), D(dt), D(1.0), P(phi)]
        orc.lib().orc_cal_center(*common, *so.args(co))
        L.cal_center_(*common, *sg.args(cg))
        assert L.fmf_last_error() == 0
        assert rel(cg, co) <= REL, step
        assert abs(sg.vel.value - so.vel.value) <= REL * max(abs(so.vel.value), 1.0) / dt, step
        assert sg.ints() == so.ints(), step
    assert so.lap.value >= 1  # the drop crossed x = xl


def _printed(capfd):
    ctypes.CDLL(None).fflush(None)
    return capfd.readouterr().out


def test_interface_dropins(orc, L, capfd):
    phi = stripes(2)
    I, D, P = orc.I, orc.D, orc.P
    cap = NI * NK
    xz = np.zeros(2 * cap)
    n = orc.lib().orc_interface_upper(I(NI), I(NJ), I(NK), P(phi), D(DX), D(1.0 / NK), D(2.0), P(xz), IP(cap))
    assert n > NK  # several crossings per row
    _printed(capfd)
    L.find_interface_positions_upper_(I(NI), I(NJ), I(NK), P(phi), D(DX), D(1.0 / NJ), D(1.0 / NK), D(2.0))
    assert L.fmf_last_error() == 0
    got = np.array([[float(t) for t in line.split()] for line in _printed(capfd).splitlines() if line.strip()])
    assert got.shape == (n, 2)
    assert rel(got, xz[:2 * n].reshape(-1, 2)) <= REL
    orc.lib().orc_interface_lower.restype = ctypes.c_double
    lo = orc.lib().orc_interface_lower(I(NI), I(NJ), I(NK), P(phi), D(DX), D(2.0))
    L.find_interface_positions_lower_(I(NI), I(NJ), I(NK), P(phi), D(DX), D(1.0 / NJ), D(1.0 / NK), D(2.0))
    assert L.fmf_last_error() == 0
    out = _printed(capfd).split()
    assert abs(float(out[-1]) - lo) <= REL * max(abs(lo), 1.0)


def test_device_variants(orc, L):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    u, v, w = (rng.normal(size=SH) for _ in range(3))
    phi = stripes(3)
    dev = [torch.from_numpy(a).cuda() for a in (u, v, w, phi)]
    out6 = torch.zeros(6, dtype=torch.float64, device="cuda")
    out4 = torch.zeros(4, dtype=torch.float64, device="cuda")
    out1 = torch.zeros(1, dtype=torch.float64, device="cuda")
    cap = NI * NK
    xz = torch.zeros(2 * cap, dtype=torch.float64, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ptr = [t.data_ptr() for t in dev]
    L.fmf_dev_cal_vel(NI, NJ, NK, 0.25, 2.0, 0.1, *ptr, out6.data_ptr())
    L.fmf_dev_cal_center_sums(NI, NJ, NK, 0, 1.0 / NJ, 2.0, 3, 1, ptr[3], out4.data_ptr())
    L.fmf_dev_interface_upper(NI, NJ, NK, ptr[3], DX, 1.0 / NK, 2.0, xz.data_ptr(), cnt.data_ptr(), cap)
    L.fmf_dev_interface_lower(NI, NJ, NK, ptr[3], DX, 2.0, out1.data_ptr())
    assert L.fmf_device_synchronize() == 0
    I, D, P = orc.I, orc.D, orc.P
    vo, ro = np.zeros(3), np.zeros(3)
    orc.lib().orc_cal_vel(I(0), I(NI), I(NJ), I(NK), D(0.25), D(2.0), D(0.1), P(u), P(v), P(w), P(phi), P(vo), P(ro))
    g6 = out6.cpu().numpy()
    assert rel(g6[:3], vo) <= REL and rel(g6[3:], ro) <= REL
    # cal_center.f:36-76 sums for area_pre1 = 3, lap = 1 (x below xl/4 moves up by xl)
    delta, xl = 1.0 / NJ, 2.0
    p = phi[3:NK + 3, 3:NJ + 3, 3:NI + 3]
    k, j, i = np.meshgrid(np.arange(1, NK + 1), np.arange(1, NJ + 1), np.arange(1, NI + 1), indexing="ij")
    x = delta * (i - 0.5)
    x = np.where(x < 0.25 * xl, x + xl, x) + xl
    ref4 = np.array([p.sum(), (p * x).sum(), (p * delta * (j - 0.5)).sum(), (p * delta * (k - 0.5)).sum()])
    assert rel(out4.cpu().numpy(), ref4) <= REL
    xo = np.zeros(2 * cap)
    n = orc.lib().orc_interface_upper(I(NI), I(NJ), I(NK), P(phi), D(DX), D(1.0 / NK), D(2.0), P(xo), IP(cap))
    assert int(cnt.item()) == n
    assert rel(xz.cpu().numpy()[:2 * n], xo[:2 * n]) <= REL
    orc.lib().orc_interface_lower.restype = ctypes.c_double
    lo = orc.lib().orc_interface_lower(I(NI), I(NJ), I(NK), P(phi), D(DX), D(2.0))
    assert abs(out1.item() - lo) <= REL * max(abs(lo), 1.0)
