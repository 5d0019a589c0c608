"""Field output on the GPU (mkvtk_*.f, mk_slice_j/k.f, mk_all.f) against the CPU
oracle on the same seeded fields.  The ghost fills and 8-point means run in the
reference's operation order without multiply-add contraction, so the values are
bit-identical: the VTK files must match byte for byte, the arrays exactly."""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MI, MJ, MK = 32, 16, 16
SH = (MK + 6, MJ + 6, MI + 6)
VP, IP, DP = ctypes.c_void_p, ctypes.c_int, ctypes.c_double


@pytest.fixture(scope="module")
def L(fmf_lib):
    from fmf import capi
    fmf_lib.fmf_set_mode(capi.FMF_COHERENT)
    fmf_lib.fmf_reset()
    yield fmf_lib
    fmf_lib.fmf_reset()
    fmf_lib.fmf_set_mode(capi.FMF_RESIDENT)


def R(x):
    return ctypes.byref(x)


def _files(d):
    return {n: open(os.path.join(d, n), "rb").read() for n in sorted(os.listdir(d))}


@pytest.mark.parametrize("kind,name", [(0, "mkvtk_phi"), (1, "mkvtk_phil"), (2, "mkvtk_p")])
def test_vtk_scalar_files(orc, L, tmp_path, monkeypatch, kind, name):
    rng = np.random.default_rng(20 + kind)
    q = rng.random(SH) * 2.0 - 0.5
    q[5, 7, 9] = 3e-120  # a three-digit exponent
    svall = (ctypes.c_int * 3)(MI, MJ, MK)
    qo, qg = q.copy(), q.copy()
    os.makedirs(tmp_path / "orc")
    os.makedirs(tmp_path / "gpu")
    monkeypatch.chdir(tmp_path / "orc")
    assert orc.lib().orc_mkvtk(kind, svall, orc.I(12), orc.D(0.0625), orc.D(0.0625), orc.D(0.0625), orc.P(qo),
                               orc.I(1)) == 0
    monkeypatch.chdir(tmp_path / "gpu")
    args = [svall, R(IP(12)), R(DP(0.0625)), R(DP(0.0625)), R(DP(0.0625)), qg.ctypes.data_as(VP)]
    if kind == 1:
        args.append(R(IP(1)))
    getattr(L, name + "_")(*args)
    assert L.fmf_last_error() == 0
    fo, fg = _files(tmp_path / "orc"), _files(tmp_path / "gpu")
    assert list(fo) == list(fg) and len(fo) == 1
    for n in fo:
        assert fo[n] == fg[n], n
    assert np.array_equal(qo, qg)  # the ghosts the reference fills in place


def test_vtk_q_files(orc, L, tmp_path, monkeypatch):
    rng = np.random.default_rng(30)
    vorx, q = rng.normal(size=SH), rng.normal(size=SH)
    svall = (ctypes.c_int * 3)(MI, MJ, MK)
    os.makedirs(tmp_path / "orc")
    os.makedirs(tmp_path / "gpu")
    monkeypatch.chdir(tmp_path / "orc")
    assert orc.lib().orc_mkvtk_q(svall, orc.I(5), orc.D(0.0625), orc.D(0.0625), orc.D(0.0625), orc.P(vorx),
                                 orc.P(q)) == 0
    monkeypatch.chdir(tmp_path / "gpu")
    L.mkvtk_q_(svall, R(IP(5)), R(DP(0.0625)), R(DP(0.0625)), R(DP(0.0625)), vorx.ctypes.data_as(VP),
               q.ctypes.data_as(VP))
    assert L.fmf_last_error() == 0
    fo, fg = _files(tmp_path / "orc"), _files(tmp_path / "gpu")
    assert list(fo) == ["q1_0000005.vtk", "q2_0000005.vtk"] == list(fg)
    for n in fo:
        assert fo[n] == fg[n], n


@pytest.mark.parametrize("axis", [1, 2])
def test_slices(orc, L, axis):
    rng = np.random.default_rng(40 + axis)
    q = rng.normal(size=SH)
    nid = (ctypes.c_int * 6)(*([-1] * 6))
    n = MK if axis == 1 else MJ
    for fixed, off in ((MJ // 2 if axis == 1 else MK // 2, (0, 1, 1)), (3, (1, 1, 0)), (1, (1, 1, 1))):
        so = np.zeros((n + 1, MI + 1))
        sg, wg = np.full((n + 1, MI + 1), 7.0), np.full((n + 1, MI + 1), 7.0)
        orc.lib().orc_mk_slice(axis, nid, orc.I(MI), orc.I(MJ), orc.I(MK), orc.I(fixed), orc.I(off[0]),
                               orc.I(off[1]), orc.I(off[2]), orc.P(q), orc.P(so))
        fn = L.mk_slice_j_ if axis == 1 else L.mk_slice_k_
        fn(R(IP(0)), R(IP(0)), nid, R(IP(1)), R(IP(MI)), R(IP(MJ)), R(IP(MK)), R(IP(fixed)), R(IP(off[0])),
           R(IP(off[1])), R(IP(off[2])), wg.ctypes.data_as(VP), q.ctypes.data_as(VP), sg.ctypes.data_as(VP))
        assert L.fmf_last_error() == 0
        assert np.array_equal(sg, so) and np.array_equal(wg, so)


def test_mk_all(L):
    rng = np.random.default_rng(50)
    q = rng.normal(size=SH)
    a, w = np.zeros(SH), np.zeros(SH)
    nid = (ctypes.c_int * 6)(*([-1] * 6))
    L.mk_all_(R(IP(0)), R(IP(0)), nid, R(IP(1)), R(IP(MI)), R(IP(MJ)), R(IP(MK)), w.ctypes.data_as(VP),
              q.ctypes.data_as(VP), a.ctypes.data_as(VP))
    assert L.fmf_last_error() == 0
    assert np.array_equal(a, q) and np.array_equal(w, q)
