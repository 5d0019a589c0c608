"""Field-output formats (no GPU): the library's and the oracle's Fortran Ew.d
formatters against hand-derived Fortran outputs, and the oracle's VTK writer
(mkvtk_phi.f) against a numpy restatement of its ghost fill and vertex means."""
import ctypes
import os

import numpy as np
import pytest

# (value, w, d, what a Fortran Ew.d edit descriptor writes)
CASES = [
    (1.0, 10, 3, " 0.100E+01"),
    (-1.0, 10, 3, "-0.100E+01"),
    (0.0, 10, 3, " 0.000E+00"),
    (123456.0, 10, 3, " 0.123E+06"),
    (9.9996, 10, 3, " 0.100E+02"),        # rounding carries into the exponent
    (1.5e-120, 10, 3, " 0.150-119"),      # three-digit exponent drops the E
    (-2.5e200, 10, 3, "-0.250+201"),
    (-1.0, 9, 3, "-.100E+01"),            # optional leading zero dropped
    (-1.0, 8, 3, "********"),             # does not fit
    (0.0625, 11, 4, " 0.6250E-01"),
    (1.0e-5, 11, 4, " 0.1000E-04"),
    (123.456, 20, 10, "    0.1234560000E+03"),
    (-0.1, 20, 10, "   -0.1000000000E+00"),
    (float("nan"), 10, 3, "       NaN"),
    (float("inf"), 10, 3, "  Infinity"),
    (-float("inf"), 10, 3, " -Infinity"),
]


@pytest.mark.parametrize("x,w,d,want", CASES)
def test_library_formatter(fmf_built, x, w, d, want):
    L = ctypes.CDLL(fmf_built)
    L.fmf_format_fortran_e.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int]
    buf = ctypes.create_string_buffer(64)
    assert L.fmf_format_fortran_e(buf, 64, x, w, d) == 0
    assert buf.value.decode() == want


@pytest.mark.parametrize("x,w,d,want", CASES)
def test_oracle_formatter(orc, x, w, d, want):
    buf = ctypes.create_string_buffer(64)
    orc.lib().orc_format_e(buf, ctypes.c_double(x), ctypes.c_int(w), ctypes.c_int(d))
    assert buf.value.decode() == want


def test_formatters_agree_on_random_values(fmf_built, orc):
    L = ctypes.CDLL(fmf_built)
    L.fmf_format_fortran_e.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(0)
    xs = rng.normal(size=2000) * 10.0 ** rng.integers(-150, 150, size=2000)
    a, b = ctypes.create_string_buffer(64), ctypes.create_string_buffer(64)
    for x in xs:
        for w, d in ((10, 3), (11, 4), (20, 10)):
            L.fmf_format_fortran_e(a, 64, float(x), w, d)
            orc.lib().orc_format_e(b, ctypes.c_double(float(x)), ctypes.c_int(w), ctypes.c_int(d))
            assert a.value == b.value, (x, w, d)


def test_oracle_vtk_phi(orc, tmp_path, monkeypatch):
    mi, mj, mk = 8, 4, 4
    rng = np.random.default_rng(1)
    q = rng.random((mk + 6, mj + 6, mi + 6))
    monkeypatch.chdir(tmp_path)
    svall = (ctypes.c_int * 3)(mi, mj, mk)
    qq = q.copy()
    assert orc.lib().orc_mkvtk(0, svall, orc.I(7), orc.D(0.25), orc.D(0.5), orc.D(0.5), orc.P(qq), orc.I(0)) == 0
    lines = open(os.path.join(tmp_path, "phi_0000007.vtk")).read().split("\n")
    assert lines[:11] == ["# vtk DataFile Version 2.0", "t=7", "ASCII", "DATASET STRUCTURED_POINTS",
                          "DIMENSIONS 9 5 5", "ORIGIN  0.0000E+00  0.0000E+00  0.0000E+00",
                          "ASPECT_RATIO  0.2500E+00  0.5000E+00  0.5000E+00", "", "POINT_DATA 225",
                          "SCALARS phi float", "LOOKUP_TABLE default"]
    vals = np.array([float(t) for t in lines[11:] if t])
    # numpy restatement: x periodic, y and z copies of the end rows, then vertex means
    r = q[2:mk + 4, 2:mj + 4, 2:mi + 4].copy()  # indices 0..m+1
    r[:, :, 0], r[:, :, mi + 1] = r[:, :, mi], r[:, :, 1]
    r[:, 0, :], r[:, mj + 1, :] = r[:, 1, :], r[:, mj, :]
    r[0, :, :], r[mk + 1, :, :] = r[1, :, :], r[mk, :, :]
    v = sum(r[a:a + mk + 1, b:b + mj + 1, c:c + mi + 1] for a in (0, 1) for b in (0, 1) for c in (0, 1)) * 0.125
    assert vals.size == v.size
    # e10.3 keeps 3 significant digits: |error| <= 0.5e-3 * 10^ex for 0.ddd x 10^ex
    ex = np.floor(np.log10(np.abs(v.ravel()))) + 1
    assert np.all(np.abs(vals - v.ravel()) <= 0.5e-3 * 10.0 ** ex * (1 + 1e-9))


def _run_in(path, monkeypatch):
    os.makedirs(path, exist_ok=True)
    monkeypatch.chdir(path)


def test_slice_files_and_logs_match_the_oracle(fmf_built, orc, tmp_path, monkeypatch):
    """uwphi/uvwp slice files and the center/velocity logs: the library's host
    writers and the oracle's produce the same bytes (values below 1e-40 written as 0)."""
    L = ctypes.CDLL(fmf_built)
    vp, dp, ip = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
    L.fmf_write_uwphi.argtypes = [ip, vp, dp, dp, vp, vp, vp]
    L.fmf_write_uvwp.argtypes = [ip, vp, dp, dp, vp, vp, vp]
    rng = np.random.default_rng(2)
    svall = (ctypes.c_int * 3)(8, 4, 4)
    s1, s2, s3 = (rng.normal(size=(5, 9)) for _ in range(3))
    s1[0, 0] = 1e-41  # clipped to 0
    vals = [rng.normal(size=3) for _ in range(3)]
    for who in ("lib", "orc"):
        _run_in(str(tmp_path / who), monkeypatch)
        for step in (3, 4):
            if who == "lib":
                assert L.fmf_write_uwphi(step, svall, 0.25, 0.5, s1.ctypes.data, s2.ctypes.data, s3.ctypes.data) == 0
                assert L.fmf_write_uvwp(step, svall, 0.25, 0.5, s1.ctypes.data, s2.ctypes.data, s3.ctypes.data) == 0
            else:
                for kind in (0, 1):
                    assert orc.lib().orc_write_slices(kind, step, svall, dp(0.25), dp(0.5), orc.P(s1), orc.P(s2),
                                                      orc.P(s3)) == 0
        for t in range(3):  # three appended records
            c, vel, re = vals[t], vals[(t + 1) % 3], vals[(t + 2) % 3]
            time, velo = dp(0.1 * t), dp(1.5 + t)
            if who == "lib":
                L.mk_center_(ctypes.byref(ip(t)), ctypes.byref(time), orc.P(c), ctypes.byref(velo), ctypes.byref(ip(1)))
                L.mk_vel_(ctypes.byref(ip(t)), ctypes.byref(time), orc.P(vel), orc.P(re), ctypes.byref(velo),
                          ctypes.byref(ip(1)))
            else:
                assert orc.lib().orc_mk_center(ctypes.byref(time), orc.P(c), ctypes.byref(velo), orc.I(1)) == 0
                assert orc.lib().orc_mk_vel(ctypes.byref(time), orc.P(vel), orc.P(re), ctypes.byref(velo), orc.I(1)) == 0
    names = ["uwphi0000003", "uwphi0000004", "uvwp0000003", "uvwp0000004", "center_01.dat", "velocity_01.dat"]
    for n in names:
        a = open(tmp_path / "lib" / n, "rb").read()
        b = open(tmp_path / "orc" / n, "rb").read()
        assert a == b and len(a) > 0, n
    first = open(tmp_path / "orc" / "uwphi0000003").readline()
    assert len(first) == 5 * 20 + 1 and float(first[40:60]) == 0.0
