"""Restart files (dataou.f / datain.f): the record layout gfortran gives an
unformatted sequential write, read back by the library and written by an
independent numpy encoder (host code, no GPU needed); and, on the GPU, the
drop-ins dataou_/datain_ with device-resident arrays."""
import ctypes
import os

import numpy as np
import pytest

NI, NJ, NK, NBUB = 16, 8, 4, 1


@pytest.fixture
def lib(fmf_built):
    L = ctypes.CDLL(fmf_built)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.fmf_write_checkpoint.argtypes = [ctypes.c_char_p, ip, ip, ip, ip, ip, dp, vp, vp]
    L.fmf_read_checkpoint.argtypes = [ctypes.c_char_p, ip, ip, ip, ip, ctypes.POINTER(ip), ctypes.POINTER(dp),
                                      vp, vp]
    return L


def _fields(seed):
    rng = np.random.default_rng(seed)
    shape = (NK + 6, NJ + 6, NI + 6)
    return [rng.standard_normal(shape) for _ in range(8)], rng.random((NBUB + 1,) + shape)


def _ptrs(arrs):
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


def _gfortran_record(payload: bytes, chunk: int) -> bytes:
    """gfortran framing of one unformatted sequential record (4-byte markers)."""
    out, off, first = [], 0, True
    while off < len(payload) or first:
        n = min(chunk, len(payload) - off)
        more = off + n < len(payload)
        out.append(np.int32(-n if more else n).tobytes())
        out.append(payload[off:off + n])
        out.append(np.int32(n if first else -n).tobytes())
        off += n
        first = False
    return b"".join(out)


def _payload(f, phi, time, nstep):
    return b"".join(a.tobytes() for a in f) + phi.tobytes() + np.float64(time).tobytes() + np.int32(nstep).tobytes()


def test_write_matches_gfortran_layout(lib, tmp_path):
    f, phi = _fields(1)
    path = str(tmp_path / "x0000042").encode()
    assert lib.fmf_write_checkpoint(path, NI, NJ, NK, NBUB, 42, 1.25e-3, _ptrs(f), phi.ctypes.data) == 0
    data = open(path, "rb").read()
    assert data == _gfortran_record(_payload(f, phi, 1.25e-3, 42), 2147483639)


def test_read_roundtrip_and_foreign_file(lib, tmp_path):
    f, phi = _fields(2)
    path = str(tmp_path / "x.inp")
    with open(path, "wb") as fh:  # written without the library
        fh.write(_gfortran_record(_payload(f, phi, 7.5, 123), 2147483639))
    g = [np.zeros_like(a) for a in f]
    ph = np.zeros_like(phi)
    ns, t = ctypes.c_int(), ctypes.c_double()
    assert lib.fmf_read_checkpoint(path.encode(), NI, NJ, NK, NBUB, ctypes.byref(ns), ctypes.byref(t), _ptrs(g),
                                   ph.ctypes.data) == 0
    assert ns.value == 123 and t.value == 7.5
    for a, b in zip(f, g):
        assert np.array_equal(a, b)
    assert np.array_equal(phi, ph)


def test_subrecords(lib, tmp_path, monkeypatch):
    """Records above 2 GiB are cut into subrecords; exercised here with a small cut."""
    f, phi = _fields(3)
    monkeypatch.setenv("FMF_RECORD_CHUNK", "1000")
    path = str(tmp_path / "x0000001").encode()
    assert lib.fmf_write_checkpoint(path, NI, NJ, NK, NBUB, 1, 0.5, _ptrs(f), phi.ctypes.data) == 0
    data = open(path, "rb").read()
    assert data == _gfortran_record(_payload(f, phi, 0.5, 1), 1000)
    g = [np.zeros_like(a) for a in f]
    ph = np.zeros_like(phi)
    ns, t = ctypes.c_int(), ctypes.c_double()
    assert lib.fmf_read_checkpoint(path, NI, NJ, NK, NBUB, ctypes.byref(ns), ctypes.byref(t), _ptrs(g),
                                   ph.ctypes.data) == 0
    assert ns.value == 1 and all(np.array_equal(a, b) for a, b in zip(f, g))


def test_size_mismatch_is_an_error(lib, tmp_path):
    f, phi = _fields(4)
    path = str(tmp_path / "x0000002").encode()
    assert lib.fmf_write_checkpoint(path, NI, NJ, NK, NBUB, 2, 0.0, _ptrs(f), phi.ctypes.data) == 0
    big = [np.zeros((NK + 6, NJ + 6, 2 * NI + 6)) for _ in range(8)]
    ph = np.zeros((NBUB + 1, NK + 6, NJ + 6, 2 * NI + 6))
    ns, t = ctypes.c_int(), ctypes.c_double()
    assert lib.fmf_read_checkpoint(path, 2 * NI, NJ, NK, NBUB, ctypes.byref(ns), ctypes.byref(t), _ptrs(big),
                                   ph.ctypes.data) != 0
    assert lib.fmf_read_checkpoint(os.path.join(str(tmp_path), "missing").encode(), NI, NJ, NK, NBUB,
                                   ctypes.byref(ns), ctypes.byref(t), _ptrs(big), ph.ctypes.data) != 0


@pytest.mark.gpu
def test_dataou_datain_resident(fmf_lib, tmp_path, monkeypatch):
    """dataou_ / datain_ with the device copies authoritative (FMF_RESIDENT,
    dataou.f:26-39, datain.f): arrays whose device mirror is newer than the host
    (a drop-in call wrote them; phi's two slices registered one by one, as the
    reference passes phi(...,l) slices) are copied back before the file is written,
    and the file is byte for byte the one fmf_write_checkpoint writes from the
    expected values; datain_ re-uploads what it read, which the next resident call
    then sees on the device."""
    from fmf import capi
    from fmf import config as C

    L = fmf_lib
    L.fmf_write_checkpoint.argtypes = [ctypes.c_char_p] + [ctypes.c_int] * 5 + [ctypes.c_double, ctypes.c_void_p,
                                                                                ctypes.c_void_p]
    monkeypatch.chdir(tmp_path)
    cfg = C.Config("restart", NI, NJ, NK, 2.0, 1.0, 1.0, dt=1e-3, steps=1)
    I = lambda x: ctypes.byref(ctypes.c_int(x))
    vp = lambda a: ctypes.c_void_p(a.ctypes.data)
    L.fmf_reset()
    L.fmf_set_mode(capi.FMF_RESIDENT)
    try:
        f, phi = _fields(5)
        host = [a.copy() for a in f]
        hphi = phi.copy()
        for a in host:
            L.bnd_periodic_(I(NI), I(NJ), I(NK), vp(a))
        for sl in range(NBUB + 1):
            L.bnd_periodic_(I(NI), I(NJ), I(NK), vp(hphi[sl]))
        assert L.fmf_last_error() == 0
        # resident: the host arrays still hold the values before the calls
        assert all(np.array_equal(a, b) for a, b in zip(host, f)) and np.array_equal(hphi, phi)
        want = [a.copy() for a in f]
        wphi = phi.copy()
        for a in want + [wphi[0], wphi[1]]:
            C.periodic(a, cfg)
        t = ctypes.byref(ctypes.c_double(0.125))
        L.dataou_(I(0), I(0), I(NI), I(NJ), I(NK), I(NBUB), I(9), t, *[vp(a) for a in host], vp(hphi))
        assert L.fmf_last_error() == 0
        assert L.fmf_write_checkpoint(b"expected", NI, NJ, NK, NBUB, 9, 0.125, _ptrs(want), wphi.ctypes.data) == 0
        assert open("x0000009", "rb").read() == open("expected", "rb").read()
        # datain_: a different state in x.inp goes to the host arrays and their mirrors
        g, gphi = _fields(6)
        assert L.fmf_write_checkpoint(b"x.inp", NI, NJ, NK, NBUB, 3, 2.5, _ptrs(g), gphi.ctypes.data) == 0
        ns, tt = ctypes.c_int(0), ctypes.c_double(0.0)
        L.datain_(I(0), I(0), I(NI), I(NJ), I(NK), I(NBUB), ctypes.byref(ns), ctypes.byref(tt),
                  *[vp(a) for a in host], vp(hphi))
        assert L.fmf_last_error() == 0
        assert ns.value == 3 and tt.value == 2.5
        assert all(np.array_equal(a, b) for a, b in zip(host, g)) and np.array_equal(hphi, gphi)
        # the device copies hold the new values: a resident copy reads them there
        for src, ref in ((host[0], g[0]), (hphi[1], gphi[1])):
            dst = np.zeros_like(ref)
            L.cpy_(I(NI), I(NJ), I(NK), vp(src), vp(dst))
            assert L.fmf_sync_to_host(vp(dst)) == 0
            assert np.array_equal(dst, ref)
    finally:
        L.fmf_reset()
        L.fmf_set_mode(capi.FMF_RESIDENT)
