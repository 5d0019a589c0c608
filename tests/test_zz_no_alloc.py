"""fmf_cal_av_noalloc: the interior mean for callers that cannot allocate device
memory while they run (code inside another framework's memory pool or a fixed
memory budget, or in the middle of its own stream-ordered work).  Its scratch
is a fixed array compiled into the library; this test checks it against the
regular, allocating cal_av_ on two calls in a row (the second with a different
field, so a stale partial sum from the first call would show), and that an
oversized grid is refused before anything runs.

This file is collected last on purpose: the device memory here comes from torch,
not from the library.
"""
import ctypes

import numpy as np
import pytest

from fmf import config as C

pytestmark = pytest.mark.gpu



def _cal_av_reference(L, q, ni, nj, nk):
    from fmf import capi
    L.fmf_set_mode(capi.FMF_COHERENT)
    av = ctypes.c_double()
    I = lambda x: ctypes.byref(ctypes.c_int(x))
    L.cal_av_(I(0), I(1), I(ni), I(nj), I(nk), ctypes.c_void_p(q.ctypes.data), ctypes.byref(av))
    L.fmf_set_mode(capi.FMF_RESIDENT)
    assert L.fmf_last_error() == 0
    return av.value


def test_noalloc_mean_matches_cal_av_twice(fmf_lib):
    torch = pytest.importorskip("torch")
    L = fmf_lib
    L.fmf_cal_av_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p]
    L.fmf_cal_av_noalloc.restype = ctypes.c_int
    ni, nj, nk = 64, 32, 16
    cfg = C.Config("noalloc", ni, nj, nk, 2.0, 1.0, 1.0, dt=1e-3, steps=1)
    rng = np.random.default_rng(7)
    stream = torch.cuda.current_stream().cuda_stream
    av_dev = torch.zeros(1, dtype=torch.float64, device="cuda")
    for call in range(2):
        q = rng.normal(loc=0.3 * (call + 1), size=cfg.shape)
        want = _cal_av_reference(L, q, ni, nj, nk)
        q_dev = torch.from_numpy(q).to("cuda")
        rc = L.fmf_cal_av_noalloc(ni, nj, nk, q_dev.data_ptr(), av_dev.data_ptr(), stream)
        torch.cuda.synchronize()
        assert rc == 0
        got = float(av_dev.item())
        # the same reduction kernels, grid and division as cal_av_: bit for bit
        assert got == want, (call, got, want)


def test_noalloc_rejects_oversized_grid(fmf_lib):
    torch = pytest.importorskip("torch")
    L = fmf_lib
    L.fmf_cal_av_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p]
    L.fmf_cal_av_noalloc.restype = ctypes.c_int
    av_dev = torch.zeros(1, dtype=torch.float64, device="cuda")
    q_dev = torch.zeros(8, dtype=torch.float64, device="cuda")
    # ceil(4096/8) * 256 = 131072 partial sums > 65536: refused before any launch
    rc = L.fmf_cal_av_noalloc(16, 4096, 256, q_dev.data_ptr(), av_dev.data_ptr(), None)
    assert rc == 2
    # 65536 k planes: within the partial-sum array (ceil(8/8) * 65536) but past the
    # launch's 65535 block rows, also refused before any launch
    rc = L.fmf_cal_av_noalloc(16, 8, 65536, q_dev.data_ptr(), av_dev.data_ptr(), None)
    assert rc == 2
