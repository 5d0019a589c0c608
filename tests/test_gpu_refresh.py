"""The one-pass wall/halo refresh kernels (k_refresh of the FP64 step, k_refresh_d on
the mixed step's FP32 corrections) against the ordered plane kernels they replace
(wall, then x halo, then z halo): the same steps run in two processes, one with
FMF_REFRESH_ORDERED set, and give the same state bit for bit."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, {pkg!r})
from fmf import capi
from fmf import config as C
cfg = C.get({name!r}, ni={ni}, nj={nj}, nk={nk})
out = {{}}
for prec, key in ((capi.FMF_FP64, "fp64"), (capi.FMF_MIXED, "mixed")):
    g = capi.Stepper(cfg, precision=prec)
    g.initial_state()
    g.step({steps})
    out[key] = g.get_state()
    g.close()
np.savez({path!r}, **out)
"""


def _run(tmp_path, tag, ordered, name, ni, nj, nk, steps):
    path = str(tmp_path / f"{tag}.npz")
    env = dict(os.environ)
    env.pop("FMF_REFRESH_ORDERED", None)
    if ordered:
        env["FMF_REFRESH_ORDERED"] = "1"
    code = SCRIPT.format(pkg=os.path.join(ROOT, "fel-multi-phase-flow_gb300"), name=name, ni=ni, nj=nj, nk=nk,
                         steps=steps, path=path)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(path)


@pytest.mark.parametrize("shape", [(32, 16, 16), (64, 32, 32)])
def test_one_pass_refresh_matches_ordered_kernels(fmf_lib, tmp_path, shape):
    ni, nj, nk = shape
    a = _run(tmp_path, "one", False, "couette32", ni, nj, nk, 4)
    b = _run(tmp_path, "ordered", True, "couette32", ni, nj, nk, 4)
    for key in ("fp64", "mixed"):
        assert np.isfinite(a[key]).all()
        assert np.array_equal(a[key], b[key]), (key, np.abs(a[key] - b[key]).max())
