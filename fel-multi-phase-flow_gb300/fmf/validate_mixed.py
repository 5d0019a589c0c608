"""Run the FP64 and the mixed-precision step side by side from the same initial
state and print the largest relative error of u, v, w, p and phi every `every`
steps (interior points, relative to the FP64 field's largest magnitude).

    python -m fmf.validate_mixed droplet512 500 50

Needs a GPU; both steppers hold a full state of the workload in device memory.
"""
import sys

import numpy as np

from fmf import build, capi
from fmf import config as C

FIELDS = {"u": 0, "v": 1, "w": 2, "p": 6, "phi": 9}


def run(name: str, steps: int, every: int) -> dict:
    build.build()
    cfg = C.get(name)
    ref = capi.Stepper(cfg)
    st = ref.initial_state()
    mix = capi.Stepper(cfg, precision=capi.FMF_MIXED)
    mix.upload(st)
    worst = {k: 0.0 for k in FIELDS}
    for s in range(every, steps + every, every):
        n = min(every, steps - (s - every))
        ref.step(n)
        mix.step(n)
        a, b = mix.get_state(), ref.get_state()
        if not np.isfinite(a).all():
            raise RuntimeError(f"non-finite mixed state after step {s}")
        errs = {}
        for k, f in FIELDS.items():
            x, y = C.interior(a[f]), C.interior(b[f])
            errs[k] = float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300))
            worst[k] = max(worst[k], errs[k])
        print(f"step {min(s, steps)}: " + " ".join(f"{k} {v:.2e}" for k, v in errs.items()), flush=True)
    ref.close()
    mix.close()
    return worst


if __name__ == "__main__":
    name = sys.argv[1] if len(sys.argv) > 1 else "droplet512"
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 500
    every = int(sys.argv[3]) if len(sys.argv) > 3 else 50
    w = run(name, steps, every)
    print("largest over the run: " + " ".join(f"{k} {v:.2e}" for k, v in w.items()))
