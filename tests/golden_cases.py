"""Loading helpers for the golden fixtures (inputs + reference outputs)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["c3d_64", "c3d_96x80", "c2d_128", "c2d_128_q", "c3d_64_ts", "c3d_64_w"]
DXY = 0.08


def load(name):
    zi = np.load(os.path.join(GOLDEN, f"in_{name}.npz"))
    zo = np.load(os.path.join(GOLDEN, f"out_{name}.npz"))
    case = dict(raw=zi["raw"], otf=zi["otf"], config=str(zi["config"]), nx=int(zi["nx"]), ny=int(zi["ny"]),
                staged=int(zi["staged"]))
    ref = {k: zo[k] for k in zo.files}
    return case, ref


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))
