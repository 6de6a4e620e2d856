"""Shared test helpers: fixture loading and field comparison metrics."""
import os

import numpy as np

from eulerianfluidsimulation_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel_l2(a, b):
    """||a - b|| / ||b|| in FP64 (absolute norm when b is zero)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    d = np.linalg.norm(a - b)
    return d / nb if nb > 0 else d


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    prm = abi.EfsParams.from_buffer_copy(z["params"].tobytes())
    dim, side, warmup, nsteps, spheres = [int(v) for v in z["meta"]]

    def snap(prefix):
        return {f: z[f"{prefix}_{f}"] for f in range(abi.FIELD_COUNT) if f"{prefix}_{f}" in z}

    return {"params": prm, "dim": dim, "side": side, "nsteps": nsteps, "state": snap("state"),
            "stages": [snap(f"stage{s}") for s in range(abi.STAGE_COUNT)], "steps": snap("steps")}


def labels(rho):
    """Fluid labels as the step reads them: liquid where rho >= 0.5."""
    return np.asarray(rho) >= 0.5
