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


def sphere_mesh(center, radius, n_lat=12, n_lon=24):
    """A closed UV sphere as triangles [n, 3, 3] (outward-facing), vertices placed off the cell-centre grid
    so no cell centre lies exactly on a face unless a test asks for it."""
    c = np.asarray(center, np.float64)
    pts = lambda th, ph: c + radius * np.array([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)])
    tris = []
    for i in range(n_lat):
        t0, t1 = np.pi * i / n_lat, np.pi * (i + 1) / n_lat
        for j in range(n_lon):
            p0, p1 = 2 * np.pi * j / n_lon + 0.1, 2 * np.pi * (j + 1) / n_lon + 0.1
            a, b, cc, d = pts(t0, p0), pts(t0, p1), pts(t1, p1), pts(t1, p0)
            if i > 0:
                tris.append((a, cc, b))
            if i < n_lat - 1:
                tris.append((a, d, cc))
    return np.asarray(tris, np.float32)


def box_mesh(lo, hi):
    """An axis-aligned box [lo, hi] as 12 triangles."""
    from eulerianfluidsimulation_gb300.scene import cube_triangles
    lo, hi = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    t = cube_triangles() > 0          # each corner takes lo or hi exactly
    return np.where(t, hi, lo).astype(np.float32)


def write_obj(path, triangles):
    """Triangles [n, 3, 3] as an OBJ file (one vertex per corner)."""
    with open(path, "w") as fh:
        for tri in np.asarray(triangles, np.float32):
            for v in tri:
                fh.write(f"v {float(v[0])!r} {float(v[1])!r} {float(v[2])!r}\n")
        for k in range(len(triangles)):
            fh.write(f"f {3 * k + 1} {3 * k + 2} {3 * k + 3}\n")
