"""Generate the golden fixtures in this folder from the reference's own CPU backend.

Runs the unmodified reference sources (built by ``oracle/Makefile`` into ``oracle/_ref/libefs_ref.so``, which
needs the reference tree) on small seeded scenes and stores, per case:
  ``state``           all eight fields after ``warmup`` full steps from the seeded scene,
  ``stage<s>``        all fields after running stage s alone from ``state`` (s = 0..6),
  ``steps``           all fields after ``nsteps`` more full steps from ``state``,
plus the parameters used.  Sizes are chosen so the reference's 32-bit advection-matrix key cannot wrap
(3D: cells^2 < 2^32; 2D: side <= 256).

Also ``ref_query.npz``: the reference's QueryNode metric loop (its own lines, compiled into the reference build by
oracle/Makefile) on a stepped 32^3 state, for a set of boxes.

Also ``ref_dropin_dam32.npz``: the reference's CPUSimulator3D driven through its ISimulator3D interface by
tests/dropin_driver.cpp (oracle/Makefile's ``dropin`` target, which needs libefs_gb300.so built first).

Usage: python tests/golden/make_golden.py      (writes ref_3d_cg.npz, ref_2d_jacobi.npz, ref_2d_cg.npz, ref_query.npz,
                                                ref_dropin_dam32.npz)
"""
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from eulerianfluidsimulation_gb300 import abi  # noqa: E402
from oracle import oracle  # noqa: E402

CASES = {
    # name: (dim, side, solver, dt, tol_rel, warmup, nsteps, spheres)
    "ref_3d_cg": (3, 24, abi.SOLVER_CG, 0.004, 0.0, 4, 2, 6),
    "ref_2d_jacobi": (2, 48, abi.SOLVER_JACOBI, 0.005, 0.0, 6, 3, 0),
    "ref_2d_cg": (2, 40, abi.SOLVER_CG, 0.005, 0.0, 6, 3, 0),
}


def case_params(dim, side, solver, dt, tol_rel):
    p = abi.params_dam(1.0 / side, dt, solver, tol_rel)
    p.cg_variant = abi.CG_REFERENCE
    if solver == abi.SOLVER_JACOBI:
        p.max_steps = 200
    return p


def scene(dim, side, spheres, seed=1):
    if dim == 3:
        return oracle.scene_dam3d(side, side, side, spheres, spheres, seed)
    return oracle.scene_dam2d(side, side)


def make(name):
    dim, side, solver, dt, tol, warmup, nsteps, spheres = CASES[name]
    prm = case_params(dim, side, solver, dt, tol)
    b, r = scene(dim, side, spheres)
    ref = oracle.RefOracle(dim, side, side, side, prm)
    ref.set_field(abi.FIELD_BOUNDARY, b)
    ref.set_field(abi.FIELD_RHO, r)
    ref.step(warmup)
    state = ref.fields()
    out = {"params": np.frombuffer(bytes(prm), np.uint8).copy(), "meta": np.array([dim, side, warmup, nsteps, spheres])}
    for f, a in state.items():
        out[f"state_{f}"] = a
    for s in range(abi.STAGE_COUNT):
        ref.set_fields(state)
        ref.stage(s)
        for f, a in ref.fields().items():
            out[f"stage{s}_{f}"] = a
    ref.set_fields(state)
    ref.step(nsteps)
    for f, a in ref.fields().items():
        out[f"steps_{f}"] = a
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), name + ".npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


# QueryNode metric boxes (position, scale, only_fluid) on a 32^3 dam break after 6 steps: the whole grid, a box in
# the liquid, one crossing the far faces (clipped), one at negative coordinates, one without liquid, the whole grid
# counting every cell, and an empty box
QUERIES = [((0, 0, 0), (32, 32, 32), 1), ((2, 2, 2), (8, 10, 12), 1), ((6, 1, 20), (40, 40, 40), 1),
           ((-3, -2, -5), (10, 12, 9), 1), ((28, 28, 28), (3, 3, 3), 1), ((0, 0, 0), (32, 32, 32), 0),
           ((5, 5, 5), (0, 4, 4), 0)]


def make_query():
    """ref_query.npz: the reference's own QueryNode metric loop (compiled into the reference build) on a stepped
    3D state, for each box of QUERIES."""
    n = 32
    prm = case_params(3, n, abi.SOLVER_CG, 0.004, 1e-6)
    b, r = scene(3, n, 8, seed=2)
    ref = oracle.RefOracle(3, n, n, n, prm)
    ref.set_field(abi.FIELD_BOUNDARY, b)
    ref.set_field(abi.FIELD_RHO, r)
    ref.step(6)
    out = {"rho": ref.field(abi.FIELD_RHO), "vel": ref.field(abi.FIELD_VEL), "pressure": ref.field(abi.FIELD_PRESSURE),
           "queries": np.array([list(p) + list(s) + [f] for p, s, f in QUERIES], np.int32)}
    res = []
    for p, s, f in QUERIES:
        m, cnt = ref.query_box(p, s, bool(f))
        res.append(np.concatenate([m["max_position"], m["min_position"], m["avg_position"], m["velocity"],
                                   [m["pressure"], cnt]]).astype(np.float64))
    out["results"] = np.array(res)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_query.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


# the C++ drop-in's comparison case: tests/dropin_driver.cpp's seeded 32^3 dam break (4 spheres, seed 3), frames
DROPIN = (32, 4)


def make_dropin():
    """ref_dropin_dam32.npz: the reference's CPUSimulator3D::update(), called through its ISimulator3D interface
    with the Properties set as the application sets them (tests/dropin_driver.cpp), for DROPIN frames; SOLVE_STEPS
    and PAUSED after each frame, the efs_params the C++ drop-in backend derives from the same Properties, and the
    fields after the last frame."""
    n, frames = DROPIN
    r = oracle.dropin_reference(n, frames)
    out = {"params": np.frombuffer(bytes(r["params"]), np.uint8).copy(), "steps": r["steps"], "paused": r["paused"],
           "meta": np.array([n, frames, 4, 4, 3])}
    for f, a in r["fields"].items():
        out[f"field_{f}"] = a
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_dropin_dam32.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    oracle.build(reference=True)
    if not oracle.reference_available():
        sys.exit("the reference tree is needed to generate golden fixtures")
    for n in CASES:
        make(n)
    make_query()
    make_dropin()
