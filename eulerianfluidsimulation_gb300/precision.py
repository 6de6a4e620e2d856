"""Precision study of the liquid step: every field's error against an FP64 pressure solve of the same
right-hand side.

Two contexts run side by side.  Context A advances the trajectory with the production settings (FP32 fields
and stencils, the mixed-precision CG: FP64-class dot products, an FP64 pressure accumulator and the FP64
residual recomputed every 64 iterations and before stopping, i.e. iterative refinement on an FP64
residual).  Before each projection the whole state of A is copied into context B, which projects with
``EFS_CG_FP64`` (p, r, d and L d in FP64, solved to ``tol_fp64``).  Both projections therefore see the same
right-hand side; the per-step report gives

- ``p_rel``: FP32 pressure field of A against B's FP64 pressure (matrix rows: rho > 0.5, not solid);
- ``p64_rel``: A's FP64 accumulator (the FP32 field before rounding) against B's FP64 pressure;
- ``vel_rel``: A's projected velocity against B's (which used B's pressure rounded to FP32);
- ``relres_a`` / ``relres_b``: the true relative residuals sqrt(r.r / b.b) each solver computed in FP64 when
  it stopped;
- ``mass_rel``: A's total liquid mass (an FP64 sum) against the first step's.

rho, gamma and beta are computed before the projection from the same state in both contexts, so their
error against the FP64 solve is zero by construction at every step; over the trajectory they carry the
pressure error of earlier steps only through the velocities, which ``vel_rel`` bounds.
"""
import numpy as np

from . import abi
from .simulator import GB300Simulator2D, GB300Simulator3D, params_dam, scene_dam2d, scene_dam3d


def _rel(a, b, mask=None):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def precision_study(dim, n, steps, spheres=16, seed=0, dt=0.004, tol_rel=1e-6, tol_fp64=1e-12, max_steps=20000,
                    on_step=None):
    """Run `steps` steps of the dam break (3D with `spheres` seeded spheres, or 2D) and return a dict with
    the per-step records and their maxima.  `on_step(record)` is called after every step."""
    prm = params_dam(1.0 / n, dt, abi.SOLVER_CG, tol_rel)
    prm.max_steps = max_steps
    prm64 = prm.copy()
    prm64.cg_variant = abi.CG_FP64
    prm64.tol_rel = tol_fp64
    prm64.max_steps = 4 * max_steps
    if dim == 3:
        boundary, rho = scene_dam3d(n, n, n, spheres, spheres, seed)
        A, B = GB300Simulator3D(n, n, n, prm), GB300Simulator3D(n, n, n, prm64)
    else:
        boundary, rho = scene_dam2d(n, n)
        A, B = GB300Simulator2D(n, n, prm), GB300Simulator2D(n, n, prm64)
    records = []
    try:
        for s in (A, B):
            s.set_field(abi.FIELD_BOUNDARY, boundary)
            s.set_field(abi.FIELD_RHO, rho)
        mass0 = None
        for k in range(steps):
            for st in range(abi.STAGE_PROJECT):
                if not (prm.disable_mask >> st) & 1:
                    A.stage(st)
            state = A.fields()
            A.project()
            B.set_fields(state)
            B.project()
            # matrix rows: liquid (rho > 0.5, the CG matrix's own test) and not solid
            rows = (state[abi.FIELD_RHO] > 0.5) & (state[abi.FIELD_BOUNDARY] == 0.0)
            pa, pa64, pb64 = A.pressure(), A.pressure_fp64(), B.pressure_fp64()
            sa, sb = A.stats(), B.stats()
            mass = A.total_mass()
            if mass0 is None:
                mass0 = mass
            rec = {
                "step": k,
                "p_rel": _rel(pa, pb64, rows),
                "p64_rel": _rel(pa64, pb64, rows),
                "vel_rel": _rel(A.vel(), B.vel()),
                "relres_a": float(np.sqrt(sa.rr / sa.bb)) if sa.bb > 0 else 0.0,
                "relres_b": float(np.sqrt(sb.rr / sb.bb)) if sb.bb > 0 else 0.0,
                "iters_a": int(sa.solve_steps),
                "iters_b": int(sb.solve_steps),
                "converged": bool(sa.converged and sb.converged),
                "mass_rel": (mass - mass0) / mass0 if mass0 else 0.0,
            }
            records.append(rec)
            if on_step:
                on_step(rec)
    finally:
        A.close()
        B.close()
    keys = ("p_rel", "p64_rel", "vel_rel", "relres_a", "relres_b")
    summary = {k: max(r[k] for r in records) for k in keys}
    summary["mass_rel_max_abs"] = max(abs(r["mass_rel"]) for r in records)
    summary["all_converged"] = all(r["converged"] for r in records)
    summary["mean_iters_a"] = float(np.mean([r["iters_a"] for r in records]))
    summary["mean_iters_b"] = float(np.mean([r["iters_b"] for r in records]))
    return {"dim": dim, "n": n, "steps": steps, "spheres": spheres if dim == 3 else 0, "seed": seed,
            "tol_rel": tol_rel, "tol_fp64": tol_fp64, "max": summary, "records": records}
