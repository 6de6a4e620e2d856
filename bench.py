#!/usr/bin/env python3
"""bench.py — steps/s of the Eulerian liquid step on a 256^3 dam break with 16 seeded solid spheres.

One step is one ISimulator::update(): the seven stages of the reference order (velocity decay disabled, as in
the reference's dam-break scene) with the pressure solved by CG to relative residual 1e-6.  The grid (about
2 GB of fields and temporaries) is larger than L2, so no flush is needed between steps.

Lines printed (rank 0, one JSON object):
  --impl gb300 (default): `value` = steps/s with the fields resident in HBM (CUDA events on the library's
      stream around K replayed step graphs); `e2e` = the same through efs_step_host with pinned host buffers
      every step; `roofline` for the pressure solve (the dominant kernel); `jacobi` and `learned_pcg` = the same
      scene stepped with Jacobi (100 sweeps) and with FCG and the committed trained network (steps/s,
      iterations and solve ms per step); `cpu_baseline` = one whole CPU step of the oracle (a port of the
      reference CPU step), measured.
  --impl reference: the reference's CPU step on the host cores (the oracle port; the reference's own sources
      need its build tree) on the same workload: one whole step, its pressure solve run to convergence.
With --gpus N (torchrun), every rank advances its own replica (weak scaling; the step has no data exchange).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "steps/s at 256\u00b3 to rel-res 1e-6: learned-PCG vs plain CG/Jacobi, HBM GB/s"
# Bytes the pressure solve must move, per matrix row (CG in its recurrence form, the default variant): per
# iteration read d, rowinfo and write t = L d (10 B), then read d, t, e, r, rowinfo and write e, r, d (30 B);
# per solve set-up read b, rowinfo and write p64, e, r, d and finally p (30 B).  Neighbour reads of the stencil
# are cache hits and count 0.
SOLVE_BYTES_PER_ROW_ITER = 40.0
SOLVE_BYTES_PER_ROW_SETUP = 30.0
# Jacobi (ping-pong): per row and sweep read rowinfo, p, b and write the other p (14 B).
JACOBI_BYTES_PER_ROW_ITER = 14.0
# DRAM bytes (read + write) the solver moved per matrix row and CG iteration in one ncu capture of k_solver on
# this workload (one launch: 950 iterations over 3,778,175 rows, 27.29 GB read + 40.74 GB written; the
# active vectors only partly fit in L2 at 256^3).  `traffic` scales it by this run's row-iterations per launch.
SOLVE_DRAM_BYTES_PER_ROW_ITER = 68.03e9 / (950 * 3778175)
# Algorithmic bytes per interior cell of the stages other than the pressure solve, 3D (each field read once and
# written once per pass: extrapolation 30 + 162, sharpen 21, advection 61 + 12 + 76 + 52, diffusion 153,
# velocity advection 50, add_force 25, divergence 22, gradient and walls 29).
STEP_BYTES_PER_CELL_3D = 693.0
# The same for 2D (vel 8 B, 4 advection weights; the 2D diffusion runs 7 iterations x 2 axes).
STEP_BYTES_PER_CELL_2D = 618.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=None, help="grid side (default 256 for dam3d, 128 for dam2d)")
    ap.add_argument("--spheres", type=int, default=16)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--dt", type=float, default=0.004)
    ap.add_argument("--solver", default=None, choices=["cg", "jacobi", "fcg"],
                    help="fcg: flexible PCG with the learned preconditioner (the committed trained network)")
    ap.add_argument("--fcg-levels", type=int, default=0,
                    help="unet workload: aggregation levels below the grid for the network (0: the whole grid; -1: FCG's "
                         "bottom grid, timed after one V-cycle descent)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-alt", action="store_true", help="skip the Jacobi and learned-PCG comparison runs")
    ap.add_argument("--alt-steps", type=int, default=4, help="timed steps of each comparison run")
    ap.add_argument("--study", default=None, choices=["precision"],
                    help="instead of the throughput line: the precision study (every field against an FP64 "
                         "pressure solve of the same right-hand side) at --size for --steps steps")
    ap.add_argument("--study-out", default=None, help="precision study: also write the per-step records here (JSON)")
    ap.add_argument("--workload", default="dam3d", choices=["dam3d", "dam2d", "batch2d", "scene", "unet"],
                    help="dam2d: the 2D dam break on one grid (Jacobi 100 sweeps unless --solver cg); batch2d: 64 "
                         "independent 2D scenes of uneven sizes advanced together (efs_batch_*)")
    ap.add_argument("--scenes", type=int, default=64)
    ap.add_argument("--batch-tuning", default=None,
                    help="batch2d: tile_x,tile_y,blocks_per_sm,solver_threads[,solver_cluster] instead of running the autotuner")
    a = ap.parse_args()
    if a.size is None:
        a.size = 128 if a.workload == "dam2d" else 256
    if a.solver is None:
        a.solver = "jacobi" if a.workload == "dam2d" else "cg"
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(ms, world):
    """The slowest rank's time (a collective: every rank calls it with its own time)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, ms, world):
    """Whole-job throughput: the units all ranks processed (each rank its own replica) over the slowest rank's
    time."""
    return units_per_rank * world / (ms / 1e3)


def workload(a):
    from eulerianfluidsimulation_gb300 import abi
    solver = abi.SOLVER_JACOBI if a.solver == "jacobi" else abi.SOLVER_CG
    prm = abi.params_dam(1.0 / a.size, a.dt, solver, 1e-6)
    # the reference's MAX_STEPS default (2000) is too small for plain CG to reach 1e-6 at 256^3; the cap
    # only guards against non-convergence here
    prm.max_steps = 200 if solver == abi.SOLVER_JACOBI else 20000
    return prm


def config(a):
    return {"workload": f"dam3d_{a.size}", "grid": [a.size] * 3, "spheres": a.spheres, "seed": a.seed, "dt": a.dt,
            "solver": a.solver + (" rel-res 1e-6, FP32 fields, FP64 dots + FP64 residual replacement" if a.solver == "cg" else " 100 sweeps"),
            "scene": "seeded synthetic: fluid x<0.4,y<0.6; spheres r~U[0.04,0.1], centres~U[0.2,0.8]^3 (PCG32)",
            "l2": "working set ~2 GB > 129 MB L2 (no flush)"}


class Clocks:
    """nvidia-smi samples every 200 ms while the timed region runs."""
    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        except OSError:
            pass
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def host_cpu():
    """The host's CPU model and logical core count (lscpu; /proc/cpuinfo as a fallback)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"model": model or "unknown", "logical_cores": os.cpu_count()}


def cpu_sample(a, prm):
    """Time one whole step of the CPU oracle (the reference CPU step restated: CPUSimulator3D.cpp's stages in the
    reference's own order, density sharpening sequential as the reference loops) on the same 256^3 scene, the
    pressure solve included and run to convergence.  The stages run on one thread, as the reference's do; the
    solver's per-cell loops (matrix products, vector updates) run on all host threads.  The solver is the CG
    variant of the CUDA path (the reference's FP32 CG stalls above rel-res 1e-6 at this size and would run to
    MAX_STEPS), so both arms do the same iterations."""
    from eulerianfluidsimulation_gb300 import abi
    from oracle import oracle
    n = a.size
    b, r = oracle.scene_dam3d(n, n, n, a.spheres, a.spheres, a.seed)
    o = oracle.Oracle(3, n, n, n, prm.copy())
    o.set_field(abi.FIELD_BOUNDARY, b)
    o.set_field(abi.FIELD_RHO, r)
    threads = oracle._load_orc().orc_threads()
    t0 = time.perf_counter()
    for s in range(abi.STAGE_PROJECT):
        if not (prm.disable_mask >> s) & 1:
            o.stage(s)
    t1 = time.perf_counter()
    o.stage(abi.STAGE_PROJECT)
    t2 = time.perf_counter()
    st = o.stats()
    step_s = t2 - t0
    return {"value": 1.0 / step_s, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": (f"one whole {n}^3 step measured (no extrapolation): stages 0-5 {t1 - t0:.2f} s on 1 thread, "
                       f"project {t2 - t1:.2f} s ({st.solve_steps} CG iterations to rel-res 1e-6, converged="
                       f"{bool(st.converged)}) with its per-cell loops on {threads} threads"),
            "step_s": step_s, "stages_s": t1 - t0, "project_s": t2 - t1, "cg_iters": st.solve_steps,
            "host": host_cpu()}


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    prm = workload(a)
    t = time.perf_counter()
    cs = cpu_sample(a, prm)
    wall = time.perf_counter() - t
    line = {"metric": METRIC, "value": cs["value"], "unit": "steps/s", "n_gpus": a.gpus, "steps": 1, "warmup": 0,
            "ms_per_step": cs["step_s"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": config(a), "impl": "reference",
            "cpu_baseline": {"value": cs["value"], "unit": "steps/s", "cores": cs["cores"], "kind": cs["kind"],
                             "sample": cs["sample"], "host": cs["host"]},
            "e2e": {"value": cs["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "sample_wall_s": wall,
            "note": "one whole step is the bounded sample (about 20-30 s on 16 Grace cores); --steps/--warmup are "
                    "not repeated on the CPU"}
    print(json.dumps(line), flush=True)


def masked_relres(div, p, rho, boundary):
    """||b - L p|| / ||b|| in FP64 for the reference's pressure matrix (CGSolver.cpp:467-497): rows are liquid
    (rho > 0.5), non-solid cells; a neighbour counts when it is inside the border and not solid, and adds its p
    when it is liquid."""
    div, p, rho, bnd = (np.asarray(x, np.float64) for x in (div, p, rho, boundary))
    D, H, W = p.shape
    row = (rho > 0.5) & (bnd != 1.0)
    inner = np.zeros(p.shape, bool)
    inner[1:D - 1, 1:H - 1, 1:W - 1] = True
    ok = inner & (bnd <= 0.5)
    liq = ok & (rho > 0.5)
    cnt = np.zeros(p.shape)
    acc = np.zeros(p.shape)
    for ax in range(3):
        for sh in (1, -1):
            okn = np.roll(ok, sh, axis=ax)
            pn = np.roll(np.where(liq, p, 0.0), sh, axis=ax)
            cnt += okn
            acc += pn
    Lp = np.where(row, acc - cnt * p, p)
    res = div - Lp
    bb = float(np.sum(div * div))
    return float(np.sqrt(np.sum(res * res) / bb)) if bb > 0 else float(np.sqrt(np.sum(res * res)))


def alt_solver_line(a, kind, b, r, cg_ms_step, cg_solve_ms, cg_iters):
    """One comparison run on the benchmark scene: `kind` = "jacobi" (100 sweeps a step, JacobiSolverCPU3D with
    MAX_STEPS 200) or "fcg" (flexible PCG with the learned U-Net preconditioner, to the same rel-res 1e-6).
    Warm-up steps then --alt-steps timed steps with CUDA events on the library's stream."""
    import eulerianfluidsimulation_gb300 as gb
    from eulerianfluidsimulation_gb300 import abi, unet_weights
    n = a.size
    prm = workload(a)
    info = {}
    if kind == "jacobi":
        prm.solver = abi.SOLVER_JACOBI
        prm.max_steps = 200
    else:
        prm.solver = abi.SOLVER_FCG_UNET
    sim = gb.GB300Simulator3D(n, n, n, prm)
    try:
        sim.set_field(abi.FIELD_BOUNDARY, b)
        sim.set_field(abi.FIELD_RHO, r)
        if kind == "fcg":
            info = unet_weights.load_into(sim)
        warm = 2
        for _ in range(warm):
            sim.update(1)
        sim.synchronize()
        st0 = sim.stats()
        k = max(1, a.alt_steps)
        sim.solve_timing_arm(k)
        sim.mark(0)
        sim.update(k)
        sim.mark(1)
        ms = sim.elapsed_ms(0, 1)
        st1 = sim.stats()
        launches, solve_ms, _, _ = sim.solve_timing_read()
        out = {"steps_per_s": k / (ms / 1e3), "ms_per_step": ms / k, "steps": k, "warmup": warm,
               "solve_iters_per_step": (st1.total_solve_steps - st0.total_solve_steps) / k,
               "solve_ms_per_step": (solve_ms / launches) if launches else None,
               "converged": bool(st1.converged), "paused": bool(st1.paused)}
        if kind == "jacobi":
            f = sim.fields()
            out["rel_res_after_100_sweeps"] = masked_relres(f[abi.FIELD_DIVERGENCE], f[abi.FIELD_PRESSURE],
                                                            f[abi.FIELD_RHO], f[abi.FIELD_BOUNDARY])
            out["note"] = "Jacobi does not reach rel-res 1e-6; it runs its fixed 100 sweeps (the reference's Jacobi)"
        else:
            out["precond_iters_last_solve"] = st1.precond_steps
            out["network"] = info
            direct, graph = sim.fcg_time_vcycle(5)
            out["preconditioner_ms"] = {"kernel_by_kernel": direct, "graph_replay": graph}
        out["vs_plain_cg"] = {"step_speedup": cg_ms_step / out["ms_per_step"],
                              "solve_speedup": (cg_solve_ms / out["solve_ms_per_step"]) if out["solve_ms_per_step"] else None,
                              "cg_iters_per_step": cg_iters}
        return out
    finally:
        sim.close()


def run_gb300(a):
    rank, world, local = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import eulerianfluidsimulation_gb300 as gb
    from eulerianfluidsimulation_gb300 import abi
    n = a.size
    prm = workload(a)
    b, r = gb.scene_dam3d(n, n, n, a.spheres, a.spheres, a.seed + rank)
    N = n ** 3
    sim = gb.GB300Simulator3D(n, n, n, prm)
    sim.set_field(abi.FIELD_BOUNDARY, b)
    sim.set_field(abi.FIELD_RHO, r)
    for _ in range(a.warmup):
        sim.update(1)
    st0 = sim.stats()
    sim.synchronize()
    kernels = sim.kernels_per_step()
    sim.solve_timing_arm(a.steps)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    with Clocks(local) as clk:
        barrier()
        sim.synchronize()
        sim.mark(0)
        sim.update(a.steps)
        sim.mark(1)
        ms = sim.elapsed_ms(0, 1)
        barrier()
    clocks = clk.summary()
    st1 = sim.stats()
    launches, solve_ms, row_iters, row_setups = sim.solve_timing_read()
    iters = st1.total_solve_steps - st0.total_solve_steps
    ms = max_over_ranks(ms, world)
    steps_per_s = job_throughput(a.steps, ms, world)
    if prm.solver == abi.SOLVER_JACOBI:
        solve_bytes = row_iters * JACOBI_BYTES_PER_ROW_ITER
    else:
        solve_bytes = row_iters * SOLVE_BYTES_PER_ROW_ITER + row_setups * SOLVE_BYTES_PER_ROW_SETUP
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = (solve_bytes / launches) / ((solve_ms / launches) / 1e3) / 1e9 if launches and solve_ms > 0 else None
    traffic = None
    if a.size == 256 and a.spheres == 16 and prm.solver == abi.SOLVER_CG and launches:
        traffic = SOLVE_DRAM_BYTES_PER_ROW_ITER * row_iters / launches
    roofline = {"kernel": "k_solver (persistent " + ("Jacobi)" if prm.solver == abi.SOLVER_JACOBI else "CG)"), "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_solver launch on this "
                                  "workload, scaled by row-iterations" if traffic else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if "hbm_gbs" in peaks else "fallback 6800 GB/s",
                "solve_ms_per_step": solve_ms / max(launches, 1), "algorithmic_bytes_per_launch": solve_bytes / max(launches, 1),
                # the DRAM bytes per launch over the launch's time: what HBM actually moves (L2 keeps about half of the
                # algorithmic bytes on chip), beside the algorithmic rate that `achieved` reports
                "dram_gbs": (traffic / ((solve_ms / launches) / 1e3) / 1e9) if traffic and solve_ms > 0 else None}
    # the whole step: the stages' algorithmic bytes per interior cell plus the solve's per matrix row
    step_bytes = STEP_BYTES_PER_CELL_3D * (n - 2) ** 3 + solve_bytes / max(launches, 1)
    step_achieved = step_bytes / (ms / a.steps / 1e3) / 1e9
    step_roofline = {"bound": "hbm", "achieved": step_achieved, "peak": peak, "unit": "GB/s", "frac": step_achieved / peak,
                     "algorithmic_bytes_per_step": step_bytes,
                     "stages_bytes_per_interior_cell": STEP_BYTES_PER_CELL_3D,
                     "stages_ms_per_step": ms / a.steps - solve_ms / max(launches, 1)}

    # e2e through the C ABI with pinned host buffers: upload, step, download every step
    e2e = None
    if not a.no_e2e:
        import torch
        def pinned(shape):
            return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()
        h = {k: pinned(s) for k, s in (("vel", (n, n, n, 3)), ("rho", (n, n, n)), ("gamma", (n, n, n)),
                                        ("boundary", (n, n, n)), ("forces", (n, n, n, 3)), ("beta", (n, n, n)),
                                        ("div", (n, n, n)), ("p", (n, n, n)))}
        sim.download_fields(vel=h["vel"], rho=h["rho"], gamma=h["gamma"], beta=h["beta"], divergence=h["div"], pressure=h["p"])
        h["boundary"][...] = b
        h["forces"][...] = 0
        k_e2e = max(2, a.steps // 2)

        def step_host():
            sim.step_host(vel=h["vel"], rho=h["rho"], gamma=h["gamma"], boundary=h["boundary"], forces=h["forces"],
                          vel_out=h["vel"], rho_out=h["rho"], gamma_out=h["gamma"], beta_out=h["beta"],
                          divergence_out=h["div"], pressure_out=h["p"])
        # untimed warm-up calls: the first call that passes a forces field recaptures the step graph with the
        # forces read (a one-time cost of the context, not of a step)
        w_e2e = 2
        for _ in range(w_e2e):
            step_host()
        sim.synchronize()
        se0 = sim.stats()
        sim.solve_timing_arm(k_e2e)
        barrier()
        sim.mark(2)
        for _ in range(k_e2e):
            step_host()
        sim.mark(3)
        ms_e2e = max_over_ranks(sim.elapsed_ms(2, 3), world)
        barrier()
        se1 = sim.stats()
        e_launches, e_solve_ms, _, _ = sim.solve_timing_read()
        # the e2e steps continue the trajectory after the timed steps: their solves may take other iteration
        # counts than the main line's, so the line carries them
        e2e = {"value": job_throughput(k_e2e, ms_e2e, world), "unit": "steps/s", "h2d_bytes_per_step": 4 * N * 9,
               "d2h_bytes_per_step": 4 * N * 8, "steps": k_e2e, "warmup": w_e2e, "ms_per_step": ms_e2e / k_e2e,
               "solve_iters_per_step": (se1.total_solve_steps - se0.total_solve_steps) / k_e2e,
               "solve_ms_per_step": (e_solve_ms / e_launches) if e_launches else None,
               "api": "efs_step_host: upload vel,rho,gamma,boundary,forces + one step + download vel,rho,gamma,beta,div,p "
                      "(page-locked buffers; gamma/forces up and rho/gamma/beta/div down overlap the step)"}
    st2 = sim.stats()
    sim.close()

    # the metric's comparison on the same scene: Jacobi (100 sweeps a step, the reference's other solver) and
    # learned-preconditioned FCG, each from the seeded scene, timed like the main line (steps, not solves alone)
    alt = {}
    if rank == 0 and world == 1 and prm.solver == abi.SOLVER_CG and not a.no_alt:
        alt["jacobi"] = alt_solver_line(a, "jacobi", b, r, ms / a.steps, roofline["solve_ms_per_step"], iters / max(a.steps, 1))
        alt["learned_pcg"] = alt_solver_line(a, "fcg", b, r, ms / a.steps, roofline["solve_ms_per_step"], iters / max(a.steps, 1))

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        cs = cpu_sample(a, prm)
        cpu = {k: cs[k] for k in ("value", "unit", "cores", "kind", "sample", "host")}

    if rank == 0:
        line = {"metric": METRIC, "value": steps_per_s, "unit": "steps/s", "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(a),
                "cell_updates_per_s": steps_per_s * (n - 2) ** 3, "cg_iters_per_step": iters / max(a.steps, 1),
                "solve_converged": bool(st1.converged), "paused": bool(st2.paused), "active_rows": st1.active_cells,
                "gpu_launches": kernels * a.steps, "kernels_per_step": kernels,
                "roofline": roofline, "step_roofline": step_roofline, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clocks}
        line.update(alt)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


UNET_LAYERS = ((16, 16, 0), (16, 32, 1), (32, 64, 2), (64, 32, 1), (32, 16, 0), (16, 16, 0))


def unet_flops(n):
    """Dense FLOPs of one U-Net forward pass on an n^3 grid (2 * 27 * cin * cout per output voxel and layer)."""
    vox = [n ** 3]
    m = n
    for _ in range(2):
        m = (m + 1) // 2
        vox.append(m ** 3)
    return [2 * 27 * ci * co * vox[lv] for ci, co, lv in UNET_LAYERS]


def run_fcg(a):
    """The learned-preconditioner line: FCG (multilevel preconditioner, the committed trained network as its
    coarsest-level solve) on the same 256^3 dam break, each step one replayed graph."""
    import eulerianfluidsimulation_gb300 as gb
    from eulerianfluidsimulation_gb300 import abi, unet_weights
    rank, world, local = dist_env()
    if rank != 0:
        return
    n = a.size
    prm = workload(a)
    prm.solver = abi.SOLVER_FCG_UNET
    b, r = gb.scene_dam3d(n, n, n, a.spheres, a.spheres, a.seed)
    sim = gb.GB300Simulator3D(n, n, n, prm)
    sim.set_field(abi.FIELD_BOUNDARY, b)
    sim.set_field(abi.FIELD_RHO, r)
    net = unet_weights.load_into(sim)
    for _ in range(a.warmup):
        sim.update(1)
    sim.synchronize()
    st0 = sim.stats()
    precond = []
    with Clocks(local) as clk:
        sim.mark(0)
        for _ in range(a.steps):
            sim.update(1)
            precond.append(sim.stats().precond_steps)
        sim.mark(1)
        ms = sim.elapsed_ms(0, 1)
    clocks = clk.summary()
    st1 = sim.stats()
    iters = (st1.total_solve_steps - st0.total_solve_steps) / max(a.steps, 1)
    # plain CG on the continuation of the same trajectory, for the iteration and time comparison
    cg = prm.copy()
    cg.solver = abi.SOLVER_CG
    sim.set_params(cg)
    sim.update(1)
    sim.synchronize()
    sc0 = sim.stats()
    sim.mark(2)
    sim.update(3)
    sim.mark(3)
    ms_cg = sim.elapsed_ms(2, 3) / 3
    sc1 = sim.stats()
    # the dominant kernel: the tcgen05 convolutions of one forward pass, timed on the device
    sim.set_params(prm)
    ms_fwd, ms_layers = sim.unet_time_forward(3)
    # one preconditioner application (V-cycle + network), kernel by kernel and as a graph replay
    vc_direct, vc_graph = sim.fcg_time_vcycle(5)
    nw = sim.unet_grid()[0]
    sim.close()
    flops = unet_flops(nw)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    conv_ms = float(sum(ms_layers))
    achieved = sum(flops) / (conv_ms / 1e3) / 1e12 if conv_ms > 0 else None
    roofline = {"kernel": f"k_conv3_slab (the 6 tcgen05 convolutions of one U-Net forward pass on the {nw}^3 bottom grid)", "bound": "tensor",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None,
                "traffic": None, "peak_source": "MEASURED_PEAKS.json bf16_tflops (measured)" if "bf16_tflops" in peaks
                else "fallback 1900 TFLOP/s", "flop_per_forward": sum(flops), "ms_per_forward": ms_fwd,
                "ms_per_layer": [round(float(x), 4) for x in ms_layers]}
    steps_per_s = a.steps / (ms / 1e3)
    cfg = config(a)
    cfg["solver"] = ("fcg_unet rel-res 1e-6 (flexible PCG, multigrid V-cycle with the U-Net 16/32/64 BF16 as its "
                     "coarsest-level solve, x as float pairs, true residual in pair arithmetic, CG fallback on stall)")
    line = {"metric": METRIC, "value": steps_per_s, "unit": "steps/s", "n_gpus": 1, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "cell_updates_per_s": steps_per_s * (n - 2) ** 3, "solve_iters_per_step": iters,
            "precond_iters_per_step": float(np.mean(precond)) if precond else 0.0,
            "fcg_converged": bool(st1.converged),
            "plain_cg_same_trajectory": {"iters_per_step": (sc1.total_solve_steps - sc0.total_solve_steps) / 3,
                                         "ms_per_step": ms_cg},
            "network": net, "preconditioner_ms": {"kernel_by_kernel": vc_direct, "graph_replay": vc_graph},
            "roofline": roofline, "clocks": clocks, "cpu_baseline": None, "e2e": None}
    print(json.dumps(line), flush=True)


def run_batch2d(a):
    """Many uneven 2D scenes advanced together: sides from {64, 96, 128, 192, 256}, 1-4 rectangles, 1-3 fluid
    circles (seeded, efs_scene.h), dx = 1/side, gravity 9.81/dx, CG to rel-res 1e-6.  Autotuned first (outside
    the timed region); the same scenes as separate single-scene simulators on their own streams are timed
    beside it."""
    import eulerianfluidsimulation_gb300 as gb
    from eulerianfluidsimulation_gb300 import abi
    rank, world, local = dist_env()
    if rank != 0:
        return
    scenes = [gb.scene_batch2d(a.seed + k) for k in range(a.scenes)]
    sides = [b.shape[0] for b, _ in scenes]
    dt = 0.005
    prm = abi.params_dam(1.0 / sides[0], dt, abi.SOLVER_CG, 1e-6)
    prm.max_steps = 20000
    grav = np.array([9.81 * s for s in sides], np.float32)
    B = gb.GB300Batch2D(sides, sides, prm, grav)
    for k, (b, r) in enumerate(scenes):
        B.set_field(k, abi.FIELD_BOUNDARY, b)
        B.set_field(k, abi.FIELD_RHO, r)
    for _ in range(a.warmup):
        B.update(1)
    B.synchronize()
    if a.batch_tuning:
        vals = [int(v) for v in a.batch_tuning.split(",")]
        tune = B.tuning()
        tune.tile_x, tune.tile_y, tune.blocks_per_sm, tune.solver_threads = vals[:4]
        tune.solver_cluster = vals[4] if len(vals) > 4 else 1
        B.set_tuning(tune)
        tune.ms_per_step = 0.0
    else:
        tune = B.autotune(3)
    st0 = [B.stats(k) for k in range(B.n)]
    with Clocks(local) as clk:
        ms = B.time_steps(a.steps)
    clocks = clk.summary()
    st1 = [B.stats(k) for k in range(B.n)]
    kernels = B.kernels_per_step()
    iters = [(st1[k].total_solve_steps - st0[k].total_solve_steps) / a.steps for k in range(B.n)]
    rows = [st1[k].active_cells for k in range(B.n)]
    conv = all(st1[k].converged for k in range(B.n))
    B.close()
    interior = sum((s - 2) ** 2 for s in sides)
    # algorithmic bytes: 618 B per interior cell for the 2D stages, 40 B per matrix row and CG iteration + 30 B
    # per row per solve
    step_bytes = 618.0 * interior + sum(40.0 * rows[k] * iters[k] + 30.0 * rows[k] for k in range(len(sides)))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = step_bytes / (ms / a.steps / 1e3) / 1e9
    # the same scenes as separate simulators, one stream each
    sims = []
    for k, (b, r) in enumerate(scenes):
        p = abi.params_dam(1.0 / sides[k], dt, abi.SOLVER_CG, 1e-6)
        p.max_steps = 20000
        S = gb.GB300Simulator2D(sides[k], sides[k], p)
        S.set_field(abi.FIELD_BOUNDARY, b)
        S.set_field(abi.FIELD_RHO, r)
        sims.append(S)
    for S in sims:
        S.update(a.warmup)
    for S in sims:
        S.synchronize()
    k_sep = max(3, a.steps // 4)
    t0 = time.perf_counter()
    for _ in range(k_sep):
        for S in sims:
            S.update(1)
    for S in sims:
        S.synchronize()
    sep_ms = (time.perf_counter() - t0) * 1e3 / k_sep
    for S in sims:
        S.close()
    cpu = None
    if not a.no_cpu:
        cpu = cpu_sample_batch([a.seed + k for k in range(a.scenes)], dt, 10)
    line = {"metric": f"scene-steps/s, {a.scenes} uneven 2D scenes (sides 64-256) to rel-res 1e-6",
            "value": a.scenes * a.steps / (ms / 1e3), "unit": "scene-steps/s", "n_gpus": 1, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch2d", "scenes": a.scenes, "seeds": [a.seed, a.seed + a.scenes - 1],
                       "sides": {str(s): sides.count(s) for s in sorted(set(sides))}, "dt": dt,
                       "solver": "cg rel-res 1e-6 (block-level, one scene per block)", "l2": "working set below L2"},
            "cell_updates_per_s": interior * a.steps / (ms / 1e3), "cg_iters_per_scene_step": float(np.mean(iters)),
            "cg_iters_max": float(np.max(iters)), "all_converged": conv, "gpu_launches": kernels * a.steps,
            "kernels_per_step": kernels, "tuning": tune.as_dict(),
            "separate_simulators": {"ms_per_step_all_scenes": sep_ms, "host_timed": True,
                                    "note": "one GB300Simulator2D per scene, each on its own stream"},
            "roofline": {"kernel": "whole batched step", "bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                         "algorithmic_bytes_per_step": step_bytes},
            "clocks": clocks, "cpu_baseline": cpu, "e2e": None}
    print(json.dumps(line), flush=True)


def _cpu_batch_scene(job):
    """Worker of cpu_sample_batch: `steps` oracle steps of one batch scene; returns the seconds they took."""
    seed, steps, dt = job
    from eulerianfluidsimulation_gb300 import abi
    from oracle import oracle
    b, r = oracle.scene_batch2d(seed)
    side = b.shape[0]
    prm = abi.params_dam(1.0 / side, dt, abi.SOLVER_CG, 1e-6)
    prm.max_steps = 20000
    o = oracle.Oracle(2, side, side, 1, prm, mode=oracle.SHARPEN_PARALLEL | oracle.DOTS_FP64)
    o.set_field(abi.FIELD_BOUNDARY, b)
    o.set_field(abi.FIELD_RHO, r)
    t0 = time.perf_counter()
    o.step(steps)
    return time.perf_counter() - t0


def _cpu_batch_warm(_):
    from oracle import oracle  # noqa: F401
    return 0


def cpu_sample_batch(seeds, dt, steps):
    """The CPU oracle (port of the reference CPUSimulator2D step) on every scene of the batch, one process per
    scene across the host cores (the reference's singletons forbid threads): `steps` steps of each scene."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    jobs = [(s, steps, dt) for s in seeds]
    with mp.get_context("spawn").Pool(cores) as pool:
        pool.map(_cpu_batch_warm, range(cores), chunksize=1)      # worker start-up and imports, untimed
        t0 = time.perf_counter()
        per_scene = pool.map(_cpu_batch_scene, jobs, chunksize=1)
        wall = time.perf_counter() - t0
    return {"value": len(seeds) * steps / wall, "unit": "scene-steps/s", "cores": cores, "kind": "port",
            "sample": f"{steps} steps of each of the {len(seeds)} scenes, one process per scene on {cores} cores "
                      f"({wall:.1f} s wall, {sum(per_scene):.1f} s of scene time)"}


def run_dam2d(a):
    """The 2D dam break on one 128^2 grid (dx = 1/128, dt = 0.005, fluid x < 0.4, y < 0.6, Jacobi 100 sweeps
    per step as MAX_STEPS = 200): steps/s with the fields resident, e2e through upload/step/download, and the
    CPU oracle timed on real steps of the same trajectory."""
    import eulerianfluidsimulation_gb300 as gb
    from eulerianfluidsimulation_gb300 import abi
    rank, world, local = dist_env()
    if rank != 0:
        return
    n = a.size
    solver = abi.SOLVER_CG if a.solver == "cg" else abi.SOLVER_JACOBI
    prm = abi.params_dam(1.0 / n, 0.005, solver, 1e-6)
    prm.max_steps = 200 if solver == abi.SOLVER_JACOBI else 20000
    b, r = gb.scene_dam2d(n, n)
    sim = gb.GB300Simulator2D(n, n, prm)
    sim.set_field(abi.FIELD_BOUNDARY, b)
    sim.set_field(abi.FIELD_RHO, r)
    sim.update(a.warmup)
    sim.synchronize()
    kernels = sim.kernels_per_step()
    st0 = sim.stats()
    with Clocks(local) as clk:
        sim.mark(0)
        sim.update(a.steps)
        sim.mark(1)
        ms = sim.elapsed_ms(0, 1)
    clocks = clk.summary()
    st1 = sim.stats()
    iters = (st1.total_solve_steps - st0.total_solve_steps) / max(a.steps, 1)
    e2e = None
    if not a.no_e2e:
        import torch
        h = {k: torch.empty(s, dtype=torch.float32, pin_memory=True).numpy()
             for k, s in (("vel", (n, n, 2)), ("rho", (n, n)), ("gamma", (n, n)), ("boundary", (n, n)),
                          ("forces", (n, n, 2)), ("beta", (n, n)), ("div", (n, n)), ("p", (n, n)))}
        sim.download_fields(vel=h["vel"], rho=h["rho"], gamma=h["gamma"], beta=h["beta"], divergence=h["div"], pressure=h["p"])
        h["boundary"][...] = b
        h["forces"][...] = 0

        def step_host():
            sim.upload_fields(vel=h["vel"], rho=h["rho"], gamma=h["gamma"], boundary=h["boundary"], forces=h["forces"])
            sim.update(1)
            sim.download_fields(vel=h["vel"], rho=h["rho"], gamma=h["gamma"], beta=h["beta"], divergence=h["div"], pressure=h["p"])
        # untimed warm-up call: the first upload of a forces field recaptures the step graph with the forces read
        step_host()
        sim.synchronize()
        sim.mark(2)
        for _ in range(a.steps):
            step_host()
        sim.mark(3)
        ms_e2e = sim.elapsed_ms(2, 3)
        e2e = {"value": a.steps / (ms_e2e / 1e3), "unit": "steps/s", "h2d_bytes_per_step": 4 * n * n * 7,
               "d2h_bytes_per_step": 4 * n * n * 7, "steps": a.steps, "warmup": 1,
               "api": "efs_upload_fields(vel,rho,gamma,boundary,forces) + efs_step + efs_download_fields(vel,rho,gamma,beta,div,p)"}
    sim.close()
    cpu = None
    if not a.no_cpu:
        cpu = cpu_sample_2d(n, prm, b, r, min(a.steps + a.warmup, 200))
    interior = (n - 2) ** 2
    per_iter = JACOBI_BYTES_PER_ROW_ITER if solver == abi.SOLVER_JACOBI else SOLVE_BYTES_PER_ROW_ITER
    step_bytes = STEP_BYTES_PER_CELL_2D * interior + per_iter * st1.active_cells * iters
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = step_bytes / (ms / a.steps / 1e3) / 1e9
    line = {"metric": f"steps/s, 2D dam break {n}^2 ({'Jacobi 100 sweeps' if solver == abi.SOLVER_JACOBI else 'CG rel-res 1e-6'})",
            "value": a.steps / (ms / 1e3), "unit": "steps/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"dam2d_{n}", "grid": [n, n], "dt": 0.005, "solver": a.solver,
                       "scene": "fluid x<0.4, y<0.6, solid border", "l2": "working set below L2 (no flush)"},
            "cell_updates_per_s": interior * a.steps / (ms / 1e3), "solve_iters_per_step": iters,
            "gpu_launches": kernels * a.steps, "kernels_per_step": kernels,
            "roofline": {"kernel": "whole step", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "algorithmic_bytes_per_step": step_bytes},
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks}
    print(json.dumps(line), flush=True)


def cpu_sample_2d(n, prm, b, r, steps):
    """The CPU oracle (port of the reference CPUSimulator2D step) on the same scene, `steps` real steps."""
    from eulerianfluidsimulation_gb300 import abi
    from oracle import oracle
    o = oracle.Oracle(2, n, n, 1, prm.copy())
    o.set_field(abi.FIELD_BOUNDARY, b)
    o.set_field(abi.FIELD_RHO, r)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    return {"value": steps / dt, "unit": "steps/s", "cores": 1, "kind": "port",
            "sample": f"{steps} steps of the {n}^2 dam break on 1 core ({dt:.2f} s)"}


def run_unet(a):
    """The U-Net preconditioner's forward pass alone on a --size^3 dam break (untrained weights; the FLOPs do
    not depend on them): ms per pass and per layer from CUDA events, TFLOP/s against the measured bf16 peak.
    One warm-up pass, then --steps timed passes of 6 convolutions each."""
    import eulerianfluidsimulation_gb300 as gb
    from eulerianfluidsimulation_gb300 import abi
    rank, world, local = dist_env()
    if rank != 0:
        return
    n = a.size
    b, r = gb.scene_dam3d(n, n, n, a.spheres, a.spheres, a.seed)
    prm = workload(a)
    prm.fcg_levels = a.fcg_levels       # 0: the network on the whole grid; < 0: on FCG's bottom grid
    sim = gb.GB300Simulator3D(n, n, n, prm)
    sim.set_field(abi.FIELD_BOUNDARY, b)
    sim.set_field(abi.FIELD_RHO, r)
    sim.update(1)
    sim.unet_init(a.seed + 7, 0)
    nw, nh, nd, level = sim.unet_grid()
    with Clocks(local) as clk:
        ms_fwd, ms_layers = sim.unet_time_forward(max(1, a.steps))
    clocks = clk.summary()
    sim.close()
    flops = unet_flops(nw)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    conv_ms = float(sum(ms_layers))
    achieved = sum(flops) / (conv_ms / 1e3) / 1e12
    per_layer = [{"layer": k, "cin_cout": list(UNET_LAYERS[k][:2]), "level": UNET_LAYERS[k][2], "ms": float(ms_layers[k]),
                  "TFLOP/s": flops[k] / (float(ms_layers[k]) / 1e3) / 1e12 if ms_layers[k] > 0 else None}
                 for k in range(len(UNET_LAYERS))]
    line = {"metric": f"U-Net forward TFLOP/s at {nw}^3 (tcgen05 convolutions)", "value": achieved,
            "unit": "TFLOP/s", "n_gpus": 1, "steps": max(1, a.steps), "warmup": 1, "ms_per_step": ms_fwd,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": f"unet_{n}", "network_grid": [nw, nh, nd], "hierarchy_level": level,
                       "channels": [16, 32, 64], "levels": 3, "kernel": "3x3x3"},
            "layers": per_layer,
            "roofline": {"kernel": "the 6 tcgen05 convolutions of one forward pass (k_conv3_halo_ws on levels at least 96 wide, k_conv3_slab below)", "bound": "tensor",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                         "flop_per_forward": sum(flops)},
            "gpu_launches": None, "clocks": clocks, "cpu_baseline": None, "e2e": None}
    print(json.dumps(line), flush=True)


def run_scene(a):
    """The scene kernels on a --size^3 grid: the mesh label (sdf.comp's test of every cell against every
    triangle of a closed sphere mesh) in cell-triangle tests/s, and the QueryNode box reduction over the whole
    grid in GB/s (rho, u, v, w, p: 20 B per cell, every cell counted).  CUDA events on the context's stream."""
    import eulerianfluidsimulation_gb300 as gb
    from eulerianfluidsimulation_gb300 import abi
    rank, world, local = dist_env()
    if rank != 0:
        return
    n = a.size
    b, r = gb.scene_dam3d(n, n, n, a.spheres, a.spheres, a.seed)
    sim = gb.GB300Simulator3D(n, n, n, workload(a))
    sim.set_field(abi.FIELD_BOUNDARY, b)
    sim.set_field(abi.FIELD_RHO, r)
    sim.update(2)
    sim.synchronize()
    # a closed UV sphere of 64 x 32 bands (4032 triangles) in the unit-cube domain
    nl, nm = 32, 64
    th = np.linspace(0, np.pi, nl + 1)
    ph = np.linspace(0, 2 * np.pi, nm + 1) + 0.1
    P = lambda i, j: 0.5 + 0.3 * np.array([np.sin(th[i]) * np.cos(ph[j]), np.cos(th[i]), np.sin(th[i]) * np.sin(ph[j])])
    tris = []
    for i in range(nl):
        for j in range(nm):
            if i > 0:
                tris.append((P(i, j), P(i + 1, j + 1), P(i, j + 1)))
            if i < nl - 1:
                tris.append((P(i, j), P(i + 1, j), P(i + 1, j + 1)))
    tris = np.asarray(tris, np.float32)
    center, size = (0.5, 0.5, 0.5), (1.0, 1.0, 1.0)
    sim.mesh_label(abi.FIELD_GAMMA, tris, center, size, 1.0, 1.0)       # warm-up
    reps = max(1, min(a.steps, 5))
    with Clocks(local) as clk:
        sim.mark(0)
        for _ in range(reps):
            sim.mesh_label(abi.FIELD_GAMMA, tris, center, size, 1.0, 1.0)
        sim.mark(1)
        ms_label = sim.elapsed_ms(0, 1) / reps
        for _ in range(3):
            sim.query_box((0, 0, 0), (n, n, n), False)
        qreps = max(3, a.steps)
        sim.mark(2)
        for _ in range(qreps):
            m = sim.query_box((0, 0, 0), (n, n, n), False)
        sim.mark(3)
        ms_query = sim.elapsed_ms(2, 3) / qreps
    clocks = clk.summary()
    sim.close()
    pairs = float((n - 1) ** 3) * len(tris)
    qcells = float((n - 1) ** 3)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    q_gbs = 20.0 * qcells / (ms_query / 1e3) / 1e9
    line = {"metric": f"mesh label cell-triangle tests/s and query-box GB/s at {n}^3", "value": pairs / (ms_label / 1e3),
            "unit": "cell-triangle tests/s", "n_gpus": 1, "steps": reps, "warmup": 1, "ms_per_step": ms_label,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"scene_{n}", "triangles": len(tris), "cells": (n - 1) ** 3,
                       "mesh": "closed UV sphere r=0.3 in the unit domain", "l2": "grid fields > L2 (query)"},
            "mesh_label_ms": ms_label, "query_box": {"ms": ms_query, "count": m.count, "GB/s": q_gbs,
                                                     "bytes_per_cell": 20},
            "roofline": {"kernel": "k_query (box reduction, every cell counted)", "bound": "hbm", "achieved": q_gbs,
                         "peak": peak, "unit": "GB/s", "frac": q_gbs / peak, "traffic": None},
            "gpu_launches": reps + 2 * qreps, "clocks": clocks, "cpu_baseline": None, "e2e": None}
    print(json.dumps(line), flush=True)


def run_precision_study(a):
    """One JSON line with the maxima of the per-step errors (the 3D dam break with --spheres spheres)."""
    from eulerianfluidsimulation_gb300.precision import precision_study
    t0 = time.time()
    rep = precision_study(3, a.size, a.steps, spheres=a.spheres, seed=a.seed, dt=a.dt)
    line = {"study": "precision", "workload": f"dam3d_{a.size}", "steps": a.steps, "spheres": a.spheres,
            "seed": a.seed, "tol_rel": rep["tol_rel"], "tol_fp64": rep["tol_fp64"], "max": rep["max"],
            "wall_s": round(time.time() - t0, 1)}
    if a.study_out:
        with open(a.study_out, "w") as f:
            json.dump(rep, f)
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.study == "precision":
        run_precision_study(a)
        return
    if a.workload == "batch2d":
        run_batch2d(a)
        return
    if a.workload == "dam2d":
        run_dam2d(a)
        return
    if a.workload == "scene":
        run_scene(a)
        return
    if a.workload == "unet":
        run_unet(a)
        return
    if a.impl == "reference":
        run_reference(a)
    elif a.solver == "fcg":
        run_fcg(a)
    else:
        run_gb300(a)


if __name__ == "__main__":
    main()
