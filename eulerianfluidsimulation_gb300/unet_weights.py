"""Trained weights of the FCG preconditioner's network, and the training run that makes them.

The network (include/efs_gb300.h, efs_unet_*) is FCG's coarsest-level solve: on the 3D dam-break grids of 128^3
and 256^3 that level is a 32^3 grid (2 and 3 aggregation levels).  One set of weights serves both, because the
network's geometry inputs are normalised by the level (face weights / 4^level).

Training data: plain-CG trajectories of the seeded dam break (include/efs_scene.h: fluid box x < 0.4, y < 0.6,
4-24 solid spheres, dt 0.004, CG to relative residual 1e-6) at 128^3 and 256^3.  After every step's projection
the right-hand side (the divergence) is carried down the V-cycle to the network's grid and stored with its
exact solution there (efs_unet_add_sample); half of every training batch are synthetic multi-scale errors on a
stored sample's matrix.  Loss: the energy-norm alignment 1 - (z.r)^2 / ((z.Az)(e.r)).

    python -m eulerianfluidsimulation_gb300.unet_weights --train     (on a GPU; writes WEIGHTS_PATH)
"""
import argparse
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS_PATH = os.path.join(HERE, "data", "unet_fcg_dam3d.npz")


def available():
    return os.path.exists(WEIGHTS_PATH)


def load():
    """(weights float32 [efs_unet_param_count], metadata dict)."""
    z = np.load(WEIGHTS_PATH)
    return z["weights"].astype(np.float32), json.loads(str(z["meta"]))


def load_into(sim):
    """Give `sim` (a GB300Simulator3D whose params select FCG's levels) the committed network.  Returns the
    metadata of the training run."""
    w, meta = load()
    sim.unet_init(0, 0)
    sim.unet_set_weights(w)
    meta = dict(meta)
    meta["network_grid"] = list(sim.unet_grid())
    return meta


def _params(n, abi):
    p = abi.params_dam(1.0 / n, 0.004, abi.SOLVER_CG, 1e-6)
    p.max_steps = 20000
    p.fcg_levels = -1
    return p


def train(sizes=(128, 256), samples=(10000, 10000), trajectory=250, rounds=6, iters_per_round=3000, batch=8,
          lr=1e-3, synthetic=0.5, seed=0, log=print):
    """Collect samples along plain-CG trajectories at each grid size (`trajectory` steps per seeded scene, new
    scene after that), then train for `rounds` rounds of `iters_per_round` Adam steps on each size's samples
    in turn.  Returns (weights, metadata)."""
    import eulerianfluidsimulation_gb300 as gb
    from eulerianfluidsimulation_gb300 import abi
    rng = np.random.default_rng(seed)
    ctxs = []
    t0 = time.perf_counter()
    total = 0
    for n, count in zip(sizes, samples):
        s = gb.GB300Simulator3D(n, n, n, _params(n, abi))
        s.unet_init(seed + 1, count)
        got, scene = 0, 0
        while got < count:
            spheres = int(rng.integers(4, 25))
            b, r = gb.scene_dam3d(n, n, n, spheres, spheres, 1000 * n + scene)
            s.reset()
            s.set_field(abi.FIELD_BOUNDARY, b)
            s.set_field(abi.FIELD_RHO, r)
            for _ in range(min(trajectory, count - got)):
                s.update(1)
                s.unet_add_sample()
                got += 1
            scene += 1
        s.synchronize()
        total += got
        log(f"{n}^3: {got} samples from {scene} trajectories, network grid {s.unet_grid()}")
        ctxs.append(s)
    t1 = time.perf_counter()
    w = ctxs[0].unet_weights()
    losses = []
    for rd in range(rounds):
        for k, s in enumerate(ctxs):
            s.unet_set_weights(w)
            loss = s.unet_train(iters_per_round, batch, lr * (0.5 ** rd), synthetic, seed + 100 * rd + k, loss_kind=1)
            w = s.unet_weights()
            losses.append(float(loss))
            log(f"round {rd} size {sizes[k]}: loss {loss:.4f}")
    t2 = time.perf_counter()
    for s in ctxs:
        s.close()
    meta = {"sizes": list(sizes), "samples": total, "samples_per_size": list(samples), "trajectory_steps": trajectory,
            "spheres": [4, 24], "rounds": rounds, "iterations": rounds * len(sizes) * iters_per_round, "batch": batch,
            "lr": lr, "synthetic_fraction": synthetic, "loss": "energy-norm alignment", "loss_last": losses[-1],
            "losses": losses, "collect_s": round(t1 - t0, 1), "train_s": round(t2 - t1, 1), "seed": seed}
    return w, meta


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", action="store_true")
    ap.add_argument("--samples", type=int, default=10000, help="samples per grid size")
    ap.add_argument("--rounds", type=int, default=6)
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--out", default=WEIGHTS_PATH)
    a = ap.parse_args()
    if not a.train:
        print(json.dumps(load()[1]) if available() else "no weights file")
        return
    w, meta = train(samples=(a.samples, a.samples), rounds=a.rounds, iters_per_round=a.iters)
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    np.savez_compressed(a.out, weights=w, meta=json.dumps(meta))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
