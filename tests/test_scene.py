"""Scene construction and queries on the GPU (efs_mesh_label, efs_mesh_cells, efs_fill_box, efs_set_cells,
efs_seal_boundary, efs_query_box) against the oracle and the CPU model of the field store.

- mesh labels (a sphere, a rotated box, a box whose faces pass through cell centres) equal the oracle's
  restatement of sdf.comp cell for cell, for a scalar field and for the boundary;
- the inside-cell list equals the oracle's labels in ascending order, with the count reported past capacity;
- fills, listed cells (vector fields, 2D, clipping) and the boundary seal equal the CPU model; an index
  outside the grid is EFS_ERR_ARG;
- query metrics: count, min and max exact, the means within 1e-6 of an FP64 numpy mean (the reference sums
  in float; the oracle's float sums are checked against the same numpy means on the CPU);
- a scene file built by Scene3D.init on the GPU equals the same calls on the CPU model, force fields and
  queries included; forces set after the step graph was captured act on the next step as in the oracle;
- a .scene2D file reset on a 2D simulator equals the CPU model.
"""
import json

import numpy as np
import pytest

from eulerianfluidsimulation_gb300 import abi
from eulerianfluidsimulation_gb300 import scene as S
from tests.helpers import box_mesh, rel_l2, sphere_mesh, write_obj
from tests.scene_grid import OracleSceneGrid

pytestmark = pytest.mark.gpu

gb = pytest.importorskip("eulerianfluidsimulation_gb300")
from oracle import oracle  # noqa: E402

SHAPE, CENTER, SIZE = (32, 36, 40), (0.1, 0.5, -0.2), (2.0, 1.8, 1.6)


def _centre(cell):
    """sdf.comp's query position of a cell, float32 operation by operation."""
    f = np.float32
    D, H, W = SHAPE
    out = []
    for k, n in zip(range(3), (W, H, D)):
        cs = f(SIZE[k]) / f(n)
        mn = f(CENTER[k]) - f(0.5) * f(SIZE[k])
        out.append(mn + cs * f(cell[k]) + cs * f(0.5))
    return np.array(out, np.float32)


def _meshes():
    rot = S.trs_matrix([0.2, 0.4, -0.1], (np.cos(0.3), 0.3, np.sin(0.3) * 0.8, 0.2), [0.6, 0.3, 0.5])
    rbox = S.transform_points(rot, S.cube_triangles().reshape(-1, 3)).reshape(-1, 3, 3)
    return {"sphere": sphere_mesh((0.0, 0.45, -0.25), 0.5), "rotated_box": rbox,
            "on_faces": box_mesh(_centre((5, 7, 4)), _centre((20, 25, 17)))}


def _sim3(params=None):
    D, H, W = SHAPE
    return gb.GB300Simulator3D(W, H, D, params or abi.params_dam(1.0 / 32, 0.004, abi.SOLVER_CG, 1e-6))


@pytest.mark.parametrize("name", ["sphere", "rotated_box", "on_faces"])
def test_mesh_label_matches_oracle(name):
    tris = _meshes()[name]
    with _sim3() as sim:
        start = np.full(SHAPE, 0.5, np.float32)
        sim.set_field(abi.FIELD_RHO, start)
        sim.mesh_label(abi.FIELD_RHO, tris, CENTER, SIZE, 0.75, 0.25)
        want = oracle.mesh_label(SHAPE, tris, CENTER, SIZE, 0.75, 0.25, out=start)
        got = sim.field(abi.FIELD_RHO)
        assert np.array_equal(got, want), int(np.sum(got != want))
        assert np.count_nonzero(want == 0.75) > 0
        sim.fill_box(abi.FIELD_BOUNDARY, (0, 0, 0), SHAPE[::-1], 0.0)
        sim.mesh_label(abi.FIELD_BOUNDARY, tris, CENTER, SIZE, 1.0, 0.0)
        lab = oracle.mesh_label(SHAPE, tris, CENTER, SIZE, 1.0, 0.0)
        assert np.array_equal(sim.field(abi.FIELD_BOUNDARY), lab)


def test_mesh_cells_ordered_and_capacity():
    tris = _meshes()["sphere"]
    lab = oracle.mesh_label(SHAPE, tris, CENTER, SIZE, 1.0, 0.0)
    want = np.nonzero(lab.ravel())[0]
    with _sim3() as sim:
        cells, n = sim.mesh_cells(tris, CENTER, SIZE)
        assert n == len(want) and np.array_equal(cells, want)
        cells, n = sim.mesh_cells(tris, CENTER, SIZE, capacity=100)
        assert n == len(want) and np.array_equal(cells, want[:100])
        cells, n = sim.mesh_cells(np.zeros((0, 3, 3), np.float32), CENTER, SIZE)
        assert n == 0 and len(cells) == 0


def test_fill_set_seal_match_the_cpu_model():
    D, H, W = SHAPE
    rng = np.random.default_rng(5)
    with _sim3() as sim:
        cpu = OracleSceneGrid(SHAPE)
        for g in (sim, cpu):
            g.reset()
            g.fill_box(abi.FIELD_RHO, (-3, 2, 4), (10, 50, 9), 1.0)
            g.fill_box(abi.FIELD_VEL, (5, 5, 5), (8, 9, 10), [1.0, -2.0, 3.0])
            g.fill_box(abi.FIELD_BOUNDARY, (12, 0, 0), (14, 30, 20), 1.0)
        cells = rng.choice(W * H * D, 500, replace=False)
        for g in (sim, cpu):
            g.set_cells(abi.FIELD_FORCES, cells, [0.5, 0.25, -1.0])
            g.set_cells(abi.FIELD_GAMMA, cells[:50], 3.0)
            g.seal_boundary()
        for f in (abi.FIELD_RHO, abi.FIELD_VEL, abi.FIELD_BOUNDARY, abi.FIELD_FORCES, abi.FIELD_GAMMA):
            assert np.array_equal(sim.field(f), cpu.field(f)), abi.FIELD_NAMES[f]
        with pytest.raises(gb.EfsError) as e:
            sim.set_cells(abi.FIELD_RHO, [0, W * H * D], 1.0)
        assert e.value.status == abi.EFS_ERR_ARG
        sim.fill_box(abi.FIELD_RHO, (0, 0, 0), (1, 1, 1), 0.0)     # the context stays usable


def _query_fp64(rho, vel, p, pos, sc, only_fluid):
    D, H, W = rho.shape
    lo = [max(0, v) for v in pos]
    hi = [min(n - 1, v + s) for v, s, n in zip(pos, sc, (W, H, D))]
    sel = np.zeros(rho.shape, bool)
    sel[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = True
    if only_fluid:
        sel &= rho >= 0.5
    z, y, x = np.nonzero(sel)
    return sel, x, y, z


@pytest.mark.parametrize("pos,sc,only_fluid", [((2, 1, 3), (20, 30, 12), True), ((-4, 5, 0), (100, 8, 100), True),
                                                ((1, 1, 1), (30, 30, 30), False), ((39, 35, 31), (4, 4, 4), True)])
def test_query_box(pos, sc, only_fluid):
    D, H, W = SHAPE
    b, r = gb.scene_dam3d(W, H, D, 3, 3, 7)
    with _sim3() as sim:
        sim.set_field(abi.FIELD_BOUNDARY, b)
        sim.set_field(abi.FIELD_RHO, r)
        sim.update(3)
        rho, vel, p = sim.rho(), sim.vel(), sim.pressure()
        m = sim.query_box(pos, sc, only_fluid)
    sel, x, y, z = _query_fp64(rho, vel, p, pos, sc, only_fluid)
    assert m.count == len(x)
    if not len(x):
        assert m.pressure == 0.0 and list(m.max_position) == [0, 0, 0]
        return
    assert list(m.max_position) == [x.max(), y.max(), z.max()]
    assert list(m.min_position) == [x.min(), y.min(), z.min()]
    assert np.allclose(m.avg_position, [x.mean(), y.mean(), z.mean()], rtol=1e-6, atol=0)
    v64 = vel[sel].astype(np.float64)
    scale = np.abs(v64).mean() + 1e-30
    assert np.all(np.abs(np.array(m.velocity) - v64.mean(0)) <= 1e-6 * scale)
    p64 = p[sel].astype(np.float64)
    assert abs(m.pressure - p64.mean()) <= 1e-6 * (np.abs(p64).mean() + 1e-30)
    mo, no = oracle.query_box(rho, vel, p, pos, sc, only_fluid)
    assert no == m.count and np.array_equal(mo["max_position"], m.max_position)


def _scene(tmp_path, W=40, H=36, D=32):
    write_obj(str(tmp_path / "ball.obj"), sphere_mesh((0.15, -0.2, 0.05), 0.35))
    doc = {"nodes": [
        {"type": "SimulationDomainNode", "position": [0.0, 0.0, 0.0], "scale": [W / 20.0, H / 20.0, D / 20.0],
         "resolution": [W, H, D]},
        {"type": "BoundingBoxFluidSpawnNode", "position": [1.0, 1.0, 1.0], "scale": [14.0, 20.0, 30.0]},
        {"type": "ModelNode", "path": "ball.obj", "boundary": True, "position": [0.0, 0.0, 0.0],
         "rotation": [0.0, 0.0, 0.0, 0.0], "scale": [1.0, 1.0, 1.0]},
        {"type": "ForceFieldNode", "position": [-0.6, -0.4, 0.0], "rotation": [0.0, 0.0, 0.38268343, 0.9238795],
         "scale": [0.3, 0.3, 0.3], "active": True, "strength": 40.0},
        {"type": "QueryNode", "position": [1.0, 1.0, 1.0], "scale": [20.0, 12.0, 30.0], "mode": 0, "onlyFluid": True},
    ], "properties": {"DT": 0.004, "Gravity": 9.81, "Cell Size": 0.05, "Lambda-": 50.0, "Lambda+": 10.0,
                      "Eta": 100.0, "D": 32.0, "Max Steps": 20000, "Disable Velocity Decay": True,
                      "Max ForceField cells": 5000}}
    path = tmp_path / "scene.json"
    path.write_text(json.dumps(doc))
    return S.Scene3D.load(str(path), assets_root=str(tmp_path))


def test_scene_build_matches_the_cpu_model(tmp_path):
    sc = _scene(tmp_path)
    W, H, D = sc.resolution
    prm = sc.params(abi.params_dam(1.0 / 20, 0.004, abi.SOLVER_CG, 1e-6))
    cpu = OracleSceneGrid(sc.shape)
    sc.init(cpu)
    sc.update(cpu, {"frames": 0, "gravity": 9.81})
    cells_cpu = sc.force_fields[0]["cells"].copy()
    hist_cpu = list(sc.queries[0].history)
    sc2 = _scene(tmp_path)
    with gb.GB300Simulator3D(W, H, D, prm) as sim:
        sc2.init(sim)
        sc2.update(sim, {"frames": 0, "gravity": 9.81})
        for f in (abi.FIELD_RHO, abi.FIELD_BOUNDARY, abi.FIELD_GAMMA, abi.FIELD_VEL, abi.FIELD_FORCES):
            assert np.array_equal(sim.field(f), cpu.field(f)), abi.FIELD_NAMES[f]
        assert np.array_equal(sc2.force_fields[0]["cells"], cells_cpu) and len(cells_cpu) > 0
        got, want = np.array(sc2.queries[0].history[0]), np.array(hist_cpu[0])
        assert np.allclose(got, want, rtol=1e-6, atol=1e-6)


def test_forces_set_after_capture_act_on_the_next_step(tmp_path):
    sc = _scene(tmp_path)
    W, H, D = sc.resolution
    prm = sc.params(abi.params_dam(1.0 / 20, 0.004, abi.SOLVER_CG, 1e-6))
    with gb.GB300Simulator3D(W, H, D, prm) as sim:
        sc.init(sim)
        sim.update(1)                                   # the step graph exists, without the force term
        state = sim.fields()
        sc.update_force_fields(sim)
        forces = sim.field(abi.FIELD_FORCES)
        assert np.any(forces != 0)
        sim.update(1)
        o = oracle.Oracle(3, W, H, D, prm, mode=oracle.SHARPEN_PARALLEL | oracle.DOTS_FP64)
        for f, a in state.items():
            o.set_field(f, a)
        o.set_field(abi.FIELD_FORCES, forces)
        o.step(1)
        for f in (abi.FIELD_VEL, abi.FIELD_RHO, abi.FIELD_PRESSURE):
            assert rel_l2(sim.field(f), o.field(f)) <= 1e-5, abi.FIELD_NAMES[f]


def test_scene2d_reset(tmp_path):
    W, H = 48, 40
    b = [i for i in range(W * H) if i % W in (0, W - 1) or i // W in (0, H - 1) or (i % W == 20 and i // W < 15)]
    fl = [y * W + x for y in range(1, 20) for x in range(1, 15)]
    path = tmp_path / "s.scene2D"
    path.write_text(json.dumps({"width": W, "height": H, "boundary": b, "fluid": fl}))
    sc = S.Scene2D.load(str(path))
    cpu = OracleSceneGrid((H, W))
    sc.reset(cpu)
    with gb.GB300Simulator2D(W, H, abi.params_dam(1.0 / W, 0.005, abi.SOLVER_CG, 1e-6)) as sim:
        sc.reset(sim)
        for f in (abi.FIELD_BOUNDARY, abi.FIELD_RHO):
            assert np.array_equal(sim.field(f), cpu.field(f))
        sim.update(2)
        assert sim.stats().converged
        m = sim.query_box((0, 0, 0), (W, H, 1), True)
        assert m.count == int(np.sum(sim.rho()[:H - 1, :W - 1] >= 0.5))
