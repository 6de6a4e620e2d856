"""Scene loading, geometry, node logic and the scene oracle, on the CPU.

- OBJ parsing (fans, negative indices, v/vt/vn), the quaternion matrix (glm::mat3_cast, zero quaternion ->
  identity) and the T*R*S transform;
- the oracle's sdf.comp label against the analytic inside test of a sphere and a box (cells away from the
  surface), and a box whose faces pass through cell centres (those cells are inside: distance 0);
- the oracle's QueryNode metrics against an FP64 numpy computation (count, min, max exact);
- a scene file written here: nodes, properties -> efs_params (GRAVITY_FORCE = GRAVITY / CELL_SIZE);
- the reference's own scene files, where the reference tree is present: every one parses, models load;
- QueryNode's three modes (history, averaging, gravity / position change, reset and pause), its CSV;
- force-field bookkeeping (first pending field, clear, capacity) and Scene2D load / reset / save, on the CPU
  model of the field store.
"""
import glob
import json
import os

import numpy as np
import pytest

from eulerianfluidsimulation_gb300 import abi
from eulerianfluidsimulation_gb300 import scene as S
from oracle import oracle
from tests.helpers import box_mesh, sphere_mesh, write_obj
from tests.scene_grid import OracleSceneGrid

REF_SCENES = os.path.join(oracle.reference_tree(), "assets", "scenes")


def _centres(shape, center, size):
    D, H, W = shape
    cs = np.asarray(size, np.float64) / np.array([W, H, D])
    mn = np.asarray(center, np.float64) - 0.5 * np.asarray(size, np.float64)
    z, y, x = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    return np.stack([mn[0] + cs[0] * (x + 0.5), mn[1] + cs[1] * (y + 0.5), mn[2] + cs[2] * (z + 0.5)], -1), cs


def _f32_centre(cell, shape, center, size):
    """sdf.comp's query position of a cell, in float32 operation by operation."""
    f = np.float32
    D, H, W = shape
    out = []
    for k, n in zip(range(3), (W, H, D)):
        cs = f(size[k]) / f(n)
        mn = f(center[k]) - f(0.5) * f(size[k])
        out.append(mn + cs * f(cell[k]) + cs * f(0.5))
    return np.array(out, np.float32)


def test_load_obj(tmp_path):
    p = tmp_path / "m.obj"
    p.write_text("# quad and a triangle\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\n"
                 "f 1//1 2//1 3//1 4//1\nf -4/1/1 -2/1/1 -1/1/1\n")
    t = S.load_obj(str(p))
    assert t.shape == (3, 3, 3)
    assert np.array_equal(t[0], [[0, 0, 0], [1, 0, 0], [1, 1, 0]])
    assert np.array_equal(t[1], [[0, 0, 0], [1, 1, 0], [0, 1, 0]])
    assert np.array_equal(t[2], [[0, 0, 0], [1, 1, 0], [0, 1, 0]])


def test_quaternion_and_transform():
    assert np.array_equal(S.quat_to_matrix(0, 0, 0, 0), np.eye(3, dtype=np.float32))
    assert np.array_equal(S.quat_to_matrix(1, 0, 0, 0), np.eye(3, dtype=np.float32))
    h = np.sqrt(0.5)
    r = S.quat_to_matrix(h, 0, 0, h)          # 90 degrees about z: x -> y
    assert np.allclose(r @ [1, 0, 0], [0, 1, 0], atol=1e-6)
    m = S.trs_matrix([1, 2, 3], (h, 0, 0, h), [2, 2, 2])
    assert np.allclose(S.transform_points(m, [[1, 0, 0]]), [[1, 4, 3]], atol=1e-6)


def test_oracle_label_sphere_and_box():
    shape, center, size = (20, 24, 28), (0.5, 0.6, 0.7), (1.4, 1.2, 1.0)
    pts, cs = _centres(shape, center, size)
    c, r = np.array([0.45, 0.55, 0.7]), 0.33
    lab = oracle.mesh_label(shape, sphere_mesh(c, r), center, size)
    d = np.linalg.norm(pts - c, axis=-1)
    far = np.abs(d - r) > 0.06          # beyond the chord error of the 12 x 24 sphere
    inner = np.zeros(shape, bool)
    inner[:-1, :-1, :-1] = True         # sdf.comp labels [0, W-1) x [0, H-1) x [0, D-1) only
    assert np.array_equal(lab[far & inner] != 0, (d < r)[far & inner])
    assert np.all(lab[~inner] == 0)
    # a box whose faces pass through cell centres (computed in float32 as sdf.comp computes them): those
    # centres are on the surface, hence inside
    lab = oracle.mesh_label(shape, box_mesh(_f32_centre((4, 5, 3), shape, center, size),
                                            _f32_centre((10, 12, 8), shape, center, size)), center, size)
    want = np.zeros(shape, bool)
    want[3:9, 5:13, 4:11] = True
    assert np.array_equal(lab != 0, want)


def test_oracle_query_matches_fp64():
    rng = np.random.default_rng(3)
    shape = (14, 16, 18)
    rho = rng.uniform(0, 1, shape).astype(np.float32)
    vel = rng.normal(size=shape + (3,)).astype(np.float32)
    p = rng.normal(size=shape).astype(np.float32)
    pos, sc = (2, 3, 1), (9, 20, 7)
    m, n = oracle.query_box(rho, vel, p, pos, sc, True)
    z0, z1, y0, y1, x0, x1 = 1, min(13, 8), 3, min(15, 23), 2, min(17, 11)
    sub = np.zeros(shape, bool)
    sub[z0:z1, y0:y1, x0:x1] = True
    sel = sub & (rho >= 0.5)
    z, y, x = np.nonzero(sel)
    assert n == len(x)
    assert np.array_equal(m["max_position"], [x.max(), y.max(), z.max()])
    assert np.array_equal(m["min_position"], [x.min(), y.min(), z.min()])
    assert np.allclose(m["avg_position"], [x.mean(), y.mean(), z.mean()], rtol=1e-6)
    assert np.allclose(m["velocity"], vel[sel].astype(np.float64).mean(0), rtol=1e-4, atol=1e-6)
    assert abs(m["pressure"] - p[sel].astype(np.float64).mean()) < 1e-5
    m0, n0 = oracle.query_box(rho, vel, p, (30, 30, 30), (2, 2, 2), True)
    assert n0 == 0 and np.all(m0["max_position"] == 0) and m0["pressure"] == 0.0


def _scene_file(tmp_path, W=24, H=20, D=16):
    write_obj(str(tmp_path / "ball.obj"), sphere_mesh((0.1, -0.1, 0.0), 0.3))
    doc = {"nodes": [
        {"type": "SimulationDomainNode", "name": "Simulation Domain", "position": [0.0, 0.0, 0.0],
         "scale": [W / 16.0, H / 16.0, D / 16.0], "resolution": [W, H, D]},
        {"type": "BoundingBoxFluidSpawnNode", "name": "Fluid Spawn", "position": [1.0, 1.0, 1.0], "scale": [8.0, 10.0, 14.0]},
        {"type": "ModelNode", "name": "Ball", "path": "ball.obj", "boundary": True, "position": [0.0, 0.0, 0.0],
         "rotation": [0.0, 0.0, 0.0, 0.0], "scale": [1.0, 1.0, 1.0]},
        {"type": "ForceFieldNode", "name": "Fan", "position": [-0.45, -0.3, 0.0], "rotation": [0.0, 0.0, 0.0, 1.0],
         "scale": [0.25, 0.25, 0.25], "active": True, "strength": 4.0},
        {"type": "QueryNode", "name": "Q", "position": [1.0, 1.0, 1.0], "scale": [10.0, 12.0, 8.0], "mode": 0,
         "onlyFluid": True, "enabled": True, "avgFrames": 5, "delayFrames": 20, "iterations": 200, "changeValue": 0.05},
        {"type": "DeletionNode", "name": "Sink", "position": [18.0, 1.0, 1.0], "scale": [4.0, 4.0, 4.0]},
        {"type": "CameraNode", "name": "Camera"},
    ], "properties": {"DT": 0.004, "Gravity": 9.81, "Cell Size": 0.0625, "Lambda-": 50.0, "Lambda+": 10.0,
                      "Eta": 100.0, "D": 32.0, "Max Steps": 3000, "Disable Velocity Decay": True,
                      "Max ForceField cells": 1000}}
    path = tmp_path / "scene.json"
    path.write_text(json.dumps(doc))
    return str(path)


def test_scene3d_load(tmp_path):
    s = S.Scene3D.load(_scene_file(tmp_path), assets_root=str(tmp_path))
    assert s.resolution == [24, 20, 16] and s.shape == (16, 20, 24)
    assert len(s.box_spawns) == 1 and len(s.boundaries) == 1 and len(s.force_fields) == 1
    assert len(s.queries) == 1 and len(s.deletions) == 1 and not s.warnings
    p = s.params()
    assert p.gravity_force == np.float32(np.float32(9.81) / np.float32(0.0625))
    assert p.max_steps == 3000 and p.disable_mask & (1 << abi.STAGE_VEL_DECAY)
    assert np.allclose(s.force_fields[0]["direction"], [1, 0, 0])


@pytest.mark.skipif(not os.path.isdir(REF_SCENES), reason="reference scene files not present")
def test_reference_scenes_parse():
    files = sorted(glob.glob(os.path.join(REF_SCENES, "*.json")))
    assert files
    for f in files:
        s = S.Scene3D.load(f)
        assert not s.warnings, (f, s.warnings)
        assert all(len(b) > 0 for b in s.boundaries), f
        p = s.params()
        assert np.isfinite(p.gravity_force) and p.dt > 0


def test_scene_init_on_the_cpu_model(tmp_path):
    s = S.Scene3D.load(_scene_file(tmp_path), assets_root=str(tmp_path))
    g = OracleSceneGrid(s.shape)
    s.init(g)
    rho, bnd = g.field(abi.FIELD_RHO), g.field(abi.FIELD_BOUNDARY)
    assert np.all(bnd[0] == 1) and np.all(bnd[:, :, -1] == 1)
    assert np.all(rho[bnd != 0] == 0)
    assert bnd[1:-1, 1:-1, 1:-1].sum() > 0                  # the ball
    assert rho[5, 5, 5] == 1.0 and rho[5, 5, 12] == 0.0      # inside / outside the spawn box (x < 9)
    state = {"frames": 0, "gravity": 9.81}
    s.update(g, state)
    f = g.field(abi.FIELD_FORCES)
    cells = s.force_fields[0]["cells"]
    assert len(cells) > 0 and not s.force_fields[0]["pending"]
    assert np.allclose(f.reshape(-1, 3)[cells], [4.0, 0.0, 0.0])
    assert np.count_nonzero(np.any(f != 0, axis=-1)) == len(cells)
    assert len(s.queries[0].history) == 1


def test_force_field_capacity(tmp_path):
    s = S.Scene3D.load(_scene_file(tmp_path), assets_root=str(tmp_path))
    g = OracleSceneGrid(s.shape)
    s.init(g)
    s.update_force_fields(g, max_cells=3)          # too many cells: skipped, nothing cleared or written
    assert s.force_fields[0]["pending"] and not np.any(g.field(abi.FIELD_FORCES))


class _Fixed:
    """query_box returns frame-dependent constant metrics."""
    dim, shape = 3, (10, 10, 10)

    def __init__(self):
        self.k = 0.0

    def query_box(self, position, scale, only_fluid=True):
        m = abi.EfsQueryMetrics()
        for key in ("max_position", "min_position", "avg_position", "velocity"):
            getattr(m, key)[:] = [self.k, self.k, self.k]
        m.pressure = self.k
        m.count = 1
        return m


def test_query_node_modes(tmp_path):
    sim = _Fixed()
    q = S.QueryNode({"mode": 0, "position": [0, 0, 0], "scale": [4, 4, 4]})
    state = {"frames": 0, "gravity": 9.81}
    for k in range(3):
        sim.k = k
        q.update(sim, state)
    state["paused"] = True
    q.update(sim, state)
    assert len(q.history) == 3 and q.history[2][0] == 2.0 and q.history[0][-1] == np.float32(9.81)

    q = S.QueryNode({"mode": 1, "delayFrames": 2, "avgFrames": 3, "iterations": 2, "changeValue": 0.5,
                     "position": [0, 0, 0], "scale": [4, 4, 4]})
    state = {"frames": 0, "gravity": 1.0}
    resets = 0
    for _ in range(20):
        if state.get("paused"):
            break
        sim.k = state["frames"]
        q.update(sim, state)
        state["frames"] += 1
        if state.pop("reset", False):
            resets += 1
            state["frames"] = 0
    # each round: frames 2, 3, 4 averaged (mean 3), kept at frame 5, then reset with gravity + 0.5
    assert resets == 2 and state["paused"] and len(q.history) == 2
    assert q.history[0][0] == 3.0 and q.history[0][-1] == 1.0 and q.history[1][-1] == 1.5
    q.export_csv(str(tmp_path / "q.csv"), 0.004, 0.0625, (10, 10, 10), {"DT": 0.004})
    lines = (tmp_path / "q.csv").read_text().splitlines()
    assert lines[0].startswith("frame,max_pos_x") and lines[0].endswith(",grid_depth,DT")
    assert len(lines) == 3 and lines[1].split(",")[0] == "0"


def test_scene2d_roundtrip(tmp_path):
    W, H = 12, 9
    b = [i for i in range(W * H) if i % W in (0, W - 1) or i // W in (0, H - 1)] + [5 * W + 5]
    fl = [2 * W + 3, 2 * W + 4, 3 * W + 3]
    path = tmp_path / "s.scene2D"
    path.write_text(json.dumps({"width": W, "height": H, "boundary": b, "fluid": fl, "properties": {"DT": 0.01}}))
    sc = S.Scene2D.load(str(path))
    assert sc.params().dt == np.float32(0.01)
    g = OracleSceneGrid((H, W))
    g.fields[abi.FIELD_RHO][...] = 0.7
    sc.reset(g)
    assert sorted(np.nonzero(g.field(abi.FIELD_BOUNDARY).ravel())[0].tolist()) == sorted(b)
    assert np.nonzero(g.field(abi.FIELD_RHO).ravel())[0].tolist() == fl

    class _Sim:
        def field(self, f):
            return g.field(f)
    sc.save(_Sim(), str(tmp_path / "t.scene2D"))
    back = S.Scene2D.load(str(tmp_path / "t.scene2D"))
    assert sorted(back.boundary.tolist()) == sorted(b) and back.fluid.tolist() == fl


# ---- Scene2D::loadImage (Scene2D.cpp:87-121) and the 8-bit grey reading it relies on ----------------------------
def _png_chunk(kind, body):
    import struct
    import zlib
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _png_filter_rows(raw, bpp):
    """PNG's five row filters applied in turn (row y uses filter y % 5), written from the PNG specification."""
    out = bytearray()
    prev = np.zeros(raw.shape[1], np.int64)
    for y, line in enumerate(raw.astype(np.int64)):
        f = y % 5
        left = np.concatenate([np.zeros(bpp, np.int64), line[:-bpp]])
        upleft = np.concatenate([np.zeros(bpp, np.int64), prev[:-bpp]])
        if f == 0:
            pred = np.zeros_like(line)
        elif f == 1:
            pred = left
        elif f == 2:
            pred = prev
        elif f == 3:
            pred = (left + prev) // 2
        else:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
        out.append(f)
        out += ((line - pred) & 0xFF).astype(np.uint8).tobytes()
        prev = line
    return bytes(out)


def _pack_rows(samples, bits):
    """(h, w * channels) integer samples -> (h, row_bytes) uint8 scanlines at `bits` per sample."""
    if bits == 8:
        return samples.astype(np.uint8)
    if bits == 16:
        s = samples.astype(np.int64)
        return np.stack([s >> 8, s & 0xFF], -1).reshape(s.shape[0], -1).astype(np.uint8)
    bitsarr = ((samples[..., None] >> np.arange(bits - 1, -1, -1)) & 1).reshape(samples.shape[0], -1)
    return np.packbits(bitsarr.astype(np.uint8), axis=1)


def _write_png(path, samples, ctype, bits, palette=None, adam7=False):
    """samples: (h, w, channels) integers; every row filter is used; Adam7 writes the seven passes in turn."""
    import struct
    import zlib
    h, w, ch = samples.shape
    bpp = max(1, ch * bits // 8)
    if adam7:
        data = b""
        for x0, y0, dx, dy in ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2),
                               (0, 1, 1, 2)):
            part = samples[y0::dy, x0::dx]
            if part.size == 0:
                continue
            data += _png_filter_rows(_pack_rows(part.reshape(part.shape[0], -1), bits), bpp)
    else:
        data = _png_filter_rows(_pack_rows(samples.reshape(h, -1), bits), bpp)
    png = b"\x89PNG\r\n\x1a\n" + _png_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, bits, ctype, 0, 0, 1 if adam7 else 0))
    if palette is not None:
        png += _png_chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    png += _png_chunk(b"IDAT", zlib.compress(data)) + _png_chunk(b"IEND", b"")
    path.write_bytes(png)


def _luma(rgb):
    rgb = rgb.astype(np.int64)
    return (rgb[..., 0] * 77 + rgb[..., 1] * 150 + rgb[..., 2] * 29) >> 8


def test_read_grey8_png_all_colour_types(tmp_path):
    from eulerianfluidsimulation_gb300.image import read_grey8
    rng = np.random.default_rng(3)
    h, w = 13, 17
    grey = rng.integers(0, 256, (h, w, 1))
    _write_png(tmp_path / "g8.png", grey, 0, 8)
    assert np.array_equal(read_grey8(str(tmp_path / "g8.png")), grey[..., 0])
    _write_png(tmp_path / "g8i.png", grey, 0, 8, adam7=True)
    assert np.array_equal(read_grey8(str(tmp_path / "g8i.png")), grey[..., 0])
    rgb = rng.integers(0, 256, (h, w, 3))
    _write_png(tmp_path / "rgb.png", rgb, 2, 8)
    assert np.array_equal(read_grey8(str(tmp_path / "rgb.png")), _luma(rgb))
    rgba = rng.integers(0, 256, (h, w, 4))
    _write_png(tmp_path / "rgba.png", rgba, 6, 8)
    assert np.array_equal(read_grey8(str(tmp_path / "rgba.png")), _luma(rgba))
    ga = rng.integers(0, 256, (h, w, 2))
    _write_png(tmp_path / "ga.png", ga, 4, 8)
    assert np.array_equal(read_grey8(str(tmp_path / "ga.png")), ga[..., 0])
    g16 = rng.integers(0, 65536, (h, w, 1))
    _write_png(tmp_path / "g16.png", g16, 0, 16)
    assert np.array_equal(read_grey8(str(tmp_path / "g16.png")), g16[..., 0] >> 8)
    rgb16 = rng.integers(0, 65536, (h, w, 3))
    _write_png(tmp_path / "rgb16.png", rgb16, 2, 16, adam7=True)
    assert np.array_equal(read_grey8(str(tmp_path / "rgb16.png")), _luma(rgb16) >> 8)
    for bits, scale in ((1, 255), (2, 85), (4, 17)):
        low = rng.integers(0, 1 << bits, (h, w, 1))
        _write_png(tmp_path / f"g{bits}.png", low, 0, bits)
        assert np.array_equal(read_grey8(str(tmp_path / f"g{bits}.png")), low[..., 0] * scale), bits
    pal = rng.integers(0, 256, (16, 3))
    idx = rng.integers(0, 16, (h, w, 1))
    _write_png(tmp_path / "p4.png", idx, 3, 4, palette=pal)
    assert np.array_equal(read_grey8(str(tmp_path / "p4.png")), _luma(pal[idx[..., 0]]))


def test_read_grey8_netpbm_and_bmp(tmp_path):
    import struct
    from eulerianfluidsimulation_gb300.image import read_grey8
    rng = np.random.default_rng(4)
    h, w = 7, 10
    g = rng.integers(0, 256, (h, w)).astype(np.uint8)
    (tmp_path / "a.pgm").write_bytes(b"P5\n# comment\n%d %d\n255\n" % (w, h) + g.tobytes())
    assert np.array_equal(read_grey8(str(tmp_path / "a.pgm")), g)
    rgb = rng.integers(0, 256, (h, w, 3)).astype(np.uint8)
    (tmp_path / "a.ppm").write_bytes(b"P6 %d %d 255\n" % (w, h) + rgb.tobytes())
    assert np.array_equal(read_grey8(str(tmp_path / "a.ppm")), _luma(rgb))
    # 24-bit BMP, rows bottom-up and padded to 4 bytes
    stride = (w * 3 + 3) // 4 * 4
    rows = b"".join(rgb[y][:, ::-1].tobytes() + b"\0" * (stride - w * 3) for y in range(h - 1, -1, -1))
    hdr = b"BM" + struct.pack("<IHHI", 54 + len(rows), 0, 0, 54) + struct.pack("<IiiHHIIiiII", 40, w, h, 1, 24, 0,
                                                                                len(rows), 0, 0, 0, 0)
    (tmp_path / "a.bmp").write_bytes(hdr + rows)
    assert np.array_equal(read_grey8(str(tmp_path / "a.bmp")), _luma(rgb))


@pytest.mark.parametrize("threshold", [128, -128, 1])
def test_scene2d_from_image(tmp_path, threshold):
    """The reference's loop: pixel i = x + y W is rho 1 when below the threshold (threshold > 0), or when at
    least |threshold| (threshold <= 0); boundary 1 on the outermost cells; the grid is the image's size."""
    rng = np.random.default_rng(5)
    h, w = 11, 16
    g = rng.integers(0, 256, (h, w, 1))
    _write_png(tmp_path / "scene.png", g, 0, 8)
    sc = S.Scene2D.from_image(str(tmp_path / "scene.png"), threshold)
    assert (sc.width, sc.height) == (w, h)
    want_rho = np.zeros(w * h, np.float32)
    want_b = np.zeros(w * h, np.float32)
    for x in range(w):
        for y in range(h):
            i = x + y * w
            p = int(g[y, x, 0])
            if threshold > 0:
                want_rho[i] = 1.0 if p < threshold else 0.0
            else:
                want_rho[i] = 0.0 if p < abs(threshold) else 1.0
            if x == 0 or x == w - 1 or y == 0 or y == h - 1:
                want_b[i] = 1.0
    grid = OracleSceneGrid((h, w))
    sc.reset(grid)
    assert np.array_equal(grid.field(abi.FIELD_RHO).ravel(), want_rho)
    assert np.array_equal(grid.field(abi.FIELD_BOUNDARY).ravel(), want_b)
