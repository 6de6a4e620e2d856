"""Scenes of the reference application on the GB300 field store: loading, building the grid, force fields and
query metrics.

The reference keeps this in its application layer (src/simulation/scene/, src/core/Editor.cpp,
src/simulation/data/Scene2D.cpp); its arithmetic over the grid runs here as CUDA kernels of the library
(``efs_mesh_label``, ``efs_mesh_cells``, ``efs_fill_box``, ``efs_set_cells``, ``efs_seal_boundary``,
``efs_query_box``), while parsing and per-node bookkeeping stay on the host, as in the reference.

- ``Scene3D.load(path)``: a 3D ``.json`` scene (Scene::loadScene, Scene.cpp:153-171; node types
  :197-225): the simulation domain, box and mesh fluid spawns, mesh boundaries (OBJ files), force fields,
  query nodes and deletion nodes, plus the saved properties.  ``Scene3D.init(sim)`` builds the grid as
  Editor::init does (Editor.cpp:21-38): initFluid, initBoundaries, force-field cells reset.
  ``Scene3D.update(sim, state)`` runs the per-frame node work of Scene::update (Scene.cpp:34-41) and
  Editor::updateForceFields (Editor.cpp:260-332).
- ``Scene2D.load(path)``: a ``.scene2D`` file of boundary and fluid cell index lists (Scene2D.cpp:41-65);
  ``Scene2D.reset(sim)`` writes them (Scene2D.cpp:67-77).
- ``QueryNode``: the metrics, its three experiment modes and the CSV export (QueryNode.cpp:31-178).

JSON is read with Python's json module (the reference uses nlohmann::json); OBJ files by ``load_obj``, which
reads vertex positions and faces as tinyobjloader does for the positions (faces of more than three vertices
split into a fan).
"""
import json
import math
import os

import numpy as np

from . import abi

# Properties (include/simulation/Properties.h, token names as saved in scenes) that the step reads.
_PARAM_FLOATS = {"DT": "dt", "Vel Decay": "vel_decay", "Lambda-": "lambda_minus", "Lambda+": "lambda_plus",
                 "Eta": "eta", "Liquid Threshold": "liquid_threshold", "D": "rho_d", "Threshold": "solver_threshold"}
_PARAM_INTS = {"Max Steps": "max_steps", "Gravity Enabled": "gravity_enabled", "Re-Calc Div": "re_calc_div"}
_DISABLE = {"Disable Velocity Decay": abi.STAGE_VEL_DECAY, "Disable Velocity Extrapolation": abi.STAGE_VEL_EXTRAPOLATE,
            "Disable Density Sharpen": abi.STAGE_RHO_SHARPEN, "Disable Density Advection": abi.STAGE_RHO_ADVECT,
            "Disable Velocity Advection": abi.STAGE_VEL_ADVECT, "Disable Add Force": abi.STAGE_ADD_FORCE,
            "Disable Projection": abi.STAGE_PROJECT}


def _f32(x):
    return float(np.float32(x))


def params_from_properties(props, base=None):
    """efs_params from a scene's saved properties.  GRAVITY_FORCE is GRAVITY / CELL_SIZE in float, as the
    application sets it every frame (Application.cpp:89)."""
    p = base.copy() if base is not None else abi.params_default()
    for k, f in _PARAM_FLOATS.items():
        if k in props:
            setattr(p, f, _f32(props[k]))
    for k, f in _PARAM_INTS.items():
        if k in props:
            setattr(p, f, int(props[k]))
    for k, bit in _DISABLE.items():
        if k in props:
            p.disable_mask = (p.disable_mask | (1 << bit)) if props[k] else (p.disable_mask & ~(1 << bit))
    if "Gravity" in props and "Cell Size" in props:
        p.gravity_force = float(np.float32(props["Gravity"]) / np.float32(props["Cell Size"]))
    elif "Gravity Force" in props:
        p.gravity_force = _f32(props["Gravity Force"])
    return p


# ---- geometry -----------------------------------------------------------------------------------------------

def quat_to_matrix(w, x, y, z):
    """Rotation matrix of a quaternion without normalising it (glm::mat3_cast; the zero quaternion that saved
    scenes hold gives the identity)."""
    f = np.float32
    w, x, y, z = f(w), f(x), f(y), f(z)
    xx, yy, zz, xz, xy, yz, wx, wy, wz = x * x, y * y, z * z, x * z, x * y, y * z, w * x, w * y, w * z
    one, two = f(1), f(2)
    return np.array([[one - two * (yy + zz), two * (xy - wz), two * (xz + wy)],
                     [two * (xy + wz), one - two * (xx + zz), two * (yz - wx)],
                     [two * (xz - wy), two * (yz + wx), one - two * (xx + yy)]], np.float32)


def trs_matrix(position, rotation_wxyz, scale):
    """T * R * S (Transform::updateTransform, Transform.cpp:67-73) as a 4x4 float32 matrix acting on columns."""
    m = np.eye(4, dtype=np.float32)
    r = quat_to_matrix(*rotation_wxyz)
    s = np.asarray(scale, np.float32)
    m[:3, :3] = r * s[None, :]
    m[:3, 3] = np.asarray(position, np.float32)
    return m


def transform_points(m, pts):
    """m * vec4(p, 1) for each point, summed column by column in float32 as glm multiplies a mat4 and a vec4."""
    p = np.asarray(pts, np.float32)
    out = m[:3, 0][None, :] * p[:, 0:1]
    out = out + m[:3, 1][None, :] * p[:, 1:2]
    out = out + m[:3, 2][None, :] * p[:, 2:3]
    out = out + m[:3, 3][None, :]
    return out.astype(np.float32)


def cube_triangles():
    """The unit cube [-0.5, 0.5]^3 as 12 outward-facing triangles (the box primitive of the reference's mesh
    library, Primitives.h BoxGeometry; any closed triangulation gives the same labels)."""
    c = np.array([[x, y, z] for z in (-0.5, 0.5) for y in (-0.5, 0.5) for x in (-0.5, 0.5)], np.float32)
    # vertex k = x + 2y + 4z bits; two triangles per face, counter-clockwise seen from outside
    faces = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    tris = []
    for a, b, cc, d in faces:
        tris.append((c[a], c[b], c[cc]))
        tris.append((c[a], c[cc], c[d]))
    return np.array(tris, np.float32)


def load_obj(path):
    """Triangles [n, 3, 3] of an OBJ file: 'v' positions and 'f' faces (1-based or negative indices,
    'v/vt/vn' forms), faces in file order, polygons split into a fan."""
    verts, tris = [], []
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if not parts:
                continue
            if parts[0] == "v":
                verts.append([float(parts[1]), float(parts[2]), float(parts[3])])
            elif parts[0] == "f":
                idx = []
                for tok in parts[1:]:
                    k = int(tok.split("/")[0])
                    idx.append(k - 1 if k > 0 else len(verts) + k)
                for j in range(1, len(idx) - 1):
                    tris.append((idx[0], idx[j], idx[j + 1]))
    v = np.asarray(verts, np.float32).reshape(-1, 3)
    return v[np.asarray(tris, np.int64)].reshape(-1, 3, 3) if tris else np.zeros((0, 3, 3), np.float32)


def _rotation(node):
    """A saved rotation [x, y, z, w] as (w, x, y, z) (ModelNode.cpp:29-30, ForceFieldNode.cpp:28-29)."""
    r = node.get("rotation", [0.0, 0.0, 0.0, 1.0])
    return (r[3], r[0], r[1], r[2])


# ---- scene nodes ----------------------------------------------------------------------------------------------

class QueryNode:
    """QueryNode (QueryNode.h, QueryNode.cpp): metrics of the cells in a box, kept per frame
    (SINGLE_SIMULATION) or averaged over `avg_frames` frames after `delay_frames` frames before the simulation
    is reset with gravity (CHANGE_GRAVITY) or the box position (CHANGE_Y_POS) changed by `change_value`, for
    `iterations` rounds."""
    SINGLE_SIMULATION, CHANGE_GRAVITY, CHANGE_Y_POS = 0, 1, 2
    COLUMNS = ["max_pos_x", "max_pos_y", "max_pos_z", "min_pos_x", "min_pos_y", "min_pos_z", "avg_pos_x",
               "avg_pos_y", "avg_pos_z", "vel_x", "vel_y", "vel_z", "pressure", "gravity"]

    def __init__(self, node=None):
        node = node or {}
        self.name = node.get("name", "QueryNode")
        self.position = [float(v) for v in node.get("position", [0.0, 0.0, 0.0])]
        self.scale = [float(v) for v in node.get("scale", [1.0, 1.0, 1.0])]
        self.enabled = bool(node.get("enabled", True))
        self.mode = int(node.get("mode", self.SINGLE_SIMULATION))
        self.avg_frames = int(node.get("avgFrames", 5))
        self.delay_frames = int(node.get("delayFrames", 20))
        self.change_value = _f32(node.get("changeValue", 0.05))
        self.iterations = int(node.get("iterations", 200))
        self.only_fluid = bool(node.get("onlyFluid", True))
        self.history = []
        self._avg_history = []

    def clamp(self, dims):
        """SimSpaceNode::update (SimSpaceNode.cpp:15-24): position rounded and clamped to [0, dim], scale
        rounded and clamped to [1, dim - position]."""
        for d in range(3):
            self.position[d] = min(max(float(np.round(np.float32(self.position[d]))), 0.0), float(dims[d]))
            self.scale[d] = min(max(float(np.round(np.float32(self.scale[d]))), 1.0), float(dims[d]) - self.position[d])

    def metrics(self, sim):
        m = sim.query_box([int(v) for v in self.position], [int(v) for v in self.scale], self.only_fluid)
        return list(m.max_position) + list(m.min_position) + list(m.avg_position) + list(m.velocity) + [m.pressure]

    def update(self, sim, state):
        """One frame (QueryNode::update, QueryNode.cpp:31-128).  `state` holds the application's properties
        that the node reads or sets: 'paused', 'frames' (SIMULATION_FRAMES), 'gravity'
        (GRAVITY_FORCE_PHYSICAL) and 'reset' (SIMULATION_RESET)."""
        self.clamp(sim.shape[::-1] if sim.dim == 3 else tuple(sim.shape[::-1]) + (1,))
        if not self.enabled or state.get("paused", False):
            return
        row = self.metrics(sim) + [float(state.get("gravity", 0.0))]
        if self.mode == self.SINGLE_SIMULATION:
            self.history.append(row)
            return
        frames = int(state.get("frames", 0))
        if frames < self.delay_frames:
            return
        if frames >= self.delay_frames + self.avg_frames:
            n = len(self._avg_history)
            mean = [float(np.float32(sum(np.float32(r[k]) for r in self._avg_history) / np.float32(n))) if n else 0.0
                    for k in range(len(row))]
            self.history.append(mean)
            self._avg_history = []
            state["reset"] = True
            if self.mode == self.CHANGE_GRAVITY:
                state["gravity"] = _f32(np.float32(state.get("gravity", 0.0)) + np.float32(self.change_value))
            elif self.mode == self.CHANGE_Y_POS:
                self.position[1] = _f32(np.float32(self.position[1]) + np.float32(self.change_value))
            self.iterations -= 1
        else:
            self._avg_history.append(row)
        if self.iterations == 0:
            state["paused"] = True

    def export_csv(self, path, dt, cell_size, dims, properties=None):
        """QueryNode::exportData (QueryNode.cpp:130-178): one row per history entry; the first row also carries
        dt, cell size, the grid size and the scene's properties (here: the saved ones, sorted by name)."""
        props = sorted((properties or {}).items())
        head = ["frame"] + self.COLUMNS + ["dt", "cell_size", "grid_width", "grid_height", "grid_depth"] + [k for k, _ in props]
        with open(path, "w") as fh:
            fh.write(",".join(head) + "\n")
            for i, row in enumerate(self.history):
                cells = [str(i)] + [repr(float(v)) for v in row]
                if i == 0:
                    cells += [repr(float(dt)), repr(float(cell_size))] + [str(int(d)) for d in dims]
                    cells += [str(v) for _, v in props]
                fh.write(",".join(cells) + "\n")


class Scene3D:
    """A 3D scene file and the grid it builds."""

    def __init__(self):
        self.properties = {}
        self.domain_center = [0.0, 0.0, 0.0]
        self.domain_size = [2.0, 2.0, 2.0]
        self.resolution = [10, 10, 10]
        self.percentage_filled = 0.0
        self.box_spawns = []            # (position, size) in cells
        self.mesh_spawns = []           # world triangles [n, 3, 3]
        self.boundaries = []            # world triangles of ModelNodes with boundary set
        self.force_fields = []          # dicts: triangles, direction, strength, active, cells, pending
        self.queries = []
        self.deletions = []             # (position, scale) in cells
        self.warnings = []

    @classmethod
    def load(cls, path, assets_root=None):
        """Parse a scene; OBJ paths are relative to `assets_root` (the reference's working directory;
        default: the directory that holds the scene's `assets` folder)."""
        with open(path) as fh:
            doc = json.load(fh)
        if assets_root is None:
            d = os.path.dirname(os.path.abspath(path))
            while d != os.path.dirname(d) and os.path.basename(d) != "assets":
                d = os.path.dirname(d)
            assets_root = os.path.dirname(d) if os.path.basename(d) == "assets" else os.path.dirname(os.path.abspath(path))
        s = cls()
        s.properties = doc.get("properties", {})
        for node in doc.get("nodes", []):
            s._add_node(node, assets_root)
        return s

    def _add_node(self, node, root):
        t = node["type"]
        if t == "SimulationDomainNode":
            self.domain_center = [float(v) for v in node.get("position", self.domain_center)]
            self.domain_size = [float(v) for v in node.get("scale", self.domain_size)]
            self.resolution = [int(v) for v in node.get("resolution", self.resolution)]
            self.percentage_filled = float(node.get("percentageFilled", 0.0))
        elif t == "BoundingBoxFluidSpawnNode":
            self.box_spawns.append(([float(v) for v in node.get("position", [0, 0, 0])],
                                    [float(v) for v in node.get("scale", [1, 1, 1])]))
        elif t in ("ModelNode", "ModelFluidSpawnNode"):
            tris = self._model(node.get("path", "assets/models/suzanne.obj"), root)
            m = trs_matrix(node.get("position", [0, 0, 0]), _rotation(node), node.get("scale", [1, 1, 1]))
            world = transform_points(m, tris.reshape(-1, 3)).reshape(-1, 3, 3)
            if t == "ModelFluidSpawnNode":
                self.mesh_spawns.append(world)
            elif node.get("boundary", False):
                self.boundaries.append(world)
        elif t == "ForceFieldNode":
            m = trs_matrix(node.get("position", [0, 0, 0]), _rotation(node), node.get("scale", [0.25, 0.25, 0.25]))
            world = transform_points(m, cube_triangles().reshape(-1, 3)).reshape(-1, 3, 3)
            axis = m[:3, 0].astype(np.float64)
            direction = (axis / np.linalg.norm(axis)).astype(np.float32)
            self.force_fields.append({"triangles": world, "direction": direction,
                                      "strength": _f32(node.get("strength", 1.0)), "active": bool(node.get("active", True)),
                                      "cells": np.zeros(0, np.int32), "pending": True})
        elif t == "QueryNode":
            self.queries.append(QueryNode(node))
        elif t == "DeletionNode":
            self.deletions.append(([float(v) for v in node.get("position", [0, 0, 0])],
                                   [float(v) for v in node.get("scale", [1, 1, 1])]))
        elif t in ("BoundingBoxNode", "CameraNode", "SkyboxNode", "FluidNode"):
            pass   # drawing only
        else:
            raise ValueError(f"Unknown node type: {t}")

    def _model(self, path, root):
        """The model's triangles; a file that cannot be found gives an empty model and a warning, as a failed
        tinyobj::LoadObj does (Model.cpp:74-85).  Paths are tried as given (relative to `root`), then as
        assets/models/<file name>."""
        for cand in (os.path.join(root, path), os.path.join(root, "assets", "models", os.path.basename(path))):
            if os.path.isfile(cand):
                return load_obj(cand)
        self.warnings.append(f"Failed to load model on path '{path}'")
        return np.zeros((0, 3, 3), np.float32)

    def params(self, base=None):
        return params_from_properties(self.properties, base)

    @property
    def shape(self):
        w, h, d = self.resolution
        return (d, h, w)

    def init(self, sim):
        """Editor::init (Editor.cpp:21-38) on a freshly reset simulator of this scene's resolution."""
        w, h, d = self.resolution
        if tuple(sim.shape) != (d, h, w):
            raise ValueError(f"simulator grid {sim.shape} is not the scene's {(d, h, w)}")
        sim.reset()
        full_lo, full_hi = (0, 0, 0), (w, h, d)
        # initFluid (Editor.cpp:84-168): cleared rho, mesh spawns (sdf.comp), initial fill, box spawns
        sim.fill_box(abi.FIELD_RHO, full_lo, full_hi, 0.0)
        if self.mesh_spawns:
            sim.mesh_label(abi.FIELD_RHO, np.concatenate(self.mesh_spawns), self.domain_center, self.domain_size, 1.0, 0.0)
        if self.percentage_filled != 0.0:
            fill_h = int(np.float32(self.percentage_filled) * np.float32(h))
            sim.fill_box(abi.FIELD_RHO, (1, 1, 1), (w - 1, min(h - 1, fill_h), d - 1), 1.0)
        for pos, size in self.box_spawns:
            lo = [int(np.float32(p)) for p in pos]
            hi = [int(np.float32(p) + np.float32(s)) for p, s in zip(pos, size)]
            sim.fill_box(abi.FIELD_RHO, lo, hi, 1.0)
        # initBoundaries (Editor.cpp:170-230): cleared boundary, mesh boundaries, solid border, no liquid in solids
        sim.fill_box(abi.FIELD_BOUNDARY, full_lo, full_hi, 0.0)
        if self.boundaries:
            sim.mesh_label(abi.FIELD_BOUNDARY, np.concatenate(self.boundaries), self.domain_center, self.domain_size, 1.0, 0.0)
        sim.seal_boundary()
        for ff in self.force_fields:
            ff["cells"] = np.zeros(0, np.int32)
            ff["pending"] = True

    def update_force_fields(self, sim, max_cells=None):
        """Editor::updateForceFields (Editor.cpp:260-332): the first pending field gets its cells; if that
        happened, the forces are cleared and every active field writes direction * strength at its cells."""
        if max_cells is None:
            max_cells = int(self.properties.get("Max ForceField cells", 1000))
        w, h, d = self.resolution
        clear = False
        for ff in self.force_fields:
            if not ff["pending"]:
                continue
            cells, n = sim.mesh_cells(ff["triangles"], self.domain_center, self.domain_size, capacity=max_cells)
            if n > max_cells:
                continue    # "ForceField exceeded maximum allowed cells!"
            if n > 0:
                ff["cells"] = cells.copy()
                ff["pending"] = False
            clear = True
            break
        if clear:
            sim.fill_box(abi.FIELD_FORCES, (0, 0, 0), (w, h, d), [0.0, 0.0, 0.0])
        for ff in self.force_fields:
            if ff["active"] and len(ff["cells"]):
                sim.set_cells(abi.FIELD_FORCES, ff["cells"], ff["direction"] * np.float32(ff["strength"]))

    def update(self, sim, state):
        """Per-frame node work (Scene::update, Scene.cpp:34-41): deletion boxes and queries, then the force
        fields.  `state` as for QueryNode.update."""
        w, h, d = self.resolution
        if not state.get("paused", False):
            for pos, scale in self.deletions:
                p = [min(max(float(np.round(np.float32(v))), 0.0), float(dim)) for v, dim in zip(pos, (w, h, d))]
                s = [min(max(float(np.round(np.float32(v))), 1.0), float(dim) - pp) for v, pp, dim in zip(scale, p, (w, h, d))]
                lo = [max(0, int(v)) for v in p]
                hi = [min(dim - 1, int(pp + ss)) for pp, ss, dim in zip(p, s, (w, h, d))]
                sim.fill_box(abi.FIELD_RHO, lo, hi, 0.0)
        for q in self.queries:
            q.update(sim, state)
        self.update_force_fields(sim)


class Scene2D:
    """A .scene2D file: grid size and the linear indices of boundary and fluid cells (Scene2D.cpp:41-65)."""

    def __init__(self, width, height, boundary, fluid, properties=None):
        self.width, self.height = int(width), int(height)
        self.boundary = np.asarray(boundary, np.int64)
        self.fluid = np.asarray(fluid, np.int64)
        self.properties = properties or {}

    @classmethod
    def load(cls, path):
        with open(path) as fh:
            doc = json.load(fh)
        return cls(doc.get("width", 0), doc.get("height", 0), doc.get("boundary", []), doc.get("fluid", []),
                   doc.get("properties", {}))

    @classmethod
    def from_image(cls, path, threshold, properties=None):
        """Scene2D::loadImage (Scene2D.cpp:87-121): the image, read as one 8-bit grey channel (image.read_grey8),
        becomes a grid of the image's width x height.  Pixel i = x + y W (row 0 the image's top row) is fluid
        when it is below `threshold` (threshold > 0), or when it is at least |threshold| (threshold <= 0); the
        outermost cells are boundary (fluid there stays fluid, as in the reference)."""
        from .image import read_grey8
        px = read_grey8(path)
        h, w = px.shape
        flat = px.reshape(-1).astype(np.int64)
        fluid = (flat < threshold) if threshold > 0 else ~(flat < abs(threshold))
        x = np.arange(w)[None, :]
        y = np.arange(h)[:, None]
        border = ((x == 0) | (x == w - 1) | (y == 0) | (y == h - 1)).reshape(-1)
        return cls(w, h, np.nonzero(border)[0], np.nonzero(fluid)[0], properties)

    def params(self, base=None):
        return params_from_properties(self.properties, base)

    def reset(self, sim):
        """Scene2D::resetScene (Scene2D.cpp:67-77): boundary and rho become the loaded cells (1) and 0
        elsewhere."""
        if tuple(sim.shape) != (self.height, self.width):
            return
        lo, hi = (0, 0, 0), (self.width, self.height, 1)
        sim.fill_box(abi.FIELD_BOUNDARY, lo, hi, 0.0)
        sim.set_cells(abi.FIELD_BOUNDARY, self.boundary, 1.0)
        sim.fill_box(abi.FIELD_RHO, lo, hi, 0.0)
        sim.set_cells(abi.FIELD_RHO, self.fluid, 1.0)

    def save(self, sim, path, properties=None):
        """Scene2D::saveScene (Scene2D.cpp:15-39): cells with boundary != 0 and rho >= 0.5."""
        b = sim.field(abi.FIELD_BOUNDARY).ravel()
        r = sim.field(abi.FIELD_RHO).ravel()
        doc = {"width": self.width, "height": self.height, "boundary": np.nonzero(b != 0.0)[0].tolist(),
               "fluid": np.nonzero(r >= 0.5)[0].tolist()}
        if properties is not None:
            doc["properties"] = properties
        with open(path, "w") as fh:
            json.dump(doc, fh)
