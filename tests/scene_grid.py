"""A CPU model of the simulator's scene calls (fill_box, set_cells, mesh_label, mesh_cells, seal_boundary,
query_box, field, reset) over numpy arrays, with the mesh label and query metrics from the oracle.  Tests run
the host scene logic on it, and compare the GPU field store against it after the same calls."""
import numpy as np

from eulerianfluidsimulation_gb300 import abi
from oracle import oracle


class OracleSceneGrid:
    def __init__(self, shape):
        self.shape = tuple(shape)
        self.dim = len(shape)
        self.fields = {}
        self.reset()

    def reset(self):
        """Grid3D / Grid2D constructor state: zero fields, gamma 1, solid border, rho 0 there."""
        s = self.shape
        self.fields = {f: np.zeros(s + ((self.dim,) if f in abi.VECTOR_FIELDS else ()), np.float32)
                       for f in range(abi.FIELD_COUNT)}
        self.fields[abi.FIELD_GAMMA][...] = 1.0
        b = self.fields[abi.FIELD_BOUNDARY]
        if self.dim == 3:
            b[0], b[-1], b[:, 0], b[:, -1], b[:, :, 0], b[:, :, -1] = 1, 1, 1, 1, 1, 1
        else:
            b[0], b[-1], b[:, 0], b[:, -1] = 1, 1, 1, 1

    def field(self, f):
        return self.fields[f].copy()

    def _view(self, f):
        a = self.fields[f]
        return a if self.dim == 3 else a[None]

    def _dims(self):
        return (self.shape[2], self.shape[1], self.shape[0]) if self.dim == 3 else (self.shape[1], self.shape[0], 1)

    def fill_box(self, f, lo, hi, value):
        W, H, D = self._dims()
        l = [max(0, int(v)) for v in lo]
        h = [min(d, int(v)) for v, d in zip(hi, (W, H, D))]
        if self.dim == 2:
            l[2], h[2] = 0, 1
        if min(b - a for a, b in zip(l, h)) <= 0:
            return
        v = np.asarray(value, np.float32)
        if f in abi.VECTOR_FIELDS:
            v = np.broadcast_to(v, (self.dim,))
        self._view(f)[l[2]:h[2], l[1]:h[1], l[0]:h[0]] = v

    def set_cells(self, f, cells, value):
        cells = np.asarray(cells, np.int64)
        n = int(np.prod(self.shape))
        if np.any((cells < 0) | (cells >= n)):
            raise IndexError("a cell index is outside the grid")
        a = self.fields[f]
        flat = a.reshape(n, -1) if f in abi.VECTOR_FIELDS else a.reshape(n)
        v = np.asarray(value, np.float32)
        flat[cells] = np.broadcast_to(v, (self.dim,)) if f in abi.VECTOR_FIELDS else v

    def mesh_label(self, f, triangles, center, size, value_inside=1.0, value_outside=0.0):
        self.fields[f] = oracle.mesh_label(self.shape, triangles, center, size, value_inside, value_outside,
                                           out=self.fields[f])

    def mesh_cells(self, triangles, center, size, capacity=None):
        lab = oracle.mesh_label(self.shape, triangles, center, size, 1.0, 0.0)
        cells = np.nonzero(lab.ravel() != 0.0)[0].astype(np.int32)
        cap = len(cells) if capacity is None else int(capacity)
        return cells[:cap], len(cells)

    def seal_boundary(self):
        b = self.fields[abi.FIELD_BOUNDARY]
        if self.dim == 3:
            b[0], b[-1], b[:, 0], b[:, -1], b[:, :, 0], b[:, :, -1] = 1, 1, 1, 1, 1, 1
        else:
            b[0], b[-1], b[:, 0], b[:, -1] = 1, 1, 1, 1
        self.fields[abi.FIELD_RHO][b != 0.0] = 0.0

    def query_box(self, position, scale, only_fluid=True):
        m, n = oracle.query_box(self.fields[abi.FIELD_RHO], self.fields[abi.FIELD_VEL],
                                self.fields[abi.FIELD_PRESSURE], position, scale, only_fluid)
        out = abi.EfsQueryMetrics()
        for k in ("max_position", "min_position", "avg_position", "velocity"):
            getattr(out, k)[:] = [float(x) for x in m[k]]
        out.pressure = m["pressure"]
        out.count = n
        return out
