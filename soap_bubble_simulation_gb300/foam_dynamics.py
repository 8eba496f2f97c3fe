"""Foam cluster dynamics on the GPU: the reference's FoamSimulator (foam_dynamics.rs:11-283) over a
BubbleCluster (foam.rs:219-424).

`FoamSimulator(position, radius)` holds the cluster on the GPU in the order of
BubbleCluster::bubbles() (ids 0..n-1, at rest, 500 nm films as Bubble::new makes them);
`step(dt)` is FoamSimulator::step (forces, semi-implicit Euler with damping and the 0.1 m/s
clamp, update_connections, coalescence when enabled) with the reference's f32 results;
`compute_forces`, `bubble_count`, `connection_count`, `connections` and `bubbles` read it back.
`couple_thickness` sets every bubble's film thickness from a batched drainage foam
(`FoamDrainage`), bubble i from batch bubble i.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

CONNECTION = np.dtype([("bubble_a", np.uint32), ("bubble_b", np.uint32), ("contact_point", np.float32, 3),
                       ("contact_normal", np.float32, 3), ("wall_curvature_radius", np.float32),
                       ("wall_thickness_nm", np.float32)])
assert CONNECTION.itemsize == 40


class FoamPhysics(C.Structure):
    """FoamSimulator's physics fields (foam_dynamics.rs:11-34), as sbs_foam_physics."""

    _fields_ = [("surface_tension", C.c_float), ("viscosity", C.c_float), ("density", C.c_float),
                ("gravity", C.c_float * 3), ("van_der_waals_strength", C.c_float),
                ("repulsion_stiffness", C.c_float), ("damping", C.c_float), ("coalescence_enabled", C.c_uint32),
                ("coalescence_threshold", C.c_float), ("padding", C.c_uint32)]

    @classmethod
    def default(cls) -> "FoamPhysics":
        """FoamSimulator::new's values (foam_dynamics.rs:38-53)."""
        p = cls()
        N.call("sbs_foam_physics_default", C.cast(C.byref(p), C.c_void_p))
        return p


assert C.sizeof(FoamPhysics) == 48


def default_cluster():
    """BubbleCluster::create_default_cluster (foam.rs:408-423): positions [5][3], radii [5]."""
    pos = np.array([[0.0, 0.0, 0.0], [0.042, 0.0, 0.0], [-0.038, 0.015, 0.0], [0.0, 0.040, 0.0],
                    [0.018, -0.038, 0.015]], dtype=np.float32)
    rad = np.array([0.025, 0.02, 0.022, 0.018, 0.02], dtype=np.float32)
    return pos, rad


class FoamSimulator:
    """FoamSimulator on the GPU (one CUDA stream per simulator)."""

    def __init__(self, position, radius, thickness_nm=None, physics: FoamPhysics | None = None):
        pos = np.ascontiguousarray(position, dtype=np.float32).reshape(-1, 3)
        n = pos.shape[0]
        rad = np.ascontiguousarray(radius, dtype=np.float32).reshape(n)
        th = None if thickness_nm is None else np.ascontiguousarray(thickness_nm, dtype=np.float32).reshape(n)
        self.physics = FoamPhysics.default() if physics is None else physics
        self._h = C.c_void_p()
        N.call("sbs_foam_sim_create", n, N.ptr(pos), N.ptr(rad), N.ptr(th), C.cast(C.byref(self.physics), C.c_void_p),
               C.byref(self._h))

    @classmethod
    def with_default_cluster(cls) -> "FoamSimulator":
        return cls(*default_cluster())

    def close(self):
        if self._h:
            N.lib().sbs_foam_sim_destroy(self._h)
            self._h = C.c_void_p()

    def reset(self) -> None:
        """FoamSimulator::reset (foam_dynamics.rs:274-276): the default cluster again, physics kept."""
        self.close()
        pos, rad = default_cluster()
        self._h = C.c_void_p()
        N.call("sbs_foam_sim_create", pos.shape[0], N.ptr(pos), N.ptr(rad), None,
               C.cast(C.byref(self.physics), C.c_void_p), C.byref(self._h))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_physics(self, physics: FoamPhysics | None = None, **fields) -> None:
        """Replaces the physics (or changes the named fields, e.g. coalescence_enabled=1); on an
        error (a non-finite value) the simulator keeps its physics."""
        p = FoamPhysics.from_buffer_copy(self.physics if physics is None else physics)
        for k, v in fields.items():
            if k == "gravity":
                p.gravity[:] = [float(x) for x in v]
            else:
                setattr(p, k, v)
        N.call("sbs_foam_sim_set_physics", self._h, C.cast(C.byref(p), C.c_void_p))
        self.physics = p

    def step(self, dt: float, steps: int = 1) -> None:
        """`steps` FoamSimulator::step(dt) calls."""
        N.call("sbs_foam_sim_step", self._h, float(dt), int(steps))

    def bubble_count(self) -> int:
        b = C.c_uint32()
        N.call("sbs_foam_sim_counts", self._h, C.byref(b), None)
        return b.value

    def connection_count(self) -> int:
        c = C.c_uint32()
        N.call("sbs_foam_sim_counts", self._h, None, C.byref(c))
        return c.value

    def bubbles(self) -> dict:
        """The cluster in its order: position, velocity [n][3], radius, thickness_nm [n], ids [n]."""
        n = self.bubble_count()
        out = dict(position=np.empty((n, 3), np.float32), velocity=np.empty((n, 3), np.float32),
                   radius=np.empty(n, np.float32), thickness_nm=np.empty(n, np.float32), ids=np.empty(n, np.uint32))
        N.call("sbs_foam_sim_get_state", self._h, N.ptr(out["position"]), N.ptr(out["velocity"]), N.ptr(out["radius"]),
               N.ptr(out["thickness_nm"]), N.ptr(out["ids"]), N.MEM_HOST)
        return out

    def set_state(self, position=None, velocity=None, radius=None, thickness_nm=None) -> None:
        n = self.bubble_count()

        def arr(a, shape):
            return None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(shape)

        p, v, r, t = arr(position, (n, 3)), arr(velocity, (n, 3)), arr(radius, (n,)), arr(thickness_nm, (n,))
        N.call("sbs_foam_sim_set_state", self._h, N.ptr(p), N.ptr(v), N.ptr(r), N.ptr(t), N.MEM_HOST)

    def compute_forces(self) -> np.ndarray:
        """compute_forces (foam_dynamics.rs:62-94) on the current state: [n][3]."""
        f = np.empty((self.bubble_count(), 3), np.float32)
        N.call("sbs_foam_sim_forces", self._h, N.ptr(f), N.MEM_HOST)
        return f

    def connections(self) -> np.ndarray:
        """BubbleCluster::connections() (foam.rs:304-307) as a structured array (CONNECTION)."""
        count = C.c_uint32()
        N.call("sbs_foam_sim_connections", self._h, None, 0, C.byref(count))
        out = np.zeros(count.value, dtype=CONNECTION)
        if count.value:
            N.call("sbs_foam_sim_connections", self._h, C.c_void_p(out.ctypes.data), count.value, C.byref(count))
        return out

    def query_nearby(self, position, radius: float) -> list:
        """BubbleCluster::query_nearby (foam.rs:314-317) over the cluster's 10 cm spatial hash as
        update_connections last rebuilt it (the current bubbles in cluster order)."""
        b = self.bubbles()
        h = SpatialHash(0.1)
        h.rebuild(b["ids"], b["position"])
        return h.query(position, radius)

    def couple_thickness(self, batch) -> None:
        """thickness_nm[i] = the sin(theta)-weighted mean of batch bubble i's thickness field, in nm."""
        N.call("sbs_foam_sim_couple_thickness", self._h, batch._h)

    @property
    def handle(self) -> C.c_void_p:
        return self._h


class SpatialHash:
    """SpatialHash (foam.rs:149-216): bubble ids binned by floor(position / cell_size) in f32;
    query returns the ids of the cells within ceil(radius / cell_size) cells of the position's,
    offsets walked x, then y, then z, each cell in insertion order. A host-side helper: the
    GPU's own spatial hash lives inside the neighbour-list build."""

    def __init__(self, cell_size: float):
        self.cell_size = np.float32(cell_size)
        self.cells: dict[tuple, list] = {}

    def cell_coords(self, position) -> tuple:
        p = np.asarray(position, dtype=np.float32).reshape(3)
        return tuple(int(np.floor(p[k] / self.cell_size)) for k in range(3))

    def clear(self) -> None:
        self.cells.clear()

    def insert(self, bubble_id: int, position) -> None:
        self.cells.setdefault(self.cell_coords(position), []).append(int(bubble_id))

    def query(self, position, radius: float) -> list:
        r = int(np.ceil(np.float32(radius) / self.cell_size))
        cx, cy, cz = self.cell_coords(position)
        out = []
        for dx in range(-r, r + 1):
            for dy in range(-r, r + 1):
                for dz in range(-r, r + 1):
                    out.extend(self.cells.get((cx + dx, cy + dy, cz + dz), ()))
        return out

    def rebuild(self, ids, positions) -> None:
        self.clear()
        for i, p in zip(ids, np.asarray(positions, dtype=np.float32).reshape(-1, 3)):
            self.insert(i, p)


def fcc_foam(count: int, spacing: float = 0.05, jitter: float = 0.1, min_radius: float = 0.015,
             max_radius: float = 0.030, seed: int = 0):
    """A face-centred cubic cluster in FoamGenerator::generate_fcc's layout and loop order
    (foam_generation.rs:307-343: 4 bubbles per cell, cells centred on the origin, jitter of
    jitter * spacing) with uniform radii (sample_uniform, foam_generation.rs:485-487); the random
    numbers come from a seeded numpy generator. Returns positions [count][3], radii [count]."""
    g = np.random.default_rng(seed)
    n = max(int(np.ceil(np.cbrt(count / 4.0))), 2)
    offset = (n - 1) * spacing / 2.0
    half = spacing / 2.0
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = np.stack([i, j, k], axis=-1).reshape(-1, 1, 3) * spacing - offset
    basis = np.array([[0, 0, 0], [half, half, 0], [half, 0, half], [0, half, half]])
    pos = (base + basis[None]).reshape(-1, 3)[:count]
    pos = pos + (g.random((count, 3)) - 0.5) * jitter * spacing
    rad = min_radius + g.random(count) * (max_radius - min_radius)
    return pos.astype(np.float32), rad.astype(np.float32)
