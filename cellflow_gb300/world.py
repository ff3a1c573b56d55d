"""Python mirror of the reference's ``ParticleSimulation`` over the C ABI.

Method names follow cuda-native/include/ParticleSimulation.cuh:10-103 so
tests and tools read like code written against the reference class; every
call goes through libcellflow.so.  Arrays are numpy; a failing call raises
``CellFlowError`` (the reference printed and exited instead).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, fields

import numpy as np

from . import _lib
from ._lib import Color, DeviceView, GridInfo, Particle, Preset, StepParams, check, load

PARTICLE_DTYPE = np.dtype(
    [("pos", "<f4", 3), ("vel", "<f4", 3), ("acc", "<f4", 3), ("ptype", "<u4"), ("pad", "<f4")]
)
assert PARTICLE_DTYPE.itemsize == 44


@dataclass
class SimulationParams:
    """Physics subset of the reference SimulationParams (SimulationParams.h:15-29)."""

    radius: float = 42.07
    delta_t: float = 0.18
    friction: float = 0.51
    repulsion: float = 64.83
    attraction: float = 3.06
    k: float = 29.45
    balance: float = 0.79
    canvas_width: float = 8000.0
    canvas_height: float = 8000.0
    canvas_depth: float = 8000.0
    num_particle_types: int = 6
    ratio_with_lfo: float = 0.0
    force_multiplier: float = 2.33
    max_expected_neighbors: int = 400

    def to_c(self) -> StepParams:
        p = StepParams()
        for f in fields(self):
            setattr(p, f.name, getattr(self, f.name))
        return p


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class ParticleSimulation:
    """One world: n particles of T types in a W x H x D periodic box."""

    def __init__(self, n: int, num_types: int = 6, width: float = 8000.0, height: float = 8000.0,
                 depth: float | None = None, seed: int = 1):
        lib = load()
        self._lib = lib
        self._h = C.c_void_p()
        depth = height if depth is None else depth  # ParticleSimulation.cu:439 uses height for depth
        check(lib.cf_create(n, num_types, width, height, depth, seed, C.byref(self._h)), "cf_create")

    # ---- lifetime -----------------------------------------------------------
    def close(self) -> None:
        if self._h:
            self._lib.cf_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def getParticleCount(self) -> int:
        n = C.c_int()
        check(self._lib.cf_particle_count(self._h, C.byref(n)), "cf_particle_count")
        return n.value

    def getNumParticleTypes(self) -> int:
        t = C.c_int()
        check(self._lib.cf_num_particle_types(self._h, C.byref(t)), "cf_num_particle_types")
        return t.value

    def setParticleCount(self, n: int, seed: int = 1) -> None:
        check(self._lib.cf_set_particle_count(self._h, n, seed), "cf_set_particle_count")

    def setNumParticleTypes(self, t: int, seed: int = 1) -> None:
        check(self._lib.cf_set_num_particle_types(self._h, t, seed), "cf_set_num_particle_types")

    def initializeParticles(self, seed: int = 1, spawn_region: float = 2000.0) -> None:
        check(self._lib.cf_initialize_particles(self._h, seed, spawn_region), "cf_initialize_particles")

    def updateCanvasDimensions(self, width: float, height: float, depth: float | None = None) -> None:
        """The box that initializeParticles spawns in and moveUniverse wraps into (depth defaults
        to height, ParticleSimulation.cu:497-503)."""
        depth = height if depth is None else depth
        check(self._lib.cf_set_canvas(self._h, width, height, depth), "cf_set_canvas")

    def moveUniverse(self, dx: float, dy: float, dz: float = 0.0) -> None:
        """Translate every particle and wrap into the box (ParticleSimulation.cu:585-592)."""
        check(self._lib.cf_move_universe(self._h, dx, dy, dz), "cf_move_universe")

    def set_stream(self, stream_ptr: int | None) -> None:
        check(self._lib.cf_set_stream(self._h, C.c_void_p(stream_ptr or 0)), "cf_set_stream")

    def sync(self) -> None:
        check(self._lib.cf_sync(self._h), "cf_sync")

    # ---- state ----------------------------------------------------------------
    def getParticleData(self) -> np.ndarray:
        """AoS records in the reference layout (ParticleSimulation.cu:558-562)."""
        n = self.getParticleCount()
        out = np.zeros(n, dtype=PARTICLE_DTYPE)
        check(self._lib.cf_get_particles(self._h, _ptr(out), n), "cf_get_particles")
        return out

    def step_host(self, params: SimulationParams, records_in, records_out=None) -> np.ndarray:
        """One step with host buffers (cf_step_host): upload `records_in` (AoS, the reference
        layout), step, read back into `records_out` (default: a new array).  Page-locked
        buffers (e.g. numpy views of pinned torch tensors) run as one CUDA graph."""
        rin = np.ascontiguousarray(records_in, dtype=PARTICLE_DTYPE)
        out = np.zeros(len(rin), dtype=PARTICLE_DTYPE) if records_out is None else records_out
        p = params.to_c()
        check(self._lib.cf_step_host(self._h, C.byref(p), _ptr(rin), _ptr(out), len(rin)), "cf_step_host")
        return out

    def setParticleData(self, records: np.ndarray) -> None:
        rec = np.ascontiguousarray(records, dtype=PARTICLE_DTYPE)
        check(self._lib.cf_set_particles(self._h, _ptr(rec), len(rec)), "cf_set_particles")

    def set_particles(self, pos: np.ndarray, types: np.ndarray, vel: np.ndarray | None = None) -> None:
        """Set positions (n, 3), types (n,) and optional velocities; counts reset to 0."""
        n = self.getParticleCount()
        pos4 = np.zeros((n, 4), dtype=np.float32)
        pos4[:, :3] = pos
        pos4[:, 3] = np.asarray(types, dtype=np.uint32).view(np.float32)
        vel4 = np.zeros((n, 4), dtype=np.float32)
        if vel is not None:
            vel4[:, :3] = vel
        counts = np.zeros(n, dtype=np.int32)
        check(self._lib.cf_set_state(self._h, _ptr(pos4), _ptr(vel4), _ptr(counts)), "cf_set_state")

    def get_state(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = self.getParticleCount()
        pos4 = np.zeros((n, 4), dtype=np.float32)
        vel4 = np.zeros((n, 4), dtype=np.float32)
        counts = np.zeros(n, dtype=np.int32)
        check(self._lib.cf_get_state(self._h, _ptr(pos4), _ptr(vel4), _ptr(counts)), "cf_get_state")
        return pos4, vel4, counts

    def set_state(self, pos4: np.ndarray, vel4: np.ndarray, counts: np.ndarray) -> None:
        pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
        vel4 = np.ascontiguousarray(vel4, dtype=np.float32)
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        check(self._lib.cf_set_state(self._h, _ptr(pos4), _ptr(vel4), _ptr(counts)), "cf_set_state")

    def getNeighborCounts(self) -> np.ndarray:
        n = self.getParticleCount()
        out = np.zeros(n, dtype=np.int32)
        check(self._lib.cf_get_neighbor_counts(self._h, _ptr(out), n), "cf_get_neighbor_counts")
        return out

    def device_buffers(self) -> DeviceView:
        v = DeviceView()
        check(self._lib.cf_device_buffers(self._h, C.byref(v)), "cf_device_buffers")
        return v

    # ---- parameter surface ------------------------------------------------------
    def getRawForceTableValues(self) -> np.ndarray:
        t = self.getNumParticleTypes()
        out = np.zeros(t * t, dtype=np.float32)
        check(self._lib.cf_get_raw_force_table(self._h, _ptr(out), t * t), "cf_get_raw_force_table")
        return out

    def setRawForceTableValues(self, raw) -> None:
        raw = np.ascontiguousarray(raw, dtype=np.float32).ravel()
        check(self._lib.cf_set_raw_force_table(self._h, _ptr(raw), raw.size), "cf_set_raw_force_table")

    def regenerateForceTable(self, seed: int = 1) -> None:
        check(self._lib.cf_regenerate_force_table(self._h, seed), "cf_regenerate_force_table")

    def updateForceTable(self, force_range: float, force_bias: float, force_offset: float) -> None:
        check(self._lib.cf_update_force_table(self._h, force_range, force_bias, force_offset),
              "cf_update_force_table")

    def setForceTable(self, table) -> None:
        table = np.ascontiguousarray(table, dtype=np.float32).ravel()
        check(self._lib.cf_set_force_table(self._h, _ptr(table), table.size), "cf_set_force_table")

    def getForceTable(self) -> np.ndarray:
        t = self.getNumParticleTypes()
        out = np.zeros(t * t, dtype=np.float32)
        check(self._lib.cf_get_force_table(self._h, _ptr(out), t * t), "cf_get_force_table")
        return out

    def getRadioByType(self) -> np.ndarray:
        t = self.getNumParticleTypes()
        out = np.zeros(t, dtype=np.float32)
        check(self._lib.cf_get_radio_by_type(self._h, _ptr(out), t), "cf_get_radio_by_type")
        return out

    def setRadioByType(self, values) -> None:
        values = np.ascontiguousarray(values, dtype=np.float32).ravel()
        check(self._lib.cf_set_radio_by_type(self._h, _ptr(values), values.size), "cf_set_radio_by_type")

    def setRadioByTypeValue(self, index: int, value: float) -> None:
        check(self._lib.cf_set_radio_by_type_value(self._h, index, value), "cf_set_radio_by_type_value")

    def rotateRadioByType(self) -> None:
        check(self._lib.cf_rotate_radio_by_type(self._h), "cf_rotate_radio_by_type")

    # ---- step ---------------------------------------------------------------------
    def simulate(self, params: SimulationParams, steps: int = 1) -> None:
        """ParticleSimulation::simulate (ParticleSimulation.cu:541-556), `steps` times; asynchronous."""
        p = params.to_c()
        check(self._lib.cf_step(self._h, C.byref(p), steps), "cf_step")

    def autotune(self, params: SimulationParams, steps: int = 3) -> int:
        """Pick the force-kernel variant by timing trial steps; the state is restored."""
        p = params.to_c()
        chosen = C.c_int()
        check(self._lib.cf_autotune_step(self._h, C.byref(p), steps, C.byref(chosen)), "cf_autotune_step")
        return chosen.value

    def set_force_variant(self, variant: int) -> None:
        check(self._lib.cf_set_force_variant(self._h, variant), "cf_set_force_variant")

    def grid(self, params: SimulationParams) -> GridInfo:
        g = GridInfo()
        p = params.to_c()
        check(self._lib.cf_get_grid(self._h, C.byref(p), C.byref(g)), "cf_get_grid")
        return g

    def cell_list(self, params: SimulationParams):
        g = self.grid(params)
        cells = g.cells[0] * g.cells[1] * g.cells[2]
        n = self.getParticleCount()
        cell_of = np.zeros(n, dtype=np.uint32)
        order = np.zeros(n, dtype=np.uint32)
        start = np.zeros(cells, dtype=np.uint32)
        end = np.zeros(cells, dtype=np.uint32)
        p = params.to_c()
        check(self._lib.cf_debug_cell_list(self._h, C.byref(p), _ptr(cell_of), _ptr(order), _ptr(start),
                                           _ptr(end), cells), "cf_debug_cell_list")
        return g, cell_of, order, start, end

    def force_work(self, params: SimulationParams) -> tuple[int, int]:
        """(candidates staged, candidate tests) of the force kernel's filter for the current state."""
        p = params.to_c()
        staged, tested = C.c_uint64(), C.c_uint64()
        check(self._lib.cf_force_work(self._h, C.byref(p), C.byref(staged), C.byref(tested)), "cf_force_work")
        return staged.value, tested.value

    def work_counters(self, params: SimulationParams) -> tuple[int, int]:
        c27 = C.c_uint64()
        inter = C.c_uint64()
        p = params.to_c()
        check(self._lib.cf_work_counters(self._h, C.byref(p), C.byref(c27), C.byref(inter)), "cf_work_counters")
        return c27.value, inter.value

    # ---- triangle mesh -----------------------------------------------------------------
    def triangle_mesh(self, distance: float, max_conn: int) -> np.ndarray:
        """Triangles of generateTriangleMesh (ParticleSimulation.cu:689-747) as index triples, shape (K, 3)."""
        count = C.c_int()
        check(self._lib.cf_triangle_mesh(self._h, distance, max_conn, None, 0, C.byref(count)), "cf_triangle_mesh")
        tris = np.zeros((max(count.value, 1), 3), dtype=np.int32)
        check(self._lib.cf_triangle_mesh(self._h, distance, max_conn, _ptr(tris), count.value, C.byref(count)),
              "cf_triangle_mesh")
        return tris[: count.value].copy()

    def _color_array(self, colors):
        """The colours as a ctypes array, rebuilt only when they change between calls."""
        key = [tuple(c) for c in colors]
        if getattr(self, "_colors_key", None) != key:
            self._colors_key = key
            self._colors_arr = (Color * len(key))(*[Color(*c) for c in key])
        return self._colors_arr

    def triangle_mesh_device(self, distance: float, max_conn: int, colors, vertices_ptr: int,
                             cap_vertices: int) -> int:
        """The reference's 9-float triangle vertices into a device buffer; returns the vertex count."""
        cols = self._color_array(colors)
        count = C.c_int()
        check(self._lib.cf_triangle_mesh_device(self._h, distance, max_conn, cols, len(colors),
                                                C.c_void_p(vertices_ptr), cap_vertices, C.byref(count)),
              "cf_triangle_mesh_device")
        return count.value

    # ---- presets ---------------------------------------------------------------------
    def loadPreset(self, source, seed: int = 1, params: SimulationParams | None = None):
        """CellFlowWidget::loadPreset (CellFlowWidget.cpp:1070-1180) on this world.  source is a path or
        the JSON text.  Returns (SimulationParams with the preset's values, the parsed Preset)."""
        from pathlib import Path

        text = str(source).encode() if str(source).lstrip().startswith("{") else Path(source).read_bytes()
        pre = parse_preset(text)
        p = (params or SimulationParams()).to_c()
        check(self._lib.cf_preset_apply(self._h, C.byref(pre), seed, C.byref(p)), "cf_preset_apply")
        return params_from_c(p), pre

    def savePreset(self, params: SimulationParams, preset: Preset | None = None, path=None) -> str:
        """CellFlowWidget::savePreset (CellFlowWidget.cpp:1182-1259): the JSON text (written to path if
        given); step parameters from params, transform / LFO / colours / other keys from preset."""
        pre = Preset() if preset is None else preset
        if preset is None:
            pre.force_range, pre.force_bias, pre.force_offset, pre.lfo_s = 0.28, -0.20, 1.0, 0.1
        pre.params = params.to_c()
        n = C.c_size_t()
        check(self._lib.cf_preset_write(self._h, C.byref(pre), None, 0, C.byref(n)), "cf_preset_write")
        buf = C.create_string_buffer(n.value + 1)
        check(self._lib.cf_preset_write(self._h, C.byref(pre), buf, n.value + 1, C.byref(n)), "cf_preset_write")
        text = buf.value.decode()
        if path is not None:
            from pathlib import Path

            Path(path).write_text(text)
        return text

    # ---- differentiable rollout (device pointers, n float4 each) -------------------
    def rollout_forward(self, params: SimulationParams, steps: int, checkpoint_every: int = 16,
                        pos4_in: int | None = None, vel4_in: int | None = None, pos4_out: int | None = None,
                        vel4_out: int | None = None) -> None:
        """cf_rollout_forward: `steps` steps keeping checkpoints for cf_rollout_backward."""
        p = params.to_c()
        vp = lambda x: C.c_void_p(x) if x else None  # noqa: E731
        check(self._lib.cf_rollout_forward(self._h, C.byref(p), vp(pos4_in), vp(vel4_in), steps, checkpoint_every,
                                           vp(pos4_out), vp(vel4_out)), "cf_rollout_forward")

    def rollout_backward(self, gpos4: int | None, gvel4: int | None, gpos4_out: int | None,
                         gvel4_out: int | None) -> tuple[np.ndarray, np.ndarray]:
        """cf_rollout_backward: fills the device outputs; returns (dL/dF (T, T), dL/dparams in GRAD_PARAMS order)."""
        T = self.getNumParticleTypes()
        gF = np.zeros(T * T, dtype=np.float32)
        gp = np.zeros(len(_lib.GRAD_PARAMS), dtype=np.float32)
        vp = lambda x: C.c_void_p(x) if x else None  # noqa: E731
        check(self._lib.cf_rollout_backward(self._h, vp(gpos4), vp(gvel4), vp(gpos4_out), vp(gvel4_out), _ptr(gF),
                                            T * T, _ptr(gp)), "cf_rollout_backward")
        return gF.reshape(T, T), gp

    def rdf(self, bins: int, r_max: float, hist: int, pos4: int | None = None) -> None:
        """cf_rdf into the device buffer `hist` (T * T * bins floats)."""
        check(self._lib.cf_rdf(self._h, C.c_void_p(pos4) if pos4 else None, bins, r_max, C.c_void_p(hist)),
              "cf_rdf")

    def rdf_backward(self, bins: int, r_max: float, ghist: int, gpos4: int, pos4: int | None = None) -> None:
        check(self._lib.cf_rdf_backward(self._h, C.c_void_p(pos4) if pos4 else None, bins, r_max,
                                        C.c_void_p(ghist), C.c_void_p(gpos4)), "cf_rdf_backward")

    # ---- proximity graph -----------------------------------------------------------
    def proximity_edges(self, distance: float, max_conn: int, cap: int | None = None) -> np.ndarray:
        """Edges (i, j) of generateProximityGraph (ParticleSimulation.cu:625-687), shape (E, 2)."""
        if cap is None:
            cap = self.getParticleCount() * max(max_conn, 0)
        edges = np.zeros((max(cap, 1), 2), dtype=np.int32)
        count = C.c_int()
        check(self._lib.cf_proximity_edges(self._h, distance, max_conn, _ptr(edges), cap, C.byref(count)),
              "cf_proximity_edges")
        return edges[: count.value].copy()

    def proximity_vertices_device(self, distance: float, max_conn: int, colors, vertices_ptr: int,
                                  cap_vertices: int) -> int:
        cols = self._color_array(colors)
        count = C.c_int()
        check(self._lib.cf_proximity_vertices_device(self._h, distance, max_conn, cols, len(colors),
                                                     C.c_void_p(vertices_ptr), cap_vertices, C.byref(count)),
              "cf_proximity_vertices_device")
        return count.value


class Batch:
    """Many independent worlds stepped together (cf_batch_*): world k owns particles
    offsets[k]:offsets[k+1] of the concatenated state and has its own force table."""

    def __init__(self, n_per_world, num_types: int, width: float = 2.0, height: float = 2.0, depth: float = 2.0,
                 seed: int = 1):
        lib = load()
        self._lib = lib
        self._h = C.c_void_p()
        counts = np.ascontiguousarray(n_per_world, dtype=np.int32)
        check(lib.cf_batch_create(len(counts), _ptr(counts), num_types, width, height, depth, seed,
                                  C.byref(self._h)), "cf_batch_create")
        worlds, total = C.c_int(), C.c_int()
        check(lib.cf_batch_info(self._h, C.byref(worlds), C.byref(total), None), "cf_batch_info")
        self.offsets = np.zeros(worlds.value + 1, dtype=np.int32)
        check(lib.cf_batch_info(self._h, None, None, _ptr(self.offsets)), "cf_batch_info")
        self.n = total.value
        self.num_types = num_types

    def close(self) -> None:
        if self._h:
            self._lib.cf_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def world_handle(self) -> C.c_void_p:
        out = C.c_void_p()
        check(self._lib.cf_batch_world(self._h, C.byref(out)), "cf_batch_world")
        return out

    def set_particles(self, pos: np.ndarray, types: np.ndarray, vel: np.ndarray | None = None) -> None:
        pos4 = np.zeros((self.n, 4), dtype=np.float32)
        pos4[:, :3] = pos
        pos4[:, 3] = np.asarray(types, dtype=np.uint32).view(np.float32)
        vel4 = np.zeros((self.n, 4), dtype=np.float32)
        if vel is not None:
            vel4[:, :3] = vel
        counts = np.zeros(self.n, dtype=np.int32)
        check(self._lib.cf_batch_set_state(self._h, _ptr(pos4), _ptr(vel4), _ptr(counts)), "cf_batch_set_state")

    def get_state(self):
        pos4 = np.zeros((self.n, 4), dtype=np.float32)
        vel4 = np.zeros((self.n, 4), dtype=np.float32)
        counts = np.zeros(self.n, dtype=np.int32)
        check(self._lib.cf_batch_get_state(self._h, _ptr(pos4), _ptr(vel4), _ptr(counts)), "cf_batch_get_state")
        return pos4, vel4, counts

    def set_force_tables(self, tables) -> None:
        t = np.ascontiguousarray(tables, dtype=np.float32).ravel()
        check(self._lib.cf_batch_set_force_tables(self._h, _ptr(t), t.size), "cf_batch_set_force_tables")

    def simulate(self, params: SimulationParams, steps: int = 1) -> None:
        p = params.to_c()
        check(self._lib.cf_batch_step(self._h, C.byref(p), steps), "cf_batch_step")

    def capture(self, params: SimulationParams, steps: int) -> None:
        p = params.to_c()
        check(self._lib.cf_batch_capture(self._h, C.byref(p), steps), "cf_batch_capture")

    def replay(self) -> None:
        check(self._lib.cf_batch_replay(self._h), "cf_batch_replay")

    def graph_info(self) -> tuple[int, int]:
        """(steps, kernel nodes) of the captured graph."""
        steps, kernels = C.c_int(), C.c_longlong()
        check(self._lib.cf_batch_graph_info(self._h, C.byref(steps), C.byref(kernels)), "cf_batch_graph_info")
        return steps.value, kernels.value

    def autotune(self, params: SimulationParams, steps: int = 2) -> int:
        p = params.to_c()
        chosen = C.c_int()
        check(self._lib.cf_batch_autotune(self._h, C.byref(p), steps, C.byref(chosen)), "cf_batch_autotune")
        return chosen.value

    def set_stream(self, stream_ptr: int | None) -> None:
        check(self._lib.cf_batch_set_stream(self._h, C.c_void_p(stream_ptr or 0)), "cf_batch_set_stream")

    def sync(self) -> None:
        check(self._lib.cf_batch_sync(self._h), "cf_batch_sync")


def parse_preset(text: str | bytes) -> Preset:
    """cf_preset_parse: a preset file's JSON text (CellFlowWidget.cpp:1070-1180 keys)."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    out = Preset()
    check(load().cf_preset_parse(data, len(data), C.byref(out)), "cf_preset_parse")
    return out


def params_from_c(p: StepParams) -> SimulationParams:
    return SimulationParams(**{f.name: getattr(p, f.name) for f in fields(SimulationParams)})


def lfo_ratio(ratio: float, lfo_a: float, lfo_s: float, t: float) -> float:
    """Caller LFO of CellFlowWidget::paintGL (CellFlowWidget.cpp:414-421)."""
    return load().cf_lfo_ratio(ratio, lfo_a, lfo_s, t)


def version() -> str:
    return load().cf_version().decode()


__all__ = ["ParticleSimulation", "SimulationParams", "PARTICLE_DTYPE", "lfo_ratio", "version", "_lib"]
