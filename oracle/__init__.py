"""The oracle: CPU restatement of the CellFlow step and the reference's own
kernel bodies run on the host.

TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py use this package, as the checker or as the timed
CPU baseline; the product path (cellflow_gb300) never imports it.

Two libraries:
  _build/libcf_oracle.so  cf_oracle.c, the restatement (always built)
  _ref/libcfref.so        the reference's own kernel bodies through
                          ref_host_shim.cu (built by build_ref.sh when the
                          reference pieces are present)
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
ORACLE_LIB = BUILD / "libcf_oracle.so"
REF_DIR = HERE / "_ref"
REF_LIB = REF_DIR / "libcfref.so"
REF_GPU_LIB = REF_DIR / "libcfref_gpu.so"


class OracleParams(C.Structure):
    _fields_ = [
        ("radius", C.c_float), ("delta_t", C.c_float), ("friction", C.c_float), ("repulsion", C.c_float),
        ("attraction", C.c_float), ("k", C.c_float), ("balance", C.c_float),
        ("w", C.c_float), ("h", C.c_float), ("d", C.c_float),
        ("num_types", C.c_int), ("ratio_with_lfo", C.c_float), ("force_multiplier", C.c_float),
        ("max_expected_neighbors", C.c_int),
    ]


class Phys64(C.Structure):
    """cfo_phys64 of cf_adjoint_oracle.c."""

    _fields_ = [
        ("repulsion", C.c_double), ("attraction", C.c_double), ("k", C.c_double),
        ("force_multiplier", C.c_double), ("balance", C.c_double), ("friction", C.c_double),
        ("delta_t", C.c_double), ("max_expected_neighbors", C.c_int),
    ]


# Order of the parameter gradients (cf_adjoint_oracle.c G_* and CF_GRAD_* of the library).
GRAD_PARAMS = ("repulsion", "attraction", "k", "force_multiplier", "balance", "friction")


def build_oracle(force: bool = False) -> Path:
    """Compile cf_oracle.c and cf_adjoint_oracle.c with contraction off (every float op rounded on its own)."""
    srcs = [HERE / "cf_oracle.c", HERE / "cf_adjoint_oracle.c"]
    if not force and ORACLE_LIB.exists() and all(ORACLE_LIB.stat().st_mtime >= s.stat().st_mtime for s in srcs):
        return ORACLE_LIB
    BUILD.mkdir(exist_ok=True)
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           *map(str, srcs), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def reference_root() -> Path:
    """The reference checkout: $CELLFLOW_REFERENCE, else a directory named `reference` beside
    this repository."""
    env = os.environ.get("CELLFLOW_REFERENCE")
    return Path(env) if env else HERE.parent.parent / "reference"


def build_ref(gpu: bool = True) -> bool:
    """Run build_ref.sh; True when oracle/_ref/libcfref.so exists afterwards."""
    inputs = [REF_DIR / "ref_step_kernel.inc", HERE / "ref_host_shim.cu", HERE / "ref_gpu_shim.cu",
              HERE / "build_ref.sh", REF_DIR / "ref_mesh_kernel.inc"]
    outputs = [REF_LIB] + ([REF_GPU_LIB] if gpu else [])
    ref_src = reference_root() / "cuda-native/src/ParticleSimulation.cu"
    if not ref_src.exists() and all(p.exists() for p in outputs + inputs[:1]):
        newest = max(p.stat().st_mtime for p in inputs if p.exists())
        if all(o.stat().st_mtime >= newest for o in outputs):
            return True
    args = [str(HERE / "build_ref.sh")] + ([] if gpu else ["--no-gpu"])
    subprocess.run(["sh", *args], check=True, env=dict(os.environ, CELLFLOW_REFERENCE=str(reference_root())))
    return REF_LIB.exists()


_oracle = None
_ref = None
_ref_gpu = None


def lib() -> C.CDLL:
    global _oracle
    if _oracle is None:
        build_oracle()
        L = C.CDLL(str(ORACLE_LIB))
        vp, P = C.c_void_p, C.POINTER(OracleParams)
        L.cfo_step_f32.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, P, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp]
        L.cfo_step_f32.restype = None
        L.cfo_step_f64.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, P, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp]
        L.cfo_step_f64.restype = None
        L.cfo_force_table.argtypes = [vp, C.c_int, C.c_float, C.c_float, C.c_float, vp]
        L.cfo_force_table.restype = None
        L.cfo_rotate.argtypes = [vp, C.c_int]
        L.cfo_rotate.restype = None
        L.cfo_lfo.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float]
        L.cfo_lfo.restype = C.c_float
        L.cfo_proximity_edges.argtypes = [C.c_int, vp, vp, C.c_float, C.c_int, vp, C.c_long]
        L.cfo_proximity_edges.restype = C.c_long
        L.cfo_cell_list.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, vp]
        L.cfo_cell_list.restype = None
        L.cfo_c27.argtypes = [C.c_int, vp, vp, vp]
        L.cfo_c27.restype = C.c_double
        L.cfo_triangle_mesh.argtypes = [C.c_int, vp, vp, C.c_float, C.c_int, vp, C.c_int, vp, vp, C.c_long]
        L.cfo_triangle_mesh.restype = C.c_long
        P64 = C.POINTER(Phys64)
        L.cfo_rollout_f64.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, C.c_int, P64, vp, C.c_int, vp, vp]
        L.cfo_rollout_f64.restype = None
        L.cfo_rollout_grad_f64.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, C.c_int, P64, vp, C.c_int, vp, vp,
                                           vp, vp, vp, vp]
        L.cfo_rollout_grad_f64.restype = None
        L.cfo_rollout_grad_traj_f64.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, C.c_int, P64, vp, C.c_int, vp, vp,
                                                vp, vp, vp, vp]
        L.cfo_rollout_grad_traj_f64.restype = None
        L.cfo_rdf_f64.argtypes = [C.c_int, vp, vp, C.c_int, vp, C.c_int, C.c_double, vp]
        L.cfo_rdf_f64.restype = None
        L.cfo_rdf_grad_f64.argtypes = [C.c_int, vp, vp, C.c_int, vp, C.c_int, C.c_double, vp, vp]
        L.cfo_rdf_grad_f64.restype = None
        _oracle = L
    return _oracle


def ref_available() -> bool:
    return REF_LIB.exists()


def ref_lib() -> C.CDLL:
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise FileNotFoundError(f"{REF_LIB} not built (oracle/build_ref.sh)")
        L = C.CDLL(str(REF_LIB))
        vp = C.c_void_p
        f = C.c_float
        L.cfref_step.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int,
                                 f, f, f, f, f, f, f, f, f, f, C.c_int, f, f, C.c_int]
        L.cfref_step.restype = None
        L.cfref_proximity.argtypes = [C.c_int, vp, f, C.c_int, vp, C.c_int, vp]
        L.cfref_proximity.restype = C.c_int
        L.cfref_triangle_mesh.argtypes = [C.c_int, vp, f, C.c_int, vp, C.c_int, vp]
        L.cfref_triangle_mesh.restype = C.c_int
        L.cfref_force_table.argtypes = [vp, C.c_int, f, f, f, vp]
        L.cfref_force_table.restype = C.c_int
        L.cfref_sizeof_particle.restype = C.c_int
        _ref = L
    return _ref


def ref_gpu_lib() -> C.CDLL:
    global _ref_gpu
    if _ref_gpu is None:
        if not REF_GPU_LIB.exists():
            raise FileNotFoundError(f"{REF_GPU_LIB} not built (oracle/build_ref.sh)")
        L = C.CDLL(str(REF_GPU_LIB))
        vp, f = C.c_void_p, C.c_float
        L.cfref_gpu_step.argtypes = [vp, vp, vp, vp, vp, C.c_int, f, f, f, f, f, f, f, f, f, f, C.c_int, f, f,
                                     C.c_int, vp]
        L.cfref_gpu_step.restype = C.c_int
        L.cfref_gpu_proximity.argtypes = [vp, C.c_int, f, C.c_int, vp, C.c_int, vp, vp, vp]
        L.cfref_gpu_proximity.restype = C.c_int
        _ref_gpu = L
    return _ref_gpu


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def to_oracle_params(p) -> OracleParams:
    """From a cellflow_gb300.world.SimulationParams (or any object with those fields)."""
    return OracleParams(p.radius, p.delta_t, p.friction, p.repulsion, p.attraction, p.k, p.balance,
                        p.canvas_width, p.canvas_height, p.canvas_depth, p.num_particle_types, p.ratio_with_lfo,
                        p.force_multiplier, p.max_expected_neighbors)


def _f32(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a if shape is None else a.reshape(shape)


def step_f32(pos, vel, types, counts, table, radio, params, rows=None):
    """Restated FP32 step.  rows = (begin, end, stride) selects particles; others stay zero."""
    pos, vel = _f32(pos, (-1, 3)), _f32(vel, (-1, 3))
    n = len(pos)
    types = np.ascontiguousarray(types, dtype=np.uint32)
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    table, radio = _f32(table).ravel(), _f32(radio).ravel()
    b, e, s = rows if rows else (0, n, 1)
    po, vo, ao = np.zeros_like(pos), np.zeros_like(pos), np.zeros_like(pos)
    co = np.zeros(n, dtype=np.int32)
    lib().cfo_step_f32(n, _p(pos), _p(vel), _p(types), _p(counts), _p(table), _p(radio),
                       C.byref(to_oracle_params(params)), b, e, s, _p(po), _p(vo), _p(ao), _p(co))
    return po, vo, ao, co


def step_f64(pos, vel, types, counts, table, radio, params, rows=None):
    """FP64 step from FP32 inputs; also returns per-particle term magnitude.
    rows = (begin, end, stride) selects particles as in step_f32."""
    pos, vel = _f32(pos, (-1, 3)), _f32(vel, (-1, 3))
    n = len(pos)
    types = np.ascontiguousarray(types, dtype=np.uint32)
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    table, radio = _f32(table).ravel(), _f32(radio).ravel()
    b, e, s = rows if rows else (0, n, 1)
    po, vo, ao = (np.zeros((n, 3)) for _ in range(3))
    co = np.zeros(n, dtype=np.int32)
    mag = np.zeros(n)
    lib().cfo_step_f64(n, _p(pos), _p(vel), _p(types), _p(counts), _p(table), _p(radio),
                       C.byref(to_oracle_params(params)), b, e, s, _p(po), _p(vo), _p(ao), _p(co), _p(mag))
    return po, vo, ao, co, mag


def force_table(raw, range_, bias, offset) -> np.ndarray:
    raw = _f32(raw).ravel()
    out = np.zeros_like(raw)
    lib().cfo_force_table(_p(raw), raw.size, range_, bias, offset, _p(out))
    return out


def rotate(values) -> np.ndarray:
    v = _f32(values).ravel().copy()
    lib().cfo_rotate(_p(v), v.size)
    return v


def lfo(ratio, lfo_a, lfo_s, t) -> float:
    return lib().cfo_lfo(ratio, lfo_a, lfo_s, t)


def proximity_edges(pos, types, distance, max_conn) -> np.ndarray:
    pos = _f32(pos, (-1, 3))
    types = np.ascontiguousarray(types, dtype=np.uint32)
    n = len(pos)
    cap = n * max(min(max_conn, 32), 0)
    edges = np.zeros((max(cap, 1), 2), dtype=np.int32)
    total = lib().cfo_proximity_edges(n, _p(pos), _p(types), distance, max_conn, _p(edges), cap)
    return edges[:total].copy()


def triangle_mesh(pos, types, distance, max_conn, colors, num_types):
    """Restated triangle mesh: (triangles (K, 3) int32, vertices (3K, 9) float32), in i order."""
    pos = _f32(pos, (-1, 3))
    types = np.ascontiguousarray(types, dtype=np.uint32)
    cols = _f32(colors, (-1, 3))
    n = len(pos)
    total = lib().cfo_triangle_mesh(n, _p(pos), _p(types), distance, max_conn, _p(cols), num_types, None, None, 0)
    tris = np.zeros((max(total, 1), 3), dtype=np.int32)
    verts = np.zeros((max(3 * total, 1), 9), dtype=np.float32)
    lib().cfo_triangle_mesh(n, _p(pos), _p(types), distance, max_conn, _p(cols), num_types, _p(tris), _p(verts),
                            total)
    return tris[:total].copy(), verts[:3 * total].copy()


def cell_list(pos, cells, inv_cell):
    pos = _f32(pos, (-1, 3))
    n = len(pos)
    m = np.ascontiguousarray(cells, dtype=np.int32)
    inv = _f32(inv_cell)
    total = int(m[0]) * int(m[1]) * int(m[2])
    cell_of = np.zeros(n, dtype=np.uint32)
    order = np.zeros(n, dtype=np.uint32)
    start = np.zeros(total, dtype=np.uint32)
    end = np.zeros(total, dtype=np.uint32)
    lib().cfo_cell_list(n, _p(pos), _p(m), _p(inv), _p(cell_of), _p(order), _p(start), _p(end))
    return cell_of, order, start, end


def c27(pos, cells, inv_cell) -> float:
    pos = _f32(pos, (-1, 3))
    m = np.ascontiguousarray(cells, dtype=np.int32)
    return lib().cfo_c27(len(pos), _p(pos), _p(m), _p(_f32(inv_cell)))


PARTICLE_DTYPE = np.dtype(
    [("pos", "<f4", 3), ("vel", "<f4", 3), ("acc", "<f4", 3), ("ptype", "<u4"), ("pad", "<f4")]
)


def to_records(pos, vel, types, acc=None) -> np.ndarray:
    pos = _f32(pos, (-1, 3))
    rec = np.zeros(len(pos), dtype=PARTICLE_DTYPE)
    rec["pos"] = pos
    rec["vel"] = _f32(vel, (-1, 3))
    if acc is not None:
        rec["acc"] = _f32(acc, (-1, 3))
    rec["ptype"] = np.asarray(types, dtype=np.uint32)
    return rec


def ref_step(records, table, radio, counts, params, rows=None):
    """The reference kernel body (ParticleSimulation.cu:69-166) on the host, Jacobi semantics."""
    rec = np.ascontiguousarray(records, dtype=PARTICLE_DTYPE)
    n = len(rec)
    out = np.zeros_like(rec)
    table, radio = _f32(table).ravel(), _f32(radio).ravel()
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    co = np.zeros(n, dtype=np.int32)
    b, e, s = rows if rows else (0, n, 1)
    p = params
    ref_lib().cfref_step(n, _p(rec), _p(table), _p(radio), _p(counts), _p(co), _p(out), b, e, s,
                         p.radius, p.delta_t, p.friction, p.repulsion, p.attraction, p.k, p.balance,
                         p.canvas_width, p.canvas_height, p.canvas_depth, p.num_particle_types, p.ratio_with_lfo,
                         p.force_multiplier, p.max_expected_neighbors)
    return out, co


def ref_proximity_vertices(records, distance, max_conn, colors, num_types) -> np.ndarray:
    """The reference proximity kernel body (ParticleSimulation.cu:188-277) on the host, in i order.
    Returns the line vertices, shape (V, 6)."""
    rec = np.ascontiguousarray(records, dtype=PARTICLE_DTYPE)
    n = len(rec)
    mc = max(min(max_conn, 32), 0)
    verts = np.zeros((max(n * 2 * mc * 2, 1), 6), dtype=np.float32)
    cols = _f32(colors, (-1, 3))
    count = ref_lib().cfref_proximity(n, _p(rec), distance, max_conn, _p(cols), num_types, _p(verts))
    return verts[:count].copy()


def ref_triangle_mesh(records, distance, max_conn, colors, num_types) -> np.ndarray:
    """The reference triangle-mesh kernel body (ParticleSimulation.cu:280-424) on the host, in i order,
    with the host wrapper's squared distance.  Returns the vertices, shape (V, 9)."""
    rec = np.ascontiguousarray(records, dtype=PARTICLE_DTYPE)
    n = len(rec)
    verts = np.zeros((max(n * 64 * 3, 1), 9), dtype=np.float32)
    cols = _f32(colors, (-1, 3))
    count = ref_lib().cfref_triangle_mesh(n, _p(rec), distance, max_conn, _p(cols), num_types, _p(verts))
    return verts[:count].copy()


def ref_force_table(raw, num_types, range_, bias, offset) -> np.ndarray:
    raw = _f32(raw).ravel()
    out = np.zeros(num_types * num_types, dtype=np.float32)
    rc = ref_lib().cfref_force_table(_p(raw), num_types, range_, bias, offset, _p(out))
    if rc:
        raise ValueError("reference force table supports T <= 10")
    return out


# ---- FP64 differentiable rollout (cf_adjoint_oracle.c)

def _f64(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def eff_table(params, radio, num_types) -> np.ndarray:
    """Effective radius of every type pair as the FP32 step rounds it (ParticleSimulation.cu:108-110)."""
    rb = _f32(radio).ravel()[:num_types]
    one, half = np.float32(1.0), np.float32(0.5)
    r = np.float32(params.radius) * (one + rb * np.float32(params.ratio_with_lfo))
    return ((r[:, None] + r[None, :]) * half).astype(np.float32)


def phys64(params, **override) -> Phys64:
    vals = {name: float(getattr(params, name)) for name in GRAD_PARAMS}
    vals["delta_t"] = float(params.delta_t)
    vals.update({k: float(v) for k, v in override.items()})
    return Phys64(vals["repulsion"], vals["attraction"], vals["k"], vals["force_multiplier"], vals["balance"],
                  vals["friction"], vals["delta_t"], int(params.max_expected_neighbors))


def _extent(params) -> np.ndarray:
    return np.array([params.canvas_width, params.canvas_height, params.canvas_depth], dtype=np.float64)


def rollout_f64(pos, vel, types, counts, table, eff, params, steps, **override):
    """FP64 rollout; returns (pos, vel, counts, min relative distance of any candidate pair to its cutoff,
    fingerprint of every step's neighbour counts)."""
    pos, vel = _f64(pos, (-1, 3)).copy(), _f64(vel, (-1, 3)).copy()
    n = len(pos)
    T = int(np.asarray(table).shape[0])
    types = np.ascontiguousarray(types, dtype=np.uint32)
    cnt = np.ascontiguousarray(counts, dtype=np.int32).copy()
    F, effa = _f64(table).ravel(), _f32(eff).ravel()
    ph, ext = phys64(params, **override), _extent(params)
    margin, fp = C.c_double(np.inf), C.c_uint64(0)
    lib().cfo_rollout_f64(n, _p(pos), _p(vel), _p(types), _p(cnt), _p(F), _p(effa), T, C.byref(ph), _p(ext), steps,
                          C.byref(margin), C.byref(fp))
    return pos, vel, cnt, margin.value, fp.value


def rollout_grad_f64(pos, vel, types, counts, table, eff, params, steps, gpos, gvel, **override):
    """FP64 adjoint of a rollout: (d/dpos0, d/dvel0, d/dF, d/dparams in GRAD_PARAMS order)."""
    pos, vel = _f64(pos, (-1, 3)), _f64(vel, (-1, 3))
    n = len(pos)
    T = int(np.asarray(table).shape[0])
    types = np.ascontiguousarray(types, dtype=np.uint32)
    cnt = np.ascontiguousarray(counts, dtype=np.int32)
    F, effa = _f64(table).ravel(), _f32(eff).ravel()
    ph, ext = phys64(params, **override), _extent(params)
    gp, gv = _f64(gpos, (-1, 3)), _f64(gvel, (-1, 3))
    g0, gv0 = np.zeros((n, 3)), np.zeros((n, 3))
    gF, gph = np.zeros(T * T), np.zeros(len(GRAD_PARAMS))
    lib().cfo_rollout_grad_f64(n, _p(pos), _p(vel), _p(types), _p(cnt), _p(F), _p(effa), T, C.byref(ph), _p(ext),
                               steps, _p(gp), _p(gv), _p(g0), _p(gv0), _p(gF), _p(gph))
    return g0, gv0, gF.reshape(T, T), gph


def rollout_grad_traj_f64(P, V, Cn, types, table, eff, params, gpos, gvel, **override):
    """FP64 adjoint along a given trajectory: P, V of shape (K+1, n, 3), Cn of shape (K+1, n)."""
    P, V = _f64(P), _f64(V)
    steps, n = P.shape[0] - 1, P.shape[1]
    T = int(np.asarray(table).shape[0])
    types = np.ascontiguousarray(types, dtype=np.uint32)
    Cn = np.ascontiguousarray(Cn, dtype=np.int32)
    F, effa = _f64(table).ravel(), _f32(eff).ravel()
    ph, ext = phys64(params, **override), _extent(params)
    gp, gv = _f64(gpos, (-1, 3)), _f64(gvel, (-1, 3))
    g0, gv0 = np.zeros((n, 3)), np.zeros((n, 3))
    gF, gph = np.zeros(T * T), np.zeros(len(GRAD_PARAMS))
    lib().cfo_rollout_grad_traj_f64(n, _p(P), _p(V), _p(Cn), _p(types), _p(F), _p(effa), T, C.byref(ph), _p(ext),
                                    steps, _p(gp), _p(gv), _p(g0), _p(gv0), _p(gF), _p(gph))
    return g0, gv0, gF.reshape(T, T), gph


def rdf_f64(pos, types, num_types, extent, bins, r_max) -> np.ndarray:
    """Soft type-resolved radial distribution, shape (T, T, bins)."""
    pos = _f64(pos, (-1, 3))
    types = np.ascontiguousarray(types, dtype=np.uint32)
    ext = _f64(extent)
    h = np.zeros(num_types * num_types * bins)
    lib().cfo_rdf_f64(len(pos), _p(pos), _p(types), num_types, _p(ext), bins, r_max, _p(h))
    return h.reshape(num_types, num_types, bins)


def rdf_grad_f64(pos, types, num_types, extent, bins, r_max, ghist) -> np.ndarray:
    pos = _f64(pos, (-1, 3))
    types = np.ascontiguousarray(types, dtype=np.uint32)
    ext, g = _f64(extent), _f64(ghist).ravel()
    out = np.zeros_like(pos)
    lib().cfo_rdf_grad_f64(len(pos), _p(pos), _p(types), num_types, _p(ext), bins, r_max, _p(g), _p(out))
    return out
