"""ctypes binding of the C ABI in include/acvd_gpu.h (libacvd_gb300.so).

`Engine` wraps one device context; the functions at module level are the
host-side set-up helpers (topology, weights, initial sampling).  There is no
fallback: if the CUDA library is missing or the device is unusable, the calls
raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

ACVD_OK = 0
ERRORS = {1: "ACVD_ERR_ARG", 2: "ACVD_ERR_CUDA", 3: "ACVD_ERR_ITER_LIMIT", 4: "ACVD_ERR_DEVICE_CHECK",
          5: "ACVD_ERR_UNSUPPORTED"}
METRICS = {"iso": 0, "isotropic": 0, "qem": 1, "aniso": 2, "quadric_anisotropic": 2}


class AcvdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("use_graphs", ctypes.c_int), ("max_loops", ctypes.c_int),
                ("max_convergences", ctypes.c_int), ("kernel_timing", ctypes.c_int), ("persistent", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("sweeps", ctypes.c_int), ("convergences", ctypes.c_int), ("moves", ctypes.c_int64),
                ("candidates", ctypes.c_int64), ("boundary_items", ctypes.c_int64),
                ("targets", ctypes.c_int64), ("visited", ctypes.c_int64), ("slots", ctypes.c_int64),
                ("disconnected", ctypes.c_int), ("unassigned", ctypes.c_int), ("device_ms", ctypes.c_double),
                ("eval_ms", ctypes.c_double), ("eval_launches", ctypes.c_int), ("energy", ctypes.c_double),
                ("eval_bytes", ctypes.c_int64), ("kernel_launches", ctypes.c_int64), ("hit_loop_cap", ctypes.c_int),
                ("reverted", ctypes.c_int64), ("relaxed_sweeps", ctypes.c_int), ("sweep_kernel_ms", ctypes.c_double),
                ("sweep_kernel_launches", ctypes.c_int)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_LIB = None
_P = ctypes.c_void_p
_i64 = ctypes.c_int64


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def lib_path() -> str:
    return _build.LIB


_LIB_PLAIN = None


def load(build_if_missing: bool = True, plain: bool = False) -> ctypes.CDLL:
    """Loads libacvd_gb300.so (building it first when it is absent).  plain=True loads
    libacvd_gb300_plain.so instead: the same C ABI, with the clustering kernels built
    with plain float32 cluster sums (no compensation), for accuracy comparisons."""
    global _LIB, _LIB_PLAIN
    if plain and _LIB_PLAIN is not None:
        return _LIB_PLAIN
    if not plain and _LIB is not None:
        return _LIB
    path = _build.LIB_PLAIN if plain else _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"CUDA library not built: {path}")
        _build.build()
    lib = ctypes.CDLL(path)
    sig = {
        "acvd_default_opts": (None, [ctypes.POINTER(Opts)]),
        "acvd_create": (_P, [ctypes.POINTER(Opts)]),
        "acvd_destroy": (None, [_P]),
        "acvd_last_error": (ctypes.c_char_p, [_P]),
        "acvd_stream": (_P, [_P]),
        "acvd_build_topology": (ctypes.c_int, [_i64, _i64, _P, _P, _P, _P, ctypes.POINTER(_i64)]),
        "acvd_vertex_weights": (ctypes.c_int, [ctypes.c_int, _i64, _P, _i64, _P, _P, _P, _P, _P, ctypes.c_double, _P]),
        "acvd_initial_sampling": (ctypes.c_int, [_i64, _P, _P, _P, ctypes.c_int32, _P]),
        "acvd_initial_sampling_fixed": (ctypes.c_int, [_i64, _P, _P, _P, ctypes.c_int32, ctypes.c_int32, _P, _P]),
        "acvd_set_fixed_clusters": (ctypes.c_int, [_P, ctypes.c_int32, _P]),
        "acvd_density_indicator": (ctypes.c_int, [ctypes.c_char_p, _i64, _P, ctypes.c_double, ctypes.c_double,
                                                  ctypes.c_double, _P]),
        "acvd_split_long_edges": (ctypes.c_int, [_i64, _P, _i64, _P, ctypes.c_double,
                                                 ctypes.POINTER(ctypes.POINTER(ctypes.c_double)),
                                                 ctypes.POINTER(_i64), ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)),
                                                 ctypes.POINTER(_i64)]),
        "acvd_set_anchor_items": (ctypes.c_int, [_P, ctypes.c_int32, _P]),
        "acvd_clean_clustering": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32)]),
        "acvd_set_mesh": (ctypes.c_int, [_P, _i64, _P, _i64, _P, _P, _P, _i64, _P]),
        "acvd_set_metric": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, ctypes.c_double]),
        "acvd_set_quadrics_optimization_level": (ctypes.c_int, [_P, ctypes.c_int]),
        "acvd_set_unconstrained_initialization": (ctypes.c_int, [_P, ctypes.c_int]),
        "acvd_set_labels": (ctypes.c_int, [_P, ctypes.c_int32, _P]),
        "acvd_minimize": (ctypes.c_int, [_P, ctypes.POINTER(Stats)]),
        "acvd_rewind": (ctypes.c_int, [_P]),
        "acvd_set_batch": (ctypes.c_int, [_P, ctypes.c_int, _P, _P]),
        "acvd_adjoint": (ctypes.c_int, [_P, _P, _P, ctypes.c_double, ctypes.c_double, _P, _P, _P, _P, _P, _P]),
        "acvd_adjoint_on_stream": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_double, _P, _P, _P, _P, _P, _P, _P]),
        "acvd_get_mesh_energies": (ctypes.c_int, [_P, _P]),
        "acvd_get_labels": (ctypes.c_int, [_P, _P]),
        "acvd_get_clusters": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
        "acvd_get_boundary_edges": (ctypes.c_int, [_P, _P, ctypes.POINTER(_i64)]),
        "acvd_get_dual_mesh": (ctypes.c_int, [_P, _P, ctypes.POINTER(_i64)]),
        "acvd_boundary_edges_noalloc": (ctypes.c_int, [_P, _i64, _P, _P, _P, _P]),
        "acvd_post_placement": (ctypes.c_int, [_P, ctypes.c_int, _P]),
        "acvd_compute_curvature": (ctypes.c_int, [_P, _P, _P]),
        "acvd_set_frozen_clusters": (ctypes.c_int, [_P, _P]),
        "acvd_check_wait_limit": (ctypes.c_int, [_P, _i64, ctypes.POINTER(ctypes.c_int32)]),
        "acvd_get_frozen_clusters": (ctypes.c_int, [_P, _P]),
        "acvd_fix_mesh_boundaries": (ctypes.c_int, [_P, _P, ctypes.POINTER(_i64), _P, ctypes.POINTER(_i64)]),
        "acvd_force_manifold_step": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32),
                                                    ctypes.POINTER(ctypes.c_int32)]),
        "acvd_read_mesh": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)),
                                          ctypes.POINTER(_i64), ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)),
                                          ctypes.POINTER(_i64)]),
        "acvd_write_mesh": (ctypes.c_int, [ctypes.c_char_p, _P, _i64, _P, _i64]),
        "acvd_free": (None, [_P]),
        "acvd_io_last_error": (ctypes.c_char_p, []),
        "acvd_subdivide_work_bytes": (_i64, [_i64]),
        "acvd_subdivide_device": (ctypes.c_int, [_P, _i64, _P, _i64, _P, _P, _P, _i64, _P, _P, _P, _P, _P, _P, _P,
                                                 _P]),
        "acvd_subdivide": (ctypes.c_int, [_P, _i64, _P, _i64, _P, _P, _P, _i64, _P, _P, _P, _P, _P, _P, _P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if plain:
        _LIB_PLAIN = lib
    else:
        _LIB = lib
    return lib


def exported_symbols() -> list[str]:
    """Entry points declared in include/acvd_gpu.h."""
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "acvd_gpu.h")
    import re
    return sorted(set(re.findall(r"\b(acvd_[a-z_0-9]+)\s*\(", open(hdr).read())))


def _check(code: int, ctx=None, what: str = ""):
    if code != ACVD_OK:
        msg = what
        if ctx:
            msg = (load().acvd_last_error(ctx) or b"").decode() or what
        raise AcvdError(code, msg)


# ---------------------------------------------------------------------------
# host-side set-up helpers
# ---------------------------------------------------------------------------

def build_topology(n_vertices: int, faces: np.ndarray):
    """Ring CSR (row, col) and edge endpoints in the reference's numbering."""
    lib = load()
    tri = np.ascontiguousarray(faces, dtype=np.int32)
    ne = _i64()
    _check(lib.acvd_build_topology(n_vertices, tri.shape[0], _ptr(tri), None, None, None, ctypes.byref(ne)),
           what="acvd_build_topology")
    row = np.empty(n_vertices + 1, dtype=np.int32)
    col = np.empty(2 * ne.value, dtype=np.int32)
    ev = np.empty(2 * ne.value, dtype=np.int32)
    _check(lib.acvd_build_topology(n_vertices, tri.shape[0], _ptr(tri), _ptr(row), _ptr(col), _ptr(ev),
                                   ctypes.byref(ne)), what="acvd_build_topology")
    return row, col, ev.reshape(-1, 2)


def read_mesh(path: str):
    """vtkSurface::CreateFromFile for triangle meshes (.ply .off .obj .stl .vtk):
    (points (nV, 3) float64, faces (nF, 3) int32)."""
    lib = load()
    xp = ctypes.POINTER(ctypes.c_double)()
    tp = ctypes.POINTER(ctypes.c_int32)()
    nv, nf = _i64(0), _i64(0)
    code = lib.acvd_read_mesh(os.fsencode(path), ctypes.byref(xp), ctypes.byref(nv), ctypes.byref(tp),
                              ctypes.byref(nf))
    if code != ACVD_OK:
        raise AcvdError(code, (lib.acvd_io_last_error() or b"").decode())
    try:
        pts = np.ctypeslib.as_array(xp, shape=(3 * nv.value,)).copy().reshape(-1, 3) if nv.value else \
            np.zeros((0, 3))
        tri = np.ctypeslib.as_array(tp, shape=(3 * nf.value,)).copy().reshape(-1, 3) if nf.value else \
            np.zeros((0, 3), dtype=np.int32)
    finally:
        lib.acvd_free(ctypes.cast(xp, ctypes.c_void_p))
        lib.acvd_free(ctypes.cast(tp, ctypes.c_void_p))
    return pts, tri


def write_mesh(path: str, points: np.ndarray, faces: np.ndarray) -> None:
    """vtkSurface::WriteToFile (.ply binary, .off, .obj, .stl binary, .vtk ascii)."""
    lib = load()
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    tri = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
    code = lib.acvd_write_mesh(os.fsencode(path), _ptr(pts), pts.shape[0], _ptr(tri), tri.shape[0])
    if code != ACVD_OK:
        raise AcvdError(code, (lib.acvd_io_last_error() or b"").decode())


def vertex_weights(metric: str, points: np.ndarray, faces: np.ndarray, indicator=None, gradation: float = 0.0):
    lib = load()
    pts = np.ascontiguousarray(points, dtype=np.float64)
    tri = np.ascontiguousarray(faces, dtype=np.int32)
    ind = None if indicator is None else np.ascontiguousarray(indicator, dtype=np.float64)
    w = np.empty(pts.shape[0], dtype=np.float64)
    _check(lib.acvd_vertex_weights(METRICS[metric], pts.shape[0], _ptr(pts), tri.shape[0], _ptr(tri), None, None,
                                   None, _ptr(ind), float(gradation), _ptr(w)), what="acvd_vertex_weights")
    return w


def density_indicator(image_path: str, points: np.ndarray, max_density: float = 1.0, min_density: float = 0.1,
                      factor: float = 0.001) -> np.ndarray:
    """The custom-density indicator of a MetaImage volume at the points
    (vtkDiscreteRemeshing's InputDensityFile): max(max - value * factor, min)."""
    lib = load()
    pts = np.ascontiguousarray(points, dtype=np.float64)
    out = np.empty(pts.shape[0], dtype=np.float64)
    code = lib.acvd_density_indicator(os.fsencode(image_path), pts.shape[0], _ptr(pts), float(max_density),
                                      float(min_density), float(factor), _ptr(out))
    if code != ACVD_OK:
        raise AcvdError(code, (lib.acvd_io_last_error() or b"").decode())
    return out


def split_long_edges(points: np.ndarray, faces: np.ndarray, ratio: float):
    """vtkSurface::SplitLongEdges: (points, faces) with every edge at most ratio x the
    input's mean edge length; vertices keep their ids, new ones are appended."""
    lib = load()
    pts = np.ascontiguousarray(points, dtype=np.float64)
    tri = np.ascontiguousarray(faces, dtype=np.int32)
    xp = ctypes.POINTER(ctypes.c_double)()
    tp = ctypes.POINTER(ctypes.c_int32)()
    nv, nf = _i64(0), _i64(0)
    _check(lib.acvd_split_long_edges(pts.shape[0], _ptr(pts), tri.shape[0], _ptr(tri), float(ratio), ctypes.byref(xp),
                                     ctypes.byref(nv), ctypes.byref(tp), ctypes.byref(nf)),
           what="acvd_split_long_edges")
    try:
        out_p = np.ctypeslib.as_array(xp, shape=(nv.value * 3,)).reshape(-1, 3).copy()
        out_t = np.ctypeslib.as_array(tp, shape=(max(nf.value, 1) * 3,))[: nf.value * 3].reshape(-1, 3).copy()
    finally:
        lib.acvd_free(ctypes.cast(xp, ctypes.c_void_p))
        lib.acvd_free(ctypes.cast(tp, ctypes.c_void_p))
    return out_p, out_t


def initial_sampling(row: np.ndarray, col: np.ndarray, weights: np.ndarray, k: int,
                     fixed: np.ndarray | None = None) -> np.ndarray:
    """ComputeInitialRandomSampling; `fixed` (vertex ids) start in clusters 0 .. F-1."""
    lib = load()
    row = np.ascontiguousarray(row, dtype=np.int32)
    col = np.ascontiguousarray(col, dtype=np.int32)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    lab = np.empty(row.shape[0] - 1, dtype=np.int32)
    if fixed is None or len(fixed) == 0:
        _check(lib.acvd_initial_sampling(row.shape[0] - 1, _ptr(row), _ptr(col), _ptr(w), int(k), _ptr(lab)),
               what="acvd_initial_sampling")
        return lab
    f = np.ascontiguousarray(fixed, dtype=np.int32)
    _check(lib.acvd_initial_sampling_fixed(row.shape[0] - 1, _ptr(row), _ptr(col), _ptr(w), int(k), f.shape[0],
                                           _ptr(f), _ptr(lab)),
           what="acvd_initial_sampling_fixed")
    return lab


# ---------------------------------------------------------------------------
# device context
# ---------------------------------------------------------------------------

class Engine:
    """One GPU clustering context (acvd_ctx)."""

    # sweep cap used unless the caller asks otherwise (the reference's own cap,
    # 5,000,000 loops, is for a sequential loop; a GPU sweep does far more work)
    DEFAULT_MAX_LOOPS = 20000

    def __init__(self, device: int = 0, use_graphs: bool = True, kernel_timing: bool = False,
                 max_loops: int | None = DEFAULT_MAX_LOOPS, persistent: bool = False,
                 max_convergences: int | None = None, plain: bool = False):
        lib = load(plain=plain)
        o = Opts()
        lib.acvd_default_opts(ctypes.byref(o))
        o.device = device
        o.use_graphs = 1 if use_graphs else 0
        o.persistent = 1 if persistent else 0
        o.kernel_timing = 1 if kernel_timing else 0
        if max_loops is not None:
            o.max_loops = int(max_loops)
        if max_convergences is not None:
            o.max_convergences = int(max_convergences)
        self._lib = lib
        self.ctx = lib.acvd_create(ctypes.byref(o))
        if not self.ctx:
            raise AcvdError(2, "acvd_create failed (no usable CUDA device?)")
        self.n = 0
        self.k = 0
        self.n_edges = 0

    def close(self):
        if getattr(self, "ctx", None):
            self._lib.acvd_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, code, what=""):
        _check(code, self.ctx, what)

    def stream(self) -> int:
        return int(self._lib.acvd_stream(self.ctx) or 0)

    def set_mesh(self, points, faces, row, col, edge_v):
        self._pts = np.ascontiguousarray(points, dtype=np.float64)
        self._tri = np.ascontiguousarray(faces, dtype=np.int32)
        row = np.ascontiguousarray(row, dtype=np.int32)
        col = np.ascontiguousarray(col, dtype=np.int32)
        ev = np.ascontiguousarray(edge_v, dtype=np.int32)
        self.n = self._pts.shape[0]
        self.n_edges = ev.size // 2
        self._ck(self._lib.acvd_set_mesh(self.ctx, self.n, _ptr(self._pts), self._tri.shape[0], _ptr(self._tri),
                                         _ptr(row), _ptr(col), self.n_edges, _ptr(ev)), "acvd_set_mesh")

    def set_metric(self, metric: str, indicator=None, principal_dirs=None, gradation: float = 0.0):
        ind = None if indicator is None else np.ascontiguousarray(indicator, dtype=np.float64)
        pd = None if principal_dirs is None else np.ascontiguousarray(principal_dirs, dtype=np.float32)
        self.metric = metric
        self._ck(self._lib.acvd_set_metric(self.ctx, METRICS[metric], _ptr(ind), _ptr(pd), float(gradation)),
                 "acvd_set_metric")

    def set_batch(self, vertex_offsets, cluster_offsets):
        vo = np.ascontiguousarray(vertex_offsets, dtype=np.int64)
        ko = np.ascontiguousarray(cluster_offsets, dtype=np.int32)
        self.nmesh = vo.shape[0] - 1
        self._ck(self._lib.acvd_set_batch(self.ctx, self.nmesh, _ptr(vo), _ptr(ko)), "acvd_set_batch")

    def mesh_energies(self) -> np.ndarray:
        out = np.empty(self.nmesh, dtype=np.float64)
        self._ck(self._lib.acvd_get_mesh_energies(self.ctx, _ptr(out)), "acvd_get_mesh_energies")
        return out

    def adjoint_raw(self, xyz_ptr: int, rho_ptr: int | None, gradation: float, g_energy: float,
                    g_centroids_ptr: int | None, centroids_ptr: int | None, grad_xyz_ptr: int | None,
                    grad_rho_ptr: int | None, cluster_energies_ptr: int | None = None) -> float:
        """acvd_adjoint on DEVICE pointers (float64); returns the energy."""
        e = ctypes.c_double()
        self._ck(self._lib.acvd_adjoint(self.ctx, xyz_ptr, rho_ptr, float(gradation), float(g_energy),
                                        g_centroids_ptr, ctypes.byref(e), cluster_energies_ptr, centroids_ptr,
                                        grad_xyz_ptr, grad_rho_ptr), "acvd_adjoint")
        return e.value

    def set_level(self, level: int):
        self._ck(self._lib.acvd_set_quadrics_optimization_level(self.ctx, int(level)))

    def set_unconstrained_initialization(self, on: int):
        self._ck(self._lib.acvd_set_unconstrained_initialization(self.ctx, int(on)))

    def set_labels(self, k: int, labels):
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        self.k = int(k)
        self._ck(self._lib.acvd_set_labels(self.ctx, self.k, _ptr(lab)), "acvd_set_labels")

    def rewind(self):
        self._ck(self._lib.acvd_rewind(self.ctx), "acvd_rewind")

    def minimize(self) -> dict:
        st = Stats()
        self._ck(self._lib.acvd_minimize(self.ctx, ctypes.byref(st)), "acvd_minimize")
        return st.as_dict()

    def compute_curvature(self, indicator: np.ndarray | None = None, principal_dirs: np.ndarray | None = None,
                          copy_out: bool = True):
        """Per-vertex curvature indicator (nV) and principal directions (nV x 6,
        float32), vtkCurvatureMeasure's polynomial fitting on the vertex 3-ring.
        Writes into the given arrays when passed (e.g. pinned buffers); with
        copy_out=False the results stay on the device and None is returned."""
        if not copy_out:
            self._ck(self._lib.acvd_compute_curvature(self.ctx, None, None), "acvd_compute_curvature")
            return None
        ind = indicator if indicator is not None else np.empty(self.n, dtype=np.float64)
        pd = principal_dirs if principal_dirs is not None else np.empty((self.n, 6), dtype=np.float32)
        if ind.dtype != np.float64 or pd.dtype != np.float32 or ind.size != self.n or pd.size != 6 * self.n \
                or not ind.flags.c_contiguous or not pd.flags.c_contiguous:
            raise ValueError("compute_curvature needs contiguous float64 (n) and float32 (n x 6) outputs")
        self._ck(self._lib.acvd_compute_curvature(self.ctx, _ptr(ind), _ptr(pd)), "acvd_compute_curvature")
        return ind, pd

    def set_frozen_clusters(self, frozen: np.ndarray | None):
        """IsClusterFreezed for the next minimize(): K flags (nonzero = frozen) or None."""
        if frozen is None:
            self._ck(self._lib.acvd_set_frozen_clusters(self.ctx, None), "acvd_set_frozen_clusters")
            return
        f = np.ascontiguousarray(frozen, dtype=np.uint8)
        if f.size != self.k:
            raise ValueError("set_frozen_clusters needs one flag per cluster")
        self._frozen = f
        self._ck(self._lib.acvd_set_frozen_clusters(self.ctx, _ptr(f)), "acvd_set_frozen_clusters")

    def set_fixed_clusters(self, vertex_ids):
        """SetFixedClusters: cluster c < len(vertex_ids) is the cluster of vertex_ids[c]
        (cleaning keeps the component holding it); empty or None clears the list."""
        f = np.ascontiguousarray([] if vertex_ids is None else vertex_ids, dtype=np.int32)
        self._fixed = f
        self._ck(self._lib.acvd_set_fixed_clusters(self.ctx, f.shape[0], _ptr(f) if f.size else None),
                 "acvd_set_fixed_clusters")

    def set_anchor_items(self, anchors):
        """QEM Cluster::AnchorItem of clusters 0 .. len(anchors)-1 (-1: none); empty or
        None clears them."""
        a = np.ascontiguousarray([] if anchors is None else anchors, dtype=np.int32)
        self._anchors = a
        self._ck(self._lib.acvd_set_anchor_items(self.ctx, a.shape[0], _ptr(a) if a.size else None),
                 "acvd_set_anchor_items")

    def clean_clustering(self) -> int:
        """CleanClustering on the current labels: the number of clusters that had
        several connected components (their smaller ones are now unassigned)."""
        n = ctypes.c_int32(0)
        self._ck(self._lib.acvd_clean_clustering(self.ctx, ctypes.byref(n)), "acvd_clean_clustering")
        return int(n.value)

    def check_wait_limit(self, max_spins: int = 1 << 18) -> bool:
        """Runs the device barrier with one block never arriving: True when its wait
        gave up (as it must) and returned."""
        g = ctypes.c_int32(0)
        self._ck(self._lib.acvd_check_wait_limit(self.ctx, int(max_spins), ctypes.byref(g)), "acvd_check_wait_limit")
        return bool(g.value)

    def frozen_clusters(self) -> np.ndarray:
        out = np.empty(self.k, dtype=np.uint8)
        self._ck(self._lib.acvd_get_frozen_clusters(self.ctx, _ptr(out)), "acvd_get_frozen_clusters")
        return out

    def force_manifold_step(self) -> int:
        """One pass of Remesh()'s ForceManifold loop: the number of topology issues (0:
        nothing changed); otherwise new clusters were added (self.k grows) and the
        others frozen for the next minimize()."""
        n, k = ctypes.c_int32(0), ctypes.c_int32(0)
        self._ck(self._lib.acvd_force_manifold_step(self.ctx, ctypes.byref(n), ctypes.byref(k)),
                 "acvd_force_manifold_step")
        self.k = int(k.value)
        return int(n.value)

    def fix_mesh_boundaries(self):
        """FixMeshBoundaries for the current clustering: (new points (n, 3) float64
        holding float values, numbered from K; new faces (m, 3) int32)."""
        n, m = _i64(0), _i64(0)
        self._ck(self._lib.acvd_fix_mesh_boundaries(self.ctx, None, ctypes.byref(n), None, ctypes.byref(m)),
                 "acvd_fix_mesh_boundaries")
        pts = np.empty((max(n.value, 1), 3), dtype=np.float64)
        tri = np.empty((max(m.value, 1), 3), dtype=np.int32)
        self._ck(self._lib.acvd_fix_mesh_boundaries(self.ctx, _ptr(pts), ctypes.byref(n), _ptr(tri), ctypes.byref(m)),
                 "acvd_fix_mesh_boundaries")
        return pts[:n.value], tri[:m.value]

    def subdivide(self, points: np.ndarray, faces: np.ndarray, row: np.ndarray, col: np.ndarray,
                  edge_v: np.ndarray, indicator: np.ndarray | None = None):
        """One level of vtkSurface::Subdivide on the device (this context's device and
        stream; its mesh is untouched).  Returns (points (nV+nE, 3) float64 holding
        float values, faces (4 nF, 3) int32, parent1 (nE), parent2 (nE), indicator
        (nV+nE) or None)."""
        pts = np.ascontiguousarray(points, dtype=np.float64)
        tri = np.ascontiguousarray(faces, dtype=np.int32)
        row = np.ascontiguousarray(row, dtype=np.int32)
        col = np.ascontiguousarray(col, dtype=np.int32)
        ev = np.ascontiguousarray(edge_v, dtype=np.int32).reshape(-1)
        nv, nf, ne = pts.shape[0], tri.shape[0], ev.size // 2
        o_pts = np.empty((nv + ne, 3), dtype=np.float64)
        o_tri = np.empty((4 * nf, 3), dtype=np.int32)
        p1 = np.empty(ne, dtype=np.int32)
        p2 = np.empty(ne, dtype=np.int32)
        ind = o_ind = None
        if indicator is not None:
            ind = np.ascontiguousarray(indicator, dtype=np.float64)
            if ind.size != nv:
                raise ValueError("subdivide: the indicator needs one value per vertex")
            o_ind = np.empty(nv + ne, dtype=np.float64)
        self._ck(self._lib.acvd_subdivide(self.ctx, nv, _ptr(pts), nf, _ptr(tri), _ptr(row), _ptr(col), ne, _ptr(ev),
                                          _ptr(ind) if ind is not None else None, _ptr(o_pts), _ptr(o_tri), _ptr(p1),
                                          _ptr(p2), _ptr(o_ind) if o_ind is not None else None), "acvd_subdivide")
        return o_pts, o_tri, p1, p2, o_ind

    def subdivide_device(self, nv: int, d_xyz: int, nf: int, d_tri: int, d_row: int, d_col: int, ne: int,
                         d_edge_v: int, d_ind: int | None, d_out_xyz: int, d_out_tri: int, d_p1: int, d_p2: int,
                         d_out_ind: int | None, d_work: int) -> None:
        """acvd_subdivide_device: device pointers (ints), enqueued on this context's stream."""
        self._ck(self._lib.acvd_subdivide_device(self.ctx, nv, d_xyz, nf, d_tri, d_row, d_col, ne, d_edge_v,
                                                 d_ind, d_out_xyz, d_out_tri, d_p1, d_p2, d_out_ind, d_work),
                 "acvd_subdivide_device")

    def subdivide_work_bytes(self, ne: int) -> int:
        return int(self._lib.acvd_subdivide_work_bytes(ne))

    def post_placement(self, level: int = 1) -> np.ndarray:
        """ACVD's quadric post-placement of the output vertices (ACVD.cxx:217-291): (K, 3)."""
        out = np.empty((self.k, 3), dtype=np.float64)
        self._ck(self._lib.acvd_post_placement(self.ctx, int(level), _ptr(out)), "acvd_post_placement")
        return out

    def labels(self, out: np.ndarray | None = None) -> np.ndarray:
        """GetClustering(); `out` (int32, n items, contiguous) may be a caller's buffer,
        e.g. in pinned host memory."""
        if out is None:
            out = np.empty(self.n, dtype=np.int32)
        elif out.dtype != np.int32 or out.shape != (self.n,) or not out.flags.c_contiguous:
            raise ValueError("labels(out=...) needs a contiguous int32 array of n items")
        self._ck(self._lib.acvd_get_labels(self.ctx, _ptr(out)), "acvd_get_labels")
        return out

    def clusters(self) -> dict:
        k = self.k
        sz = np.empty(k, dtype=np.int32)
        S = np.empty(3 * k); W = np.empty(k); Q = np.empty(9 * k); C = np.empty(3 * k); E = np.empty(k)
        tot = ctypes.c_double()
        self._ck(self._lib.acvd_get_clusters(self.ctx, _ptr(sz), _ptr(S), _ptr(W), _ptr(Q), _ptr(C), _ptr(E),
                                             ctypes.byref(tot)), "acvd_get_clusters")
        return {"size": sz, "S": S.reshape(k, 3), "W": W, "Q": Q.reshape(k, 9), "centroid": C.reshape(k, 3),
                "energy": E, "energy_total": tot.value}

    def boundary_edges(self) -> np.ndarray:
        n = _i64()
        self._ck(self._lib.acvd_get_boundary_edges(self.ctx, None, ctypes.byref(n)))
        out = np.empty(max(n.value, 1), dtype=np.int32)
        self._ck(self._lib.acvd_get_boundary_edges(self.ctx, _ptr(out), ctypes.byref(n)))
        return out[:n.value]

    def dual_mesh(self) -> np.ndarray:
        n = _i64()
        self._ck(self._lib.acvd_get_dual_mesh(self.ctx, None, ctypes.byref(n)))
        out = np.empty(3 * max(n.value, 1), dtype=np.int32)
        self._ck(self._lib.acvd_get_dual_mesh(self.ctx, _ptr(out), ctypes.byref(n)))
        return out[:3 * n.value].reshape(-1, 3)
