"""ORACLE / TEST INFRASTRUCTURE ONLY.

ctypes front-end over the two CPU checkers built by oracle/Makefile:

* ``Port``  -- the C++ restatement (oracle/acvd_port.cpp, library _build/libacvd_port.so)
* ``Ref``   -- the reference's own headers compiled against the VTK shim
               (oracle/ref_driver.cpp, library _ref/libacvdref.so; only where the
               reference tree is present)

Both expose the same methods.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of bench.py use this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libacvd_port.so")
REF_LIB = os.path.join(HERE, "_ref", "libacvdref.so")
REF_MT_LIB = os.path.join(HERE, "_ref", "libacvdref_mt.so")
REF_ROOT = os.environ.get("ACVD_REFERENCE_ROOT", "/root/reference")

METRICS = {"iso": 0, "qem": 1, "aniso": 2}

_P = ctypes.c_void_p
_pd = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_pf = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_pi = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(ref: bool | None = None) -> None:
    """Build the restatement (always) and the reference library (when the
    reference tree is present, or when ``ref`` is True)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    if ref is None:
        ref = os.path.isdir(os.path.join(REF_ROOT, "Common"))
    if ref:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={REF_ROOT}"],
                              stderr=subprocess.DEVNULL)


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def _bind(lib, prefix):
    def f(name, res, *args):
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = list(args)
        return fn
    fns = {
        "create": f("create", _P, ctypes.c_int, ctypes.c_longlong, _pd, ctypes.c_longlong, _pi,
                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int),
        "destroy": f("destroy", None, _P),
        "set_option": f("set_option", ctypes.c_int, _P, ctypes.c_char_p, ctypes.c_double),
        "init": f("init", None, _P, ctypes.c_void_p),
        "run": f("run", ctypes.c_double, _P),
        "get_labels": f("get_labels", None, _P, _pi),
        "set_labels": f("set_labels", None, _P, _pi),
        "evaluate": f("evaluate", None, _P, _pi, ctypes.c_int),
        "global_energy": f("global_energy", ctypes.c_double, _P),
        "get_clusters": f("get_clusters", None, _P, _pd, _pd, _pd, _pd, _pd, _pi),
        "clean": f("clean", ctypes.c_int, _P),
        "fill_holes": f("fill_holes", ctypes.c_int, _P),
        "post_placement": f("post_placement", None, _P, ctypes.c_int, _pd),
        "curvature": f("curvature", None, _P, _pd, np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")),
        "set_fixed": f("set_fixed", None, _P, ctypes.c_int, _pi),
        "set_anchors": f("set_anchors", ctypes.c_int, _P, ctypes.c_int, _pi),
    }
    return fns


class _Base:
    _lib = None
    _prefix = ""
    _libpath = ""

    @classmethod
    def _load(cls):
        if cls._lib is None:
            if not os.path.exists(cls._libpath):
                raise RuntimeError(f"oracle library missing: {cls._libpath}")
            cls._lib = ctypes.CDLL(cls._libpath)
            cls._fns = _bind(cls._lib, cls._prefix)
            cls._extra(cls._lib)
        return cls._fns

    @classmethod
    def _extra(cls, lib):
        pass

    def __init__(self, metric: str, points: np.ndarray, faces: np.ndarray, k: int,
                 gradation: float = 0.0, indicator: np.ndarray | None = None,
                 principal_dirs: np.ndarray | None = None, level: int | None = None,
                 unconstrained_init: int = 0):
        self.f = self._load()
        self.metric = metric
        self.k = int(k)
        self.points = np.ascontiguousarray(points, dtype=np.float64)
        self.faces = np.ascontiguousarray(faces, dtype=np.int32)
        self.n = self.points.shape[0]
        self._ind = None if indicator is None else np.ascontiguousarray(indicator, dtype=np.float64)
        self._pd = None if principal_dirs is None else np.ascontiguousarray(principal_dirs, dtype=np.float32).reshape(-1)
        self.h = self.f["create"](METRICS[metric], self.n, self.points.reshape(-1), self.faces.shape[0],
                                  self.faces.reshape(-1),
                                  None if self._ind is None else self._ind.ctypes.data,
                                  None if self._pd is None else self._pd.ctypes.data,
                                  float(gradation), self.k)
        if level is not None:
            self.set_option("level", level)
        if unconstrained_init:
            self.set_option("unconstrained_init", unconstrained_init)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.f["destroy"](h)
            self.h = None

    def set_option(self, name: str, value: float) -> None:
        self.f["set_option"](self.h, name.encode(), float(value))

    def set_fixed(self, ids) -> None:
        """SetFixedClusters: cluster c < len(ids) holds vertex ids[c] (before init)."""
        a = np.ascontiguousarray(ids, dtype=np.int32)
        self._fixed = a
        self.f["set_fixed"](self.h, a.shape[0], a)

    def set_anchors(self, anchors) -> None:
        """QEM Cluster::AnchorItem of clusters 0 .. len(anchors)-1 (-1: none)."""
        a = np.ascontiguousarray(anchors, dtype=np.int32)
        if self.f["set_anchors"](self.h, a.shape[0], a) != 0:
            raise ValueError("anchor items exist for the QEM metric only")

    def init(self, initial: np.ndarray | None = None) -> None:
        if initial is None:
            self.f["init"](self.h, None)
        else:
            self._initial = np.ascontiguousarray(initial, dtype=np.int32)
            self.f["init"](self.h, self._initial.ctypes.data)

    def run(self) -> float:
        return float(self.f["run"](self.h))

    def labels(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.int32)
        self.f["get_labels"](self.h, out)
        return out

    def set_labels(self, lab: np.ndarray) -> None:
        self.f["set_labels"](self.h, np.ascontiguousarray(lab, dtype=np.int32))

    def evaluate(self, lab: np.ndarray, constrained: int = 1) -> None:
        self.f["evaluate"](self.h, np.ascontiguousarray(lab, dtype=np.int32), int(constrained))

    def global_energy(self) -> float:
        return float(self.f["global_energy"](self.h))

    def clusters(self) -> dict:
        k = self.k
        S = np.empty(3 * k); W = np.empty(k); Q = np.empty(9 * k); C = np.empty(3 * k); E = np.empty(k)
        sz = np.empty(k, dtype=np.int32)
        self.f["get_clusters"](self.h, S, W, Q, C, E, sz)
        return {"S": S.reshape(k, 3), "W": W, "Q": Q.reshape(k, 9), "centroid": C.reshape(k, 3),
                "energy": E, "size": sz}

    def clean(self) -> int:
        return int(self.f["clean"](self.h))

    def post_placement(self, level: int = 1) -> np.ndarray:
        """ACVD's quadric post-placement of the output vertices (ACVD.cxx:217-291) for
        the current clustering and cluster statistics (call evaluate first)."""
        out = np.empty((self.k, 3), dtype=np.float64)
        self.f["post_placement"](self.h, int(level), out.ravel())
        return out

    def curvature_range(self, v0: int, v1: int):
        """curvature() for the vertices [v0, v1) only (full-size outputs, others zero)."""
        ind = np.zeros(self.n, dtype=np.float64)
        pd = np.zeros(6 * self.n, dtype=np.float32)
        fn = self._lib.port_curvature_range
        fn.restype = None
        fn.argtypes = [_P, ctypes.c_longlong, ctypes.c_longlong, _pd,
                       np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")]
        fn(self.h, int(v0), int(v1), ind, pd)
        return ind, pd.reshape(-1, 6)

    def curvature(self):
        """Per-vertex curvature indicator (nV) and principal directions (nV x 6, float32)
        of the mesh, vtkCurvatureMeasure's polynomial fitting on the vertex 3-ring."""
        ind = np.empty(self.n, dtype=np.float64)
        pd = np.empty(6 * self.n, dtype=np.float32)
        self.f["curvature"](self.h, ind, pd)
        return ind, pd.reshape(-1, 6)

    def fill_holes(self) -> int:
        return int(self.f["fill_holes"](self.h))


class Port(_Base):
    _prefix = "port_"
    _libpath = PORT_LIB

    @classmethod
    def _extra(cls, lib):
        lib.port_get_items.argtypes = [_P, _pd, _pd, _pd]
        lib.port_get_items.restype = None
        lib.port_get_aniso_items.argtypes = [_P, _pf, _pf]
        lib.port_get_aniso_items.restype = None
        lib.port_connexity_problem.argtypes = [_P, ctypes.c_longlong, ctypes.c_int]
        lib.port_connexity_problem.restype = ctypes.c_int
        lib.port_topology.argtypes = [_P, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.port_topology.restype = ctypes.c_longlong
        lib.port_stats.argtypes = [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                   ctypes.POINTER(ctypes.c_longlong)]
        lib.port_stats.restype = None
        lib.port_dual_mesh.argtypes = [_P, ctypes.c_void_p, ctypes.c_void_p]
        lib.port_dual_mesh.restype = ctypes.c_longlong
        lib.port_detect_nonmanifold.argtypes = [_P, ctypes.POINTER(ctypes.c_int)]
        lib.port_detect_nonmanifold.restype = ctypes.c_int
        lib.port_get_frozen.argtypes = [_P, ctypes.c_void_p]
        lib.port_get_frozen.restype = None
        lib.port_manifold_flags.argtypes = [_P, ctypes.c_void_p, ctypes.c_void_p]
        lib.port_manifold_flags.restype = None
        lib.port_force_manifold.argtypes = [_P, ctypes.c_int]
        lib.port_force_manifold.restype = ctypes.c_int
        lib.port_set_frozen.argtypes = [_P, ctypes.c_void_p]
        lib.port_set_frozen.restype = None
        lib.port_minimize.argtypes = [_P]
        lib.port_minimize.restype = None
        lib.port_get_k.argtypes = [_P]
        lib.port_get_k.restype = ctypes.c_int
        lib.port_fix_mesh_boundaries.argtypes = [_P, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.POINTER(ctypes.c_longlong)]
        lib.port_fix_mesh_boundaries.restype = ctypes.c_longlong

    def items(self) -> dict:
        n = self.n
        V = np.empty(3 * n); W = np.empty(n); Q = np.empty(9 * n)
        self._lib.port_get_items(self.h, V, W, Q)
        d = {"value": V.reshape(n, 3), "weight": W, "quadric": Q.reshape(n, 9)}
        if self.metric == "aniso":
            T = np.empty(6 * n, dtype=np.float32); TX = np.empty(3 * n, dtype=np.float32)
            self._lib.port_get_aniso_items(self.h, T, TX)
            d["tensor"] = T.reshape(n, 6)
            d["tensor_x"] = TX.reshape(n, 3)
        return d

    def connexity_problem(self, item: int, cluster: int) -> int:
        return int(self._lib.port_connexity_problem(self.h, item, cluster))

    def topology(self):
        ne = int(self._lib.port_topology(self.h, None, None, None))
        ev = np.empty(2 * ne, dtype=np.int32)
        row = np.empty(self.n + 1, dtype=np.int32)
        col = np.empty(2 * ne, dtype=np.int32)
        self._lib.port_topology(self.h, ev.ctypes.data, row.ctypes.data, col.ctypes.data)
        return ev.reshape(ne, 2), row, col

    def stats(self) -> dict:
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        self._lib.port_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return {"loops": a.value, "convergences": b.value, "moves": c.value}

    def detect_nonmanifold(self) -> int:
        """DetectNonManifoldOutputVertices on the current clustering: the number of
        issues; new clusters added (self.k), IsClusterFreezed set (frozen())."""
        k = ctypes.c_int(0)
        n = int(self._lib.port_detect_nonmanifold(self.h, ctypes.byref(k)))
        self.k = int(k.value)
        return n

    def set_frozen(self, frozen: np.ndarray) -> None:
        self._frozen_in = np.ascontiguousarray(frozen, dtype=np.uint8)
        self._lib.port_set_frozen(self.h, self._frozen_in.ctypes.data)

    def minimize(self) -> None:
        """MinimizeEnergy again (connectivity constraint off first), keeping IsClusterFreezed."""
        self._lib.port_minimize(self.h)

    def frozen(self) -> np.ndarray:
        out = np.empty(self.k, dtype=np.uint8)
        self._lib.port_get_frozen(self.h, out.ctypes.data)
        return out

    def manifold_flags(self):
        """IsVertexManifold of every coarse-surface vertex (ForceManifold edges
        included) and of every input vertex."""
        d = np.empty(self.k, dtype=np.uint8)
        i = np.empty(self.n, dtype=np.uint8)
        self._lib.port_manifold_flags(self.h, d.ctypes.data, i.ctypes.data)
        return d, i

    def force_manifold(self, max_rounds: int = 1000) -> int:
        """Remesh()'s ForceManifold loop after run(): the passes that found issues."""
        r = int(self._lib.port_force_manifold(self.h, int(max_rounds)))
        self.k = int(self._lib.port_get_k(self.h))
        return r

    def fix_mesh_boundaries(self):
        """FixMeshBoundaries for the current clustering: (new points (n, 3), faces (m, 3))."""
        n = ctypes.c_longlong(0)
        nf = int(self._lib.port_fix_mesh_boundaries(self.h, None, None, ctypes.byref(n)))
        pts = np.empty((max(n.value, 1), 3))
        tri = np.empty((max(nf, 1), 3), dtype=np.int32)
        self._lib.port_fix_mesh_boundaries(self.h, pts.ctypes.data, tri.ctypes.data, ctypes.byref(n))
        return pts[:n.value], tri[:nf]

    def dual_mesh(self):
        nt = int(self._lib.port_dual_mesh(self.h, None, None))
        tris = np.empty(3 * max(nt, 1), dtype=np.int32)
        verts = np.empty(3 * self.k)
        self._lib.port_dual_mesh(self.h, tris.ctypes.data, verts.ctypes.data)
        return tris[:3 * nt].reshape(nt, 3), verts.reshape(self.k, 3)


class Ref(_Base):
    _prefix = "ref_"
    _libpath = REF_LIB

    @classmethod
    def _extra(cls, lib):
        lib.ref_process.argtypes = [_P, ctypes.c_void_p]
        lib.ref_process.restype = ctypes.c_double
        lib.ref_loops.argtypes = [_P]
        lib.ref_loops.restype = ctypes.c_int

    def process(self, initial: np.ndarray | None = None) -> float:
        """The reference's own ProcessClustering() (Init + InitSamples + MinimizeEnergy)."""
        if initial is None:
            return float(self._lib.ref_process(self.h, None))
        self._initial = np.ascontiguousarray(initial, dtype=np.int32)
        return float(self._lib.ref_process(self.h, self._initial.ctypes.data))

    def loops(self) -> int:
        return int(self._lib.ref_loops(self.h))


class RefThreaded(_Base):
    """The reference built with DOmultithread: vtkThreadedClustering (ACVDQP's
    engine) under the same driver.  Options "threads" and "pooling_ratio"."""
    _prefix = "refmt_"
    _libpath = REF_MT_LIB
    _lib = None

    @classmethod
    def _extra(cls, lib):
        lib.refmt_loops.argtypes = [_P]
        lib.refmt_loops.restype = ctypes.c_int

    def loops(self) -> int:
        return int(self._lib.refmt_loops(self.h))


def ref_threaded_available() -> bool:
    return os.path.exists(REF_MT_LIB)


def subdivide(points: np.ndarray, faces: np.ndarray, indicator: np.ndarray | None = None, timing: list | None = None):
    """vtkSurface::Subdivide restated (acvd_port.cpp ``port_subdivide``), with the
    parent interpolation of the indicator.  Returns (points (nV+nE, 3), faces (4 nF', 3),
    parent1 (nE), parent2 (nE), indicator (nV+nE) or None).  ``timing`` (a list) gets the
    seconds of the subdivision proper, after the edge table is built."""
    Port._load()
    lib = Port._lib
    fn = lib.port_subdivide
    fn.restype = ctypes.c_longlong
    fn.argtypes = [ctypes.c_longlong, _pd, ctypes.c_longlong, _pi, _pd, _pi, _pi, _pi, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    pts = np.ascontiguousarray(points, dtype=np.float64)
    tri = np.ascontiguousarray(faces, dtype=np.int32)
    nv, nf = pts.shape[0], tri.shape[0]
    ne = int(Port("iso", pts, tri, 1).topology()[0].shape[0])
    o_pts = np.empty(3 * (nv + ne))
    o_tri = np.empty(12 * max(nf, 1), dtype=np.int32)
    p1 = np.empty(max(ne, 1), dtype=np.int32)
    p2 = np.empty(max(ne, 1), dtype=np.int32)
    ind = o_ind = None
    if indicator is not None:
        ind = np.ascontiguousarray(indicator, dtype=np.float64)
        o_ind = np.empty(nv + ne)
    secs = ctypes.c_double(0.0)
    nt = int(fn(nv, pts.reshape(-1), nf, tri.reshape(-1), o_pts, o_tri, p1, p2,
                None if ind is None else ind.ctypes.data, None if o_ind is None else o_ind.ctypes.data,
                ctypes.addressof(secs)))
    if timing is not None:
        timing.append(secs.value)   # the subdivision proper, after the edge table is built
    return o_pts.reshape(-1, 3), o_tri[:3 * nt].reshape(-1, 3), p1[:ne], p2[:ne], o_ind
