"""Batched clustering: many meshes packed into one CSR (acvd_set_batch).

The meshes are independent; vertex, face and edge ranges follow one another,
labels are offset so that mesh m owns clusters [k_off[m], k_off[m+1]).  The CPU
analogue in the reference runs one remesher per mesh on host threads
(DiscreteRemeshing/Examples/VolumeAnalysis.cxx:153-240).
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import engine as _eng
from . import synth


@dataclasses.dataclass
class Batch:
    meshes: list
    ks: np.ndarray            # clusters per mesh
    points: np.ndarray
    faces: np.ndarray
    v_off: np.ndarray         # int64, n_mesh + 1
    f_off: np.ndarray
    k_off: np.ndarray         # int32, n_mesh + 1
    labels0: np.ndarray       # packed initial labels (null = K_total)
    k_total: int
    metric: str
    gradation: float
    indicator: np.ndarray | None

    @property
    def n_mesh(self) -> int:
        return len(self.meshes)

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    def mesh_labels(self, packed: np.ndarray, m: int) -> np.ndarray:
        """Labels of mesh m in its own numbering (null = its own K)."""
        lab = packed[self.v_off[m]:self.v_off[m + 1]].astype(np.int64) - self.k_off[m]
        k = int(self.ks[m])
        lab[(lab < 0) | (lab >= k)] = k
        return lab.astype(np.int32)


def build_batch(meshes, ks, metric: str = "qem", gradation: float = 0.0) -> Batch:
    ks = np.asarray(ks, dtype=np.int64)
    v_off = np.zeros(len(meshes) + 1, dtype=np.int64)
    f_off = np.zeros(len(meshes) + 1, dtype=np.int64)
    k_off = np.zeros(len(meshes) + 1, dtype=np.int64)
    for m, mesh in enumerate(meshes):
        v_off[m + 1] = v_off[m] + mesh.n_points
        f_off[m + 1] = f_off[m] + mesh.n_faces
        k_off[m + 1] = k_off[m] + ks[m]
    k_total = int(k_off[-1])
    points = np.concatenate([m.points for m in meshes], axis=0)
    faces = np.concatenate([m.faces.astype(np.int64) + v_off[i] for i, m in enumerate(meshes)], axis=0)
    use_ind = gradation != 0.0 if metric == "aniso" else gradation > 0.0
    ind = np.concatenate([m.indicator for m in meshes]) if use_ind else None
    labels = np.empty(int(v_off[-1]), dtype=np.int32)
    for i, mesh in enumerate(meshes):
        row, col, _ = _eng.build_topology(mesh.n_points, mesh.faces)
        w = _eng.vertex_weights(metric, mesh.points, mesh.faces, mesh.indicator if use_ind else None, gradation)
        lab = _eng.initial_sampling(row, col, w, int(ks[i])).astype(np.int64)
        lab = np.where(lab >= ks[i], k_total, lab + k_off[i])
        labels[v_off[i]:v_off[i + 1]] = lab
    return Batch(list(meshes), ks, points, faces.astype(np.int32), v_off, f_off, k_off.astype(np.int32), labels,
                 k_total, metric, gradation, ind)


def spec_items(spec) -> int:
    """Vertex count of a batch mesh spec (kind, size parameters) without building it."""
    kind, kw = spec
    if kind == "icosphere":
        return 10 * 4 ** kw["level"] + 2
    if kind == "torus":
        return kw["nu"] * kw["nv"]
    return kw["n"] * kw["n"]


def spec_faces(spec) -> int:
    """Triangle count of a batch mesh spec without building it."""
    kind, kw = spec
    if kind == "icosphere":
        return 20 * 4 ** kw["level"]
    if kind == "torus":
        return 2 * kw["nu"] * kw["nv"]
    return 2 * (kw["n"] - 1) ** 2


def mesh_from_spec(spec, with_curvature: bool):
    kind, kw = spec
    if kind == "icosphere":
        return synth.icosphere(kw["level"], seed=kw["seed"], with_curvature=with_curvature)
    if kind == "torus":
        return synth.torus(kw["nu"], kw["nv"], seed=kw["seed"], with_curvature=with_curvature)
    return synth.heightfield(kw["n"], seed=kw["seed"], with_curvature=with_curvature)


def batch_from_specs(specs, metric: str = "qem", gradation: float = 0.0, items_per_cluster: int = 20) -> Batch:
    """The batch of the given mesh specs, K = vertices / items_per_cluster per mesh."""
    curv = gradation != 0.0 or metric == "aniso"
    meshes = [mesh_from_spec(s, curv) for s in specs]
    ks = [max(1, m.n_points // items_per_cluster) for m in meshes]
    return build_batch(meshes, ks, metric, gradation)


def synthetic_batch(n_meshes: int = 256, seed: int = 0, lo: int = 2000, hi: int = 500000,
                    items_per_cluster: int = 20, metric: str = "qem", gradation: float = 0.0) -> Batch:
    """The batched workload: generator type uniform over icosphere / torus / heightfield,
    vertex count log-uniform in [lo, hi], K = vertices / 20 per mesh."""
    return batch_from_specs(synth.batch_specs(n_meshes, seed, lo, hi), metric, gradation, items_per_cluster)


def run_on_gpu(b: Batch, engine: "_eng.Engine | None" = None, unconstrained_init: int = 1):
    """Packs the batch into one context and minimises every mesh in the same sweeps."""
    e = engine or _eng.Engine()
    row, col, ev = _eng.build_topology(b.n_points, b.faces)
    e.set_mesh(b.points, b.faces, row, col, ev)
    e.set_batch(b.v_off, b.k_off)
    e.set_metric(b.metric, b.indicator, None, b.gradation)
    e.set_unconstrained_initialization(unconstrained_init)
    e.set_labels(b.k_total, b.labels0)
    stats = e.minimize()
    return e, stats
