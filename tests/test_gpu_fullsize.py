"""Parity at the benchmark configurations' full sizes (needs a GB300).

(a) Identical assignment at the sizes where FP32 item records and compensated
    sums have to hold: the converged GPU clustering of the ACVDQ torus 1024x512
    (K = 20,000, 26 items per cluster) and of a 1024^2 slice of the anisotropic
    heightfield (K = 12,500, 84 items per cluster), loaded back into the engine
    and into the oracle: cluster sizes, boundary-edge ids and dual triangles
    bit-exact; S, W, the quadric and the energies within 1e-6 of the oracle's FP64
    evaluation (the reference's load path, DiscreteRemeshing/vtkDiscreteRemeshing.h:
    915-932, and ReComputeStatistics, Common/vtkUniformClustering.h:353-403).
(b) Full runs against tests/golden/fullsize/ (the oracle's converged solves from the
    reference's own initial sampling, written by tests/golden/gen_fullsize.py): the
    GPU starts from the same initial clustering (SHA-256 of the labels), and the
    oracle's evaluation of its result lands within 0.1 % of the fixture's energy,
    with every cluster connected and every item assigned -- for the torus, the
    4096^2 heightfield (16.8 M items, K = 200,000) and all 256 meshes of the batch.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import batch as B
from acvd_gb300 import synth

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(__file__), "golden", "fullsize")
REL_ACC = 1e-6      # accumulators / energies vs FP64, identical assignment
REL_ENERGY = 1e-3   # converged energy vs the reference run


def _sha(lab):
    return hashlib.sha256(np.ascontiguousarray(lab, dtype=np.int32).tobytes()).hexdigest()


def _fixture(name):
    with open(os.path.join(FIX, name + ".json")) as f:
        return json.load(f)


def _solve(m, metric, k, grad, ind, pd, uinit, lab0):
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    e = acvd_gb300.Engine()
    e.set_mesh(m.points, m.faces, row, col, ev)
    e.set_metric(metric, ind, pd, grad)
    e.set_unconstrained_initialization(uinit)
    e.set_labels(k, lab0)
    e.minimize()
    lab = e.labels()
    return e, lab, (row, col, ev)


def _initial(m, metric, k, grad, ind):
    row, col, _ = acvd_gb300.build_topology(m.n_points, m.faces)
    w = acvd_gb300.vertex_weights(metric, m.points, m.faces, ind, grad)
    return acvd_gb300.initial_sampling(row, col, w, k)


def _rel(a, b, scale):
    scale = np.maximum(scale, 1e-300)
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)) / scale))


SLICES = [
    # name, generator, metric, K, gradation, unconstrained init
    ("torus_1024x512_qem", lambda: synth.torus(1024, 512, seed=0), "qem", 20000, 1.5, 1),
    ("heightfield_1024_aniso", lambda: synth.heightfield(1024, seed=0), "aniso", 12500, 1.5, 0),
]


@pytest.mark.parametrize("case", SLICES, ids=[c[0] for c in SLICES])
def test_identical_assignment_full_size(oracle_lib, case):
    name, mk, metric, k, grad, uinit = case
    m = mk()
    ind = m.indicator
    pd = m.principal_dirs if metric == "aniso" else None
    lab0 = _initial(m, metric, k, grad, ind)
    e, lab, (row, col, ev) = _solve(m, metric, k, grad, ind, pd, uinit, lab0)
    assert np.all(lab < k)
    # the converged clustering, loaded back (placement on, as the reference loads one)
    e.set_labels(k, lab)
    cl = e.clusters()
    p = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind, pd)
    p.evaluate(lab, 1)
    ref = p.clusters()
    np.testing.assert_array_equal(cl["size"], np.bincount(lab, minlength=k))
    np.testing.assert_array_equal(cl["size"], ref["size"])
    assert _rel(cl["W"], ref["W"], np.abs(ref["W"])) < REL_ACC
    assert _rel(cl["S"], ref["S"], np.linalg.norm(ref["S"], axis=1, keepdims=True)) < REL_ACC
    assert _rel(cl["Q"], ref["Q"], np.max(np.abs(ref["Q"]), axis=1, keepdims=True)) < REL_ACC
    assert _rel(cl["energy"], ref["energy"], np.abs(ref["energy"])) < REL_ACC
    e_ref = p.global_energy()
    assert abs(cl["energy_total"] - e_ref) < REL_ACC * abs(e_ref)
    # boundary edges in the reference's edge ids, and the dual mesh, bit for bit
    want = np.nonzero(lab[ev[:, 0]] != lab[ev[:, 1]])[0]
    np.testing.assert_array_equal(e.boundary_edges(), want)
    tris, _ = p.dual_mesh()
    np.testing.assert_array_equal(e.dual_mesh(), tris)
    e.close()


FULL = [
    ("torus_1024x512_qem", lambda: synth.torus(1024, 512, seed=0)),
    ("heightfield_4096_aniso", lambda: synth.heightfield(4096, seed=0)),
]


@pytest.mark.parametrize("case", FULL, ids=[c[0] for c in FULL])
def test_full_size_energy_against_fixture(oracle_lib, case):
    name, mk = case
    fx = _fixture(name)
    m = mk()
    metric, k, grad, uinit = fx["metric"], fx["clusters"], fx["gradation"], fx["unconstrained_init"]
    ind = m.indicator
    pd = m.principal_dirs if metric == "aniso" else None
    lab0 = _initial(m, metric, k, grad, ind)
    assert _sha(lab0) == fx["labels0_sha256"], "initial clustering differs from the reference's sampling"
    e, lab, _ = _solve(m, metric, k, grad, ind, pd, uinit, lab0)
    e.close()
    assert np.all(lab < k), "unassigned items left"
    ev = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind, pd)
    ev.evaluate(lab, 1)
    e_gpu = ev.global_energy()
    e_ref = fx["reference_energy"]
    assert e_gpu <= e_ref + REL_ENERGY * abs(e_ref), (e_gpu, e_ref)
    assert ev.clean() == 0, "disconnected clusters"


def test_batch_every_mesh_against_fixture(oracle_lib):
    fx = _fixture("batch_256_qem")
    specs = synth.batch_specs(len(fx["meshes"]), 0)
    b = B.batch_from_specs(specs, fx["metric"], fx["gradation"], fx["items_per_cluster"])
    e, _ = B.run_on_gpu(b, unconstrained_init=fx["unconstrained_init"])
    packed = e.labels()
    e.close()
    worst = -1.0
    for g, ref in enumerate(fx["meshes"]):
        m = b.meshes[g]
        assert int(b.ks[g]) == ref["clusters"]
        assert _sha(b.mesh_labels(b.labels0, g)) == ref["labels0_sha256"], g
        lab = b.mesh_labels(packed, g)
        assert np.all(lab < ref["clusters"]), g
        ev = oracle_lib.Port(fx["metric"], m.points, m.faces, ref["clusters"], fx["gradation"])
        ev.evaluate(lab, 1)
        e_gpu = ev.global_energy()
        rel = (e_gpu - ref["reference_energy"]) / abs(ref["reference_energy"])
        worst = max(worst, rel)
        assert rel <= REL_ENERGY, (g, e_gpu, ref["reference_energy"])
        assert ev.clean() == 0, g
