"""Fixed vertices and cleaning on the CUDA path against the oracle (needs a GB300).

ACVDQ's fixed vertices (DiscreteRemeshing/Examples/ACVDQ.cxx:327-334): SetFixedClusters
puts vertex ids[c] in cluster c, and the QEM metric's cluster c carries AnchorItem =
ids[c], so that its output vertex is that vertex, its energy W |p|^2 - 2 p.S, and a move
of the vertex out of it is never taken (vtkQEMetricForClustering.h:194-275).
(a) records: for one assignment, the anchored clusters' vertices equal the fixed
    vertices bit for bit and every cluster energy the reference arithmetic's to 1e-6;
(b) full runs: the fixed vertices stay in their clusters and in place in the coarse
    mesh, and the reference arithmetic's energy of the GPU clustering is within 0.1 %
    of the oracle's converged run with the same fixed vertices;
(c) CleanClustering alone: the labels after cleaning equal the oracle's bit for bit,
    with and without fixed vertices (a fixed vertex's component is the one kept).
"""
import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import synth
from acvd_gb300.remesh import QIsotropicDiscreteRemeshing, Surface

pytestmark = pytest.mark.gpu

REL_ACC = 1e-6
REL_ENERGY = 1e-3


def _fixed_ids(n, count, seed):
    return np.sort(np.random.default_rng(seed).choice(n, size=count, replace=False)).astype(np.int32)


def _engine(m, metric, ind, grad, uinit=0):
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    e = acvd_gb300.Engine()
    e.set_mesh(m.points, m.faces, row, col, ev)
    e.set_metric(metric, ind, None, grad)
    e.set_level(3)
    e.set_unconstrained_initialization(uinit)
    return e, (row, col, ev)


def _oracle(O, metric, m, k, grad, ind, fixed, uinit=0):
    p = O.Port(metric, m.points, m.faces, k, grad, ind, None, unconstrained_init=uinit)
    p.set_fixed(fixed)
    if metric == "qem":
        p.set_anchors(fixed)
    return p


def test_anchored_cluster_records(oracle_lib):
    m = synth.torus(80, 40, seed=1)
    nfix, k = 12, 312
    fixed = _fixed_ids(m.n_points, nfix, 7)
    run = _oracle(oracle_lib, "qem", m, k, 1.5, m.indicator, fixed, uinit=1)
    run.init(None)
    run.run()
    lab = run.labels()          # converged: the anchored clusters hold many vertices
    assert np.min(np.bincount(lab, minlength=k)[:nfix]) > 1
    p = _oracle(oracle_lib, "qem", m, k, 1.5, m.indicator, fixed)
    p.evaluate(lab, 1)
    want = p.clusters()
    e, _ = _engine(m, "qem", m.indicator, 1.5)
    e.set_labels(k, lab)
    e.set_fixed_clusters(fixed)
    e.set_anchor_items(fixed)
    cl = e.clusters()
    np.testing.assert_array_equal(cl["centroid"][:nfix], m.points[fixed])
    np.testing.assert_array_equal(want["centroid"][:nfix], m.points[fixed])
    scale = np.maximum(np.abs(want["energy"]), 1e-300)
    assert np.max(np.abs(cl["energy"] - want["energy"]) / scale) < REL_ACC
    assert abs(cl["energy_total"] - p.global_energy()) < REL_ACC * abs(p.global_energy())
    # cleared, the same clusters are placed freely, as the oracle places them
    e.set_anchor_items(None)
    free = e.clusters()
    q = oracle_lib.Port("qem", m.points, m.faces, k, 1.5, m.indicator)
    q.evaluate(lab, 1)
    want_free = q.clusters()
    assert np.max(np.abs(free["energy"] - want_free["energy"]) / np.maximum(np.abs(want_free["energy"]), 1e-300)) < REL_ACC
    assert not np.array_equal(free["centroid"][:nfix], m.points[fixed])
    e.close()


@pytest.mark.parametrize("mk,k,nfix,grad,uinit", [
    (lambda: synth.torus(96, 48, seed=2), 300, 16, 1.5, 1),
    (lambda: synth.heightfield(48, seed=3), 150, 9, 0.0, 0),
])
def test_fixed_vertices_run_vs_oracle(oracle_lib, mk, k, nfix, grad, uinit):
    m = mk()
    ind = m.indicator if grad > 0 else None
    fixed = _fixed_ids(m.n_points, nfix, k)
    K = k + nfix
    p = _oracle(oracle_lib, "qem", m, K, grad, ind, fixed, uinit)
    p.init(None)
    lab0 = p.labels()
    p.run()
    ref_lab = p.labels()
    np.testing.assert_array_equal(ref_lab[fixed], np.arange(nfix))
    ev = _oracle(oracle_lib, "qem", m, K, grad, ind, fixed)
    ev.evaluate(ref_lab, 1)
    e_ref = ev.global_energy()

    e, (row, col, _) = _engine(m, "qem", ind, grad, uinit)
    w = acvd_gb300.vertex_weights("qem", m.points, m.faces, ind, grad)
    lab_gpu0 = acvd_gb300.initial_sampling(row, col, w, K, fixed=fixed)
    np.testing.assert_array_equal(lab_gpu0, lab0)
    e.set_labels(K, lab_gpu0)
    e.set_fixed_clusters(fixed)
    e.set_anchor_items(fixed)
    stats = e.minimize()
    lab = e.labels()
    assert stats["unassigned"] == 0 and np.all(lab < K)
    np.testing.assert_array_equal(lab[fixed], np.arange(nfix))
    cl = e.clusters()
    np.testing.assert_array_equal(cl["centroid"][:nfix], m.points[fixed])
    ev2 = _oracle(oracle_lib, "qem", m, K, grad, ind, fixed)
    ev2.evaluate(lab, 1)
    e_gpu = ev2.global_energy()
    assert e_gpu <= e_ref + REL_ENERGY * abs(e_ref), (e_gpu, e_ref)
    e.close()


def test_remesh_keeps_fixed_vertices():
    """The Python mirror of ACVDQ's flow: SetFixedClusters, NumberOfClusters raised by
    the fixed count, GetCluster(i).AnchorItem; the fixed vertices are the first output
    vertices, unchanged (the check of ACVDQ.cxx:341-363)."""
    m = synth.torus(64, 32, seed=4)
    pts = m.points.astype(np.float32).astype(np.float64)   # a float vtkPoints input
    fixed = _fixed_ids(m.n_points, 10, 3)
    r = QIsotropicDiscreteRemeshing()
    r.SetInput(Surface(pts, m.faces))
    r.SetFixedClusters(fixed)
    r.SetNumberOfClusters(150 + len(fixed))
    for i, v in enumerate(fixed):
        r.GetCluster(i).AnchorItem = int(v)
    r.SetUnconstrainedInitialization(1)
    r.GetMetric().SetGradation(0.0)
    r.Remesh()
    out = r.GetOutput()
    np.testing.assert_array_equal(out.points[: len(fixed)], pts[fixed])
    np.testing.assert_array_equal(r.GetClustering()[fixed], np.arange(len(fixed)))


@pytest.mark.parametrize("union_tries", [None, 0])
@pytest.mark.parametrize("with_fixed", [False, True])
def test_clean_clustering_equals_oracle(oracle_lib, with_fixed, union_tries, monkeypatch):
    # the components by union-find (default), and by the min-id propagation it falls back
    # to when a link gives up (ACVD_UNION_TRIES=0, read when the engine is created)
    if union_tries is None:
        monkeypatch.delenv("ACVD_UNION_TRIES", raising=False)
    else:
        monkeypatch.setenv("ACVD_UNION_TRIES", str(union_tries))
    m = synth.icosphere(4, seed=3)
    rng = np.random.default_rng(5)
    k = 60
    lab = rng.integers(0, k - 1, size=m.n_points).astype(np.int32)   # many components per cluster
    # the reference never cleans the cluster whose first component starts at vertex 0
    # (its VisitedCluster test, vtkUniformClustering.h:463): give vertex 0 a cluster of its own
    lab[0] = k - 1
    fixed = np.array([int(np.flatnonzero(lab == c)[-1]) for c in range(8)], dtype=np.int32)
    p = oracle_lib.Port("iso", m.points, m.faces, k)
    if with_fixed:
        p.set_fixed(fixed)
    p.init(lab)
    n_ref = p.clean()
    want = p.labels()
    e, _ = _engine(m, "iso", None, 0.0)
    e.set_labels(k, lab)
    if with_fixed:
        e.set_fixed_clusters(fixed)
    n = e.clean_clustering()
    got = e.labels()
    assert n == n_ref and n > 0
    np.testing.assert_array_equal(got, want)
    if with_fixed:
        np.testing.assert_array_equal(got[fixed], np.arange(8))
    e.close()


def test_fixed_argument_errors():
    m = synth.torus(32, 16, seed=1)
    e, _ = _engine(m, "iso", None, 0.0)
    with pytest.raises(acvd_gb300.AcvdError):
        e.set_anchor_items(np.array([0, 1], dtype=np.int32))      # iso clusters have no anchor
    with pytest.raises(acvd_gb300.AcvdError):
        e.set_fixed_clusters(np.array([m.n_points], dtype=np.int32))
    e.set_labels(4, np.zeros(m.n_points, dtype=np.int32))
    with pytest.raises(acvd_gb300.AcvdError):
        e.set_fixed_clusters(np.arange(5, dtype=np.int32))       # more fixed vertices than clusters
    e.close()


@pytest.mark.parametrize("schedule", ["host_loop", "persistent"])
def test_fixed_vertices_same_under_every_schedule(oracle_lib, schedule, monkeypatch):
    """The anchored clusters run through the same device functions whatever drives the
    sweeps: the device-side loop (default), the host loop and the persistent kernel give
    bitwise the same clustering and energy."""
    m = synth.torus(96, 48, seed=2)
    k, nfix = 316, 16
    fixed = _fixed_ids(m.n_points, nfix, 300)
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    w = acvd_gb300.vertex_weights("qem", m.points, m.faces, m.indicator, 1.5)
    lab0 = acvd_gb300.initial_sampling(row, col, w, k, fixed=fixed)
    out = []
    for variant in ("default", schedule):
        if variant == "host_loop":
            monkeypatch.setenv("ACVD_HOST_LOOP", "1")
        else:
            monkeypatch.delenv("ACVD_HOST_LOOP", raising=False)
        e = acvd_gb300.Engine(persistent=(variant == "persistent"))
        e.set_mesh(m.points, m.faces, row, col, ev)
        e.set_metric("qem", m.indicator, None, 1.5)
        e.set_unconstrained_initialization(1)
        e.set_labels(k, lab0)
        e.set_fixed_clusters(fixed)
        e.set_anchor_items(fixed)
        st = e.minimize()
        out.append((e.labels(), st))
        e.close()
    (lab_a, st_a), (lab_b, st_b) = out
    np.testing.assert_array_equal(lab_a, lab_b)
    np.testing.assert_array_equal(lab_a[fixed], np.arange(nfix))
    assert st_a["energy"] == st_b["energy"] and st_a["sweeps"] == st_b["sweeps"]
