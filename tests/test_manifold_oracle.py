"""The oracle's restatement of the ForceManifold and FixMeshBoundaries steps
(DiscreteRemeshing/vtkDiscreteRemeshing.h:165-383, 426-579, 937-950;
Common/vtkSurfaceBase.cxx:259-315 IsVertexManifold) on the CPU: manifoldness of
closed and open meshes, the detection pass's bookkeeping, the loop's end state and
the boundary passes' counts.  The GPU side is compared with it in
test_gpu_manifold.py."""
import numpy as np

import acvd_gb300
from acvd_gb300 import synth


def test_vertex_manifold_closed_and_open(oracle_lib):
    m = synth.torus(30, 14, seed=2)
    p = oracle_lib.Port("qem", m.points, m.faces, 50, 0.0)
    p.init(None)
    _, inp = p.manifold_flags()
    assert inp.all()                          # a closed surface: every vertex manifold
    h = synth.heightfield(20, seed=1)
    p = oracle_lib.Port("qem", h.points, h.faces, 30, 0.0)
    p.init(None)
    _, inp = p.manifold_flags()
    row, col, ev = acvd_gb300.build_topology(h.n_points, h.faces)
    # boundary vertices (an edge with one face) fail IsVertexManifold, the others pass
    faces_per_edge = {}
    for f in h.faces:
        for a, b in ((f[0], f[1]), (f[1], f[2]), (f[2], f[0])):
            key = (min(a, b), max(a, b))
            faces_per_edge[key] = faces_per_edge.get(key, 0) + 1
    on_boundary = np.zeros(h.n_points, dtype=bool)
    for (a, b), n in faces_per_edge.items():
        if n == 1:
            on_boundary[a] = on_boundary[b] = True
    np.testing.assert_array_equal(inp == 0, on_boundary)


def test_detection_pass_bookkeeping(oracle_lib):
    m = synth.torus(60, 30, seed=1)
    k = 600
    p = oracle_lib.Port("qem", m.points, m.faces, k, 0.0)
    p.init(None)
    p.fill_holes()
    before = p.labels()
    dual, _ = p.manifold_flags()
    n = p.detect_nonmanifold()
    after = p.labels()
    frozen = p.frozen()
    assert n == int((dual == 0).sum()) > 0    # closed input: every failing vertex is an issue
    added = p.k - k
    assert 0 < added <= n
    moved = np.nonzero(before != after)[0]
    assert moved.size == added                # each new cluster takes one item
    assert set(after[moved]) == set(range(k, p.k))
    assert not frozen[k:].any()               # new clusters are free
    assert not frozen[np.nonzero(dual == 0)[0]].any()


def test_loop_ends_without_issue(oracle_lib):
    m = synth.torus(60, 30, seed=1)
    p = oracle_lib.Port("qem", m.points, m.faces, 450, 0.0)
    p.init(None)
    p.fill_holes()
    rounds = p.force_manifold(50)
    assert rounds >= 1
    assert p.detect_nonmanifold() == 0


def test_boundary_fixing_counts(oracle_lib):
    h = synth.heightfield(30, seed=4)
    p = oracle_lib.Port("qem", h.points, h.faces, 60, 0.0)
    p.init(None)
    p.run()
    lab = p.labels()
    pts, tri = p.fix_mesh_boundaries()
    # pass 1: one new vertex per boundary edge between two clusters
    cnt = {}
    for f in h.faces:
        for a, b in ((f[0], f[1]), (f[1], f[2]), (f[2], f[0])):
            key = (min(a, b), max(a, b))
            cnt[key] = cnt.get(key, 0) + 1
    split = sum(1 for (a, b), n in cnt.items() if n == 1 and lab[a] != lab[b])
    assert pts.shape[0] == split > 0
    assert np.all(tri[:split, 0] == 60 + np.arange(split))
    assert tri.max() < 60 + split
    # the new vertices are float values on the boundary edges' midpoints
    np.testing.assert_array_equal(pts, pts.astype(np.float32).astype(np.float64))
    # closed mesh: nothing to add
    m = synth.torus(30, 14, seed=2)
    q = oracle_lib.Port("qem", m.points, m.faces, 40, 0.0)
    q.init(None)
    q.run()
    a, b = q.fix_mesh_boundaries()
    assert a.shape[0] == 0 and b.shape[0] == 0
