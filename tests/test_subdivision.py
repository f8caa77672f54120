"""Midpoint subdivision before clustering (vtkSurface::Subdivide,
Common/vtkSurface.cxx:605-677; vtkDiscreteRemeshing::CheckSubsamplingRatio,
DiscreteRemeshing/vtkDiscreteRemeshing.h:841-875; the indicator interpolation,
:731-745).  CPU: the oracle's restatement against a hand-worked case and the
counting identities of 1-to-4 subdivision; the C-ABI entry point is exported.
The GPU side is compared with the oracle in test_gpu_parity.py."""
import numpy as np

import acvd_gb300
from acvd_gb300 import synth


def test_tetrahedron_known_answer(oracle_lib):
    P = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    F = np.array([[0, 1, 2], [0, 3, 1], [0, 2, 3], [1, 3, 2]], dtype=np.int32)
    ind = np.array([1.0, 2.0, 4.0, 8.0])
    pts, tri, p1, p2, oind = oracle_lib.subdivide(P, F, ind)
    # edges in creation order: 01 12 20 03 31 23
    np.testing.assert_array_equal(p1, [0, 1, 2, 0, 3, 2])
    np.testing.assert_array_equal(p2, [1, 2, 0, 3, 1, 3])
    np.testing.assert_array_equal(pts[4:], [[.5, 0, 0], [.5, .5, 0], [0, .5, 0], [0, 0, .5], [.5, 0, .5],
                                            [0, .5, .5]])
    # face 0 = (0, 1, 2): children of 01 / 12 / 20 are 4 / 5 / 6
    np.testing.assert_array_equal(tri[:4], [[0, 4, 6], [4, 1, 5], [5, 2, 6], [4, 5, 6]])
    # face 3 = (1, 3, 2): children of 13 / 32 / 21 are 8 / 9 / 5
    np.testing.assert_array_equal(tri[12:], [[1, 8, 5], [8, 3, 9], [9, 2, 5], [8, 9, 5]])
    np.testing.assert_array_equal(oind, [1, 2, 4, 8, 1.5, 3, 2.5, 4.5, 5, 6])


def test_counts_and_float_rounding(oracle_lib):
    m = synth.torus(30, 14, seed=2)
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    ne = ev.shape[0]
    pts, tri, p1, p2, _ = oracle_lib.subdivide(m.points, m.faces)
    assert pts.shape == (m.n_points + ne, 3) and tri.shape == (4 * m.faces.shape[0], 3)
    # E' = 2E + 3F, and the Euler characteristic is unchanged (torus: 0)
    _, _, ev2 = acvd_gb300.build_topology(pts.shape[0], tri)
    assert ev2.shape[0] == 2 * ne + 3 * m.faces.shape[0]
    assert pts.shape[0] - ev2.shape[0] + tri.shape[0] == 0
    # every new vertex is the float nearest to its parents' midpoint
    mid = 0.5 * (m.points[p1] + m.points[p2])
    np.testing.assert_array_equal(pts[m.n_points:], mid.astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(pts[:m.n_points], m.points.astype(np.float32).astype(np.float64))
    # the parents are the edge list in the reference's numbering
    np.testing.assert_array_equal(np.stack([p1, p2], 1), ev)


def test_entry_point_exported():
    lib = acvd_gb300.engine.load()
    assert hasattr(lib, "acvd_subdivide")
