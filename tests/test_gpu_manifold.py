"""ForceManifold and FixMeshBoundaries on the GPU against the oracle (needs a GB300).

* one detection pass (DetectNonManifoldOutputVertices,
  DiscreteRemeshing/vtkDiscreteRemeshing.h:165-383) on the same clustering: the same
  number of issues, the same new labels and K, the same frozen set -- bit-exact;
* MinimizeEnergy with frozen clusters (vtkUniformClustering.h:912-915): no item leaves
  a frozen cluster, and the energy reached is as good as the reference arithmetic's
  own run with the same frozen set;
* the whole loop ends with no issue the reference would find;
* FixMeshBoundaries (:426-579): the same new vertices (bit-exact) and faces.
"""
import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import synth

pytestmark = pytest.mark.gpu

REL_ENERGY = 1e-3

MESHES = {
    "torus": lambda: synth.torus(60, 30, seed=1),
    "icosphere": lambda: synth.icosphere(3, seed=2),
    "heightfield": lambda: synth.heightfield(40, seed=3),
}


def _unconverged(oracle_lib, m, k, metric="qem"):
    """The reference's initial sampling with its holes filled: a clustering with
    plenty of non-manifold output vertices."""
    p = oracle_lib.Port(metric, m.points, m.faces, k, 0.0)
    p.init(None)
    p.fill_holes()
    return p


def _engine(m, metric="qem"):
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    e = acvd_gb300.Engine()
    e.set_mesh(m.points, m.faces, row, col, ev)
    e.set_metric(metric)
    return e


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("ratio", [3, 8])
def test_detection_pass_matches_oracle(oracle_lib, name, ratio):
    m = MESHES[name]()
    k = m.n_points // ratio
    p = _unconverged(oracle_lib, m, k)
    lab = p.labels()
    e = _engine(m)
    e.set_labels(k, lab)
    n_gpu = e.force_manifold_step()
    n_ref = p.detect_nonmanifold()
    # the torus has issues here; on the open heightfield every failing output vertex
    # holds a boundary vertex (itself non-manifold), which excuses it
    assert n_ref > 0 or name != "torus"
    assert n_gpu == n_ref
    assert e.k == p.k
    np.testing.assert_array_equal(e.labels(), p.labels())
    if n_ref:
        # (with no issue the reference leaves every cluster frozen; Remesh() stops there,
        # and the engine keeps its frozen set as it was)
        np.testing.assert_array_equal(e.frozen_clusters(), p.frozen())
    e.close()


def test_converged_clustering_has_no_issue(oracle_lib):
    m = MESHES["torus"]()
    k = 300
    p = oracle_lib.Port("qem", m.points, m.faces, k, 0.0)
    p.init(None)
    p.run()
    e = _engine(m)
    e.set_labels(k, p.labels())
    assert e.force_manifold_step() == 0 == p.detect_nonmanifold()
    assert e.k == k
    e.close()


def test_minimize_keeps_frozen_clusters(oracle_lib):
    m = MESHES["torus"]()
    k = 600
    p = _unconverged(oracle_lib, m, k)
    lab = p.labels()
    frozen = (np.arange(k) % 3 == 0).astype(np.uint8)
    e = _engine(m)
    e.set_labels(k, lab)
    e.set_frozen_clusters(frozen)
    np.testing.assert_array_equal(e.frozen_clusters(), frozen)
    e.minimize()
    out = e.labels()
    # items never leave a frozen cluster (hole filling may still add some)
    for c in np.nonzero(frozen)[0][:200]:
        assert np.all(out[lab == c] == c)
    p.set_frozen(frozen)
    p.minimize()
    ev = oracle_lib.Port("qem", m.points, m.faces, k, 0.0)
    ev.evaluate(out, 1)
    e_gpu, e_ref = ev.global_energy(), p.global_energy()
    assert e_gpu <= e_ref + REL_ENERGY * abs(e_ref), (e_gpu, e_ref)
    e.close()


@pytest.mark.parametrize("name", ["torus", "heightfield"])
def test_force_manifold_loop_ends_clean(oracle_lib, name):
    m = MESHES[name]()
    k = m.n_points // 4
    p = _unconverged(oracle_lib, m, k)
    e = _engine(m)
    e.set_labels(k, p.labels())
    passes = 0
    while e.force_manifold_step():
        e.minimize()
        passes += 1
        assert passes < 50
    assert e.k >= k and (passes >= 1 or name != "torus")
    # the reference's own detection finds nothing on the result
    chk = oracle_lib.Port("qem", m.points, m.faces, e.k, 0.0)
    chk.evaluate(e.labels(), 1)
    assert chk.detect_nonmanifold() == 0
    assert chk.clean() == 0
    e.close()


def test_remesh_force_manifold_and_boundary_fixing():
    m = MESHES["heightfield"]()
    r = acvd_gb300.QIsotropicDiscreteRemeshing()
    r.SetInput(acvd_gb300.Surface(m.points, m.faces))
    r.SetNumberOfClusters(150)
    r.SetSubsamplingThreshold(5)
    r.SetForceManifold(1)
    r.SetBoundaryFixing(1)
    r.Remesh()
    out = r.GetOutput()
    k = r.GetNumberOfClusters()
    assert k >= 150 and out.GetNumberOfPoints() > k       # boundary vertices appended
    assert out.faces.max() < out.GetNumberOfPoints()
    # the output points are the float values the reference's vtkPoints holds
    np.testing.assert_array_equal(out.points, out.points.astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("variant", ["heightfield", "heightfield_shuffled", "torus"])
@pytest.mark.parametrize("k", [40, 200])
def test_fix_mesh_boundaries_matches_oracle(oracle_lib, variant, k):
    m = MESHES["heightfield" if variant.startswith("heightfield") else variant]()
    pts, faces = m.points, m.faces
    if variant.endswith("shuffled"):
        # interior edges first: the reference's GetNumberOfBoundaries then skips pass 3
        faces = faces[np.random.default_rng(7).permutation(faces.shape[0])]
    p = oracle_lib.Port("qem", pts, faces, k, 0.0)
    p.init(None)
    p.run()
    row, col, ev = acvd_gb300.build_topology(pts.shape[0], faces)
    e = acvd_gb300.Engine()
    e.set_mesh(pts, faces, row, col, ev)
    e.set_metric("qem")
    e.set_labels(k, p.labels())
    g_pts, g_tri = e.fix_mesh_boundaries()
    r_pts, r_tri = p.fix_mesh_boundaries()
    np.testing.assert_array_equal(g_pts, r_pts)
    np.testing.assert_array_equal(g_tri, r_tri)
    if variant == "torus":
        assert g_pts.shape[0] == 0 and g_tri.shape[0] == 0
    else:
        assert g_pts.shape[0] > 0
    e.close()
