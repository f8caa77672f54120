"""Reference setters of the Python remesher that act before any solve: initial sampling
type, convergence cap, energy-driven loop, energy log, the remaining stored or refused
options, cluster sizes and a dual item's clusters (CPU), and two solves on the GPU."""
import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import remesh
from acvd_gb300 import synth


def _remesher(cls=acvd_gb300.IsotropicDiscreteRemeshing):
    r = cls.New()
    m = synth.icosphere(2, seed=0)
    r.SetInput(acvd_gb300.Surface(m.points, m.faces))
    r.SetNumberOfClusters(20)
    return r


def test_initial_sampling_types():
    r = _remesher()
    assert r.InitialSamplingType == 1                       # the reference's default
    r.SetInitialClustering(np.zeros(r.GetNumberOfItems(), dtype=np.int32))
    assert r.InitialSamplingType == 2                       # SetInitialClustering selects type 2
    r.SetInitialSamplingType(-1)
    assert r.InitialSamplingType == -1
    with pytest.raises(acvd_gb300.AcvdError) as err:
        r.SetInitialSamplingType(0)                         # vtkMath::Random's sequence: refused
    assert err.value.code == 5
    with pytest.raises(acvd_gb300.AcvdError):
        r.SetInitialSamplingType(3)
    assert r.InitialSamplingType == -1


def test_identity_sampling():
    np.testing.assert_array_equal(remesh.initial_identity_sampling(5, 3), [0, 1, 2, 3, 3])
    np.testing.assert_array_equal(remesh.initial_identity_sampling(3, 3), [0, 1, 2])
    for n, k in ((3, 4), (3, 0)):
        with pytest.raises(acvd_gb300.AcvdError):
            remesh.initial_identity_sampling(n, k)


def test_loop_options_and_refusals():
    r = _remesher(acvd_gb300.QIsotropicDiscreteRemeshing)
    assert r.MaxNumberOfConvergences == 1000000000
    r.SetMaxNumberOfConvergences(3)
    assert r.MaxNumberOfConvergences == 3
    r.SetMinimizeUsingEnergy(True)
    r.SetWriteToGlobalEnergyLog(0)
    for call in (lambda: r.SetMinimizeUsingEnergy(False), lambda: r.SetWriteToGlobalEnergyLog(1)):
        with pytest.raises(acvd_gb300.AcvdError) as err:
            call()
        assert err.value.code == 5


def test_cluster_sizes():
    r = _remesher()
    assert r.GetNumberOfItems() == 162
    with pytest.raises(acvd_gb300.AcvdError):
        r.GetClusterSize(0)
    r.Clustering = np.repeat(np.arange(20, dtype=np.int32), 9)[:162]
    assert [r.GetClusterSize(c) for c in (0, 17, 18, 19)] == [9, 9, 0, 0]
    assert sum(r.GetClusterSize(c) for c in range(20)) == 162
    with pytest.raises(IndexError):
        r.GetClusterSize(20)
    assert acvd_gb300.IsotropicDiscreteRemeshing.New().GetNumberOfItems() == 0


def test_remaining_reference_setters():
    """SetEdgeOptimization and SetOutputDirectory are stored (nothing on the path reads
    them); SetComputeAndSaveEnergy is SetWriteToGlobalEnergyLog; SetFileLoadSaveOption's
    interactive prompts are refused; FixClusteringToVoronoi is the reference's no-op."""
    r = _remesher()
    assert r.EdgeOptimization == 0 and r.OutputDirectory is None and r.FileLoadSaveOption == 0
    r.SetEdgeOptimization(1)
    r.SetOutputDirectory("/tmp/out")
    r.SetComputeAndSaveEnergy(0)
    r.SetFileLoadSaveOption(0)
    assert r.EdgeOptimization == 1 and r.OutputDirectory == "/tmp/out"
    for call in (lambda: r.SetComputeAndSaveEnergy(1), lambda: r.SetFileLoadSaveOption(1)):
        with pytest.raises(acvd_gb300.AcvdError) as err:
            call()
        assert err.value.code == 5
    r.Clustering = np.arange(162, dtype=np.int32) % 20
    before = r.Clustering.copy()
    assert r.FixClusteringToVoronoi() is None
    np.testing.assert_array_equal(r.Clustering, before)


def test_dual_item_neighbour_clusters():
    """A face's distinct clusters in its vertex order, unassigned vertices left out
    (vtkDiscreteRemeshing.h:956-1000)."""
    r = _remesher()
    with pytest.raises(acvd_gb300.AcvdError):
        r.GetDualItemNeighbourClusters(0)
    faces = r.Input.faces
    lab = np.full(162, 20, dtype=np.int32)          # all unassigned
    a, b, c = (int(v) for v in faces[5])
    lab[a], lab[b], lab[c] = 7, 3, 7
    r.Clustering = lab
    assert r.GetDualItemNeighbourClusters(5) == [7, 3]
    lab[b] = 20
    assert r.GetDualItemNeighbourClusters(5) == [7]
    lab[a] = lab[c] = 20
    assert r.GetDualItemNeighbourClusters(5) == []


def test_manifold_detection_needs_a_clustering():
    r = _remesher()
    with pytest.raises(acvd_gb300.AcvdError):
        r.DetectNonManifoldOutputVertices()


def test_engine_takes_the_convergence_cap():
    o = acvd_gb300.engine.Opts()
    assert [f[0] for f in o._fields_].index("max_convergences") == 3


@pytest.mark.gpu
def test_identity_sampling_solves_and_cap_stops_the_loop(oracle_lib):
    """Type -1 (item i seeds cluster i, the rest unassigned,
    Common/vtkUniformClustering.h:1139-1157) through a whole Remesh(): hole filling
    assigns every item and the clusters come out connected; and
    SetMaxNumberOfConvergences(1) ends a real solve at its first convergence."""
    m = synth.icosphere(3, seed=4)
    k = 40
    r = acvd_gb300.IsotropicDiscreteRemeshing.New()
    r.SetInput(acvd_gb300.Surface(m.points, m.faces))
    r.SetNumberOfClusters(k)
    r.SetInitialSamplingType(-1)
    r.Remesh()
    lab = np.asarray(r.GetClustering())
    assert np.all(lab < k)
    ev = oracle_lib.Port("iso", m.points, m.faces, k)
    ev.evaluate(lab, 1)
    assert ev.clean() == 0
    # with unconstrained initialisation the first convergence only switches the
    # placement on (:778-781), so an uncapped solve converges at least twice
    t = synth.torus(64, 32, seed=1)

    def qem(cap):
        r = acvd_gb300.QIsotropicDiscreteRemeshing.New()
        r.SetInput(acvd_gb300.Surface(t.points, t.faces))
        r.SetNumberOfClusters(k)
        r.SetUnconstrainedInitialization(1)
        if cap:
            r.SetMaxNumberOfConvergences(cap)
        r.Remesh()
        return r.Stats["convergences"]

    assert qem(None) > 1
    assert qem(1) == 1


@pytest.mark.gpu
def test_hole_filling_paths_agree(monkeypatch):
    """Hole filling (Common/vtkUniformClustering.h:552-633) over the unassigned items of
    type -1 sampling (K seeds, every other item unassigned): all rounds in one
    single-block launch, and one launch per colour class and round (ACVD_FILL_BLOCK_MAX=0,
    read when a context is created), give the same labels after a whole solve."""
    t = synth.torus(128, 64, seed=3)

    def run(block_max):
        if block_max is None:
            monkeypatch.delenv("ACVD_FILL_BLOCK_MAX", raising=False)
        else:
            monkeypatch.setenv("ACVD_FILL_BLOCK_MAX", str(block_max))
        r = acvd_gb300.QIsotropicDiscreteRemeshing.New()
        r.SetInput(acvd_gb300.Surface(t.points, t.faces))
        r.SetNumberOfClusters(300)
        r.SetInitialSamplingType(-1)
        r.Remesh()
        return np.asarray(r.GetClustering()).copy(), r.Stats

    lab_block, st_block = run(None)
    lab_rounds, st_rounds = run(0)
    assert np.all(lab_block < 300)
    assert np.array_equal(lab_block, lab_rounds)
    assert st_block["sweeps"] == st_rounds["sweeps"]
