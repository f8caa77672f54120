"""CUDA path against the oracle (needs a GB300).

(a) identical assignment: cluster sizes, boundary-edge set and dual-mesh
    triangles bit-exact; accumulators and energies within 1e-6 relative of the
    FP64 evaluation;
(b) full runs from the same initial clustering: the reference arithmetic's
    energy of the GPU clustering is within 0.1 % of the reference CPU run's
    converged energy, every cluster connected, nothing unassigned;
plus determinism (two runs bitwise identical) and the error paths.
"""
import glob
import os

import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import synth

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
REL_ACC = 1e-6      # accumulators / energies vs FP64
REL_ENERGY = 1e-3   # converged energy vs the reference run


def _load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


def _engine(points, faces, metric, ind, pd, grad, level=3, uinit=0):
    row, col, ev = acvd_gb300.build_topology(points.shape[0], faces)
    e = acvd_gb300.Engine()
    e.set_mesh(points, faces, row, col, ev)
    e.set_metric(metric, ind, pd, grad)
    e.set_level(level)
    e.set_unconstrained_initialization(uinit)
    return e, (row, col, ev)


def _rel(a, b, scale):
    return np.max(np.abs(np.asarray(a) - np.asarray(b)) / scale)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_identical_assignment(oracle_lib, path):
    g = _load(path)
    metric = str(g["metric"])
    k = int(g["k"])
    grad = float(g["gradation"])
    ind = g.get("indicator")
    pd = g.get("principal_dirs")
    e, (row, col, ev) = _engine(g["points"], g["faces"], metric, ind if (grad > 0 or metric == "aniso") else None,
                                pd, grad)
    lab = g["fixed_labels"]
    e.set_labels(k, lab)
    cl = e.clusters()
    sizes = np.bincount(lab[lab < k], minlength=k)
    np.testing.assert_array_equal(cl["size"], sizes)
    # accumulators vs the reference's FP64 sums
    assert _rel(cl["W"], g["fixed_W"], np.abs(g["fixed_W"])) < REL_ACC
    sc = np.linalg.norm(g["fixed_S"], axis=1, keepdims=True)
    assert _rel(cl["S"], g["fixed_S"], sc) < REL_ACC
    if metric != "iso":
        qs = np.max(np.abs(g["fixed_Q"]), axis=1, keepdims=True)
        assert _rel(cl["Q"], g["fixed_Q"], qs) < REL_ACC
    # energies (per cluster, and the total)
    assert _rel(cl["energy"], g["fixed_cluster_energy"], np.abs(g["fixed_cluster_energy"])) < REL_ACC
    assert abs(cl["energy_total"] - float(g["fixed_energy"])) < REL_ACC * abs(float(g["fixed_energy"]))
    # boundary edges: exact set, reference edge ids
    want = np.nonzero(lab[ev[:, 0]] != lab[ev[:, 1]])[0]
    np.testing.assert_array_equal(e.boundary_edges(), want)
    # dual mesh: exact triangles, order and corner order of the reference rule
    p = oracle_lib.Port(metric, g["points"], g["faces"], k, grad, ind if (grad > 0 or metric == "aniso") else None, pd)
    p.evaluate(lab, 1)
    tris, _ = p.dual_mesh()
    np.testing.assert_array_equal(e.dual_mesh(), tris)
    e.close()


RUNS = [
    # name, metric, mesh, K, gradation, unconstrained init, seeds-init
    ("iso_icosphere5_k1000_seeds", "iso", lambda: synth.icosphere(5, seed=0), 1000, 0.0, 0, True),
    ("iso_icosphere4_k200", "iso", lambda: synth.icosphere(4, seed=1), 200, 0.0, 0, False),
    ("qem_torus128x64_k600_g15", "qem", lambda: synth.torus(128, 64, seed=0), 600, 1.5, 1, False),
    ("qem_torus96x48_k300_g0", "qem", lambda: synth.torus(96, 48, seed=2), 300, 0.0, 0, False),
    ("aniso_heightfield64_k300_g15", "aniso", lambda: synth.heightfield(64, seed=0), 300, 1.5, 0, False),
]


def _evaluated(oracle_lib, metric, points, faces, k, grad, ind, pd, labels):
    """The reference's evaluation of a final clustering: Init, load the labels,
    ReComputeStatistics with the placement on (vtkDiscreteRemeshing.h:915-932).
    Both the CPU run's and the GPU run's clusterings are compared through it: the
    reference may stop at its first convergence, right after switching the
    placement on, with cluster records still computed without it."""
    ev = oracle_lib.Port(metric, points, faces, k, grad, ind, pd)
    ev.evaluate(labels, 1)
    return ev.global_energy()


def _run_case(oracle_lib, case):
    name, metric, mk, k, grad, uinit, seeds = case
    m = mk()
    ind = m.indicator if (grad > 0 or metric == "aniso") else None
    pd = m.principal_dirs if metric == "aniso" else None
    init = synth.seed_labels(m.n_points, k, seed=11) if seeds else None
    ref = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind, pd, unconstrained_init=uinit)
    ref.init(init)
    lab0 = ref.labels()
    ref.run()
    e_ref = _evaluated(oracle_lib, metric, m.points, m.faces, k, grad, ind, pd, ref.labels())
    e, topo = _engine(m.points, m.faces, metric, ind, pd, grad, uinit=uinit)
    e.set_labels(k, lab0)
    stats = e.minimize()
    lab = e.labels()
    return m, ind, pd, lab, stats, e_ref, e


@pytest.mark.parametrize("case", RUNS, ids=[c[0] for c in RUNS])
def test_full_run_energy_and_connectivity(oracle_lib, case):
    name, metric, mk, k, grad, uinit, seeds = case
    m, ind, pd, lab, stats, e_ref, e = _run_case(oracle_lib, case)
    assert np.all(lab < k), "unassigned items left"
    ev = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind, pd)
    ev.evaluate(lab, 1)
    e_gpu = ev.global_energy()
    # lower is better; within 0.1 % of the reference's converged energy
    assert e_gpu <= e_ref + REL_ENERGY * abs(e_ref), (e_gpu, e_ref, stats)
    # every cluster connected (the reference's CleanClustering finds nothing to split)
    assert ev.clean() == 0
    assert np.all(ev.clusters()["size"] > 0)
    # the GPU's own FP64 energy of its clustering agrees with the reference arithmetic
    assert abs(stats["energy"] - e_gpu) < REL_ACC * abs(e_gpu)
    e.close()


def test_determinism(oracle_lib):
    case = RUNS[2]
    out = []
    for _ in range(2):
        m, ind, pd, lab, stats, e_ref, e = _run_case(oracle_lib, case)
        out.append((lab, stats["energy"], stats["moves"], stats["sweeps"]))
        e.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    assert out[0][1:] == out[1][1:]


def test_remesh_api_end_to_end():
    m = synth.torus(96, 48, seed=4)
    mesh = acvd_gb300.Surface(m.points, m.faces)
    r = acvd_gb300.QIsotropicDiscreteRemeshing()
    r.SetInput(mesh)
    r.SetNumberOfClusters(300)
    r.SetSubsamplingThreshold(10)
    r.GetMetric().SetGradation(1.5)
    r.SetCurvatureInfo(m.indicator)
    r.SetUnconstrainedInitialization(1)
    r.Remesh()
    out = r.GetOutput()
    assert out.GetNumberOfPoints() == 300
    # closed torus: the coarse mesh is a closed surface of genus 1 when it is clean
    assert out.GetNumberOfCells() > 500
    lab = r.GetClustering()
    assert lab.shape == (m.n_points,) and lab.max() < 300
    # the ACVD driver's quadric post-placement moves the output vertices in place
    before = out.points.copy()
    placed = acvd_gb300.QuadricPostPlacement(r, 1)
    assert placed is out and np.all(np.isfinite(placed.points))
    assert not np.array_equal(before, placed.points)


def test_error_paths():
    m = synth.icosphere(3)
    e = acvd_gb300.Engine()
    with pytest.raises(acvd_gb300.AcvdError):
        e.minimize()                       # nothing set
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    e.set_mesh(m.points, m.faces, row, col, ev)
    with pytest.raises(acvd_gb300.AcvdError):
        e.set_metric("qem", None, None, 1.5)   # gradation without indicator
    with pytest.raises(acvd_gb300.AcvdError):
        e.set_metric("aniso", m.points[:, 0].copy(), None, 1.0)  # no principal directions
    e.set_metric("iso")
    with pytest.raises(acvd_gb300.AcvdError):
        e.set_labels(10, np.full(m.n_points, 11, dtype=np.int32))  # label > K
    r = acvd_gb300.AnisotropicDiscreteRemeshing()
    r.SetInput(acvd_gb300.Surface(m.points, m.faces))
    r.SetNumberOfClusters(500)                 # 642 < 10 * 500: needs subdivision, which the
    with pytest.raises(acvd_gb300.AcvdError):  # reference's aniso path cannot take
        r.Remesh()
    e.close()


def test_batched_meshes_match_individual_runs(oracle_lib):
    """Several meshes packed in one CSR: each converges like its own CPU run."""
    from acvd_gb300 import batch as B
    meshes = [synth.icosphere(3, seed=1), synth.torus(40, 24, seed=2), synth.heightfield(30, seed=3),
              synth.torus(64, 30, seed=4), synth.icosphere(4, seed=5)]
    ks = [m.n_points // 20 for m in meshes]
    b = B.build_batch(meshes, ks, "qem", 0.0)
    e, stats = B.run_on_gpu(b, unconstrained_init=1)
    packed = e.labels()
    mesh_e = e.mesh_energies()
    for m, mesh in enumerate(meshes):
        lab = b.mesh_labels(packed, m)
        k = int(ks[m])
        assert np.all(lab < k)
        ref = oracle_lib.Port("qem", mesh.points, mesh.faces, k, 0.0, unconstrained_init=1)
        ref.init(b.mesh_labels(b.labels0, m))
        ref.run()
        e_ref = _evaluated(oracle_lib, "qem", mesh.points, mesh.faces, k, 0.0, None, None, ref.labels())
        chk = oracle_lib.Port("qem", mesh.points, mesh.faces, k, 0.0)
        chk.evaluate(lab, 1)
        e_gpu = chk.global_energy()
        assert e_gpu <= e_ref + REL_ENERGY * abs(e_ref), (m, e_gpu, e_ref)
        assert chk.clean() == 0
        assert abs(mesh_e[m] - e_gpu) < REL_ACC * abs(e_gpu)
    e.close()


@pytest.mark.parametrize("case", [RUNS[0], RUNS[2], RUNS[4]], ids=[RUNS[i][0] for i in (0, 2, 4)])
def test_persistent_schedule_matches_per_phase_kernels(oracle_lib, case):
    """The persistent sweep kernel (one cooperative launch per phase of the
    minimisation) runs the same device functions in the same order as the
    per-phase kernels: the clusterings, energies and counts are identical."""
    name, metric, mk, k, grad, uinit, seeds = case
    m = mk()
    ind = m.indicator if (grad > 0 or metric == "aniso") else None
    pd = m.principal_dirs if metric == "aniso" else None
    init = synth.seed_labels(m.n_points, k, seed=11) if seeds else None
    ref = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind, pd, unconstrained_init=uinit)
    ref.init(init)
    lab0 = ref.labels()
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    out = []
    for persistent in (True, False):
        e = acvd_gb300.Engine(persistent=persistent)
        e.set_mesh(m.points, m.faces, row, col, ev)
        e.set_metric(metric, ind, pd, grad)
        e.set_unconstrained_initialization(uinit)
        e.set_labels(k, lab0)
        st = e.minimize()
        out.append((e.labels(), st))
        e.close()
    (lab_p, st_p), (lab_k, st_k) = out
    assert st_p["sweep_kernel_launches"] >= 1 and st_k["sweep_kernel_launches"] == 0
    np.testing.assert_array_equal(lab_p, lab_k)
    for key in ("sweeps", "moves", "relaxed_sweeps", "convergences", "candidates", "reverted"):
        assert st_p[key] == st_k[key], (key, st_p[key], st_k[key])
    assert st_p["energy"] == st_k["energy"]


@pytest.mark.parametrize("case", [RUNS[0], RUNS[2], RUNS[4]], ids=[RUNS[i][0] for i in (0, 2, 4)])
def test_device_loop_matches_host_loop(oracle_lib, case, monkeypatch):
    """The sweeps between convergence events looped on the device (graph WHILE node
    with decision kernels) take the host loop's decisions: the clusterings, energies
    and counts are identical."""
    name, metric, mk, k, grad, uinit, seeds = case
    m = mk()
    ind = m.indicator if (grad > 0 or metric == "aniso") else None
    pd = m.principal_dirs if metric == "aniso" else None
    init = synth.seed_labels(m.n_points, k, seed=11) if seeds else None
    ref = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind, pd, unconstrained_init=uinit)
    ref.init(init)
    lab0 = ref.labels()
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    out = []
    for host_loop in (True, False):
        if host_loop:
            monkeypatch.setenv("ACVD_HOST_LOOP", "1")
        else:
            monkeypatch.delenv("ACVD_HOST_LOOP", raising=False)
        e = acvd_gb300.Engine()
        e.set_mesh(m.points, m.faces, row, col, ev)
        e.set_metric(metric, ind, pd, grad)
        e.set_unconstrained_initialization(uinit)
        e.set_labels(k, lab0)
        st = e.minimize()
        out.append((e.labels(), st))
        e.close()
    (lab_h, st_h), (lab_d, st_d) = out
    np.testing.assert_array_equal(lab_h, lab_d)
    for key in ("sweeps", "moves", "relaxed_sweeps", "convergences", "candidates", "reverted"):
        assert st_h[key] == st_d[key], (key, st_h[key], st_d[key])
    assert st_h["energy"] == st_d["energy"]


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_post_placement_matches_reference(path):
    """ACVD's quadric post-placement (ACVD.cxx:217-291) of the reference's fixed
    assignment against the reference's own output (golden).  The face quadrics and the
    placement are FP64; the start points are the metric's cluster centroids, built from
    the float32 item records like every accumulator here, hence REL_ACC relative to the
    mesh size (a placement with fewer than three singular values keeps the start point
    along the unused directions)."""
    g = _load(path)
    metric = str(g["metric"])
    grad = float(g["gradation"])
    ind = g.get("indicator")
    e, _ = _engine(g["points"], g["faces"], metric, ind if (grad > 0 or metric == "aniso") else None,
                   g.get("principal_dirs"), grad)
    e.set_labels(int(g["k"]), g["fixed_labels"])
    scale = float(np.ptp(g["points"], axis=0).max())
    for level, key in ((1, "fixed_post1"), (3, "fixed_post3")):
        got = e.post_placement(level)
        np.testing.assert_allclose(got, g[key], rtol=0, atol=REL_ACC * scale)
    e.close()


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_curvature_matches_reference(path):
    """Per-vertex curvature (vtkCurvatureMeasure, polynomial fitting on the vertex
    3-ring) on the GPU against the reference's own output, bit for bit: the kernel is
    FP64 without FMA contraction and keeps the reference's operation order."""
    g = _load(path)
    row, col, ev = acvd_gb300.build_topology(g["points"].shape[0], g["faces"])
    e = acvd_gb300.Engine()
    e.set_mesh(g["points"], g["faces"], row, col, ev)
    ind, pd = e.compute_curvature()
    np.testing.assert_array_equal(ind, g["curv_indicator"])
    np.testing.assert_array_equal(pd, g["curv_dirs"])
    e.close()


@pytest.mark.parametrize("mk", [lambda: synth.torus(96, 48, seed=4), lambda: synth.icosphere(5, seed=2),
                                lambda: synth.heightfield(64, seed=3)], ids=["torus", "icosphere", "heightfield"])
def test_curvature_matches_oracle(oracle_lib, mk):
    m = mk()
    ref_ind, ref_pd = oracle_lib.Port("iso", m.points, m.faces, 10, 0.0).curvature()
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    e = acvd_gb300.Engine()
    e.set_mesh(m.points, m.faces, row, col, ev)
    ind, pd = e.compute_curvature()
    np.testing.assert_array_equal(ind, ref_ind)
    np.testing.assert_array_equal(pd, ref_pd)
    e.close()


def test_remesh_computes_curvature_like_the_reference(oracle_lib):
    """Remesh() without SetCurvatureInfo computes the curvature on the GPU (the
    reference's SamplingPreProcessing); it is bit-identical to the reference's, so the
    remesh equals one fed with the oracle's curvature."""
    m = synth.torus(96, 48, seed=6)
    ind, pd = oracle_lib.Port("qem", m.points, m.faces, 10, 0.0).curvature()
    outs = []
    for given in (True, False):
        r = acvd_gb300.QIsotropicDiscreteRemeshing()
        r.SetInput(acvd_gb300.Surface(m.points, m.faces))
        r.SetNumberOfClusters(300)
        r.GetMetric().SetGradation(1.5)
        r.SetUnconstrainedInitialization(1)
        if given:
            r.SetCurvatureInfo(ind)
        r.Remesh()
        outs.append(r.GetClustering())
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.parametrize("mk", [lambda: synth.torus(40, 20, seed=3), lambda: synth.icosphere(3, seed=1),
                                lambda: synth.heightfield(24, seed=5), synth.tetrahedron],
                         ids=["torus", "icosphere", "heightfield", "tetrahedron"])
def test_subdivision_matches_oracle(oracle_lib, mk):
    """vtkSurface::Subdivide on the GPU: points (float-rounded midpoints), faces, parents
    and the interpolated indicator bit-exact against the restatement, two levels."""
    m = mk()
    e = acvd_gb300.Engine()
    pts, tri = m.points, m.faces
    ind = np.linspace(0.5, 2.0, m.n_points) ** 1.7
    for _ in range(2):
        row, col, ev = acvd_gb300.build_topology(pts.shape[0], tri)
        g = e.subdivide(pts, tri, row, col, ev, indicator=ind)
        o = oracle_lib.subdivide(pts, tri, ind)
        for a, b in zip(g, o):
            np.testing.assert_array_equal(a, b)
        pts, tri, ind = g[0], g[1], g[4]
    e.close()


def test_remesh_subdivides_like_the_reference(oracle_lib):
    """Remesh() on a mesh with fewer than SubsamplingThreshold x K vertices: two levels
    of subdivision (CheckSubsamplingRatio), the curvature of the original mesh
    interpolated to the new vertices, and a clustering of the subdivided mesh as good as
    the reference arithmetic's own run on it."""
    m = synth.icosphere(2, seed=3)                  # 162 vertices; 10 x 100 needs 2 levels
    k, grad = 100, 1.0
    r = acvd_gb300.QIsotropicDiscreteRemeshing()
    r.SetInput(acvd_gb300.Surface(m.points, m.faces))
    r.SetNumberOfClusters(k)
    r.GetMetric().SetGradation(grad)
    r.Remesh()
    assert r.NumberOfSubdivisionsBeforeClustering == 2
    assert r.OriginalInput.GetNumberOfPoints() == m.n_points
    # the mesh and indicator the reference would cluster
    ind0, _ = oracle_lib.Port("qem", m.points, m.faces, 10, 0.0).curvature()
    pts, tri, ind = m.points, m.faces, ind0
    for _ in range(2):
        pts, tri, _, _, ind = oracle_lib.subdivide(pts, tri, ind)
    sub = r.GetInput()
    np.testing.assert_array_equal(sub.points, pts)
    np.testing.assert_array_equal(sub.faces, tri)
    np.testing.assert_array_equal(r.Indicator, ind)
    assert sub.GetNumberOfPoints() >= 10 * k
    lab = r.GetClustering()
    assert lab.shape == (pts.shape[0],) and lab.max() < k
    ev = oracle_lib.Port("qem", pts, tri, k, grad, ind)
    ev.evaluate(lab, 1)
    e_gpu = ev.global_energy()
    assert ev.clean() == 0 and np.all(ev.clusters()["size"] > 0)
    ref = oracle_lib.Port("qem", pts, tri, k, grad, ind)
    ref.init(None)
    ref.run()
    e_ref = ref.global_energy()
    assert e_gpu <= e_ref + 0.02 * abs(e_ref), (e_gpu, e_ref)
    assert r.GetOutput().GetNumberOfPoints() == k


def test_subdivide_device_matches_host_call():
    """acvd_subdivide_device (device buffers, the context's stream, no allocation) gives
    the host call's outputs; an out-of-range vertex id is reported, not read."""
    torch = pytest.importorskip("torch")
    m = synth.torus(40, 20, seed=3)
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    ind = np.linspace(0.5, 2.0, m.n_points)
    e = acvd_gb300.Engine()
    ref = e.subdivide(m.points, m.faces, row, col, ev, indicator=ind)
    nv, nf, ne = m.n_points, m.faces.shape[0], ev.shape[0]
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).cuda()
    d = [t(m.points, np.float64), t(m.faces, np.int32), t(row, np.int32), t(col, np.int32), t(ev, np.int32),
         t(ind, np.float64)]
    o = [torch.empty((nv + ne, 3), dtype=torch.float64, device="cuda"),
         torch.empty((4 * nf, 3), dtype=torch.int32, device="cuda"),
         torch.empty(ne, dtype=torch.int32, device="cuda"), torch.empty(ne, dtype=torch.int32, device="cuda"),
         torch.empty(nv + ne, dtype=torch.float64, device="cuda")]
    work = torch.empty(e.subdivide_work_bytes(ne), dtype=torch.uint8, device="cuda")

    def run(tri):
        e.subdivide_device(nv, d[0].data_ptr(), nf, tri.data_ptr(), d[2].data_ptr(), d[3].data_ptr(), ne,
                           d[4].data_ptr(), d[5].data_ptr(), o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(),
                           o[3].data_ptr(), o[4].data_ptr(), work.data_ptr())
        torch.cuda.synchronize()
        return int(work[8 * ne:8 * ne + 4].view(torch.int32).item())

    assert run(d[1]) == 0
    for got, want in zip(o, ref):
        np.testing.assert_array_equal(got.cpu().numpy(), want)
    bad = d[1].clone()
    bad[5, 1] = nv + 7                         # a vertex that does not exist
    assert run(bad) == 1
    e.close()


@pytest.mark.parametrize("case", RUNS, ids=[c[0] for c in RUNS])
def test_split_evaluation_matches_fused_kernel(oracle_lib, case, monkeypatch):
    """The split evaluation (a screen pass over the colour class that settles the
    items with nothing to do, then the evaluation over the forwarded work list) takes
    every item's decision as the fused evaluation kernel does: forced on every class
    of a small mesh, the clustering, energy and counts equal the fused run's."""
    name, metric, mk, k, grad, uinit, seeds = case
    m = mk()
    ind = m.indicator if (grad > 0 or metric == "aniso") else None
    pd = m.principal_dirs if metric == "aniso" else None
    init = synth.seed_labels(m.n_points, k, seed=11) if seeds else None
    ref = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind, pd, unconstrained_init=uinit)
    ref.init(init)
    lab0 = ref.labels()
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    out = []
    for split_min in ("1", "0"):          # every class split / none split
        monkeypatch.setenv("ACVD_SPLIT_MIN", split_min)
        e = acvd_gb300.Engine()
        e.set_mesh(m.points, m.faces, row, col, ev)
        e.set_metric(metric, ind, pd, grad)
        e.set_unconstrained_initialization(uinit)
        e.set_labels(k, lab0)
        st = e.minimize()
        out.append((e.labels(), st))
        e.close()
    (lab_s, st_s), (lab_f, st_f) = out
    np.testing.assert_array_equal(lab_s, lab_f)
    assert st_s["energy"] == st_f["energy"]
    for key in ("sweeps", "moves", "relaxed_sweeps", "convergences", "candidates", "reverted", "boundary_items",
                "targets", "visited"):
        assert st_s[key] == st_f[key], (key, st_s[key], st_f[key])
    assert st_s["kernel_launches"] > st_f["kernel_launches"]


def test_plain_fp32_form_runs_through_the_same_abi(oracle_lib):
    """libacvd_gb300_plain (cluster sums in plain float32, no compensation) is the
    comparison form of the benchmark: same C ABI, a connected clustering within the
    0.1 % bar of the reference's converged energy on a small QEM torus."""
    case = RUNS[2]
    name, metric, mk, k, grad, uinit, seeds = case
    m = mk()
    ind = m.indicator
    ref = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind, unconstrained_init=uinit)
    ref.init(None)
    lab0 = ref.labels()
    ref.run()
    e_ref = _evaluated(oracle_lib, metric, m.points, m.faces, k, grad, ind, None, ref.labels())
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    e = acvd_gb300.Engine(plain=True)
    assert e._lib._name.endswith("libacvd_gb300_plain.so")
    e.set_mesh(m.points, m.faces, row, col, ev)
    e.set_metric(metric, ind, None, grad)
    e.set_unconstrained_initialization(uinit)
    e.set_labels(k, lab0)
    e.minimize()
    lab = e.labels()
    e.close()
    assert np.all(lab < k)
    chk = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind)
    chk.evaluate(lab, 1)
    assert chk.global_energy() <= e_ref + REL_ENERGY * abs(e_ref)
    assert chk.clean() == 0
