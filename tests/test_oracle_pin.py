"""The C++ restatement against the reference's own code, run live.

Only where the reference tree is present: the reference's clustering headers are
compiled unmodified against the VTK shim (oracle/Makefile target `ref`) and both
libraries run the same seeded inputs; every output must agree bit for bit.
"""
import numpy as np
import pytest

from acvd_gb300 import synth


def _need_ref(O):
    if not O.ref_available():
        pytest.skip("reference tree not present; golden fixtures cover this case")


CASES = [
    ("iso", lambda: synth.icosphere(4, seed=5), 120, 0.0, 0, False),
    ("iso", lambda: synth.torus(40, 20, seed=2), 60, 1.0, 0, False),
    ("iso", lambda: synth.heightfield(30, seed=4), 40, 0.0, 0, True),
    ("qem", lambda: synth.torus(80, 40, seed=1), 300, 1.5, 1, False),
    ("qem", lambda: synth.heightfield(32, seed=2), 80, 0.0, 1, True),
    ("qem", lambda: synth.icosphere(3, seed=9), 40, 0.0, 0, True),
    ("aniso", lambda: synth.heightfield(36, seed=6), 90, 1.5, 0, False),
    ("aniso", lambda: synth.torus(40, 24, seed=8), 70, 0.0, 0, True),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_restatement_equals_reference(oracle_lib, case):
    O = oracle_lib
    _need_ref(O)
    metric, mk, k, grad, uinit, seeds = CASES[case]
    m = mk()
    if metric == "aniso" and m.principal_dirs is None:
        pytest.skip("no principal directions")
    ind = m.indicator if (grad > 0 or metric == "aniso") else None
    pd = m.principal_dirs if metric == "aniso" else None
    initial = synth.seed_labels(m.n_points, k, seed=case) if seeds else None
    out = []
    for cls in (O.Port, O.Ref):
        o = cls(metric, m.points, m.faces, k, grad, ind, pd, unconstrained_init=uinit)
        o.init(initial)
        l0 = o.labels()
        o.run()
        out.append((l0, o.labels(), o.global_energy(), o.clusters()))
    (pl0, pl, pe, pc), (rl0, rl, re, rc) = out
    np.testing.assert_array_equal(pl0, rl0)
    np.testing.assert_array_equal(pl, rl)
    assert pe == re
    for key in ("S", "W", "Q", "centroid", "energy", "size"):
        np.testing.assert_array_equal(pc[key], rc[key])


def test_clean_and_fill_equal_reference(oracle_lib):
    O = oracle_lib
    _need_ref(O)
    m = synth.icosphere(3, seed=3)
    rng = np.random.default_rng(0)
    k = 30
    lab = rng.integers(0, k, size=m.n_points).astype(np.int32)   # many disconnected pieces
    res = []
    for cls in (O.Port, O.Ref):
        o = cls("iso", m.points, m.faces, k)
        o.init(lab)
        n_disc = o.clean()
        after_clean = o.labels()
        n_bad = o.fill_holes()
        res.append((n_disc, after_clean, n_bad, o.labels()))
    assert res[0][0] == res[1][0]
    np.testing.assert_array_equal(res[0][1], res[1][1])
    assert res[0][2] == res[1][2]
    np.testing.assert_array_equal(res[0][3], res[1][3])


@pytest.mark.parametrize("case", [0, 3, 6])
def test_post_placement_equals_reference(oracle_lib, case):
    """ACVD's quadric post-placement (ACVD.cxx:217-291): the restatement against the
    same loop over the reference's own vtkQuadricTools, bit for bit."""
    O = oracle_lib
    _need_ref(O)
    metric, mk, k, grad, uinit, seeds = CASES[case]
    m = mk()
    ind = m.indicator if (grad > 0 or metric == "aniso") else None
    pd = m.principal_dirs if metric == "aniso" else None
    r = O.Ref(metric, m.points, m.faces, k, grad, ind, pd, unconstrained_init=uinit)
    r.init(None)
    r.run()
    lab = r.labels()
    out = []
    for cls in (O.Port, O.Ref):
        p = cls(metric, m.points, m.faces, k, grad, ind, pd)
        p.evaluate(lab, 1)
        out.append((p.post_placement(1), p.post_placement(3)))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])



@pytest.mark.parametrize("case", range(len(CASES)))
def test_curvature_equals_reference(oracle_lib, case):
    """vtkCurvatureMeasure (Common/vtkCurvatureMeasure.cxx, compiled unmodified against
    the shim) and the restatement, bit for bit."""
    O = oracle_lib
    _need_ref(O)
    metric, mk, k, grad, uinit, seeds = CASES[case]
    m = mk()
    a = O.Port(metric, m.points, m.faces, k, 0.0).curvature()
    b = O.Ref(metric, m.points, m.faces, k, 0.0).curvature()
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


FIXED_CASES = [
    ("qem", lambda: synth.torus(80, 40, seed=1), 300, 1.5, 1, 12),
    ("qem", lambda: synth.heightfield(32, seed=2), 80, 0.0, 0, 5),
    ("iso", lambda: synth.icosphere(4, seed=5), 120, 0.0, 0, 9),
]


def _fixed_ids(n, count, seed):
    return np.sort(np.random.default_rng(seed).choice(n, size=count, replace=False)).astype(np.int32)


@pytest.mark.parametrize("case", range(len(FIXED_CASES)))
def test_fixed_vertices_equal_reference(oracle_lib, case):
    """Fixed vertices as ACVDQ.cxx:327-334 sets them (SetFixedClusters, and for QEM
    the clusters' AnchorItem): initial sampling, converged clustering, energies and
    cluster records bit for bit; the anchored clusters' centroids are their vertices."""
    O = oracle_lib
    _need_ref(O)
    metric, mk, k, grad, uinit, nfix = FIXED_CASES[case]
    m = mk()
    ind = m.indicator if grad > 0 else None
    fixed = _fixed_ids(m.n_points, nfix, 100 + case)
    out = []
    for cls in (O.Port, O.Ref):
        o = cls(metric, m.points, m.faces, k + nfix, grad, ind, None, unconstrained_init=uinit)
        o.set_fixed(fixed)
        if metric == "qem":
            o.set_anchors(fixed)
        o.init(None)
        l0 = o.labels()
        o.run()
        out.append((l0, o.labels(), o.global_energy(), o.clusters()))
    (pl0, pl, pe, pc), (rl0, rl, re, rc) = out
    np.testing.assert_array_equal(pl0, rl0)
    np.testing.assert_array_equal(pl0[fixed], np.arange(nfix))
    np.testing.assert_array_equal(pl, rl)
    assert pe == re
    for key in ("S", "W", "Q", "centroid", "energy", "size"):
        np.testing.assert_array_equal(pc[key], rc[key])
    np.testing.assert_array_equal(pl[fixed], np.arange(nfix))
    if metric == "qem":
        np.testing.assert_array_equal(pc["centroid"][:nfix], m.points[fixed])


def test_clean_with_fixed_items_equals_reference(oracle_lib):
    """CleanClustering keeps the component holding a cluster's fixed item, however
    small (vtkUniformClustering.h:439-447)."""
    O = oracle_lib
    _need_ref(O)
    m = synth.icosphere(3, seed=3)
    rng = np.random.default_rng(1)
    k = 30
    lab = rng.integers(0, k, size=m.n_points).astype(np.int32)
    fixed = np.array([int(np.flatnonzero(lab == c)[-1]) for c in range(6)], dtype=np.int32)
    res = []
    for cls in (O.Port, O.Ref):
        o = cls("iso", m.points, m.faces, k)
        o.set_fixed(fixed)
        o.init(lab)
        n_disc = o.clean()
        res.append((n_disc, o.labels()))
    assert res[0][0] == res[1][0]
    np.testing.assert_array_equal(res[0][1], res[1][1])
    np.testing.assert_array_equal(res[0][1][fixed], np.arange(6))


THREADED = [
    ("iso", lambda: synth.icosphere(4, seed=5), 120, 0.0, 0),
    ("qem", lambda: synth.torus(128, 64, seed=0), 600, 1.5, 1),
    ("aniso", lambda: synth.heightfield(48, seed=6), 120, 1.5, 0),
]


@pytest.mark.parametrize("case", range(len(THREADED)))
@pytest.mark.parametrize("threads", [1, 4])
def test_threaded_restatement_lands_with_the_reference(oracle_lib, case, threads):
    """ACVDQP (vtkThreadedClustering, DOmultithread) restated in the oracle against the
    reference's own threaded engine built against the shim.  Both are
    non-deterministic (the thread schedule follows measured region times) and both,
    run after run, sometimes stop a few tenths of a percent above the sequential
    engine's energy, so they are pinned by the distribution of their energies: four
    runs of each, every run connected, fully assigned and within 1 % of the
    reference's sequential energy, and the best run of each within 0.1 % of it."""
    O = oracle_lib
    _need_ref(O)
    if not O.ref_threaded_available():
        pytest.skip("threaded reference build not present")
    metric, mk, k, grad, uinit = THREADED[case]
    m = mk()
    ind = m.indicator if (grad > 0 or metric == "aniso") else None
    pd = m.principal_dirs if metric == "aniso" else None

    def energy(lab):
        ev = O.Port(metric, m.points, m.faces, k, grad, ind, pd)
        ev.evaluate(lab, 1)
        assert ev.clean() == 0
        assert np.all(lab < k)
        return ev.global_energy()

    def solve(cls, opts):
        p = cls(metric, m.points, m.faces, k, grad, ind, pd, unconstrained_init=uinit)
        for a, v in opts.items():
            p.set_option(a, v)
        p.init(None)
        p.run()
        return energy(p.labels())

    seq = solve(O.Ref, {})
    for cls in (O.RefThreaded, O.Port):
        runs = [solve(cls, {"threads": threads}) for _ in range(4)]
        assert all(abs(e - seq) <= 1e-2 * abs(seq) for e in runs), (cls.__name__, runs, seq)
        assert abs(min(runs) - seq) <= 1e-3 * abs(seq), (cls.__name__, runs, seq)
