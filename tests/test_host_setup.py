"""Host-side set-up of the product library against the oracle (CPU only).

Edge numbering / vertex rings, vertex weights and the default initial sampling
run on the host before MinimizeEnergy(); they must equal the restatement (and so
the reference) exactly.  Also checks that the CUDA library loads and exports
every entry point declared in include/acvd_gpu.h (no device calls).
"""
import ctypes

import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import engine as E
from acvd_gb300 import synth

MESHES = [
    ("icosphere3", lambda: synth.icosphere(3, seed=0)),
    ("torus40x20", lambda: synth.torus(40, 20, seed=1)),
    ("heightfield25", lambda: synth.heightfield(25, seed=2)),
    ("grid9", lambda: synth.grid(9, seed=3)),
    ("tetrahedron", synth.tetrahedron),
    ("octahedron", synth.octahedron),
]


@pytest.fixture(scope="module")
def lib():
    return E.load()


def test_library_exports_header_symbols(lib):
    names = E.exported_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert ctypes.cast(getattr(lib, n), ctypes.c_void_p).value


@pytest.mark.parametrize("name,mk", MESHES, ids=[m[0] for m in MESHES])
def test_topology_matches_reference_numbering(oracle_lib, lib, name, mk):
    m = mk()
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    p = oracle_lib.Port("iso", m.points, m.faces, 1)
    pev, prow, pcol = p.topology()
    np.testing.assert_array_equal(ev, pev)
    np.testing.assert_array_equal(row, prow)
    np.testing.assert_array_equal(col, pcol)


@pytest.mark.parametrize("metric,grad", [("iso", 0.0), ("iso", 1.0), ("qem", 0.0), ("qem", 1.5), ("aniso", 1.5)])
def test_weights_match_metric_build(oracle_lib, lib, metric, grad):
    m = synth.torus(48, 24, seed=5)
    ind = m.indicator if (grad > 0 or metric == "aniso") else None
    w = acvd_gb300.vertex_weights(metric, m.points, m.faces, ind, grad)
    p = oracle_lib.Port(metric, m.points, m.faces, 10, grad, ind, m.principal_dirs if metric == "aniso" else None)
    p.init(None)
    np.testing.assert_array_equal(w, p.items()["weight"])


@pytest.mark.parametrize("metric,k,grad", [("iso", 60, 0.0), ("qem", 150, 1.5), ("aniso", 80, 1.5), ("iso", 7, 0.0)])
def test_initial_sampling_matches_reference(oracle_lib, lib, metric, k, grad):
    m = synth.torus(56, 28, seed=2)
    ind = m.indicator if (grad > 0 or metric == "aniso") else None
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    w = acvd_gb300.vertex_weights(metric, m.points, m.faces, ind, grad)
    lab = acvd_gb300.initial_sampling(row, col, w, k)
    p = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind, m.principal_dirs if metric == "aniso" else None)
    p.init(None)
    np.testing.assert_array_equal(lab, p.labels())


def test_bad_inputs_raise(lib):
    with pytest.raises(acvd_gb300.AcvdError):
        acvd_gb300.build_topology(3, np.array([[0, 1, 5]], dtype=np.int32))
    with pytest.raises(acvd_gb300.AcvdError):
        acvd_gb300.initial_sampling(np.array([0, 0], dtype=np.int32), np.zeros(0, dtype=np.int32),
                                    np.ones(1), 0)


@pytest.mark.parametrize("metric,k,nfix,grad", [("qem", 150, 12, 1.5), ("iso", 60, 5, 0.0), ("qem", 40, 40, 0.0),
                                                 ("iso", 9, 3, 0.0)])
def test_initial_sampling_with_fixed_vertices_matches_reference(oracle_lib, lib, metric, k, nfix, grad):
    """SetFixedClusters before InitSamples: the fixed vertices take clusters 0 .. F-1
    and the grown regions the labels above (vtkUniformClustering.h:1186-1316)."""
    m = synth.torus(56, 28, seed=2)
    ind = m.indicator if grad > 0 else None
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    w = acvd_gb300.vertex_weights(metric, m.points, m.faces, ind, grad)
    fixed = np.random.default_rng(k).choice(m.n_points, size=nfix, replace=False).astype(np.int32)
    lab = acvd_gb300.initial_sampling(row, col, w, k, fixed=fixed)
    p = oracle_lib.Port(metric, m.points, m.faces, k, grad, ind)
    p.set_fixed(fixed)
    p.init(None)
    np.testing.assert_array_equal(lab, p.labels())
    np.testing.assert_array_equal(lab[fixed], np.arange(nfix))
    with pytest.raises(acvd_gb300.AcvdError):
        acvd_gb300.initial_sampling(row, col, w, k, fixed=np.array([m.n_points], dtype=np.int32))
    with pytest.raises(acvd_gb300.AcvdError):
        acvd_gb300.initial_sampling(row, col, w, nfix - 1, fixed=fixed)
