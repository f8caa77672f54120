"""acvd_boundary_edges_noalloc against acvd_get_boundary_edges (needs a GB300).

The allocation-free entry point takes device buffers and the caller's stream;
its ids must equal the allocating entry point's, bit for bit (integer output),
on two calls in a row with different clusterings.  Its first call in a process
does the per-device set-up.
"""
import ctypes

import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import synth

pytestmark = pytest.mark.gpu

ACVD_ERR_ARG = 1
ACVD_ERR_UNSUPPORTED = 5
MAX_EDGES = 1 << 26


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _noalloc(lib, torch, ev_d, ne, lab_d):
    ids = torch.full((max(ne, 1),), -1, dtype=torch.int32, device="cuda")
    cnt = torch.full((1,), 0xFFFF, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.acvd_boundary_edges_noalloc(_vp(ev_d), ne, _vp(lab_d), _vp(ids), _vp(cnt), stream)
    assert rc == 0
    torch.cuda.synchronize()
    n = int(cnt.cpu()[0])
    return ids[:n].cpu().numpy()


@pytest.mark.parametrize("nu,nv", [(8, 4), (256, 128), (2048, 1024)])
def test_noalloc_matches_allocating_entry_point(nu, nv):
    torch = pytest.importorskip("torch")
    lib = acvd_gb300.load()
    m = synth.torus(nu, nv, seed=3, with_curvature=False)
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    ne = int(ev.shape[0])
    k = max(2, m.n_points // 20)
    lab_a = acvd_gb300.initial_sampling(row, col, np.ones(m.n_points), k).astype(np.int32)
    lab_b = synth.seed_labels(m.n_points, k, seed=7).astype(np.int32)
    e = acvd_gb300.Engine()
    e.set_mesh(m.points, m.faces, row, col, ev)
    e.set_metric("iso")
    want = []
    for lab in (lab_a, lab_b):
        e.set_labels(k, lab)
        want.append(e.boundary_edges())
    e.close()
    ev_d = torch.from_numpy(np.ascontiguousarray(ev, dtype=np.int32)).cuda()
    got = []
    for lab in (lab_a, lab_b):    # two calls in a row
        got.append(_noalloc(lib, torch, ev_d, ne, torch.from_numpy(lab).cuda()))
    for g, w in zip(got, want):
        assert g.size > 0
        np.testing.assert_array_equal(g, w)


def test_noalloc_rejects_oversized_and_bad_arguments():
    torch = pytest.importorskip("torch")
    lib = acvd_gb300.load()
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # checked on the host before anything is enqueued
    assert lib.acvd_boundary_edges_noalloc(_vp(buf), MAX_EDGES + 1, _vp(buf), _vp(buf), _vp(buf), s) \
        == ACVD_ERR_UNSUPPORTED
    assert lib.acvd_boundary_edges_noalloc(_vp(buf), -1, _vp(buf), _vp(buf), _vp(buf), s) == ACVD_ERR_ARG
    assert lib.acvd_boundary_edges_noalloc(None, 4, _vp(buf), _vp(buf), _vp(buf), s) == ACVD_ERR_ARG
    # no edges: count 0
    cnt = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    assert lib.acvd_boundary_edges_noalloc(None, 0, None, None, _vp(cnt), s) == 0
    torch.cuda.synchronize()
    assert int(cnt.cpu()[0]) == 0
