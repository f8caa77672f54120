"""Failure detection without a GPU fault (needs a GB300): faults are injected on the
host -- corrupt mesh arrays, labels out of range, NaN metric inputs -- and must come
back as error statuses with the context still usable; the device's bounded wait is
made to run out (one block never arrives) and must report that it gave up."""
import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import synth

pytestmark = pytest.mark.gpu


def _mesh():
    m = synth.torus(40, 20, seed=3)
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    return m, row, col, ev


def _solve(e, m, row, col, ev, k=60):
    e.set_mesh(m.points, m.faces, row, col, ev)
    e.set_metric("qem")
    lab = acvd_gb300.initial_sampling(row, col, acvd_gb300.vertex_weights("qem", m.points, m.faces), k)
    e.set_labels(k, lab)
    return e.minimize()


def test_wait_limit_gives_up_and_context_stays_usable():
    m, row, col, ev = _mesh()
    with acvd_gb300.Engine() as e:
        assert e.check_wait_limit(1 << 16) is True
        st = _solve(e, m, row, col, ev)
        assert st["sweeps"] > 0 and not st["hit_loop_cap"]
        with pytest.raises(acvd_gb300.AcvdError):
            e.check_wait_limit(1 << 30)        # above the limit's cap: refused, nothing launched


@pytest.mark.parametrize("what", ["face", "ring", "edge", "offsets", "total"])
def test_corrupt_mesh_arrays_are_rejected(what):
    m, row, col, ev = _mesh()
    tri, row2, col2, ev2 = m.faces.copy(), row.copy(), col.copy(), ev.copy()
    n = m.n_points
    if what == "face":
        tri[7, 2] = n + 3
    elif what == "ring":
        col2[11] = -5
    elif what == "edge":
        ev2[4, 1] = n
    elif what == "offsets":
        row2[10], row2[11] = row2[11], row2[10]   # decreasing, same total
    else:
        row2[-1] -= 1                             # the CSR does not hold 2 n_edges slots
    with acvd_gb300.Engine() as e:
        with pytest.raises(acvd_gb300.AcvdError):
            e.set_mesh(m.points, tri, row2, col2, ev2)
        with pytest.raises(acvd_gb300.AcvdError):
            e.minimize()                          # nothing usable was set
        st = _solve(e, m, row, col, ev)           # the same context takes a good mesh
        assert st["sweeps"] > 0


def test_labels_out_of_range_and_nan_inputs():
    m, row, col, ev = _mesh()
    with acvd_gb300.Engine(max_loops=500) as e:
        e.set_mesh(m.points, m.faces, row, col, ev)
        e.set_metric("qem")
        with pytest.raises(acvd_gb300.AcvdError):
            e.set_labels(30, np.full(m.n_points, -2, dtype=np.int32))
        with pytest.raises(acvd_gb300.AcvdError):
            e.minimize()                          # the rejected labels left no clustering
        # NaN coordinates poison the energies: the minimisation still ends, bounded
        pts = m.points.copy()
        pts[::17] = np.nan
        e.set_mesh(pts, m.faces, row, col, ev)
        e.set_metric("qem")
        lab = acvd_gb300.initial_sampling(row, col, np.ones(m.n_points), 60)
        e.set_labels(60, lab)
        try:
            st = e.minimize()
            assert st["sweeps"] <= 501
        except acvd_gb300.AcvdError as err:
            assert err.code in (3, 4)             # iteration cap or a device check, not a crash
        st = _solve(e, m, row, col, ev)
        assert st["sweeps"] > 0
