"""Schedule autotuner on the GPU: it times the exact schedules on a small QEM torus,
the schedule it picks gives the default schedule's clustering, and a second call is
answered from its cache (needs a GB300)."""
import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import autotune as at
from acvd_gb300 import synth

pytestmark = pytest.mark.gpu


def test_tuned_schedule_keeps_the_clustering(tmp_path):
    m = synth.torus(96, 48, seed=2)
    k = 300
    lab0 = synth.seed_labels(m.n_points, k, seed=11)
    topo = acvd_gb300.build_topology(m.n_points, m.faces)
    tuner = at.Autotuner(str(tmp_path / "tune.json"))
    kw = dict(indicator=m.indicator, gradation=1.5, level=3, unconstrained_init=1, repeats=2, topology=topo)
    s, rep = at.tune_problem(m.points, m.faces, "qem", k, lab0, tuner=tuner, **kw)
    assert not rep["cached"]
    trials = {t["schedule"]: t for t in rep["trials"]}
    assert set(trials) == {"graphs", "host_loop", "persistent", "fused", "blocks3", "blocks4", "blocks5",
                           "threads128"}
    assert trials["graphs"]["accepted"] and trials["graphs"]["ms"] > 0
    for t in trials.values():   # every exact schedule reaches the same clustering
        assert t["accepted"] or t["reason"].startswith("error"), t

    outs = []
    for sched in (at.DEFAULT, s):
        with at.ScheduledEngine(sched) as e:
            e.set_mesh(m.points, m.faces, *topo)
            e.set_metric("qem", m.indicator, None, 1.5)
            e.set_level(3)
            e.set_unconstrained_initialization(1)
            e.set_labels(k, lab0)
            st = e.minimize()
            outs.append((e.labels(), st["energy"]))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    assert outs[0][1] == outs[1][1]

    s2, rep2 = at.tune_problem(m.points, m.faces, "qem", k, lab0, tuner=at.Autotuner(str(tmp_path / "tune.json")), **kw)
    assert rep2["cached"] and s2 == s


def test_approximate_colourings_within_the_energy_bar(tmp_path):
    """With the opt-in candidates (vertex-order and squeezed colourings, exact-only
    sweeps, two claim rounds) and the end-to-end objective, the chosen schedule assigns
    every item and lands within 1e-3 of the default schedule's energy."""
    m = synth.torus(128, 64, seed=3)
    k = 600
    topo = acvd_gb300.build_topology(m.n_points, m.faces)
    w = acvd_gb300.vertex_weights("qem", m.points, m.faces, m.indicator, 1.5)
    lab0 = acvd_gb300.initial_sampling(topo[0], topo[1], w, k)
    tuner = at.Autotuner(str(tmp_path / "tune.json"), include_approximate=True, objective="end_to_end")
    kw = dict(indicator=m.indicator, gradation=1.5, level=3, unconstrained_init=1, repeats=2, topology=topo)
    s, rep = at.tune_problem(m.points, m.faces, "qem", k, lab0, tuner=tuner, **kw)
    trials = {t["schedule"]: t for t in rep["trials"]}
    assert {"order_colors", "squeeze_colors"} <= set(trials)
    base = trials["graphs"]["energy"]
    for name in ("order_colors", "squeeze_colors"):
        t = trials[name]
        assert t["accepted"] == (abs(t["energy"] - base) <= 1e-3 * abs(base)), t
    with at.ScheduledEngine(s) as e:
        e.set_mesh(m.points, m.faces, *topo)
        e.set_metric("qem", m.indicator, None, 1.5)
        e.set_level(3)
        e.set_unconstrained_initialization(1)
        e.set_labels(k, lab0)
        st = e.minimize()
        lab = e.labels()
    assert np.all(lab < k)
    assert abs(st["energy"] - base) <= 1e-3 * abs(base)
