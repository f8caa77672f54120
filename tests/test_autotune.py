"""Schedule autotuner: choice, acceptance rules, cache and environment scoping (CPU only;
the measurements are fakes, so no solve runs)."""
import json
import os

import pytest

from acvd_gb300 import autotune as at
from acvd_gb300.engine import AcvdError


def _fake(times, energies=None, digests=None, unassigned=None, fail=(), setup=None):
    calls = []

    def measure(s):
        calls.append(s.name)
        if s.name in fail:
            raise AcvdError(4, "cooperative launch refused")
        return {"ms": times.get(s.name, [50.0]), "energy": (energies or {}).get(s.name, -2.0),
                "setup_ms": (setup or {}).get(s.name, 0.0),
                "digest": (digests or {}).get(s.name, "same"),
                "unassigned": (unassigned or {}).get(s.name, 0)}
    return measure, calls


def test_fastest_exact_schedule_chosen_and_cached(tmp_path):
    path = str(tmp_path / "tune.json")
    measure, calls = _fake({"graphs": [3.0, 2.9, 3.1], "host_loop": [4.0, 4.1, 3.9], "persistent": [2.0, 2.2, 2.1]})
    s, rep = at.Autotuner(path).tune("gb300|qem|n2^19_k2^14", measure)
    assert s == at.BY_NAME["persistent"] and not rep["cached"]
    assert calls == ["graphs", "host_loop", "persistent", "fused", "blocks3", "blocks4", "blocks5", "threads128"]
    assert rep["ms"] == pytest.approx(2.1)
    with open(path) as f:
        assert json.load(f)["gb300|qem|n2^19_k2^14"]["schedule"] == "persistent"
    # a fresh tuner on the same file answers from the cache without measuring
    measure2, calls2 = _fake({})
    s2, rep2 = at.Autotuner(path).tune("gb300|qem|n2^19_k2^14", measure2)
    assert s2 == s and rep2["cached"] and calls2 == []
    # retune measures again
    measure3, calls3 = _fake({"graphs": [1.0], "host_loop": [4.0], "persistent": [2.0]})
    s3, _ = at.Autotuner(path).tune("gb300|qem|n2^19_k2^14", measure3, retune=True)
    assert s3 == at.DEFAULT and len(calls3) == 8


def test_exact_schedule_with_another_clustering_is_rejected():
    measure, _ = _fake({"graphs": [3.0], "host_loop": [1.0], "persistent": [2.0]},
                       digests={"graphs": "a", "host_loop": "b", "persistent": "a"})
    s, rep = at.Autotuner().tune("k", measure)
    assert s.name == "persistent"
    trial = {t["schedule"]: t for t in rep["trials"]}
    assert not trial["host_loop"]["accepted"] and "differs" in trial["host_loop"]["reason"]


def test_approximate_schedules_opt_in_and_energy_bar():
    times = {"graphs": [3.0], "host_loop": [3.5], "persistent": [3.2], "exact_sweeps": [1.0], "match2": [2.0]}
    measure, calls = _fake(times)
    assert at.Autotuner().tune("k", measure)[0] == at.DEFAULT
    assert "exact_sweeps" not in calls
    # exact_sweeps 0.2 % above the default energy: rejected; match2 0.05 %: accepted
    energies = {"graphs": -2.0, "host_loop": -2.0, "persistent": -2.0, "exact_sweeps": -2.0 * 0.998,
                "match2": -2.0 * 0.9995}
    measure, _ = _fake(times, energies=energies, digests={"exact_sweeps": "x", "match2": "y"})
    s, rep = at.Autotuner(include_approximate=True).tune("k", measure)
    assert s.name == "match2"
    trial = {t["schedule"]: t for t in rep["trials"]}
    assert "outside" in trial["exact_sweeps"]["reason"]


def test_cached_approximate_choice_not_returned_to_a_default_tuner(tmp_path):
    path = str(tmp_path / "tune.json")
    times = {"graphs": [3.0], "host_loop": [3.5], "persistent": [3.2], "exact_sweeps": [2.5], "match2": [1.0]}
    measure, _ = _fake(times, digests={"exact_sweeps": "x", "match2": "y"})
    s, _ = at.Autotuner(path, include_approximate=True).tune("k", measure)
    assert s.name == "match2"
    # a default (exact-only) tuner on the same file must not answer with match2
    measure2, calls2 = _fake(times)
    s2, rep2 = at.Autotuner(path).tune("k", measure2)
    assert s2.exact and not rep2["cached"] and calls2 == ["graphs", "host_loop", "persistent", "fused", "blocks3",
                                                           "blocks4", "blocks5", "threads128"]
    # an opt-in tuner with a tighter tolerance than the cached choice's measures again
    at.Autotuner(path, include_approximate=True).tune("k2", _fake(times, digests={"match2": "y"})[0])
    tight = at.Autotuner(path, include_approximate=True, energy_rel_tol=1e-4)
    assert tight.lookup("k2") is None
    # the same tolerance answers from the cache
    assert at.Autotuner(path, include_approximate=True).lookup("k2").name == "match2"


def test_unassigned_items_and_errors_reject_a_candidate():
    measure, _ = _fake({"graphs": [3.0], "host_loop": [1.0], "persistent": [2.0]},
                       unassigned={"host_loop": 5}, fail=("persistent",))
    s, rep = at.Autotuner().tune("k", measure)
    assert s == at.DEFAULT
    trial = {t["schedule"]: t for t in rep["trials"]}
    assert "unassigned" in trial["host_loop"]["reason"]
    assert trial["persistent"]["reason"].startswith("error")


def test_default_schedule_failure_is_raised():
    measure, _ = _fake({}, fail=("graphs",))
    with pytest.raises(AcvdError):
        at.Autotuner().tune("k", measure)


def test_default_always_measured_first():
    tuner = at.Autotuner(candidates=(at.BY_NAME["persistent"], at.BY_NAME["match2"]))
    assert [s.name for s in tuner.candidates] == ["graphs", "persistent", "match2"]


def test_environment_switches_scoped(monkeypatch):
    monkeypatch.setenv("ACVD_HOST_LOOP", "7")
    monkeypatch.delenv("ACVD_RELAXED", raising=False)
    with at.environ({"ACVD_HOST_LOOP": None, "ACVD_RELAXED": "0"}):
        assert "ACVD_HOST_LOOP" not in os.environ and os.environ["ACVD_RELAXED"] == "0"
    assert os.environ["ACVD_HOST_LOOP"] == "7" and "ACVD_RELAXED" not in os.environ
    with pytest.raises(RuntimeError):
        with at.environ({"ACVD_RELAXED": "0"}):
            raise RuntimeError
    assert "ACVD_RELAXED" not in os.environ


def test_schedule_switches_are_the_engines():
    assert at.BY_NAME["host_loop"].run_env() == {"ACVD_HOST_LOOP": "1"}
    assert at.DEFAULT.run_env() == {"ACVD_HOST_LOOP": None}
    assert at.BY_NAME["exact_sweeps"].create_env()["ACVD_RELAXED"] == "0"
    assert at.BY_NAME["match2"].create_env()["ACVD_MATCH_ROUNDS"] == "2"
    assert at.DEFAULT.create_env() == {"ACVD_RELAXED": None, "ACVD_MATCH_ROUNDS": None, "ACVD_EVAL_BLOCKS": None,
                                       "ACVD_EVAL_THREADS": None}
    assert at.BY_NAME["persistent"].persistent and all(s.exact for s in at.EXACT_SCHEDULES)
    assert not any(s.exact for s in at.APPROX_SCHEDULES)


def test_size_class_groups_nearby_sizes():
    assert at.size_class(524288, 20000) == at.size_class(600000, 18000) == "n2^19_k2^14"
    assert at.size_class(10242, 1000) != at.size_class(524288, 1000)
    assert at.size_class(0, 0) == "n2^0_k2^0"


def test_mesh_switches_and_end_to_end_objective():
    # colouring and split threshold are read by acvd_set_mesh: scoped to set_mesh
    assert at.BY_NAME["order_colors"].mesh_env() == {"ACVD_COLORING": "order", "ACVD_SPLIT_MIN": None}
    assert at.BY_NAME["fused"].mesh_env() == {"ACVD_COLORING": None, "ACVD_SPLIT_MIN": "0"}
    assert at.BY_NAME["fused"].exact and not at.BY_NAME["order_colors"].exact
    assert at.BY_NAME["blocks3"].create_env()["ACVD_EVAL_BLOCKS"] == "3" and at.BY_NAME["blocks3"].exact
    times = {"graphs": [10.0], "host_loop": [12.0], "persistent": [12.0], "fused": [11.0], "order_colors": [8.0]}
    setup = {"order_colors": 5.0, "graphs": 1.0, "fused": 1.0}
    dig = {"order_colors": "o"}
    s, _ = at.Autotuner(include_approximate=True).tune("k", _fake(times, digests=dig, setup=setup)[0])
    assert s.name == "order_colors"          # fastest solve
    s, rep = at.Autotuner(include_approximate=True, objective="end_to_end").tune(
        "k", _fake(times, digests=dig, setup=setup)[0])
    assert s.name == "graphs" and rep["score"] == 11.0   # 10 + 1 beats 8 + 5
    with pytest.raises(ValueError):
        at.Autotuner(objective="wall")
