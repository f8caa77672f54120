"""Schedule autotuner for the clustering engine.

The engine can run the minimisation (the seam of vtkUniformClustering::MinimizeEnergy,
Common/vtkUniformClustering.h:725-830) under several sweep schedules. Which one is fastest
depends on the mesh size, the cluster count, the metric and the GPU. The tuner times
converged solves of the caller's own problem under each candidate, keeps the fastest
acceptable one, and caches the choice in a JSON file keyed by device, metric and size class.

Two families of candidates:

* exact schedules give the default schedule's clustering bit for bit, so a tuned run never
  changes a result:
    - ``graphs``: per-phase kernels, sweeps between convergence events looped on the device
      inside one CUDA graph (the default);
    - ``host_loop``: the same kernels, one graph launch per sweep decided on the host;
    - ``persistent``: one cooperative kernel per phase with grid barriers;
    - ``fused``: the launch shape of the evaluation -- every colour class through the one
      fused evaluation kernel, where the default splits large classes into a screen pass
      and an evaluation over the forwarded work list;
    - ``blocks3`` / ``blocks4`` / ``blocks5``: the evaluation kernels compiled for 3, 4 or 5
      blocks of 256 threads per SM (80, 64 or 48 registers per thread) instead of the
      per-kernel defaults;
    - ``threads128``: the evaluation kernels in blocks of 128 threads (8 per SM, 64
      registers): a block waits at its tile's barriers, and smaller blocks let more of them
      be in different phases.
  A candidate of this family whose labels differ from the default's is rejected, since that
  would mean a broken guarantee rather than a faster schedule.
* approximate schedules (opt-in) reach a different deterministic clustering:
    - ``exact_sweeps``: no relaxed multi-move sweeps, claim-based sweeps only;
    - ``match2``: two claim / commit rounds per colour step;
    - ``order_colors``: the colour classes of a greedy colouring in vertex order (4 balanced
      classes on grid-like meshes, against the hashed Jones-Plassmann colouring's 6-7 with
      a few nearly empty ones): fewer colour steps per sweep;
    - ``squeeze_colors``: the Jones-Plassmann colouring with its highest classes emptied
      where a local recolouring allows it.
  One of them is accepted only when every item is assigned and its energy is within
  ``energy_rel_tol`` (default 1e-3, the 0.1 % bar against the reference's converged energy)
  of the default schedule's energy on the same input.

The objective is the median device time of a converged solve (``solve``), or that plus the
wall time of the engine's set-up for the problem (``end_to_end``: the host colourings cost
set-up time that a one-off solve pays).

The schedules' switches are the engine's own (the ``persistent`` option of ``acvd_opts`` and the
``ACVD_HOST_LOOP`` / ``ACVD_RELAXED`` / ``ACVD_MATCH_ROUNDS`` / ``ACVD_EVAL_BLOCKS`` /
``ACVD_EVAL_THREADS`` / ``ACVD_COLORING`` / ``ACVD_SPLIT_MIN`` environment switches). The engine
reads ``ACVD_RELAXED``, ``ACVD_MATCH_ROUNDS``, ``ACVD_EVAL_BLOCKS`` and ``ACVD_EVAL_THREADS``
when a context is created, ``ACVD_COLORING`` and ``ACVD_SPLIT_MIN`` when it
takes a mesh and ``ACVD_HOST_LOOP`` when it minimises, so ``ScheduledEngine`` sets them only
around those calls and puts the environment back afterwards.
"""
from __future__ import annotations

import contextlib
import dataclasses
import hashlib
import json
import math
import os
import statistics
import tempfile
import time
from typing import Callable

import numpy as np

from .engine import AcvdError, Engine, build_topology


@dataclasses.dataclass(frozen=True)
class Schedule:
    name: str
    persistent: bool = False
    host_loop: bool = False
    relaxed: bool = True
    match_rounds: int = 1
    coloring: str = "jp"           # jp (device Jones-Plassmann) | order | squeeze
    split_min: int | None = None   # None: the engine's threshold; 0: never split
    eval_blocks: int | None = None  # evaluation kernels' blocks per SM (3, 4, 5); None: the defaults
    eval_threads: int | None = None  # evaluation kernels' threads per block (128); None: 256
    exact: bool = True   # same clustering as the default schedule, bit for bit

    def create_env(self) -> dict:
        """Switches the engine reads in acvd_create (None = unset)."""
        return {"ACVD_RELAXED": None if self.relaxed else "0",
                "ACVD_MATCH_ROUNDS": None if self.match_rounds == 1 else str(int(self.match_rounds)),
                "ACVD_EVAL_BLOCKS": None if self.eval_blocks is None else str(int(self.eval_blocks)),
                "ACVD_EVAL_THREADS": None if self.eval_threads is None else str(int(self.eval_threads))}

    def mesh_env(self) -> dict:
        """Switches the engine reads in acvd_set_mesh."""
        return {"ACVD_COLORING": None if self.coloring == "jp" else self.coloring,
                "ACVD_SPLIT_MIN": None if self.split_min is None else str(int(self.split_min))}

    def run_env(self) -> dict:
        """Switches the engine reads in acvd_minimize."""
        return {"ACVD_HOST_LOOP": "1" if self.host_loop else None}


DEFAULT = Schedule("graphs")
EXACT_SCHEDULES = (DEFAULT, Schedule("host_loop", host_loop=True), Schedule("persistent", persistent=True),
                   Schedule("fused", split_min=0), Schedule("blocks3", eval_blocks=3),
                   Schedule("blocks4", eval_blocks=4), Schedule("blocks5", eval_blocks=5),
                   Schedule("threads128", eval_threads=128))
APPROX_SCHEDULES = (Schedule("exact_sweeps", relaxed=False, exact=False),
                    Schedule("match2", match_rounds=2, exact=False),
                    Schedule("order_colors", coloring="order", exact=False),
                    Schedule("squeeze_colors", coloring="squeeze", exact=False))
BY_NAME = {s.name: s for s in EXACT_SCHEDULES + APPROX_SCHEDULES}


@contextlib.contextmanager
def environ(values: dict):
    """Sets (or, for None, removes) environment variables, and restores them on exit."""
    saved = {k: os.environ.get(k) for k in values}
    try:
        for k, v in values.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        yield
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


class ScheduledEngine(Engine):
    """An Engine whose context is created, and whose minimisations run, under a schedule."""

    def __init__(self, schedule: Schedule = DEFAULT, **kw):
        self.schedule = schedule
        with environ(schedule.create_env()):
            super().__init__(persistent=schedule.persistent, **kw)

    def set_mesh(self, *a, **kw):
        with environ(self.schedule.mesh_env()):
            return super().set_mesh(*a, **kw)

    def minimize(self) -> dict:
        with environ(self.schedule.run_env()):
            return super().minimize()


def size_class(n_items: int, k: int) -> str:
    """Problems within a factor of about 1.4 in items and clusters share a tuned schedule."""
    return "n2^%d_k2^%d" % (round(math.log2(max(int(n_items), 1))), round(math.log2(max(int(k), 1))))


def labels_digest(labels: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(labels, dtype=np.int32).tobytes()).hexdigest()


@dataclasses.dataclass
class Trial:
    schedule: str
    ms: float | None = None          # median device time of the timed solves
    setup_ms: float = 0.0            # wall time of the engine's set-up for the problem
    score: float | None = None       # what the objective minimises
    energy: float | None = None
    accepted: bool = False
    reason: str = ""


class Autotuner:
    """Chooses a schedule per key by measurement and caches the choice.

    ``measure(schedule)`` runs one problem under ``schedule`` and returns a dict with
    ``ms`` (a list of timed solves, device milliseconds), ``energy``, ``unassigned`` and
    ``digest`` (labels_digest of the final clustering); it may raise AcvdError, which
    rejects that candidate. The default schedule is always measured first: it is the
    yardstick for the others, and a failure there is raised to the caller.
    """

    def __init__(self, cache_path: str | None = None, include_approximate: bool = False,
                 energy_rel_tol: float = 1e-3, candidates=None, objective: str = "solve"):
        if objective not in ("solve", "end_to_end"):
            raise ValueError("objective is 'solve' or 'end_to_end'")
        self.cache_path = cache_path
        self.objective = objective
        self.energy_rel_tol = float(energy_rel_tol)
        if candidates is None:
            candidates = EXACT_SCHEDULES + (APPROX_SCHEDULES if include_approximate else ())
        names = [s.name for s in candidates]
        if DEFAULT.name not in names:
            candidates = (DEFAULT,) + tuple(candidates)
        self.candidates = tuple(sorted(candidates, key=lambda s: s.name != DEFAULT.name))
        self.cache = self._load()

    def _load(self) -> dict:
        if not self.cache_path or not os.path.exists(self.cache_path):
            return {}
        with open(self.cache_path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}

    def _save(self) -> None:
        if not self.cache_path:
            return
        d = os.path.dirname(os.path.abspath(self.cache_path))
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=d, prefix=".autotune-", suffix=".json")
        with os.fdopen(fd, "w") as f:
            json.dump(self.cache, f, indent=1, sort_keys=True)
        os.replace(tmp, self.cache_path)

    def lookup(self, key: str) -> Schedule | None:
        """The cached choice for key, if this tuner could have made it: a schedule outside
        this tuner's candidates (an approximate one cached by an opt-in tuner, seen by a
        default one) or an approximate one accepted under a looser energy tolerance than
        this tuner's is a miss, so that a default tuner never returns a schedule that
        changes the clustering."""
        entry = self.cache.get(key)
        if entry is None:
            return None
        s = BY_NAME.get(entry.get("schedule"))
        if s is None or s not in self.candidates:
            return None
        if not s.exact:
            tol = entry.get("energy_rel_tol")
            if tol is None or float(tol) > self.energy_rel_tol:
                return None
        if entry.get("objective", "solve") != self.objective:
            return None
        return s

    def tune(self, key: str, measure: Callable[[Schedule], dict], retune: bool = False) -> tuple[Schedule, dict]:
        """Returns (chosen schedule, report). A cached key is not measured again unless retune."""
        if not retune:
            hit = self.lookup(key)
            if hit is not None:
                return hit, dict(self.cache[key], cached=True)
        trials: list[Trial] = []
        base = None
        for s in self.candidates:
            t = Trial(s.name)
            try:
                r = measure(s)
            except AcvdError as err:
                if s.name == DEFAULT.name:
                    raise
                t.reason = "error: %s" % err
                trials.append(t)
                continue
            t.ms = float(statistics.median(r["ms"]))
            t.setup_ms = float(r.get("setup_ms", 0.0))
            t.score = t.ms + (t.setup_ms if self.objective == "end_to_end" else 0.0)
            t.energy = float(r["energy"])
            if s.name == DEFAULT.name:
                base = r
                t.accepted = True
            elif r.get("unassigned", 0):
                t.reason = "%d items unassigned" % r["unassigned"]
            elif s.exact and r["digest"] != base["digest"]:
                t.reason = "clustering differs from the default schedule's"
            elif not s.exact and abs(t.energy - base["energy"]) > self.energy_rel_tol * abs(base["energy"]):
                t.reason = "energy %.9g outside %.1e of %.9g" % (t.energy, self.energy_rel_tol, base["energy"])
            else:
                t.accepted = True
            trials.append(t)
        best = min((t for t in trials if t.accepted), key=lambda t: t.score)
        report = {"schedule": best.schedule, "ms": best.ms, "score": best.score,
                  "energy_rel_tol": self.energy_rel_tol, "objective": self.objective,
                  "trials": [dataclasses.asdict(t) for t in trials]}
        self.cache[key] = report
        self._save()
        return BY_NAME[best.schedule], dict(report, cached=False)


def device_name(device: int = 0) -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(device)
    except Exception:  # torch absent or without CUDA: the ordinal still keys the cache
        pass
    return "cuda:%d" % device


def problem_key(metric: str, n_items: int, k: int, device: int = 0) -> str:
    return "%s|%s|%s" % (device_name(device), metric, size_class(n_items, k))


def solve_measure(points, faces, metric: str, k: int, labels, indicator=None, principal_dirs=None,
                  gradation: float = 0.0, level: int = 3, unconstrained_init: int = 0,
                  repeats: int = 3, device: int = 0, topology=None, batch=None) -> Callable[[Schedule], dict]:
    """A measure() for Autotuner.tune: one context per schedule, its set-up for the problem
    done three times and the shorter of the two warm ones kept (wall clock), one untimed solve (graph instantiation, first-touch), then
    ``repeats`` converged solves from the same initial clustering (acvd_rewind), each timed
    on the device by the engine's own CUDA events.  batch: (v_off, k_off) of a packed batch
    (acvd_set_batch)."""
    row, col, ev = topology if topology is not None else build_topology(np.asarray(points).shape[0], faces)
    lab0 = np.ascontiguousarray(labels, dtype=np.int32)

    def setup(e):
        e.set_mesh(points, faces, row, col, ev)
        if batch is not None:
            e.set_batch(*batch)
        e.set_metric(metric, indicator, principal_dirs, gradation)
        e.set_level(level)
        e.set_unconstrained_initialization(unconstrained_init)
        e.set_labels(k, lab0)

    def measure(s: Schedule) -> dict:
        with ScheduledEngine(s, device=device) as e:
            # the first set-up pays the context's allocations; the next two are timed and
            # the shorter one kept (host-side noise is of the order of the set-up itself)
            setup(e)
            setup_ms = float("inf")
            for _ in range(2):
                t0 = time.perf_counter()
                setup(e)
                setup_ms = min(setup_ms, 1000.0 * (time.perf_counter() - t0))
            e.minimize()
            ms = []
            for _ in range(max(1, int(repeats))):
                e.rewind()
                st = e.minimize()
                ms.append(st["device_ms"])
            return {"ms": ms, "setup_ms": setup_ms, "energy": st["energy"], "unassigned": st["unassigned"],
                    "digest": labels_digest(e.labels())}

    return measure


def default_cache_path() -> str:
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "acvd_gb300", "autotune.json")


def tune_problem(points, faces, metric: str, k: int, labels, tuner: Autotuner | None = None,
                 retune: bool = False, **kw) -> tuple[Schedule, dict]:
    """Tunes (or looks up) the schedule for one problem; keywords go to solve_measure."""
    tuner = tuner if tuner is not None else Autotuner(default_cache_path())
    key = problem_key(metric, np.asarray(points).shape[0], k, kw.get("device", 0))
    return tuner.tune(key, solve_measure(points, faces, metric, k, labels, **kw), retune=retune)
