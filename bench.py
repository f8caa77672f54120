"""Benchmark: time to a converged ACVDQ clustering on one GB300.

Workload (default): ACVDQ -- QEM metric, curvature gradation 1.5, unconstrained
initialisation -- on the seeded synthetic torus R=1, r=0.3, 1024 x 512 vertices
(524,288 items, 1,048,576 triangles), 20,000 clusters, the reference's default
initial sampling.  One "step" is one full minimisation (MinimizeEnergy) from the
same initial clustering, inputs resident in HBM.  The metric is items/s =
items / time-to-converge.  The GPU clustering's energy, evaluated with the
reference arithmetic (oracle), must be within 0.1 % of the CPU run's converged
energy.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank solves its own replica (a single mesh does not
shard); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from acvd_gb300 import replicas  # noqa: E402  (after the repository root is on the path)

METRIC = "time to converged ACVDQ energy (<=0.1% of ref), items/s, batched meshes/s"
L2_BYTES = 129 * 1024 * 1024

WORKLOADS = {
    "torus_1024x512_qem": dict(kind="torus", mesh=dict(nu=1024, nv=512, seed=0), metric="qem", k=20000,
                               gradation=1.5, uinit=1,
                               desc="ACVDQ torus R=1 r=0.3 1024x512 (524,288 items), K=20,000, gradation 1.5"),
    "icosphere_l5_iso": dict(kind="icosphere", mesh=dict(level=5, seed=0), metric="iso", k=1000,
                             gradation=0.0, uinit=0, init="seeds",
                             desc="ACVD icosphere level 5 (10,242 items), K=1,000 single-item seeds from a "
                                  "seeded shuffle (others unassigned), isotropic"),
    "torus_512x512_qem": dict(kind="torus", mesh=dict(nu=512, nv=512, seed=0), metric="qem", k=10000,
                              gradation=1.0, uinit=1, density=True,
                              desc="ACVDQ torus 512x512 (262,144 items), K=10,000, densities U[0.5,2], gradation 1"),
    "heightfield_4096_aniso": dict(kind="heightfield", mesh=dict(n=4096, seed=0), metric="aniso", k=200000,
                                   gradation=1.5, uinit=0,
                                   desc="quadric-anisotropic heightfield 4096^2 (16,777,216 items), K=200,000",
                                   # the sequential CPU solve of the full mesh takes far longer than the
                                   # bench budget: time a 1024^2 patch with the same items per cluster
                                   cpu_sample=dict(mesh=dict(n=1024, seed=0), k=12500)),
    # the 4096^2 workload at a quarter of the items (same items per cluster): small enough
    # for multi-pass ncu captures, whose per-launch figures scale to the full mesh
    "heightfield_2048_aniso": dict(kind="heightfield", mesh=dict(n=2048, seed=0), metric="aniso", k=50000,
                                   gradation=1.5, uinit=0,
                                   desc="quadric-anisotropic heightfield 2048^2 (4,194,304 items), K=50,000",
                                   cpu_sample=dict(mesh=dict(n=512, seed=0), k=3125)),
}


BATCH_WORKLOADS = {
    "batch_256_qem": dict(n_meshes=256, seed=0, metric="qem", gradation=0.0, uinit=1,
                          desc="256 meshes (icosphere / torus / heightfield, type uniform, vertices "
                               "log-uniform in [2,000, 500,000]), ACVDQ, K = vertices / 20 per mesh",
                          cpu_every=16),
}


ADJOINT_WORKLOADS = {
    "torus_512x512_adjoint": dict(mesh=dict(nu=512, nv=512, seed=0), k=10000, gradation=1.0,
                                  desc="adjoint of ACVDQ on the torus 512x512 (262,144 items), densities "
                                       "U[0.5, 2] with gradation 1, K=10,000 converged then fixed: gradients "
                                       "of the energy and of the placed vertices w.r.t. positions and densities"),
}


CURVATURE_WORKLOADS = {
    "curvature_torus_1024x512": dict(kind="torus", mesh=dict(nu=1024, nv=512, seed=0),
                                     desc="vertex curvature (vtkCurvatureMeasure polynomial fitting on the "
                                          "3-ring) of the torus 1024x512 (524,288 vertices)"),
    "curvature_heightfield_4096": dict(kind="heightfield", mesh=dict(n=4096, seed=0),
                                       desc="vertex curvature (vtkCurvatureMeasure polynomial fitting on the "
                                            "3-ring) of the heightfield 4096^2 (16,777,216 vertices)"),
}
CURV_CHECK = 4096        # vertices compared bit for bit with the oracle

SUBDIVISION_WORKLOADS = {
    "subdivide_torus_1024x512": dict(kind="torus", mesh=dict(nu=1024, nv=512, seed=0),
                                     desc="one level of midpoint subdivision (vtkSurface::Subdivide) with the "
                                          "indicator's parent interpolation, torus 1024x512 (524,288 vertices, "
                                          "1,048,576 faces -> 2,097,152 vertices, 4,194,304 faces)"),
}


MANIFOLD_WORKLOADS = {
    "force_manifold_torus_1024x512": dict(kind="torus", mesh=dict(nu=1024, nv=512, seed=0), k=20000,
                                          desc="one ForceManifold detection pass (DetectNonManifoldOutputVertices) "
                                               "on the torus 1024x512 (524,288 items), K=20,000, from the "
                                               "reference's initial sampling with its holes filled"),
}


def run_manifold_arm(args):
    """One detection pass of the ForceManifold loop: the device checks (dual triangles,
    manifold tests of output and input vertices) and the host's new-cluster bookkeeping,
    timed on the wall clock around the call (the pass ends with a device-to-host read)."""
    import torch
    import acvd_gb300
    from acvd_gb300 import engine as E
    from acvd_gb300 import synth
    from oracle import oracle

    ws, rank, local = _dist()
    device = local
    torch.cuda.set_device(device)
    w = MANIFOLD_WORKLOADS[args.workload]
    m = synth.make(w["kind"], with_curvature=False, **w["mesh"])
    k = w["k"]
    oracle.build(ref=False)
    p = oracle.Port("qem", m.points, m.faces, k, 0.0)
    p.init(None)
    p.fill_holes()
    lab = p.labels()
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    eng = E.Engine(device=device)
    eng.set_mesh(m.points, m.faces, row, col, ev)
    eng.set_metric("qem")
    for _ in range(args.warmup):
        eng.set_labels(k, lab)
        eng.force_manifold_step()
    step_ms, issues = [], 0
    with ClockSampler(device) as clk:
        for _ in range(args.steps):
            eng.set_labels(k, lab)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            issues = eng.force_manifold_step()
            step_ms.append(1000.0 * (time.perf_counter() - t0))
    g_lab, g_k, g_frozen = eng.labels(), eng.k, eng.frozen_clusters()
    eng.close()
    if rank != 0:
        return
    t0 = time.perf_counter()
    n_ref = p.detect_nonmanifold()
    secs = time.perf_counter() - t0
    exact = n_ref == issues and p.k == g_k and np.array_equal(p.labels(), g_lab) and \
        np.array_equal(p.frozen(), g_frozen)
    ms = statistics.mean(step_ms)
    n = m.n_points
    cpu = None if args.no_cpu_baseline else {
        "value": n / secs, "unit": "items/s", "cores": 1, "kind": "port",
        "sample": f"the same pass on the same clustering, one core ({secs:.3f} s)"}
    print(json.dumps({
        "metric": "ForceManifold detection pass throughput (items of the clustering per second)",
        "value": n / (ms / 1000.0), "unit": "items/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": {"workload": args.workload, "description": w["desc"], "items": n, "clusters": k,
                   "issues": issues, "timing": "wall clock around acvd_force_manifold_step (host-synchronous)"},
        "roofline": None,
        "roofline_note": "a pass of short kernels (dual mesh sort, incidence lists, per-vertex fan walks) and "
                         "host bookkeeping; no single kernel dominates",
        "parity": {"identical_to_oracle": bool(exact), "issues_oracle": n_ref},
        "cpu_baseline": cpu,
        "e2e": {"value": n / (ms / 1000.0), "unit": "items/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(4 * n), "ms_per_step": ms},
        "clocks": clk.summary(),
    }), flush=True)


def run_manifold_reference_arm(args):
    """Reference arm of the ForceManifold workload: the restated detection pass
    (sequential, as the reference's), one per step from the same clustering."""
    ws, rank, local = _dist()
    if rank != 0:
        return
    from acvd_gb300 import synth
    from oracle import oracle
    oracle.build(ref=False)
    w = MANIFOLD_WORKLOADS[args.workload]
    m = synth.make(w["kind"], with_curvature=False, **w["mesh"])
    base = oracle.Port("qem", m.points, m.faces, w["k"], 0.0)
    base.init(None)
    base.fill_holes()
    lab = base.labels()
    secs = []
    for it in range(args.warmup + args.steps):
        p = oracle.Port("qem", m.points, m.faces, w["k"], 0.0)
        p.init(lab)
        p.fill_holes()
        t0 = time.perf_counter()
        p.detect_nonmanifold()
        if it >= args.warmup:
            secs.append(time.perf_counter() - t0)
    ms = 1000.0 * statistics.mean(secs)
    value = m.n_points / (ms / 1000.0)
    print(json.dumps({
        "impl": "reference", "metric": "ForceManifold detection pass throughput (items of the clustering per second)",
        "value": value, "unit": "items/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic", "config": {"workload": args.workload, "description": w["desc"]},
        "cpu_baseline": {"value": value, "unit": "items/s", "cores": 1, "kind": "port",
                         "sample": "the whole pass per step, one core"},
        "e2e": {"value": value, "unit": "items/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def subdivision_bytes(nv, ne, nf):
    """Compulsory bytes of one subdivision launch sequence: points (24 B), indicator (8 B),
    ring offsets (4 B) per vertex, faces (12 B), ring slots and edge ends (2 x 8 B per edge)
    read once; new points and indicator (32 B per output vertex), parents (8 B per edge),
    faces (48 B per input face) written once; the slot-to-edge table written and read (16 B
    per edge)."""
    return (24 + 8 + 4) * nv + 12 * nf + 16 * ne + 32 * (nv + ne) + 8 * ne + 48 * nf + 16 * ne


def run_subdivision_reference_arm(args):
    """Reference arm of the subdivision workload: the restatement of vtkSurface::Subdivide
    (sequential, one core -- the reference's loop is not threaded), after the edge table is
    built, one full subdivision per step."""
    ws, rank, local = _dist()
    if rank != 0:
        return
    from acvd_gb300 import synth
    from oracle import oracle
    oracle.build(ref=False)
    w = SUBDIVISION_WORKLOADS[args.workload]
    m = synth.make(w["kind"], with_curvature=False, **w["mesh"])
    ind = np.random.default_rng(0).uniform(0.5, 2.0, size=m.n_points)
    for _ in range(args.warmup):
        oracle.subdivide(m.points, m.faces, ind)
    secs = []
    for _ in range(args.steps):
        out = oracle.subdivide(m.points, m.faces, ind, timing=secs)
    n_out = out[0].shape[0]
    ms = 1000.0 * statistics.mean(secs)
    value = n_out / (ms / 1000.0)
    print(json.dumps({
        "impl": "reference", "metric": "midpoint subdivision throughput (vtkSurface::Subdivide + indicator "
                                       "interpolation)",
        "value": value, "unit": "output vertices/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": args.workload, "description": w["desc"]},
        "cpu_baseline": {"value": value, "unit": "output vertices/s", "cores": 1, "kind": "port",
                         "sample": "the whole mesh per step, one core, after the edge table is built"},
        "e2e": {"value": value, "unit": "output vertices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def run_subdivision_arm(args):
    """One level of subdivision on the GPU: resident (device pointers, CUDA events on the
    context's stream, L2 flushed between steps) and end to end (host buffers)."""
    import torch
    import acvd_gb300
    from acvd_gb300 import engine as E
    from acvd_gb300 import synth

    ws, rank, local = _dist()
    device = local
    torch.cuda.set_device(device)
    w = SUBDIVISION_WORKLOADS[args.workload]
    m = synth.make(w["kind"], with_curvature=False, **w["mesh"])
    nv, nf = m.n_points, m.n_faces
    row, col, ev = acvd_gb300.build_topology(nv, m.faces)
    ne = ev.shape[0]
    ind = np.random.default_rng(0).uniform(0.5, 2.0, size=nv)
    dev = f"cuda:{device}"
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)
    d_xyz, d_tri, d_row, d_col, d_ev, d_ind = (t(m.points, np.float64), t(m.faces, np.int32), t(row, np.int32),
                                               t(col, np.int32), t(ev, np.int32), t(ind, np.float64))
    o_xyz = torch.empty((nv + ne, 3), dtype=torch.float64, device=dev)
    o_tri = torch.empty((4 * nf, 3), dtype=torch.int32, device=dev)
    o_p1 = torch.empty(ne, dtype=torch.int32, device=dev)
    o_p2 = torch.empty(ne, dtype=torch.int32, device=dev)
    o_ind = torch.empty(nv + ne, dtype=torch.float64, device=dev)
    eng = E.Engine(device=device)
    work = torch.empty(eng.subdivide_work_bytes(ne), dtype=torch.uint8, device=dev)
    stream = torch.cuda.ExternalStream(eng.stream(), device=device)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    def call():
        eng.subdivide_device(nv, d_xyz.data_ptr(), nf, d_tri.data_ptr(), d_row.data_ptr(), d_col.data_ptr(), ne,
                             d_ev.data_ptr(), d_ind.data_ptr(), o_xyz.data_ptr(), o_tri.data_ptr(),
                             o_p1.data_ptr(), o_p2.data_ptr(), o_ind.data_ptr(), work.data_ptr())

    for _ in range(args.warmup):
        call()
    torch.cuda.synchronize()
    step_ms = []
    with ClockSampler(device) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            call()
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
    ms = statistics.mean(step_ms)
    faults = int(work[8 * ne:8 * ne + 4].view(torch.int32).item())
    g_xyz, g_tri, g_p1, g_p2, g_ind = (o_xyz.cpu().numpy(), o_tri.cpu().numpy(), o_p1.cpu().numpy(),
                                       o_p2.cpu().numpy(), o_ind.cpu().numpy())
    e2e = None
    if not args.no_e2e:
        c = np.ascontiguousarray
        h_pts, h_faces, h_row, h_col, h_ev, h_ind = (pinned(torch, a) for a in (
            c(m.points, dtype=np.float64), c(m.faces, dtype=np.int32), c(row, dtype=np.int32),
            c(col, dtype=np.int32), c(ev, dtype=np.int32), c(ind, dtype=np.float64)))
        e2e_ms = []
        for it in range(args.warmup + max(1, args.steps)):   # untimed warm-up calls first
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = eng.subdivide(h_pts, h_faces, h_row, h_col, h_ev, indicator=h_ind)
            if it >= args.warmup:
                e2e_ms.append(1000.0 * (time.perf_counter() - t0))
        assert np.array_equal(out[0], g_xyz) and np.array_equal(out[1], g_tri), "end-to-end subdivision differs"
        e2e = {"value": (nv + ne) / (statistics.mean(e2e_ms) / 1000.0), "unit": "output vertices/s",
               "h2d_bytes_per_step": int(h_pts.nbytes + h_faces.nbytes + h_row.nbytes + h_col.nbytes + h_ev.nbytes +
                                         h_ind.nbytes),
               "d2h_bytes_per_step": int(out[0].nbytes + out[1].nbytes + out[2].nbytes + out[3].nbytes +
                                         out[4].nbytes),
               "ms_per_step": statistics.mean(e2e_ms),
               "includes": "host->device inputs, the three kernels, device->host outputs (pageable results)"}
    eng.close()
    if rank != 0:
        return
    from oracle import oracle
    oracle.build(ref=False)
    secs = []
    r = oracle.subdivide(m.points, m.faces, ind, timing=secs)
    exact = (faults == 0 and np.array_equal(r[0], g_xyz) and np.array_equal(r[1], g_tri) and
             np.array_equal(r[2], g_p1) and np.array_equal(r[3], g_p2) and np.array_equal(r[4], g_ind))
    cpu = None
    if not args.no_cpu_baseline:
        cpu = {"value": (nv + ne) / secs[0], "unit": "output vertices/s", "cores": 1, "kind": "port",
               "sample": f"the whole mesh, one core, after the edge table is built ({secs[0]:.3f} s)"}
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    alg = subdivision_bytes(nv, ne, nf)
    achieved = alg / 1e9 / (ms / 1000.0)
    line = {
        "metric": "midpoint subdivision throughput (vtkSurface::Subdivide + indicator interpolation)",
        "value": (nv + ne) / (ms / 1000.0), "unit": "output vertices/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "description": w["desc"], "vertices": nv, "edges": ne, "faces": nf,
                   "l2": "flushed between timed steps (256 MB write)"},
        "roofline": {"bound": "hbm", "kernel": "subdiv_* (three kernels and a memset, timed together)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback",
                     "traffic": None, "algorithmic_bytes_per_launch": alg},
        "parity": {"bit_exact_vs_oracle": bool(exact), "faces_reported": faults},
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": 4 * (args.steps + args.warmup),
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
CURV_CPU_SAMPLE = 65536  # vertices of the single-core CPU baseline


def run_curvature_arm(args):
    """Per-vertex curvature on the GPU: resident (device time) and end to end (set_mesh
    from pinned host buffers, outputs back into pinned buffers)."""
    import torch
    import acvd_gb300
    from acvd_gb300 import engine as E
    from acvd_gb300 import synth

    ws, rank, local = _dist()
    device = local
    torch.cuda.set_device(device)
    w = CURVATURE_WORKLOADS[args.workload]
    m = synth.make(w["kind"], with_curvature=False, **w["mesh"])
    n = m.n_points
    row, col, ev = acvd_gb300.build_topology(n, m.faces)
    eng = E.Engine(device=device)
    eng.set_mesh(m.points, m.faces, row, col, ev)
    stream = torch.cuda.ExternalStream(eng.stream(), device=device)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{device}")
    for _ in range(args.warmup):
        eng.compute_curvature(copy_out=False)
    torch.cuda.synchronize()
    step_ms = []
    with ClockSampler(device) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.compute_curvature(copy_out=False)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
    ms = statistics.mean(step_ms)
    ind, pd = eng.compute_curvature()
    eng.close()
    e2e = None
    if not args.no_e2e:
        c = np.ascontiguousarray
        h_pts, h_faces, h_row, h_col, h_ev = (pinned(torch, a) for a in (
            c(m.points, dtype=np.float64), c(m.faces, dtype=np.int32), c(row, dtype=np.int32),
            c(col, dtype=np.int32), c(ev, dtype=np.int32)))
        o_ind = pinned(torch, np.zeros(n, dtype=np.float64))
        o_pd = pinned(torch, np.zeros((n, 6), dtype=np.float32))
        eng2 = E.Engine(device=device)
        e2e_ms = []
        for it in range(args.warmup + max(1, args.steps)):   # untimed warm-up calls first
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            eng2.set_mesh(h_pts, h_faces, h_row, h_col, h_ev)
            eng2.compute_curvature(o_ind, o_pd)
            if it >= args.warmup:
                e2e_ms.append(1000.0 * (time.perf_counter() - t0))
        eng2.close()
        assert np.array_equal(o_ind, ind) and np.array_equal(o_pd, pd), "end-to-end curvature differs"
        e2e = {"value": n / (statistics.mean(e2e_ms) / 1000.0), "unit": "vertices/s",
               "h2d_bytes_per_step": int(h_pts.nbytes + h_faces.nbytes + h_row.nbytes + h_col.nbytes + h_ev.nbytes),
               "d2h_bytes_per_step": int(o_ind.nbytes + o_pd.nbytes), "ms_per_step": statistics.mean(e2e_ms),
               "includes": "acvd_set_mesh (topology upload, colouring, item order, vertex-face CSR) + curvature"}
    if rank != 0:
        return
    from oracle import oracle
    oracle.build(ref=False)
    port = oracle.Port("iso", m.points, m.faces, 10, 0.0)
    step = max(1, n // CURV_CHECK)
    chk = np.arange(0, n, step)[:CURV_CHECK]
    exact = True
    for v in chk[:64]:
        ci, cp = port.curvature_range(int(v), int(v) + 1)
        exact &= bool(ci[v] == ind[v]) and bool(np.array_equal(cp[v], pd[v]))
    cpu = None
    if not args.no_cpu_baseline:
        sample = min(n, CURV_CPU_SAMPLE)
        t0 = time.perf_counter()
        port.curvature_range(0, sample)
        secs = time.perf_counter() - t0
        cpu = {"value": sample / secs, "unit": "vertices/s", "cores": 1, "kind": "port",
               "sample": f"vertices 0..{sample} of the workload mesh, one core ({secs:.2f} s)"}
    line = {
        "metric": "vertex curvature throughput (vtkCurvatureMeasure polynomial fitting, 3-ring)",
        "value": n / (ms / 1000.0), "unit": "vertices/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "description": w["desc"], "vertices": n, "faces": m.n_faces,
                   "l2": "flushed between timed steps (256 MB write)"},
        "roofline": None,
        "roofline_note": "FP64-ALU bound (one thread per vertex, about 8,000 FP64 operations each); "
                         "MEASURED_PEAKS.json holds no FP64 peak",
        "parity": {"vertices_checked_bit_exact_vs_oracle": 64, "bit_exact": exact},
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": 3,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def _curv_job(a):
    """Reference-arm worker: curvature of the vertices [v0, v1) of the workload mesh."""
    name, v0, v1 = a
    from acvd_gb300 import synth
    from oracle import oracle
    global _CURV_PORT
    if _CURV_PORT is None or _CURV_PORT[0] != name:
        w = CURVATURE_WORKLOADS[name]
        m = synth.make(w["kind"], with_curvature=False, **w["mesh"])
        _CURV_PORT = (name, oracle.Port("iso", m.points, m.faces, 10, 0.0))
    t0 = time.perf_counter()
    _CURV_PORT[1].curvature_range(v0, v1)
    return time.perf_counter() - t0


_CURV_PORT = None


def run_curvature_reference_arm(args):
    """CPU arm for the curvature workloads: the restatement of vtkCurvatureMeasure with
    the vertices dealt to every host core, as the reference's threads deal them."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import multiprocessing as mp
    from acvd_gb300 import synth
    from oracle import oracle
    oracle.build(ref=False)
    cores = os.cpu_count() or 1
    w = CURVATURE_WORKLOADS[args.workload]
    m = synth.make(w["kind"], with_curvature=False, **w["mesh"])
    n = m.n_points
    bounds = [(args.workload, (n * c) // cores, (n * (c + 1)) // cores) for c in range(cores)]
    times = []
    with mp.get_context("spawn").Pool(cores) as pool:
        pool.map(_curv_job, [(args.workload, 0, 1)] * cores)   # every worker builds its mesh first
        for step in range(args.warmup + args.steps):
            t = pool.map(_curv_job, bounds)
            if step >= args.warmup:
                times.append(max(t))
    ms = 1000.0 * statistics.mean(times)
    value = n / (ms / 1000.0)
    print(json.dumps({"impl": "reference", "metric": "vertex curvature throughput (vtkCurvatureMeasure polynomial "
                      "fitting, 3-ring)", "value": value, "unit": "vertices/s", "n_gpus": ws,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                      "config": {"workload": args.workload, "description": w["desc"], "vertices": n},
                      "cpu_baseline": {"value": value, "unit": "vertices/s", "cores": cores, "kind": "port",
                                       "sample": f"all {n} vertices dealt over {cores} cores"},
                      "e2e": {"value": value, "unit": "vertices/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)


def run_adjoint_arm(args):
    """Adjoint workload: converge, fix the clustering, time forward + backward of
    E + sum_k G_k . c_k, and check 64 random coordinates against FP64 central
    differences (step 1e-6) and the whole gradient against the FP64 torch reference."""
    import torch
    import acvd_gb300
    from acvd_gb300 import engine as E
    from acvd_gb300 import synth
    from acvd_gb300.adjoint import ClusteringEnergy, cluster_energies, reference_energy

    ws, rank, local = _dist()
    device = local
    torch.cuda.set_device(device)
    w = ADJOINT_WORKLOADS[args.workload]
    m = synth.torus(**w["mesh"], with_curvature=False)
    rho = np.random.default_rng(1).uniform(0.5, 2.0, m.n_points)
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    wts = acvd_gb300.vertex_weights("qem", m.points, m.faces, rho, w["gradation"])
    lab0 = acvd_gb300.initial_sampling(row, col, wts, w["k"])
    eng = E.Engine(device=device)
    eng.set_mesh(m.points, m.faces, row, col, ev)
    eng.set_metric("qem", rho, None, w["gradation"])
    eng.set_unconstrained_initialization(1)
    eng.set_labels(w["k"], lab0)
    conv = eng.minimize()
    lab = eng.labels()
    eng.set_labels(w["k"], lab)            # the converged clustering, held fixed
    G = torch.tensor(np.random.default_rng(7).normal(size=(w["k"], 3)), dtype=torch.float64, device="cuda")
    x = torch.tensor(m.points, dtype=torch.float32, device="cuda", requires_grad=True)   # fp32 input positions
    r = torch.tensor(rho, dtype=torch.float32, device="cuda", requires_grad=True)

    def step():
        x.grad = None
        r.grad = None
        En, C = ClusteringEnergy.apply(x, r, eng, w["gradation"])
        (En + (C * G).sum()).backward()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    times = []
    with ClockSampler(device) as clk:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            step()
            torch.cuda.synchronize()
            times.append(1000.0 * (time.perf_counter() - t0))
    ms = statistics.mean(times)
    # checks at full size
    x64 = torch.tensor(m.points, dtype=torch.float64, device="cuda", requires_grad=True)
    r64 = torch.tensor(rho, dtype=torch.float64, device="cuda", requires_grad=True)
    En, C = ClusteringEnergy.apply(x64, r64, eng, w["gradation"])
    En.backward()
    gx, gr = x64.grad.cpu().numpy(), r64.grad.cpu().numpy()
    rng = np.random.default_rng(11)
    h = 1e-6
    xb = torch.tensor(m.points, dtype=torch.float64, device="cuda")
    rb = torch.tensor(rho, dtype=torch.float64, device="cuda")
    worst_fd = 0.0
    for _ in range(64):
        i, d = int(rng.integers(m.n_points)), int(rng.integers(3))
        xp, xm = xb.clone(), xb.clone()
        xp[i, d] += h
        xm[i, d] -= h
        fd = float((cluster_energies(eng, xp, rb, w["gradation"]) - cluster_energies(eng, xm, rb, w["gradation"])).sum()) / (2 * h)
        worst_fd = max(worst_fd, abs(fd - gx[i, d]) / max(abs(fd), 1e-3 * np.abs(gx).max()))
    xr = torch.tensor(m.points, dtype=torch.float64, requires_grad=True)
    rr = torch.tensor(rho, dtype=torch.float64, requires_grad=True)
    Er, _ = reference_energy(xr, m.faces, lab, w["k"], rr, w["gradation"])
    Er.backward()
    ref_x = float(np.max(np.abs(gx - xr.grad.numpy())) / np.max(np.abs(xr.grad.numpy())))
    ref_r = float(np.max(np.abs(gr - rr.grad.numpy())) / np.max(np.abs(rr.grad.numpy())))
    if rank != 0:
        return
    line = {"metric": METRIC, "value": 1000.0 / ms, "unit": "gradient evaluations/s (forward + backward)",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "description": w["desc"], "items": m.n_points, "clusters": w["k"]},
            "convergence": {"sweeps": conv["sweeps"], "device_ms": conv["device_ms"]},
            "checks": {"fd_coordinates": 64, "fd_step": h, "worst_fd_rel_err": worst_fd,
                       "ref_grad_rel_err_xyz": ref_x, "ref_grad_rel_err_rho": ref_r,
                       "within_1e-4": bool(worst_fd <= 1e-4 and ref_x <= 1e-4 and ref_r <= 1e-4),
                       "energy": float(En)},
            "cpu_baseline": None, "e2e": None, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def _dist():
    return replicas.world()


def make_workload(name):
    from acvd_gb300 import synth
    w = WORKLOADS[name]
    m = synth.make(w["kind"], **w["mesh"])
    ind = m.indicator
    if w.get("density"):
        ind = np.random.default_rng(1).uniform(0.5, 2.0, size=m.n_points)
    use_ind = w["gradation"] != 0.0 if w["metric"] == "aniso" else w["gradation"] > 0.0
    return m, (ind if use_ind else None), (m.principal_dirs if w["metric"] == "aniso" else None), w


def initial_labels(m, metric, ind, grad, k, init=None):
    """The GPU arm's initial clustering: the library's host port of the reference's
    ComputeInitialRandomSampling (or the seeded single-item seeds)."""
    import acvd_gb300
    from acvd_gb300 import synth
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    if init == "seeds":
        return synth.seed_labels(m.n_points, k, seed=0), (row, col, ev)
    w = acvd_gb300.vertex_weights(metric, m.points, m.faces, ind, grad)
    return acvd_gb300.initial_sampling(row, col, w, k), (row, col, ev)


def reference_seeds(m, w):
    """The CPU side's initial-clustering input: the seeded single-item seeds of the
    seeded workload, else None (the oracle runs the reference's own sampling)."""
    from acvd_gb300 import synth    # numpy only: the CUDA library is not loaded
    return synth.seed_labels(m.n_points, w["k"], seed=0) if w.get("init") == "seeds" else None


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap,utilization.gpu",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = []
        for line in (self.out or "").strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[2:6], float(parts[6])))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = [r for r in rows if r[3] > 0] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in loaded for i, v in enumerate(r[2]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in loaded), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "samples_under_load": len(loaded)}


def cpu_reference_run(m, ind, pd, w, seeds):
    """The oracle's restatement of the reference's sequential MinimizeEnergy, started
    from the reference's own initial sampling (or the given seeds).  Nothing of the
    CUDA library runs here.  Returns the solver, the minimisation's seconds and the
    initial clustering."""
    from oracle import oracle
    oracle.build(ref=False)
    p = oracle.Port(w["metric"], m.points, m.faces, w["k"], w["gradation"], ind, pd, unconstrained_init=w["uinit"])
    p.init(seeds)
    lab_init = p.labels()
    secs = p.run()
    return p, secs, lab_init


def evaluated_energy(w, points, faces, k, ind, pd, labels):
    """The reference's evaluation of a final clustering (Init, labels, ReComputeStatistics
    with the placement on); CPU and GPU clusterings are both compared through it."""
    from oracle import oracle
    ev = oracle.Port(w["metric"], points, faces, k, w["gradation"], ind, pd)
    ev.evaluate(labels, 1)
    return ev.global_energy(), ev


FIXTURE_DIR = os.path.join(ROOT, "tests", "golden", "fullsize")
L2_NOTE = "GPU arm: L2 flushed between timed steps (256 MB write)"
EXTRA_STEPS = 5     # timed steps of the extra workloads of the default run


def fullsize_fixture(name):
    """The oracle's converged energy for a full-size workload from the reference's own
    initial sampling, precomputed by tests/golden/gen_fullsize.py (the sequential CPU
    solve is far longer than a bench run)."""
    try:
        with open(os.path.join(FIXTURE_DIR, name + ".json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def labels_sha(lab) -> str:
    return hashlib.sha256(np.ascontiguousarray(lab, dtype=np.int32).tobytes()).hexdigest()


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def workload_config(name, desc, items, clusters, faces, ws, batch=False):
    """The config block both arms print for a workload (identical keys and values)."""
    par = "single"
    if ws > 1:
        par = f"meshes sharded over {ws} ranks" if batch else f"{ws} replicas"
    return {"workload": name, "description": desc, "items": int(items), "clusters": int(clusters),
            "faces": int(faces), "parallelism": par, "l2": L2_NOTE}


def _batch_port_job(a):
    """Reference-arm worker for the batch: one mesh, one sequential converged solve."""
    spec, metric, grad, uinit, ipc = a
    from acvd_gb300 import batch as B
    from oracle import oracle
    m = B.mesh_from_spec(spec, grad != 0.0 or metric == "aniso")
    k = max(1, m.n_points // ipc)
    use_ind = grad != 0.0 if metric == "aniso" else grad > 0.0
    p = oracle.Port(metric, m.points, m.faces, k, grad, m.indicator if use_ind else None, None,
                    unconstrained_init=uinit)
    p.init(None)
    secs = p.run()
    return m.n_points, secs


def run_batch_reference_arm(args):
    """CPU arm of the batch: one mesh per host core at a time, as the reference's
    VolumeAnalysis hands one label to each thread (VolumeAnalysis.cxx:153).  Each step
    solves a bounded sample of the batch (every 16th mesh); the step time is the sum of
    the sample's solve times over the cores (a perfect packing of the meshes on the
    cores, which favours the CPU)."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import multiprocessing as mp
    from acvd_gb300 import batch as B
    from acvd_gb300 import synth
    from oracle import oracle
    oracle.build(ref=False)
    w = BATCH_WORKLOADS[args.workload]
    cores = os.cpu_count() or 1
    specs = synth.batch_specs(w["n_meshes"] * ws, w["seed"])
    sample = list(range(0, len(specs), w["cpu_every"]))
    jobs = sorted(((specs[i], w["metric"], w["gradation"], w["uinit"], 20) for i in sample),
                  key=lambda j: -B.spec_items(j[0]))
    times = []
    with mp.get_context("spawn").Pool(cores) as pool:
        for step in range(args.warmup + args.steps):
            res = pool.map(_batch_port_job, jobs, chunksize=1)
            if step >= args.warmup:
                times.append(sum(r[1] for r in res) / cores)
    ms = 1000.0 * statistics.mean(times)
    value = len(sample) / (ms / 1000.0)
    items = sum(B.spec_items(s) for s in specs)
    faces = sum(B.spec_faces(s) for s in specs)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "meshes/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.workload, w["desc"], items, sum(max(1, B.spec_items(s) // 20)
                                                                            for s in specs), faces, ws, batch=True),
            "cpu_baseline": {"value": value, "unit": "meshes/s", "cores": cores, "kind": "port",
                             "sample": f"every {w['cpu_every']}th mesh ({len(sample)} meshes) per step, one mesh "
                                       f"per core at a time, sequential reference algorithm restated in C++; "
                                       f"step time = summed solve time / {cores} cores"},
            "e2e": {"value": value, "unit": "meshes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_arm(args):
    """CPU arm: the reference's own parallel engine for one mesh, ACVDQP
    (vtkThreadedClustering: thread regions from the engine's random sampling,
    per-cluster locks, the cross-region edges run serially after each loop;
    DiscreteRemeshing/vtkThreadedClustering.h), restated in the oracle and run with
    every host core as a thread, one converged solve per step from the reference's
    own initial sampling.  The reference's timer brackets MinimizeEnergy; the thread
    layout is built in Init, outside it.  Where the full CPU solve exceeds the bench
    budget (the 4096^2 heightfield) each step solves the bounded sample mesh of the
    workload.  The CUDA library is never loaded on this arm."""
    if args.workload in BATCH_WORKLOADS:
        run_batch_reference_arm(args)
        return
    ws, rank, _ = _dist()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    m, ind, pd, w = make_workload(args.workload)
    cfg = workload_config(args.workload, w["desc"], m.n_points, w["k"], m.n_faces, ws)
    sample = "the full workload mesh"
    fx = fullsize_fixture(args.workload)
    if w.get("cpu_sample"):
        from acvd_gb300 import synth
        k = w["cpu_sample"]["k"]
        m = synth.make(w["kind"], **w["cpu_sample"]["mesh"])
        ind = m.indicator if ind is not None else None
        pd = m.principal_dirs if pd is not None else None
        w = dict(w, k=k)
        sample = f"{w['kind']} {w['cpu_sample']['mesh']} with K={k} (same items per cluster)"
        fx = None
    from oracle import oracle
    oracle.build(ref=False)
    seeds = reference_seeds(m, w)
    times, lab = [], None
    for step in range(args.warmup + args.steps):
        p = oracle.Port(w["metric"], m.points, m.faces, w["k"], w["gradation"], ind, pd, unconstrained_init=w["uinit"])
        p.set_option("threads", cores)
        p.init(seeds)
        secs = p.run()
        if step >= args.warmup:
            times.append(secs)
        lab = p.labels()
    n = m.n_points
    ms = 1000.0 * statistics.mean(times)
    value = n / (ms / 1000.0)
    e_acvdqp, chk = evaluated_energy(w, m.points, m.faces, w["k"], ind, pd, lab)
    energy = {"acvdqp_energy": e_acvdqp, "all_clusters_connected": bool(chk.clean() == 0)}
    if fx is not None:
        energy.update({"sequential_reference_energy": fx["reference_energy"],
                       "rel_diff_vs_sequential": (e_acvdqp - fx["reference_energy"]) / abs(fx["reference_energy"])})
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "items/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": "items/s", "cores": cores, "kind": "port",
                             "sample": f"ACVDQP (the reference's threaded engine, restated) with {cores} threads and "
                                       f"pooling ratio 5, one converged solve of {sample} per step, from the "
                                       f"reference's own initial sampling"},
            "e2e": {"value": value, "unit": "items/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "energy": energy}
    print(json.dumps(line), flush=True)


STEP_KEYS = ("eval_ms", "eval_bytes", "eval_launches", "kernel_launches", "sweeps", "moves", "hit_loop_cap",
             "reverted", "relaxed_sweeps", "sweep_kernel_ms", "sweep_kernel_launches")


def run_steps(torch, e, steps, warmup, device, ws, flush):
    """`warmup` untimed minimisations, then `steps` minimisations (rewind + minimize
    on resident inputs) timed with CUDA events on the engine's stream, the L2
    flushed before each (outside the events).  Returns per-step ms, summed stats and
    the last step's stats."""
    stream = torch.cuda.ExternalStream(e.stream(), device=device)
    for _ in range(warmup):
        e.rewind()
        e.minimize()
    torch.cuda.synchronize()
    replicas.barrier()
    step_ms = []
    tot = {k: 0 for k in STEP_KEYS}
    st = None
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        e.rewind()
        st = e.minimize()
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        for k in tot:
            tot[k] += st[k]
    torch.cuda.synchronize()
    return step_ms, tot, st


def pinned(torch, a):
    """A copy of numpy array `a` in pinned (page-locked) host memory, as a numpy view."""
    if a is None:
        return None
    t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
    out = t.numpy()          # the view's base keeps the pinned tensor alive
    out[...] = a
    return out


def roofline_kernel(persistent, tot_t):
    """The dominant kernel and its event-timed duration from the instrumented pass:
    the evaluation kernel on the per-phase schedule, the persistent sweep kernel
    (all evaluation bytes over its duration) on the persistent one."""
    if persistent:
        return "sweep_run_kernel", tot_t["sweep_kernel_ms"], tot_t["sweep_kernel_launches"]
    return "eval_kernel", tot_t["eval_ms"], tot_t["eval_launches"]


def eval_traffic(workload, coloring):
    """DRAM bytes per evaluation launch of a workload under a colouring, from the
    committed ncu summaries (profiles/eval_traffic.json): (bytes, how measured), or
    (None, None) where no capture covers that evaluation."""
    tpath = os.path.join(ROOT, "profiles", "eval_traffic.json")
    try:
        with open(tpath) as f:
            entry = json.load(f).get(workload, {}).get(coloring)
    except (OSError, ValueError, AttributeError):
        return None, None
    if not entry:
        return None, None
    return entry.get("bytes_per_launch"), entry.get("how")


def roofline_block(persistent, tot_t, workload, coloring="jp"):
    """The dominant kernel's roofline from the instrumented pass, and its DRAM traffic
    per launch from the committed ncu summary (profiles/eval_traffic.json) of the same
    evaluation (workload and colouring)."""
    peaks = load_peaks()
    peak = peaks.get("hbm_gbs", 6800.0)
    kname, kms, klaunch = roofline_kernel(persistent, tot_t)
    achieved = (tot_t["eval_bytes"] / 1e9) / (kms / 1000.0) if kms > 0 else None
    traffic, how = (None, None) if persistent else eval_traffic(workload, coloring)
    return {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback",
            "traffic": traffic, "traffic_source": how, "launches": klaunch,
            "algorithmic_bytes_per_launch": tot_t["eval_bytes"] / max(1, klaunch),
            "avg_launch_us": 1000.0 * kms / max(1, klaunch),
            "timing": "CUDA events around each launch, in a second pass of the same steps "
                      "(the headline pass carries no events)"}


def choose_schedule(args, metric, n, k, device, measure_kw):
    """The schedule a line runs: 'tuned' (default) times the candidate schedules of the
    project's autotuner on this very problem before the timed steps (a fresh tuning per
    run, end-to-end objective: set-up plus converged solve; the approximate candidates
    only within 1e-3 of the default schedule's energy), 'phases' is the default schedule,
    'persistent' the persistent kernel.  Returns (schedule, tuning report or None)."""
    import tempfile
    from acvd_gb300 import autotune as AT
    if args.schedule == "persistent":
        return AT.BY_NAME["persistent"], None
    if args.schedule == "phases":
        return AT.DEFAULT, None
    with tempfile.TemporaryDirectory() as td:
        tuner = AT.Autotuner(os.path.join(td, "tune.json"), include_approximate=True, objective="end_to_end")
        t0 = time.perf_counter()
        sched, rep = tuner.tune(AT.problem_key(metric, n, k, device), AT.solve_measure(device=device, **measure_kw))
        secs = time.perf_counter() - t0
    trials = [{"schedule": t["schedule"], "solve_ms": t["ms"], "setup_ms": t["setup_ms"], "accepted": t["accepted"],
               "reason": t["reason"]} for t in rep["trials"]]
    return sched, {"chosen": sched.name, "objective": rep["objective"], "tuning_s": secs, "trials": trials}


def roofline_by_phase(make_engine, peak):
    """The evaluation's roofline split by sweep kind, from one more converged solve with
    the per-sweep log on (ACVD_SWEEP_LOG: CUDA events around every evaluation, the
    host loop): relaxed sweeps (no connectivity constraint, many moves) and exact
    sweeps (claims, the connectivity phase's long tail)."""
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "sweeps.jsonl")
        old = os.environ.get("ACVD_SWEEP_LOG")
        os.environ["ACVD_SWEEP_LOG"] = path
        try:
            e = make_engine(False)
            e.minimize()
            e.close()
        finally:
            if old is None:
                os.environ.pop("ACVD_SWEEP_LOG", None)
            else:
                os.environ["ACVD_SWEEP_LOG"] = old
        with open(path) as f:
            rows = [json.loads(line) for line in f if '"event"' not in line]
    out = {}
    for mode in ("relaxed", "exact"):
        sel = [r for r in rows if r["mode"] == mode]
        ms = sum(r["eval_ms"] for r in sel)
        by = sum(r["eval_bytes"] for r in sel)
        gbs = by / 1e6 / ms if ms > 0 else None
        out[mode] = {"sweeps": len(sel), "eval_ms": ms, "algorithmic_bytes": by, "achieved_gbs": gbs,
                     "frac": (gbs / peak) if gbs else None}
    return out


def batch_line(args, name, steps, warmup, e2e_on, cpu_on):
    """Batched workload: the rank's share of the meshes (balanced by items) in one packed
    CSR, one minimisation per step.  At N ranks the batch holds N x 256 meshes (the
    first 256 are the single-GPU batch), so the work per GPU stays fixed.  Per-mesh
    labels and energies are gathered on rank 0 after the timed steps.  Returns the
    JSON line on rank 0, None elsewhere."""
    import torch
    from acvd_gb300 import batch as B
    from acvd_gb300 import engine as E
    from acvd_gb300 import shards
    from acvd_gb300 import synth

    ws, rank, device = _dist()
    w = BATCH_WORKLOADS[name]
    specs = synth.batch_specs(w["n_meshes"] * ws, w["seed"])
    parts = shards.balanced_partition([B.spec_items(s) for s in specs], ws)
    mine = parts[rank]
    t0 = time.perf_counter()
    b = B.batch_from_specs([specs[i] for i in mine], w["metric"], w["gradation"])
    gen_s = time.perf_counter() - t0
    from acvd_gb300 import autotune as AT
    row, col, ev = E.build_topology(b.n_points, b.faces)
    sched, tuning = choose_schedule(args, w["metric"], b.n_points, b.k_total, device, dict(
        points=b.points, faces=b.faces, metric=w["metric"], k=b.k_total, labels=b.labels0, indicator=b.indicator,
        gradation=w["gradation"], unconstrained_init=w["uinit"], topology=(row, col, ev), batch=(b.v_off, b.k_off)))
    persistent = sched.persistent
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{device}")

    def make_engine(kernel_timing):
        e = AT.ScheduledEngine(sched, device=device, kernel_timing=kernel_timing)
        e.set_mesh(b.points, b.faces, row, col, ev)
        e.set_batch(b.v_off, b.k_off)
        e.set_metric(w["metric"], b.indicator, None, w["gradation"])
        e.set_unconstrained_initialization(w["uinit"])
        e.set_labels(b.k_total, b.labels0)
        return e

    # pass 1 (the headline): no instrumentation; pass 2: events around the evaluation kernels
    eng = make_engine(False)
    with ClockSampler(device) as clk:
        step_ms, tot, st = run_steps(torch, eng, steps, warmup, device, ws, flush)
    engt = make_engine(True)
    _, tot_t, _ = run_steps(torch, engt, steps, 1, device, ws, flush)
    engt.close()
    by_phase = None if persistent else roofline_by_phase(make_engine, load_peaks().get("hbm_gbs", 6800.0))
    ms = statistics.mean(step_ms)
    ms = replicas.max_over_ranks(ms, device=f"cuda:{device}")   # the slowest rank
    value = len(specs) / (ms / 1000.0)
    packed = eng.labels()
    mesh_e = eng.mesh_energies()
    eng.close()
    e2e = None
    if e2e_on:
        h2d = (b.points.nbytes + b.faces.nbytes + row.nbytes + col.nbytes + ev.nbytes + b.labels0.nbytes +
               (b.indicator.nbytes if b.indicator is not None else 0))
        e2e_ms = []
        eng2 = AT.ScheduledEngine(sched, device=device)
        # the step's inputs and its output buffer in pinned host memory
        c = np.ascontiguousarray
        h_pts, h_faces, h_row, h_col, h_ev = (pinned(torch, a) for a in (
            c(b.points, dtype=np.float64), c(b.faces, dtype=np.int32), c(row, dtype=np.int32),
            c(col, dtype=np.int32), c(ev, dtype=np.int32)))
        h_ind = pinned(torch, None if b.indicator is None else c(b.indicator, dtype=np.float64))
        h_lab0 = pinned(torch, c(b.labels0, dtype=np.int32))
        out = pinned(torch, c(b.labels0, dtype=np.int32))
        # untimed warm-up calls first (the engine's device buffers are allocated on the first)
        for it in range(warmup + max(1, steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            eng2.set_mesh(h_pts, h_faces, h_row, h_col, h_ev)
            eng2.set_batch(b.v_off, b.k_off)
            eng2.set_metric(w["metric"], h_ind, None, w["gradation"])
            eng2.set_unconstrained_initialization(w["uinit"])
            eng2.set_labels(b.k_total, h_lab0)
            eng2.minimize()
            eng2.labels(out=out)
            torch.cuda.synchronize()
            if it >= warmup:
                e2e_ms.append(1000.0 * (time.perf_counter() - t0))
        eng2.close()
        assert np.array_equal(out, packed), "end-to-end batch run differs from the resident run"
        e2e_t = replicas.max_over_ranks(statistics.mean(e2e_ms), device=f"cuda:{device}")
        e2e = {"value": len(specs) / (e2e_t / 1000.0), "unit": "meshes/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(b.labels0.nbytes),
               "ms_per_step": e2e_t, "warmup_calls": warmup}
    # per-mesh results of this rank, gathered on rank 0 (after the timed steps)
    lab_m = shards.split_packed(packed, b.v_off, b.k_off, b.ks)
    lab0_m = shards.split_packed(b.labels0, b.v_off, b.k_off, b.ks)
    local = {g: (lab_m[j], float(mesh_e[j]), labels_sha(lab0_m[j])) for j, g in enumerate(mine)}
    results = shards.gather_meshes(local, len(specs), rank, ws)
    loads = shards.part_loads([B.spec_items(s) for s in specs], parts)
    replicas.barrier()
    if rank != 0:
        return None
    energy = {}
    fx = fullsize_fixture(name)
    if fx is not None:
        # every mesh of the fixture's batch: the GPU clustering evaluated by the oracle
        # against the oracle's own converged solve from the reference's sampling
        t0 = time.perf_counter()
        worst, n_ok, n_conn, n_init, n_chk = -1e300, 0, 0, 0, 0
        for g, ref in enumerate(fx["meshes"][:len(specs)]):
            m = B.mesh_from_spec(specs[g], False)
            lab, _, sha0 = results[g]
            e_gpu, chk = evaluated_energy(w, m.points, m.faces, ref["clusters"], None, None, lab)
            rel = (e_gpu - ref["reference_energy"]) / abs(ref["reference_energy"])
            worst = max(worst, rel)
            n_ok += rel <= 1e-3
            n_conn += chk.clean() == 0
            n_init += sha0 == ref["labels0_sha256"]
            n_chk += 1
        energy = {"meshes_checked": n_chk, "worst_rel_diff_vs_reference": worst,
                  "meshes_within_0.1pct": n_ok, "within_0.1pct": bool(n_ok == n_chk),
                  "meshes_all_clusters_connected": n_conn, "all_clusters_connected": bool(n_conn == n_chk),
                  "meshes_initial_clustering_identical_to_reference": n_init,
                  "reference": "tests/golden/fullsize/" + name + ".json (oracle converged solve per mesh from the "
                               "reference's own initial sampling)",
                  "check_s": time.perf_counter() - t0}
    cpu = None
    if cpu_on:
        from oracle import oracle
        oracle.build(ref=False)
        secs = 0.0
        n_items = 0
        sample = list(range(0, w["n_meshes"], w["cpu_every"]))
        for g in sample:
            m = B.mesh_from_spec(specs[g], False)
            k = max(1, m.n_points // 20)
            p = oracle.Port(w["metric"], m.points, m.faces, k, w["gradation"], unconstrained_init=w["uinit"])
            p.init(None)
            secs += p.run()
            n_items += m.n_points
        cpu = {"value": len(sample) / secs, "unit": "meshes/s", "cores": 1, "kind": "port",
               "sample": f"every {w['cpu_every']}th mesh of the batch ({len(sample)} meshes, {n_items} vertices), "
                         f"sequential converged solves from the reference's own sampling ({secs:.2f} s)"}
    cfg = workload_config(name, w["desc"], sum(B.spec_items(s) for s in specs),
                          sum(max(1, B.spec_items(s) // 20) for s in specs),
                          sum(B.spec_faces(s) for s in specs), ws, batch=True)
    return {
        "metric": METRIC, "value": value, "unit": "meshes/s", "n_gpus": ws, "steps": steps,
        "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
        "schedule": sched.name, "tuning": tuning, "meshes_per_rank": [len(p) for p in parts], "items_per_rank": loads,
        "generation_s": gen_s,
        "roofline": dict(roofline_block(persistent, tot_t, name, sched.coloring), by_sweep_kind=by_phase),
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(tot["kernel_launches"]),
        "sweeps_per_step": tot["sweeps"] / max(1, steps),
        "relaxed_sweeps_per_step": tot["relaxed_sweeps"] / max(1, steps),
        "items_per_s": cfg["items"] / (ms / 1000.0),
        "energy": energy, "mesh_energy_total_rank0": float(np.sum(mesh_e)), "clocks": clk.summary(),
    }


def run_batch_arm(args):
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        replicas.init("nccl")
    line = batch_line(args, args.workload, args.steps, args.warmup, not args.no_e2e, not args.no_cpu_baseline)
    if line is not None:
        print(json.dumps(line), flush=True)


def clustering_line(args, name, steps, warmup, e2e_on, cpu_on):
    """One single-mesh clustering workload on this rank's GPU: the headline pass, the
    instrumented pass (roofline), the end-to-end pass through the C ABI from pinned
    host buffers, and on rank 0 the checks against the oracle.  Returns the JSON line
    on rank 0, None elsewhere."""
    import torch
    from acvd_gb300 import engine as E

    ws, rank, device = _dist()
    m, ind, pd, w = make_workload(name)
    lab0, (row, col, ev) = initial_labels(m, w["metric"], ind, w["gradation"], w["k"], w.get("init"))
    n = m.n_points
    from acvd_gb300 import autotune as AT
    sched, tuning = choose_schedule(args, w["metric"], n, w["k"], device, dict(
        points=m.points, faces=m.faces, metric=w["metric"], k=w["k"], labels=lab0, indicator=ind,
        principal_dirs=pd, gradation=w["gradation"], unconstrained_init=w["uinit"], topology=(row, col, ev)))
    persistent = sched.persistent
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{device}")

    def make_engine(kernel_timing):
        e = AT.ScheduledEngine(sched, device=device, kernel_timing=kernel_timing)
        e.set_mesh(m.points, m.faces, row, col, ev)
        e.set_metric(w["metric"], ind, pd, w["gradation"])
        e.set_unconstrained_initialization(w["uinit"])
        e.set_labels(w["k"], lab0)
        return e

    # pass 1 (the headline): no instrumentation inside the sweeps
    eng = make_engine(False)
    with ClockSampler(device) as clk:
        step_ms, tot, st = run_steps(torch, eng, steps, warmup, device, ws, flush)
    ms = statistics.mean(step_ms)
    lab = eng.labels()
    eng.close()
    # pass 2 (the roofline): the same steps with CUDA events around every evaluation
    # kernel (event nodes inside the sweep graph; on the persistent schedule the
    # events bracket each persistent launch)
    engt = make_engine(True)
    _, tot_t, _ = run_steps(torch, engt, steps, 1, device, ws, flush)
    engt.close()
    by_phase = None if persistent else roofline_by_phase(make_engine, load_peaks().get("hbm_gbs", 6800.0))
    ms = replicas.max_over_ranks(ms, device=f"cuda:{device}")   # the slowest replica
    value = ws * n / (ms / 1000.0)
    gpu_energy_fp64 = st["energy"]

    # end to end through the C ABI with host buffers (copies inside the timed region)
    e2e = None
    if e2e_on:
        h2d = (m.points.nbytes + m.faces.astype(np.int32).nbytes + row.nbytes + col.nbytes + ev.nbytes +
               (ind.nbytes if ind is not None else 0) + (pd.nbytes if pd is not None else 0) + lab0.nbytes)
        d2h = lab0.nbytes
        e2e_ms = []
        eng2 = AT.ScheduledEngine(sched, device=device)
        # the step's inputs and its output buffer in pinned host memory
        c = np.ascontiguousarray
        h_pts, h_faces, h_row, h_col, h_ev = (pinned(torch, a) for a in (
            c(m.points, dtype=np.float64), c(m.faces, dtype=np.int32), c(row, dtype=np.int32),
            c(col, dtype=np.int32), c(ev, dtype=np.int32)))
        h_ind = pinned(torch, None if ind is None else c(ind, dtype=np.float64))
        h_pd = pinned(torch, None if pd is None else c(pd, dtype=np.float32))
        h_lab0 = pinned(torch, c(lab0, dtype=np.int32))
        out = pinned(torch, c(lab0, dtype=np.int32))
        parts = {"set_mesh": [], "set_metric": [], "set_labels": [], "minimize": [], "labels": []}
        # untimed warm-up calls first (the engine's device buffers are allocated on the first)
        for it in range(warmup + max(1, steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            eng2.set_mesh(h_pts, h_faces, h_row, h_col, h_ev)
            t1 = time.perf_counter()
            eng2.set_metric(w["metric"], h_ind, h_pd, w["gradation"])
            t2 = time.perf_counter()
            eng2.set_unconstrained_initialization(w["uinit"])
            eng2.set_labels(w["k"], h_lab0)
            t3 = time.perf_counter()
            eng2.minimize()
            t4 = time.perf_counter()
            eng2.labels(out=out)
            torch.cuda.synchronize()
            t5 = time.perf_counter()
            if it >= warmup:
                e2e_ms.append(1000.0 * (t5 - t0))
                for key, a, b_ in (("set_mesh", t0, t1), ("set_metric", t1, t2), ("set_labels", t2, t3),
                                   ("minimize", t3, t4), ("labels", t4, t5)):
                    parts[key].append(1000.0 * (b_ - a))
        eng2.close()
        assert np.array_equal(out, lab), "end-to-end run differs from the resident run"
        e2e_t = replicas.max_over_ranks(statistics.mean(e2e_ms), device=f"cuda:{device}")
        e2e = {"value": ws * n / (e2e_t / 1000.0), "unit": "items/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_t, "warmup_calls": warmup,
               "breakdown_ms": {k: statistics.mean(v) for k, v in parts.items()}}

    replicas.barrier()
    if rank != 0:
        return None

    # the CPU side: a sequential converged solve from the reference's own initial
    # sampling (oracle only), or the precomputed fixture where that solve is out of budget
    cpu = None
    fx = fullsize_fixture(name)
    seeds = reference_seeds(m, w)
    e_ref, ref_src, init_same = None, None, None
    if w.get("cpu_sample"):
        if cpu_on:
            # bounded sample of the same workload (same generator, same items per cluster)
            smp = dict(w)
            smp.update(mesh=w["cpu_sample"]["mesh"], k=w["cpu_sample"]["k"])
            from acvd_gb300 import synth
            ms_ = synth.make(w["kind"], **smp["mesh"])
            ind_s = ms_.indicator if ind is not None else None
            pd_s = ms_.principal_dirs if pd is not None else None
            _, secs, _ = cpu_reference_run(ms_, ind_s, pd_s, smp, None)
            cpu = {"value": ms_.n_points / secs, "unit": "items/s", "cores": 1, "kind": "port",
                   "sample": f"{w['kind']} {smp['mesh']} with K={smp['k']} (same items per cluster), one "
                             f"sequential converged solve from the reference's own sampling ({secs:.2f} s)"}
    elif cpu_on or fx is None:
        p, secs, lab_init = cpu_reference_run(m, ind, pd, w, seeds)
        init_same = bool(np.array_equal(lab_init, lab0))
        e_ref, _ = evaluated_energy(w, m.points, m.faces, w["k"], ind, pd, p.labels())
        ref_src = "CPU solve in this run (oracle, from the reference's own initial sampling)"
        if cpu_on:
            cpu = {"value": n / secs, "unit": "items/s", "cores": 1, "kind": "port",
                   "sample": f"full workload, one sequential converged solve ({secs:.2f} s)"}
    if e_ref is None and fx is not None:
        e_ref = fx["reference_energy"]
        init_same = labels_sha(lab0) == fx["labels0_sha256"] if seeds is None else None
        ref_src = ("tests/golden/fullsize/" + name + ".json (oracle converged solve from the reference's own "
                   "initial sampling, precomputed)")
    energy = {"gpu_energy_fp64_device": gpu_energy_fp64}
    if e_ref is not None:
        t0 = time.perf_counter()
        e_gpu, chk = evaluated_energy(w, m.points, m.faces, w["k"], ind, pd, lab)
        connected = chk.clean() == 0
        energy.update({
            "reference_energy": e_ref, "reference_source": ref_src,
            "gpu_energy_reference_arithmetic": e_gpu,
            "rel_diff": (e_gpu - e_ref) / abs(e_ref),
            "within_0.1pct": bool(e_gpu <= e_ref + 1e-3 * abs(e_ref)),
            "all_clusters_connected": bool(connected),
            "all_items_assigned": bool(np.all(lab < w["k"])),
            "initial_clustering_identical_to_reference": init_same,
            # the device's FP32-item / compensated-sum energy of the same clustering against
            # the FP64 evaluation
            "device_vs_fp64_rel_err": abs(gpu_energy_fp64 - e_gpu) / abs(e_gpu),
            "check_s": time.perf_counter() - t0})
    return {
        "metric": METRIC, "value": value, "unit": "items/s", "n_gpus": ws, "steps": steps,
        "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(name, w["desc"], n, w["k"], m.n_faces, ws),
        "schedule": sched.name, "tuning": tuning,
        "roofline": dict(roofline_block(persistent, tot_t, name, sched.coloring), by_sweep_kind=by_phase),
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(tot["kernel_launches"]),
        "sweeps_per_step": tot["sweeps"] / max(1, steps),
        "moves_per_step": tot["moves"] / max(1, steps),
        "hit_loop_cap": bool(tot["hit_loop_cap"]),
        "reverted_per_step": tot["reverted"] / max(1, steps),
        "relaxed_sweeps_per_step": tot["relaxed_sweeps"] / max(1, steps),
        "energy": energy,
        "clocks": clk.summary(),
    }


def plain_form_block(args, steps, warmup):
    """The plain float32 form (libacvd_gb300_plain: uncompensated cluster sums) beside
    the compensated one: the torus workload solved with each library from the same
    initial clustering (time, converged energy against the reference, the device
    energy's error against the FP64 evaluation of the same clustering), and the 256
    meshes of the batch solved one at a time with the plain form (summed device time)
    beside their single batched solve."""
    import torch
    from acvd_gb300 import batch as B
    from acvd_gb300 import engine as E
    from acvd_gb300 import synth
    _, _, device = _dist()
    name = DEFAULT_WORKLOAD
    m, ind, pd, w = make_workload(name)
    lab0, (row, col, ev) = initial_labels(m, w["metric"], ind, w["gradation"], w["k"], w.get("init"))
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{device}")
    fx = fullsize_fixture(name)
    out = {}
    for form in ("plain", "compensated"):
        e = E.Engine(device=device, plain=form == "plain")
        e.set_mesh(m.points, m.faces, row, col, ev)
        e.set_metric(w["metric"], ind, pd, w["gradation"])
        e.set_unconstrained_initialization(w["uinit"])
        e.set_labels(w["k"], lab0)
        step_ms, tot, st = run_steps(torch, e, steps, warmup, device, 1, flush)
        lab = e.labels()
        e.close()
        e_gpu, chk = evaluated_energy(w, m.points, m.faces, w["k"], ind, pd, lab)
        rec = {"ms_per_step": statistics.mean(step_ms), "sweeps_per_step": tot["sweeps"] / max(1, steps),
               "reverted_per_step": tot["reverted"] / max(1, steps),
               "gpu_energy_reference_arithmetic": e_gpu, "gpu_energy_device": st["energy"],
               "device_vs_fp64_rel_err": abs(st["energy"] - e_gpu) / abs(e_gpu),
               "all_clusters_connected": bool(chk.clean() == 0)}
        if fx is not None:
            rec["rel_diff_vs_reference"] = (e_gpu - fx["reference_energy"]) / abs(fx["reference_energy"])
            rec["within_0.1pct"] = bool(rec["rel_diff_vs_reference"] <= 1e-3)
        out[f"{name}_{form}"] = rec
    # the batch's meshes one at a time with the plain form
    bw = BATCH_WORKLOADS["batch_256_qem"]
    specs = synth.batch_specs(bw["n_meshes"], bw["seed"])
    total_ms, worst = 0.0, -1e300
    bfx = fullsize_fixture("batch_256_qem")
    for g, spec in enumerate(specs):
        mesh = B.mesh_from_spec(spec, False)
        k = max(1, mesh.n_points // 20)
        r, c_, ev_ = E.build_topology(mesh.n_points, mesh.faces)
        wts = E.vertex_weights(bw["metric"], mesh.points, mesh.faces, None, bw["gradation"])
        l0 = E.initial_sampling(r, c_, wts, k)
        e = E.Engine(device=device, plain=True)
        e.set_mesh(mesh.points, mesh.faces, r, c_, ev_)
        e.set_metric(bw["metric"], None, None, bw["gradation"])
        e.set_unconstrained_initialization(bw["uinit"])
        e.set_labels(k, l0)
        e.minimize()                       # untimed: graph instantiation
        e.rewind()
        st = e.minimize()
        total_ms += st["device_ms"]
        if bfx is not None:
            e_m, _ = evaluated_energy(bw, mesh.points, mesh.faces, k, None, None, e.labels())
            ref = bfx["meshes"][g]["reference_energy"]
            worst = max(worst, (e_m - ref) / abs(ref))
        e.close()
    out["batch_256_qem_plain_one_at_a_time"] = {
        "ms_total": total_ms, "meshes_per_s": len(specs) / (total_ms / 1000.0),
        "worst_rel_diff_vs_reference": worst if bfx is not None else None,
        "timing": "device time of one converged solve per mesh (engine CUDA events), summed"}
    return out


DEFAULT_WORKLOAD = "torus_1024x512_qem"
# the default run adds the configurations whose evaluation is HBM-bound (single GPU only)
EXTRA_WORKLOADS = ("heightfield_4096_aniso", "batch_256_qem")


def run_gpu_arm(args):
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        replicas.init("nccl")
    line = clustering_line(args, args.workload, args.steps, args.warmup, not args.no_e2e, not args.no_cpu_baseline)
    if args.workload == DEFAULT_WORKLOAD and ws == 1 and not args.no_extra:
        extra = {}
        xs = min(args.steps, EXTRA_STEPS)
        for name in EXTRA_WORKLOADS:
            if name in BATCH_WORKLOADS:
                extra[name] = batch_line(args, name, xs, 3, not args.no_e2e, False)
            else:
                extra[name] = clustering_line(args, name, xs, 3, not args.no_e2e, False)
        line["extra_workloads"] = extra
        line["plain_form"] = plain_form_block(args, xs, 3)
    if line is not None:
        print(json.dumps(line), flush=True)


def solve_once(args):
    """One engine set-up and one converged solve of a clustering workload (or the batch),
    untimed: the program that ncu captures are taken on (launch lists, per-launch DRAM
    traffic)."""
    import acvd_gb300
    from acvd_gb300 import engine as E
    if args.workload in BATCH_WORKLOADS:
        from acvd_gb300 import batch as B
        w = BATCH_WORKLOADS[args.workload]
        b = B.synthetic_batch(w["n_meshes"], w["seed"], metric=w["metric"], gradation=w["gradation"])
        e, st = B.run_on_gpu(b, unconstrained_init=w["uinit"])
        e.close()
        print(json.dumps({"workload": args.workload, "sweeps": st["sweeps"], "moves": st["moves"],
                          "device_ms": st["device_ms"], "eval_bytes": st["eval_bytes"],
                          "kernel_launches": st["kernel_launches"]}), flush=True)
        return
    m, ind, pd, w = make_workload(args.workload)
    lab0, (row, col, ev) = initial_labels(m, w["metric"], ind, w["gradation"], w["k"], w.get("init"))
    e = E.Engine()
    e.set_mesh(m.points, m.faces, row, col, ev)
    e.set_metric(w["metric"], ind, pd, w["gradation"])
    e.set_unconstrained_initialization(w["uinit"])
    e.set_labels(w["k"], lab0)
    st = e.minimize()
    e.close()
    print(json.dumps({"workload": args.workload, "sweeps": st["sweeps"], "moves": st["moves"],
                      "device_ms": st["device_ms"], "eval_bytes": st["eval_bytes"],
                      "kernel_launches": st["kernel_launches"]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--schedule", default="tuned", choices=["tuned", "phases", "persistent"],
                    help="sweep schedule of the clustering workloads: chosen by the autotuner on the "
                         "workload before the timed steps (default), the default per-phase kernels in "
                         "CUDA graphs, or one persistent cooperative kernel between convergence events")
    ap.add_argument("--workload", default="torus_1024x512_qem",
                    choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS) + sorted(ADJOINT_WORKLOADS) +
                    sorted(CURVATURE_WORKLOADS) + sorted(SUBDIVISION_WORKLOADS) + sorted(MANIFOLD_WORKLOADS))
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="default workload only: skip the heightfield 4096^2 and batch lines added to it")
    ap.add_argument("--solve-once", action="store_true",
                    help="set up and run one converged solve of a clustering workload, untimed (for ncu)")
    args = ap.parse_args()
    if args.solve_once:
        if args.workload not in WORKLOADS and args.workload not in BATCH_WORKLOADS:
            raise SystemExit("--solve-once takes a clustering or batch workload")
        solve_once(args)
        return
    if args.impl == "reference" and args.workload in SUBDIVISION_WORKLOADS:
        run_subdivision_reference_arm(args)
    elif args.impl == "reference" and args.workload in MANIFOLD_WORKLOADS:
        run_manifold_reference_arm(args)
    elif args.impl == "reference" and args.workload in CURVATURE_WORKLOADS:
        run_curvature_reference_arm(args)
    elif args.impl == "reference":
        run_reference_arm(args)
    elif args.workload in CURVATURE_WORKLOADS:
        run_curvature_arm(args)
    elif args.workload in SUBDIVISION_WORKLOADS:
        run_subdivision_arm(args)
    elif args.workload in MANIFOLD_WORKLOADS:
        run_manifold_arm(args)
    elif args.workload in BATCH_WORKLOADS:
        run_batch_arm(args)
    elif args.workload in ADJOINT_WORKLOADS:
        run_adjoint_arm(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
