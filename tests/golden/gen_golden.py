"""Generate the golden fixtures in this directory from the reference's own code.

The reference's clustering headers are compiled unmodified against the VTK shim
(``make -C oracle ref``; needs the reference tree, default /root/reference or
$ACVD_REFERENCE_ROOT).  For each small case below this script stores the inputs
(so that no platform's libm is needed to regenerate them) and the reference's
outputs: the initial sampling, the converged labels, global energy, per-cluster
sizes / centroids / energies, the accumulators of a fixed assignment and its
quadric post-placement (the ACVD driver's last step) at levels 1 and 3, and the
reference's curvature indicator / principal directions of the mesh.  The fixtures
under fixed_vertices/ hold runs with fixed vertices as ACVDQ sets them
(SetFixedClusters, and the QEM clusters' AnchorItem) and a CleanClustering with fixed
vertices.

    python tests/golden/gen_golden.py           # every fixture
    python tests/golden/gen_golden.py fixed     # the fixed-vertex fixtures only
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from acvd_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = [
    # name, metric, mesh builder, K, gradation, unconstrained_init, initial labels
    ("iso_icosphere3_k50", "iso", lambda: synth.icosphere(3, seed=0), 50, 0.0, 0, None),
    ("iso_icosphere4_k300_seeds", "iso", lambda: synth.icosphere(4, seed=1), 300, 0.0, 0, "seeds"),
    ("iso_grid12_k10", "iso", lambda: synth.grid(12, seed=0), 10, 0.0, 0, None),
    ("qem_torus64x32_k200_g15", "qem", lambda: synth.torus(64, 32, seed=0), 200, 1.5, 1, None),
    ("qem_torus48x24_k100_g0", "qem", lambda: synth.torus(48, 24, seed=3), 100, 0.0, 0, None),
    ("aniso_heightfield40_k100_g15", "aniso", lambda: synth.heightfield(40, seed=0), 100, 1.5, 0, None),
]


FIXED_CASES = [
    # name, metric, mesh builder, K (fixed vertices included), gradation, unconstrained_init, fixed count
    ("qem_torus64x32_k212_fixed12_g15", "qem", lambda: synth.torus(64, 32, seed=0), 212, 1.5, 1, 12),
    ("iso_icosphere4_k130_fixed10", "iso", lambda: synth.icosphere(4, seed=1), 130, 0.0, 0, 10),
]


def fixed_ids(n, count, seed):
    return np.sort(np.random.default_rng(seed).choice(n, size=count, replace=False)).astype(np.int32)


def main_fixed():
    O.build(ref=True)
    out_dir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fixed_vertices")
    os.makedirs(out_dir, exist_ok=True)
    for name, metric, mk, k, grad, uinit, nfix in FIXED_CASES:
        m = mk()
        ind = m.indicator if grad > 0 else None
        fixed = fixed_ids(m.n_points, nfix, k)
        r = O.Ref(metric, m.points, m.faces, k, grad, ind, None, unconstrained_init=uinit)
        r.set_fixed(fixed)
        if metric == "qem":
            r.set_anchors(fixed)
        r.init(None)
        lab_init = r.labels()
        r.run()
        cl = r.clusters()
        # CleanClustering alone on a scattered assignment, the fixed vertices last in their clusters
        lab_r = np.random.default_rng(3).integers(0, k, size=m.n_points).astype(np.int32)
        fixed_c = np.array([int(np.flatnonzero(lab_r == c)[-1]) for c in range(nfix)], dtype=np.int32)
        c = O.Ref(metric, m.points, m.faces, k, grad, ind, None)
        c.set_fixed(fixed_c)
        c.init(lab_r)
        n_split = c.clean()
        d = dict(points=m.points, faces=m.faces, k=k, gradation=grad, unconstrained_init=uinit, metric=metric,
                 fixed=fixed, labels_init=lab_init, labels=r.labels(), energy=r.global_energy(),
                 size=cl["size"], centroid=cl["centroid"], cluster_energy=cl["energy"],
                 clean_labels_in=lab_r, clean_fixed=fixed_c, clean_labels_out=c.labels(), clean_split=n_split)
        if ind is not None:
            d["indicator"] = ind
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **d)
        print(f"{name}: N={m.n_points} K={k} fixed={nfix} E={d['energy']:.12g}")


def main():
    O.build(ref=True)
    out_dir = os.path.dirname(os.path.abspath(__file__))
    for name, metric, mk, k, grad, uinit, init in CASES:
        m = mk()
        ind = m.indicator if (grad > 0 or metric == "aniso") else None
        pd = m.principal_dirs if metric == "aniso" else None
        initial = synth.seed_labels(m.n_points, k, seed=7) if init == "seeds" else None
        r = O.Ref(metric, m.points, m.faces, k, grad, ind, pd, unconstrained_init=uinit)
        r.init(initial)
        lab_init = r.labels()
        seconds = r.run()
        lab = r.labels()
        e = r.global_energy()
        cl = r.clusters()
        # accumulators of a fixed assignment: the initial sampling with holes filled,
        # evaluated on a fresh object (the anisotropic metric's BuildMetric writes its
        # tensors into the principal-direction array, so Init() must run only once)
        r1 = O.Ref(metric, m.points, m.faces, k, grad, ind, pd)
        r1.init(lab_init)
        r1.fill_holes()
        fixed = r1.labels()
        r2 = O.Ref(metric, m.points, m.faces, k, grad, ind, pd)
        r2.evaluate(fixed, 1)
        cf = r2.clusters()
        d = dict(points=m.points, faces=m.faces, k=k, gradation=grad, unconstrained_init=uinit,
                 metric=metric, labels_init=lab_init, labels=lab, energy=e,
                 size=cl["size"], centroid=cl["centroid"], cluster_energy=cl["energy"],
                 fixed_labels=fixed, fixed_S=cf["S"], fixed_W=cf["W"], fixed_Q=cf["Q"],
                 fixed_centroid=cf["centroid"], fixed_cluster_energy=cf["energy"],
                 fixed_energy=r2.global_energy(),
                 # ACVD's quadric post-placement (ACVD.cxx:217-291) of the fixed assignment
                 fixed_post1=r2.post_placement(1), fixed_post3=r2.post_placement(3))
        # the reference's curvature of the mesh (vtkCurvatureMeasure, polynomial fitting,
        # vertices, 3-ring), as vtkDiscreteRemeshing's pre-processing computes it
        d["curv_indicator"], d["curv_dirs"] = O.Ref(metric, m.points, m.faces, k, 0.0).curvature()
        if initial is not None:
            d["initial"] = initial
        if ind is not None:
            d["indicator"] = ind
        if pd is not None:
            d["principal_dirs"] = pd
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **d)
        print(f"{name}: N={m.n_points} K={k} E={e:.12g} ({seconds:.3f} s)")


if __name__ == "__main__":
    if sys.argv[1:] != ["fixed"]:
        main()
    main_fixed()
