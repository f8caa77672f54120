"""Command-line drivers with the reference programs' arguments, on the GPU engine.

    python -m acvd_gb300.acvd  file nvertices gradation [options]   # DiscreteRemeshing/Examples/ACVD.cxx
    python -m acvd_gb300.acvdq file nvertices gradation [options]   # DiscreteRemeshing/Examples/ACVDQ.cxx
    python -m acvd_gb300.anisotropic_remeshing_q file nvertices gradation [options]
                                         # DiscreteRemeshing/Examples/AnisotropicRemeshingQ.cxx

Options are "-key value" pairs as in the reference:

    -b 0/1    boundary fixing (default 0)
    -m 0/1    manifold output (ForceManifold, default 0; not an AnisotropicRemeshingQ option)
    -s t      subsampling threshold (default 10)
    -o dir    output directory
    -of name  output file name (default simplification.ply)
    -q n      ACVD: eigenvalues of the quadric post-placement (default 1, 0 = none);
              ACVDQ, AnisotropicRemeshingQ: the metric's QuadricsOptimizationLevel (default 3)
    -d 0      display (only 0: there is no graphics stack)
    -np n     threads of the reference's threaded engine (accepted, unused)
    -p n      its thread pooling ratio (accepted, unused)
    -l ratio  split the edges longer than ratio x the mean edge length first
              (vtkSurface::SplitLongEdges)
    -cd file  ACVD, ACVDQ: MetaImage volume whose values replace the curvature indicator
    -cmax v, -cmin v, -cf v
              its mapping max(cmax - value * cf, cmin) (defaults 1, 0.1, 0.001)
    -fv file  ACVDQ: vertex ids (whitespace separated) that stay output vertices
    -ft file  ACVDQ: face ids whose three vertices stay output vertices

-l, -fv and -ft act on the mesh in the order given, as the reference's argument loop
does.  The option of the reference that needs a part this package does not build,
-w (energy log), stops with an error rather than being ignored.  Other keys are ignored, as the reference programs
ignore them.

Outputs follow the reference: ACVD writes <dir>smooth_<name> before the post-placement
and <dir>/<name> after it, in the format the name's extension selects; ACVDQ writes
<dir><name> as binary PLY whatever the extension; AnisotropicRemeshingQ writes
<dir>Remeshing.ply.
"""
from __future__ import annotations

import os
import sys

import numpy as np

from . import engine as _eng
from .remesh import (AnisotropicDiscreteRemeshing, IsotropicDiscreteRemeshing, QIsotropicDiscreteRemeshing,
                     QuadricPostPlacement, Surface)

_UNBUILT = {
    "-w": "the global energy log (which the reference's ACVD / ACVDQ write through an uninitialised "
          "timer, vtkUniformClustering.h:1384-1395)",
}


def _usage(prog: str) -> str:
    return (f"Usage : {prog} file nvertices gradation [options]\n"
            "nvertices is the desired number of vertices\n"
            "gradation defines the influence of local curvature (0=uniform meshing)\n"
            "options: -b 0/1, -m 0/1, -s threshold, -o directory, -of file, -q level, -d 0")


def _parse(argv: list[str], prog: str):
    if len(argv) < 3:
        raise SystemExit(_usage(prog))
    opts = {"file": argv[0], "n": int(argv[1]), "gradation": float(argv[2])}
    rest = argv[3:]
    if len(rest) % 2:
        raise SystemExit(f"{prog}: option {rest[-1]} without a value")
    opts["_order"] = []
    for key, value in zip(rest[0::2], rest[1::2]):
        if key in _UNBUILT:
            raise SystemExit(f"{prog}: option {key} needs {_UNBUILT[key]}, which this build does not have")
        if key == "-d" and int(value) != 0:
            raise SystemExit(f"{prog}: display needs a graphics stack; only -d 0 is available")
        opts[key] = value
        opts["_order"].append((key, value))
    return opts


def _mesh_options(opts, mesh: Surface, fixed_vertices: bool):
    """-l, -fv and -ft in the order given (ACVD.cxx:151-155, ACVDQ.cxx:192-280): a split
    replaces the mesh, -ft maps face ids of the mesh as it is at that point."""
    fixed = None
    for key, value in opts.get("_order", []):
        if key == "-l":
            print(f"Splitting edges longer than {float(value)} times the average edge length")
            pts, tri = _eng.split_long_edges(mesh.points, mesh.faces, float(value))
            mesh = Surface(pts, tri)
        elif key == "-fv" and fixed_vertices:
            fixed = np.asarray(_read_ids(value), dtype=np.int32)
        elif key == "-ft" and fixed_vertices:
            faces = _read_ids(value)
            mark = np.zeros(mesh.GetNumberOfPoints(), dtype=bool)
            for f in faces:
                mark[mesh.faces[f]] = True
            fixed = np.nonzero(mark)[0].astype(np.int32)
            print(f"Added {len(faces)} constraints on triangles")
    return mesh, fixed


def _remesh(opts, cls, console: int, manifold: bool = True, fixed_vertices: bool = False, density: bool = True):
    mesh = Surface.CreateFromFile(opts["file"])
    mesh.DisplayMeshProperties()
    mesh, fixed = _mesh_options(opts, mesh, fixed_vertices)
    r = cls()
    r._cli_fixed = fixed
    r.SetForceManifold(int(opts.get("-m", 0)) if manifold else 0)
    r.SetBoundaryFixing(int(opts.get("-b", 0)))
    r.SetInput(mesh)
    r.SetNumberOfClusters(opts["n"])
    r.SetConsoleOutput(console)
    r.SetSubsamplingThreshold(int(opts.get("-s", 10)))
    r.GetMetric().SetGradation(opts["gradation"])
    if density:
        if "-cd" in opts:
            r.SetInputDensityFile(opts["-cd"])
        if "-cmax" in opts:
            r.SetMaxCustomDensity(float(opts["-cmax"]))
        if "-cmin" in opts:
            r.SetMinCustomDensity(float(opts["-cmin"]))
        if "-cf" in opts:
            r.SetCustomDensityMultiplicationFactor(float(opts["-cf"]))
    return r


def main_acvd(argv: list[str] | None = None) -> int:
    """ACVD (DiscreteRemeshing/Examples/ACVD.cxx): isotropic metric, then the quadric
    post-placement of the output vertices with -q eigenvalues."""
    argv = sys.argv[1:] if argv is None else argv
    opts = _parse(argv, "ACVD")
    level = int(opts.get("-q", 1))
    outdir = opts.get("-o")
    outfile = opts.get("-of", "simplification.ply")
    r = _remesh(opts, IsotropicDiscreteRemeshing, 2)
    r.Remesh()
    if level != 0:
        r.GetOutput().WriteToFile((outdir or "") + "smooth_" + outfile)
        QuadricPostPlacement(r, level)
        print("After Quadrics Post-processing : ")
        r.GetOutput().DisplayMeshProperties()
    r.GetOutput().WriteToFile((outdir + "/" if outdir else "") + outfile)
    return 0


def _read_ids(path: str) -> list[int]:
    """Integers read one after the other until one does not parse (`input >> id`); an
    unreadable file gives none."""
    ids = []
    try:
        with open(path) as f:
            for tok in f.read().split():
                try:
                    ids.append(int(tok))
                except ValueError:
                    break
    except OSError:
        pass
    return ids


def _fixed_vertices(opts, mesh: Surface):
    """-fv / -ft (ACVDQ.cxx:246-280): the last of them given wins; None without either."""
    return _mesh_options({"_order": [kv for kv in opts.get("_order", []) if kv[0] != "-l"]}, mesh, True)[1]


def main_acvdq(argv: list[str] | None = None) -> int:
    """ACVDQ (DiscreteRemeshing/Examples/ACVDQ.cxx): QEM metric with the unconstrained
    first phase; the output is written as binary PLY.  With -fv / -ft the fixed vertices
    are the first output vertices, anchored in place (:327-363)."""
    argv = sys.argv[1:] if argv is None else argv
    opts = _parse(argv, "ACVDQ")
    r = _remesh(opts, QIsotropicDiscreteRemeshing, 2, fixed_vertices=True)
    if "-q" in opts:
        r.GetMetric().SetQuadricsOptimizationLevel(int(opts["-q"]))
    r.SetUnconstrainedInitialization(1)
    mesh = r.GetInput()
    fixed = r._cli_fixed
    if fixed is not None:
        r.SetFixedClusters(fixed)
        r.SetNumberOfClusters(opts["n"] + len(fixed))
        print(f"Read {len(fixed)} fixed Ids")
        for i, v in enumerate(fixed):
            r.GetCluster(i).AnchorItem = int(v)
    r.Remesh()
    out = r.GetOutput()
    if fixed is not None:
        for i, v in enumerate(fixed):
            if not np.array_equal(mesh.points[v], out.points[i]):
                print(f"Error, vertex {v} has been lost")
                return 1
        print("Constraints on vertices have been checked")
    path = (opts.get("-o") or "") + opts.get("-of", "simplification.ply")
    # the reference writes with vtkPLYWriter whatever the name says
    tmp = path if ".ply" in path.lower() and ".vtk" not in path.lower() else \
        os.path.join(os.path.dirname(path) or ".", f".acvdq_{os.getpid()}.ply")
    _eng.write_mesh(tmp, out.points, out.faces)
    if tmp != path:
        os.replace(tmp, path)
    return 0


def main_anisotropic_remeshing_q(argv: list[str] | None = None) -> int:
    """AnisotropicRemeshingQ (DiscreteRemeshing/Examples/AnisotropicRemeshingQ.cxx): the
    quadric-anisotropic metric with options -s, -o, -q, -b, -d 0; the output is
    <dir>Remeshing.ply."""
    argv = sys.argv[1:] if argv is None else argv
    opts = _parse(argv, "AnisotropicRemeshingQ")
    r = _remesh(opts, AnisotropicDiscreteRemeshing, 2, manifold=False, density=False)
    if "-q" in opts:
        r.GetMetric().SetQuadricsOptimizationLevel(int(opts["-q"]))
    r.Remesh()
    _eng.write_mesh((opts.get("-o") or "") + "Remeshing.ply", r.GetOutput().points, r.GetOutput().faces)
    return 0
