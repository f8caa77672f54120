"""Python mirror of the reference's remeshing API for the clustering path.

Same class and method names as the reference's C++ classes
(DiscreteRemeshing/vtkIsotropicDiscreteRemeshing.h:55-102,
vtkAnisotropicDiscreteRemeshing.h:49-71), backed by the GPU engine:

    mesh = Surface(points, faces)
    r = QIsotropicDiscreteRemeshing()            # ACVDQ
    r.SetInput(mesh)
    r.SetNumberOfClusters(20000)
    r.SetSubsamplingThreshold(10)
    r.GetMetric().SetGradation(1.5)
    r.SetCurvatureInfo(indicator)                # optional: otherwise computed on the GPU
    r.SetUnconstrainedInitialization(1)
    r.Remesh()
    coarse = r.GetOutput()                       # Surface
    labels = r.GetClustering()

Remesh() computes the curvature indicator / principal directions the metric needs
on the GPU (vtkCurvatureMeasure's polynomial fitting, as the reference's
SamplingPreProcessing does); SetCurvatureInfo supplies them instead.  Differences
from the reference, by design: meshes that would need subdivision
(N < threshold * K) are rejected; display options must stay 0.
"""
from __future__ import annotations

import numpy as np

from . import engine as _eng


class Surface:
    """Triangle mesh with the reference's edge numbering (vtkSurface subset)."""

    def __init__(self, points, faces):
        self.points = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        self.faces = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
        self._topo = None

    def GetNumberOfPoints(self) -> int:
        return int(self.points.shape[0])

    def GetNumberOfCells(self) -> int:
        return int(self.faces.shape[0])

    def topology(self):
        if self._topo is None:
            self._topo = _eng.build_topology(self.GetNumberOfPoints(), self.faces)
        return self._topo

    def GetNumberOfEdges(self) -> int:
        return int(self.topology()[2].shape[0])

    def GetPointCoordinates(self, i: int):
        return self.points[i].copy()


class _Metric:
    def __init__(self, owner):
        self._o = owner
        self.Gradation = 0.0
        self.QuadricsOptimizationLevel = 3

    def SetGradation(self, g: float):
        self.Gradation = float(g)

    def GetGradation(self) -> float:
        return self.Gradation

    def SetQuadricsOptimizationLevel(self, level: int):
        self.QuadricsOptimizationLevel = int(level)

    def SetConstrainedClustering(self, c: int):
        self._o._constrained_request = int(c)


class _DiscreteRemeshing:
    _metric_name = "iso"

    def __init__(self, device: int = 0):
        self._device = device
        self.Input = None
        self.NumberOfClusters = 0
        self.SubsamplingThreshold = 10
        self.UnconstrainedInitialization = 0
        self.ConsoleOutput = 0
        self.Display = 0
        self.MaxNumberOfLoops = 5000000
        self.InitialClustering = None
        self.Indicator = None
        self.PrincipalDirections = None
        self.Output = None
        self.Clustering = None
        self.Stats = None
        self._metric = _Metric(self)
        self._engine = None
        self._constrained_request = None

    @classmethod
    def New(cls, device: int = 0):
        return cls(device)

    # -- setters of the reference API --
    def SetInput(self, mesh: Surface):
        self.Input = mesh

    def GetInput(self) -> Surface:
        return self.Input

    def SetNumberOfClusters(self, k: int):
        self.NumberOfClusters = int(k)

    def GetNumberOfClusters(self) -> int:
        return self.NumberOfClusters

    def SetSubsamplingThreshold(self, t: int):
        self.SubsamplingThreshold = int(t)

    def SetUnconstrainedInitialization(self, on: int):
        self.UnconstrainedInitialization = int(on)

    def SetInitialClustering(self, labels):
        self.InitialClustering = np.ascontiguousarray(labels, dtype=np.int32)

    def SetConsoleOutput(self, v: int):
        self.ConsoleOutput = int(v)

    def SetDisplay(self, v: int):
        if v:
            raise _eng.AcvdError(5, "display needs a graphics stack; only Display = 0 is available")
        self.Display = 0

    def SetMaxNumberOfLoops(self, n: int):
        self.MaxNumberOfLoops = int(n)

    def SetCurvatureInfo(self, indicator, principal_dirs=None):
        self.Indicator = None if indicator is None else np.ascontiguousarray(indicator, dtype=np.float64)
        self.PrincipalDirections = (None if principal_dirs is None
                                    else np.ascontiguousarray(principal_dirs, dtype=np.float32).reshape(-1, 6))

    def GetMetric(self) -> _Metric:
        return self._metric

    # -- processing --
    def _needs_indicator(self) -> bool:
        g = self._metric.Gradation
        return g != 0.0 if self._metric_name == "aniso" else g > 0.0

    def _prepare(self):
        if self.Input is None:
            raise _eng.AcvdError(1, "SetInput first")
        k = self.NumberOfClusters
        if k <= 0:
            raise _eng.AcvdError(1, "must set NumberOfClusters to more than zero")
        n = self.Input.GetNumberOfPoints()
        if n < self.SubsamplingThreshold * k:
            raise _eng.AcvdError(5, f"{n} vertices < SubsamplingThreshold * K = {self.SubsamplingThreshold * k}: "
                                    "the input would need subdivision, which this build does not do")
        row, col, ev = self.Input.topology()
        if self._engine is None:
            self._engine = _eng.Engine(self._device, max_loops=self.MaxNumberOfLoops)
        e = self._engine
        e.set_mesh(self.Input.points, self.Input.faces, row, col, ev)
        # SamplingPreProcessing (vtkDiscreteRemeshing.h:583-700): the curvature the
        # metric needs, computed here (on the GPU) unless SetCurvatureInfo gave it
        need_pd = self._metric_name == "aniso"
        if (self._needs_indicator() and self.Indicator is None) or (need_pd and self.PrincipalDirections is None):
            ind_c, pd_c = e.compute_curvature()
            if self.Indicator is None:
                self.Indicator = ind_c
            if need_pd and self.PrincipalDirections is None:
                self.PrincipalDirections = pd_c
        ind = self.Indicator if self._needs_indicator() else None
        e.set_metric(self._metric_name, ind, self.PrincipalDirections, self._metric.Gradation)
        e.set_level(self._metric.QuadricsOptimizationLevel)
        e.set_unconstrained_initialization(self.UnconstrainedInitialization)
        if self.InitialClustering is not None:
            lab = self.InitialClustering
        else:
            w = _eng.vertex_weights(self._metric_name, self.Input.points, self.Input.faces, ind,
                                    self._metric.Gradation)
            lab = _eng.initial_sampling(row, col, w, k)
        e.set_labels(k, lab)
        return e

    def ProcessClustering(self):
        e = self._prepare()
        self.Stats = e.minimize()
        self.Clustering = e.labels()
        if self.ConsoleOutput:
            print(f"The clustering took :{self.Stats['device_ms'] / 1000.0} seconds.")
            print(f"Number of loops:\t{self.Stats['sweeps']}")
        return self.Clustering

    def BuildDelaunayTriangulation(self):
        e = self._engine
        cl = e.clusters()
        sizes = cl["size"]
        verts = cl["centroid"].copy()
        nonempty = np.nonzero(sizes > 0)[0]
        valid = int(nonempty[0]) if nonempty.size else 0
        verts[sizes == 0] = verts[valid]
        self.Output = Surface(verts, e.dual_mesh())
        self.Energy = cl["energy_total"]
        return self.Output

    def Remesh(self):
        self.ProcessClustering()
        self.BuildDelaunayTriangulation()

    def GetOutput(self) -> Surface:
        return self.Output

    def GetClustering(self) -> np.ndarray:
        return self.Clustering

    def GetBoundaryEdges(self) -> np.ndarray:
        return self._engine.boundary_edges()


class IsotropicDiscreteRemeshing(_DiscreteRemeshing):
    """vtkIsotropicDiscreteRemeshing (ACVD): isotropic metric."""
    _metric_name = "iso"


class QIsotropicDiscreteRemeshing(_DiscreteRemeshing):
    """vtkQIsotropicDiscreteRemeshing (ACVDQ): quadric error metric."""
    _metric_name = "qem"


class AnisotropicDiscreteRemeshing(_DiscreteRemeshing):
    """vtkAnisotropicDiscreteRemeshing: quadric-anisotropic metric."""
    _metric_name = "aniso"


def QuadricPostPlacement(remesh: _DiscreteRemeshing, level: int = 1) -> Surface:
    """The ACVD driver's step after Remesh() (DiscreteRemeshing/Examples/ACVD.cxx:217-291,
    run there when QuadricsOptimizationLevel != 0; its default is 1): every output
    vertex moves to the point minimising the summed plane quadrics of the faces
    around its cluster's items.  Updates remesh.GetOutput() in place and returns it."""
    if level == 0:
        return remesh.Output
    pts = remesh._engine.post_placement(level)
    remesh.Output.points = pts
    return remesh.Output


# the reference's class names
vtkIsotropicDiscreteRemeshing = IsotropicDiscreteRemeshing
vtkQIsotropicDiscreteRemeshing = QIsotropicDiscreteRemeshing
vtkAnisotropicDiscreteRemeshing = AnisotropicDiscreteRemeshing
vtkSurface = Surface
