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

Remesh() first subdivides the input on the GPU while it has fewer than
SubsamplingThreshold x K vertices (CheckSubsamplingRatio, vtkSurface::Subdivide);
GetInput() is then the subdivided mesh and OriginalInput the given one.  It computes
the curvature indicator / principal directions the metric needs on the GPU
(vtkCurvatureMeasure's polynomial fitting on the original mesh, as the reference's
SamplingPreProcessing does, the indicator interpolated to the subdivided vertices);
SetCurvatureInfo supplies them instead.  Differences from the reference, by design:
the quadric-anisotropic metric on a mesh that needs subdivision is rejected (the
reference keeps the original mesh's principal-direction array and reads past its
end); display options must stay 0.
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

    @classmethod
    def CreateFromFile(cls, path: str) -> "Surface":
        """vtkSurface::CreateFromFile (Common/vtkSurface.cxx:2013-2132), triangle meshes."""
        pts, tri = _eng.read_mesh(path)
        return cls(pts, tri)

    def WriteToFile(self, path: str) -> None:
        """vtkSurface::WriteToFile (Common/vtkSurface.cxx:1958-2009)."""
        _eng.write_mesh(path, self.points, self.faces)

    def DisplayMeshProperties(self) -> None:
        print(f"Mesh with {self.GetNumberOfPoints()} vertices, {self.GetNumberOfCells()} faces, "
              f"{self.GetNumberOfEdges()} edges")


def initial_identity_sampling(n_items: int, k: int) -> np.ndarray:
    """Initial sampling type -1 (vtkUniformClustering.h:1139-1157): item i seeds cluster i
    for i < K, every other item is unassigned (label K)."""
    if not 0 < k <= n_items:
        raise _eng.AcvdError(1, "initial sampling type -1 needs 0 < NumberOfClusters <= items")
    lab = np.full(n_items, k, dtype=np.int32)
    lab[:k] = np.arange(k, dtype=np.int32)
    return lab


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
        self.OriginalInput = None
        self.NumberOfSubdivisionsBeforeClustering = 0
        self.VerticesParent1 = None
        self.VerticesParent2 = None
        self.NumberOfClusters = 0
        self.RequestedNumberOfClusters = 0
        self.SubsamplingThreshold = 10
        self.UnconstrainedInitialization = 0
        self.ConsoleOutput = 0
        self.Display = 0
        self.MaxNumberOfLoops = 5000000
        self.InitialClustering = None
        self.InitialSamplingType = 1        # vtkUniformClustering.h:108, default :1409
        self.MaxNumberOfConvergences = 1000000000   # :99, default :1406
        self._resume = False              # LoadClustering: take the clustering as computed
        self.ForceManifold = False
        self.BoundaryFixing = 0          # the constructor's value (vtkDiscreteRemeshing.h:1192)
        self.MaxNumberOfManifoldPasses = 1000
        self.Indicator = None
        self.PrincipalDirections = None
        self.Output = None
        self.Clustering = None
        self.Stats = None
        self._metric = _Metric(self)
        self._engine = None
        self._constrained_request = None
        self.FixedClusters = None         # SetFixedClusters (vtkUniformClustering.h:134)
        # custom density (vtkDiscreteRemeshing.h:80-83, defaults :1203-1206)
        self.InputDensityFile = None
        self.MaxCustomDensity = 1.0
        self.MinCustomDensity = 0.1
        self.CustomDensityMultiplicationFactor = 0.001
        self._anchors = {}                # QEM Cluster::AnchorItem, by cluster
        self.EdgeOptimization = 0          # vtkDiscreteRemeshing.h:74, default :1193 (stored, never read)
        self.OutputDirectory = None        # vtkUniformClustering.h:126, default :1412
        self.FileLoadSaveOption = 0        # vtkDiscreteRemeshing.h:67

    @classmethod
    def New(cls, device: int = 0):
        return cls(device)

    # -- setters of the reference API --
    def SetInput(self, mesh: Surface):
        self.Input = mesh
        self.OriginalInput = None
        self.NumberOfSubdivisionsBeforeClustering = 0

    def GetInput(self) -> Surface:
        return self.Input

    def SetNumberOfClusters(self, k: int):
        self.NumberOfClusters = int(k)
        self.RequestedNumberOfClusters = int(k)

    def GetNumberOfClusters(self) -> int:
        return self.NumberOfClusters

    def SetSubsamplingThreshold(self, t: int):
        self.SubsamplingThreshold = int(t)

    def SetUnconstrainedInitialization(self, on: int):
        self.UnconstrainedInitialization = int(on)

    def SetInitialClustering(self, labels):
        """Start from these labels (NumberOfClusters = unassigned); like the reference, this
        also selects initial sampling type 2 (vtkUniformClustering.h:337-342)."""
        self.InitialClustering = np.ascontiguousarray(labels, dtype=np.int32)
        self.InitialSamplingType = 2

    def SetInitialSamplingType(self, t: int):
        """InitSamples (vtkUniformClustering.h:1124-1175): 1 = weighted region growing from a
        seeded shuffle (the default), 2 = the labels of SetInitialClustering, -1 = item i seeds
        cluster i. Type 0 draws seeds from VTK's vtkMath::Random sequence, which is not
        restated here (VTK is not pinned), and is refused."""
        t = int(t)
        if t == 0:
            raise _eng.AcvdError(5, "initial sampling type 0 draws from VTK's vtkMath::Random sequence, "
                                    "which is not available; use type 1, 2 or -1")
        if t not in (-1, 1, 2):
            raise _eng.AcvdError(1, "initial sampling type must be -1, 0, 1 or 2")
        self.InitialSamplingType = t

    def SetMaxNumberOfConvergences(self, n: int):
        """Convergence events after which the minimisation stops (:99, :773-824)."""
        self.MaxNumberOfConvergences = int(n)
        if self._engine is not None:   # the cap is a context option: the next Remesh makes a new context
            self._engine.close()
            self._engine = None

    def SetMinimizeUsingEnergy(self, on):
        """Only the energy-driven loop (ProcessOneLoop, the reference's default, :1416) is
        built; the distance-driven ProcessOneLoopWithDistances (:1002-) is not."""
        if not on:
            raise _eng.AcvdError(5, "only energy minimisation (MinimizeUsingEnergy on) is available")

    def SetWriteToGlobalEnergyLog(self, on: int):
        """The per-loop energy log (ComputeAndSaveEnergy, :123, :1386-) is not written:
        only 0 is accepted; the final energy is in Stats['energy']."""
        if on:
            raise _eng.AcvdError(5, "the global energy log is not available; read Stats['energy']")

    def SetComputeAndSaveEnergy(self, on: int):
        """The setter behind SetWriteToGlobalEnergyLog (vtkUniformClustering.h:123, :307)."""
        self.SetWriteToGlobalEnergyLog(on)

    def SetEdgeOptimization(self, on: int):
        """Stored as the reference stores it (vtkDiscreteRemeshing.h:74); nothing reads it."""
        self.EdgeOptimization = int(on)

    def SetOutputDirectory(self, path):
        """Stored (vtkUniformClustering.h:126).  The reference uses it only to name the
        global energy log (:670-675), which is not written here."""
        self.OutputDirectory = None if path is None else str(path)

    def SetFileLoadSaveOption(self, on: int):
        """The reference's FileLoadSaveOption asks on standard input whether to compute the
        curvature and the clustering or load them from curvature.dat / clustering.dat
        (vtkDiscreteRemeshing.h:591-700, :885-932).  The interactive prompts are not kept:
        0 is accepted; the files are read and written by SaveCurvature / LoadCurvature /
        SaveClustering / LoadClustering."""
        if on:
            raise _eng.AcvdError(5, "FileLoadSaveOption's prompts are not available; use SaveClustering / "
                                    "LoadClustering / SaveCurvature / LoadCurvature")
        self.FileLoadSaveOption = 0

    def FixClusteringToVoronoi(self):
        """A no-op, as in the reference, whose body is commented out
        (vtkDiscreteRemeshing.h:386-423)."""

    def GetDualItemNeighbourClusters(self, face: int) -> list:
        """The distinct clusters of a dual item -- an input face when the items are vertices
        -- in the order of its vertices, unassigned vertices left out
        (vtkDiscreteRemeshing.h:956-1000, ClusteringType 1)."""
        if self.Clustering is None or self.Input is None:
            raise _eng.AcvdError(1, "no clustering")
        k = self.NumberOfClusters
        out = []
        for v in self.Input.faces[int(face)]:
            c = int(self.Clustering[int(v)])
            if c < k and c not in out:
                out.append(c)
        return out

    def GetNumberOfItems(self) -> int:
        return 0 if self.Input is None else self.Input.GetNumberOfPoints()

    def GetClusterSize(self, c: int) -> int:
        """Items in cluster c of the current clustering (ClustersSizes, :132)."""
        if self.Clustering is None:
            raise _eng.AcvdError(1, "no clustering yet: call Remesh or ProcessClustering first")
        if not 0 <= int(c) < self.NumberOfClusters:
            raise IndexError("cluster index outside [0, NumberOfClusters)")
        return int(np.count_nonzero(np.asarray(self.Clustering) == int(c)))

    def SetConsoleOutput(self, v: int):
        self.ConsoleOutput = int(v)

    def SetDisplay(self, v: int):
        if v:
            raise _eng.AcvdError(5, "display needs a graphics stack; only Display = 0 is available")
        self.Display = 0

    def SetForceManifold(self, on):
        """ForceManifold: after the clustering, add clusters next to non-manifold output
        vertices and minimise again until none is left (vtkDiscreteRemeshing.h:937-950)."""
        self.ForceManifold = bool(on)

    def SetBoundaryFixing(self, on: int):
        """Close the coarse mesh along the input's boundary (FixMeshBoundaries)."""
        self.BoundaryFixing = int(on)

    def SetInputDensityFile(self, path):
        """A MetaImage volume whose values replace the curvature indicator: at each vertex
        max(MaxCustomDensity - value * CustomDensityMultiplicationFactor, MinCustomDensity)
        (vtkDiscreteRemeshing.h:603-640)."""
        self.InputDensityFile = path

    def SetMaxCustomDensity(self, v: float):
        self.MaxCustomDensity = float(v)

    def SetMinCustomDensity(self, v: float):
        self.MinCustomDensity = float(v)

    def SetCustomDensityMultiplicationFactor(self, v: float):
        self.CustomDensityMultiplicationFactor = float(v)

    def SetFixedClusters(self, vertex_ids):
        """Cluster c < len(vertex_ids) is the cluster of vertex vertex_ids[c]: the initial
        sampling places it there and cleaning keeps its component (vtkUniformClustering.h:
        134, 439-447, 1186-1190).  None clears the list."""
        self.FixedClusters = None if vertex_ids is None else np.asarray(vertex_ids, dtype=np.int32).copy()

    def GetCluster(self, c: int) -> "_ClusterRef":
        """The cluster record whose AnchorItem ACVDQ sets (ACVDQ.cxx:333-334)."""
        if not 0 <= int(c) < self.NumberOfClusters:
            raise IndexError("cluster index outside [0, NumberOfClusters)")
        return _ClusterRef(self, int(c))

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

    def _check_subsampling_ratio(self, e, indicator):
        """CheckSubsamplingRatio (vtkDiscreteRemeshing.h:841-875): subdivide on the GPU
        while the mesh has fewer than SubsamplingThreshold x K vertices; the indicator
        (of the original mesh, or None) is carried through each level by the parent
        interpolation of vtkDiscreteRemeshing.h:731-745.  Returns the indicator of the
        mesh that is clustered."""
        mesh = self.Input
        k = self.NumberOfClusters
        levels = []
        while mesh.GetNumberOfPoints() < self.SubsamplingThreshold * k:
            if self._metric_name == "aniso":
                raise _eng.AcvdError(5, "the quadric-anisotropic metric on a mesh that needs subdivision: the "
                                        "reference does not interpolate the principal directions")
            if mesh.GetNumberOfCells() == 0 or len(levels) >= 99:
                raise _eng.AcvdError(1, "the mesh cannot be subdivided to SubsamplingThreshold x K vertices")
            if self.ConsoleOutput:
                print("Subdividing mesh")
            row, col, ev = mesh.topology()
            pts, tri, p1, p2, indicator = e.subdivide(mesh.points, mesh.faces, row, col, ev, indicator=indicator)
            levels.append((mesh.GetNumberOfPoints(), p1, p2))
            mesh = Surface(pts, tri)
        if levels:
            self.OriginalInput = self.Input
            self.Input = mesh
            self.NumberOfSubdivisionsBeforeClustering = len(levels)
            # VerticesParent1/2, indexed by vertex id (-1 for the original vertices)
            n = mesh.GetNumberOfPoints()
            self.VerticesParent1 = np.full(n, -1, dtype=np.int32)
            self.VerticesParent2 = np.full(n, -1, dtype=np.int32)
            for n0, p1, p2 in levels:
                self.VerticesParent1[n0:n0 + p1.size] = p1
                self.VerticesParent2[n0:n0 + p2.size] = p2
        return indicator

    def _prepare(self):
        if self.Input is None:
            raise _eng.AcvdError(1, "SetInput first")
        k = self.NumberOfClusters
        if k <= 0:
            raise _eng.AcvdError(1, "must set NumberOfClusters to more than zero")
        if self._engine is None:
            self._engine = _eng.Engine(self._device, max_loops=self.MaxNumberOfLoops,
                                       max_convergences=self.MaxNumberOfConvergences)
        e = self._engine
        # SamplingPreProcessing (vtkDiscreteRemeshing.h:583-753): the curvature the
        # metric needs, computed here on the GPU on the original mesh unless
        # SetCurvatureInfo gave it
        need_pd = self._metric_name == "aniso"
        on_device = None
        if self._needs_indicator() and self.Indicator is None and self.InputDensityFile and not need_pd:
            # the custom density replaces the curvature (vtkDiscreteRemeshing.h:603-640)
            src = self.OriginalInput if self.OriginalInput is not None else self.Input
            self.Indicator = _eng.density_indicator(self.InputDensityFile, src.points, self.MaxCustomDensity,
                                                    self.MinCustomDensity, self.CustomDensityMultiplicationFactor)
        if (self._needs_indicator() and self.Indicator is None) or (need_pd and self.PrincipalDirections is None):
            src = self.OriginalInput if self.OriginalInput is not None else self.Input
            row, col, ev = src.topology()
            e.set_mesh(src.points, src.faces, row, col, ev)
            on_device = src
            ind_c, pd_c = e.compute_curvature()
            if self.Indicator is None:
                self.Indicator = ind_c
            if need_pd and self.PrincipalDirections is None:
                self.PrincipalDirections = pd_c
        if self.OriginalInput is None:
            carry = self.Indicator if self._needs_indicator() else None
            if carry is not None and carry.size != self.Input.GetNumberOfPoints():
                raise _eng.AcvdError(1, "the curvature indicator needs one value per input vertex")
            carry = self._check_subsampling_ratio(e, carry)
            if carry is not None:
                self.Indicator = carry
        n = self.Input.GetNumberOfPoints()
        ind = self.Indicator if self._needs_indicator() else None
        if ind is not None and ind.size != n:
            raise _eng.AcvdError(1, "the curvature indicator needs one value per clustered vertex")
        row, col, ev = self.Input.topology()
        if on_device is not self.Input:
            e.set_mesh(self.Input.points, self.Input.faces, row, col, ev)
        e.set_metric(self._metric_name, ind, self.PrincipalDirections, self._metric.Gradation)
        e.set_level(self._metric.QuadricsOptimizationLevel)
        e.set_unconstrained_initialization(self.UnconstrainedInitialization)
        if self.InitialSamplingType == 2:
            if self.InitialClustering is None:
                raise _eng.AcvdError(1, "initial sampling type 2 needs SetInitialClustering")
            lab = self.InitialClustering
        elif self.InitialSamplingType == -1:
            lab = initial_identity_sampling(n, k)
        else:
            w = _eng.vertex_weights(self._metric_name, self.Input.points, self.Input.faces, ind,
                                    self._metric.Gradation)
            lab = _eng.initial_sampling(row, col, w, k, fixed=self.FixedClusters)
        e.set_labels(k, lab)
        if self.FixedClusters is not None:
            e.set_fixed_clusters(self.FixedClusters)
        if self._anchors:
            anchors = np.full(max(self._anchors) + 1, -1, dtype=np.int32)
            for c, v in self._anchors.items():
                anchors[c] = v
            e.set_anchor_items(anchors)
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
        """The coarse mesh (vtkDiscreteRemeshing.h:1003-1112): one vertex per cluster at
        its metric centroid (the first non-empty cluster's for an empty one), stored
        float-rounded as the output's float vtkPoints holds it, and the dual triangles."""
        e = self._engine
        cl = e.clusters()
        sizes = cl["size"]
        verts = cl["centroid"].copy()
        nonempty = np.nonzero(sizes > 0)[0]
        valid = int(nonempty[0]) if nonempty.size else 0
        verts[sizes == 0] = verts[valid]
        self.Output = Surface(verts.astype(np.float32).astype(np.float64), e.dual_mesh())
        self.Energy = cl["energy_total"]
        return self.Output

    def _force_manifold(self):
        """Remesh()'s ForceManifold loop (vtkDiscreteRemeshing.h:937-950): while
        DetectNonManifoldOutputVertices finds issues, MinimizeEnergy again with the
        other clusters frozen."""
        e = self._engine
        passes = 0
        while True:
            n = self.DetectNonManifoldOutputVertices()
            if n == 0:
                break
            if self.ConsoleOutput:
                print(f"{n} topology issues, restarting minimization")
            st = e.minimize()
            for key in ("sweeps", "moves", "device_ms"):
                if self.Stats is not None and key in self.Stats:
                    self.Stats[key] += st[key]
            passes += 1
            if passes >= self.MaxNumberOfManifoldPasses:
                raise _eng.AcvdError(3, f"ForceManifold: issues left after {passes} passes")
        self.NumberOfManifoldPasses = passes
        self.NumberOfClusters = e.k
        self.Clustering = e.labels()

    def DetectNonManifoldOutputVertices(self) -> int:
        """One detection pass of the ForceManifold loop (vtkDiscreteRemeshing.h:166-383) on
        the current clustering: the issues found, with the reference's side effects (the
        new clusters, the frozen set) applied to the context."""
        if self._engine is None:
            raise _eng.AcvdError(1, "no clustering: call ProcessClustering or Remesh first")
        return self._engine.force_manifold_step()

    def FixMeshBoundaries(self) -> bool:
        """FixMeshBoundaries (vtkDiscreteRemeshing.h:426-579): appends the boundary
        vertices and faces to GetOutput(); True when it added any."""
        if not self.BoundaryFixing:
            return False
        pts, tri = self._engine.fix_mesh_boundaries()
        if pts.shape[0] == 0 and tri.shape[0] == 0:
            return False
        self.Output = Surface(np.concatenate([self.Output.points, pts]), np.concatenate([self.Output.faces, tri]))
        return pts.shape[0] > 0

    def Remesh(self):
        if self._resume:
            e = self._prepare()                    # uploads the loaded clustering
            self.Clustering = e.labels()
            self.Stats = None
        else:
            self.ProcessClustering()
        if self.ForceManifold:
            self._force_manifold()
        self.BuildDelaunayTriangulation()
        self.FixMeshBoundaries()

    def GetOutput(self) -> Surface:
        return self.Output

    def GetClustering(self) -> np.ndarray:
        return self.Clustering

    def GetBoundaryEdges(self) -> np.ndarray:
        return self._engine.boundary_edges()

    # -- checkpoint / resume: the reference's FileLoadSaveOption files
    # (vtkDiscreteRemeshing.h:899-932 clustering.dat, :655-700 curvature.dat), raw
    # native-endian int32 / float64 per item, without the interactive prompts --
    def SaveClustering(self, path: str = "clustering.dat") -> None:
        if self.Clustering is None:
            raise _eng.AcvdError(1, "no clustering to save")
        np.ascontiguousarray(self.Clustering, dtype=np.int32).tofile(path)

    def LoadClustering(self, path: str = "clustering.dat") -> np.ndarray:
        """Reads a clustering written by SaveClustering (or the reference): the next
        Remesh() takes it as computed and skips the minimisation, as the reference's load
        path does (Init, read, ReComputeStatistics, then the coarse mesh).  The number of
        values must match the mesh that is clustered (after any subdivision)."""
        lab = np.fromfile(path, dtype=np.int32)
        self.SetInitialClustering(lab)
        self._resume = True
        return lab

    def SaveCurvature(self, path: str = "curvature.dat") -> None:
        if self.Indicator is None:
            raise _eng.AcvdError(1, "no curvature indicator to save")
        np.ascontiguousarray(self.Indicator, dtype=np.float64).tofile(path)

    def LoadCurvature(self, path: str = "curvature.dat") -> np.ndarray:
        ind = np.fromfile(path, dtype=np.float64)
        self.SetCurvatureInfo(ind, self.PrincipalDirections)
        return ind


class _ClusterRef:
    """GetCluster(c): the metric's cluster record, here its AnchorItem only -- a member of
    the QEM metric's clusters (vtkQEMetricForClustering.h:127-128), -1 when unset."""

    def __init__(self, owner: _DiscreteRemeshing, c: int):
        self._owner = owner
        self._c = c

    @property
    def AnchorItem(self) -> int:
        self._check()
        return self._owner._anchors.get(self._c, -1)

    @AnchorItem.setter
    def AnchorItem(self, v: int):
        self._check()
        v = int(v)
        if v < -1:
            raise ValueError("AnchorItem is a vertex id, or -1")
        if v == -1:
            self._owner._anchors.pop(self._c, None)
        else:
            self._owner._anchors[self._c] = v

    def _check(self):
        if self._owner._metric_name != "qem":
            raise AttributeError("AnchorItem is a member of the QEM metric's clusters only")


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
    # the driver moves its NumberOfSamples vertices only (clusters ForceManifold added and
    # FixMeshBoundaries' vertices keep their place) and stores them in the output's float
    # vtkPoints
    k = min(remesh.RequestedNumberOfClusters, pts.shape[0])
    out = remesh.Output.points.copy()
    out[:k] = pts[:k].astype(np.float32).astype(np.float64)
    remesh.Output.points = out
    return remesh.Output


# the reference's class names
vtkIsotropicDiscreteRemeshing = IsotropicDiscreteRemeshing
vtkQIsotropicDiscreteRemeshing = QIsotropicDiscreteRemeshing
vtkAnisotropicDiscreteRemeshing = AnisotropicDiscreteRemeshing
vtkSurface = Surface
