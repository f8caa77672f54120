"""The reference-side binding (include/vtkGPUClustering.h) against the reference.

Compiles the binding together with the reference's own clustering headers (the
VTK shim stands in for VTK) and links it with libacvd_gb300.so, for all three
metric plugins.  The program then runs the reference's own ProcessClustering()
with the GPU engine in place of MinimizeEnergy(): on a machine without a GPU it
must stop with the C ABI's error (no CPU fallback); with a GPU it must return
a clustering.  Only where the reference tree is present.
"""
import os
import shutil
import subprocess
import textwrap

import pytest

from acvd_gb300 import build as cuda_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("ACVD_REFERENCE_ROOT", "/root/reference")

PROGRAM = textwrap.dedent(r"""
    #include "vtkSurfaceClustering.h"
    #include "vtkVerticesProcessing.h"
    #include "vtkIsotropicMetricForClustering.h"
    #include "vtkQEMetricForClustering.h"
    #include "vtkQuadricAnisotropicMetricForClustering.h"
    #include "vtkGPUClustering.h"
    #include <cstdio>
    typedef vtkGPUMetric<vtkQEMetricForClustering> GQ;
    typedef vtkGPUClustering<vtkVerticesProcessing<vtkSurfaceClustering<GQ> >, GQ> GPUQ;
    typedef vtkGPUMetric<vtkIsotropicMetricForClustering> GI;
    typedef vtkGPUClustering<vtkVerticesProcessing<vtkSurfaceClustering<GI> >, GI> GPUI;
    typedef vtkGPUMetric<vtkQuadricAnisotropicMetricForClustering> GA;
    typedef vtkGPUClustering<vtkVerticesProcessing<vtkSurfaceClustering<GA> >, GA> GPUA;
    int main() {
        static_assert(GQ::acvd_metric == ACVD_METRIC_QEM, "qem");
        static_assert(GI::acvd_metric == ACVD_METRIC_ISOTROPIC, "iso");
        static_assert(GA::acvd_metric == ACVD_METRIC_QUADRIC_ANISOTROPIC, "aniso");
        // AnchorItem is forwarded for the QEM metric's clusters only
        static_assert(acvd_has_anchor<GQ::Cluster>::value, "qem anchors");
        static_assert(!acvd_has_anchor<GI::Cluster>::value, "iso has no anchors");
        static_assert(!acvd_has_anchor<GA::Cluster>::value, "aniso has no anchors");
        GPUI::New()->Delete();   // instantiates the iso engine's MinimizeEnergy too
        // octahedron subdivided once: 18 vertices, 32 faces
        const double P[18][3] = {{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{0,0,1},{0,0,-1},
            {.7,.7,0},{-.7,.7,0},{-.7,-.7,0},{.7,-.7,0},{.7,0,.7},{0,.7,.7},{-.7,0,.7},{0,-.7,.7},
            {.7,0,-.7},{0,.7,-.7},{-.7,0,-.7},{0,-.7,-.7}};
        const int T[8][3] = {{0,2,4},{2,1,4},{1,3,4},{3,0,4},{2,0,5},{1,2,5},{3,1,5},{0,3,5}};
        auto mid = [](int a, int b) -> int {
            const int e[12][3] = {{0,2,6},{2,1,7},{1,3,8},{3,0,9},{0,4,10},{2,4,11},{1,4,12},{3,4,13},
                                  {0,5,14},{2,5,15},{1,5,16},{3,5,17}};
            for (auto& r : e) if ((r[0]==a && r[1]==b) || (r[0]==b && r[1]==a)) return r[2];
            return -1; };
        std::vector<int> tri;
        for (auto& t : T) {
            int a = t[0], b = t[1], c = t[2], ab = mid(a,b), bc = mid(b,c), ca = mid(c,a);
            int q[4][3] = {{a,ab,ca},{b,bc,ab},{c,ca,bc},{ab,bc,ca}};
            for (auto& f : q) for (int j = 0; j < 3; j++) tri.push_back(f[j]);
        }
        vtkSurface* mesh = vtkSurface::New();
        mesh->CreateFromArrays(18, &P[0][0], 32, tri.data());
        GPUQ* r = GPUQ::New();
        r->SetInput(mesh);
        r->SetNumberOfClusters(3);
        r->SetUnconstrainedInitialization(1);
        int rc = 0;
        try {
            r->ProcessClustering();
            std::printf("clustered: %d sweeps\n", r->GetLastStats().sweeps);
        } catch (const std::exception& e) {
            std::printf("GPU engine error: %s\n", e.what());
            rc = 3;
        }
        r->Delete();
        mesh->Delete();
        return rc;
    }
""")


def test_binding_compiles_and_runs_reference_flow(tmp_path, oracle_lib):
    if not os.path.isdir(os.path.join(REF, "Common")):
        pytest.skip("reference tree not present")
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    lib = cuda_build.build()
    src = tmp_path / "binding.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "binding"
    cmd = ["g++", "-std=c++17", "-w", "-include", os.path.join(ROOT, "oracle", "shim", "preinclude.h"),
           "-I" + os.path.join(ROOT, "oracle", "shim"), "-I" + os.path.join(REF, "Common"),
           "-I" + os.path.join(REF, "DiscreteRemeshing"), "-I" + os.path.join(ROOT, "include"),
           str(src), os.path.join(REF, "Common", "vtkQuadricTools.cxx"),
           "-L" + os.path.dirname(lib), "-lacvd_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    if r.returncode == 3:
        assert "GPU engine error" in r.stdout and "CUDA" in r.stdout
    else:
        assert r.returncode == 0, r.stdout + r.stderr
        assert "clustered" in r.stdout
