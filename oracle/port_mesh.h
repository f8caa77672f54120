// ORACLE / TEST INFRASTRUCTURE ONLY.
// Mesh connectivity restated from Common/vtkSurfaceBase.cxx and the area/quadric
// helpers of Common/vtkSurface.cxx / Common/vtkQuadricTools.cxx.  Shared by the
// C++ restatement (acvd_port.cpp) and the shim's vtkSurface (shim/vtkSurface.h),
// so both see the same edge numbering and vertex-ring order.
#pragma once
#include <vector>
#include "restated_math.h"

namespace port {

typedef long long idt;

// ---------------------------------------------------------------------------
// Edge-oriented triangle mesh (Common/vtkSurfaceBase.cxx:1166-1221 AddEdge,
// :1057-1068 InsertEdgeInRing, :1407-1468 CreateFromPolyData)
// ---------------------------------------------------------------------------
struct Mesh {
    idt nV = 0, nF = 0;
    std::vector<double> P;                 // 3 nV
    std::vector<idt> F;                    // 3 nF
    std::vector<idt> ev1, ev2, poly1, poly2;
    std::vector<std::vector<idt>> nonmanifold;  // per edge, extra faces (rare)
    std::vector<std::vector<idt>> ring;    // per vertex: incident edge ids, creation order

    idt n_edges() const { return (idt)ev1.size(); }

    idt is_edge(idt v1, idt v2) const {
        const std::vector<idt>& r = ring[v1];
        for (idt k = (idt)r.size() - 1; k >= 0; k--) {
            const idt e = r[k];
            if (v2 == ev1[e] || v2 == ev2[e]) return e;
        }
        return -1;
    }

    void add_edge(idt v1, idt v2, idt f) {
        if (v1 == v2) return;
        idt e = is_edge(v1, v2);
        if (e >= 0) {
            if (poly1[e] < 0) { poly1[e] = f; return; }
            if (poly2[e] >= 0) { nonmanifold[e].push_back(f); return; }
            poly2[e] = f;
            return;
        }
        e = (idt)ev1.size();
        ev1.push_back(v1); ev2.push_back(v2); poly1.push_back(f); poly2.push_back(-1);
        nonmanifold.emplace_back();
        insert_in_ring(e, v1);
        insert_in_ring(e, v2);
    }

    void insert_in_ring(idt e, idt v) {
        std::vector<idt>& r = ring[v];
        for (idt x : r) if (x == e) return;
        r.push_back(e);
    }

    void build(idt nv, const double* pts, idt nf, const int* tri) {
        nV = nv; nF = nf;
        P.assign(pts, pts + 3 * nv);
        F.resize(3 * nf);
        for (idt i = 0; i < 3 * nf; i++) F[i] = tri[i];
        ring.assign(nv, {});
        for (idt f = 0; f < nf; f++) {
            const idt* v = &F[3 * f];
            if (v[0] == v[1]) continue;  // inactive face (vtkSurfaceBase.cxx:1439)
            for (int j = 0; j < 3; j++) add_edge(v[j], v[(j + 1) % 3], f);
        }
    }

    void point(idt i, double* p) const { p[0] = P[3 * i]; p[1] = P[3 * i + 1]; p[2] = P[3 * i + 2]; }

    // vtkSurfaceBase::GetVertexNeighbourFaces (.cxx:964-984)
    void vertex_faces(idt v, std::vector<idt>& out) const {
        out.clear();
        auto ins = [&](idt f) { for (idt x : out) if (x == f) return; out.push_back(f); };
        for (idt e : ring[v]) {
            if (poly1[e] >= 0) ins(poly1[e]);
            if (poly2[e] >= 0) ins(poly2[e]);
            for (idt f : nonmanifold[e]) ins(f);
        }
    }

    // vtkSurfaceBase::GetVertexNeighbours (.cxx:988-1000)
    void vertex_neighbours(idt v, std::vector<idt>& out) const {
        out.clear();
        for (idt e : ring[v]) out.push_back(ev1[e] == v ? ev2[e] : ev1[e]);
    }

    // vtkSurface::GetFaceArea (.cxx:1319-1340), triangles only
    double face_area(idt f) const {
        double a[3], b[3], c[3];
        point(F[3 * f], a); point(F[3 * f + 1], b); point(F[3 * f + 2], c);
        return rmath::tri_area(a, b, c);
    }

    // vtkSurface::GetVertexArea (.cxx:1342-1359)
    double vertex_area(idt v) const {
        std::vector<idt> fl;
        vertex_faces(v, fl);
        double area = 0;
        for (idt f : fl) area += face_area(f) / 3.0;
        return area;
    }

    // vtkQuadricTools::AddTriangleQuadric with FullQuadric=false (.cxx:56-79)
    void add_triangle_quadric(double* Q, idt f) const {
        double x1[3], x2[3], x3[3], q[4][4];
        point(F[3 * f], x1); point(F[3 * f + 1], x2); point(F[3 * f + 2], x3);
        rmath::tri_quadric(x1, x2, x3, q);
        Q[0] += q[0][0]; Q[1] += q[0][1]; Q[2] += q[0][2]; Q[3] += q[0][3];
        Q[4] += q[1][1]; Q[5] += q[1][2]; Q[6] += q[1][3]; Q[7] += q[2][2]; Q[8] += q[2][3];
    }
};

}  // namespace port
