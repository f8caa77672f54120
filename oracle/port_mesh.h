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

    // an empty surface of n vertices grown by add_face / add_edge (the coarse mesh of
    // BuildDelaunayTriangulation; no coordinates)
    void start(idt n) {
        nV = n; nF = 0;
        P.clear(); F.clear(); ev1.clear(); ev2.clear(); poly1.clear(); poly2.clear(); nonmanifold.clear();
        ring.assign(n, {});
    }

    // vtkSurfaceBase::AddFace -> AddPolygon (.cxx:1236-1320): edges in corner order
    idt add_face(idt a, idt b, idt c) {
        const idt f = nF++;
        F.push_back(a); F.push_back(b); F.push_back(c);
        add_edge(a, b, f); add_edge(b, c, f); add_edge(c, a, f);
        return f;
    }

    // vtkSurfaceBase::GetThirdPoint (vtkSurfaceBase.h:384-400)
    idt third_point(idt f, idt v1, idt v2) const {
        const idt v3 = F[3 * f], v4 = F[3 * f + 1], v5 = F[3 * f + 2];
        if (v1 != v3 && v2 != v3) return v3;
        if (v1 != v4 && v2 != v4) return v4;
        return v5;
    }

    // vtkSurfaceBase::IsFace (.cxx:724-764)
    idt is_face(idt v1, idt v2, idt v3) const {
        const idt e = is_edge(v1, v2);
        if (e < 0) return -1;
        const idt f1 = poly1[e], f2 = poly2[e];
        if (f1 < 0) return -1;
        if (v3 == third_point(f1, v1, v2)) return f1;
        if (f2 < 0) return -1;
        if (v3 == third_point(f2, v1, v2)) return f2;
        for (idt k = (idt)nonmanifold[e].size() - 1; k >= 0; k--)
            if (v3 == third_point(nonmanifold[e][k], v1, v2)) return nonmanifold[e][k];
        return -1;
    }

    // vtkSurfaceBase::Conquer (vtkSurfaceBase.h:402-426)
    void conquer(idt f1, idt v1, idt v2, idt& f2, idt& v3) const {
        const idt e = is_edge(v1, v2);
        if (e < 0) { f2 = -1; v3 = -1; return; }
        f2 = poly2[e];
        if (f2 == -1) { v3 = -1; return; }
        if (f2 == f1) f2 = poly1[e];
        v3 = third_point(f2, v1, v2);
    }

    // vtkSurfaceBase::IsEdgeManifold (vtkSurfaceBase.h:521-528)
    bool is_edge_manifold(idt e) const { return poly2[e] >= 0 && nonmanifold[e].empty(); }

    // vtkSurfaceBase::IsVertexManifold (.cxx:259-315), walk for walk
    bool is_vertex_manifold(idt iV) const {
        const std::vector<idt>& edges = ring[iV];
        idt remaining = (idt)edges.size();
        if (remaining < 2) return false;
        for (idt e : edges) if (!is_edge_manifold(e)) return false;
        const idt first_edge = edges[0];
        idt first_vertex = ev1[first_edge], v1 = ev2[first_edge];
        if (first_vertex == iV) first_vertex = v1;
        v1 = first_vertex;
        remaining--;
        idt f1 = poly1[first_edge], f2 = poly2[first_edge], f3;
        idt v2 = third_point(f1, iV, first_vertex);
        do {
            if (--remaining == 0) return true;
            conquer(f1, iV, v2, f3, v1);
            f1 = f3;
            v2 = v1;
        } while (f1 >= 0 && v2 != first_vertex);
        if (f2 < 0 || v2 == first_vertex) return false;
        v1 = first_vertex;
        v2 = third_point(f2, iV, first_vertex);
        do {
            if (--remaining == 0) return true;
            conquer(f2, iV, v2, f3, v1);
            f2 = f3;
            v2 = v1;
        } while (f2 >= 0 && v2 != first_vertex);
        return false;
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
