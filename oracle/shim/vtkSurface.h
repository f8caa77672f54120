// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// Stand-in for the reference's vtkSurface (Common/vtkSurface.h), which derives
// from VTK's vtkPolyData.  It exposes only the members the clustering headers
// call, on top of the restated edge table in ../port_mesh.h (edge numbering and
// vertex-ring order as in Common/vtkSurfaceBase.cxx:1166-1221,1407-1468).
#pragma once
#include "vtk_shim.h"
#include "../port_mesh.h"

class vtkSurface : public vtkPolyData {
public:
    static vtkSurface* New() { return new vtkSurface; }

    void CreateFromArrays(vtkIdType nV, const double* pts, vtkIdType nF, const int* tri) {
        M.build(nV, pts, nF, tri);
        for (int k = 0; k < 3; k++) { Pts.B[2 * k] = 1e300; Pts.B[2 * k + 1] = -1e300; }
        for (vtkIdType v = 0; v < nV; v++)
            for (int k = 0; k < 3; k++) {
                Pts.B[2 * k] = std::min(Pts.B[2 * k], pts[3 * v + k]);
                Pts.B[2 * k + 1] = std::max(Pts.B[2 * k + 1], pts[3 * v + k]);
            }
        Faces.assign(M.F.begin(), M.F.end());
        Ring.resize(nV);
        for (vtkIdType v = 0; v < nV; v++) Ring[v].assign(M.ring[v].begin(), M.ring[v].end());
    }
    void CreateFromPolyData(vtkPolyData*) {
        std::cerr << "shim vtkSurface: CreateFromPolyData is not available" << std::endl;
        std::abort();
    }

    vtkIdType GetNumberOfPoints() { return M.nV; }
    // the point set's bounding box (vtkCurvatureMeasure reads it)
    vtkPoints* GetPoints() { return &Pts; }
    vtkIdType GetNumberOfCells() { return M.nF; }
    vtkIdType GetNumberOfEdges() { return M.n_edges(); }
    bool IsFaceActive(vtkIdType) { return true; }

    void GetFaceVertices(vtkIdType f, vtkIdType& n, vtkIdType*& v) { n = 3; v = Faces.data() + 3 * f; }
    void GetFaceVertices(vtkIdType f, vtkIdType& v1, vtkIdType& v2, vtkIdType& v3) {
        v1 = Faces[3 * f]; v2 = Faces[3 * f + 1]; v3 = Faces[3 * f + 2];
    }
    void GetEdgeVertices(vtkIdType e, vtkIdType& v1, vtkIdType& v2) { v1 = M.ev1[e]; v2 = M.ev2[e]; }
    void GetEdgeFaces(vtkIdType e, vtkIdType& f1, vtkIdType& f2) { f1 = M.poly1[e]; f2 = M.poly2[e]; }
    // the faces of an edge as a list (the face-clustering branch of GetEdgeItemsSure,
    // compiled in the threaded engine, never run for vertex clustering)
    void GetEdgeFaces(vtkIdType e, vtkIdList* out) {
        out->Reset();
        if (M.poly1[e] >= 0) out->InsertNextId(M.poly1[e]);
        if (M.poly2[e] >= 0) out->InsertNextId(M.poly2[e]);
    }
    void GetVertexNeighbourEdges(vtkIdType v, vtkIdType& n, vtkIdType*& e) {
        n = (vtkIdType)Ring[v].size(); e = Ring[v].data();
    }
    void GetVertexNeighbourEdges(vtkIdType v, vtkIdList* out) {
        out->Reset();
        for (vtkIdType e : Ring[v]) out->InsertNextId(e);
    }
    void GetVertexNeighbours(vtkIdType v, vtkIdList* out) {
        out->Reset();
        std::vector<port::idt> nb;
        M.vertex_neighbours(v, nb);
        for (port::idt x : nb) out->InsertNextId(x);
    }
    void GetVertexNeighbourFaces(vtkIdType v, vtkIdList* out) {
        out->Reset();
        std::vector<port::idt> fl;
        M.vertex_faces(v, fl);
        for (port::idt x : fl) out->InsertNextId(x);
    }
    int GetValence(vtkIdType v) { return (int)Ring[v].size(); }
    void GetPoint(vtkIdType i, double* p) { M.point(i, p); }
    void GetPointCoordinates(vtkIdType i, double* p) { M.point(i, p); }
    double GetFaceArea(vtkIdType f) { return M.face_area(f); }
    // vtkSurface::GetCellMassProperties (Common/vtkSurface.cxx:1380-1419), triangles:
    // area-weighted vertex mean, divided by the area when it is positive
    void GetCellMassProperties(vtkIdType f, double& area, double* bary) {
        double p1[3], p2[3], p3[3];
        M.point(Faces[3 * f], p1); M.point(Faces[3 * f + 1], p2); M.point(Faces[3 * f + 2], p3);
        area = 0;
        bary[0] = bary[1] = bary[2] = 0;
        const double a2 = rmath::tri_area(p1, p2, p3);
        for (int i = 0; i < 3; i++) bary[i] += a2 * (p1[i] + p2[i] + p3[i]) / 3.0;
        area += a2;
        if (area > 0)
            for (int i = 0; i < 3; i++) bary[i] /= area;
    }
    vtkIdType IsEdge(vtkIdType a, vtkIdType b) { return M.is_edge(a, b); }
    vtkIdType GetThirdPoint(vtkIdType f, vtkIdType a, vtkIdType b) {
        for (int j = 0; j < 3; j++) {
            const vtkIdType v = Faces[3 * f + j];
            if (v != a && v != b) return v;
        }
        return -1;
    }
    vtkDoubleArray* GetEdgeLengths() {
        std::cerr << "shim vtkSurface: GetEdgeLengths (display only) is not available" << std::endl;
        std::abort();
    }
    double GetVertexArea(vtkIdType v) { return M.vertex_area(v); }
    vtkDoubleArray* GetVerticesAreas() {
        if (!Areas) {
            Areas = vtkDoubleArray::New();
            Areas->SetNumberOfValues(M.nV);
            for (vtkIdType i = 0; i < M.nV; i++) Areas->SetValue(i, M.vertex_area(i));
        }
        return Areas;
    }
    ~vtkSurface() override { if (Areas) Areas->Delete(); }

    port::Mesh M;
private:
    vtkPoints Pts;
    std::vector<vtkIdType> Faces;
    std::vector<std::vector<vtkIdType>> Ring;
    vtkDoubleArray* Areas = nullptr;
};
