// ORACLE / TEST INFRASTRUCTURE ONLY.
// Headless stand-in for the reference's VTK/OpenGL RenderWindow (Common/RenderWindow.h).
// There is no graphics stack on either machine; every run uses Display = 0, so
// these members only have to exist.
#pragma once
#include "vtk_shim.h"

class vtkSurface;

class RenderWindow : public vtkObject {
public:
    static RenderWindow* New() { return new RenderWindow; }
    void SetInputData(vtkPolyData*) {}
    void SetInputEdges(vtkPolyData*) {}
    void AttachToRenderWindow(RenderWindow*) {}
    void DisplayRandomColors(int) {}
    void DisplayInputEdges() {}
    void Render() {}
    void SetWindowName(const char*) {}
    void Interact() {}
    void Capture(const char*) {}
    void SetLookupTable(vtkLookupTable* = nullptr) {}
};
