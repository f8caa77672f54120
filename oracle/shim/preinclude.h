// ORACLE / TEST INFRASTRUCTURE ONLY.
// Force-included (g++ -include) ahead of every reference translation unit: it
// brings in the shim's vtkSurface and headless RenderWindow and defines the
// include guards of the reference's VTK-bound Common/vtkSurface.h,
// Common/vtkSurfaceBase.h and Common/RenderWindow.h, so that those files are
// skipped when the reference headers include them by relative path.
#pragma once
#include "vtkSurface.h"
#include "RenderWindow.h"
#define __vtkSurface_h
#define __vtkSurfaceBase_h
#define _RENDERWINDOW_H_
