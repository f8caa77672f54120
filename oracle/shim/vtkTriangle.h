// ORACLE shim: forwards to vtk_shim.h
#pragma once
#include "vtk_shim.h"
