// Selects the GPU solvers in the reference simulator's solver factory.
//
// Compile the reference's src/Simulation.cpp, unmodified, with
//     -include sph_gpu_select.h
// and Simulation::setSimulationMethod (src/Simulation.cpp:207-231) creates
// GpuWCSPHSolver / GpuPCISPHSolver / GpuDFSPHSolver for the method ids 0, 1
// and 2; importScene's setters (src/Simulation.cpp:354-378) cast to the
// same classes, which derive from the CPU solvers.  The reference's solver
// headers are included first, so their include guards keep the class
// definitions as they are; only the names the translation unit writes after
// this header are redirected.  The three lines a maintainer would otherwise
// change in setSimulationMethod are exactly these substitutions.
#pragma once

#include "DFSPHSolver.h"
#include "PCISPHSolver.h"
#include "WCSPHSolver.h"
#include "sph_gpu_solvers.h"

#define WCSPHSolver GpuWCSPHSolver
#define PCISPHSolver GpuPCISPHSolver
#define DFSPHSolver GpuDFSPHSolver
