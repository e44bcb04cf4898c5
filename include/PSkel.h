// PSkel drop-in for GB300: umbrella header.
//
// Include this instead of the reference's PSkel.h (PSkel.h:57-106). It pulls
// in the same API (Array*, Mask*, Args*, Stencil2D/3D) backed by
// libpskel_gb300.so; link with -lpskel_gb300 -lcudart. Applications that use
// their own stencilKernel functors must be compiled with nvcc
// (-gencode arch=compute_103a,code=sm_103a -std=c++17); define PSKEL_OMP (and
// compile with OpenMP) to keep the host runIterativeCPU methods.
#ifndef PSKEL_H
#define PSKEL_H

#include <cstdio>
#include <cstdlib>
#include <iostream>

#ifdef PSKEL_OMP
#include <omp.h>
#endif

#include "PSkelDefs.h"
#include "PSkelArray.h"
#include "PSkelArgs.h"
#include "PSkelMask.h"
#include "PSkelStencil.h"

#endif  // PSKEL_H
