// metric.h -- device face-metric builder (metric.cu), internal to the library.
#pragma once
#include <cuda_runtime.h>

#include "mg_device.cuh"

namespace ples {
// FP64 face metric t*inv_div (g11..g33) of a level whose nodes are the fine
// nodes sub-sampled with strides (sx,sy,sz), into nine ghosted-box arrays of
// geometry g, from node coordinates (0:jx,0:jy,0:jz) already on the device.
// With all strides 1 the result is metrica's; with sx = sy = sz = pot and
// inv_div = 1/pot it is mul_met's.
cudaError_t launch_metric(const double* xn, const double* yn, const double* zn, int jx, int jy, int jz,
                          int ip, int jp, int kp, int sx, int sy, int sz, double inv_div, Geom g,
                          double* const gout[9], cudaStream_t st);
// Fine-level face normals J grad(csi), J grad(eta), J grad(zeta) on their
// faces (csx,csy,csz on csi faces; etx,ety,etz; ztx,zty,ztz) into nine boxes
// of geometry g, and the cell Jacobian giac at the cells.
cudaError_t launch_normals(const double* xn, const double* yn, const double* zn, int jx, int jy, int jz, int ip,
                           int jp, int kp, Geom g, double* const nout[9], double* giac, cudaStream_t st);
}  // namespace ples
