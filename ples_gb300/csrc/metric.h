// metric.h -- device face-metric builder (metric.cu), internal to the library.
#pragma once
#include <cuda_runtime.h>

#include "mg_device.cuh"

namespace ples {
// Raw FP64 face metric of `level` (g11..g33, unscaled, t/pot for level >= 2)
// into nine ghosted-box arrays of geometry g, from node coordinates
// (0:jx,0:jy,0:jz) already on the device.
cudaError_t launch_metric(const double* xn, const double* yn, const double* zn, int jx, int jy, int jz,
                          int ip, int jp, int kp, int level, Geom g, double* const gout[9],
                          cudaStream_t st);
}  // namespace ples
