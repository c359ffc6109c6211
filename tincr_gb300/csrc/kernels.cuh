// Declarations of the A.X product kernels defined in tda.cu, for other translation units.
#pragma once

namespace tincr {

__global__ void diag_dots_kernel(int n, int v, const double *__restrict__ H, const double *__restrict__ Rv,
                                 double *d3, double *d2);
__global__ void coulomb_kernel(int n, int n_atoms, const int *__restrict__ ao_off, const double *__restrict__ gamma,
                               const double *__restrict__ d3, const double *__restrict__ d2, double *zao, double *F,
                               double *y_out, double scale);
__global__ void scale_rows_kernel(int n, int v, const double *__restrict__ zao, const double *__restrict__ Rv,
                                  double *G);

}  // namespace tincr
