// Declarations of the A.X product kernels defined in tda.cu, for other translation units.
#pragma once

namespace tincr {

__global__ void diag_dots_kernel(int n, int v, const double *__restrict__ H, long long ldh, long long sbh,
                                 const double *__restrict__ Rv, double *d3, double *d2);
// Coulomb part of A.X for kc vectors: y_b(A) = (1/2) sum_{mu in A} (d3 + d2)_b(mu) (into y_out when
// given), z_b(A) = scale sum_B gamma_AB y_b(B), written per AO into zao and/or onto the diagonals of
// F_b ([2n x 2n]); grid (atoms / COULOMB_ATOMS, kc), one warp per atom.
constexpr int COULOMB_ATOMS = 8;
void launch_coulomb(cudaStream_t st, int kc, int n, int n_atoms, const int *ao_off, const double *gamma,
                    const double *d3, const double *d2, double *zao, double *F, double *y_out, double scale);
__global__ void scale_rows_kernel(int n, int v, const double *__restrict__ zao, const double *__restrict__ Rv,
                                  double *G);

}  // namespace tincr
