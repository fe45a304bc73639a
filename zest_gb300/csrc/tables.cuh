// Device-generated FP64 tables of the GLQ path (see tables.cu).
#pragma once

#include <cuda_runtime.h>

namespace zgpu {

// Gauss-Legendre nodes (cos style) and weights on the host, layouts of
// include/gauss_legendre.hpp:32-66 (unpacked ascending from -1; packed =
// non-negative nodes ascending from 0).
void gl_nodes_weights(long n, bool packed, double* nodes, double* weights);
// The same nodes as colatitudes theta = arccos(x) (angle style), ordered as
// the unpacked nodes (x ascending, theta descending from near pi).
void gl_colatitudes(long n, double* theta);

// P_lm(z_i) in the reference vector layout out[idx(l,m) * nz + i].
// complex_basis: P_lm of PlmRecursion::plm_complex (no sqrt(2) for m > 0)
int launch_plm_ref(cudaStream_t s, int L, int sh_norm, int sh_phase, int nz, const double* z, double* out,
                   bool complex_basis = false);
// P_lm(z_i) * scale[i] * (m > 0 ? mscale : 1) in the folded GEMM layout:
// row off[2m + ((l-m)&1)] + ((l-m)>>1), column i (ld columns); rows l >= Lrows skipped.
int launch_plm_gemm(cudaStream_t s, int L, int Lrows, int sh_norm, int sh_phase, int nz, const double* z,
                    double* out, const long long* off, const double* scale, int ld, double mscale);
// R_nl(r_k) in the reference vector layout out[(floor((n+1)^2/4) + l/2) * nr + k].
int launch_radial_ref(cudaStream_t s, int L, int zernike_norm, int nr, const double* r, double* out);
// R_nl(r_k) * scale[k] * (unnormed_factor ? 2n+3 : 1) at row off[l] + (n-l)/2; rows n >= Lrows skipped.
int launch_radial_gemm(cudaStream_t s, int L, int Lrows, int zernike_norm, int nr, const double* r, double* out,
                       const long long* off, const double* scale, int unnormed_factor);
// d^l_{m1 m2}(pi/2) for l < L in the reference layout (l(l+1)(2l+1)/6 + (l+1) m1 + m2).
int launch_wignerd(cudaStream_t s, int L, double* out);

}  // namespace zgpu
