// Evaluation at arbitrary points and power spectra (evaluate.cu).  Device
// pointers; the points arrive as host vectors of cos(colatitude), (cos, sin)
// of each longitude and the radii.
#pragma once

#include <vector>

struct zest_gpu_context;

namespace zgpu {

// values [b][lon][lat][rad] of `batch` Zernike expansions of order L
int zt_evaluate_dev(zest_gpu_context* ctx, int zn, int sn, int sp, int L, int batch, const double* coeffs,
                    const std::vector<double>& z, const std::vector<double>& cs, const std::vector<double>& r,
                    double* values);
// values [b][lon][lat] of `batch` SH expansions of order L
int st_evaluate_dev(zest_gpu_context* ctx, int sn, int sp, int L, int batch, const double* coeffs,
                    const std::vector<double>& z, const std::vector<double>& cs, double* values);
// out[b * out_stride + l], l < nl: SH cross power spectrum of a and b (b = a for the power spectrum)
int st_spectrum_dev(zest_gpu_context* ctx, int sn, int L, int batch, const double* a, const double* b, int nl,
                    long long out_stride, double* out);
// out[b * floor((L+1)^2/4) + floor((n+1)^2/4) + l/2] for l < n < L
int zt_spectrum_dev(zest_gpu_context* ctx, int sn, int L, int batch, const double* c, double* out);

}  // namespace zgpu
