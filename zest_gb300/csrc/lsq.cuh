// Least-squares fits of expansions to scattered data (lsq.cu).
#pragma once

#include <vector>

struct zest_gpu_context;

namespace zgpu {

struct LsqState;  // solver handles and scratch, defined in lsq.cu
void destroy_lsq(LsqState* s);
struct LsqDeleter {
    void operator()(LsqState* s) const { destroy_lsq(s); }
};

// kind 0: Zernike (points r, lon, and z = cos(colatitude)); kind 1: SH
// (points lon and z = sin(latitude)).  data [batch][npts] and coeffs
// [batch][pairs][2] are device pointers; coefficients of all orders < L are
// written (the sin part of m = 0 as 0).
int lsq_dev(zest_gpu_context* ctx, int kind, int zn, int sn, int sp, int L, int npts, int batch, const double* data,
            const std::vector<double>& z, const std::vector<double>& lon, const std::vector<double>& r,
            double* coeffs);

}  // namespace zgpu
