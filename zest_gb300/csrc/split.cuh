// Split-precision (BF16 fixed-point slices on tcgen05) form of the Zernike
// contractions and of the SH Legendre sums; see split.cu.
#pragma once

#include <vector>

struct zest_gpu_context;

namespace zgpu {

struct ZtPlan;
struct StPlan;
struct SplitState;  // per-context state of the split path, defined in split.cu
void destroy_split(SplitState* s);
struct SplitDeleter {
    void operator()(SplitState* s) const { destroy_split(s); }
};

// ZEST_GPU_OK when the split path is available on the current device.
int split_available();
int split_zt_forward(zest_gpu_context* ctx, ZtPlan& plan, int Lg, int Le, int Lm, int batch, const double* grids,
                     double* coeffs);
int split_zt_backward(zest_gpu_context* ctx, ZtPlan& plan, int Le, int Lg, int Lm, int batch, const double* coeffs,
                      double* grids);
// True when the split SH path also runs the longitude DFT (on the tensor
// cores, in place of the FP64 FFT): LonLat grids of order 2 and above.
inline bool split_st_tensor_dft(bool latlon, int Lg) { return !latlon && Lg >= 2; }
// SH transforms in split precision (6 slices).  Forward: grids -> the spectra
// X[b][m][lat][2] (by the tensor-core DFT where split_st_tensor_dft; else X
// already holds the forward FFT's output) -> coefficients of degrees < Lm.
// Backward: coefficients -> grids where split_st_tensor_dft (X is scratch);
// else -> X, for the caller's inverse FFT.
int split_st_forward(zest_gpu_context* ctx, StPlan& plan, int Lg, int Lm, int batch, const double* grids, double* X,
                     double* coeffs, long long csz);
int split_st_backward(zest_gpu_context* ctx, StPlan& plan, int Lg, int Lm, int batch, const double* coeffs,
                      long long csz, double* X, double* grids);
// Rotor::rotate of a batch of real expansions (Zernike, SH or row-skipping,
// of equal or different orders) with the two X(+-pi/2) products of every
// rotated vector as split GEMMs (orders up to 256): vecs = the
// {item, n, l, first coefficient of the vector within its item} vectors
// sorted by l, vector rows [voff[l], voff[l+1]) of order l; coff = each
// item's coefficient offset; phase = scratch for the [item][3][Lmax] phase
// tables.
int split_rotate_ragged(zest_gpu_context* ctx, int Lmax, int items, long long nvec, const int4* vecs,
                        const std::vector<long long>& voff, const long long* coff, double* coeffs, const double* wig,
                        const double* euler, int type, double* phase);
// C = A B^T (A: M x K, B: N x K, C: M x N, row-major FP64 device buffers)
int split_dense_gemm(zest_gpu_context* ctx, int M, int N, int K, const double* A, const double* B, double* C);
// BF16 tensor-core flops of the split GEMM launches since the last reset
// (counted while profiling is enabled): useful = valid rows x table rows x K,
// issued = whole 128-row tiles as executed.
void split_flops(zest_gpu_context* ctx, bool reset, double* useful, double* issued);
// Synchronizes the context stream and reports (and clears) a bounded-wait
// timeout recorded by the split GEMMs launched since the last check.
int split_check_flag(zest_gpu_context* ctx);
// End of a split-path call: split_check_flag, except while the stream is
// being captured into a graph (whose replays are checked by the caller).
int split_finish(zest_gpu_context* ctx);
// Makes one bounded mbarrier wait run out after limit_ns (nothing arrives on
// it) and reports it as the GEMMs' timeouts are reported: ZEST_GPU_ERR_TIMEOUT.
int split_wait_selftest(zest_gpu_context* ctx, long long limit_ns);

}  // namespace zgpu
