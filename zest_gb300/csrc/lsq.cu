// Least-squares fits of expansions to data at scattered points:
//   st::LSQTransformer::transform   lsq_transformer.hpp:57-110 (RealSHGenerator::generate,
//                                   sh_generator.hpp:69-120; LinearMultifit, src/linearfit.cpp)
//   zt::LSQTransformer::transform   lsq_transformer.hpp:119-187 (ZernikeGenerator::generate,
//                                   zernike_generator.hpp:64-140)
//
// The reference builds the design matrix (one row per point, one column per
// real basis function) and solves it with LAPACK's dgels (Householder QR).
// Here the design matrix is built on the device from the P_lm and R_nl
// tables at the points (the same table kernels as everywhere else) and
// cos/sin(m lon) -- the reference's generators take std::cos/std::sin of
// m * lon -- and solved by QR with cuSOLVER (geqrf, ormqr) and a triangular
// solve (cuBLAS trsm).  `batch` data vectors at the same points are the
// right-hand sides of one factorisation.  As dgels, no rank check: the
// points must determine the expansion (at least as many points as unknowns).
//
// SH basis: P_lm(z) cos(m lon), P_lm(z) sin(m lon) with z = sin(latitude),
// as RealSHGenerator::generate (it evaluates P_lm at the sine of its angle
// argument, which LSQTransformer passes latitudes to).  Zernike basis:
// R_nl(r) P_lm(cos colatitude) {cos, sin}(m lon), as ZernikeGenerator
// evaluates it.  (The reference's Zernike fit passes its arguments to the
// generator in another order and regroups the solution by l alone; the fit
// here is the one its interface describes.)
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <vector>

#include "context.cuh"
#include "lsq.cuh"
#include "tables.cuh"

namespace zgpu {

struct LsqState {
    cusolverDnHandle_t sol = nullptr;
    cublasHandle_t blas = nullptr;
    DevBuf A, tau, work, info, b, cols, P, R, z, r, lon;
    ~LsqState() {
        if (sol) cusolverDnDestroy(sol);
        if (blas) cublasDestroy(blas);
    }
};
void destroy_lsq(LsqState* s) { delete s; }

namespace {

#define ZG_SOLVER_TRY(expr)                                                                             \
    do {                                                                                                 \
        const cusolverStatus_t _st = (expr);                                                            \
        if (_st != CUSOLVER_STATUS_SUCCESS)                                                              \
            return fail(ZEST_GPU_ERR_CUDA, std::string(#expr) + ": cuSOLVER status " + std::to_string(int(_st))); \
    } while (0)
#define ZG_BLAS_TRY(expr)                                                                               \
    do {                                                                                                 \
        const cublasStatus_t _st = (expr);                                                              \
        if (_st != CUBLAS_STATUS_SUCCESS)                                                                \
            return fail(ZEST_GPU_ERR_CUDA, std::string(#expr) + ": cuBLAS status " + std::to_string(int(_st))); \
    } while (0)

// A[col][i] (column-major, lda = npts) for columns {n, l, m, c} (n < 0: SH).
__global__ void design_kernel(int npts, int ncol, const int4* __restrict__ cols, const double* __restrict__ P,
                              const double* __restrict__ R, const double* __restrict__ lon, double* __restrict__ A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npts) return;
    for (int j = blockIdx.y; j < ncol; j += gridDim.y) {
        const int4 c = cols[j];
        double sn, cs;
        sincos(double(c.z) * lon[i], &sn, &cs);
        double v = P[tri_idx(c.y, c.z) * npts + i] * (c.w ? sn : cs);
        if (c.x >= 0) v *= R[((((long long)c.x + 1) * (c.x + 1)) >> 2) * npts + (c.y >> 1) * (long long)npts + i];
        A[(long long)j * npts + i] = v;
    }
}

// coeffs[b][k][c] = x[b][col(k, c)] (the first ncol entries of right-hand side b)
__global__ void scatter_kernel(int ncol, int batch, const int4* __restrict__ cols, const int* __restrict__ pair,
                               const double* __restrict__ X, long long ldx, double* __restrict__ coeffs,
                               long long cstride) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)ncol * batch) return;
    const int b = int(t / ncol), j = int(t - (long long)b * ncol);
    coeffs[b * cstride + 2 * (long long)pair[j] + cols[j].w] = X[b * ldx + j];
}

}  // namespace

int lsq_dev(zest_gpu_context* ctx, int kind, int zn, int sn, int sp, int L, int npts, int batch, const double* data,
            const std::vector<double>& z, const std::vector<double>& lon, const std::vector<double>& r,
            double* coeffs) {
    if (batch == 0 || L == 0) return ZEST_GPU_OK;
    cudaStream_t s = ctx->stream;
    if (!ctx->lsq) {
        ctx->lsq.reset(new LsqState());
        ZG_SOLVER_TRY(cusolverDnCreate(&ctx->lsq->sol));
        ZG_BLAS_TRY(cublasCreate(&ctx->lsq->blas));
    }
    LsqState& Q = *ctx->lsq;
    ZG_SOLVER_TRY(cusolverDnSetStream(Q.sol, s));
    ZG_BLAS_TRY(cublasSetStream(Q.blas, s));
    // columns: every (n, l, m) cos term, and the sin term for m > 0
    std::vector<int4> cols;
    std::vector<int> pair;
    if (kind == 0) {
        for (int n = 0; n < L; ++n)
            for (int l = n & 1; l <= n; l += 2)
                for (int m = 0; m <= l; ++m)
                    for (int c = 0; c < (m ? 2 : 1); ++c) {
                        cols.push_back(make_int4(n, l, m, c));
                        pair.push_back(int(zidx(n, l, m)));
                    }
    } else {
        for (int l = 0; l < L; ++l)
            for (int m = 0; m <= l; ++m)
                for (int c = 0; c < (m ? 2 : 1); ++c) {
                    cols.push_back(make_int4(-1, l, m, c));
                    pair.push_back(int(tri_idx(l, m)));
                }
    }
    const int ncol = int(cols.size());
    if (npts < ncol)
        return fail(ZEST_GPU_ERR_UNSUPPORTED, "least-squares fit: fewer points (" + std::to_string(npts) +
                                                  ") than unknowns (" + std::to_string(ncol) + ")");
    DevBuf dpair;
    ZG_TRY(upload(Q.cols, cols, s));
    ZG_TRY(upload(dpair, pair, s));
    ZG_TRY(upload(Q.z, z, s));
    ZG_TRY(upload(Q.lon, lon, s));
    ZG_TRY(Q.P.ensure((size_t)tri_size(L) * npts * sizeof(double)));
    ZG_TRY(launch_plm_ref(s, L, sn, sp, npts, Q.z.as<double>(), Q.P.as<double>()));
    if (kind == 0) {
        ZG_TRY(upload(Q.r, r, s));
        ZG_TRY(Q.R.ensure((size_t)((((size_t)L + 1) * (L + 1)) >> 2) * npts * sizeof(double)));
        ZG_TRY(launch_radial_ref(s, L, zn, npts, Q.r.as<double>(), Q.R.as<double>()));
    }
    ZG_TRY(Q.A.ensure((size_t)ncol * npts * sizeof(double)));
    {
        StageScope sc(ctx, ST_EVAL_TABLES);
        dim3 grid((npts + 127) / 128, std::min(ncol, 65535));
        design_kernel<<<grid, 128, 0, s>>>(npts, ncol, Q.cols.as<int4>(), Q.P.as<double>(),
                                           kind == 0 ? Q.R.as<double>() : nullptr, Q.lon.as<double>(),
                                           Q.A.as<double>());
        ZG_TRY(launch_check("design_kernel"));
    }
    // right-hand sides: the data vectors, npts each (overwritten by Q^T b)
    ZG_TRY(Q.b.ensure((size_t)npts * batch * sizeof(double)));
    ZG_CUDA_TRY(cudaMemcpyAsync(Q.b.p, data, (size_t)npts * batch * sizeof(double), cudaMemcpyDeviceToDevice, s));
    ZG_TRY(Q.tau.ensure((size_t)ncol * sizeof(double)));
    ZG_TRY(Q.info.ensure(sizeof(int)));
    int lw1 = 0, lw2 = 0;
    double* A = Q.A.as<double>();
    double* tau = Q.tau.as<double>();
    double* b = Q.b.as<double>();
    ZG_SOLVER_TRY(cusolverDnDgeqrf_bufferSize(Q.sol, npts, ncol, A, npts, &lw1));
    ZG_SOLVER_TRY(cusolverDnDormqr_bufferSize(Q.sol, CUBLAS_SIDE_LEFT, CUBLAS_OP_T, npts, batch, ncol, A, npts, tau, b,
                                              npts, &lw2));
    const int lwork = std::max(lw1, lw2);
    ZG_TRY(Q.work.ensure((size_t)std::max(lwork, 1) * sizeof(double)));
    {
        StageScope sc(ctx, ST_EVAL_LEG);
        ZG_SOLVER_TRY(cusolverDnDgeqrf(Q.sol, npts, ncol, A, npts, tau, Q.work.as<double>(), lwork, Q.info.as<int>()));
        ZG_SOLVER_TRY(cusolverDnDormqr(Q.sol, CUBLAS_SIDE_LEFT, CUBLAS_OP_T, npts, batch, ncol, A, npts, tau, b, npts,
                                       Q.work.as<double>(), lwork, Q.info.as<int>()));
        const double one = 1.0;
        ZG_BLAS_TRY(cublasDtrsm(Q.blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT,
                                ncol, batch, &one, A, npts, b, npts));
    }
    int info = 0;
    ZG_CUDA_TRY(cudaMemcpyAsync(&info, Q.info.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    ZG_CUDA_TRY(cudaStreamSynchronize(s));
    if (info != 0) return fail(ZEST_GPU_ERR_CUDA, "least-squares fit: QR reported info " + std::to_string(info));
    const long long csz = 2 * (kind == 0 ? zsize(L) : tri_size(L));
    ZG_CUDA_TRY(cudaMemsetAsync(coeffs, 0, (size_t)csz * batch * sizeof(double), s));
    const long long n = (long long)ncol * batch;
    scatter_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(ncol, batch, Q.cols.as<int4>(), dpair.as<int>(), b, npts,
                                                            coeffs, csz);
    ZG_TRY(launch_check("scatter_kernel"));
    ZG_CUDA_TRY(cudaStreamSynchronize(s));  // dpair is local
    return ZEST_GPU_OK;
}

}  // namespace zgpu
