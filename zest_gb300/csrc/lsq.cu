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
// m * lon -- and solved by the method of dgels, written here in FP64 kernels
// of this file: blocked Householder QR (panels of 32 columns, the reflectors
// of a panel applied to the trailing columns in the compact WY form
// I - V T V^T), the right-hand sides carried as extra trailing columns so
// that they receive Q^T, and back substitution with R.  `batch` data vectors
// at the same points are the right-hand sides of one factorisation.  As
// dgels, no rank check: the points must determine the expansion (at least as
// many points as unknowns).
//
// SH basis: P_lm(z) cos(m lon), P_lm(z) sin(m lon) with z = sin(latitude),
// as RealSHGenerator::generate (it evaluates P_lm at the sine of its angle
// argument, which LSQTransformer passes latitudes to).  Zernike basis:
// R_nl(r) P_lm(cos colatitude) {cos, sin}(m lon), as ZernikeGenerator
// evaluates it.  (The reference's Zernike fit passes its arguments to the
// generator in another order and regroups the solution by l alone; the fit
// here is the one its interface describes.)
#include <algorithm>
#include <cmath>
#include <vector>

#include "context.cuh"
#include "lsq.cuh"
#include "tables.cuh"

namespace zgpu {

struct LsqState {
    DevBuf A, b, cols, P, R, z, r, lon;
    DevBuf part, T, W;  // QR: reduction partials, the panel's T, the panel's T^T V^T C
};
void destroy_lsq(LsqState* s) { delete s; }

namespace {

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


// ---------------------------------------------------------------------------
// Householder QR least squares in FP64 (the method of LAPACK dgels).  The
// m x n matrix A (column-major, lda = m, m >= n) is factored in panels of
// QR_NB columns; reflector k is H_k = I - tau_k v_k v_k^T with v_k[k] = 1,
// v_k[i] = 0 for i < k and v_k[i > k] stored below the diagonal of A, as
// dgeqrf stores it; R is left in the upper triangle.  After each panel its
// reflectors are applied to the trailing columns of A and to the nrhs
// right-hand sides B (m x nrhs, ldb = m) at once, as
// C <- (I - V T V^T)^T C = C - V (T^T (V^T C)).  Every reduction is summed in
// a fixed order (per-block partials, then one pass over the blocks), so the
// result does not depend on the launch.
constexpr int QR_NB = 32;           // panel width
constexpr int QR_PROWS = 256;       // rows per block of the panel reductions (one per thread)
constexpr int QR_CROWS = 512;       // rows per block of V^T C
constexpr int QR_CCOLS = 64;        // columns per block of V^T C and of the update

// column c of the trailing part: columns of A from a0 on, then those of B
struct QrCols {
    double* A;
    long long lda;
    int na;  // trailing columns of A
    double* B;
    long long ldb;
    __device__ double* col(int c) const { return c < na ? A + (long long)c * lda : B + (long long)(c - na) * ldb; }
};

// Reflector k of a panel, first pass: over rows i > k, s = sum x_i^2 and
// d_c = sum x_i a_c[i] for the panel's columns c = k+1 .. k+nc (x = column k);
// block 0 also records row k (alpha = A[k][k] and a_c[k]), which the second
// pass overwrites.  part[blk][0] = s, part[blk][1 + c'] = d; rowk[0..nc].
__global__ void __launch_bounds__(256) qr_panel_dots(const double* __restrict__ A, long long lda, int m, int k,
                                                     int nc, double* __restrict__ part, double* __restrict__ rowk) {
    const double* x = A + (long long)k * lda;
    double acc[QR_NB];
#pragma unroll
    for (int c = 0; c < QR_NB; ++c) acc[c] = 0.0;
    const int i0 = k + 1 + blockIdx.x * QR_PROWS, i1 = min(m, i0 + QR_PROWS);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const double xi = x[i];
        acc[0] = fma(xi, xi, acc[0]);
#pragma unroll
        for (int c = 1; c < QR_NB; ++c)
            if (c <= nc) acc[c] = fma(xi, A[(long long)(k + c) * lda + i], acc[c]);
    }
    __shared__ double red[8][QR_NB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < QR_NB; ++c) {
        double v = acc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][c] = v;
    }
    __syncthreads();
    if (threadIdx.x <= nc) {
        double v = 0.0;
        for (int w = 0; w < 8; ++w) v += red[w][threadIdx.x];
        part[(long long)blockIdx.x * QR_NB + threadIdx.x] = v;
    }
    if (blockIdx.x == 0 && threadIdx.x <= nc) rowk[threadIdx.x] = A[(long long)(k + threadIdx.x) * lda + k];
}

// Block reduction of QR_NB per-thread sums; thread t <= n then holds the
// block's sum of entry t in red[0][t].
__device__ __forceinline__ void qr_block_sums(double (&acc)[QR_NB], double (*red)[QR_NB]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < QR_NB; ++c) {
        double v = acc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < QR_NB) {
        double v = 0.0;
        for (int w = 0; w < 8; ++w) v += red[w][threadIdx.x];
        red[0][threadIdx.x] = v;  // only warp 0 reads and writes red[0] from here on
    }
    __syncthreads();
}

// Reflector k, second pass, fused with the first pass of reflector k + 1.
// Every block sums the partials of reflector k in the same order, forms beta,
// tau and the scale 1 / (alpha - beta) of v, stores v below the diagonal and
// beta on it, and applies H_k to the panel's columns k+1 .. k+nc on its rows
// (rows k .. m-1, QR_PROWS per block, one per thread).  As dlarfg: tau = 0
// (H_k = I) when the column below the diagonal is zero.  Then, on the same
// rows (those below k + 1), it sums the first pass of reflector k + 1 into
// part_out and block 0 records row k + 1 in rowk_out.
__global__ void __launch_bounds__(256) qr_panel_step(double* __restrict__ A, long long lda, int m, int k, int nc,
                                                     int nblk, const double* __restrict__ part,
                                                     const double* __restrict__ rowk, double* __restrict__ part_out,
                                                     double* __restrict__ rowk_out, double* __restrict__ tau) {
    __shared__ double sum[QR_NB];
    __shared__ double w[QR_NB];
    __shared__ double scale_s;
    __shared__ double red[8][QR_NB];
    if (threadIdx.x <= nc) {
        double v = 0.0;
        for (int b = 0; b < nblk; ++b) v += part[(long long)b * QR_NB + threadIdx.x];
        sum[threadIdx.x] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double alpha = rowk[0], s = sum[0];
        double t = 0.0, scale = 0.0, beta = alpha;
        if (s > 0.0) {
            beta = -copysign(sqrt(fma(alpha, alpha, s)), alpha);
            t = (beta - alpha) / beta;
            scale = 1.0 / (alpha - beta);
        }
        scale_s = scale;
        // w_c = tau v^T a_c = tau (a_c[k] + scale d_c)
        for (int c = 1; c <= nc; ++c) w[c] = t * fma(scale, sum[c], rowk[c]);
        w[0] = beta;
        if (blockIdx.x == 0) tau[k] = t;
    }
    __syncthreads();
    const double scale = scale_s;
    const int i = k + blockIdx.x * QR_PROWS + threadIdx.x;  // this thread's row
    const bool own = i < m && threadIdx.x < QR_PROWS;
    if (own) {
        double* x = A + (long long)k * lda;
        double v;
        if (i == k) {
            v = 1.0;
            x[i] = w[0];
        } else {
            v = x[i] * scale;
            x[i] = v;
        }
        for (int c = 1; c <= nc; ++c) {
            double* a = A + (long long)(k + c) * lda;
            a[i] = fma(-v, w[c], a[i]);
        }
    }
    if (nc == 0) return;  // the panel's last reflector
    // first pass of reflector k + 1 over this block's rows below k + 1
    double acc[QR_NB];
#pragma unroll
    for (int c = 0; c < QR_NB; ++c) acc[c] = 0.0;
    if (own && i > k + 1) {
        const double xi = A[(long long)(k + 1) * lda + i];
        acc[0] = xi * xi;
#pragma unroll
        for (int c = 1; c < QR_NB; ++c)
            if (c < nc) acc[c] = xi * A[(long long)(k + 1 + c) * lda + i];
    }
    qr_block_sums(acc, red);  // also orders row k + 1's update before the read below
    if (threadIdx.x < nc) part_out[(long long)blockIdx.x * QR_NB + threadIdx.x] = red[0][threadIdx.x];
    if (blockIdx.x == 0 && threadIdx.x < nc) rowk_out[threadIdx.x] = A[(long long)(k + 1 + threadIdx.x) * lda + k + 1];
}

// v_a[i] of a panel starting at column j0 (v_a[j0 + a] = 1, 0 above)
__device__ __forceinline__ double qr_v(const double* __restrict__ A, long long lda, int j0, int a, int i) {
    const int d = j0 + a;
    return i < d ? 0.0 : (i == d ? 1.0 : A[(long long)d * lda + i]);
}

// Gram matrix of the panel's reflectors, per-block partials over rows
// j0 .. m-1: part[blk][a][b] = sum_i v_a[i] v_b[i] (a, b < jb).
__global__ void __launch_bounds__(256) qr_gram(const double* __restrict__ A, long long lda, int m, int j0, int jb,
                                               double* __restrict__ part) {
    __shared__ double Vs[64][QR_NB + 1];
    const int a = threadIdx.x >> 3, b0 = (threadIdx.x & 7) * 4;  // this thread: G[a][b0 .. b0+3]
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int r0 = j0 + blockIdx.x * QR_PROWS, r1 = min(m, r0 + QR_PROWS);
    for (int c0 = r0; c0 < r1; c0 += 64) {
        for (int e = threadIdx.x; e < 64 * QR_NB; e += blockDim.x) {
            const int i = e & 63, q = e >> 6;
            Vs[i][q] = (c0 + i < r1 && q < jb) ? qr_v(A, lda, j0, q, c0 + i) : 0.0;
        }
        __syncthreads();
        const int nrow = min(64, r1 - c0);
        for (int i = 0; i < nrow; ++i) {
            const double va = Vs[i][a];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] = fma(va, Vs[i][b0 + q], acc[q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) part[(long long)blockIdx.x * QR_NB * QR_NB + a * QR_NB + b0 + q] = acc[q];
}

// T of the compact WY form (dlarft, forward, columnwise): T[i][i] = tau_i,
// T[0:i][i] = -tau_i T[0:i][0:i] G[0:i][i], with G the summed Gram partials.
// One block of QR_NB x QR_NB threads; T is written row-major (QR_NB x QR_NB).
__global__ void qr_tmat(const double* __restrict__ part, int nblk, int jb, const double* __restrict__ tau, int j0,
                        double* __restrict__ T) {
    __shared__ double G[QR_NB][QR_NB];
    __shared__ double Ts[QR_NB][QR_NB];
    const int a = threadIdx.y, b = threadIdx.x;
    double v = 0.0;
    for (int blk = 0; blk < nblk; ++blk) v += part[(long long)blk * QR_NB * QR_NB + a * QR_NB + b];
    G[a][b] = v;
    Ts[a][b] = 0.0;
    __syncthreads();
    for (int i = 0; i < jb; ++i) {
        const double ti = tau[j0 + i];
        // thread (a, 0) for a < i: T[a][i] = -tau_i sum_{q=a}^{i-1} T[a][q] G[q][i]
        double t = 0.0;
        if (b == 0 && a < i) {
            for (int q = a; q < i; ++q) t = fma(Ts[a][q], G[q][i], t);
        }
        __syncthreads();
        if (b == 0 && a < i) Ts[a][i] = -ti * t;
        if (a == 0 && b == 0) Ts[i][i] = ti;
        __syncthreads();
    }
    T[a * QR_NB + b] = (a < jb && b < jb) ? Ts[a][b] : 0.0;
}

// Per-block partials of V^T C over rows j0 .. m-1: part[blk][a][c] for the
// block's QR_CCOLS trailing columns (a < jb).  Thread (ty, tx): rows a =
// 4 ty .. 4 ty + 3 of V^T, columns tx and tx + 32 of the tile.
__global__ void __launch_bounds__(256) qr_vtc(const double* __restrict__ A, long long lda, int m, int j0, int jb,
                                              QrCols C, int ncols, double* __restrict__ part) {
    __shared__ double Vs[32][QR_NB + 1];
    __shared__ double Cs[32][QR_CCOLS + 1];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int c0 = blockIdx.x * QR_CCOLS;
    double acc[4][2] = {};
    const int r0 = j0 + blockIdx.y * QR_CROWS, r1 = min(m, r0 + QR_CROWS);
    for (int q0 = r0; q0 < r1; q0 += 32) {
        for (int e = threadIdx.x; e < 32 * QR_NB; e += blockDim.x) {
            const int i = e & 31, a = e >> 5;
            Vs[i][a] = (q0 + i < r1 && a < jb) ? qr_v(A, lda, j0, a, q0 + i) : 0.0;
        }
        for (int e = threadIdx.x; e < 32 * QR_CCOLS; e += blockDim.x) {
            const int i = e & 31, c = e >> 5;
            Cs[i][c] = (q0 + i < r1 && c0 + c < ncols) ? C.col(c0 + c)[q0 + i] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int i = 0; i < 32; ++i) {
            double va[4], cb[2];
#pragma unroll
            for (int p = 0; p < 4; ++p) va[p] = Vs[i][4 * ty + p];
            cb[0] = Cs[i][tx];
            cb[1] = Cs[i][tx + 32];
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                acc[p][0] = fma(va[p], cb[0], acc[p][0]);
                acc[p][1] = fma(va[p], cb[1], acc[p][1]);
            }
        }
        __syncthreads();
    }
    double* out = part + (long long)blockIdx.y * QR_NB * ncols;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        const int a = 4 * ty + p;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int c = c0 + tx + 32 * q;
            if (a < jb && c < ncols) out[(long long)a * ncols + c] = acc[p][q];
        }
    }
}

// W = T^T (sum over the row blocks of V^T C).  A block of 32 x 8 threads
// takes 8 trailing columns: thread (a, c) sums entry (a, c) over the row
// blocks in a fixed order, then forms (T^T u)_a = sum_{q <= a} T[q][a] u_q.
__global__ void __launch_bounds__(256) qr_wmat(const double* __restrict__ part, int nblk, int jb, int ncols,
                                               const double* __restrict__ T, double* __restrict__ W) {
    __shared__ double Ts[QR_NB][QR_NB];
    __shared__ double u[8][QR_NB];
    const int a = threadIdx.x, cl = threadIdx.y;
    for (int e = threadIdx.y * QR_NB + threadIdx.x; e < QR_NB * QR_NB; e += QR_NB * 8) Ts[e / QR_NB][e % QR_NB] = T[e];
    const int c = blockIdx.x * 8 + cl;
    double v = 0.0;
    if (c < ncols && a < jb)
        for (int b = 0; b < nblk; ++b) v += part[((long long)b * QR_NB + a) * ncols + c];
    u[cl][a] = v;
    __syncthreads();
    if (c >= ncols || a >= jb) return;
    double w = 0.0;
    for (int q = 0; q <= a; ++q) w = fma(Ts[q][a], u[cl][q], w);  // T upper triangular
    W[(long long)a * ncols + c] = w;
}

// C[i][c] -= sum_a v_a[i] W[a][c] for rows j0 .. m-1: 64 x 64 tiles; thread
// (tx, ty) updates rows i0 + tx + 32 p (p < 2) of columns c0 + ty + 8 q
// (q < 8), so that the lanes of a warp touch 32 consecutive rows of a column.
__global__ void __launch_bounds__(256) qr_update(const double* __restrict__ A, long long lda, int m, int j0, int jb,
                                                 QrCols C, int ncols, const double* __restrict__ W) {
    __shared__ double Vs[QR_NB][64 + 1];
    __shared__ double Ws[QR_NB][64 + 1];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i0 = j0 + blockIdx.y * 64, c0 = blockIdx.x * 64;
    for (int e = threadIdx.x; e < 64 * QR_NB; e += blockDim.x) {
        const int i = e & 63, a = e >> 6;
        Vs[a][i] = (i0 + i < m && a < jb) ? qr_v(A, lda, j0, a, i0 + i) : 0.0;
        Ws[a][i] = (c0 + i < ncols && a < jb) ? W[(long long)a * ncols + c0 + i] : 0.0;
    }
    __syncthreads();
    double acc[2][8] = {};
#pragma unroll 4
    for (int a = 0; a < QR_NB; ++a) {
        double vv[2], ww[8];
#pragma unroll
        for (int p = 0; p < 2; ++p) vv[p] = Vs[a][tx + 32 * p];
#pragma unroll
        for (int q = 0; q < 8; ++q) ww[q] = Ws[a][ty + 8 * q];
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
            for (int q = 0; q < 8; ++q) acc[p][q] = fma(vv[p], ww[q], acc[p][q]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int c = c0 + ty + 8 * q;
        if (c >= ncols) continue;
        double* col = C.col(c);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const int i = i0 + tx + 32 * p;
            if (i < m) col[i] -= acc[p][q];
        }
    }
}

// Back substitution R x = y for each right-hand side (one block each): y =
// B[0:n][r] (the first n entries of Q^T b), R the upper triangle of A; x
// overwrites y.  Column-oriented: x_j = y_j / R_jj, then y_i -= R_ij x_j for
// i < j, from j = n-1 down.
__global__ void __launch_bounds__(1024) qr_backsub(const double* __restrict__ A, long long lda, int n,
                                                   double* __restrict__ B, long long ldb) {
    extern __shared__ double y[];
    double* b = B + (long long)blockIdx.x * ldb;
    for (int i = threadIdx.x; i < n; i += blockDim.x) y[i] = b[i];
    __syncthreads();
    for (int j = n - 1; j >= 0; --j) {
        const double* col = A + (long long)j * lda;
        const double xj = y[j] / col[j];
        __syncthreads();  // every thread has read y[j]
        for (int i = threadIdx.x; i < j; i += blockDim.x) y[i] = fma(-col[i], xj, y[i]);
        if (threadIdx.x == 0) y[j] = xj;
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) b[i] = y[i];
}

// Least-squares solution of A x = B (m x n, m >= n, nrhs right-hand sides):
// A is overwritten by its QR factors, B's first n rows by the solutions.
int qr_solve(zest_gpu_context* ctx, LsqState& Q, double* A, int m, int n, double* B, int nrhs) {
    cudaStream_t s = ctx->stream;
    const long long lda = m;
    const int pblk = (m + QR_PROWS - 1) / QR_PROWS;
    const int cblk = (m + QR_CROWS - 1) / QR_CROWS;
    const int ncol_max = n + nrhs;
    const size_t part_half = (size_t)pblk * QR_NB;  // panel partials, two halves
    const size_t part_n = std::max<size_t>({2 * part_half, (size_t)pblk * QR_NB * QR_NB,
                                            (size_t)cblk * QR_NB * ncol_max});
    ZG_TRY(Q.part.ensure((part_n + 2 * QR_NB + 8) * sizeof(double)));
    ZG_TRY(Q.T.ensure((QR_NB * QR_NB + n + 8) * sizeof(double)));
    ZG_TRY(Q.W.ensure((size_t)QR_NB * ncol_max * sizeof(double)));
    double* part = Q.part.as<double>();
    double* rowk = part + part_n;
    double* T = Q.T.as<double>();
    double* tau = T + QR_NB * QR_NB;
    double* W = Q.W.as<double>();
    for (int j0 = 0; j0 < n; j0 += QR_NB) {
        const int jb = std::min(QR_NB, n - j0);
        // first pass of the panel's first reflector, then one fused launch per
        // reflector (its second pass and the next one's first pass), the
        // partials alternating between two halves of the buffer
        int nprev = std::max(1, (m - j0 - 1 + QR_PROWS - 1) / QR_PROWS);
        qr_panel_dots<<<nprev, 256, 0, s>>>(A, lda, m, j0, jb - 1, part, rowk);
        ZG_TRY(launch_check("qr_panel_dots"));
        for (int k = j0; k < j0 + jb; ++k) {
            const int nc = j0 + jb - 1 - k;  // panel columns right of k
            const int cur = (k - j0) & 1;
            const int nb = (m - k + QR_PROWS - 1) / QR_PROWS;
            qr_panel_step<<<nb, 256, 0, s>>>(A, lda, m, k, nc, nprev, part + (size_t)cur * part_half,
                                             rowk + cur * QR_NB, part + (size_t)(cur ^ 1) * part_half,
                                             rowk + (cur ^ 1) * QR_NB, tau);
            ZG_TRY(launch_check("qr_panel_step"));
            nprev = nb;
        }
        const int ntrail = (n - j0 - jb) + nrhs;
        if (ntrail == 0) continue;
        const int gb = (m - j0 + QR_PROWS - 1) / QR_PROWS;
        qr_gram<<<gb, 256, 0, s>>>(A, lda, m, j0, jb, part);
        ZG_TRY(launch_check("qr_gram"));
        qr_tmat<<<1, dim3(QR_NB, QR_NB), 0, s>>>(part, gb, jb, tau, j0, T);
        ZG_TRY(launch_check("qr_tmat"));
        const QrCols C{A + (long long)(j0 + jb) * lda, lda, n - j0 - jb, B, lda};
        const int vb = (m - j0 + QR_CROWS - 1) / QR_CROWS;
        qr_vtc<<<dim3((ntrail + QR_CCOLS - 1) / QR_CCOLS, vb), 256, 0, s>>>(A, lda, m, j0, jb, C, ntrail, part);
        ZG_TRY(launch_check("qr_vtc"));
        qr_wmat<<<(ntrail + 7) / 8, dim3(QR_NB, 8), 0, s>>>(part, vb, jb, ntrail, T, W);
        ZG_TRY(launch_check("qr_wmat"));
        qr_update<<<dim3((ntrail + 63) / 64, (m - j0 + 63) / 64), 256, 0, s>>>(A, lda, m, j0, jb, C, ntrail, W);
        ZG_TRY(launch_check("qr_update"));
    }
    const size_t ysmem = (size_t)n * sizeof(double);
    if (ysmem > 200 * 1024) return fail(ZEST_GPU_ERR_UNSUPPORTED, "least-squares fit: more than 25600 unknowns");
    if (ysmem > 48 * 1024)
        ZG_CUDA_TRY(cudaFuncSetAttribute(qr_backsub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ysmem));
    qr_backsub<<<nrhs, 1024, ysmem, s>>>(A, lda, n, B, lda);
    return launch_check("qr_backsub");
}

}  // namespace

int lsq_dev(zest_gpu_context* ctx, int kind, int zn, int sn, int sp, int L, int npts, int batch, const double* data,
            const std::vector<double>& z, const std::vector<double>& lon, const std::vector<double>& r,
            double* coeffs) {
    if (batch == 0 || L == 0) return ZEST_GPU_OK;
    cudaStream_t s = ctx->stream;
    if (!ctx->lsq) ctx->lsq.reset(new LsqState());
    LsqState& Q = *ctx->lsq;
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
    {
        StageScope sc(ctx, ST_EVAL_LEG);
        ZG_TRY(qr_solve(ctx, Q, Q.A.as<double>(), npts, ncol, Q.b.as<double>(), batch));
    }
    double* b = Q.b.as<double>();
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
