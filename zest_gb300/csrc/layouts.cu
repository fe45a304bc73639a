// Coefficient layouts beside the transforms: the in-place conversions between
// real and complex expansions (with a change of normalisation and phase
// conventions), and the expansion of a row-skipping (single-parity) SH
// expansion into the full triangle layout.
//
//   * to_complex_expansion / to_real_expansion: SH spans
//     (include/real_sh_expansion.hpp:345-436), Zernike spans
//     (include/zernike_expansion.hpp:484-634) and per-n Zernike SH spans in
//     the row-skipping layout (include/zernike_expansion.hpp:636-775).  Every
//     coefficient pair is multiplied by one factor per component, computed
//     with the same operations in the same order as the reference computes
//     it, so the results are bit-identical to the reference's.
//   * the row-skipping SH backward transform
//     (include/sh_glq_transformer.hpp:680-754): the rows of the expansion's
//     parity go to the triangle layout, the other rows are zero.
#include "common.cuh"
#include "kernels.cuh"

namespace zgpu {
namespace {

// (l, m) of pair j of a row-skipping triangle whose rows have parity p:
// j = floor(l^2 / 4) + m (include/layout.hpp:364-370)
__device__ inline void rowskip_lm(i64 j, int p, int& l, int& m) {
    if (p == 0) {  // l = 2k: j = k^2 + m, m <= 2k
        i64 k = i64(sqrt(double(j)));
        while (k * k > j) --k;
        while ((k + 1) * (k + 1) <= j) ++k;
        l = int(2 * k);
        m = int(j - k * k);
    } else {  // l = 2k + 1: j = k (k + 1) + m, m <= 2k + 1
        i64 k = i64((sqrt(4.0 * double(j) + 1.0) - 1.0) * 0.5);
        while (k * (k + 1) > j) --k;
        while ((k + 1) * (k + 2) <= j) ++k;
        l = int(2 * k + 1);
        m = int(j - k * (k + 1));
    }
}

// (l, m) of pair j of the triangle layout, j = l (l + 1) / 2 + m
__device__ inline void tri_lm(i64 j, int& l, int& m) {
    i64 k = i64((sqrt(8.0 * double(j) + 1.0) - 1.0) * 0.5);
    while (tri_idx(k, 0) > j) --k;
    while (tri_idx(k + 1, 0) <= j) ++k;
    l = int(k);
    m = int(j - tri_idx(k, 0));
}

// n of pair j of the Zernike tetrahedral layout: zsize(n) <= j < zsize(n + 1)
__device__ inline int zt_n(i64 j) {
    i64 n = i64(cbrt(12.0 * double(j)));
    while (n > 0 && zsize(n) > j) --n;
    while (zsize(n + 1) <= j) ++n;
    return int(n);
}

__global__ void convert_kernel(ConvertParams P, int batch, double* __restrict__ c) {
    const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.pairs * batch) return;
    const i64 j = i % P.pairs;
    int n = 0, l = 0, m = 0;
    if (P.kind == CONVERT_SH) {
        tri_lm(j, l, m);
    } else if (P.kind == CONVERT_ROWS) {
        rowskip_lm(j, P.parity, l, m);
    } else {
        n = zt_n(j);
        rowskip_lm(j - zsize(n), n & 1, l, m);
    }
    // the factors of the reference: shnorm for m = 0; for m > 0 +-norm, the
    // sign alternating with m when the phase convention changes; a Zernike
    // normalisation change multiplies both by conversion_factor(n)
    double f0 = P.shnorm, fm = P.norm;
    if (P.zconv != 0) {
        const double zf = P.zconv > 0 ? sqrt(double(2 * n + 3)) : 1.0 / sqrt(double(2 * n + 3));
        f0 = P.shnorm * zf;
        fm = P.norm * zf;
    }
    double* p = c + 2 * i;
    if (m == 0) {
        p[0] *= f0;
        p[1] *= f0;
    } else {
        const double pre = (P.phase_change && (m & 1)) ? -fm : fm;
        p[0] *= pre;
        p[1] *= -pre;
    }
}

// Row-skipping SH expansions of order Lm (rows l = (Lm - 1) mod 2, + 2, ...)
// to triangle expansions of order Lm, the other rows zero.
__global__ void rows_to_triangle_kernel(int Lm, i64 src_pairs, int batch, const double* __restrict__ src,
                                        double* __restrict__ dst) {
    const i64 tri = tri_size(Lm);
    const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tri * batch) return;
    const i64 b = i / tri, j = i - b * tri;
    int l, m;
    tri_lm(j, l, m);
    double2 v = make_double2(0.0, 0.0);
    if ((l & 1) == ((Lm - 1) & 1)) {
        const double* s = src + 2 * (b * src_pairs + ((i64(l) * l) >> 2) + m);
        v = make_double2(s[0], s[1]);
    }
    reinterpret_cast<double2*>(dst)[i] = v;
}

}  // namespace

int launch_convert(cudaStream_t s, const ConvertParams& P, int batch, double* coeffs) {
    const i64 total = P.pairs * batch;
    if (total == 0) return ZEST_GPU_OK;
    convert_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(P, batch, coeffs);
    return launch_check("convert_kernel");
}

int launch_rows_to_triangle(cudaStream_t s, int Lm, long long src_pairs, int batch, const double* src,
                            double* dst) {
    const i64 total = tri_size(Lm) * batch;
    if (total == 0) return ZEST_GPU_OK;
    rows_to_triangle_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(Lm, src_pairs, batch, src, dst);
    return launch_check("rows_to_triangle_kernel");
}

}  // namespace zgpu
