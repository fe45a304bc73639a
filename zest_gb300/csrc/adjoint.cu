// Diagonal factors of the adjoint (vector-Jacobian) products of the GLQ
// transforms.  No counterpart in the reference, which has no derivatives.
//
// With B the backward transform (coefficients -> grid values, the real basis
// sampled at the quadrature nodes), W the quadrature weights of the grid and
// G the Gram diagonal of the basis under that quadrature, the forward
// transform of the reference is the quadrature projection
//     F = G^+ B^T W                    (zernike_glq_transformer.hpp:640-655, 710-865)
// (G^+ inverts the non-zero diagonal; the sin part of m = 0 has G = 0 and is
// never written).  Its adjoints are therefore
//     F^T cbar = W B (G^+ cbar),     B^T gbar = G F (W^-1 gbar),
// i.e. a backward (forward) transform between two diagonal scalings:
//   G = S * (1 for normed, 1/(2n+3) for unnormed Zernike), S = 4 pi (geo) or 1 (qm);
//   W = (2 pi / nlon) * w_lat(j) * (w_rad(k) r_k^2 / 2)   Zernike grid
//     = (2 pi / nlon) * w_lat(j)                         SH grid
// with the GL weights of the grid's own node counts.  The reference's SH fold
// of an odd LatLon grid counts the middle latitude twice
// (sh_glq_transformer.hpp:797-884); its weight is doubled in W so that the
// adjoint is the exact transpose of the forward transform as computed.
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace zgpu {

namespace {

// one block per (n, item) of a Zernike expansion
__global__ void zt_gram_kernel(const double* __restrict__ in, double* __restrict__ out, int L, double S, int unnormed,
                               int inverse) {
    const int n = blockIdx.x, b = blockIdx.y;
    const long long base = (long long)b * 2 * zsize(L);
    const double g = unnormed ? S / double(2 * n + 3) : S;
    const double f = inverse ? 1.0 / g : g;
    for (int l = n & 1; l <= n; l += 2)
        for (int m = threadIdx.x; m <= l; m += blockDim.x) {
            const long long i = base + 2 * zidx(n, l, m);
            out[i] = f * in[i];
            out[i + 1] = m ? f * in[i + 1] : 0.0;
        }
}

// one block per (l, item) of an SH expansion
__global__ void st_gram_kernel(const double* __restrict__ in, double* __restrict__ out, int L, double S, int inverse) {
    const int l = blockIdx.x, b = blockIdx.y;
    const long long base = (long long)b * 2 * tri_size(L);
    const double f = inverse ? 1.0 / S : S;
    for (int m = threadIdx.x; m <= l; m += blockDim.x) {
        const long long i = base + 2 * tri_idx(l, m);
        out[i] = f * in[i];
        out[i + 1] = m ? f * in[i + 1] : 0.0;
    }
}

__global__ void grid_weights_kernel(const double* __restrict__ in, double* __restrict__ out, long long n,
                                    const double* __restrict__ w, long long slab, int divide) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double wi = w[i % slab];
        out[i] = divide ? in[i] / wi : in[i] * wi;
    }
}

constexpr double kPi = 3.14159265358979323846264338327950288;

}  // namespace

int launch_zt_gram(cudaStream_t s, const double* in, double* out, int L, int batch, int sh_norm, int zernike_norm,
                   int inverse) {
    if (L <= 0 || batch <= 0) return ZEST_GPU_OK;
    const double S = sh_norm == ZEST_SH_GEO ? 4.0 * kPi : 1.0;
    zt_gram_kernel<<<dim3(L, batch), 128, 0, s>>>(in, out, L, S, zernike_norm == ZEST_ZERNIKE_UNNORMED, inverse);
    return launch_check("zt_gram_kernel");
}

int launch_st_gram(cudaStream_t s, const double* in, double* out, int L, int batch, int sh_norm, int inverse) {
    if (L <= 0 || batch <= 0) return ZEST_GPU_OK;
    const double S = sh_norm == ZEST_SH_GEO ? 4.0 * kPi : 1.0;
    st_gram_kernel<<<dim3(L, batch), 128, 0, s>>>(in, out, L, S, inverse);
    return launch_check("st_gram_kernel");
}

int launch_grid_weights(cudaStream_t s, const double* in, double* out, long long n, const double* w, long long slab,
                        int divide) {
    if (n <= 0) return ZEST_GPU_OK;
    const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
    grid_weights_kernel<<<(unsigned)blocks, 256, 0, s>>>(in, out, n, w, slab, divide);
    return launch_check("grid_weights_kernel");
}

}  // namespace zgpu
