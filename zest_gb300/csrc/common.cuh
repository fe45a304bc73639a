// Shared definitions for the zest GB300 kernels: index math of the reference
// layouts, grid shapes, and error plumbing for the C-ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "zest_gpu.h"

namespace zgpu {

using i64 = long long;

// ---- index math (restated from the reference layouts) ----------------------
// TriangleLayout<nonnegative>::idx, include/layout.hpp:232-237
__host__ __device__ inline i64 tri_idx(i64 l, i64 m) { return ((l * (l + 1)) >> 1) + m; }
__host__ __device__ inline i64 tri_size(i64 L) { return (L * (L + 1)) >> 1; }
// ZernikeTetrahedralLayout<nonnegative>::idx, include/layout.hpp:414-417
__host__ __device__ inline i64 zidx(i64 n, i64 l, i64 m) {
    return (n + 1) * (n + 3) * (2 * n + 1) / 24 + ((l * l) >> 2) + m;
}
__host__ __device__ inline i64 zsize(i64 L) { return (L + 1) * (L + 3) * (2 * L + 1) / 24; }
// offset of the d^l(pi/2) block, include/wignerd_collection.hpp:102-106
__host__ __device__ inline i64 wig_off(i64 l) { return l * (l + 1) * (2 * l + 1) / 6; }
__host__ __device__ inline i64 pad8(i64 n) { return (n + 7) & ~i64(7); }

// ---- grid shapes ------------------------------------------------------------
// LonLatRadLayout, include/zernike_glq_transformer.hpp:50-131
struct ZtShape {
    i64 L, nlon, nlat, nrad;
    __host__ __device__ i64 size() const { return nlon * nlat * nrad; }
};
inline ZtShape zt_shape(i64 L) { return ZtShape{L, L ? 2 * L - 1 : 0, L + 1, pad8(L + 1)}; }

// LonLatLayout / LatLonLayout, include/sh_glq_transformer.hpp:48-197.  For
// LatLon the transform runs over the padded longitude count (lon stride =
// transform length), as the reference's pocketfft call does.
struct StShape {
    i64 L, nlon, nlat;
    int latlon;
    __host__ __device__ i64 size() const { return nlon * nlat; }
};
inline StShape st_shape(i64 L, int latlon) {
    if (latlon) return StShape{L, pad8(L ? 2 * L - 1 : 0), L, 1};
    return StShape{L, L ? 2 * L - 1 : 0, pad8(L), 0};
}

// ---- error plumbing -----------------------------------------------------------
struct Status {
    int code = ZEST_GPU_OK;
    std::string msg;
};

}  // namespace zgpu

#define ZG_CUDA_TRY(expr)                                                                  \
    do {                                                                                   \
        cudaError_t _e = (expr);                                                           \
        if (_e != cudaSuccess) {                                                           \
            return ::zgpu::fail(ZEST_GPU_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
        }                                                                                  \
    } while (0)

#define ZG_TRY(expr)                                                                       \
    do {                                                                                   \
        int _s = (expr);                                                                   \
        if (_s != ZEST_GPU_OK) return _s;                                                  \
    } while (0)

namespace zgpu {
// records the message in the thread-local last-error slot and returns code
int fail(int code, const std::string& msg);
// checks the last launch; every kernel launch of the library goes through it
// (it also counts launches, see zest_gpu_launch_count)
int launch_check(const char* what);

// pipeline stages timed by the context profiler (zest_gpu_profile_*)
enum Stage {
    ST_FFT_FWD = 0, ST_FFT_INV, ST_LEG_FWD, ST_LEG_BWD, ST_RAD_FWD, ST_RAD_BWD, ST_ROTATE,
    ST_SPLIT_SLICE, ST_SPLIT_GEMM, ST_COPY_H2D, ST_COPY_D2H, ST_MEMSET, ST_EVAL_TABLES, ST_EVAL_RAD, ST_EVAL_LEG,
    ST_EVAL_LON, ST_SPECTRUM, ST_COUNT
};
inline const char* stage_name(int s) {
    static const char* names[ST_COUNT] = {"fft_fwd", "fft_inv", "legendre_fwd", "legendre_bwd", "radial_fwd",
                                          "radial_bwd", "rotate", "split_slice", "split_gemm", "copy_h2d",
                                          "copy_d2h", "memset", "eval_tables", "eval_radial", "eval_legendre",
                                          "eval_longitude", "spectrum"};
    return (s >= 0 && s < ST_COUNT) ? names[s] : "?";
}
}  // namespace zgpu
