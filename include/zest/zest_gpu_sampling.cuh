// Sampling of device functors on the quadrature grids, for code compiled with
// nvcc: the GPU counterpart of BallGLQGridPoints::generate_values and
// ZernikeTransformer::transform (zernike_glq_transformer.hpp:388-427,
// 1054-1178), and of SphereGLQGridPoints::generate_values and
// SHTransformer::transform (sh_glq_transformer.hpp:431-481, 1257-1351).
//
// A functor with a __device__ call operator is evaluated at every grid point
// by one thread each, straight into device memory, and the forward transform
// then runs on device memory: no grid crosses the host link.  The points are
// the library's (zest_gpu_zt_grid_points / zest_gpu_st_grid_points), the same
// as the host-side classes use.
//
//     struct Gaussian {
//         double s;
//         __device__ double operator()(double lon, double colat, double r) const { ... }
//     };
//     zest::zt::DeviceZernikeTransformer<ZernikeNorm::unnormed, SHNorm::geo, SHPhase::none> t(order);
//     auto expansion = t.transform(Gaussian{0.3}, radius, order);
//
// Batched form: a functor taking the item first, f(item, lon, colat, r),
// samples `batch` functions into consecutive grids.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "zest_gpu.hpp"

namespace zest {

namespace detail {

inline void cuda_check(cudaError_t e) {
    if (e != cudaSuccess) throw GPUError(ZEST_GPU_ERR_CUDA, cudaGetErrorString(e));
}

// Device buffer of doubles owned by the sampler.
class DeviceDoubles {
public:
    DeviceDoubles() = default;
    DeviceDoubles(const DeviceDoubles&) = delete;
    DeviceDoubles& operator=(const DeviceDoubles&) = delete;
    ~DeviceDoubles() {
        if (m_p) cudaFree(m_p);
    }
    void resize(std::size_t n) {
        if (n <= m_n && m_p) return;
        if (m_p) cudaFree(m_p);
        m_p = nullptr;
        m_n = 0;
        cuda_check(cudaMalloc(&m_p, (n ? n : 1) * sizeof(double)));
        m_n = n;
    }
    void upload(const double* h, std::size_t n, cudaStream_t s) {
        resize(n);
        if (n) cuda_check(cudaMemcpyAsync(m_p, h, n * sizeof(double), cudaMemcpyHostToDevice, s));
        cuda_check(cudaStreamSynchronize(s));
    }
    [[nodiscard]] double* data() const noexcept { return m_p; }

private:
    double* m_p = nullptr;
    std::size_t m_n = 0;
};

// One thread per grid point, the fastest grid axis across consecutive threads.
template <typename F>
__global__ void zt_sample_kernel(F f, double radius, int nlon, int nlat, int nrad, const double* __restrict__ lon,
                                 const double* __restrict__ colat, const double* __restrict__ rad,
                                 double* __restrict__ grid, int batch) {
    const long long per = (long long)nlon * nlat * nrad;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= per * batch) return;
    const long long b = t / per, p = t - b * per;
    const int k = int(p % nrad), j = int((p / nrad) % nlat), i = int(p / ((long long)nrad * nlat));
    grid[t] = f((std::size_t)b, lon[i], colat[j], rad[k] * radius);
}

template <typename F>
__global__ void st_sample_kernel(F f, int nlon, int nlat, int lon_fast, const double* __restrict__ lon,
                                 const double* __restrict__ colat, double* __restrict__ grid, int batch) {
    const long long per = (long long)nlon * nlat;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= per * batch) return;
    const long long b = t / per, p = t - b * per;
    int i, j;
    if (lon_fast) { i = int(p % nlon); j = int(p / nlon); }  // [lat][lon]
    else { j = int(p % nlat); i = int(p / nlat); }           // [lon][lat]
    grid[t] = f((std::size_t)b, lon[i], colat[j]);
}

// Adapters from single-function functors to the batched form.
template <typename F>
struct ZtOne {
    F f;
    __device__ double operator()(std::size_t, double lon, double colat, double r) const { return f(lon, colat, r); }
};
template <typename F>
struct StOne {
    F f;
    __device__ double operator()(std::size_t, double lon, double colat) const { return f(lon, colat); }
};

}  // namespace detail

namespace zt {

// Zernike transforms of device functors: sample on the GPU, transform on the GPU.
template <ZernikeNorm zernike_norm_param, st::SHNorm sh_norm_param, st::SHPhase sh_phase_param,
          typename GridLayoutType = DefaultLayout>
class DeviceZernikeTransformer {
public:
    using GridLayout = GridLayoutType;
    using Expansion = RealZernikeExpansion<zernike_norm_param, sh_norm_param, sh_phase_param>;

    explicit DeviceZernikeTransformer(std::size_t order = 0, int device = 0, cudaStream_t stream = nullptr)
        : m_transformer(order, device, stream), m_stream(stream) {
        resize(order);
    }
    void resize(std::size_t order) {
        m_transformer.resize(order);
        if (order == m_order && m_points_ready) return;
        BallGLQGridPoints<GridLayout> pts(order);
        m_lon.upload(pts.longitudes().data(), pts.longitudes().size(), m_stream);
        m_colat.upload(pts.lat_glq_nodes().data(), pts.lat_glq_nodes().size(), m_stream);
        m_rad.upload(pts.rad_glq_nodes().data(), pts.rad_glq_nodes().size(), m_stream);
        m_order = order;
        m_points_ready = true;
    }
    [[nodiscard]] GLQTransformer<zernike_norm_param, sh_norm_param, sh_phase_param, GridLayout>& transformer() noexcept {
        return m_transformer;
    }

    // f(item, lon, colat, r * radius) for item < batch into `grids` (device), item b at
    // b * grid_size(order), on the transformer's stream.
    template <typename F>
    void generate_values_batch(F f, double radius, std::size_t order, std::size_t batch, double* grids) {
        resize(order);
        const auto sh = GridLayout::shape(order);
        const long long n = (long long)sh[0] * sh[1] * sh[2] * (long long)batch;
        if (n == 0) return;
        zest::detail::zt_sample_kernel<<<unsigned((n + 255) / 256), 256, 0, m_stream>>>(
            f, radius, int(sh[0]), int(sh[1]), int(sh[2]), m_lon.data(), m_colat.data(), m_rad.data(), grids,
            int(batch));
        zest::detail::cuda_check(cudaGetLastError());
    }
    // `batch` functions f(item, lon, colat, r) -> `batch` expansions (device memory, contiguous)
    template <typename F>
    void transform_batch(F f, double radius, std::size_t order, std::size_t batch, double* coeffs_dev) {
        const std::size_t gsz = GridLayout::size(order);
        m_grid.resize(gsz * batch);
        generate_values_batch(f, radius, order, batch, m_grid.data());
        m_transformer.forward_transform_batch(m_grid.data(), order, coeffs_dev, order, batch, MemoryKind::device);
    }
    // one function f(lon, colat, r) -> a host expansion
    template <typename F>
    void transform(F f, double radius,
                   RealZernikeSpan<std::array<double, 2>, zernike_norm_param, sh_norm_param, sh_phase_param> expansion) {
        const std::size_t order = expansion.order();
        m_coeffs.resize(2 * expansion.size());
        transform_batch(zest::detail::ZtOne<F>{f}, radius, order, 1, m_coeffs.data());
        zest::detail::cuda_check(cudaMemcpyAsync(expansion.data(), m_coeffs.data(), 2 * expansion.size() * sizeof(double),
                                           cudaMemcpyDeviceToHost, m_stream));
        zest::detail::cuda_check(cudaStreamSynchronize(m_stream));
    }
    template <typename F>
    [[nodiscard]] Expansion transform(F f, double radius, std::size_t order) {
        Expansion expansion(order);
        transform(f, radius, expansion);
        return expansion;
    }

private:
    GLQTransformer<zernike_norm_param, sh_norm_param, sh_phase_param, GridLayout> m_transformer;
    cudaStream_t m_stream = nullptr;
    zest::detail::DeviceDoubles m_lon, m_colat, m_rad, m_grid, m_coeffs;
    std::size_t m_order = 0;
    bool m_points_ready = false;
};

}  // namespace zt

namespace st {

// SH transforms of device functors f(lon, colat): sample on the GPU, transform on the GPU.
template <SHNorm sh_norm_param, SHPhase sh_phase_param, typename GridLayoutType = DefaultLayout>
class DeviceSHTransformer {
public:
    using GridLayout = GridLayoutType;
    using Expansion = RealSHExpansion<sh_norm_param, sh_phase_param>;

    explicit DeviceSHTransformer(std::size_t order = 0, int device = 0, cudaStream_t stream = nullptr)
        : m_transformer(order, device, stream), m_stream(stream) {
        resize(order);
    }
    void resize(std::size_t order) {
        m_transformer.resize(order);
        if (order == m_order && m_points_ready) return;
        SphereGLQGridPoints<GridLayout> pts(order);
        m_lon.upload(pts.longitudes().data(), pts.longitudes().size(), m_stream);
        m_colat.upload(pts.glq_nodes().data(), pts.glq_nodes().size(), m_stream);
        m_order = order;
        m_points_ready = true;
    }

    template <typename F>
    void generate_values_batch(F f, std::size_t order, std::size_t batch, double* grids) {
        resize(order);
        const auto sh = GridLayout::shape(order);
        const std::size_t nlon = sh[GridLayout::lon_axis], nlat = sh[GridLayout::lat_axis];
        const long long n = (long long)nlon * nlat * (long long)batch;
        if (n == 0) return;
        zest::detail::st_sample_kernel<<<unsigned((n + 255) / 256), 256, 0, m_stream>>>(
            f, int(nlon), int(nlat), GridLayout::lon_axis == 1, m_lon.data(), m_colat.data(), grids, int(batch));
        zest::detail::cuda_check(cudaGetLastError());
    }
    template <typename F>
    void transform_batch(F f, std::size_t order, std::size_t batch, double* coeffs_dev) {
        m_grid.resize(GridLayout::size(order) * batch);
        generate_values_batch(f, order, batch, m_grid.data());
        m_transformer.forward_transform_batch(m_grid.data(), order, coeffs_dev, order, batch, MemoryKind::device);
    }
    template <typename F>
    void transform(F f, RealSHSpan<std::array<double, 2>, sh_norm_param, sh_phase_param> expansion) {
        m_coeffs.resize(2 * expansion.size());
        transform_batch(zest::detail::StOne<F>{f}, expansion.order(), 1, m_coeffs.data());
        zest::detail::cuda_check(cudaMemcpyAsync(expansion.data(), m_coeffs.data(), 2 * expansion.size() * sizeof(double),
                                           cudaMemcpyDeviceToHost, m_stream));
        zest::detail::cuda_check(cudaStreamSynchronize(m_stream));
    }
    template <typename F>
    [[nodiscard]] Expansion transform(F f, std::size_t order) {
        Expansion expansion(order);
        transform(f, expansion);
        return expansion;
    }

private:
    GLQTransformer<sh_norm_param, sh_phase_param, GridLayout> m_transformer;
    cudaStream_t m_stream = nullptr;
    zest::detail::DeviceDoubles m_lon, m_colat, m_grid, m_coeffs;
    std::size_t m_order = 0;
    bool m_points_ready = false;
};

}  // namespace st

}  // namespace zest
