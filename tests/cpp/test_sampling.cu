// Test of the sampling front-ends, compiled with nvcc against include/zest/.
//
//   test_sampling <dir>           writes raw doubles into <dir>:
//     zt_device.bin   DeviceZernikeTransformer::transform of the order-20
//                     function f = r exp(-(sin colat cos lon)^2) (device functor)
//     zt_host.bin     ZernikeTransformer::transform of the same host lambda
//     zt_cart.bin     ZernikeTransformer::transform of its Cartesian form, radius 2
//     zt_batch.bin    transform_batch of f_b = (b + 1) f, 3 items
//     st_device.bin / st_host.bin / st_latlon.bin
//                     SH transforms of g = exp(-(sin colat cos lon)^2), order 12,
//                     device functor / host lambda / LatLon layout
//     points.bin      BallGLQGridPoints of order 20: lon, colat, rad
//   test_sampling --time L B      times device sampling + forward transform of
//                                 B functions of order L, FP64 and split precision
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "zest/zest_gpu_sampling.cuh"

namespace {

using namespace zest;

void write_doubles(const std::string& path, const double* p, std::size_t n) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), std::streamsize(n * sizeof(double)));
}

struct Config1 {
    __host__ __device__ double operator()(double lon, double colat, double r) const {
        const double x = sin(colat) * cos(lon);
        return r * exp(-x * x);
    }
};
struct Config1Batch {
    __device__ double operator()(std::size_t b, double lon, double colat, double r) const {
        return double(b + 1) * Config1{}(lon, colat, r);
    }
};
// a functor of a few flops: the sampler's own cost (one store per point)
struct Cheap {
    __device__ double operator()(std::size_t b, double lon, double colat, double r) const {
        return r * r + double(b) * lon * colat;
    }
};
struct Sphere1 {
    __host__ __device__ double operator()(double lon, double colat) const {
        const double x = sin(colat) * cos(lon);
        return exp(-x * x);
    }
};

using ZN = zt::ZernikeNorm;
using SN = st::SHNorm;
using SP = st::SHPhase;

int run_parity(const std::string& dir) {
    const std::size_t L = 20;
    zt::DeviceZernikeTransformer<ZN::unnormed, SN::geo, SP::none> dev(L);
    const auto ed = dev.transform(Config1{}, 1.0, L);
    write_doubles(dir + "/zt_device.bin", reinterpret_cast<const double*>(ed.data()), 2 * ed.size());

    zt::ZernikeTransformer<ZN::unnormed, SN::geo, SP::none> host(L);
    const auto eh = host.transform([](double lon, double colat, double r) { return Config1{}(lon, colat, r); }, 1.0, L);
    write_doubles(dir + "/zt_host.bin", reinterpret_cast<const double*>(eh.data()), 2 * eh.size());

    // the same function in Cartesian form on a ball of radius 2: f(x) = |x| exp(-(x_0 / |x|)^2)
    const auto ec = host.transform(
        [](std::array<double, 3> x) {
            const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            const double c = x[0] / r;
            return r * std::exp(-c * c);
        },
        2.0, L);
    write_doubles(dir + "/zt_cart.bin", reinterpret_cast<const double*>(ec.data()), 2 * ec.size());

    // three items f_b = (b + 1) f in one launch, coefficients on the device
    const std::size_t B = 3, csz = zt::RealZernikeExpansionGeo::size(L);
    zest::detail::DeviceDoubles coeffs;
    coeffs.resize(2 * csz * B);
    dev.transform_batch(Config1Batch{}, 1.0, L, B, coeffs.data());
    std::vector<double> cb(2 * csz * B);
    zest::detail::cuda_check(cudaMemcpy(cb.data(), coeffs.data(), cb.size() * sizeof(double), cudaMemcpyDeviceToHost));
    write_doubles(dir + "/zt_batch.bin", cb.data(), cb.size());

    const std::size_t Ls = 12;
    st::DeviceSHTransformer<SN::geo, SP::none> sdev(Ls);
    const auto sd = sdev.transform(Sphere1{}, Ls);
    write_doubles(dir + "/st_device.bin", reinterpret_cast<const double*>(sd.data()), 2 * sd.size());
    st::SHTransformer<SN::geo, SP::none> shost(Ls);
    const auto sh = shost.transform([](double lon, double colat) { return Sphere1{}(lon, colat); }, Ls);
    write_doubles(dir + "/st_host.bin", reinterpret_cast<const double*>(sh.data()), 2 * sh.size());
    st::DeviceSHTransformer<SN::geo, SP::none, st::LatLonLayout<>> slat(Ls);
    const auto sl = slat.transform(Sphere1{}, Ls);
    write_doubles(dir + "/st_latlon.bin", reinterpret_cast<const double*>(sl.data()), 2 * sl.size());

    zt::BallGLQGridPoints<> pts(L);
    std::vector<double> p;
    for (auto v : pts.longitudes()) p.push_back(v);
    for (auto v : pts.lat_glq_nodes()) p.push_back(v);
    for (auto v : pts.rad_glq_nodes()) p.push_back(v);
    write_doubles(dir + "/points.bin", p.data(), p.size());
    std::puts("sampling parity jobs done");
    return 0;
}

int run_timing(std::size_t L, std::size_t B) {
    zt::DeviceZernikeTransformer<ZN::unnormed, SN::geo, SP::none> dev(L);
    const std::size_t csz = zt::RealZernikeExpansionGeo::size(L);
    zest::detail::DeviceDoubles coeffs;
    coeffs.resize(2 * csz * B);
    cudaEvent_t e0, e1;
    zest::detail::cuda_check(cudaEventCreate(&e0));
    zest::detail::cuda_check(cudaEventCreate(&e1));
    for (int precision = 0; precision < 2; ++precision) {
        dev.transformer().set_precision(precision ? Precision::split : Precision::fp64);
        for (int w = 0; w < 3; ++w) dev.transform_batch(Config1Batch{}, 1.0, L, B, coeffs.data());
        zest::detail::cuda_check(cudaDeviceSynchronize());
        const int reps = 5;
        float ms_sample = 0.0f, ms_all = 0.0f;
        zest::detail::DeviceDoubles grids;
        grids.resize(zt::LonLatRadLayout<>::size(L) * B);
        for (int r = 0; r < reps; ++r) {
            float ms = 0.0f;
            zest::detail::cuda_check(cudaEventRecord(e0, nullptr));
            dev.generate_values_batch(Config1Batch{}, 1.0, L, B, grids.data());
            zest::detail::cuda_check(cudaEventRecord(e1, nullptr));
            zest::detail::cuda_check(cudaEventSynchronize(e1));
            zest::detail::cuda_check(cudaEventElapsedTime(&ms, e0, e1));
            ms_sample += ms;
            zest::detail::cuda_check(cudaEventRecord(e0, nullptr));
            dev.transform_batch(Config1Batch{}, 1.0, L, B, coeffs.data());
            zest::detail::cuda_check(cudaEventRecord(e1, nullptr));
            zest::detail::cuda_check(cudaEventSynchronize(e1));
            zest::detail::cuda_check(cudaEventElapsedTime(&ms, e0, e1));
            ms_all += ms;
        }
        float ms_cheap = 0.0f;
        for (int r = 0; r < reps; ++r) {
            float ms = 0.0f;
            zest::detail::cuda_check(cudaEventRecord(e0, nullptr));
            dev.generate_values_batch(Cheap{}, 1.0, L, B, grids.data());
            zest::detail::cuda_check(cudaEventRecord(e1, nullptr));
            zest::detail::cuda_check(cudaEventSynchronize(e1));
            zest::detail::cuda_check(cudaEventElapsedTime(&ms, e0, e1));
            ms_cheap += ms;
        }
        const double gbytes = double(zt::LonLatRadLayout<>::size(L)) * B * 8.0 / 1e9;
        std::printf("{\"functor\": \"r*r + b*lon*colat\", \"sample_ms\": %.3f, \"sample_gbs\": %.1f}\n",
                    ms_cheap / reps, gbytes / (ms_cheap / reps * 1e-3));
        std::printf("{\"precision\": \"%s\", \"order\": %zu, \"batch\": %zu, \"sample_ms\": %.3f, "
                    "\"sample_gbs\": %.1f, \"sample_plus_forward_ms\": %.3f, \"functions_per_s\": %.1f}\n",
                    precision ? "split" : "fp64", L, B, ms_sample / reps, gbytes / (ms_sample / reps * 1e-3),
                    ms_all / reps, B / (ms_all / reps * 1e-3));
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    try {
        if (argc >= 4 && std::string(argv[1]) == "--time")
            return run_timing(std::strtoul(argv[2], nullptr, 10), std::strtoul(argv[3], nullptr, 10));
        if (argc < 2) {
            std::puts("usage: test_sampling <dir> | --time L B");
            return 2;
        }
        return run_parity(argv[1]);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "failed: %s\n", e.what());
        return 1;
    }
}
