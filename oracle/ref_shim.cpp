// C entry points over the reference zest library (sebsassi/zest), used ONLY as
// test infrastructure: to generate golden fixtures under tests/golden/ and as
// the timed CPU baseline of bench.py's reference arm.  It is compiled from the
// reference's own headers and sources by oracle/build_ref.py into oracle/_ref/.
// Nothing in the product (zest_gb300/, include/) links or calls this file.
//
// Every function calls the reference's public API unchanged:
//   zest::zt::GLQTransformer<...>   include/zernike_glq_transformer.hpp:511-965
//   zest::st::GLQTransformer<...>   include/sh_glq_transformer.hpp:513-1213
//   zest::Rotor                     include/rotor.hpp:95-401
//   zest::WignerdPiHalfCollection   include/wignerd_collection.hpp:66-110
//   zest::st::PlmRecursion          include/plm_recursion.hpp:62-362
//   zest::zt::RadialZernikeRecursion include/radial_zernike_recursion.hpp:38-297
//   zest::gl::gl_nodes_and_weights  include/gauss_legendre.hpp:1549-1565
//   zest::{zt,st}::GridEvaluator    include/grid_evaluator.hpp:52-325
//   zest::zt::power_spectrum        include/power_spectra.hpp:124-146
#include <algorithm>
#include <array>
#include <barrier>
#include <chrono>
#include <complex>
#include <memory>
#include <utility>
#include <cstddef>
#include <cstring>
#include <thread>
#include <vector>

#include "zernike_glq_transformer.hpp"
#include "sh_glq_transformer.hpp"
#include "rotor.hpp"
#include "wignerd_collection.hpp"
#include "grid_evaluator.hpp"
#include "power_spectra.hpp"

using zest::zt::ZernikeNorm;
using zest::st::SHNorm;
using zest::st::SHPhase;

namespace {

template <typename F>
int dispatch_zt(int zn, int sn, int sp, F&& f) {
    const int code = (zn & 1) | ((sn & 1) << 1) | ((sp & 1) << 2);
    switch (code) {
    case 0: f.template operator()<ZernikeNorm::normed, SHNorm::geo, SHPhase::none>(); return 0;
    case 1: f.template operator()<ZernikeNorm::unnormed, SHNorm::geo, SHPhase::none>(); return 0;
    case 2: f.template operator()<ZernikeNorm::normed, SHNorm::qm, SHPhase::none>(); return 0;
    case 3: f.template operator()<ZernikeNorm::unnormed, SHNorm::qm, SHPhase::none>(); return 0;
    case 4: f.template operator()<ZernikeNorm::normed, SHNorm::geo, SHPhase::cs>(); return 0;
    case 5: f.template operator()<ZernikeNorm::unnormed, SHNorm::geo, SHPhase::cs>(); return 0;
    case 6: f.template operator()<ZernikeNorm::normed, SHNorm::qm, SHPhase::cs>(); return 0;
    case 7: f.template operator()<ZernikeNorm::unnormed, SHNorm::qm, SHPhase::cs>(); return 0;
    }
    return -1;
}

template <typename F>
int dispatch_st(int sn, int sp, F&& f) {
    const int code = (sn & 1) | ((sp & 1) << 1);
    switch (code) {
    case 0: f.template operator()<SHNorm::geo, SHPhase::none>(); return 0;
    case 1: f.template operator()<SHNorm::qm, SHPhase::none>(); return 0;
    case 2: f.template operator()<SHNorm::geo, SHPhase::cs>(); return 0;
    case 3: f.template operator()<SHNorm::qm, SHPhase::cs>(); return 0;
    }
    return -1;
}

zest::RotationType rot_type(int t) {
    return t ? zest::RotationType::coordinate : zest::RotationType::object;
}

using ZtLayout = zest::zt::DefaultLayout;
using StLonLat = zest::st::LonLatLayout<>;
using StLatLon = zest::st::LatLonLayout<>;

}  // namespace

extern "C" {

int ref_gl_nodes_weights(std::size_t n, int packed, int angle_style, double* nodes, double* weights) {
    namespace gl = zest::gl;
    const std::size_t parity = n & 1;
    const std::size_t sz = packed ? gl::PackedLayout::size(n) : n;
    std::vector<double> nd(sz), wt(sz);
    if (packed) {
        if (angle_style) gl::gl_nodes_and_weights<gl::PackedLayout, gl::GLNodeStyle::angle>(nd, wt, parity);
        else gl::gl_nodes_and_weights<gl::PackedLayout, gl::GLNodeStyle::cos>(nd, wt, parity);
    } else {
        if (angle_style) gl::gl_nodes_and_weights<gl::UnpackedLayout, gl::GLNodeStyle::angle>(nd, wt, parity);
        else gl::gl_nodes_and_weights<gl::UnpackedLayout, gl::GLNodeStyle::cos>(nd, wt, parity);
    }
    std::memcpy(nodes, nd.data(), sz * sizeof(double));
    std::memcpy(weights, wt.data(), sz * sizeof(double));
    return 0;
}

int ref_plm_real(std::size_t order, int sn, int sp, std::size_t nz, const double* z, double* out) {
    return dispatch_st(sn, sp, [&]<SHNorm N, SHPhase P>() {
        zest::st::PlmRecursion rec(order);
        std::vector<double> zz(z, z + nz);
        std::vector<double> buf(zest::st::PlmLayout::size(order) * nz);
        zest::st::PlmVecSpan<double, N, P> plm(buf, order, nz);
        rec.plm_real(std::span<const double>(zz), plm);
        std::memcpy(out, buf.data(), buf.size() * sizeof(double));
    });
}

int ref_radial_zernike(std::size_t order, int zn, std::size_t nr, const double* r, double* out) {
    std::vector<double> rr(r, r + nr);
    std::vector<double> buf(zest::zt::RadialZernikeLayout::size(order) * nr);
    zest::zt::RadialZernikeRecursion rec(order);
    if (zn == 0) {
        zest::zt::RadialZernikeVecSpan<double, ZernikeNorm::normed> span(buf, order, nr);
        rec.zernike<ZernikeNorm::normed>(std::span<const double>(rr), span);
    } else {
        zest::zt::RadialZernikeVecSpan<double, ZernikeNorm::unnormed> span(buf, order, nr);
        rec.zernike<ZernikeNorm::unnormed>(std::span<const double>(rr), span);
    }
    std::memcpy(out, buf.data(), buf.size() * sizeof(double));
    return 0;
}

int ref_zt_grid_points(std::size_t order, double* lon, double* colat, double* r) {
    zest::zt::BallGLQGridPoints<ZtLayout> pts(order);
    auto a = pts.longitudes();
    auto b = pts.lat_glq_nodes();
    auto c = pts.rad_glq_nodes();
    std::memcpy(lon, a.data(), a.size() * sizeof(double));
    std::memcpy(colat, b.data(), b.size() * sizeof(double));
    std::memcpy(r, c.data(), c.size() * sizeof(double));
    return 0;
}

int ref_zt_forward(int zn, int sn, int sp, std::size_t grid_order, std::size_t exp_order,
                   const double* grid, double* coeffs) {
    return dispatch_zt(zn, sn, sp, [&]<ZernikeNorm Z, SHNorm N, SHPhase P>() {
        zest::zt::GLQTransformer<Z, N, P, ZtLayout> tr(grid_order);
        zest::zt::BallGLQGridSpan<const double, ZtLayout> g(grid, grid_order);
        zest::zt::RealZernikeSpan<std::array<double, 2>, Z, N, P> e(
            reinterpret_cast<std::array<double, 2>*>(coeffs), exp_order);
        tr.forward_transform(g, e);
    });
}

int ref_zt_backward(int zn, int sn, int sp, std::size_t exp_order, std::size_t grid_order,
                    const double* coeffs, double* grid) {
    return dispatch_zt(zn, sn, sp, [&]<ZernikeNorm Z, SHNorm N, SHPhase P>() {
        zest::zt::GLQTransformer<Z, N, P, ZtLayout> tr(grid_order);
        zest::zt::BallGLQGridSpan<double, ZtLayout> g(grid, grid_order);
        zest::zt::RealZernikeSpan<const std::array<double, 2>, Z, N, P> e(
            reinterpret_cast<const std::array<double, 2>*>(coeffs), exp_order);
        tr.backward_transform(e, g);
    });
}

int ref_st_grid_points(std::size_t order, int latlon, double* lon, double* colat) {
    auto copy = [&](auto& pts) {
        auto a = pts.longitudes();
        auto b = pts.glq_nodes();
        std::memcpy(lon, a.data(), a.size() * sizeof(double));
        std::memcpy(colat, b.data(), b.size() * sizeof(double));
    };
    if (latlon) { zest::st::SphereGLQGridPoints<StLatLon> p(order); copy(p); }
    else { zest::st::SphereGLQGridPoints<StLonLat> p(order); copy(p); }
    return 0;
}

int ref_st_forward(int sn, int sp, int latlon, std::size_t grid_order, std::size_t exp_order,
                   const double* grid, double* coeffs) {
    return dispatch_st(sn, sp, [&]<SHNorm N, SHPhase P>() {
        auto run = [&]<typename Lay>() {
            zest::st::GLQTransformer<N, P, Lay> tr(grid_order);
            zest::st::SphereGLQGridSpan<const double, Lay> g(grid, grid_order);
            zest::st::RealSHSpan<std::array<double, 2>, N, P> e(
                reinterpret_cast<std::array<double, 2>*>(coeffs), exp_order);
            tr.forward_transform(g, e);
        };
        if (latlon) run.template operator()<StLatLon>();
        else run.template operator()<StLonLat>();
    });
}

int ref_st_backward(int sn, int sp, int latlon, std::size_t exp_order, std::size_t grid_order,
                    const double* coeffs, double* grid) {
    return dispatch_st(sn, sp, [&]<SHNorm N, SHPhase P>() {
        auto run = [&]<typename Lay>() {
            zest::st::GLQTransformer<N, P, Lay> tr(grid_order);
            zest::st::SphereGLQGridSpan<double, Lay> g(grid, grid_order);
            zest::st::RealSHSpan<const std::array<double, 2>, N, P> e(
                reinterpret_cast<const std::array<double, 2>*>(coeffs), exp_order);
            tr.backward_transform(e, g);
        };
        if (latlon) run.template operator()<StLatLon>();
        else run.template operator()<StLonLat>();
    });
}

int ref_wignerd(std::size_t order, double* out) {
    zest::WignerdPiHalfCollection w(order);
    auto m = w.matrices();
    std::memcpy(out, m.data(), m.size() * sizeof(double));
    return 0;
}

int ref_zt_rotate(int zn, int sn, int sp, std::size_t order, double* coeffs, const double* euler, int type) {
    return dispatch_zt(zn, sn, sp, [&]<ZernikeNorm Z, SHNorm N, SHPhase P>() {
        zest::WignerdPiHalfCollection w(order);
        zest::Rotor rot(order);
        zest::zt::RealZernikeSpan<std::array<double, 2>, Z, N, P> e(
            reinterpret_cast<std::array<double, 2>*>(coeffs), order);
        rot.rotate(e, w, std::array<double, 3>{euler[0], euler[1], euler[2]}, rot_type(type));
    });
}

// Rotor::rotate of a per-n Zernike SH span (row-skipping layout, rotor.hpp:165-193).
int ref_rows_rotate(int sn, int sp, std::size_t order, double* coeffs, const double* euler, int type) {
    return dispatch_st(sn, sp, [&]<SHNorm N, SHPhase P>() {
        using Span = zest::zt::ZernikeSHSpan<std::array<double, 2>,
                                             zest::RowSkippingTriangleLayout<zest::IndexingMode::nonnegative>,
                                             ZernikeNorm::normed, N, P>;
        zest::WignerdPiHalfCollection w(order);
        zest::Rotor rot(order);
        Span e(reinterpret_cast<std::array<double, 2>*>(coeffs), order);
        rot.rotate(e, w, std::array<double, 3>{euler[0], euler[1], euler[2]}, rot_type(type));
    });
}

// st::GLQTransformer::backward_transform of a per-n Zernike SH span
// (sh_glq_transformer.hpp:680-700).
int ref_st_backward_rows(int sn, int sp, int latlon, std::size_t exp_order, std::size_t grid_order,
                         const double* coeffs, double* grid) {
    return dispatch_st(sn, sp, [&]<SHNorm N, SHPhase P>() {
        using Span = zest::zt::ZernikeSHSpan<const std::array<double, 2>,
                                             zest::RowSkippingTriangleLayout<zest::IndexingMode::nonnegative>,
                                             ZernikeNorm::normed, N, P>;
        Span e(reinterpret_cast<const std::array<double, 2>*>(coeffs), exp_order);
        auto run = [&]<typename Layout>() {
            zest::st::GLQTransformer<N, P, Layout> tr(grid_order);
            zest::st::SphereGLQGridSpan<double, Layout> g(grid, grid_order);
            tr.backward_transform(e, g);
        };
        if (latlon) run.template operator()<StLatLon>();
        else run.template operator()<StLonLat>();
    });
}

// to_complex_expansion (to_complex = 1) / to_real_expansion (0) of a Zernike
// (kind 0), SH (kind 1) or per-n Zernike SH span (kind 2) from the source to
// the destination conventions, in place (zernike_expansion.hpp:484-775,
// real_sh_expansion.hpp:345-436).
int ref_convert(int kind, std::size_t order, double* coeffs, int szn, int ssn, int ssp, int dzn, int dsn, int dsp,
                int to_complex) {
    using Row = zest::RowSkippingTriangleLayout<zest::IndexingMode::nonnegative>;
    return dispatch_zt(szn, ssn, ssp, [&]<ZernikeNorm SZ, SHNorm SN, SHPhase SP>() {
        dispatch_zt(dzn, dsn, dsp, [&]<ZernikeNorm DZ, SHNorm DN, SHPhase DP>() {
            auto* a = reinterpret_cast<std::array<double, 2>*>(coeffs);
            auto* c = reinterpret_cast<std::complex<double>*>(coeffs);
            if (kind == 0) {
                if (to_complex)
                    zest::zt::to_complex_expansion<DZ, DN, DP>(zest::zt::RealZernikeSpan<std::array<double, 2>, SZ, SN, SP>(a, order));
                else
                    zest::zt::to_real_expansion<DZ, DN, DP>(zest::zt::RealZernikeSpan<std::complex<double>, SZ, SN, SP>(c, order));
            } else if (kind == 1) {
                if (to_complex)
                    zest::st::to_complex_expansion<DN, DP>(zest::st::RealSHSpan<std::array<double, 2>, SN, SP>(a, order));
                else
                    zest::st::to_real_expansion<DN, DP>(zest::st::RealSHSpan<std::complex<double>, SN, SP>(c, order));
            } else {
                if (to_complex)
                    zest::zt::to_complex_expansion<DN, DP>(
                        zest::zt::ZernikeSHSpan<std::array<double, 2>, Row, SZ, SN, SP>(a, order));
                else
                    zest::zt::to_real_expansion<DN, DP>(
                        zest::zt::ZernikeSHSpan<std::complex<double>, Row, SZ, SN, SP>(c, order));
            }
        });
    });
}

int ref_zt_rotate_matrix(int zn, int sn, int sp, std::size_t order, double* coeffs, const double* mat, int type) {
    return dispatch_zt(zn, sn, sp, [&]<ZernikeNorm Z, SHNorm N, SHPhase P>() {
        zest::WignerdPiHalfCollection w(order);
        zest::Rotor rot(order);
        zest::zt::RealZernikeSpan<std::array<double, 2>, Z, N, P> e(
            reinterpret_cast<std::array<double, 2>*>(coeffs), order);
        std::array<std::array<double, 3>, 3> m{};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) m[i][j] = mat[3 * i + j];
        rot.rotate(e, w, m, rot_type(type));
    });
}

int ref_st_rotate(int sn, int sp, std::size_t order, double* coeffs, const double* euler, int type) {
    return dispatch_st(sn, sp, [&]<SHNorm N, SHPhase P>() {
        zest::WignerdPiHalfCollection w(order);
        zest::Rotor rot(order);
        zest::st::RealSHSpan<std::array<double, 2>, N, P> e(
            reinterpret_cast<std::array<double, 2>*>(coeffs), order);
        rot.rotate(e, w, std::array<double, 3>{euler[0], euler[1], euler[2]}, rot_type(type));
    });
}

int ref_zt_polar_rotate(int zn, int sn, int sp, std::size_t order, double* coeffs, double angle, int type) {
    return dispatch_zt(zn, sn, sp, [&]<ZernikeNorm Z, SHNorm N, SHPhase P>() {
        zest::Rotor rot(order);
        zest::zt::RealZernikeSpan<std::array<double, 2>, Z, N, P> e(
            reinterpret_cast<std::array<double, 2>*>(coeffs), order);
        rot.polar_rotate(e, angle, rot_type(type));
    });
}

int ref_st_polar_rotate(int sn, int sp, std::size_t order, double* coeffs, double angle, int type) {
    return dispatch_st(sn, sp, [&]<SHNorm N, SHPhase P>() {
        zest::Rotor rot(order);
        zest::st::RealSHSpan<std::array<double, 2>, N, P> e(
            reinterpret_cast<std::array<double, 2>*>(coeffs), order);
        rot.polar_rotate(e, angle, rot_type(type));
    });
}

int ref_zt_evaluate(int zn, int sn, int sp, std::size_t order, const double* coeffs,
                    std::size_t nlon, const double* lon, std::size_t nlat, const double* colat,
                    std::size_t nrad, const double* rad, double* out) {
    return dispatch_zt(zn, sn, sp, [&]<ZernikeNorm Z, SHNorm N, SHPhase P>() {
        zest::zt::GridEvaluator ev(order, nlon, nlat, nrad);
        zest::zt::RealZernikeSpan<const std::array<double, 2>, Z, N, P> e(
            reinterpret_cast<const std::array<double, 2>*>(coeffs), order);
        auto res = ev.evaluate(e, std::span<const double>(lon, nlon), std::span<const double>(colat, nlat),
                               std::span<const double>(rad, nrad));
        std::memcpy(out, res.data(), res.size() * sizeof(double));
    });
}

int ref_st_evaluate(int sn, int sp, std::size_t order, const double* coeffs, std::size_t nlon, const double* lon,
                    std::size_t nlat, const double* colat, double* out) {
    return dispatch_st(sn, sp, [&]<SHNorm N, SHPhase P>() {
        zest::st::GridEvaluator ev(order, nlon, nlat);
        zest::st::RealSHSpan<const std::array<double, 2>, N, P> e(
            reinterpret_cast<const std::array<double, 2>*>(coeffs), order);
        auto res = ev.evaluate(e, std::span<const double>(lon, nlon), std::span<const double>(colat, nlat));
        std::memcpy(out, res.data(), res.size() * sizeof(double));
    });
}

// zt::power_spectrum takes its expansion as a forwarding reference and reads
// ExpansionType::sh_norm, so the span is passed as a prvalue.  (The SH
// spectra, power_spectra.hpp:38-104, read ExpansionType::sh_norm too, which
// the SH spans do not have -- they name it `norm` -- so they do not compile
// and are not wrapped here.)
int ref_zt_power_spectrum(int sn, std::size_t order, const double* coeffs, double* out) {
    return dispatch_zt(1, sn, 0, [&]<ZernikeNorm Z, SHNorm N, SHPhase P>() {
        using Span = zest::zt::RealZernikeSpan<const std::array<double, 2>, Z, N, P>;
        zest::zt::power_spectrum(Span(reinterpret_cast<const std::array<double, 2>*>(coeffs), order),
                                 zest::zt::RadialZernikeSpan<double, Z>(out, order));
    });
}

// CPU baseline: `nsteps` steps of forward then backward transform of `batch`
// Zernike functions of one order on `nthreads` std::threads, items
// b = t, t + nthreads, ... on thread t.  Each thread builds its reference
// transformer (the O(L^3) tables) once, before the first step; only the
// steps are timed.  Writes each step's seconds to step_secs[0..nsteps).
int ref_zt_fwd_bwd_steps(int zn, int sn, int sp, std::size_t order, std::size_t batch, const double* grids,
                         double* coeffs, double* grids_out, int nthreads, int nsteps, double* step_secs) {
    const std::size_t gsz = ZtLayout::size(order);
    const std::size_t csz = zest::zt::RealZernikeExpansionGeo::size(order);
    return dispatch_zt(zn, sn, sp, [&]<ZernikeNorm Z, SHNorm N, SHPhase P>() {
        std::barrier sync(nthreads + 1);
        std::vector<std::thread> pool;
        for (int t = 0; t < nthreads; ++t) {
            pool.emplace_back([&, t]() {
                zest::zt::GLQTransformer<Z, N, P, ZtLayout> tr(order);
                sync.arrive_and_wait();  // tables built
                for (int step = 0; step < nsteps; ++step) {
                    sync.arrive_and_wait();  // step starts
                    for (std::size_t b = t; b < batch; b += nthreads) {
                        zest::zt::BallGLQGridSpan<const double, ZtLayout> g(grids + b * gsz, order);
                        zest::zt::RealZernikeSpan<std::array<double, 2>, Z, N, P> e(
                            reinterpret_cast<std::array<double, 2>*>(coeffs + 2 * b * csz), order);
                        tr.forward_transform(g, e);
                        zest::zt::BallGLQGridSpan<double, ZtLayout> go(grids_out + b * gsz, order);
                        tr.backward_transform(e, go);
                    }
                    sync.arrive_and_wait();  // step ends
                }
            });
        }
        sync.arrive_and_wait();
        for (int step = 0; step < nsteps; ++step) {
            const auto t0 = std::chrono::steady_clock::now();
            sync.arrive_and_wait();
            sync.arrive_and_wait();
            step_secs[step] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        for (auto& th : pool) th.join();
    });
}

// CPU baseline of the SH workload: `nsteps` steps of backward then forward
// transform of `batch` SH expansions of one order (LonLat grids) on
// `nthreads` std::threads, items b = t, t + nthreads, ... on thread t.  Each
// thread builds its reference transformer once, before the first step; only
// the steps are timed.  Writes each step's seconds to step_secs[0..nsteps).
int ref_st_bwd_fwd_steps(int sn, int sp, std::size_t order, std::size_t batch, const double* coeffs,
                         double* grids, double* coeffs_out, int nthreads, int nsteps, double* step_secs) {
    const std::size_t gsz = StLonLat::size(order);
    const std::size_t csz = order * (order + 1) / 2;
    return dispatch_st(sn, sp, [&]<SHNorm N, SHPhase P>() {
        std::barrier sync(nthreads + 1);
        std::vector<std::thread> pool;
        for (int t = 0; t < nthreads; ++t) {
            pool.emplace_back([&, t]() {
                zest::st::GLQTransformer<N, P, StLonLat> tr(order);
                sync.arrive_and_wait();  // tables built
                for (int step = 0; step < nsteps; ++step) {
                    sync.arrive_and_wait();  // step starts
                    for (std::size_t b = t; b < batch; b += nthreads) {
                        zest::st::RealSHSpan<const std::array<double, 2>, N, P> e(
                            reinterpret_cast<const std::array<double, 2>*>(coeffs + 2 * b * csz), order);
                        zest::st::SphereGLQGridSpan<double, StLonLat> g(grids + b * gsz, order);
                        tr.backward_transform(e, g);
                        zest::st::SphereGLQGridSpan<const double, StLonLat> gi(grids + b * gsz, order);
                        zest::st::RealSHSpan<std::array<double, 2>, N, P> eo(
                            reinterpret_cast<std::array<double, 2>*>(coeffs_out + 2 * b * csz), order);
                        tr.forward_transform(gi, eo);
                    }
                    sync.arrive_and_wait();  // step ends
                }
            });
        }
        sync.arrive_and_wait();
        for (int step = 0; step < nsteps; ++step) {
            const auto t0 = std::chrono::steady_clock::now();
            sync.arrive_and_wait();
            sync.arrive_and_wait();
            step_secs[step] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        for (auto& th : pool) th.join();
    });
}

// CPU baseline of batches of uneven order: Rotor::rotate (in place) then
// backward_transform of item i to a grid of its own order, for n_items items
// sorted by order.  Thread t takes a contiguous run of items of about equal
// cost (order^4).  Before timing, each thread builds its Rotor and
// WignerdPiHalfCollection for the largest order of its run and one
// transformer per order in its run, as a reference user with a ragged batch
// would keep them.  With grids_out null each thread overwrites one grid of
// its own (the results are discarded).  Returns the seconds of the timed run.
double ref_zt_rotate_backward_ragged(int zn, int sn, int sp, std::size_t n_items, const int* orders,
                                     double* coeffs, const double* euler, int rtype, double* grids_out,
                                     int nthreads) {
    std::vector<std::size_t> coff(n_items + 1, 0), goff(n_items + 1, 0);
    std::vector<double> cost(n_items + 1, 0.0);
    for (std::size_t i = 0; i < n_items; ++i) {
        const std::size_t L = std::size_t(orders[i]);
        coff[i + 1] = coff[i] + 2 * zest::zt::RealZernikeExpansionGeo::size(L);
        goff[i + 1] = goff[i] + ZtLayout::size(L);
        cost[i + 1] = cost[i] + double(L) * double(L) * double(L) * double(L);
    }
    std::vector<std::size_t> first(nthreads + 1, n_items);
    first[0] = 0;
    for (int t = 1; t < nthreads; ++t) {
        const double target = cost[n_items] * t / nthreads;
        first[t] = std::size_t(std::lower_bound(cost.begin(), cost.end(), target) - cost.begin());
        first[t] = std::min(std::max(first[t], first[t - 1]), n_items);
    }
    double secs = 0.0;
    dispatch_zt(zn, sn, sp, [&]<ZernikeNorm Z, SHNorm N, SHPhase P>() {
        using Tr = zest::zt::GLQTransformer<Z, N, P, ZtLayout>;
        std::barrier sync(nthreads + 1);
        std::vector<std::thread> pool;
        for (int t = 0; t < nthreads; ++t) {
            pool.emplace_back([&, t]() {
                const std::size_t i0 = first[t], i1 = first[t + 1];
                std::size_t lmax = 1;
                for (std::size_t i = i0; i < i1; ++i) lmax = std::max(lmax, std::size_t(orders[i]));
                zest::Rotor rotor(lmax);
                zest::WignerdPiHalfCollection wig(lmax);
                std::vector<std::pair<int, std::unique_ptr<Tr>>> trs;
                for (std::size_t i = i0; i < i1; ++i)
                    if (trs.empty() || trs.back().first != orders[i])
                        trs.emplace_back(orders[i], std::make_unique<Tr>(std::size_t(orders[i])));
                std::vector<double> own(grids_out ? 0 : ZtLayout::size(lmax));
                sync.arrive_and_wait();  // set-up done
                sync.arrive_and_wait();  // timed run starts
                std::size_t k = 0;
                for (std::size_t i = i0; i < i1; ++i) {
                    const std::size_t L = std::size_t(orders[i]);
                    while (trs[k].first != orders[i]) ++k;
                    zest::zt::RealZernikeSpan<std::array<double, 2>, Z, N, P> e(
                        reinterpret_cast<std::array<double, 2>*>(coeffs + coff[i]), L);
                    rotor.rotate(e, wig, std::array<double, 3>{euler[3 * i], euler[3 * i + 1], euler[3 * i + 2]},
                                 rot_type(rtype));
                    zest::zt::BallGLQGridSpan<double, ZtLayout> g(grids_out ? grids_out + goff[i] : own.data(), L);
                    trs[k].second->backward_transform(
                        zest::zt::RealZernikeSpan<const std::array<double, 2>, Z, N, P>(e), g);
                }
                sync.arrive_and_wait();  // timed run ends
            });
        }
        sync.arrive_and_wait();
        const auto t0 = std::chrono::steady_clock::now();
        sync.arrive_and_wait();
        sync.arrive_and_wait();
        secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (auto& th : pool) th.join();
    });
    return secs;
}

}  // extern "C"
