// Test of the C++20 interface (include/zest/*.hpp), written the way a user of
// the reference writes it.
//
// Compile-time part: the conventions are part of the types, so a transformer
// accepts only grids and expansions of its own conventions, and the rotor
// only expansions of std::array<double, 2>.
//
// Run-time part (needs a GPU): `test_cpp_api <dir>` reads <dir>/jobs.txt, one
// job per line,
//     <op> <conventions> <order> <input file> <output file> [extra file]
// runs it through the C++ interface and writes the result as raw doubles.
// The test harness compares the outputs with the golden fixtures.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "zest/grid_evaluator.hpp"
#include "zest/power_spectra.hpp"
#include "zest/rotor.hpp"
#include "zest/sh_glq_transformer.hpp"
#include "zest/zernike_glq_transformer.hpp"

namespace {

using namespace zest;

template <typename T, typename Grid, typename Exp>
concept can_forward = requires(T t, Grid g, Exp e) { t.forward_transform(g, e); };
template <typename T, typename Exp, typename Grid>
concept can_backward = requires(T t, Exp e, Grid g) { t.backward_transform(e, g); };
template <typename E>
concept can_rotate = requires(Rotor r, E e, WignerdPiHalfCollection w, std::array<double, 3> a) {
    r.rotate(e, w, a, RotationType::object);
};

using ZGeo = zt::GLQTransformerGeo<>;
static_assert(can_forward<ZGeo&, zt::BallGLQGrid<double>&, zt::RealZernikeExpansionGeo&>);
static_assert(can_backward<ZGeo&, zt::RealZernikeExpansionGeo&, zt::BallGLQGrid<double>&>);
static_assert(!can_forward<ZGeo&, zt::BallGLQGrid<double>&, zt::RealZernikeExpansionQM&>,
              "expansion of other conventions must be rejected");
static_assert(!can_forward<ZGeo&, zt::BallGLQGrid<double>&, zt::RealZernikeExpansionNormalGeo&>,
              "Zernike normalisation must match");
static_assert(!can_backward<zt::GLQTransformerNormalQM<>&, zt::RealZernikeExpansionQM&, zt::BallGLQGrid<double>&>);
static_assert(!can_forward<st::GLQTransformerGeo<>&, st::SphereGLQGrid<double>&, st::RealSHExpansionQM&>);
static_assert(!can_forward<st::GLQTransformerGeo<st::LatLonLayout<>>&, st::SphereGLQGrid<double>&,
                           st::RealSHExpansionGeo&>,
              "grid layout must match");
static_assert(can_forward<st::GLQTransformerGeo<st::LatLonLayout<>>&,
                          st::SphereGLQGrid<double, st::LatLonLayout<>>&, st::RealSHExpansionGeo&>);
static_assert(can_rotate<zt::RealZernikeExpansionGeo&> && can_rotate<st::RealSHExpansionQM&>);
static_assert(!can_rotate<const zt::RealZernikeExpansionGeo&>, "a const expansion cannot be rotated");
static_assert(zt::LonLatRadLayout<>::shape(200) == std::array<std::size_t, 3>{399, 201, 208});
static_assert(st::LonLatLayout<>::shape(1024) == std::array<std::size_t, 2>{2047, 1024});
static_assert(st::LatLonLayout<>::shape(7) == std::array<std::size_t, 2>{7, 16});
static_assert(zt::RealZernikeExpansionGeo::size(20) == 825);
static_assert(int(st::SHPhase::none) == -1 && int(st::SHPhase::cs) == 1);
static_assert(zt::RadialZernikeSpan<double, zt::ZernikeNorm::unnormed>::size(4) == 6);
static_assert(zt::RadialZernikeSpan<double, zt::ZernikeNorm::unnormed>::idx(3, 3) == 5);

std::vector<double> read_doubles(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    f.seekg(0, std::ios::end);
    const std::streamsize n = f.tellg();
    f.seekg(0);
    std::vector<double> v(std::size_t(n) / sizeof(double));
    f.read(reinterpret_cast<char*>(v.data()), n);
    return v;
}
void write_doubles(const std::string& path, const double* p, std::size_t n) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), std::streamsize(n * sizeof(double)));
}

template <typename Transformer>
void zt_job(const std::string& op, std::size_t order, const std::vector<double>& in, const std::string& out) {
    using Exp = typename Transformer::Expansion;
    Transformer t(order);
    if (op == "zt_fwd") {
        zt::BallGLQGrid<double> grid(order);
        std::copy(in.begin(), in.end(), grid.data());
        Exp e = t.forward_transform(grid, order);
        write_doubles(out, reinterpret_cast<const double*>(e.data()), 2 * e.size());
    } else {
        Exp e(order);
        std::copy(in.begin(), in.end(), reinterpret_cast<double*>(e.data()));
        zt::BallGLQGrid<double> grid = t.backward_transform(e, order);
        write_doubles(out, grid.data(), grid.size());
    }
}

template <typename Transformer>
void st_job(const std::string& op, std::size_t order, const std::vector<double>& in, const std::string& out) {
    using Layout = typename Transformer::GridLayout;
    Transformer t(order);
    using Exp = st::RealSHExpansion<Transformer::sh_norm, Transformer::phase>;
    if (op == "st_fwd") {
        st::SphereGLQGrid<double, Layout> grid(order);
        std::copy(in.begin(), in.end(), grid.data());
        Exp e = t.forward_transform(grid, order);
        write_doubles(out, reinterpret_cast<const double*>(e.data()), 2 * e.size());
    } else {
        Exp e(order);
        std::copy(in.begin(), in.end(), reinterpret_cast<double*>(e.data()));
        st::SphereGLQGrid<double, Layout> grid = t.backward_transform(e, order);
        write_doubles(out, grid.data(), grid.size());
    }
}

// conventions "zn sn sp" as digits of the C-ABI values, e.g. "100" = GLQTransformerGeo
void run_zt(const std::string& op, const std::string& conv, std::size_t order, const std::vector<double>& in,
            const std::string& out) {
    using ZN = zt::ZernikeNorm;
    using SN = st::SHNorm;
    using SP = st::SHPhase;
    if (conv == "000") zt_job<zt::GLQTransformer<ZN::normed, SN::geo, SP::none>>(op, order, in, out);
    else if (conv == "100") zt_job<zt::GLQTransformer<ZN::unnormed, SN::geo, SP::none>>(op, order, in, out);
    else if (conv == "010") zt_job<zt::GLQTransformer<ZN::normed, SN::qm, SP::none>>(op, order, in, out);
    else if (conv == "110") zt_job<zt::GLQTransformer<ZN::unnormed, SN::qm, SP::none>>(op, order, in, out);
    else if (conv == "001") zt_job<zt::GLQTransformer<ZN::normed, SN::geo, SP::cs>>(op, order, in, out);
    else if (conv == "101") zt_job<zt::GLQTransformer<ZN::unnormed, SN::geo, SP::cs>>(op, order, in, out);
    else if (conv == "011") zt_job<zt::GLQTransformer<ZN::normed, SN::qm, SP::cs>>(op, order, in, out);
    else if (conv == "111") zt_job<zt::GLQTransformer<ZN::unnormed, SN::qm, SP::cs>>(op, order, in, out);
    else throw std::runtime_error("bad conventions " + conv);
}

// conventions "layout sn sp", layout 0 = LonLat, 1 = LatLon
void run_st(const std::string& op, const std::string& conv, std::size_t order, const std::vector<double>& in,
            const std::string& out) {
    using SN = st::SHNorm;
    using SP = st::SHPhase;
    using LL = st::LonLatLayout<>;
    using TL = st::LatLonLayout<>;
    if (conv == "000") st_job<st::GLQTransformer<SN::geo, SP::none, LL>>(op, order, in, out);
    else if (conv == "010") st_job<st::GLQTransformer<SN::qm, SP::none, LL>>(op, order, in, out);
    else if (conv == "001") st_job<st::GLQTransformer<SN::geo, SP::cs, LL>>(op, order, in, out);
    else if (conv == "011") st_job<st::GLQTransformer<SN::qm, SP::cs, LL>>(op, order, in, out);
    else if (conv == "100") st_job<st::GLQTransformer<SN::geo, SP::none, TL>>(op, order, in, out);
    else if (conv == "110") st_job<st::GLQTransformer<SN::qm, SP::none, TL>>(op, order, in, out);
    else if (conv == "101") st_job<st::GLQTransformer<SN::geo, SP::cs, TL>>(op, order, in, out);
    else if (conv == "111") st_job<st::GLQTransformer<SN::qm, SP::cs, TL>>(op, order, in, out);
    else throw std::runtime_error("bad conventions " + conv);
}

// conventions "zn sn sp" -> f.template operator()<ZN, SN, SP>()
template <typename F>
void dispatch_zt_conv(const std::string& conv, F&& f) {
    using ZN = zt::ZernikeNorm;
    using SN = st::SHNorm;
    using SP = st::SHPhase;
    if (conv == "000") f.template operator()<ZN::normed, SN::geo, SP::none>();
    else if (conv == "100") f.template operator()<ZN::unnormed, SN::geo, SP::none>();
    else if (conv == "010") f.template operator()<ZN::normed, SN::qm, SP::none>();
    else if (conv == "110") f.template operator()<ZN::unnormed, SN::qm, SP::none>();
    else if (conv == "001") f.template operator()<ZN::normed, SN::geo, SP::cs>();
    else if (conv == "101") f.template operator()<ZN::unnormed, SN::geo, SP::cs>();
    else if (conv == "011") f.template operator()<ZN::normed, SN::qm, SP::cs>();
    else if (conv == "111") f.template operator()<ZN::unnormed, SN::qm, SP::cs>();
    else throw std::runtime_error("bad conventions " + conv);
}

// zt::GridEvaluator / st::GridEvaluator on the points of `pts` =
// [nlon, nlat, nrad, lon..., colat..., rad...]; zt::power_spectrum
void run_eval(const std::string& op, const std::string& conv, std::size_t order, const std::vector<double>& in,
              const std::string& out, const std::vector<double>& pts) {
    const std::size_t nlon = std::size_t(pts[0]), nlat = std::size_t(pts[1]), nrad = std::size_t(pts[2]);
    const std::span<const double> lon(pts.data() + 3, nlon), colat(lon.data() + nlon, nlat),
        rad(colat.data() + nlat, nrad);
    if (op == "zt_eval") {
        dispatch_zt_conv(conv, [&]<zt::ZernikeNorm Z, st::SHNorm N, st::SHPhase P>() {
            zt::RealZernikeExpansion<Z, N, P> e(order);
            std::copy(in.begin(), in.end(), reinterpret_cast<double*>(e.data()));
            zt::GridEvaluator ev(order, nlon, nlat, nrad);
            const std::vector<double> v = ev.evaluate(e, lon, colat, rad);
            write_doubles(out, v.data(), v.size());
        });
    } else if (op == "st_eval") {
        dispatch_zt_conv("0" + conv, [&]<zt::ZernikeNorm Z, st::SHNorm N, st::SHPhase P>() {
            st::RealSHExpansion<N, P> e(order);
            std::copy(in.begin(), in.end(), reinterpret_cast<double*>(e.data()));
            st::GridEvaluator ev(order, nlon, nlat);
            const std::vector<double> v = ev.evaluate(e, lon, colat);
            write_doubles(out, v.data(), v.size());
        });
    } else if (op == "zt_ps") {
        dispatch_zt_conv("1" + conv + "0", [&]<zt::ZernikeNorm Z, st::SHNorm N, st::SHPhase P>() {
            zt::RealZernikeExpansion<Z, N, P> e(order);
            std::copy(in.begin(), in.end(), reinterpret_cast<double*>(e.data()));
            const std::vector<double> v = zt::power_spectrum(e);
            write_doubles(out, v.data(), v.size());
        });
    } else {
        throw std::runtime_error("bad op " + op);
    }
}

// rotations of GLQTransformerGeo-convention expansions; conv = rotation type digit
void run_rot(const std::string& op, const std::string& conv, std::size_t order, const std::vector<double>& in,
             const std::string& out, const std::vector<double>& extra) {
    const RotationType type = conv == "1" ? RotationType::coordinate : RotationType::object;
    Rotor rotor(order);
    WignerdPiHalfCollection wigner(order);
    if (op.rfind("zt_", 0) == 0) {
        zt::RealZernikeExpansionGeo e(order);
        std::copy(in.begin(), in.end(), reinterpret_cast<double*>(e.data()));
        if (op == "zt_rot") rotor.rotate(e, wigner, std::array<double, 3>{extra[0], extra[1], extra[2]}, type);
        else if (op == "zt_polar") rotor.polar_rotate(e, extra[0], type);
        else if (op == "zt_rot_matrix") {
            std::array<std::array<double, 3>, 3> m{};
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) m[i][j] = extra[3 * i + j];
            rotor.rotate(e, wigner, m, type);
        } else throw std::runtime_error("bad op " + op);
        write_doubles(out, reinterpret_cast<const double*>(e.data()), 2 * e.size());
    } else {
        st::RealSHExpansionGeo e(order);
        std::copy(in.begin(), in.end(), reinterpret_cast<double*>(e.data()));
        if (op == "st_rot") rotor.rotate(e, wigner, std::array<double, 3>{extra[0], extra[1], extra[2]}, type);
        else if (op == "st_polar") rotor.polar_rotate(e, extra[0], type);
        else throw std::runtime_error("bad op " + op);
        write_doubles(out, reinterpret_cast<const double*>(e.data()), 2 * e.size());
    }
}

// Transpose identities through the C++ adjoints, written as relative
// differences: <F g, c> vs <g, F^T c>, <B c, g> vs <c, B^T g>,
// <rotate(x), y> vs <x, rotate^T y>.
void run_vjp_checks(const std::string& out) {
    const std::size_t L = 9;
    zt::GLQTransformerGeo<> t(L);
    zt::BallGLQGrid<double> g(L), gt(L), bc(L);
    zt::RealZernikeExpansionGeo c(L), fg(L), ct(L), x(L), y(L), xt(L);
    std::uint64_t s = 12345;
    auto rnd = [&]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return double(s >> 11) / double(1ull << 53) - 0.5;
    };
    for (auto& v : g.flatten()) v = rnd();
    for (std::size_t n = 0; n < L; ++n)
        for (std::size_t l = n & 1; l <= n; l += 2)
            for (std::size_t m = 0; m <= l; ++m) {
                c(n, l, m) = {rnd(), m ? rnd() : 0.0};
                x(n, l, m) = {rnd(), m ? rnd() : 0.0};
                y(n, l, m) = {rnd(), m ? rnd() : 0.0};
            }
    t.forward_transform(g, fg);
    t.forward_transform_vjp(c, gt);
    t.backward_transform(c, bc);
    t.backward_transform_vjp(g, ct);
    auto dot_c = [&](const auto& a, const auto& b) {
        double d = 0.0;
        for (std::size_t i = 0; i < a.size(); ++i) d += a.data()[i][0] * b.data()[i][0] + a.data()[i][1] * b.data()[i][1];
        return d;
    };
    auto dot_g = [&](const auto& a, const auto& b) {
        double d = 0.0;
        for (std::size_t i = 0; i < a.size(); ++i) d += a.data()[i] * b.data()[i];
        return d;
    };
    auto rel = [](double a, double b) { return std::abs(a - b) / std::max({std::abs(a), std::abs(b), 1e-300}); };
    double r[4];
    r[0] = rel(dot_c(fg, c), dot_g(g, gt));
    r[1] = rel(dot_g(bc, g), dot_c(c, ct));
    Rotor rotor(L);
    WignerdPiHalfCollection w(L);
    const std::array<double, 3> e{0.3, 1.1, -2.0};
    zt::RealZernikeExpansionGeo rx = x;
    rotor.rotate(rx, w, e, RotationType::object);
    const std::array<double, 3> grad = rotor.rotate_vjp(x, w, e, RotationType::object, y,
                                                        reinterpret_cast<double*>(xt.data()));
    r[2] = rel(dot_c(rx, y), dot_c(x, xt));
    // the angle gradient against a central difference of <rotate(x, e), y>
    const double h = 1e-6;
    double worst = 0.0;
    for (int k = 0; k < 3; ++k) {
        std::array<double, 3> ep = e, em = e;
        ep[k] += h;
        em[k] -= h;
        zt::RealZernikeExpansionGeo xp = x, xm = x;
        rotor.rotate(xp, w, ep, RotationType::object);
        rotor.rotate(xm, w, em, RotationType::object);
        const double fd = (dot_c(xp, y) - dot_c(xm, y)) / (2 * h);
        worst = std::max(worst, std::abs(fd - grad[k]) / std::max(std::abs(fd), 1e-3));
    }
    r[3] = worst;
    write_doubles(out, r, 4);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::puts("compile-time checks passed");
        return 0;
    }
    const std::string dir = argv[1];
    std::ifstream jobs(dir + "/jobs.txt");
    std::string line;
    int n = 0;
    try {
        while (std::getline(jobs, line)) {
            if (line.empty()) continue;
            std::istringstream ss(line);
            std::string op, conv, in, out, extra;
            std::size_t order = 0;
            ss >> op >> conv >> order >> in >> out >> extra;
            const std::vector<double> x = read_doubles(dir + "/" + in);
            if (op == "vjp_checks") {
                run_vjp_checks(dir + "/" + out);
                ++n;
                continue;
            }
            if (op == "zt_fwd" || op == "zt_bwd") run_zt(op, conv, order, x, dir + "/" + out);
            else if (op == "st_fwd" || op == "st_bwd") run_st(op, conv, order, x, dir + "/" + out);
            else if (op == "zt_eval" || op == "st_eval" || op == "zt_ps")
                run_eval(op, conv, order, x, dir + "/" + out, read_doubles(dir + "/" + extra));
            else run_rot(op, conv, order, x, dir + "/" + out, read_doubles(dir + "/" + extra));
            ++n;
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "job failed (%s): %s\n", line.c_str(), e.what());
        return 1;
    }
    std::printf("%d jobs done\n", n);
    return 0;
}
