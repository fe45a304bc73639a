// C++20 interface of zest_gb300 with the reference's API (sebsassi/zest):
// the same namespaces, class templates, aliases and member functions for the
// Gauss-Legendre-quadrature transforms and rotations, each call forwarded to
// the C-ABI of libzest_gb300 (zest_gpu.h), which runs it on the GPU.
//
// Code written against the reference's
//     zest::zt::GLQTransformerGeo<> transformer(order);
//     transformer.forward_transform(grid, expansion);
//     zest::Rotor rotor(order);
//     rotor.rotate(expansion, wigner_d_pi2, euler_angles, zest::RotationType::object);
// compiles unchanged against these headers.  The conventions are template
// parameters, so a grid, an expansion and a transformer of different
// conventions do not combine: the mismatch is a compile-time error, as in the
// reference.
//
// Interfaces kept (reference file:line):
//   zt::LonLatRadLayout, BallGLQGridSpan, BallGLQGrid     zernike_glq_transformer.hpp:50-501
//   zt::GLQTransformer and its aliases                     zernike_glq_transformer.hpp:510-1025
//   zt::RealZernikeSpan, RealZernikeExpansion + aliases    zernike_expansion.hpp:156-447
//   st::LonLatLayout, LatLonLayout, SphereGLQGrid(Span)    sh_glq_transformer.hpp:48-504
//   st::GLQTransformer and its aliases                     sh_glq_transformer.hpp:520-1240
//   st::RealSHSpan, RealSHExpansion + aliases              real_sh_expansion.hpp:49-292
//   WignerdPiHalfCollection                                wignerd_collection.hpp:66-110
//   Rotor, RotationType, euler_angles_from_rotation_matrix rotor.hpp:38-395
//   st::GridEvaluator, zt::GridEvaluator                   grid_evaluator.hpp:52-325
//   st::power_spectrum, cross_power_spectrum, zt::power_spectrum, zt::RadialZernikeSpan
//                                                          power_spectra.hpp:38-163
//
// Additions of this implementation:
//   * GPUContext: the device, stream and cached tables behind a transformer or
//     rotor (zest_gpu_ctx_create).  Every transformer and rotor owns one; like
//     the reference's transformers they are not thread-safe.
//   * transformer.set_precision(Precision::split): the tensor-core form of the
//     Zernike contractions.
//   * *_batch member functions: many grids / expansions in one call, on host
//     or device memory.
// Errors throw zest::GPUError carrying the library's status code and message.
#pragma once

#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <complex>
#include <concepts>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <new>
#include <numbers>
#include <span>
#include <stdexcept>
#include <type_traits>
#include <utility>
#include <vector>

#include "../zest_gpu.h"

namespace zest {

// ---------------------------------------------------------------------------
// Errors, device context, storage
// ---------------------------------------------------------------------------
class GPUError : public std::runtime_error {
public:
    GPUError(int code, const char* message) : std::runtime_error(message), m_code(code) {}
    [[nodiscard]] int code() const noexcept { return m_code; }

private:
    int m_code;
};

namespace detail {
inline void check(int status) {
    if (status != ZEST_GPU_OK) throw GPUError(status, zest_gpu_last_error());
}
constexpr std::size_t pad8(std::size_t n) noexcept { return (n + 7) & ~std::size_t(7); }
}  // namespace detail

enum class Precision { fp64 = ZEST_PRECISION_FP64, split = ZEST_PRECISION_SPLIT };
enum class MemoryKind { device = ZEST_MEM_DEVICE, host = ZEST_MEM_HOST };

// Owner of one zest_gpu_context: a device, a stream (nullptr = the default
// stream), cached tables and scratch.
class GPUContext {
public:
    explicit GPUContext(int device = 0, void* stream = nullptr) {
        detail::check(zest_gpu_ctx_create(&m_ctx, device, stream));
    }
    ~GPUContext() {
        if (m_ctx) zest_gpu_ctx_destroy(m_ctx);
    }
    GPUContext(GPUContext&& other) noexcept : m_ctx(std::exchange(other.m_ctx, nullptr)) {}
    GPUContext& operator=(GPUContext&& other) noexcept {
        std::swap(m_ctx, other.m_ctx);
        return *this;
    }
    GPUContext(const GPUContext&) = delete;
    GPUContext& operator=(const GPUContext&) = delete;

    [[nodiscard]] zest_gpu_context* get() const noexcept { return m_ctx; }
    void set_precision(Precision precision, int slices = 0) {
        detail::check(zest_gpu_set_precision(m_ctx, int(precision), slices));
    }
    void synchronize() { detail::check(zest_gpu_synchronize(m_ctx)); }
    void set_autotune(bool enable) { detail::check(zest_gpu_set_autotune(m_ctx, int(enable))); }
    void set_host_chunk_bytes(std::size_t bytes) { detail::check(zest_gpu_set_host_chunk_bytes(m_ctx, bytes)); }

private:
    zest_gpu_context* m_ctx = nullptr;
};

namespace detail {
// The reference's free functions (spectra, expansion conversions) run on a
// context per thread.
inline GPUContext& thread_context() {
    thread_local GPUContext ctx(0);
    return ctx;
}
}  // namespace detail

// ---------------------------------------------------------------------------
// Coefficient layouts, include/layout.hpp:36-420
// ---------------------------------------------------------------------------
enum class IndexingMode { negative, nonnegative };
enum class Parity { even = 0, odd = 1 };

// (l, m), 0 <= m <= l (or -l <= m <= l) at l(l+1)/2 + m (l(l+1) + m)
template <IndexingMode indexing_mode_param>
struct TriangleLayout {
    using index_type = std::conditional_t<indexing_mode_param == IndexingMode::negative, int, std::size_t>;
    using size_type = std::size_t;
    static constexpr IndexingMode indexing_mode = indexing_mode_param;
    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept {
        if constexpr (indexing_mode == IndexingMode::nonnegative) return (order * (order + 1)) >> 1;
        else return order * order;
    }
    [[nodiscard]] static constexpr std::size_t idx(index_type l, index_type m) noexcept {
        if constexpr (indexing_mode == IndexingMode::nonnegative) return ((l * (l + 1)) >> 1) + m;
        else return std::size_t(l * (l + 1) + m);
    }
};

// Rows of one parity of l only, (l, m) at floor(l^2/4) + m (l(l+1)/2 + m):
// the (l, m) coefficients of one radial index n of a Zernike expansion
template <IndexingMode indexing_mode_param>
struct RowSkippingTriangleLayout {
    using index_type = std::conditional_t<indexing_mode_param == IndexingMode::negative, int, std::size_t>;
    using size_type = std::size_t;
    static constexpr IndexingMode indexing_mode = indexing_mode_param;
    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept {
        if constexpr (indexing_mode == IndexingMode::nonnegative) return ((order + 1) * (order + 1)) >> 2;
        else return (order * (order + 1)) >> 1;
    }
    [[nodiscard]] static constexpr std::size_t idx(index_type l, index_type m) noexcept {
        if constexpr (indexing_mode == IndexingMode::nonnegative) return ((l * l) >> 2) + m;
        else return std::size_t(((l * (l + 1)) >> 1) + m);
    }
};

// (n, l, m), l = n mod 2, .., n: (n+1)(n+3)(2n+1)/24 + floor(l^2/4) + m
template <IndexingMode indexing_mode_param>
struct ZernikeTetrahedralLayout {
    using index_type = std::conditional_t<indexing_mode_param == IndexingMode::negative, int, std::size_t>;
    using size_type = std::size_t;
    static constexpr IndexingMode indexing_mode = indexing_mode_param;
    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept {
        if constexpr (indexing_mode == IndexingMode::nonnegative) return (order + 1) * (order + 3) * (2 * order + 1) / 24;
        else return order * (order + 1) * (order + 2) / 6;
    }
    [[nodiscard]] static constexpr std::size_t idx(index_type n, index_type l, index_type m) noexcept {
        if constexpr (indexing_mode == IndexingMode::nonnegative)
            return (n + 1) * (n + 3) * (2 * n + 1) / 24 + ((l * l) >> 2) + m;
        else
            return std::size_t(n * (n + 1) * (n + 2) / 6 + ((l * (l + 1)) >> 1) + m);
    }
};

// Containers are cache-line (64-byte) aligned, as the reference's.
template <typename T>
struct CacheLineAllocator {
    using value_type = T;
    CacheLineAllocator() noexcept = default;
    template <typename U>
    CacheLineAllocator(const CacheLineAllocator<U>&) noexcept {}
    T* allocate(std::size_t n) { return static_cast<T*>(::operator new(n * sizeof(T), std::align_val_t(64))); }
    void deallocate(T* p, std::size_t) noexcept { ::operator delete(p, std::align_val_t(64)); }
    template <typename U>
    bool operator==(const CacheLineAllocator<U>&) const noexcept { return true; }
};
template <typename T>
using AlignedVector = std::vector<T, CacheLineAllocator<T>>;

// Grid alignment policy of the layouts: the fastest axis padded to 8 doubles.
struct CacheLineAlignment {};

enum class RotationType { object, coordinate };

// ---------------------------------------------------------------------------
// Spherical harmonics
// ---------------------------------------------------------------------------
namespace st {

enum class SHPhase { none = -1, cs = 1 };
enum class SHNorm { geo, qm };

namespace detail {
constexpr int abi(SHNorm n) noexcept { return n == SHNorm::geo ? ZEST_SH_GEO : ZEST_SH_QM; }
constexpr int abi(SHPhase p) noexcept { return p == SHPhase::none ? ZEST_SH_PHASE_NONE : ZEST_SH_PHASE_CS; }
inline constexpr double inv_sqrtpi = 0.564189583547756286948079451560772586;
}  // namespace detail

// Normalisation constant of the SH coefficients, sh_conventions.hpp:56-63:
// 1 (qm) or 1/(4 pi) (geo).
template <SHNorm sh_norm_param>
[[nodiscard]] constexpr double normalization() noexcept {
    if constexpr (sh_norm_param == SHNorm::qm) return 1.0;
    else return 1.0 / (4.0 * 3.141592653589793238462643383279502884);
}

// Factor converting coefficients between SH normalisations,
// sh_conventions.hpp:73-96 (the same operations, so the same double).
template <SHNorm from, SHNorm to>
[[nodiscard]] constexpr double conversion_const() noexcept {
    if constexpr (from == to) {
        return 1.0;
    } else {
        constexpr double inv_sqrt_4pi = 0.5 * detail::inv_sqrtpi;
        constexpr double sqrt_4pi = 1.0 / inv_sqrt_4pi;
        double norm = from == SHNorm::qm ? 1.0 : sqrt_4pi;
        norm *= to == SHNorm::qm ? 1.0 : inv_sqrt_4pi;
        return norm;
    }
}

// An expansion holding the rows of one parity of l in the row-skipping layout
// (a zt::ZernikeSHSpan), real_sh_expansion.hpp:309-316.
template <typename T>
concept row_skipping_real_sh_expansion =
    std::same_as<typename std::remove_cvref_t<T>::Layout, RowSkippingTriangleLayout<IndexingMode::nonnegative>> &&
    requires {
        { std::remove_cvref_t<T>::norm } -> std::convertible_to<SHNorm>;
        { std::remove_cvref_t<T>::phase } -> std::convertible_to<SHPhase>;
    };

// [lon][lat]: (2L - 1, pad8(L))
template <typename AlignmentType = CacheLineAlignment>
struct LonLatLayout {
    using Alignment = AlignmentType;
    static constexpr int abi = ZEST_LAYOUT_LONLAT;
    [[nodiscard]] static constexpr std::size_t lon_size(std::size_t order) noexcept {
        return 2 * order - std::min<std::size_t>(1, order);
    }
    [[nodiscard]] static constexpr std::size_t lat_size(std::size_t order) noexcept { return zest::detail::pad8(order); }
    [[nodiscard]] static constexpr std::array<std::size_t, 2> shape(std::size_t order) noexcept {
        return {lon_size(order), lat_size(order)};
    }
    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept {
        return lon_size(order) * lat_size(order);
    }
    static constexpr std::size_t lat_axis = 1;
    static constexpr std::size_t lon_axis = 0;
};

// [lat][lon]: (L, pad8(2L - 1))
template <typename AlignmentType = CacheLineAlignment>
struct LatLonLayout {
    using Alignment = AlignmentType;
    static constexpr int abi = ZEST_LAYOUT_LATLON;
    [[nodiscard]] static constexpr std::size_t lat_size(std::size_t order) noexcept { return order; }
    [[nodiscard]] static constexpr std::size_t lon_size(std::size_t order) noexcept {
        return zest::detail::pad8(2 * order - std::min<std::size_t>(1, order));
    }
    [[nodiscard]] static constexpr std::array<std::size_t, 2> shape(std::size_t order) noexcept {
        return {lat_size(order), lon_size(order)};
    }
    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept {
        return lon_size(order) * lat_size(order);
    }
    static constexpr std::size_t lat_axis = 0;
    static constexpr std::size_t lon_axis = 1;
};

using DefaultLayout = LonLatLayout<>;

// Non-owning view of grid values on the sphere.
template <typename ElementType, typename LayoutType = DefaultLayout>
class SphereGLQGridSpan {
public:
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    using Layout = LayoutType;
    using ConstView = SphereGLQGridSpan<const value_type, Layout>;

    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept { return Layout::size(order); }
    [[nodiscard]] static constexpr std::array<std::size_t, 2> shape(std::size_t order) noexcept {
        return Layout::shape(order);
    }

    SphereGLQGridSpan() noexcept = default;
    constexpr SphereGLQGridSpan(element_type* data, std::size_t order) noexcept : m_data(data), m_order(order) {}
    constexpr SphereGLQGridSpan(std::span<element_type> buffer, std::size_t order) noexcept
        : m_data(buffer.data()), m_order(order) {}

    [[nodiscard]] constexpr std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] constexpr std::array<std::size_t, 2> shape() const noexcept { return Layout::shape(m_order); }
    [[nodiscard]] constexpr std::size_t size() const noexcept { return Layout::size(m_order); }
    [[nodiscard]] constexpr element_type* data() const noexcept { return m_data; }
    [[nodiscard]] constexpr std::span<element_type> flatten() const noexcept { return {m_data, size()}; }
    [[nodiscard]] constexpr element_type& operator()(std::size_t i, std::size_t j) const noexcept {
        return m_data[i * shape()[1] + j];
    }
    [[nodiscard]] constexpr operator ConstView() const noexcept
        requires(!std::is_const_v<ElementType>)
    {
        return ConstView(m_data, m_order);
    }

private:
    element_type* m_data = nullptr;
    std::size_t m_order = 0;
};

// Owning grid on the sphere.
template <typename ElementType = double, typename LayoutType = DefaultLayout>
class SphereGLQGrid {
public:
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    using Layout = LayoutType;
    using View = SphereGLQGridSpan<element_type, Layout>;
    using ConstView = SphereGLQGridSpan<const element_type, Layout>;

    SphereGLQGrid() = default;
    explicit SphereGLQGrid(std::size_t order) : m_values(Layout::size(order)), m_order(order) {}

    [[nodiscard]] std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] std::array<std::size_t, 2> shape() const noexcept { return Layout::shape(m_order); }
    [[nodiscard]] std::size_t size() const noexcept { return m_values.size(); }
    [[nodiscard]] element_type* data() noexcept { return m_values.data(); }
    [[nodiscard]] const element_type* data() const noexcept { return m_values.data(); }
    [[nodiscard]] std::span<element_type> flatten() noexcept { return m_values; }
    [[nodiscard]] std::span<const element_type> flatten() const noexcept { return m_values; }
    [[nodiscard]] element_type& operator()(std::size_t i, std::size_t j) noexcept {
        return m_values[i * shape()[1] + j];
    }
    void resize(std::size_t order) {
        m_values.resize(Layout::size(order));
        m_order = order;
    }
    [[nodiscard]] operator View() noexcept { return View(m_values.data(), m_order); }
    [[nodiscard]] operator ConstView() const noexcept { return ConstView(m_values.data(), m_order); }

private:
    AlignedVector<element_type> m_values;
    std::size_t m_order = 0;
};

// Either grid type of the sphere, sh_glq_transformer.hpp:367-377.
template <typename T>
concept sphere_glq_grid =
    std::same_as<std::remove_cvref_t<T>, SphereGLQGridSpan<typename std::remove_cvref_t<T>::element_type,
                                                           typename std::remove_cvref_t<T>::Layout>> ||
    std::same_as<std::remove_cvref_t<T>, SphereGLQGrid<typename std::remove_cvref_t<T>::element_type,
                                                       typename std::remove_cvref_t<T>::Layout>>;

// Real SH coefficients {cos, sin} of degree l and order m at l(l+1)/2 + m.
template <typename ElementType, SHNorm sh_norm_param, SHPhase sh_phase_param>
class RealSHSpan {
public:
    using Layout = TriangleLayout<IndexingMode::nonnegative>;
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    using ConstView = RealSHSpan<const value_type, sh_norm_param, sh_phase_param>;
    static constexpr SHNorm norm = sh_norm_param;
    static constexpr SHPhase phase = sh_phase_param;

    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept { return order * (order + 1) / 2; }
    [[nodiscard]] static constexpr std::size_t idx(std::size_t l, std::size_t m) noexcept {
        return l * (l + 1) / 2 + m;
    }

    RealSHSpan() noexcept = default;
    constexpr RealSHSpan(element_type* data, std::size_t order) noexcept : m_data(data), m_order(order) {}
    constexpr RealSHSpan(std::span<element_type> buffer, std::size_t order) noexcept
        : m_data(buffer.data()), m_order(order) {}

    [[nodiscard]] constexpr std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] constexpr std::size_t size() const noexcept { return size(m_order); }
    [[nodiscard]] constexpr element_type* data() const noexcept { return m_data; }
    [[nodiscard]] constexpr std::span<element_type> flatten() const noexcept { return {m_data, size()}; }
    [[nodiscard]] constexpr element_type& operator()(std::size_t l, std::size_t m) const noexcept {
        return m_data[idx(l, m)];
    }
    [[nodiscard]] constexpr operator ConstView() const noexcept
        requires(!std::is_const_v<ElementType>)
    {
        return ConstView(m_data, m_order);
    }

private:
    element_type* m_data = nullptr;
    std::size_t m_order = 0;
};

template <SHNorm sh_norm_param, SHPhase sh_phase_param, typename ElementType = std::array<double, 2>>
class RealSHExpansion {
public:
    using Layout = TriangleLayout<IndexingMode::nonnegative>;
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    using View = RealSHSpan<element_type, sh_norm_param, sh_phase_param>;
    using ConstView = RealSHSpan<const element_type, sh_norm_param, sh_phase_param>;
    static constexpr SHNorm norm = sh_norm_param;
    static constexpr SHPhase phase = sh_phase_param;

    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept { return order * (order + 1) / 2; }

    RealSHExpansion() = default;
    explicit RealSHExpansion(std::size_t order) : m_coeffs(size(order)), m_order(order) {}

    [[nodiscard]] std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] std::size_t size() const noexcept { return m_coeffs.size(); }
    [[nodiscard]] element_type* data() noexcept { return m_coeffs.data(); }
    [[nodiscard]] const element_type* data() const noexcept { return m_coeffs.data(); }
    [[nodiscard]] std::span<element_type> flatten() noexcept { return m_coeffs; }
    [[nodiscard]] std::span<const element_type> flatten() const noexcept { return m_coeffs; }
    [[nodiscard]] element_type& operator()(std::size_t l, std::size_t m) noexcept {
        return m_coeffs[View::idx(l, m)];
    }
    [[nodiscard]] const element_type& operator()(std::size_t l, std::size_t m) const noexcept {
        return m_coeffs[View::idx(l, m)];
    }
    void resize(std::size_t order) {
        m_coeffs.resize(size(order));
        m_order = order;
    }
    [[nodiscard]] operator View() noexcept { return View(m_coeffs.data(), m_order); }
    [[nodiscard]] operator ConstView() const noexcept { return ConstView(m_coeffs.data(), m_order); }

private:
    AlignedVector<element_type> m_coeffs;
    std::size_t m_order = 0;
};

template <typename ElementType>
using RealSHSpanAcoustics = RealSHSpan<ElementType, SHNorm::qm, SHPhase::none>;
template <typename ElementType>
using RealSHSpanQM = RealSHSpan<ElementType, SHNorm::qm, SHPhase::cs>;
template <typename ElementType>
using RealSHSpanGeo = RealSHSpan<ElementType, SHNorm::geo, SHPhase::none>;
using RealSHExpansionAcoustics = RealSHExpansion<SHNorm::qm, SHPhase::none>;
using RealSHExpansionQM = RealSHExpansion<SHNorm::qm, SHPhase::cs>;
using RealSHExpansionGeo = RealSHExpansion<SHNorm::geo, SHPhase::none>;

// An SH expansion type: its conventions are static members and it converts
// to the span of those conventions.
template <typename T>
concept real_sh_expansion = requires {
    { std::remove_cvref_t<T>::norm } -> std::convertible_to<SHNorm>;
    { std::remove_cvref_t<T>::phase } -> std::convertible_to<SHPhase>;
} && std::convertible_to<T, RealSHSpan<typename std::remove_cvref_t<T>::element_type,
                                       std::remove_cvref_t<T>::norm, std::remove_cvref_t<T>::phase>>;

namespace detail {
// In-place conversion of host (or device) coefficients on the device.
inline void convert(int kind, std::size_t order, void* data, int src_zn, int src_sn, int src_sp, int dst_zn,
                    int dst_sn, int dst_sp, bool to_complex, MemoryKind mem = MemoryKind::host) {
    zest::detail::check(zest_gpu_convert_expansion(zest::detail::thread_context().get(), kind, order, 1,
                                                   static_cast<double*>(data), src_zn, src_sn, src_sp, dst_zn,
                                                   dst_sn, dst_sp, int(to_complex), int(mem)));
}
}  // namespace detail

// Real SH expansion -> complex expansion of the destination conventions, in
// place (the input is modified; the result views the same data),
// real_sh_expansion.hpp:345-387.
template <SHNorm dest_sh_norm, SHPhase dest_sh_phase, real_sh_expansion ExpansionType>
RealSHSpan<std::complex<double>, dest_sh_norm, dest_sh_phase> to_complex_expansion(ExpansionType&& expansion) {
    using E = std::remove_cvref_t<ExpansionType>;
    detail::convert(ZEST_EXPANSION_SH, expansion.order(), expansion.data(), 0, detail::abi(E::norm),
                    detail::abi(E::phase), 0, detail::abi(dest_sh_norm), detail::abi(dest_sh_phase), true);
    return RealSHSpan<std::complex<double>, dest_sh_norm, dest_sh_phase>(
        reinterpret_cast<std::complex<double>*>(expansion.data()), expansion.order());
}

// Complex SH expansion -> real expansion of the destination conventions, in
// place, real_sh_expansion.hpp:399-436.
template <SHNorm dest_sh_norm, SHPhase dest_sh_phase, real_sh_expansion ExpansionType>
RealSHSpan<std::array<double, 2>, dest_sh_norm, dest_sh_phase> to_real_expansion(ExpansionType&& expansion) {
    using E = std::remove_cvref_t<ExpansionType>;
    detail::convert(ZEST_EXPANSION_SH, expansion.order(), expansion.data(), 0, detail::abi(E::norm),
                    detail::abi(E::phase), 0, detail::abi(dest_sh_norm), detail::abi(dest_sh_phase), false);
    return RealSHSpan<std::array<double, 2>, dest_sh_norm, dest_sh_phase>(
        reinterpret_cast<std::array<double, 2>*>(expansion.data()), expansion.order());
}

// Spherical-harmonic transforms on the GLQ grid, sh_glq_transformer.hpp:520-754.
template <SHNorm sh_norm_param, SHPhase sh_phase_param, typename GridLayoutType = DefaultLayout>
class GLQTransformer {
public:
    using GridLayout = GridLayoutType;
    static constexpr SHNorm sh_norm = sh_norm_param;
    static constexpr SHPhase phase = sh_phase_param;

    GLQTransformer() : GLQTransformer(0) {}
    explicit GLQTransformer(std::size_t order, int device = 0, void* stream = nullptr)
        : m_ctx(device, stream), m_order(order) {}

    [[nodiscard]] std::size_t order() const noexcept { return m_order; }
    void resize(std::size_t order) { m_order = order; }
    [[nodiscard]] GPUContext& context() noexcept { return m_ctx; }

    void forward_transform(SphereGLQGridSpan<const double, GridLayout> values,
                           RealSHSpan<std::array<double, 2>, sh_norm_param, sh_phase_param> expansion) {
        resize(values.order());
        forward_transform_batch(values.data(), values.order(), reinterpret_cast<double*>(expansion.data()),
                                expansion.order(), 1, MemoryKind::host);
    }
    void backward_transform(RealSHSpan<const std::array<double, 2>, sh_norm_param, sh_phase_param> expansion,
                            SphereGLQGridSpan<double, GridLayout> values) {
        resize(values.order());
        backward_transform_batch(reinterpret_cast<const double*>(expansion.data()), expansion.order(),
                                 values.data(), values.order(), 1, MemoryKind::host);
    }
    [[nodiscard]] RealSHExpansion<sh_norm_param, sh_phase_param> forward_transform(
        SphereGLQGridSpan<const double, GridLayout> values, std::size_t order) {
        RealSHExpansion<sh_norm_param, sh_phase_param> expansion(order);
        forward_transform(values, expansion);
        return expansion;
    }
    [[nodiscard]] SphereGLQGrid<double, GridLayout> backward_transform(
        RealSHSpan<const std::array<double, 2>, sh_norm_param, sh_phase_param> expansion, std::size_t order) {
        SphereGLQGrid<double, GridLayout> grid(order);
        backward_transform(expansion, grid);
        return grid;
    }

    // Backward transform of an expansion of one parity of l (a zt::ZernikeSHSpan),
    // sh_glq_transformer.hpp:680-700 and :743-754.
    template <row_skipping_real_sh_expansion Expansion>
        requires(std::remove_cvref_t<Expansion>::norm == sh_norm_param) &&
                (std::remove_cvref_t<Expansion>::phase == sh_phase_param) &&
                std::same_as<typename std::remove_cvref_t<Expansion>::value_type, std::array<double, 2>>
    void backward_transform(Expansion&& expansion, SphereGLQGridSpan<double, GridLayout> values) {
        resize(values.order());
        zest::detail::check(zest_gpu_st_backward_rows(
            m_ctx.get(), detail::abi(sh_norm_param), detail::abi(sh_phase_param), GridLayout::abi, expansion.order(),
            values.order(), 1, reinterpret_cast<const double*>(expansion.data()), values.data(), ZEST_MEM_HOST));
    }
    template <row_skipping_real_sh_expansion Expansion>
        requires(std::remove_cvref_t<Expansion>::norm == sh_norm_param) &&
                (std::remove_cvref_t<Expansion>::phase == sh_phase_param) &&
                std::same_as<typename std::remove_cvref_t<Expansion>::value_type, std::array<double, 2>>
    [[nodiscard]] SphereGLQGrid<double, GridLayout> backward_transform(Expansion&& expansion, std::size_t order) {
        SphereGLQGrid<double, GridLayout> grid(order);
        backward_transform(std::forward<Expansion>(expansion), grid);
        return grid;
    }

    // `batch` contiguous grids of grid_order -> expansions of exp_order.
    void forward_transform_batch(const double* grids, std::size_t grid_order, double* coeffs, std::size_t exp_order,
                                 std::size_t batch, MemoryKind mem) {
        zest::detail::check(zest_gpu_st_forward(m_ctx.get(), detail::abi(sh_norm_param), detail::abi(sh_phase_param),
                                                GridLayout::abi, grid_order, exp_order, batch, grids, coeffs,
                                                int(mem)));
    }
    void backward_transform_batch(const double* coeffs, std::size_t exp_order, double* grids, std::size_t grid_order,
                                  std::size_t batch, MemoryKind mem) {
        zest::detail::check(zest_gpu_st_backward(m_ctx.get(), detail::abi(sh_norm_param), detail::abi(sh_phase_param),
                                                 GridLayout::abi, exp_order, grid_order, batch, coeffs, grids,
                                                 int(mem)));
    }

    // Vector-Jacobian products (adjoints) of the two transforms: the grid
    // cotangent of forward_transform from its coefficient cotangent, and the
    // coefficient cotangent of backward_transform from its grid cotangent.
    void forward_transform_vjp(RealSHSpan<const std::array<double, 2>, sh_norm_param, sh_phase_param> expansion_cot,
                               SphereGLQGridSpan<double, GridLayout> values_cot) {
        zest::detail::check(zest_gpu_st_forward_vjp(
            m_ctx.get(), detail::abi(sh_norm_param), detail::abi(sh_phase_param), GridLayout::abi, values_cot.order(),
            expansion_cot.order(), 1, reinterpret_cast<const double*>(expansion_cot.data()), values_cot.data(),
            ZEST_MEM_HOST));
    }
    void backward_transform_vjp(SphereGLQGridSpan<const double, GridLayout> values_cot,
                                RealSHSpan<std::array<double, 2>, sh_norm_param, sh_phase_param> expansion_cot) {
        zest::detail::check(zest_gpu_st_backward_vjp(
            m_ctx.get(), detail::abi(sh_norm_param), detail::abi(sh_phase_param), GridLayout::abi,
            expansion_cot.order(), values_cot.order(), 1, values_cot.data(),
            reinterpret_cast<double*>(expansion_cot.data()), ZEST_MEM_HOST));
    }

private:
    GPUContext m_ctx;
    std::size_t m_order;
};

template <typename GridLayout = DefaultLayout>
using GLQTransformerAcoustics = GLQTransformer<SHNorm::qm, SHPhase::none, GridLayout>;
template <typename GridLayout = DefaultLayout>
using GLQTransformerQM = GLQTransformer<SHNorm::qm, SHPhase::cs, GridLayout>;
template <typename GridLayout = DefaultLayout>
using GLQTransformerGeo = GLQTransformer<SHNorm::geo, SHPhase::none, GridLayout>;

}  // namespace st

// ---------------------------------------------------------------------------
// 3D Zernike functions on the unit ball
// ---------------------------------------------------------------------------
namespace zt {

enum class ZernikeNorm { normed, unnormed };

namespace detail {
constexpr int abi(ZernikeNorm n) noexcept {
    return n == ZernikeNorm::normed ? ZEST_ZERNIKE_NORMED : ZEST_ZERNIKE_UNNORMED;
}
}  // namespace detail

// Normalisation of the radial Zernike functions, zernike_conventions.hpp:44-51.
template <ZernikeNorm zernike_norm_param>
[[nodiscard]] inline double normalization(std::size_t n) noexcept {
    if constexpr (zernike_norm_param == ZernikeNorm::normed) return 1.0;
    else return double(2 * n + 3);
}

// Factor converting coefficients between Zernike normalisations,
// zernike_conventions.hpp:61-76.
template <ZernikeNorm from, ZernikeNorm to>
[[nodiscard]] inline double conversion_factor(std::size_t n) noexcept {
    if constexpr (from == to) return 1.0;
    else if constexpr (to == ZernikeNorm::normed) return 1.0 / std::sqrt(double(2 * n + 3));
    else return std::sqrt(double(2 * n + 3));
}

// The (l, m) coefficients of one radial index n of a Zernike expansion: a
// span of `order` = n + 1 in the row-skipping layout (rows l = n mod 2, .., n),
// zernike_expansion.hpp:103-140.
template <typename ElementType, typename LayoutType, ZernikeNorm zernike_norm_param, st::SHNorm sh_norm_param,
          st::SHPhase sh_phase_param>
    requires std::same_as<LayoutType, RowSkippingTriangleLayout<LayoutType::indexing_mode>>
class ZernikeSHSpan {
public:
    using Layout = LayoutType;
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    using index_type = typename Layout::index_type;
    using ConstView = ZernikeSHSpan<const value_type, LayoutType, zernike_norm_param, sh_norm_param, sh_phase_param>;
    static constexpr ZernikeNorm zernike_norm = zernike_norm_param;
    static constexpr st::SHNorm norm = sh_norm_param;
    static constexpr st::SHPhase phase = sh_phase_param;

    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept { return Layout::size(order); }

    constexpr ZernikeSHSpan() noexcept = default;
    constexpr ZernikeSHSpan(element_type* data, std::size_t order) noexcept
        : m_data(data), m_size(Layout::size(order)), m_order(order) {}
    constexpr ZernikeSHSpan(std::span<element_type> buffer, std::size_t order) noexcept
        : m_data(buffer.data()), m_size(Layout::size(order)), m_order(order) {}
    constexpr ZernikeSHSpan(element_type* data, std::size_t size, std::size_t order) noexcept
        : m_data(data), m_size(size), m_order(order) {}

    [[nodiscard]] constexpr std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] constexpr std::size_t size() const noexcept { return m_size; }
    [[nodiscard]] constexpr element_type* data() const noexcept { return m_data; }
    [[nodiscard]] constexpr std::span<element_type> flatten() const noexcept { return {m_data, m_size}; }
    // rows of the parity of order - 1
    [[nodiscard]] constexpr Parity parity() const noexcept { return Parity((m_order & 1) ^ 1); }
    [[nodiscard]] constexpr element_type& operator()(index_type l, index_type m) const noexcept {
        return m_data[Layout::idx(l, m)];
    }
    [[nodiscard]] constexpr operator ConstView() const noexcept
        requires(!std::is_const_v<ElementType>)
    {
        return ConstView(m_data, m_size, m_order);
    }

private:
    element_type* m_data = nullptr;
    std::size_t m_size = 0;
    std::size_t m_order = 0;
};

// [lon][lat][rad]: (2L - 1, L + 1, pad8(L + 1))
template <typename AlignmentType = CacheLineAlignment>
struct LonLatRadLayout {
    using Alignment = AlignmentType;
    [[nodiscard]] static constexpr std::size_t lon_size(std::size_t order) noexcept {
        return 2 * order - std::min<std::size_t>(1, order);
    }
    [[nodiscard]] static constexpr std::size_t lat_size(std::size_t order) noexcept { return order + 1; }
    [[nodiscard]] static constexpr std::size_t rad_size(std::size_t order) noexcept {
        return zest::detail::pad8(order + 1);
    }
    [[nodiscard]] static constexpr std::array<std::size_t, 3> shape(std::size_t order) noexcept {
        return {lon_size(order), lat_size(order), rad_size(order)};
    }
    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept {
        return lon_size(order) * lat_size(order) * rad_size(order);
    }
};

using DefaultLayout = LonLatRadLayout<>;

template <typename ElementType, typename LayoutType = DefaultLayout>
class BallGLQGridSpan {
public:
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    using Layout = LayoutType;
    using ConstView = BallGLQGridSpan<const value_type, Layout>;

    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept { return Layout::size(order); }
    [[nodiscard]] static constexpr std::array<std::size_t, 3> shape(std::size_t order) noexcept {
        return Layout::shape(order);
    }

    BallGLQGridSpan() noexcept = default;
    constexpr BallGLQGridSpan(element_type* data, std::size_t order) noexcept : m_data(data), m_order(order) {}
    constexpr BallGLQGridSpan(std::span<element_type> buffer, std::size_t order) noexcept
        : m_data(buffer.data()), m_order(order) {}

    [[nodiscard]] constexpr std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] constexpr std::array<std::size_t, 3> shape() const noexcept { return Layout::shape(m_order); }
    [[nodiscard]] constexpr std::size_t size() const noexcept { return Layout::size(m_order); }
    [[nodiscard]] constexpr element_type* data() const noexcept { return m_data; }
    [[nodiscard]] constexpr std::span<element_type> flatten() const noexcept { return {m_data, size()}; }
    [[nodiscard]] constexpr element_type& operator()(std::size_t i, std::size_t j, std::size_t k) const noexcept {
        const auto s = shape();
        return m_data[(i * s[1] + j) * s[2] + k];
    }
    [[nodiscard]] constexpr operator ConstView() const noexcept
        requires(!std::is_const_v<ElementType>)
    {
        return ConstView(m_data, m_order);
    }

private:
    element_type* m_data = nullptr;
    std::size_t m_order = 0;
};

template <typename ElementType = double, typename LayoutType = DefaultLayout>
class BallGLQGrid {
public:
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    using Layout = LayoutType;
    using View = BallGLQGridSpan<element_type, Layout>;
    using ConstView = BallGLQGridSpan<const element_type, Layout>;

    BallGLQGrid() = default;
    explicit BallGLQGrid(std::size_t order) : m_values(Layout::size(order)), m_order(order) {}

    [[nodiscard]] std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] std::array<std::size_t, 3> shape() const noexcept { return Layout::shape(m_order); }
    [[nodiscard]] std::size_t size() const noexcept { return m_values.size(); }
    [[nodiscard]] element_type* data() noexcept { return m_values.data(); }
    [[nodiscard]] const element_type* data() const noexcept { return m_values.data(); }
    [[nodiscard]] std::span<element_type> flatten() noexcept { return m_values; }
    [[nodiscard]] std::span<const element_type> flatten() const noexcept { return m_values; }
    [[nodiscard]] element_type& operator()(std::size_t i, std::size_t j, std::size_t k) noexcept {
        const auto s = shape();
        return m_values[(i * s[1] + j) * s[2] + k];
    }
    void resize(std::size_t order) {
        m_values.resize(Layout::size(order));
        m_order = order;
    }
    [[nodiscard]] operator View() noexcept { return View(m_values.data(), m_order); }
    [[nodiscard]] operator ConstView() const noexcept { return ConstView(m_values.data(), m_order); }

private:
    AlignedVector<element_type> m_values;
    std::size_t m_order = 0;
};

// Either grid type of the ball, zernike_glq_transformer.hpp:318-328.
template <typename T>
concept ball_glq_grid =
    std::same_as<std::remove_cvref_t<T>, BallGLQGridSpan<typename std::remove_cvref_t<T>::element_type,
                                                         typename std::remove_cvref_t<T>::Layout>> ||
    std::same_as<std::remove_cvref_t<T>, BallGLQGrid<typename std::remove_cvref_t<T>::element_type,
                                                     typename std::remove_cvref_t<T>::Layout>>;

// Real Zernike coefficients {cos, sin} of (n, l, m), n - l even, at
// (n+1)(n+3)(2n+1)/24 + floor(l^2/4) + m.
template <typename ElementType, ZernikeNorm zernike_norm_param, st::SHNorm sh_norm_param,
          st::SHPhase sh_phase_param>
class RealZernikeSpan {
public:
    using Layout = ZernikeTetrahedralLayout<IndexingMode::nonnegative>;
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    using ConstView = RealZernikeSpan<const value_type, zernike_norm_param, sh_norm_param, sh_phase_param>;
    using SubSpan = ZernikeSHSpan<ElementType, RowSkippingTriangleLayout<IndexingMode::nonnegative>,
                                  zernike_norm_param, sh_norm_param, sh_phase_param>;
    static constexpr ZernikeNorm zernike_norm = zernike_norm_param;
    static constexpr st::SHNorm sh_norm = sh_norm_param;
    static constexpr st::SHPhase sh_phase = sh_phase_param;

    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept {
        return (order + 1) * (order + 3) * (2 * order + 1) / 24;
    }
    [[nodiscard]] static constexpr std::size_t idx(std::size_t n, std::size_t l, std::size_t m) noexcept {
        return (n + 1) * (n + 3) * (2 * n + 1) / 24 + (l * l) / 4 + m;
    }

    RealZernikeSpan() noexcept = default;
    constexpr RealZernikeSpan(element_type* data, std::size_t order) noexcept : m_data(data), m_order(order) {}
    constexpr RealZernikeSpan(std::span<element_type> buffer, std::size_t order) noexcept
        : m_data(buffer.data()), m_order(order) {}

    [[nodiscard]] constexpr std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] constexpr std::size_t size() const noexcept { return size(m_order); }
    [[nodiscard]] constexpr element_type* data() const noexcept { return m_data; }
    [[nodiscard]] constexpr std::span<element_type> flatten() const noexcept { return {m_data, size()}; }
    [[nodiscard]] constexpr element_type& operator()(std::size_t n, std::size_t l, std::size_t m) const noexcept {
        return m_data[idx(n, l, m)];
    }
    // the (l, m) coefficients of radial index n, zernike_expansion.hpp:186-190
    [[nodiscard]] constexpr SubSpan operator[](std::size_t n) const noexcept {
        return SubSpan(m_data + idx(n, 0, 0), n + 1);
    }
    [[nodiscard]] constexpr operator ConstView() const noexcept
        requires(!std::is_const_v<ElementType>)
    {
        return ConstView(m_data, m_order);
    }

private:
    element_type* m_data = nullptr;
    std::size_t m_order = 0;
};

template <ZernikeNorm zernike_norm_param, st::SHNorm sh_norm_param, st::SHPhase sh_phase_param,
          typename ElementType = std::array<double, 2>>
class RealZernikeExpansion {
public:
    using Layout = ZernikeTetrahedralLayout<IndexingMode::nonnegative>;
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    using View = RealZernikeSpan<element_type, zernike_norm_param, sh_norm_param, sh_phase_param>;
    using ConstView = RealZernikeSpan<const element_type, zernike_norm_param, sh_norm_param, sh_phase_param>;
    static constexpr ZernikeNorm zernike_norm = zernike_norm_param;
    static constexpr st::SHNorm sh_norm = sh_norm_param;
    static constexpr st::SHPhase sh_phase = sh_phase_param;

    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept { return View::size(order); }

    RealZernikeExpansion() = default;
    explicit RealZernikeExpansion(std::size_t order) : m_coeffs(size(order)), m_order(order) {}

    [[nodiscard]] std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] std::size_t size() const noexcept { return m_coeffs.size(); }
    [[nodiscard]] element_type* data() noexcept { return m_coeffs.data(); }
    [[nodiscard]] const element_type* data() const noexcept { return m_coeffs.data(); }
    [[nodiscard]] std::span<element_type> flatten() noexcept { return m_coeffs; }
    [[nodiscard]] std::span<const element_type> flatten() const noexcept { return m_coeffs; }
    [[nodiscard]] element_type& operator()(std::size_t n, std::size_t l, std::size_t m) noexcept {
        return m_coeffs[View::idx(n, l, m)];
    }
    [[nodiscard]] const element_type& operator()(std::size_t n, std::size_t l, std::size_t m) const noexcept {
        return m_coeffs[View::idx(n, l, m)];
    }
    void resize(std::size_t order) {
        m_coeffs.resize(size(order));
        m_order = order;
    }
    [[nodiscard]] operator View() noexcept { return View(m_coeffs.data(), m_order); }
    [[nodiscard]] operator ConstView() const noexcept { return ConstView(m_coeffs.data(), m_order); }

private:
    AlignedVector<element_type> m_coeffs;
    std::size_t m_order = 0;
};

// Aliases of the reference, zernike_expansion.hpp:233-447 (its
// RealZernikeSpanNormalAcoustics names ZernikeNorm::unnormed; kept so).
template <typename ElementType>
using RealZernikeSpanAcoustics = RealZernikeSpan<ElementType, ZernikeNorm::unnormed, st::SHNorm::qm, st::SHPhase::none>;
template <typename ElementType>
using RealZernikeSpanNormalAcoustics
    = RealZernikeSpan<ElementType, ZernikeNorm::unnormed, st::SHNorm::qm, st::SHPhase::none>;
template <typename ElementType>
using RealZernikeSpanQM = RealZernikeSpan<ElementType, ZernikeNorm::unnormed, st::SHNorm::qm, st::SHPhase::cs>;
template <typename ElementType>
using RealZernikeSpanNormalQM = RealZernikeSpan<ElementType, ZernikeNorm::normed, st::SHNorm::qm, st::SHPhase::cs>;
template <typename ElementType>
using RealZernikeSpanGeo = RealZernikeSpan<ElementType, ZernikeNorm::unnormed, st::SHNorm::geo, st::SHPhase::none>;
template <typename ElementType>
using RealZernikeSpanNormalGeo = RealZernikeSpan<ElementType, ZernikeNorm::normed, st::SHNorm::geo, st::SHPhase::none>;
using RealZernikeExpansionAcoustics = RealZernikeExpansion<ZernikeNorm::unnormed, st::SHNorm::qm, st::SHPhase::none>;
using RealZernikeExpansionNormalAcoustics = RealZernikeExpansion<ZernikeNorm::normed, st::SHNorm::qm, st::SHPhase::none>;
using RealZernikeExpansionQM = RealZernikeExpansion<ZernikeNorm::unnormed, st::SHNorm::qm, st::SHPhase::cs>;
using RealZernikeExpansionNormalQM = RealZernikeExpansion<ZernikeNorm::normed, st::SHNorm::qm, st::SHPhase::cs>;
using RealZernikeExpansionGeo = RealZernikeExpansion<ZernikeNorm::unnormed, st::SHNorm::geo, st::SHPhase::none>;
using RealZernikeExpansionNormalGeo = RealZernikeExpansion<ZernikeNorm::normed, st::SHNorm::geo, st::SHPhase::none>;

template <typename T>
concept real_zernike_expansion = requires {
    { std::remove_cvref_t<T>::zernike_norm } -> std::convertible_to<ZernikeNorm>;
    { std::remove_cvref_t<T>::sh_norm } -> std::convertible_to<st::SHNorm>;
    { std::remove_cvref_t<T>::sh_phase } -> std::convertible_to<st::SHPhase>;
} && std::convertible_to<T, RealZernikeSpan<typename std::remove_cvref_t<T>::element_type,
                                            std::remove_cvref_t<T>::zernike_norm, std::remove_cvref_t<T>::sh_norm,
                                            std::remove_cvref_t<T>::sh_phase>>;

// Real Zernike expansion -> complex expansion of the destination conventions,
// in place (the input is modified; the result views the same data),
// zernike_expansion.hpp:484-557.
template <ZernikeNorm dest_zernike_norm, st::SHNorm dest_sh_norm, st::SHPhase dest_sh_phase,
          real_zernike_expansion ExpansionType>
RealZernikeSpan<std::complex<double>, dest_zernike_norm, dest_sh_norm, dest_sh_phase> to_complex_expansion(
    ExpansionType&& expansion) {
    using E = std::remove_cvref_t<ExpansionType>;
    st::detail::convert(ZEST_EXPANSION_ZERNIKE, expansion.order(), expansion.data(), detail::abi(E::zernike_norm),
                        st::detail::abi(E::sh_norm), st::detail::abi(E::sh_phase), detail::abi(dest_zernike_norm),
                        st::detail::abi(dest_sh_norm), st::detail::abi(dest_sh_phase), true);
    return RealZernikeSpan<std::complex<double>, dest_zernike_norm, dest_sh_norm, dest_sh_phase>(
        reinterpret_cast<std::complex<double>*>(expansion.data()), expansion.order());
}

// Complex Zernike expansion -> real expansion, in place, zernike_expansion.hpp:568-634.
template <ZernikeNorm dest_zernike_norm, st::SHNorm dest_sh_norm, st::SHPhase dest_sh_phase,
          real_zernike_expansion ExpansionType>
RealZernikeSpan<std::array<double, 2>, dest_zernike_norm, dest_sh_norm, dest_sh_phase> to_real_expansion(
    ExpansionType&& expansion) {
    using E = std::remove_cvref_t<ExpansionType>;
    st::detail::convert(ZEST_EXPANSION_ZERNIKE, expansion.order(), expansion.data(), detail::abi(E::zernike_norm),
                        st::detail::abi(E::sh_norm), st::detail::abi(E::sh_phase), detail::abi(dest_zernike_norm),
                        st::detail::abi(dest_sh_norm), st::detail::abi(dest_sh_phase), false);
    return RealZernikeSpan<std::array<double, 2>, dest_zernike_norm, dest_sh_norm, dest_sh_phase>(
        reinterpret_cast<std::array<double, 2>*>(expansion.data()), expansion.order());
}

// The same for the coefficients of one radial index (a ZernikeSHSpan): only
// the SH conventions change, zernike_expansion.hpp:644-775.
template <st::SHNorm dest_sh_norm, st::SHPhase dest_sh_phase, typename ExpansionType>
    requires st::row_skipping_real_sh_expansion<ExpansionType> &&
             std::same_as<typename std::remove_cvref_t<ExpansionType>::value_type, std::array<double, 2>>
auto to_complex_expansion(ExpansionType&& expansion) {
    using E = std::remove_cvref_t<ExpansionType>;
    st::detail::convert(ZEST_EXPANSION_ZERNIKE_ROW, expansion.order(), expansion.data(), detail::abi(E::zernike_norm),
                        st::detail::abi(E::norm), st::detail::abi(E::phase), detail::abi(E::zernike_norm),
                        st::detail::abi(dest_sh_norm), st::detail::abi(dest_sh_phase), true);
    return ZernikeSHSpan<std::complex<double>, typename E::Layout, E::zernike_norm, dest_sh_norm, dest_sh_phase>(
        reinterpret_cast<std::complex<double>*>(expansion.data()), expansion.order());
}
template <st::SHNorm dest_sh_norm, st::SHPhase dest_sh_phase, typename ExpansionType>
    requires st::row_skipping_real_sh_expansion<ExpansionType> &&
             std::same_as<typename std::remove_cvref_t<ExpansionType>::value_type, std::complex<double>>
auto to_real_expansion(ExpansionType&& expansion) {
    using E = std::remove_cvref_t<ExpansionType>;
    st::detail::convert(ZEST_EXPANSION_ZERNIKE_ROW, expansion.order(), expansion.data(), detail::abi(E::zernike_norm),
                        st::detail::abi(E::norm), st::detail::abi(E::phase), detail::abi(E::zernike_norm),
                        st::detail::abi(dest_sh_norm), st::detail::abi(dest_sh_phase), false);
    return ZernikeSHSpan<std::array<double, 2>, typename E::Layout, E::zernike_norm, dest_sh_norm, dest_sh_phase>(
        reinterpret_cast<std::array<double, 2>*>(expansion.data()), expansion.order());
}

// Zernike transforms on the GLQ grid of the ball, zernike_glq_transformer.hpp:510-707.
template <ZernikeNorm zernike_norm_param, st::SHNorm sh_norm_param, st::SHPhase sh_phase_param,
          typename GridLayoutType = DefaultLayout>
class GLQTransformer {
public:
    using GridLayout = GridLayoutType;
    static constexpr ZernikeNorm zernike_norm = zernike_norm_param;
    static constexpr st::SHNorm sh_norm = sh_norm_param;
    static constexpr st::SHPhase phase = sh_phase_param;
    using Expansion = RealZernikeExpansion<zernike_norm_param, sh_norm_param, sh_phase_param>;

    GLQTransformer() : GLQTransformer(0) {}
    explicit GLQTransformer(std::size_t order, int device = 0, void* stream = nullptr)
        : m_ctx(device, stream), m_order(order) {}

    [[nodiscard]] std::size_t order() const noexcept { return m_order; }
    void resize(std::size_t order) { m_order = order; }
    [[nodiscard]] GPUContext& context() noexcept { return m_ctx; }
    // the contractions' arithmetic: FP64 (default) or split precision on the tensor cores
    void set_precision(Precision precision, int slices = 0) { m_ctx.set_precision(precision, slices); }

    void forward_transform(
        BallGLQGridSpan<const double, GridLayout> values,
        RealZernikeSpan<std::array<double, 2>, zernike_norm_param, sh_norm_param, sh_phase_param> expansion) {
        resize(values.order());
        forward_transform_batch(values.data(), values.order(), reinterpret_cast<double*>(expansion.data()),
                                expansion.order(), 1, MemoryKind::host);
    }
    void backward_transform(
        RealZernikeSpan<const std::array<double, 2>, zernike_norm_param, sh_norm_param, sh_phase_param> expansion,
        BallGLQGridSpan<double, GridLayout> values) {
        resize(values.order());
        backward_transform_batch(reinterpret_cast<const double*>(expansion.data()), expansion.order(),
                                 values.data(), values.order(), 1, MemoryKind::host);
    }
    [[nodiscard]] Expansion forward_transform(BallGLQGridSpan<const double, GridLayout> values, std::size_t order) {
        Expansion expansion(order);
        forward_transform(values, expansion);
        return expansion;
    }
    [[nodiscard]] BallGLQGrid<double, GridLayout> backward_transform(
        RealZernikeSpan<const std::array<double, 2>, zernike_norm_param, sh_norm_param, sh_phase_param> expansion,
        std::size_t order) {
        BallGLQGrid<double, GridLayout> grid(order);
        backward_transform(expansion, grid);
        return grid;
    }

    // `batch` contiguous grids of grid_order -> expansions of exp_order.
    void forward_transform_batch(const double* grids, std::size_t grid_order, double* coeffs, std::size_t exp_order,
                                 std::size_t batch, MemoryKind mem) {
        zest::detail::check(zest_gpu_zt_forward(m_ctx.get(), detail::abi(zernike_norm_param),
                                                st::detail::abi(sh_norm_param), st::detail::abi(sh_phase_param),
                                                grid_order, exp_order, batch, grids, coeffs, int(mem)));
    }
    void backward_transform_batch(const double* coeffs, std::size_t exp_order, double* grids, std::size_t grid_order,
                                  std::size_t batch, MemoryKind mem) {
        zest::detail::check(zest_gpu_zt_backward(m_ctx.get(), detail::abi(zernike_norm_param),
                                                 st::detail::abi(sh_norm_param), st::detail::abi(sh_phase_param),
                                                 exp_order, grid_order, batch, coeffs, grids, int(mem)));
    }

    // Vector-Jacobian products (adjoints): the grid cotangent of
    // forward_transform, W B(G^+ c), and the coefficient cotangent of
    // backward_transform, G F(W^-1 g) (W quadrature weights, G Gram diagonal).
    void forward_transform_vjp(
        RealZernikeSpan<const std::array<double, 2>, zernike_norm_param, sh_norm_param, sh_phase_param> expansion_cot,
        BallGLQGridSpan<double, GridLayout> values_cot) {
        forward_transform_vjp_batch(reinterpret_cast<const double*>(expansion_cot.data()), expansion_cot.order(),
                                    values_cot.data(), values_cot.order(), 1, MemoryKind::host);
    }
    void backward_transform_vjp(
        BallGLQGridSpan<const double, GridLayout> values_cot,
        RealZernikeSpan<std::array<double, 2>, zernike_norm_param, sh_norm_param, sh_phase_param> expansion_cot) {
        backward_transform_vjp_batch(values_cot.data(), values_cot.order(),
                                     reinterpret_cast<double*>(expansion_cot.data()), expansion_cot.order(), 1,
                                     MemoryKind::host);
    }
    void forward_transform_vjp_batch(const double* coeffs_cot, std::size_t exp_order, double* grids_cot,
                                     std::size_t grid_order, std::size_t batch, MemoryKind mem) {
        zest::detail::check(zest_gpu_zt_forward_vjp(m_ctx.get(), detail::abi(zernike_norm_param),
                                                    st::detail::abi(sh_norm_param), st::detail::abi(sh_phase_param),
                                                    grid_order, exp_order, batch, coeffs_cot, grids_cot, int(mem)));
    }
    void backward_transform_vjp_batch(const double* grids_cot, std::size_t grid_order, double* coeffs_cot,
                                      std::size_t exp_order, std::size_t batch, MemoryKind mem) {
        zest::detail::check(zest_gpu_zt_backward_vjp(m_ctx.get(), detail::abi(zernike_norm_param),
                                                     st::detail::abi(sh_norm_param), st::detail::abi(sh_phase_param),
                                                     exp_order, grid_order, batch, grids_cot, coeffs_cot, int(mem)));
    }

private:
    GPUContext m_ctx;
    std::size_t m_order;
};

template <typename GridLayout = DefaultLayout>
using GLQTransformerAcoustics = GLQTransformer<ZernikeNorm::unnormed, st::SHNorm::qm, st::SHPhase::none, GridLayout>;
template <typename GridLayout = DefaultLayout>
using GLQTransformerNormalAcoustics
    = GLQTransformer<ZernikeNorm::normed, st::SHNorm::qm, st::SHPhase::none, GridLayout>;
template <typename GridLayout = DefaultLayout>
using GLQTransformerQM = GLQTransformer<ZernikeNorm::unnormed, st::SHNorm::qm, st::SHPhase::cs, GridLayout>;
template <typename GridLayout = DefaultLayout>
using GLQTransformerNormalQM = GLQTransformer<ZernikeNorm::normed, st::SHNorm::qm, st::SHPhase::cs, GridLayout>;
template <typename GridLayout = DefaultLayout>
using GLQTransformerGeo = GLQTransformer<ZernikeNorm::unnormed, st::SHNorm::geo, st::SHPhase::none, GridLayout>;
template <typename GridLayout = DefaultLayout>
using GLQTransformerNormalGeo = GLQTransformer<ZernikeNorm::normed, st::SHNorm::geo, st::SHPhase::none, GridLayout>;

}  // namespace zt

// ---------------------------------------------------------------------------
// Rotations
// ---------------------------------------------------------------------------

// Wigner d^l_{m1 m2}(pi/2) for 0 <= m1, m2 <= l < max_order, generated on the
// device (wignerd_collection.hpp:66-110); block l at l(l+1)(2l+1)/6, row m1.
class WignerdPiHalfCollection {
public:
    WignerdPiHalfCollection() = default;
    explicit WignerdPiHalfCollection(std::size_t max_order, int device = 0) : m_device(device) { expand(max_order); }

    void expand(std::size_t max_order) {
        if (max_order <= m_max_order && !m_matrices.empty()) return;
        GPUContext ctx(m_device);
        m_matrices.assign(max_order * (max_order + 1) * (2 * max_order + 1) / 6, 0.0);
        if (max_order) zest::detail::check(zest_gpu_wignerd_table(ctx.get(), max_order, m_matrices.data(), ZEST_MEM_HOST));
        m_max_order = max_order;
    }
    [[nodiscard]] std::span<const double> matrices() const noexcept { return m_matrices; }
    [[nodiscard]] std::size_t max_order() const noexcept { return m_max_order; }
    [[nodiscard]] double operator()(std::size_t l, std::size_t m1, std::size_t m2) const noexcept {
        return m_matrices[l * (l + 1) * (2 * l + 1) / 6 + (l + 1) * m1 + m2];
    }

private:
    std::vector<double> m_matrices;
    std::size_t m_max_order = 0;
    int m_device = 0;
};

// Euler angles (intrinsic ZYZ) of a rotation matrix, rotor.hpp:53-63.
[[nodiscard]] inline std::array<double, 3> euler_angles_from_rotation_matrix(
    const std::array<std::array<double, 3>, 3>& matrix) {
    double m[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m[3 * i + j] = matrix[i][j];
    std::array<double, 3> euler{};
    zest::detail::check(zest_gpu_euler_from_matrix(m, euler.data()));
    return euler;
}

// Rotations of real Zernike and SH expansions, rotor.hpp:95-395.  The rotor
// owns a device context, which holds its own copy of the Wigner d(pi/2)
// tables (the same values as `wigner_d_pi2`, generated by the same kernel).
class Rotor {
public:
    Rotor() : Rotor(0) {}
    explicit Rotor(std::size_t max_order, int device = 0, void* stream = nullptr)
        : m_ctx(device, stream), m_max_order(max_order) {}

    void expand(std::size_t max_order) { m_max_order = std::max(m_max_order, max_order); }
    [[nodiscard]] std::size_t max_order() const noexcept { return m_max_order; }
    [[nodiscard]] GPUContext& context() noexcept { return m_ctx; }

    template <zt::real_zernike_expansion ExpansionType>
        requires std::same_as<typename std::remove_cvref_t<ExpansionType>::value_type, std::array<double, 2>>
    void rotate(ExpansionType&& expansion, const WignerdPiHalfCollection& wigner_d_pi2,
                const std::array<double, 3>& euler_angles, RotationType type) {
        auto span = as_zt_span(expansion);
        check_wigner(wigner_d_pi2, span.order());
        expand(span.order());
        zest::detail::check(zest_gpu_zt_rotate(m_ctx.get(), span.order(), 1, reinterpret_cast<double*>(span.data()),
                                               euler_angles.data(), abi(type), ZEST_MEM_HOST));
    }
    template <st::real_sh_expansion ExpansionType>
        requires std::same_as<typename std::remove_cvref_t<ExpansionType>::value_type, std::array<double, 2>>
    void rotate(ExpansionType&& expansion, const WignerdPiHalfCollection& wigner_d_pi2,
                const std::array<double, 3>& euler_angles, RotationType type) {
        auto span = as_st_span(expansion);
        check_wigner(wigner_d_pi2, span.order());
        expand(span.order());
        zest::detail::check(zest_gpu_st_rotate(m_ctx.get(), span.order(), 1, reinterpret_cast<double*>(span.data()),
                                               euler_angles.data(), abi(type), ZEST_MEM_HOST));
    }
    // An expansion of one parity of l in the row-skipping layout (the
    // coefficients of one radial index of a Zernike expansion), rotor.hpp:165-193.
    template <st::row_skipping_real_sh_expansion ExpansionType>
        requires std::same_as<typename std::remove_cvref_t<ExpansionType>::value_type, std::array<double, 2>>
    void rotate(ExpansionType&& expansion, const WignerdPiHalfCollection& wigner_d_pi2,
                const std::array<double, 3>& euler_angles, RotationType type) {
        check_wigner(wigner_d_pi2, expansion.order());
        expand(expansion.order());
        zest::detail::check(zest_gpu_rows_rotate(m_ctx.get(), expansion.order(), 1,
                                                 reinterpret_cast<double*>(expansion.data()), euler_angles.data(),
                                                 abi(type), ZEST_MEM_HOST));
    }
    template <typename ExpansionType>
        requires zt::real_zernike_expansion<ExpansionType> || st::real_sh_expansion<ExpansionType>
    void rotate(ExpansionType&& expansion, const WignerdPiHalfCollection& wigner_d_pi2,
                const std::array<std::array<double, 3>, 3>& matrix, RotationType type) {
        rotate(std::forward<ExpansionType>(expansion), wigner_d_pi2, euler_angles_from_rotation_matrix(matrix), type);
    }

    template <zt::real_zernike_expansion ExpansionType>
        requires std::same_as<typename std::remove_cvref_t<ExpansionType>::value_type, std::array<double, 2>>
    void polar_rotate(ExpansionType&& expansion, double angle, RotationType type) {
        auto span = as_zt_span(expansion);
        zest::detail::check(zest_gpu_zt_polar_rotate(m_ctx.get(), span.order(), 1,
                                                     reinterpret_cast<double*>(span.data()), &angle, abi(type),
                                                     ZEST_MEM_HOST));
    }
    template <st::real_sh_expansion ExpansionType>
        requires std::same_as<typename std::remove_cvref_t<ExpansionType>::value_type, std::array<double, 2>>
    void polar_rotate(ExpansionType&& expansion, double angle, RotationType type) {
        auto span = as_st_span(expansion);
        zest::detail::check(zest_gpu_st_polar_rotate(m_ctx.get(), span.order(), 1,
                                                     reinterpret_cast<double*>(span.data()), &angle, abi(type),
                                                     ZEST_MEM_HOST));
    }

    // Vector-Jacobian product of y = rotate(expansion, euler_angles): writes
    // D^T out_cot into expansion_cot (if non-empty) and returns the gradient
    // of <out_cot, y> with respect to the three Euler angles.
    template <typename ExpansionType, typename CotangentType>
        requires(zt::real_zernike_expansion<ExpansionType> || st::real_sh_expansion<ExpansionType>)
    std::array<double, 3> rotate_vjp(const ExpansionType& expansion, const WignerdPiHalfCollection& wigner_d_pi2,
                                     const std::array<double, 3>& euler_angles, RotationType type,
                                     const CotangentType& out_cot, double* expansion_cot = nullptr) {
        std::array<double, 3> grad{};
        const double* x = reinterpret_cast<const double*>(expansion.data());
        const double* y = reinterpret_cast<const double*>(out_cot.data());
        check_wigner(wigner_d_pi2, expansion.order());
        if constexpr (zt::real_zernike_expansion<ExpansionType>)
            zest::detail::check(zest_gpu_zt_rotate_vjp(m_ctx.get(), expansion.order(), 1, x, euler_angles.data(),
                                                       abi(type), y, expansion_cot, grad.data(), ZEST_MEM_HOST));
        else
            zest::detail::check(zest_gpu_st_rotate_vjp(m_ctx.get(), expansion.order(), 1, x, euler_angles.data(),
                                                       abi(type), y, expansion_cot, grad.data(), ZEST_MEM_HOST));
        return grad;
    }

    // `batch` contiguous Zernike expansions of one order, one Euler triple each.
    void rotate_batch(double* coeffs, std::size_t order, std::size_t batch, const double* euler_angles,
                      RotationType type, MemoryKind mem) {
        zest::detail::check(
            zest_gpu_zt_rotate(m_ctx.get(), order, batch, coeffs, euler_angles, abi(type), int(mem)));
    }

private:
    static constexpr int abi(RotationType t) noexcept {
        return t == RotationType::object ? ZEST_ROTATION_OBJECT : ZEST_ROTATION_COORDINATE;
    }
    static void check_wigner(const WignerdPiHalfCollection& w, std::size_t order) {
        if (w.max_order() < order)
            throw GPUError(ZEST_GPU_ERR_INVALID, "WignerdPiHalfCollection is smaller than the expansion order");
    }
    template <typename E>
    static auto as_zt_span(E& e) {
        using T = std::remove_cvref_t<E>;
        return zt::RealZernikeSpan<std::array<double, 2>, T::zernike_norm, T::sh_norm, T::sh_phase>(e);
    }
    template <typename E>
    static auto as_st_span(E& e) {
        using T = std::remove_cvref_t<E>;
        return st::RealSHSpan<std::array<double, 2>, T::norm, T::phase>(e);
    }

    GPUContext m_ctx;
    std::size_t m_max_order;
};

// ---------------------------------------------------------------------------
// Evaluation at arbitrary points and power spectra
// ---------------------------------------------------------------------------

namespace st {

// Evaluation of SH expansions on the product grid of arbitrary longitudes and
// colatitudes, grid_evaluator.hpp:52-133.  Values [lon][lat], row-major.
class GridEvaluator {
public:
    GridEvaluator() : GridEvaluator(0) {}
    explicit GridEvaluator(std::size_t max_order, int device = 0, void* stream = nullptr)
        : m_ctx(device, stream), m_max_order(max_order) {}
    GridEvaluator(std::size_t max_order, std::size_t lon_size, std::size_t lat_size) : GridEvaluator(max_order) {
        resize(max_order, lon_size, lat_size);
    }
    void resize(std::size_t max_order, std::size_t lon_size, std::size_t lat_size) {
        m_max_order = max_order;
        m_lon_size = lon_size;
        m_lat_size = lat_size;
    }
    [[nodiscard]] GPUContext& context() noexcept { return m_ctx; }

    template <real_sh_expansion ExpansionType>
    [[nodiscard]] std::vector<double> evaluate(ExpansionType&& expansion, std::span<const double> longitudes,
                                               std::span<const double> colatitudes) {
        using E = std::remove_cvref_t<ExpansionType>;
        if (longitudes.empty() || colatitudes.empty()) return {};
        resize(expansion.order(), longitudes.size(), colatitudes.size());
        std::vector<double> res(longitudes.size() * colatitudes.size());
        evaluate_batch<E::norm, E::phase>(reinterpret_cast<const double*>(expansion.data()), expansion.order(), 1,
                                          longitudes.data(), longitudes.size(), colatitudes.data(),
                                          colatitudes.size(), res.data(), MemoryKind::host);
        return res;
    }
    // `batch` contiguous expansions; coefficients, points and values all host or all device memory
    template <SHNorm sh_norm, SHPhase sh_phase>
    void evaluate_batch(const double* coeffs, std::size_t order, std::size_t batch, const double* lon,
                        std::size_t nlon, const double* colat, std::size_t nlat, double* values, MemoryKind mem) {
        zest::detail::check(zest_gpu_st_evaluate(m_ctx.get(), detail::abi(sh_norm), detail::abi(sh_phase), order,
                                                 batch, coeffs, nlon, lon, nlat, colat, values, int(mem)));
    }

private:
    GPUContext m_ctx;
    std::size_t m_max_order = 0, m_lon_size = 0, m_lat_size = 0;
};

// power_spectra.hpp:38-104.  (The reference's own SH spectra name the
// convention ExpansionType::sh_norm, which its SH spans do not define; here
// they read the span's `norm`, which is what they mean.)
template <real_sh_expansion ExpansionType>
void cross_power_spectrum(ExpansionType&& a, ExpansionType&& b, std::span<double> out) {
    using E = std::remove_cvref_t<ExpansionType>;
    if (a.order() != b.order())
        throw GPUError(ZEST_GPU_ERR_INVALID, "cross_power_spectrum: expansions of different orders");
    zest::detail::check(zest_gpu_st_cross_power_spectrum(
        zest::detail::thread_context().get(), detail::abi(E::norm), a.order(), 1,
        reinterpret_cast<const double*>(a.data()), reinterpret_cast<const double*>(b.data()), out.size(), out.data(),
        ZEST_MEM_HOST));
}
template <real_sh_expansion ExpansionType>
[[nodiscard]] std::vector<double> cross_power_spectrum(ExpansionType&& a, ExpansionType&& b) {
    std::vector<double> out(std::min(a.order(), b.order()));
    cross_power_spectrum(std::forward<ExpansionType>(a), std::forward<ExpansionType>(b), out);
    return out;
}
template <real_sh_expansion ExpansionType>
void power_spectrum(ExpansionType&& expansion, std::span<double> out) {
    using E = std::remove_cvref_t<ExpansionType>;
    if (out.size() < expansion.order()) throw GPUError(ZEST_GPU_ERR_INVALID, "power_spectrum: output too small");
    zest::detail::check(zest_gpu_st_power_spectrum(zest::detail::thread_context().get(), detail::abi(E::norm),
                                                   expansion.order(), 1,
                                                   reinterpret_cast<const double*>(expansion.data()), out.data(),
                                                   ZEST_MEM_HOST));
}
template <real_sh_expansion ExpansionType>
[[nodiscard]] std::vector<double> power_spectrum(ExpansionType&& expansion) {
    std::vector<double> out(expansion.order());
    power_spectrum(std::forward<ExpansionType>(expansion), out);
    return out;
}

}  // namespace st

namespace zt {

// Values R_nl of one radial index (n, l), n - l even, at floor((n+1)^2/4) + l/2
// (RadialZernikeSpan over RadialZernikeLayout, zernike_expansion.hpp:43-75,
// layout.hpp:254-289).
template <typename ElementType, ZernikeNorm zernike_norm_param>
class RadialZernikeSpan {
public:
    using element_type = ElementType;
    static constexpr ZernikeNorm zernike_norm = zernike_norm_param;
    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept { return ((order + 1) * (order + 1)) >> 2; }
    [[nodiscard]] static constexpr std::size_t idx(std::size_t n, std::size_t l) noexcept {
        return (((n + 1) * (n + 1)) >> 2) + (l >> 1);
    }
    RadialZernikeSpan() noexcept = default;
    constexpr RadialZernikeSpan(element_type* data, std::size_t order) noexcept : m_data(data), m_order(order) {}
    constexpr RadialZernikeSpan(std::span<element_type> buffer, std::size_t order) noexcept
        : m_data(buffer.data()), m_order(order) {}
    [[nodiscard]] constexpr std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] constexpr std::size_t size() const noexcept { return size(m_order); }
    [[nodiscard]] constexpr element_type* data() const noexcept { return m_data; }
    [[nodiscard]] constexpr element_type& operator()(std::size_t n, std::size_t l) const noexcept {
        return m_data[idx(n, l)];
    }

private:
    element_type* m_data = nullptr;
    std::size_t m_order = 0;
};

// Evaluation of Zernike expansions on the product grid of arbitrary
// longitudes, colatitudes and radii, grid_evaluator.hpp:147-325.
// Values [lon][lat][rad], row-major.
class GridEvaluator {
public:
    GridEvaluator() : GridEvaluator(0) {}
    explicit GridEvaluator(std::size_t max_order, int device = 0, void* stream = nullptr)
        : m_ctx(device, stream), m_max_order(max_order) {}
    GridEvaluator(std::size_t max_order, std::size_t lon_size, std::size_t lat_size, std::size_t rad_size)
        : GridEvaluator(max_order) {
        resize(max_order, lon_size, lat_size, rad_size);
    }
    void resize(std::size_t max_order, std::size_t lon_size, std::size_t lat_size, std::size_t rad_size) {
        m_max_order = max_order;
        m_lon_size = lon_size;
        m_lat_size = lat_size;
        m_rad_size = rad_size;
    }
    [[nodiscard]] GPUContext& context() noexcept { return m_ctx; }

    template <real_zernike_expansion ExpansionType>
    [[nodiscard]] std::vector<double> evaluate(ExpansionType&& expansion, std::span<const double> longitudes,
                                               std::span<const double> colatitudes, std::span<const double> radii) {
        using E = std::remove_cvref_t<ExpansionType>;
        if (longitudes.empty() || colatitudes.empty() || radii.empty()) return {};
        resize(expansion.order(), longitudes.size(), colatitudes.size(), radii.size());
        std::vector<double> res(longitudes.size() * colatitudes.size() * radii.size());
        evaluate_batch<E::zernike_norm, E::sh_norm, E::sh_phase>(
            reinterpret_cast<const double*>(expansion.data()), expansion.order(), 1, longitudes.data(),
            longitudes.size(), colatitudes.data(), colatitudes.size(), radii.data(), radii.size(), res.data(),
            MemoryKind::host);
        return res;
    }
    template <ZernikeNorm zernike_norm, st::SHNorm sh_norm, st::SHPhase sh_phase>
    void evaluate_batch(const double* coeffs, std::size_t order, std::size_t batch, const double* lon,
                        std::size_t nlon, const double* colat, std::size_t nlat, const double* rad, std::size_t nrad,
                        double* values, MemoryKind mem) {
        zest::detail::check(zest_gpu_zt_evaluate(m_ctx.get(), detail::abi(zernike_norm), st::detail::abi(sh_norm),
                                                 st::detail::abi(sh_phase), order, batch, coeffs, nlon, lon, nlat,
                                                 colat, nrad, rad, values, int(mem)));
    }

private:
    GPUContext m_ctx;
    std::size_t m_max_order = 0, m_lon_size = 0, m_lat_size = 0, m_rad_size = 0;
};

// power_spectra.hpp:124-163: out(n, l) = norm sum_m |c_nlm|^2 for l = n&1, .. < n
// (the reference's bound: the l = n entries are not written).
template <real_zernike_expansion ExpansionType>
void power_spectrum(ExpansionType&& expansion,
                    RadialZernikeSpan<double, std::remove_cvref_t<ExpansionType>::zernike_norm> out) {
    using E = std::remove_cvref_t<ExpansionType>;
    const std::size_t order = std::min(out.order(), expansion.order());
    if (order == 0) return;
    if (order == expansion.order()) {
        zest::detail::check(zest_gpu_zt_power_spectrum(zest::detail::thread_context().get(),
                                                       st::detail::abi(E::sh_norm), order, 1,
                                                       reinterpret_cast<const double*>(expansion.data()),
                                                       out.data(), ZEST_MEM_HOST));
        return;
    }
    // a smaller output: the leading orders of the expansion, copied contiguously
    using Span = RealZernikeSpan<const std::array<double, 2>, E::zernike_norm, E::sh_norm, E::sh_phase>;
    const Span full(reinterpret_cast<const std::array<double, 2>*>(expansion.data()), expansion.order());
    std::vector<std::array<double, 2>> head(Span::size(order));
    for (std::size_t n = 0; n < order; ++n)
        for (std::size_t l = n & 1; l <= n; l += 2)
            for (std::size_t m = 0; m <= l; ++m) head[Span::idx(n, l, m)] = full(n, l, m);
    zest::detail::check(zest_gpu_zt_power_spectrum(zest::detail::thread_context().get(), st::detail::abi(E::sh_norm),
                                                   order, 1, reinterpret_cast<const double*>(head.data()),
                                                   out.data(), ZEST_MEM_HOST));
}
template <real_zernike_expansion ExpansionType>
[[nodiscard]] std::vector<double> power_spectrum(ExpansionType&& expansion) {
    using E = std::remove_cvref_t<ExpansionType>;
    std::vector<double> res(RadialZernikeSpan<double, E::zernike_norm>::size(expansion.order()));
    power_spectrum(std::forward<ExpansionType>(expansion),
                   RadialZernikeSpan<double, E::zernike_norm>(res, expansion.order()));
    return res;
}

}  // namespace zt

// ---------------------------------------------------------------------------
// Sampling front-ends: the quadrature points, generate_values, and the
// transformers of functions (zernike_glq_transformer.hpp:336-501, 1027-1178;
// sh_glq_transformer.hpp:385-504, 1242-1351).  Functions are host callables
// here, sampled on the host as in the reference; zest_gpu_sampling.cuh samples
// device functors on the GPU instead.
// ---------------------------------------------------------------------------

namespace st {

template <typename Func>
concept spherical_function = requires(Func f, double lon, double colat) {
    { f(lon, colat) } -> std::same_as<double>;
};
template <typename Func>
concept cartesian_function = requires(Func f, std::array<double, 3> x) {
    { f(x) } -> std::same_as<double>;
};

// Longitudes and GL colatitudes of the grid of a layout (counts from the
// layout's shape, padding included, as the reference).
template <typename LayoutType = DefaultLayout>
class SphereGLQGridPoints {
public:
    using GridLayout = LayoutType;
    SphereGLQGridPoints() = default;
    explicit SphereGLQGridPoints(std::size_t order) { resize(order); }
    void resize(std::size_t order) {
        if (order == m_order && !m_longitudes.empty()) return;
        const auto shape = GridLayout::shape(order);
        m_longitudes.assign(shape[GridLayout::lon_axis], 0.0);
        m_glq_nodes.assign(shape[GridLayout::lat_axis], 0.0);
        zest::detail::check(zest_gpu_st_grid_points(order, GridLayout::abi, m_longitudes.data(), m_glq_nodes.data()));
        m_order = order;
    }
    [[nodiscard]] std::array<std::size_t, 2> shape() const noexcept { return {m_glq_nodes.size(), m_longitudes.size()}; }
    [[nodiscard]] std::span<const double> longitudes() const noexcept { return m_longitudes; }
    [[nodiscard]] std::span<const double> glq_nodes() const noexcept { return m_glq_nodes; }

    template <typename GridType, typename FuncType>
        requires std::same_as<typename std::remove_cvref_t<GridType>::Layout, GridLayout>
    void generate_values(GridType&& grid, FuncType&& f) {
        resize(grid.order());
        for (std::size_t i = 0; i < m_longitudes.size(); ++i)
            for (std::size_t j = 0; j < m_glq_nodes.size(); ++j) {
                const double v = f(m_longitudes[i], m_glq_nodes[j]);
                if constexpr (GridLayout::lon_axis == 0) grid(i, j) = v;
                else grid(j, i) = v;
            }
    }
    template <typename FuncType>
    [[nodiscard]] auto generate_values(FuncType&& f, std::size_t order) {
        SphereGLQGrid<double, GridLayout> grid(order);
        generate_values(grid, f);
        return grid;
    }

private:
    std::vector<double> m_longitudes, m_glq_nodes;
    std::size_t m_order = 0;
};

// SH expansions of functions on the sphere (sh_glq_transformer.hpp:1257-1351).
template <SHNorm sh_norm_param, SHPhase sh_phase_param, typename GridLayoutType = DefaultLayout>
class SHTransformer {
public:
    using GridLayout = GridLayoutType;
    SHTransformer() = default;
    explicit SHTransformer(std::size_t order) : m_grid(order), m_points(order), m_transformer(order) {}
    void resize(std::size_t order) {
        m_points.resize(order);
        if (m_grid.order() != order) m_grid = SphereGLQGrid<double, GridLayout>(order);
        m_transformer.resize(order);
    }
    [[nodiscard]] GLQTransformer<sh_norm_param, sh_phase_param, GridLayout>& transformer() noexcept {
        return m_transformer;
    }

    template <spherical_function FuncType>
    void transform(FuncType&& f, RealSHSpan<std::array<double, 2>, sh_norm_param, sh_phase_param> expansion) {
        resize(expansion.order());
        m_points.generate_values(m_grid, f);
        m_transformer.forward_transform(m_grid, expansion);
    }
    template <spherical_function FuncType>
    [[nodiscard]] RealSHExpansion<sh_norm_param, sh_phase_param> transform(FuncType&& f, std::size_t order) {
        RealSHExpansion<sh_norm_param, sh_phase_param> expansion(order);
        transform(std::forward<FuncType>(f), expansion);
        return expansion;
    }
    template <cartesian_function FuncType>
    void transform(FuncType&& f, RealSHSpan<std::array<double, 2>, sh_norm_param, sh_phase_param> expansion) {
        transform(spherical(f), expansion);
    }
    template <cartesian_function FuncType>
    [[nodiscard]] RealSHExpansion<sh_norm_param, sh_phase_param> transform(FuncType&& f, std::size_t order) {
        return transform(spherical(f), order);
    }

private:
    template <typename F>
    static auto spherical(F& f) {
        return [&f](double lon, double colat) -> double {
            const double scolat = std::sin(colat);
            const std::array<double, 3> x = {scolat * std::cos(lon), scolat * std::sin(lon), std::cos(colat)};
            return f(x);
        };
    }
    SphereGLQGrid<double, GridLayout> m_grid;
    SphereGLQGridPoints<GridLayout> m_points;
    GLQTransformer<sh_norm_param, sh_phase_param, GridLayout> m_transformer;
};

}  // namespace st

namespace zt {

template <typename Func>
concept spherical_function = requires(Func f, double lon, double colat, double r) {
    { f(lon, colat, r) } -> std::same_as<double>;
};
template <typename Func>
concept cartesian_function = requires(Func f, std::array<double, 3> x) {
    { f(x) } -> std::same_as<double>;
};

// Longitudes, GL colatitudes and GL radii of the ball grid.
template <typename LayoutType = DefaultLayout>
class BallGLQGridPoints {
public:
    using GridLayout = LayoutType;
    BallGLQGridPoints() = default;
    explicit BallGLQGridPoints(std::size_t order) { resize(order); }
    void resize(std::size_t order) {
        if (order == m_order && !m_longitudes.empty()) return;
        const auto shape = GridLayout::shape(order);
        m_longitudes.assign(shape[0], 0.0);
        m_lat_glq_nodes.assign(shape[1], 0.0);
        m_rad_glq_nodes.assign(shape[2], 0.0);
        zest::detail::check(
            zest_gpu_zt_grid_points(order, m_longitudes.data(), m_lat_glq_nodes.data(), m_rad_glq_nodes.data()));
        m_order = order;
    }
    [[nodiscard]] std::span<const double> longitudes() const noexcept { return m_longitudes; }
    [[nodiscard]] std::span<const double> lat_glq_nodes() const noexcept { return m_lat_glq_nodes; }
    [[nodiscard]] std::span<const double> rad_glq_nodes() const noexcept { return m_rad_glq_nodes; }

    template <typename GridType, typename FuncType>
        requires std::same_as<typename std::remove_cvref_t<GridType>::Layout, GridLayout>
    void generate_values(GridType&& grid, FuncType&& f) {
        resize(grid.order());
        for (std::size_t i = 0; i < m_longitudes.size(); ++i)
            for (std::size_t j = 0; j < m_lat_glq_nodes.size(); ++j)
                for (std::size_t k = 0; k < m_rad_glq_nodes.size(); ++k)
                    grid(i, j, k) = f(m_longitudes[i], m_lat_glq_nodes[j], m_rad_glq_nodes[k]);
    }
    template <typename FuncType>
    [[nodiscard]] auto generate_values(FuncType&& f, std::size_t order) {
        BallGLQGrid<double, GridLayout> grid(order);
        generate_values(grid, f);
        return grid;
    }

private:
    std::vector<double> m_longitudes, m_lat_glq_nodes, m_rad_glq_nodes;
    std::size_t m_order = 0;
};

// Zernike expansions of functions on balls of any radius
// (zernike_glq_transformer.hpp:1054-1178).
template <ZernikeNorm zernike_norm_param, st::SHNorm sh_norm_param, st::SHPhase sh_phase_param,
          typename GridLayoutType = DefaultLayout>
class ZernikeTransformer {
public:
    using GridLayout = GridLayoutType;
    using Expansion = RealZernikeExpansion<zernike_norm_param, sh_norm_param, sh_phase_param>;
    ZernikeTransformer() = default;
    explicit ZernikeTransformer(std::size_t order) : m_grid(order), m_points(order), m_transformer(order) {}
    void resize(std::size_t order) {
        m_points.resize(order);
        if (m_grid.order() != order) m_grid = BallGLQGrid<double, GridLayout>(order);
        m_transformer.resize(order);
    }
    [[nodiscard]] GLQTransformer<zernike_norm_param, sh_norm_param, sh_phase_param, GridLayout>& transformer() noexcept {
        return m_transformer;
    }

    template <spherical_function FuncType>
    void transform(FuncType&& f, double radius,
                   RealZernikeSpan<std::array<double, 2>, zernike_norm_param, sh_norm_param, sh_phase_param> expansion) {
        auto f_scaled = [&](double lon, double colat, double r) { return f(lon, colat, r * radius); };
        resize(expansion.order());
        m_points.generate_values(m_grid, f_scaled);
        m_transformer.forward_transform(m_grid, expansion);
    }
    template <spherical_function FuncType>
    [[nodiscard]] Expansion transform(FuncType&& f, double radius, std::size_t order) {
        Expansion expansion(order);
        transform(std::forward<FuncType>(f), radius, expansion);
        return expansion;
    }
    template <cartesian_function FuncType>
    void transform(FuncType&& f, double radius,
                   RealZernikeSpan<std::array<double, 2>, zernike_norm_param, sh_norm_param, sh_phase_param> expansion) {
        auto f_spherical = [&](double lon, double colat, double r) -> double {
            const double rad = r * radius;
            const double scolat = std::sin(colat);
            const std::array<double, 3> x = {rad * scolat * std::cos(lon), rad * scolat * std::sin(lon),
                                             rad * std::cos(colat)};
            return f(x);
        };
        resize(expansion.order());
        m_points.generate_values(m_grid, f_spherical);
        m_transformer.forward_transform(m_grid, expansion);
    }
    template <cartesian_function FuncType>
    [[nodiscard]] Expansion transform(FuncType&& f, double radius, std::size_t order) {
        Expansion expansion(order);
        transform(std::forward<FuncType>(f), radius, expansion);
        return expansion;
    }

private:
    BallGLQGrid<double, GridLayout> m_grid;
    BallGLQGridPoints<GridLayout> m_points;
    GLQTransformer<zernike_norm_param, sh_norm_param, sh_phase_param, GridLayout> m_transformer;
};

}  // namespace zt
// ---------------------------------------------------------------------------
// Least-squares fits to scattered data (lsq_transformer.hpp:38-190)
// ---------------------------------------------------------------------------

namespace st {

class LSQTransformer {
public:
    LSQTransformer() : LSQTransformer(0) {}
    explicit LSQTransformer(std::size_t order, int device = 0, void* stream = nullptr)
        : m_ctx(device, stream), m_order(order) {}
    [[nodiscard]] std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] GPUContext& context() noexcept { return m_ctx; }

    // data at (latitude, longitude) points
    template <SHNorm sh_norm_param, SHPhase sh_phase_param>
    void transform(std::span<const double> data, std::span<const double> lat, std::span<const double> lon,
                   RealSHSpan<std::array<double, 2>, sh_norm_param, sh_phase_param> expansion) {
        if (lat.size() != data.size() || lon.size() != data.size())
            throw GPUError(ZEST_GPU_ERR_INVALID, "LSQTransformer: data and points differ in length");
        m_order = expansion.order();
        zest::detail::check(zest_gpu_st_lsq(m_ctx.get(), detail::abi(sh_norm_param), detail::abi(sh_phase_param),
                                            expansion.order(), data.size(), 1, data.data(), lat.data(), lon.data(),
                                            reinterpret_cast<double*>(expansion.data()), ZEST_MEM_HOST));
    }
    template <SHNorm sh_norm_param, SHPhase sh_phase_param>
    [[nodiscard]] auto transform(std::span<const double> data, std::span<const double> lat,
                                 std::span<const double> lon, std::size_t order) {
        RealSHExpansion<sh_norm_param, sh_phase_param> expansion(order);
        transform<sh_norm_param, sh_phase_param>(data, lat, lon, expansion);
        return expansion;
    }

private:
    GPUContext m_ctx;
    std::size_t m_order;
};

}  // namespace st

namespace zt {

class LSQTransformer {
public:
    LSQTransformer() : LSQTransformer(0) {}
    explicit LSQTransformer(std::size_t order, int device = 0, void* stream = nullptr)
        : m_ctx(device, stream), m_order(order) {}
    [[nodiscard]] std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] GPUContext& context() noexcept { return m_ctx; }

    // data at (r, longitude, colatitude) points
    template <ZernikeNorm zernike_norm_param, st::SHNorm sh_norm_param, st::SHPhase sh_phase_param>
    void transform(std::span<const double> data, std::span<const double> r, std::span<const double> lon,
                   std::span<const double> colat,
                   RealZernikeSpan<std::array<double, 2>, zernike_norm_param, sh_norm_param, sh_phase_param> expansion) {
        if (r.size() != data.size() || lon.size() != data.size() || colat.size() != data.size())
            throw GPUError(ZEST_GPU_ERR_INVALID, "LSQTransformer: data and points differ in length");
        m_order = expansion.order();
        zest::detail::check(zest_gpu_zt_lsq(m_ctx.get(), detail::abi(zernike_norm_param),
                                            st::detail::abi(sh_norm_param), st::detail::abi(sh_phase_param),
                                            expansion.order(), data.size(), 1, data.data(), r.data(), lon.data(),
                                            colat.data(), reinterpret_cast<double*>(expansion.data()),
                                            ZEST_MEM_HOST));
    }
    template <ZernikeNorm zernike_norm_param, st::SHNorm sh_norm_param, st::SHPhase sh_phase_param>
    [[nodiscard]] auto transform(std::span<const double> data, std::span<const double> r,
                                 std::span<const double> lon, std::span<const double> colat, std::size_t order) {
        RealZernikeExpansion<zernike_norm_param, sh_norm_param, sh_phase_param> expansion(order);
        transform<zernike_norm_param, sh_norm_param, sh_phase_param>(data, r, lon, colat, expansion);
        return expansion;
    }

private:
    GPUContext m_ctx;
    std::size_t m_order;
};

}  // namespace zt


// ---------------------------------------------------------------------------
// Tables: Gauss-Legendre nodes and weights, the P_lm and R_nl recursions
// ---------------------------------------------------------------------------
namespace gl {

// Nodes of both halves (UnpackedLayout) or of the non-negative half only
// (PackedLayout), gauss_legendre.hpp:43-86.
struct PackedLayout {
    [[nodiscard]] static constexpr std::size_t size(std::size_t num_total_nodes) noexcept {
        return (num_total_nodes + 1) >> 1;
    }
    [[nodiscard]] static constexpr std::size_t total_nodes(std::size_t size, std::size_t parity) noexcept {
        return 2 * size - parity;
    }
};
struct UnpackedLayout {
    [[nodiscard]] static constexpr std::size_t size(std::size_t num_total_nodes) noexcept { return num_total_nodes; }
    [[nodiscard]] static constexpr std::size_t total_nodes(std::size_t size, std::size_t) noexcept { return size; }
};

// Nodes as cosines x in [-1, 1] (ascending) or as angles arccos(x).
enum class GLNodeStyle { angle, cos };

// Gauss-Legendre nodes and weights, gauss_legendre.hpp:1549-1565: as many as
// `nodes` holds, of a rule of Layout::total_nodes(nodes.size(), parity) nodes.
// The nodes come from a double-double Newton solve (within 2 ulp of the
// reference's tables and Bogaert formulas); angle-style nodes are the
// colatitudes of the quadrature grids.
template <typename Layout, GLNodeStyle node_style_param, typename R>
void gl_nodes_and_weights(R&& nodes, R&& weights, std::size_t parity) {
    const std::size_t size = std::size(nodes);
    if (size == 0) return;
    const std::size_t n = Layout::total_nodes(size, parity);
    constexpr bool packed = std::same_as<Layout, PackedLayout>;
    zest::detail::check(zest_gpu_gl_nodes_weights(n, packed, std::data(nodes), std::data(weights)));
    if constexpr (node_style_param == GLNodeStyle::angle) {
        // the LatLon SH grid of order n has the n angle-style nodes as its colatitudes
        std::vector<double> lon(zest_gpu_st_grid_size(n, ZEST_LAYOUT_LATLON) / n), colat(n);
        zest::detail::check(zest_gpu_st_grid_points(n, ZEST_LAYOUT_LATLON, lon.data(), colat.data()));
        std::copy(colat.end() - std::ptrdiff_t(size), colat.end(), std::data(nodes));
    }
}

}  // namespace gl

namespace st {

using PlmLayout = TriangleLayout<IndexingMode::nonnegative>;

// P_lm of one point at PlmLayout::idx(l, m), plm_recursion.hpp:46-48.
template <typename ElementType, SHNorm sh_norm_param, SHPhase sh_phase_param>
class PlmSpan {
public:
    using Layout = PlmLayout;
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    static constexpr SHNorm norm = sh_norm_param;
    static constexpr SHPhase phase = sh_phase_param;
    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept { return Layout::size(order); }
    constexpr PlmSpan() noexcept = default;
    constexpr PlmSpan(element_type* data, std::size_t order) noexcept : m_data(data), m_order(order) {}
    constexpr PlmSpan(std::span<element_type> buffer, std::size_t order) noexcept
        : m_data(buffer.data()), m_order(order) {}
    [[nodiscard]] constexpr std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] constexpr std::size_t size() const noexcept { return size(m_order); }
    [[nodiscard]] constexpr element_type* data() const noexcept { return m_data; }
    [[nodiscard]] constexpr std::span<element_type> flatten() const noexcept { return {m_data, size()}; }
    [[nodiscard]] constexpr element_type& operator()(std::size_t l, std::size_t m) const noexcept {
        return m_data[Layout::idx(l, m)];
    }

private:
    element_type* m_data = nullptr;
    std::size_t m_order = 0;
};

// P_lm of vec_size points: the values of (l, m) contiguous at
// PlmLayout::idx(l, m) * vec_size, plm_recursion.hpp:53-55.
template <typename ElementType, SHNorm sh_norm_param, SHPhase sh_phase_param>
class PlmVecSpan {
public:
    using Layout = PlmLayout;
    using element_type = ElementType;
    using value_type = std::remove_cv_t<ElementType>;
    static constexpr SHNorm norm = sh_norm_param;
    static constexpr SHPhase phase = sh_phase_param;
    [[nodiscard]] static constexpr std::size_t size(std::size_t order, std::size_t vec_size) noexcept {
        return Layout::size(order) * vec_size;
    }
    constexpr PlmVecSpan() noexcept = default;
    constexpr PlmVecSpan(element_type* data, std::size_t order, std::size_t vec_size) noexcept
        : m_data(data), m_order(order), m_vec_size(vec_size) {}
    constexpr PlmVecSpan(std::span<element_type> buffer, std::size_t order, std::size_t vec_size) noexcept
        : m_data(buffer.data()), m_order(order), m_vec_size(vec_size) {}
    [[nodiscard]] constexpr std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] constexpr std::size_t vec_size() const noexcept { return m_vec_size; }
    [[nodiscard]] constexpr std::size_t size() const noexcept { return size(m_order, m_vec_size); }
    [[nodiscard]] constexpr element_type* data() const noexcept { return m_data; }
    [[nodiscard]] constexpr std::span<element_type> flatten() const noexcept { return {m_data, size()}; }
    [[nodiscard]] constexpr std::span<element_type> operator()(std::size_t l, std::size_t m) const noexcept {
        return {m_data + Layout::idx(l, m) * m_vec_size, m_vec_size};
    }

private:
    element_type* m_data = nullptr;
    std::size_t m_order = 0;
    std::size_t m_vec_size = 0;
};

// The associated Legendre recursion, plm_recursion.hpp:62-362, evaluated on
// the device in FP64 with the reference's operations in its order (the
// tables are bit-identical to the reference's).
class PlmRecursion {
public:
    PlmRecursion() = default;
    explicit PlmRecursion(std::size_t max_order) : m_max_order(max_order) {}
    [[nodiscard]] std::size_t max_order() const noexcept { return m_max_order; }
    void expand(std::size_t max_order) { m_max_order = std::max(m_max_order, max_order); }
    void expand_vec(std::size_t) {}

    template <SHNorm sh_norm_param, SHPhase sh_phase_param>
    void plm_real(double z, PlmSpan<double, sh_norm_param, sh_phase_param> plm) {
        run(false, sh_norm_param, sh_phase_param, plm.order(), 1, &z, plm.data());
    }
    template <SHNorm sh_norm_param, SHPhase sh_phase_param>
    void plm_real(std::span<const double> z, PlmVecSpan<double, sh_norm_param, sh_phase_param> plm) {
        run(false, sh_norm_param, sh_phase_param, plm.order(), z.size(), z.data(), plm.data());
    }
    template <SHNorm sh_norm_param, SHPhase sh_phase_param>
    void plm_complex(double z, PlmSpan<double, sh_norm_param, sh_phase_param> plm) {
        run(true, sh_norm_param, sh_phase_param, plm.order(), 1, &z, plm.data());
    }
    template <SHNorm sh_norm_param, SHPhase sh_phase_param>
    void plm_complex(std::span<const double> z, PlmVecSpan<double, sh_norm_param, sh_phase_param> plm) {
        run(true, sh_norm_param, sh_phase_param, plm.order(), z.size(), z.data(), plm.data());
    }

private:
    void run(bool complex_basis, SHNorm norm, SHPhase phase, std::size_t order, std::size_t nz, const double* z,
             double* out) {
        expand(order);
        auto* ctx = zest::detail::thread_context().get();
        zest::detail::check(complex_basis
                                ? zest_gpu_plm_complex_table(ctx, order, detail::abi(norm), detail::abi(phase), nz,
                                                             z, out, ZEST_MEM_HOST)
                                : zest_gpu_plm_table(ctx, order, detail::abi(norm), detail::abi(phase), nz, z, out,
                                                     ZEST_MEM_HOST));
    }
    std::size_t m_max_order = 0;
};

}  // namespace st

namespace zt {

// R_nl at index floor((n+1)^2/4) + floor(l/2), zernike_expansion.hpp:43-75.
struct RadialZernikeLayout {
    using index_type = std::size_t;
    using size_type = std::size_t;
    [[nodiscard]] static constexpr std::size_t size(std::size_t order) noexcept {
        return ((order + 1) * (order + 1)) >> 2;
    }
    [[nodiscard]] static constexpr std::size_t idx(std::size_t n, std::size_t l) noexcept {
        return (((n + 1) * (n + 1)) >> 2) + (l >> 1);
    }
};

// R_nl of vec_size radii: the values of (n, l) contiguous.
template <typename ElementType, ZernikeNorm zernike_norm_param>
class RadialZernikeVecSpan {
public:
    using Layout = RadialZernikeLayout;
    using element_type = ElementType;
    static constexpr ZernikeNorm zernike_norm = zernike_norm_param;
    constexpr RadialZernikeVecSpan() noexcept = default;
    constexpr RadialZernikeVecSpan(element_type* data, std::size_t order, std::size_t vec_size) noexcept
        : m_data(data), m_order(order), m_vec_size(vec_size) {}
    constexpr RadialZernikeVecSpan(std::span<element_type> buffer, std::size_t order, std::size_t vec_size) noexcept
        : m_data(buffer.data()), m_order(order), m_vec_size(vec_size) {}
    [[nodiscard]] constexpr std::size_t order() const noexcept { return m_order; }
    [[nodiscard]] constexpr std::size_t vec_size() const noexcept { return m_vec_size; }
    [[nodiscard]] constexpr std::size_t size() const noexcept { return Layout::size(m_order) * m_vec_size; }
    [[nodiscard]] constexpr element_type* data() const noexcept { return m_data; }
    [[nodiscard]] constexpr std::span<element_type> flatten() const noexcept { return {m_data, size()}; }
    [[nodiscard]] constexpr std::span<element_type> operator()(std::size_t n, std::size_t l) const noexcept {
        return {m_data + Layout::idx(n, l) * m_vec_size, m_vec_size};
    }

private:
    element_type* m_data = nullptr;
    std::size_t m_order = 0;
    std::size_t m_vec_size = 0;
};

// The radial Zernike recursion, radial_zernike_recursion.hpp:38-297, on the
// device in FP64 (bit-identical to the reference's values).
class RadialZernikeRecursion {
public:
    RadialZernikeRecursion() = default;
    explicit RadialZernikeRecursion(std::size_t max_order) : m_max_order(max_order) {}
    [[nodiscard]] std::size_t max_order() const noexcept { return m_max_order; }
    void expand(std::size_t max_order) { m_max_order = std::max(m_max_order, max_order); }

    template <ZernikeNorm zernike_norm_param>
    void zernike(double r, RadialZernikeSpan<double, zernike_norm_param> out) {
        run(zernike_norm_param, out.order(), 1, &r, out.data());
    }
    template <ZernikeNorm zernike_norm_param>
    void zernike(std::span<const double> r, RadialZernikeVecSpan<double, zernike_norm_param> out) {
        run(zernike_norm_param, out.order(), r.size(), r.data(), out.data());
    }

private:
    void run(ZernikeNorm norm, std::size_t order, std::size_t nr, const double* r, double* out) {
        expand(order);
        zest::detail::check(zest_gpu_radial_table(zest::detail::thread_context().get(), order, detail::abi(norm), nr,
                                                  r, out, ZEST_MEM_HOST));
    }
    std::size_t m_max_order = 0;
};

}  // namespace zt

}  // namespace zest
