/*
 * zest_gpu.h -- C-ABI of the GB300-native Gauss-Legendre-quadrature transform
 * and rotation path of zest (sebsassi/zest).
 *
 * The reference exposes this path only as a C++20 template API; the C++
 * headers under include/zest/ keep that API and forward every call to the
 * entry points declared here.  Each entry point names the reference interface
 * it replaces (file:line in the reference repository).
 *
 * Conventions
 *   - Every function returns an int status (ZEST_GPU_OK == 0).  Nothing aborts
 *     or traps; on failure zest_gpu_last_error() holds a message.
 *   - Buffers are plain pointers + sizes.  `mem` says whether the data
 *     pointers are host (ZEST_MEM_HOST) or device (ZEST_MEM_DEVICE) memory;
 *     host buffers are staged through device scratch owned by the context.
 *   - A context is bound to one device and one CUDA stream and is not
 *     thread-safe (like the reference's transformers, which hold scratch).
 *     Calls are asynchronous on that stream for device buffers and
 *     synchronous for host buffers.
 *   - Batches are contiguous: item b of a batch of grids starts at
 *     grids + b * grid_size(order); item b of a batch of expansions starts at
 *     coeffs + 2 * b * coeff_size(order) (pairs {cos, sin} as in the
 *     reference's std::array<double, 2> elements).
 *
 * Data layouts (identical to the reference):
 *   Zernike grid   [lon][lat][rad] = (2L-1, L+1, pad8(L+1))
 *                  include/zernike_glq_transformer.hpp:50-131
 *   Zernike coeffs idx(n,l,m) = (n+1)(n+3)(2n+1)/24 + floor(l^2/4) + m
 *                  include/layout.hpp:385-420
 *   SH grid        LonLat [lon][lat] = (2L-1, pad8(L));
 *                  LatLon [lat][lon] = (L, pad8(2L-1))
 *                  include/sh_glq_transformer.hpp:48-197
 *   SH coeffs      idx(l,m) = l(l+1)/2 + m, include/layout.hpp:203-240
 */
#ifndef ZEST_GPU_H
#define ZEST_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define ZEST_GPU_OK 0
#define ZEST_GPU_ERR_INVALID 1     /* invalid argument (order, size, enum, null pointer) */
#define ZEST_GPU_ERR_OOM 2         /* device allocation failed */
#define ZEST_GPU_ERR_CUDA 3        /* a CUDA runtime call or kernel launch failed */
#define ZEST_GPU_ERR_TIMEOUT 4     /* a bounded in-kernel wait gave up */
#define ZEST_GPU_ERR_UNSUPPORTED 5 /* valid request the library does not support */

/* ---- conventions: zest::zt::ZernikeNorm (zernike_conventions.hpp:35),
 *      zest::st::SHNorm, zest::st::SHPhase (sh_conventions.hpp:35-47) ---- */
#define ZEST_ZERNIKE_NORMED 0
#define ZEST_ZERNIKE_UNNORMED 1
#define ZEST_SH_GEO 0
#define ZEST_SH_QM 1
#define ZEST_SH_PHASE_NONE 0
#define ZEST_SH_PHASE_CS 1
/* zest::RotationType, include/rotor.hpp:38-44 */
#define ZEST_ROTATION_OBJECT 0
#define ZEST_ROTATION_COORDINATE 1
/* SH grid layouts: LonLatLayout (the default) / LatLonLayout */
#define ZEST_LAYOUT_LONLAT 0
#define ZEST_LAYOUT_LATLON 1
/* expansion layouts of zest_gpu_convert_expansion */
#define ZEST_EXPANSION_ZERNIKE 0     /* RealZernikeSpan: ZernikeTetrahedralLayout, layout.hpp:385-420 */
#define ZEST_EXPANSION_SH 1          /* RealSHSpan: TriangleLayout, layout.hpp:203-240 */
#define ZEST_EXPANSION_ZERNIKE_ROW 2 /* zt::ZernikeSHSpan: RowSkippingTriangleLayout, layout.hpp:334-371 */
/* arithmetic of the contractions */
#define ZEST_PRECISION_FP64 0  /* FP64 everywhere (plain form) */
#define ZEST_PRECISION_SPLIT 1 /* BF16 fixed-point slices on tcgen05, exact FP32 partial sums, FP64 recombination */
/* memory kinds of data pointers */
#define ZEST_MEM_DEVICE 0
#define ZEST_MEM_HOST 1

typedef struct zest_gpu_context zest_gpu_context;

/* ---- context ---- */
/* Creates a context on `device` bound to `stream` (a cudaStream_t; NULL = the
 * legacy default stream).  Replaces the scratch/caches a reference
 * transformer holds (zernike_glq_transformer.hpp:951-964).  A new context
 * computes in FP64, or in the split-precision form (six slices) when the
 * environment variable ZEST_GPU_PRECISION is "split". */
int zest_gpu_ctx_create(zest_gpu_context** ctx, int device, void* stream);
int zest_gpu_ctx_destroy(zest_gpu_context* ctx);
/* Message of the last failing call on this thread ("" if none). */
const char* zest_gpu_last_error(void);
/* Precision of the dense contractions; `slices` = number of BF16 digit
 * slices per operand for ZEST_PRECISION_SPLIT (4..6, 0 = default 6), 8-bit
 * digits, sums longer than 256 terms in chunks of at most 256. */
int zest_gpu_set_precision(zest_gpu_context* ctx, int precision, int slices);
int zest_gpu_synchronize(zest_gpu_context* ctx);
/* Releases cached tables and scratch (they are rebuilt on demand). */
int zest_gpu_trim(zest_gpu_context* ctx);

/* ---- profiling (no reference counterpart: the reference times whole calls
 *      with nanobench, benchmarks/benchmark_zernike_glq_forward_transform.cpp) ----
 * When enabled, every pipeline stage launched on the context stream is
 * bracketed by CUDA events; zest_gpu_profile_read synchronizes the stream and
 * returns the accumulated milliseconds and stage counts for the first n
 * stages (reset != 0 clears them). */
int zest_gpu_profile_enable(zest_gpu_context* ctx, int enable);
int zest_gpu_profile_read(zest_gpu_context* ctx, int reset, double* ms, long long* count, int n);
int zest_gpu_profile_stage_count(void);
/* BF16 tensor-core flops of the split-precision products issued while
 * profiling: `useful` counts valid rows x table rows x K x slice products,
 * `issued` the whole 128-row tiles as executed (reset != 0 clears them). */
int zest_gpu_profile_flops(zest_gpu_context* ctx, int reset, double* useful, double* issued);
const char* zest_gpu_profile_stage_name(int stage);
/* Number of kernels this library has launched in this process. */
unsigned long long zest_gpu_launch_count(void);

/* ---- sizes (doubles for grids, pairs for coefficients) ---- */
size_t zest_gpu_zt_grid_size(size_t order);
size_t zest_gpu_zt_coeff_size(size_t order);
size_t zest_gpu_st_grid_size(size_t order, int layout);
size_t zest_gpu_st_coeff_size(size_t order);

/* ---- Zernike GLQ transforms ----
 * forward: zt::GLQTransformer<...>::forward_transform(BallGLQGridSpan<const double>,
 *          RealZernikeSpan<std::array<double,2>,...>)  zernike_glq_transformer.hpp:640-655
 *          (and the container-returning overload :687-693).  The expansion is
 *          truncated to min(exp_order, grid_order); as in the reference, coefficients of
 *          higher orders are not written (the SH forward transform likewise).
 * backward: ::backward_transform(RealZernikeSpan<const ...>, BallGLQGridSpan<double>)
 *          zernike_glq_transformer.hpp:663-679 (and :701-707). */
int zest_gpu_zt_forward(zest_gpu_context* ctx, int zernike_norm, int sh_norm, int sh_phase,
                        size_t grid_order, size_t exp_order, size_t batch,
                        const double* grids, double* coeffs, int mem);
int zest_gpu_zt_backward(zest_gpu_context* ctx, int zernike_norm, int sh_norm, int sh_phase,
                         size_t exp_order, size_t grid_order, size_t batch,
                         const double* coeffs, double* grids, int mem);

/* ---- SH GLQ transforms ----
 * st::GLQTransformer<...>::forward_transform  sh_glq_transformer.hpp:632-647 (:709-714)
 * st::GLQTransformer<...>::backward_transform sh_glq_transformer.hpp:655-668 (:723-728) */
int zest_gpu_st_forward(zest_gpu_context* ctx, int sh_norm, int sh_phase, int layout,
                        size_t grid_order, size_t exp_order, size_t batch,
                        const double* grids, double* coeffs, int mem);
int zest_gpu_st_backward(zest_gpu_context* ctx, int sh_norm, int sh_phase, int layout,
                         size_t exp_order, size_t grid_order, size_t batch,
                         const double* coeffs, double* grids, int mem);

/* st::GLQTransformer<...>::backward_transform of a row-skipping SH expansion
 * (one parity of l), sh_glq_transformer.hpp:680-700 (:743-754): coefficients
 * in the row-skipping layout of exp_order ((exp_order + 1)^2 / 4 pairs per
 * item).  As the reference, the expansion is read as the row-skipping span of
 * order min(exp_order, grid_order), whose rows have the parity of that order;
 * the rows of the other parity contribute nothing. */
int zest_gpu_st_backward_rows(zest_gpu_context* ctx, int sh_norm, int sh_phase, int layout,
                              size_t exp_order, size_t grid_order, size_t batch,
                              const double* coeffs, double* grids, int mem);

/* ---- real <-> complex expansions (in place) ----
 * to_complex_expansion (to_complex = 1) / to_real_expansion (0) of
 *   SH expansions, real_sh_expansion.hpp:345-436 (kind ZEST_EXPANSION_SH);
 *   Zernike expansions, zernike_expansion.hpp:484-634 (ZEST_EXPANSION_ZERNIKE);
 *   per-n Zernike SH spans, zernike_expansion.hpp:636-775
 *   (ZEST_EXPANSION_ZERNIKE_ROW; no Zernike normalisation change).
 * The coefficients of `batch` expansions of `order` are rescaled from the
 * source conventions (src_*) to the destination ones (dst_*): m = 0 pairs by
 * st::conversion_const (times zt::conversion_factor(n) when the Zernike
 * normalisation changes), m > 0 pairs (a, b) to (f a, -f b) with
 * f = conversion_const / sqrt(2) (to complex) or conversion_const sqrt(2) (to
 * real), negated for odd m when the phase convention changes.  Each factor is
 * computed as the reference computes it, so the results are bit-identical. */
int zest_gpu_convert_expansion(zest_gpu_context* ctx, int kind, size_t order, size_t batch, double* coeffs,
                               int src_zernike_norm, int src_sh_norm, int src_sh_phase,
                               int dst_zernike_norm, int dst_sh_norm, int dst_sh_phase,
                               int to_complex, int mem);

/* ---- rotations (in place) ----
 * Rotor::rotate(real Zernike expansion, WignerdPiHalfCollection, euler, type)
 *   rotor.hpp:214-243; (real SH expansion) rotor.hpp:125-141.
 * `euler` holds 3 angles (alpha, beta, gamma, intrinsic ZYZ) per batch item.
 * The rotation-matrix overloads (rotor.hpp:264-300) map to
 * zest_gpu_euler_from_matrix followed by these calls. */
int zest_gpu_zt_rotate(zest_gpu_context* ctx, size_t order, size_t batch,
                       double* coeffs, const double* euler, int rotation_type, int mem);
int zest_gpu_st_rotate(zest_gpu_context* ctx, size_t order, size_t batch,
                       double* coeffs, const double* euler, int rotation_type, int mem);
/* Rotor::rotate of a row-skipping (single-parity) SH expansion, rotor.hpp:165-193:
 * a zt::ZernikeSHSpan of `order` (the n = order - 1 row of a Zernike
 * expansion: rows l = (order - 1) mod 2, + 2, .., < order, pair
 * floor(l^2/4) + m, (order + 1)^2 / 4 pairs per item), l = 0 included. */
int zest_gpu_rows_rotate(zest_gpu_context* ctx, size_t order, size_t batch,
                         double* coeffs, const double* euler, int rotation_type, int mem);
/* Rotor::polar_rotate, rotor.hpp:316-378 (one angle per batch item). */
int zest_gpu_zt_polar_rotate(zest_gpu_context* ctx, size_t order, size_t batch,
                             double* coeffs, const double* angles, int rotation_type, int mem);
int zest_gpu_st_polar_rotate(zest_gpu_context* ctx, size_t order, size_t batch,
                             double* coeffs, const double* angles, int rotation_type, int mem);
/* euler_angles_from_rotation_matrix, rotor.hpp:53-63 (row-major 3x3, host). */
int zest_gpu_euler_from_matrix(const double* matrix, double* euler);

/* ---- points of the quadrature grids (host arrays, no context) ----
 * BallGLQGridPoints (zernike_glq_transformer.hpp:336-501): 2L-1 longitudes
 * 2 pi i / (2L-1), L+1 colatitudes (the GL nodes in angle style, descending
 * from near pi) and pad8(L+1) radii (1 + x_k)/2.  SphereGLQGridPoints
 * (sh_glq_transformer.hpp:385-504): the longitudes and colatitudes of the
 * layout's shape, padding included, as the reference (LonLat: 2L-1 and
 * pad8(L); LatLon: pad8(2L-1) and L). */
int zest_gpu_zt_grid_points(size_t order, double* lon, double* colat, double* rad);
int zest_gpu_st_grid_points(size_t order, int layout, double* lon, double* colat);

/* ---- evaluation at arbitrary points ----
 * zt::GridEvaluator::evaluate, grid_evaluator.hpp:228-266 (sums in
 * src/grid_evaluator.cpp:180-257): the values of `batch` Zernike expansions of
 * `order` on the product grid of nlon longitudes, nlat colatitudes and nrad
 * radii, values[b][i][j][k] row-major, item b at b * nlon * nlat * nrad.
 * `coeffs`, `values` and the three point arrays are all host or all device
 * memory (`mem`).  Like the reference, cos(colatitude), cos(longitude) and
 * sin(longitude) are taken with the host's std::cos and std::sin, and the
 * multiples cos/sin(m lon) by its recurrence (src/grid_evaluator.cpp:43-66).
 * Unlike the reference, whose st::GridEvaluator keeps adding into a buffer it
 * never clears (src/grid_evaluator.cpp:95-151), every call starts afresh. */
int zest_gpu_zt_evaluate(zest_gpu_context* ctx, int zernike_norm, int sh_norm, int sh_phase, size_t order,
                         size_t batch, const double* coeffs, size_t nlon, const double* lon, size_t nlat,
                         const double* colat, size_t nrad, const double* rad, double* values, int mem);
/* st::GridEvaluator::evaluate, grid_evaluator.hpp:84-133: values[b][i][j],
 * nlon x nlat per item. */
int zest_gpu_st_evaluate(zest_gpu_context* ctx, int sh_norm, int sh_phase, size_t order, size_t batch,
                         const double* coeffs, size_t nlon, const double* lon, size_t nlat, const double* colat,
                         double* values, int mem);

/* ---- least-squares fits to scattered data (lsq_transformer.hpp) ----
 * `batch` data vectors of npoints values at the same points; coefficients of
 * every order below `order` are written, item b at b * 2 * coeff_size(order).
 * Solved by Householder QR of the design matrix (as the reference's LAPACK
 * dgels, src/linearfit.cpp), on the device; at least as many points as
 * unknowns (L^2 for SH, L(L+1)(L+2)/6 for Zernike).
 * st::LSQTransformer::transform, :57-110: points (latitude, longitude); the
 * basis P_lm(sin latitude) {cos, sin}(m longitude), as RealSHGenerator. */
int zest_gpu_st_lsq(zest_gpu_context* ctx, int sh_norm, int sh_phase, size_t order, size_t npoints, size_t batch,
                    const double* data, const double* lat, const double* lon, double* coeffs, int mem);
/* zt::LSQTransformer::transform, :119-187: points (r, longitude, colatitude);
 * the basis R_nl(r) P_lm(cos colatitude) {cos, sin}(m longitude), as
 * ZernikeGenerator.  (The reference's version of this fit passes the points
 * to its generator in another order and regroups the solution by l only;
 * this is the fit its interface describes.) */
int zest_gpu_zt_lsq(zest_gpu_context* ctx, int zernike_norm, int sh_norm, int sh_phase, size_t order, size_t npoints,
                    size_t batch, const double* data, const double* r, const double* lon, const double* colat,
                    double* coeffs, int mem);

/* ---- power spectra (power_spectra.hpp) ----
 * norm = 1/(4 pi) for ZEST_SH_GEO, 1 for ZEST_SH_QM (sh_conventions.hpp). */
/* st::power_spectrum, :88-104: out[b * order + l] = norm sum_m |c_lm|^2, l < order. */
int zest_gpu_st_power_spectrum(zest_gpu_context* ctx, int sh_norm, size_t order, size_t batch,
                               const double* coeffs, double* out, int mem);
/* st::cross_power_spectrum, :38-52: out[b * out_len + l] = norm sum_m a_lm . b_lm
 * for l < min(order, out_len - 1), as the reference; other entries untouched
 * (its vector overload, :62-69, passes out_len = order). */
int zest_gpu_st_cross_power_spectrum(zest_gpu_context* ctx, int sh_norm, size_t order, size_t batch,
                                     const double* a, const double* b, size_t out_len, double* out, int mem);
/* zt::power_spectrum, :124-146: out[b * floor((order+1)^2/4) + floor((n+1)^2/4) + l/2]
 * = norm sum_m |c_nlm|^2.  As in the reference, l runs over n&1, n&1+2, .. < n,
 * so the l = n entries are not written. */
int zest_gpu_zt_power_spectrum(zest_gpu_context* ctx, int sh_norm, size_t order, size_t batch,
                               const double* coeffs, double* out, int mem);

/* ---- Zernike rotation that allocates no device memory ----
 * No counterpart in the reference: its rotations run on the host.  Same
 * operation and result as zest_gpu_zt_rotate with ZEST_MEM_DEVICE (the same
 * kernels, in place on `coeffs`), for callers that must not allocate device
 * memory while they run: a process whose device memory is owned by another
 * allocator that reserved it up front (a framework's caching allocator, a
 * server that sized its pools at start-up), where an allocation from inside
 * a library can fail or squeeze those pools; and a caller with latency-bound
 * work on other streams, because cudaFree and a growing cudaMalloc can
 * synchronize the whole device.
 *
 * All pointers are device memory of the current device; `stream` is a
 * cudaStream_t of that device (NULL: the default stream).  `wignerd` is a
 * Wigner d(pi/2) table of order `wignerd_order` >= `order`, as written by
 * zest_gpu_wignerd_table, allocated and filled by the caller beforehand.
 * There is no context: the call allocates nothing, neither through this
 * library nor through any allocating library routine.  Its scratch (the
 * list of rotated (n, l) vectors and the phase tables) is one fixed array
 * of ZEST_GPU_NOALLOC_SCRATCH_BYTES inside the library's device image, one
 * per device; nothing in it has to start at zero, since each call writes
 * every byte it reads.  A call needs 8 nvec(order) bytes (rounded up to 256)
 * plus 48 order batch bytes, nvec(order) ~ order^2 / 4; larger requests
 * return ZEST_GPU_ERR_UNSUPPORTED and do nothing.  The largest order that
 * fits is 1435 at batch 1; order 200 fits up to batch 428, order 64 up to
 * batch 1362.
 *
 * The first call on each device sets up: it looks up the array's address
 * with cudaGetSymbolAddress, which also loads the library's kernels onto the
 * device.  Make that first call with the device current and before any
 * stream capture on it.  The address is kept with the id of the CUDA context
 * it belongs to; after the device's context is replaced (cudaDeviceReset, or
 * the primary context released and retained again) the next call sets up
 * again in the new context.  Other calls only launch kernels.
 *
 * The array is shared by every caller in the process: two calls that can
 * run at the same time on one device (on streams without ordering between
 * them, or from different host threads) race on it and give wrong results.
 * Issue them on one stream, or order them with events.  The call returns
 * once its kernels are queued; synchronize `stream` before reading. */
#define ZEST_GPU_NOALLOC_SCRATCH_BYTES 4194304
int zest_gpu_zt_rotate_noalloc(void* stream, size_t order, size_t batch, double* coeffs,
                               const double* euler, int rotation_type,
                               const double* wignerd, size_t wignerd_order);

/* ---- batches of expansions of different orders (no reference counterpart;
 *      the reference runs one Rotor::rotate + backward_transform per expansion,
 *      rotor.hpp:214-243, zernike_glq_transformer.hpp:663-679) ----
 * Rotates expansion i by euler[3i..3i+2] (in place) and backward-transforms it
 * to a grid of its own order, for n_items expansions.  `orders` (host) must be
 * non-decreasing; `coeffs`, `euler` and `grids` are device buffers, expansions
 * and grids packed back to back in item order.  The first call for a given
 * (orders, buffers, conventions, precision) runs the work eagerly and records
 * it into a CUDA graph on the context; a later identical call replays the
 * graph (recorded anew if any of the context's device buffers was freed or
 * reallocated since, e.g. by zest_gpu_trim).  Results are those of
 * zest_gpu_zt_rotate + zest_gpu_zt_backward per item; in
 * ZEST_PRECISION_SPLIT (orders up to 256) the rotation's d(pi/2) products
 * also run in split precision on the tensor cores, within 1e-11 of FP64. */
int zest_gpu_zt_rotate_backward_ragged(zest_gpu_context* ctx, int zernike_norm, int sh_norm, int sh_phase,
                                       size_t n_items, const int* orders, double* coeffs, const double* euler,
                                       int rotation_type, double* grids);
/* Autotuning of the contraction tile shapes: when enabled (the default), the
 * first run of each Zernike stage at a new size times the candidate shapes on
 * the context stream and keeps the fastest (the FP64 tile shapes; in
 * ZEST_PRECISION_SPLIT the column tile, 80 or 32, of each single-sum tensor
 * core stage); disabled, a size rule picks them.  The shapes change only how
 * the output is tiled, not any result. */
int zest_gpu_set_autotune(zest_gpu_context* ctx, int enable);
/* Pipelining of host-memory Zernike transforms (mem = ZEST_MEM_HOST): a
 * batch whose per-item input or output exceeds `bytes` in total is cut into
 * chunks of about `bytes`, and the upload of one chunk, the transform of the
 * previous one and the download of the one before run at the same time (two
 * copy streams of the context and two device slots per direction).  The
 * default is 256 MiB; 0 turns the pipelining off.  Results do not depend on it.
 * Host buffers should be pinned for the copies to overlap. */
int zest_gpu_set_host_chunk_bytes(zest_gpu_context* ctx, size_t bytes);
/* Pins (page-locks) caller-owned host memory for the copies of ZEST_MEM_HOST
 * calls, so that they run asynchronously and overlap the transforms
 * (cudaHostRegister on the current device's context; no reference
 * counterpart: the reference transforms host memory in place), e.g. a
 * std::vector's data, for callers that do not link the CUDA runtime
 * themselves.  Unregister before freeing the memory. */
int zest_gpu_host_register(void* ptr, size_t bytes);
int zest_gpu_host_unregister(void* ptr);
/* Self-test of the failure path of the split GEMMs' bounded waits: one
 * kernel waits, for `seconds` (1 ms .. 2 s), on an mbarrier that nothing
 * arrives on, and a second wait in the same kernel gives up as soon as the
 * first has set the error flag.  Returns ZEST_GPU_ERR_TIMEOUT, reported
 * exactly as a timed-out GEMM is; the flag is cleared and the context stays
 * usable. */
int zest_gpu_selftest_wait_timeout(zest_gpu_context* ctx, double seconds);

/* ---- adjoints: vector-Jacobian products (no reference counterpart; the
 *      reference has no derivatives) ----
 * The transforms are linear; these return the transpose applied to a
 * cotangent, for gradients of losses through them.  With B the backward
 * transform, W the grid's quadrature weights and G the Gram diagonal of the
 * real basis, the reference's forward transform (zernike_glq_transformer.hpp:
 * 640-655, sh_glq_transformer.hpp:632-647) is F = G^+ B^T W, so
 *   forward_vjp:  grids_cot  = F^T coeffs_cot = W B (G^+ coeffs_cot)
 *   backward_vjp: coeffs_cot = B^T grids_cot  = G F (W^-1 grids_cot)
 * (the sin part of m = 0, and orders a transform does not use, get 0).
 * Orders, batching and memory kinds as for the transforms. */
int zest_gpu_zt_forward_vjp(zest_gpu_context* ctx, int zernike_norm, int sh_norm, int sh_phase,
                            size_t grid_order, size_t exp_order, size_t batch,
                            const double* coeffs_cot, double* grids_cot, int mem);
int zest_gpu_zt_backward_vjp(zest_gpu_context* ctx, int zernike_norm, int sh_norm, int sh_phase,
                             size_t exp_order, size_t grid_order, size_t batch,
                             const double* grids_cot, double* coeffs_cot, int mem);
int zest_gpu_st_forward_vjp(zest_gpu_context* ctx, int sh_norm, int sh_phase, int layout,
                            size_t grid_order, size_t exp_order, size_t batch,
                            const double* coeffs_cot, double* grids_cot, int mem);
int zest_gpu_st_backward_vjp(zest_gpu_context* ctx, int sh_norm, int sh_phase, int layout,
                             size_t exp_order, size_t grid_order, size_t batch,
                             const double* grids_cot, double* coeffs_cot, int mem);
/* Rotor::rotate (rotor.hpp:214-243 / 125-141) as y = D(euler) x, per batch
 * item: coeffs_cot = D^T out_cot (the inverse rotation of out_cot) and
 * euler_cot[3 b + k] = sum over coefficients of out_cot * d y / d euler_k.
 * Either output may be NULL; `coeffs` (x) is needed only for euler_cot.
 * The angle gradient supports orders up to 1024. */
int zest_gpu_zt_rotate_vjp(zest_gpu_context* ctx, size_t order, size_t batch, const double* coeffs,
                           const double* euler, int rotation_type, const double* out_cot,
                           double* coeffs_cot, double* euler_cot, int mem);
int zest_gpu_st_rotate_vjp(zest_gpu_context* ctx, size_t order, size_t batch, const double* coeffs,
                           const double* euler, int rotation_type, const double* out_cot,
                           double* coeffs_cot, double* euler_cot, int mem);

/* ---- split-precision dense product (no reference counterpart) ----
 * C = A B^T for row-major FP64 A (M x K) and B (N x K), K <= 2048, evaluated
 * with the context's slice count on the tcgen05 path used by
 * ZEST_PRECISION_SPLIT (BF16 fixed-point slices, exact FP32 partial sums,
 * FP64 recombination).  Exposed to test and measure the emulation itself. */
int zest_gpu_split_gemm(zest_gpu_context* ctx, size_t M, size_t N, size_t K, const double* A, const double* B,
                        double* C, int mem);

/* ---- tables (device generated, FP64) ----
 * gl::gl_nodes_and_weights<Layout, GLNodeStyle::cos>, gauss_legendre.hpp:1549-1565
 *   (host solve; packed = 1 for PackedLayout).  */
int zest_gpu_gl_nodes_weights(size_t n, int packed, double* nodes, double* weights);
/* st::PlmRecursion::plm_real(span z, PlmVecSpan), plm_recursion.hpp:109-113;
 * out[idx(l,m) * nz + i]. */
int zest_gpu_plm_table(zest_gpu_context* ctx, size_t order, int sh_norm, int sh_phase,
                       size_t nz, const double* z, double* out, int mem);
/* st::PlmRecursion::plm_complex(span z, PlmVecSpan), plm_recursion.hpp:133-139:
 * the same table without the sqrt(2) of the real basis for m > 0. */
int zest_gpu_plm_complex_table(zest_gpu_context* ctx, size_t order, int sh_norm, int sh_phase,
                               size_t nz, const double* z, double* out, int mem);
/* zt::RadialZernikeRecursion::zernike(span r, RadialZernikeVecSpan),
 * radial_zernike_recursion.hpp:152-288; out[(floor((n+1)^2/4) + l/2) * nr + k]. */
int zest_gpu_radial_table(zest_gpu_context* ctx, size_t order, int zernike_norm,
                          size_t nr, const double* r, double* out, int mem);
/* WignerdPiHalfCollection(order).matrices(), wignerd_collection.hpp:66-110,
 * src/wignerd_collection.cpp:29-98; size order(order+1)(2order+1)/6. */
int zest_gpu_wignerd_table(zest_gpu_context* ctx, size_t order, double* out, int mem);

#ifdef __cplusplus
}
#endif

#endif /* ZEST_GPU_H */
