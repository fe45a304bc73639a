// Launchers of the FP64 kernels of the GLQ path (fft.cu, gemm64.cu, rotate.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace zgpu {

// ---- longitude FFT ----------------------------------------------------------
struct FftPlan {
    int N = 0;            // transform length
    int nst = 0;          // number of Stockham stages
    int radix[24] = {};   // radix of each stage (product = N)
    const double2* tw = nullptr;  // device table W_t = exp(-2 pi i t / N), t < N
};
size_t fft_smem_bytes(int N, int NC);
// forward: x(b, i, col) at x + b*xb + i*si + col*sc, i < N, col < C
//          -> F[((b*nm + m)*C + col)*2 + {re,im}] = conj(X_m), m < nm
int launch_rfft_fwd(cudaStream_t s, const FftPlan& plan, const double* x, long long xb, long long si, long long sc,
                    int C, int nm, int batch, int lon_fast, double* F);
// inverse (Hermitian, factor 1): F as above -> x
int launch_rfft_inv(cudaStream_t s, const FftPlan& plan, const double* F, int C, int nm, int batch, int lon_fast,
                    double* x, long long xb, long long si, long long sc);

// ---- grouped FP64 contractions ------------------------------------------------
// Per-call metadata of the folded Legendre / radial stages, all device pointers.
struct LegMeta {
    const double* P = nullptr;      // folded Legendre table (rows x ld)
    const long long* off = nullptr; // row offset of group (m, p) = 2m + p
    const int* cnt = nullptr;       // rows of group (m, p) with l < Lm
    int ld = 0;                     // = number of folded nodes Kh
    int j0u = 0, j0d = 0;           // latitude index of folded node 0, north / south
};
struct RadMeta {
    const double* R = nullptr;      // radial table (rows x nr)
    const long long* off = nullptr; // row offset of group l
    const int* cnt = nullptr;       // rows (n = l, l+2, .. < Lm) of group l
};
struct TileList {
    const int4* tiles = nullptr;    // {group, row0, col0, -}
    int count = 0;
    int variant = 0;                // tile shape of the Zernike sums (zt_tile_shape)
};

// Zernike (G: [b][m][lat][rad][2], flm: [tri(l,m)][b][rad][2], coeffs: [b][zidx][2])
int launch_zt_leg_fwd(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* G, double* flm, int Lg,
                      int nlat, int nrad, int batch);
int launch_zt_leg_bwd(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* flm, double* G, int Lg,
                      int nlat, int nrad, int batch);
int launch_zt_rad_fwd(cudaStream_t s, const RadMeta& rm, const TileList& tl, const double* flm, double* coeffs,
                      int nrad, int batch, long long coeff_stride);
int launch_zt_rad_bwd(cudaStream_t s, const RadMeta& rm, const TileList& tl, const double* coeffs, double* flm,
                      int nrad, int batch, long long coeff_stride);
// SH (X: [b][m][lat][2], coeffs: [b][tri][2])
int launch_st_leg_fwd(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* X, double* coeffs,
                      int Lg, int nlat, int batch, long long coeff_stride);
int launch_st_leg_bwd(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* coeffs, double* X,
                      int Lg, int nlat, int batch, long long coeff_stride);
// Evaluation at arbitrary points: unfolded Legendre sums over all nlat nodes
// (lm.ld = nlat) into G [b][m][lat][rad][2] (Zernike) or G [b][m][lat][2]
// (SH); then the longitude sum into values [b][lon][lat * rad] with
// trig [lon][m][cos, sin].  Zernike tile shapes (variant) for ev_zt_leg and
// ev_lon, SH shapes for ev_st_leg.
int launch_ev_zt_leg(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* flm, double* G, int L,
                     int nlat, int nrad, int batch);
int launch_ev_st_leg(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* coeffs, double* G, int L,
                     int nlat, int batch, long long coeff_stride);
int launch_ev_lon(cudaStream_t s, const TileList& tl, const double* trig, const double* G, double* values, int L,
                  int nlon, int npts);
// tile shapes (rows x cols per CTA) of the launches above
void zt_tile_shape(int variant, int& bm, int& bn);
constexpr int kZtTileVariants = 3;
void st_tile_shape(int& bm, int& bn);

// ---- rotations ------------------------------------------------------------------
// Rotor::rotate on a batch of real expansions (in place).  kind 0 = Zernike,
// 1 = SH, 2 = SH rows of one parity in the row-skipping layout (a per-n
// Zernike SH span); vec_list holds the nvec rotated (n, l) vectors of one
// expansion.
// phase_scratch: 6 * L * batch doubles.
int launch_rotate_vectors(cudaStream_t s, int kind, int L, int batch, double* coeffs, long long cstride,
                          const int2* vec_list, int nvec, const double* wigner, const double* euler, int type,
                          double* phase_scratch);
int launch_polar_vectors(cudaStream_t s, int kind, int L, int batch, double* coeffs, long long cstride,
                         const int2* vec_list, int nvec, const double* angles, int type);
// Gradient of <ybar, rotate(x, euler)> with respect to the Euler angles of each
// batch item -> grad[3 * batch].  part: 3 * nvec * batch doubles of scratch.
int launch_rotate_euler_grad(cudaStream_t s, int kind, int L, int batch, const double* x, const double* ybar,
                             long long cstride, const int2* vec_list, int nvec, const double* wigner,
                             const double* euler, int type, double* phase_scratch, double* part, double* grad);
// Rotations of `items` expansions of different orders in one launch: work
// entries {item, n, l, -}, item i's coefficients at coeffs + coff[i]; phase
// scratch 6 * Lmax * items doubles.
int launch_rotate_ragged(cudaStream_t s, int kind, int Lmax, int items, double* coeffs, const long long* coff,
                         const int4* work, long long nwork, const double* wigner, const double* euler, int type,
                         double* phase_scratch);
// The phase tables e^{-i m angle} [item][alpha', beta', gamma'][m < Lmax] of a
// ragged rotation (double2 entries in phase_scratch).
int launch_phases(cudaStream_t s, int Lmax, int items, const double* euler, int type, double* phase_scratch);
// Euler angles (3 per item) of the inverse rotations.
int launch_invert_euler(cudaStream_t s, int batch, const double* euler, double* out);

// ---- adjoints of the transforms (adjoint.cu) --------------------------------------
// c_out = G c_in (inverse = 0) or G^+ c_in (inverse = 1) for the Gram diagonal of
// the real basis under the quadrature: G = S (1 if normed, 1/(2n+3) if unnormed)
// for Zernike, S for SH, S = 4 pi (geo) or 1 (qm); 0 for the sin part of m = 0.
int launch_zt_gram(cudaStream_t s, const double* in, double* out, int L, int batch, int sh_norm, int zernike_norm,
                   int inverse);
int launch_st_gram(cudaStream_t s, const double* in, double* out, int L, int batch, int sh_norm, int inverse);
// out[i] = in[i] * w[i % slab] (divide = 0) or in[i] / w[i % slab] (divide = 1) over n values.
int launch_grid_weights(cudaStream_t s, const double* in, double* out, long long n, const double* w, long long slab,
                        int divide);

// ---- coefficient layouts (layouts.cu) ------------------------------------------------
enum { CONVERT_ZERNIKE = 0, CONVERT_SH = 1, CONVERT_ROWS = 2 };
// In-place real <-> complex conversion of `pairs` coefficient pairs per item:
// m = 0 pairs times shnorm, m > 0 pairs (x, y) -> (f x, -f y) with f = norm,
// negated for odd m when phase_change; zconv = +1 / -1 multiplies both by
// sqrt(2n + 3) / 1 / sqrt(2n + 3) (Zernike normalisation change), 0 not.
// parity: the row parity of a row-skipping (CONVERT_ROWS) expansion.
struct ConvertParams {
    int kind = 0;
    int parity = 0;
    int zconv = 0;
    int phase_change = 0;
    long long pairs = 0;
    double shnorm = 1.0;
    double norm = 1.0;
};
int launch_convert(cudaStream_t s, const ConvertParams& P, int batch, double* coeffs);
// Row-skipping SH expansions of order Lm (src_pairs pairs apart) -> triangle
// expansions of order Lm, the rows of the other parity zero.
int launch_rows_to_triangle(cudaStream_t s, int Lm, long long src_pairs, int batch, const double* src, double* dst);

}  // namespace zgpu
