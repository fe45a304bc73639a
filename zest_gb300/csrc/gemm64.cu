// Grouped FP64 contractions of the GLQ path (the plain form).
//
// One templated tiled kernel, instantiated for the six quadrature sums:
//   Zernike  Legendre forward  integrate_latitudinal  zernike_glq_transformer.hpp:778-817
//            Legendre backward sum_l                  zernike_glq_transformer.hpp:901-941
//            radial forward    integrate_radial       zernike_glq_transformer.hpp:819-865
//            radial backward   sum_n                  zernike_glq_transformer.hpp:867-899
//   SH       Legendre forward  integrate_latitudinal  sh_glq_transformer.hpp:886-974
//            Legendre backward sum_l                  sh_glq_transformer.hpp:976-1051
//
// Every sum is a small dense matrix product per group (per m, per parity of
// l-m, or per l), so the kernel walks a host-built list of output tiles
// {group, row0, col0}.  The Legendre sums are folded over the equatorial
// symmetry P_lm(-z) = (-1)^(l+m) P_lm(z): the forward operand is
// G(z) +- G(-z) over the ceil(nlat/2) non-negative nodes, the backward
// output is E_0 +- E_1 written to the north/south node pair.  This halves the
// FP64 work of the dominant stage (the reference folds only the SH sum,
// sh_glq_transformer.hpp:797-884; the quadrature result is the same).
//
// FP64 on GB300 runs at ~1.2 TFLOP/s, so the kernel is DFMA-bound: tiles
// staged through shared memory, a register micro-tile per thread.
#include "common.cuh"
#include "kernels.cuh"

namespace zgpu {

namespace {

template <class Prob, int BM, int BN, int TM, int TN, int BK>
__global__ void __launch_bounds__((BM / TM) * (BN / TN)) gemm64_kernel(const Prob P, const int4* __restrict__ tiles) {
    constexpr int NT = (BM / TM) * (BN / TN);
    constexpr int NA = Prob::NACC;
    __shared__ double As[BK][BM];
    __shared__ double Bs[BK][BN];
    const int4 t = tiles[blockIdx.x];
    const int g = t.x, row0 = t.y, col0 = t.z;
    const int M = P.M(g), N = P.N(g);
    const int tx = threadIdx.x % (BN / TN);
    const int ty = threadIdx.x / (BN / TN);
    double acc[NA][TM][TN];
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) acc[a][i][j] = 0.0;

#pragma unroll
    for (int par = 0; par < NA; ++par) {
        const int K = P.K(g, par);
        for (int k0 = 0; k0 < K; k0 += BK) {
            for (int e = threadIdx.x; e < BM * BK; e += NT) {
                int i, k;
                if (Prob::A_K_FAST) { k = e % BK; i = e / BK; }
                else { i = e % BM; k = e / BM; }
                double v = 0.0;
                if (row0 + i < M && k0 + k < K) v = P.a(g, par, row0 + i, k0 + k);
                As[k][i] = v;
            }
            for (int e = threadIdx.x; e < BN * BK; e += NT) {
                const int n = e % BN, k = e / BN;
                double v = 0.0;
                if (col0 + n < N && k0 + k < K) v = P.b(g, par, k0 + k, col0 + n);
                Bs[k][n] = v;
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < BK; ++k) {
                double av[TM], bv[TN];
#pragma unroll
                for (int i = 0; i < TM; ++i) av[i] = As[k][ty * TM + i];
#pragma unroll
                for (int j = 0; j < TN; ++j) bv[j] = Bs[k][tx * TN + j];
#pragma unroll
                for (int i = 0; i < TM; ++i)
#pragma unroll
                    for (int j = 0; j < TN; ++j) acc[par][i][j] = fma(av[i], bv[j], acc[par][i][j]);
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        const int r = row0 + ty * TM + i;
        if (r >= M) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int c = col0 + tx * TN + j;
            if (c >= N) continue;
            double v[NA];
#pragma unroll
            for (int a = 0; a < NA; ++a) v[a] = acc[a][i][j];
            P.store(g, r, c, v);
        }
    }
}

// ---------------------------------------------------------------------------
// Zernike, Legendre forward: group g = 2m + p, rows l = m + p + 2i (l < Lm),
// K = folded nodes, columns (b, rad, re/im).
struct ZtLegFwd {
    static constexpr int NACC = 1;
    static constexpr bool A_K_FAST = true;
    LegMeta lm;
    const double* G;
    double* flm;
    int Lg, nlat, nr2, batch;
    __device__ int M(int g) const { return lm.cnt[g]; }
    __device__ int N(int) const { return batch * nr2; }
    __device__ int K(int, int) const { return lm.ld; }
    __device__ double a(int g, int, int i, int k) const { return lm.P[(lm.off[g] + i) * lm.ld + k]; }
    __device__ double b(int g, int, int k, int n) const {
        const int m = g >> 1, p = g & 1;
        const int bb = n / nr2, kc = n - bb * nr2;
        const double* base = G + ((long long)bb * Lg + m) * nlat * nr2 + kc;
        const double up = base[(long long)(lm.j0u + k) * nr2];
        const double dn = base[(long long)(lm.j0d - k) * nr2];
        return p ? up - dn : up + dn;
    }
    __device__ void store(int g, int i, int n, const double* v) const {
        const int m = g >> 1, p = g & 1;
        const int l = m + p + 2 * i;
        const int bb = n / nr2, kc = n - bb * nr2;
        flm[(tri_idx(l, m) * batch + bb) * nr2 + kc] = v[0];
    }
};

// Zernike, Legendre backward: group m, rows = folded nodes, two accumulations
// (p = 0, 1) over l = m + p + 2i; output north = E0 + E1, south = E0 - E1,
// conjugated (the reference's sum_l writes {w re, -w im}).
struct ZtLegBwd {
    static constexpr int NACC = 2;
    static constexpr bool A_K_FAST = false;
    LegMeta lm;
    const double* flm;
    double* G;
    int Lg, nlat, nr2, batch;
    __device__ int M(int) const { return lm.ld; }
    __device__ int N(int) const { return batch * nr2; }
    __device__ int K(int g, int p) const { return lm.cnt[2 * g + p]; }
    __device__ double a(int g, int p, int i, int k) const { return lm.P[(lm.off[2 * g + p] + k) * lm.ld + i]; }
    __device__ double b(int g, int p, int k, int n) const {
        const int l = g + p + 2 * k;
        const int bb = n / nr2, kc = n - bb * nr2;
        return flm[(tri_idx(l, g) * batch + bb) * nr2 + kc];
    }
    __device__ void store(int g, int i, int n, const double* v) const {
        const int bb = n / nr2, kc = n - bb * nr2;
        const double s = (kc & 1) ? -1.0 : 1.0;
        double* base = G + ((long long)bb * Lg + g) * nlat * nr2 + kc;
        base[(long long)(lm.j0u + i) * nr2] = s * (v[0] + v[1]);
        base[(long long)(lm.j0d - i) * nr2] = s * (v[0] - v[1]);
    }
};

// Zernike, radial forward: group l, rows n = l + 2i, K = rad nodes, columns
// (m, b, re/im) -> coefficients of item b.
struct ZtRadFwd {
    static constexpr int NACC = 1;
    static constexpr bool A_K_FAST = true;
    RadMeta rm;
    const double* flm;
    double* coeffs;
    int nr, batch;
    long long cstride;  // doubles per expansion in the coefficient batch
    __device__ int M(int g) const { return rm.cnt[g]; }
    __device__ int N(int g) const { return (g + 1) * batch * 2; }
    __device__ int K(int, int) const { return nr; }
    __device__ double a(int g, int, int i, int k) const { return rm.R[(rm.off[g] + i) * nr + k]; }
    __device__ double b(int g, int, int k, int n) const {
        const int c = n & 1, mb = n >> 1;
        return flm[(tri_idx(g, 0) * batch + mb) * (2LL * nr) + 2 * k + c];
    }
    __device__ void store(int g, int i, int n, const double* v) const {
        const int c = n & 1, mb = n >> 1;
        const int m = mb / batch, bb = mb - m * batch;
        coeffs[bb * cstride + zidx(g + 2 * i, g, m) * 2 + c] = v[0];
    }
};

// Zernike, radial backward (sum_n): group l, rows = rad nodes, K = n of that l.
struct ZtRadBwd {
    static constexpr int NACC = 1;
    static constexpr bool A_K_FAST = false;
    RadMeta rm;
    const double* coeffs;
    double* flm;
    int nr, batch;
    long long cstride;
    __device__ int M(int) const { return nr; }
    __device__ int N(int g) const { return (g + 1) * batch * 2; }
    __device__ int K(int g, int) const { return rm.cnt[g]; }
    __device__ double a(int g, int, int i, int k) const { return rm.R[(rm.off[g] + k) * nr + i]; }
    __device__ double b(int g, int, int k, int n) const {
        const int c = n & 1, mb = n >> 1;
        const int m = mb / batch, bb = mb - m * batch;
        return coeffs[bb * cstride + zidx(g + 2 * k, g, m) * 2 + c];
    }
    __device__ void store(int g, int i, int n, const double* v) const {
        const int c = n & 1, mb = n >> 1;
        flm[(tri_idx(g, 0) * batch + mb) * (2LL * nr) + 2 * i + c] = v[0];
    }
};

// SH, Legendre forward: group 2m + p, K = unique nodes, columns (b, re/im).
struct StLegFwd {
    static constexpr int NACC = 1;
    static constexpr bool A_K_FAST = true;
    LegMeta lm;
    const double* X;
    double* coeffs;
    int Lg, nlat, batch;
    long long cstride;
    __device__ int M(int g) const { return lm.cnt[g]; }
    __device__ int N(int) const { return batch * 2; }
    __device__ int K(int, int) const { return lm.ld; }
    __device__ double a(int g, int, int i, int k) const { return lm.P[(lm.off[g] + i) * lm.ld + k]; }
    __device__ double b(int g, int, int k, int n) const {
        const int m = g >> 1, p = g & 1;
        const int bb = n >> 1, c = n & 1;
        const double* base = X + ((long long)bb * Lg + m) * nlat * 2 + c;
        const double up = base[(long long)(lm.j0u + k) * 2];
        const double dn = base[(long long)(lm.j0d - k) * 2];
        return p ? up - dn : up + dn;
    }
    __device__ void store(int g, int i, int n, const double* v) const {
        const int m = g >> 1, p = g & 1;
        const int l = m + p + 2 * i;
        const int bb = n >> 1, c = n & 1;
        coeffs[bb * cstride + tri_idx(l, m) * 2 + c] = v[0];
    }
};

struct StLegBwd {
    static constexpr int NACC = 2;
    static constexpr bool A_K_FAST = false;
    LegMeta lm;
    const double* coeffs;
    double* X;
    int Lg, nlat, batch;
    long long cstride;
    __device__ int M(int) const { return lm.ld; }
    __device__ int N(int) const { return batch * 2; }
    __device__ int K(int g, int p) const { return lm.cnt[2 * g + p]; }
    __device__ double a(int g, int p, int i, int k) const { return lm.P[(lm.off[2 * g + p] + k) * lm.ld + i]; }
    __device__ double b(int g, int p, int k, int n) const {
        const int l = g + p + 2 * k;
        const int bb = n >> 1, c = n & 1;
        return coeffs[bb * cstride + tri_idx(l, g) * 2 + c];
    }
    __device__ void store(int g, int i, int n, const double* v) const {
        const int bb = n >> 1, c = n & 1;
        const double s = c ? -1.0 : 1.0;
        double* base = X + ((long long)bb * Lg + g) * nlat * 2 + c;
        base[(long long)(lm.j0u + i) * 2] = s * (v[0] + v[1]);
        base[(long long)(lm.j0d - i) * 2] = s * (v[0] - v[1]);
    }
};

// ---------------------------------------------------------------------------
// Evaluation at arbitrary points (zt::GridEvaluator, st::GridEvaluator,
// grid_evaluator.hpp:52-325, src/grid_evaluator.cpp:95-257).  The colatitudes
// have no equatorial symmetry, so the Legendre sums run over every node: one
// group per m, rows = nodes, the two parities of l - m accumulated apart and
// added (f_m = sum_l P_lm(z_j) flm, sum_l of the reference, no conjugation).

// Zernike: flm [tri(l,m)][b][rad][2] -> G [b][m][lat][rad][2]
struct EvZtLeg {
    static constexpr int NACC = 2;
    static constexpr bool A_K_FAST = false;
    LegMeta lm;
    const double* flm;
    double* G;
    int L, nlat, nr2, batch;
    __device__ int M(int) const { return lm.ld; }
    __device__ int N(int) const { return batch * nr2; }
    __device__ int K(int g, int p) const { return lm.cnt[2 * g + p]; }
    __device__ double a(int g, int p, int i, int k) const { return lm.P[(lm.off[2 * g + p] + k) * lm.ld + i]; }
    __device__ double b(int g, int p, int k, int n) const {
        const int l = g + p + 2 * k;
        const int bb = n / nr2, kc = n - bb * nr2;
        return flm[(tri_idx(l, g) * batch + bb) * nr2 + kc];
    }
    __device__ void store(int g, int i, int n, const double* v) const {
        const int bb = n / nr2, kc = n - bb * nr2;
        G[(((long long)bb * L + g) * nlat + i) * nr2 + kc] = v[0] + v[1];
    }
};

// SH: coeffs [b][tri][2] -> G [b][m][lat][2]
struct EvStLeg {
    static constexpr int NACC = 2;
    static constexpr bool A_K_FAST = false;
    LegMeta lm;
    const double* coeffs;
    double* G;
    int L, nlat, batch;
    long long cstride;
    __device__ int M(int) const { return lm.ld; }
    __device__ int N(int) const { return batch * 2; }
    __device__ int K(int g, int p) const { return lm.cnt[2 * g + p]; }
    __device__ double a(int g, int p, int i, int k) const { return lm.P[(lm.off[2 * g + p] + k) * lm.ld + i]; }
    __device__ double b(int g, int p, int k, int n) const {
        const int l = g + p + 2 * k;
        const int bb = n >> 1, c = n & 1;
        return coeffs[bb * cstride + tri_idx(l, g) * 2 + c];
    }
    __device__ void store(int g, int i, int n, const double* v) const {
        const int bb = n >> 1, c = n & 1;
        G[(((long long)bb * L + g) * nlat + i) * 2 + c] = v[0] + v[1];
    }
};

// Longitude sum (sum_m of the reference): group = item b, rows = longitudes i,
// K = 2L pairs (m, cos/sin), columns = (lat, rad) points:
// values[b][i][j][k] = sum_m G[b][m][j][k].re cos(m phi_i) + G[b][m][j][k].im sin(m phi_i).
struct EvLon {
    static constexpr int NACC = 1;
    static constexpr bool A_K_FAST = true;
    const double* trig;  // [i][m][cos, sin]
    const double* G;     // [b][m][lat * rad][2]
    double* values;      // [b][i][lat * rad]
    int L, nlon, npts;
    __device__ int M(int) const { return nlon; }
    __device__ int N(int) const { return npts; }
    __device__ int K(int, int) const { return 2 * L; }
    __device__ double a(int, int, int i, int k) const { return trig[(long long)i * 2 * L + k]; }
    __device__ double b(int g, int, int k, int n) const {
        const int m = k >> 1, c = k & 1;
        return G[(((long long)g * L + m) * npts + n) * 2 + c];
    }
    __device__ void store(int g, int i, int n, const double* v) const {
        values[((long long)g * nlon + i) * npts + n] = v[0];
    }
};

// tile shapes: Zernike sums have few rows and many columns; SH sums have
// many rows (or K) and 2*batch columns.  The Zernike sums come in three
// shapes of 256 threads (the autotuner picks one per stage and size): groups
// have (L - m)/2 or (L + 1)/2 rows, so small orders waste most of a 64-row tile.
//   variant 0: 64 x 64 (4 x 4 per thread), 1: 32 x 128 (2 x 8), 2: 16 x 128 (1 x 8)
constexpr int ZBK = 8;
constexpr int SBM = 128, SBN = 16, STM = 4, STN = 2, SBK = 8;

template <class Prob, int BM, int BN, int TM, int TN, int BK>
int run(cudaStream_t s, const Prob& p, const TileList& tl, const char* name) {
    if (tl.count <= 0) return ZEST_GPU_OK;
    gemm64_kernel<Prob, BM, BN, TM, TN, BK><<<tl.count, (BM / TM) * (BN / TN), 0, s>>>(p, tl.tiles);
    return launch_check(name);
}

template <class Prob>
int run_zt(cudaStream_t s, const Prob& p, const TileList& tl, const char* name) {
    switch (tl.variant) {
    case 1: return run<Prob, 32, 128, 2, 8, ZBK>(s, p, tl, name);
    case 2: return run<Prob, 16, 128, 1, 8, ZBK>(s, p, tl, name);
    default: return run<Prob, 64, 64, 4, 4, ZBK>(s, p, tl, name);
    }
}

}  // namespace

int launch_ev_zt_leg(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* flm, double* G, int L,
                     int nlat, int nrad, int batch) {
    EvZtLeg p{lm, flm, G, L, nlat, 2 * nrad, batch};
    return run_zt(s, p, tl, "ev_zt_leg");
}
int launch_ev_st_leg(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* coeffs, double* G, int L,
                     int nlat, int batch, long long coeff_stride) {
    EvStLeg p{lm, coeffs, G, L, nlat, batch, coeff_stride};
    return run<EvStLeg, SBM, SBN, STM, STN, SBK>(s, p, tl, "ev_st_leg");
}
int launch_ev_lon(cudaStream_t s, const TileList& tl, const double* trig, const double* G, double* values, int L,
                  int nlon, int npts) {
    EvLon p{trig, G, values, L, nlon, npts};
    return run_zt(s, p, tl, "ev_lon");
}

void zt_tile_shape(int variant, int& bm, int& bn) {
    bm = variant == 1 ? 32 : (variant == 2 ? 16 : 64);
    bn = variant == 0 ? 64 : 128;
}
void st_tile_shape(int& bm, int& bn) { bm = SBM; bn = SBN; }

int launch_zt_leg_fwd(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* G, double* flm, int Lg,
                      int nlat, int nrad, int batch) {
    ZtLegFwd p{lm, G, flm, Lg, nlat, 2 * nrad, batch};
    return run_zt(s, p, tl, "zt_leg_fwd");
}
int launch_zt_leg_bwd(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* flm, double* G, int Lg,
                      int nlat, int nrad, int batch) {
    ZtLegBwd p{lm, flm, G, Lg, nlat, 2 * nrad, batch};
    return run_zt(s, p, tl, "zt_leg_bwd");
}
int launch_zt_rad_fwd(cudaStream_t s, const RadMeta& rm, const TileList& tl, const double* flm, double* coeffs,
                      int nrad, int batch, long long coeff_stride) {
    ZtRadFwd p{rm, flm, coeffs, nrad, batch, coeff_stride};
    return run_zt(s, p, tl, "zt_rad_fwd");
}
int launch_zt_rad_bwd(cudaStream_t s, const RadMeta& rm, const TileList& tl, const double* coeffs, double* flm,
                      int nrad, int batch, long long coeff_stride) {
    ZtRadBwd p{rm, coeffs, flm, nrad, batch, coeff_stride};
    return run_zt(s, p, tl, "zt_rad_bwd");
}
int launch_st_leg_fwd(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* X, double* coeffs, int Lg,
                      int nlat, int batch, long long coeff_stride) {
    StLegFwd p{lm, X, coeffs, Lg, nlat, batch, coeff_stride};
    return run<StLegFwd, SBM, SBN, STM, STN, SBK>(s, p, tl, "st_leg_fwd");
}
int launch_st_leg_bwd(cudaStream_t s, const LegMeta& lm, const TileList& tl, const double* coeffs, double* X, int Lg,
                      int nlat, int batch, long long coeff_stride) {
    StLegBwd p{lm, coeffs, X, Lg, nlat, batch, coeff_stride};
    return run<StLegBwd, SBM, SBN, STM, STN, SBK>(s, p, tl, "st_leg_bwd");
}

}  // namespace zgpu
