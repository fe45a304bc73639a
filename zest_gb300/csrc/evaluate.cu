// Expansions evaluated at arbitrary points, and power spectra.
//
//   zt::GridEvaluator::evaluate   grid_evaluator.hpp:228-266, src/grid_evaluator.cpp:160-257
//   st::GridEvaluator::evaluate   grid_evaluator.hpp:84-133,  src/grid_evaluator.cpp:95-151
//   detail::recursive_trig        src/grid_evaluator.cpp:43-66
//   st::power_spectrum            power_spectra.hpp:88-104
//   st::cross_power_spectrum      power_spectra.hpp:38-52
//   zt::power_spectrum            power_spectra.hpp:124-146
//
// The evaluation is the backward transform's three contractions with tables
// built at the caller's points instead of the quadrature nodes: the radial sum
// (gemm64 ZtRadBwd, R_nl at the radii), the Legendre sum over every colatitude
// (gemm64 EvZtLeg / EvStLeg, no equatorial folding: arbitrary points have no
// symmetry) and the longitude sum, a direct product with the cos/sin table of
// the longitudes (gemm64 EvLon; arbitrary longitudes rule out an FFT).  All
// FP64.  The reference computes cos(colatitude) and cos/sin(longitude) with
// std::cos / std::sin on the host; so does the caller of these functions.
#include <algorithm>
#include <vector>

#include "context.cuh"
#include "evaluate.cuh"
#include "tables.cuh"

namespace zgpu {

namespace {

// cos(m phi_i), sin(m phi_i) for m < L by the reference's recurrence:
// t_0 = (1, 0), t_1 = (cos phi, sin phi) (given), t_m = t_{m-1} * t_1 with each
// product and sum rounded as written.  trig[i][m][2].
__global__ void trig_kernel(int L, int nlon, const double* __restrict__ cs, double* __restrict__ trig) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nlon) return;
    double* t = trig + (long long)i * 2 * L;
    t[0] = 1.0;
    t[1] = 0.0;
    if (L < 2) return;
    const double c = cs[2 * i], s = cs[2 * i + 1];
    t[2] = c;
    t[3] = s;
    double pc = c, ps = s;
    for (int m = 2; m < L; ++m) {
        const double nc = __dsub_rn(__dmul_rn(pc, c), __dmul_rn(ps, s));
        const double ns = __dadd_rn(__dmul_rn(pc, s), __dmul_rn(ps, c));
        t[2 * m] = nc;
        t[2 * m + 1] = ns;
        pc = nc;
        ps = ns;
    }
}

// SH (cross) power spectrum: one thread per (item, l < nl),
// out = norm * (a_l0 b_l0 + sum_{m >= 1} (a_lm.c b_lm.c + a_lm.s b_lm.s)),
// summed over m in the reference's order.
__global__ void st_spectrum_kernel(int nl, int batch, const double* __restrict__ a, const double* __restrict__ b,
                                   long long cstride, double* __restrict__ out, long long ostride, double norm) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)nl * batch) return;
    const int bb = int(t / nl), l = int(t - (long long)bb * nl);
    const double* pa = a + bb * cstride + 2 * tri_idx(l, 0);
    const double* pb = b + bb * cstride + 2 * tri_idx(l, 0);
    double s = __dmul_rn(pa[0], pb[0]);
    for (int m = 1; m <= l; ++m)
        s = __dadd_rn(s, __dadd_rn(__dmul_rn(pa[2 * m], pb[2 * m]), __dmul_rn(pa[2 * m + 1], pb[2 * m + 1])));
    out[bb * ostride + l] = __dmul_rn(s, norm);
}

// Zernike power spectrum: one thread per (item, radial index (n, l)), n < L.
// The reference sums l = n&1, n&1 + 2, .. < n (power_spectra.hpp:136), so the
// l = n entries are left as they were; kept for identical results.
__global__ void zt_spectrum_kernel(int L, int batch, const double* __restrict__ c, long long cstride,
                                   double* __restrict__ out, long long ostride, double norm) {
    const long long nidx = ((long long)(L + 1) * (L + 1)) >> 2;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= nidx * batch) return;
    const int bb = int(t / nidx);
    const long long idx = t - (long long)bb * nidx;
    // n = the largest with floor((n+1)^2/4) <= idx
    int n = max(0, int(2.0 * sqrt(double(idx))) - 2);
    while ((((long long)(n + 2) * (n + 2)) >> 2) <= idx) ++n;
    while (n > 0 && (((long long)(n + 1) * (n + 1)) >> 2) > idx) --n;
    const int l = 2 * int(idx - ((((long long)(n + 1) * (n + 1)) >> 2))) + (n & 1);
    if (l >= n) return;
    const double* p = c + bb * cstride + 2 * zidx(n, l, 0);
    double s = __dmul_rn(p[0], p[0]);
    for (int m = 1; m <= l; ++m) s = __dadd_rn(s, __dadd_rn(__dmul_rn(p[2 * m], p[2 * m]), __dmul_rn(p[2 * m + 1], p[2 * m + 1])));
    out[bb * ostride + idx] = __dmul_rn(s, norm);
}

int upload_tiles(zest_gpu_context* ctx, DevBuf& buf, const std::vector<int4>& v, TileList* tl) {
    if (v.size() > 0x7fffffff) return fail(ZEST_GPU_ERR_UNSUPPORTED, "tile count overflow");
    ZG_TRY(upload(buf, v, ctx->stream));
    tl->tiles = buf.as<int4>();
    tl->count = int(v.size());
    tl->variant = 0;
    return ZEST_GPU_OK;
}

void add_tiles(std::vector<int4>& v, int g, long long M, long long N, int bm, int bn) {
    for (long long r = 0; r < M; r += bm)
        for (long long c = 0; c < N; c += bn) v.push_back(make_int4(g, int(r), int(c), 0));
}

// Legendre table P_lm(z_j) at every point, groups (m, parity of l - m) as in
// the transforms (l < L), with the group counts.
int eval_leg_table(zest_gpu_context* ctx, int L, int sn, int sp, const std::vector<double>& z, LegMeta* lm) {
    EvalBufs& E = ctx->eval;
    cudaStream_t s = ctx->stream;
    const int nz = int(z.size());
    std::vector<long long> off(2 * (size_t)L + 1, 0);
    std::vector<int> cnt(2 * (size_t)L, 0);
    long long rows = 0;
    for (int m = 0; m < L; ++m)
        for (int p = 0; p < 2; ++p) {
            off[2 * m + p] = rows;
            cnt[2 * m + p] = (L - m - p > 0) ? (L - m - p + 1) / 2 : 0;
            rows += cnt[2 * m + p];
        }
    off[2 * (size_t)L] = rows;
    ZG_TRY(upload(E.offP, off, s));
    ZG_TRY(upload(E.cntP, cnt, s));
    ZG_TRY(upload(E.z, z, s));
    ZG_TRY(E.P.ensure((size_t)rows * nz * sizeof(double)));
    ZG_TRY(launch_plm_gemm(s, L, L, sn, sp, nz, E.z.as<double>(), E.P.as<double>(), E.offP.as<long long>(), nullptr,
                           nz, 1.0));
    lm->P = E.P.as<double>();
    lm->off = E.offP.as<long long>();
    lm->cnt = E.cntP.as<int>();
    lm->ld = nz;
    lm->j0u = lm->j0d = 0;
    return ZEST_GPU_OK;
}

int eval_trig_table(zest_gpu_context* ctx, int L, const std::vector<double>& cs) {
    EvalBufs& E = ctx->eval;
    const int nlon = int(cs.size() / 2);
    ZG_TRY(upload(E.cs, cs, ctx->stream));
    ZG_TRY(E.trig.ensure((size_t)nlon * 2 * L * sizeof(double)));
    trig_kernel<<<(nlon + 127) / 128, 128, 0, ctx->stream>>>(L, nlon, E.cs.as<double>(), E.trig.as<double>());
    return launch_check("trig_kernel");
}

// items per pass so that the intermediate sums stay within about 4 GiB
int eval_items_per_pass(size_t bytes_per_item, int batch) {
    const size_t budget = size_t(4) << 30;
    return int(std::max<size_t>(1, std::min<size_t>(size_t(batch), budget / std::max<size_t>(bytes_per_item, 1))));
}

}  // namespace

int zt_evaluate_dev(zest_gpu_context* ctx, int zn, int sn, int sp, int L, int batch, const double* coeffs,
                    const std::vector<double>& z, const std::vector<double>& cs, const std::vector<double>& r,
                    double* values) {
    const int nlat = int(z.size()), nlon = int(cs.size() / 2), nrad = int(r.size());
    const long long npts = (long long)nlat * nrad;
    if (batch == 0 || nlat == 0 || nlon == 0 || nrad == 0) return ZEST_GPU_OK;
    cudaStream_t s = ctx->stream;
    if (L == 0) {
        ZG_CUDA_TRY(cudaMemsetAsync(values, 0, (size_t)batch * nlon * npts * sizeof(double), s));
        return ZEST_GPU_OK;
    }
    EvalBufs& E = ctx->eval;
    LegMeta lm;
    RadMeta rm;
    {
        StageScope sc(ctx, ST_EVAL_TABLES);
        ZG_TRY(eval_leg_table(ctx, L, sn, sp, z, &lm));
        // radial table R_nl(r_k), groups l, rows n = l, l + 2, .. < L
        std::vector<long long> off((size_t)L + 1, 0);
        std::vector<int> cnt((size_t)L, 0);
        long long rows = 0;
        for (int l = 0; l < L; ++l) {
            off[l] = rows;
            cnt[l] = (L - l + 1) / 2;
            rows += cnt[l];
        }
        off[L] = rows;
        ZG_TRY(upload(E.offR, off, s));
        ZG_TRY(upload(E.cntR, cnt, s));
        ZG_TRY(upload(E.r, r, s));
        ZG_TRY(E.R.ensure((size_t)rows * nrad * sizeof(double)));
        ZG_TRY(launch_radial_gemm(s, L, L, zn, nrad, E.r.as<double>(), E.R.as<double>(), E.offR.as<long long>(),
                                  nullptr, 0));
        rm.R = E.R.as<double>();
        rm.off = E.offR.as<long long>();
        rm.cnt = E.cntR.as<int>();
        ZG_TRY(eval_trig_table(ctx, L, cs));
    }
    const long long csz = 2 * zsize(L);
    const size_t per_item = ((size_t)L * nlat + (size_t)tri_size(L)) * nrad * 2 * sizeof(double);
    const int per = eval_items_per_pass(per_item, batch);
    ZG_TRY(E.flm.ensure((size_t)tri_size(L) * per * nrad * 2 * sizeof(double)));
    ZG_TRY(E.G.ensure((size_t)L * nlat * per * nrad * 2 * sizeof(double)));
    int bm, bn;
    zt_tile_shape(0, bm, bn);
    int tiled_for = -1;
    TileList tr, tg, tn;
    for (int b0 = 0; b0 < batch; b0 += per) {
        const int nb = std::min(per, batch - b0);
        if (nb != tiled_for) {
            std::vector<int4> v;
            for (int l = 0; l < L; ++l) add_tiles(v, l, nrad, (long long)(l + 1) * nb * 2, bm, bn);
            ZG_TRY(upload_tiles(ctx, E.tiles[0], v, &tr));
            v.clear();
            for (int m = 0; m < L; ++m) add_tiles(v, m, nlat, (long long)nb * 2 * nrad, bm, bn);
            ZG_TRY(upload_tiles(ctx, E.tiles[1], v, &tg));
            v.clear();
            for (int b = 0; b < nb; ++b) add_tiles(v, b, nlon, npts, bm, bn);
            ZG_TRY(upload_tiles(ctx, E.tiles[2], v, &tn));
            tiled_for = nb;
        }
        {
            StageScope sc(ctx, ST_EVAL_RAD);
            ZG_TRY(launch_zt_rad_bwd(s, rm, tr, coeffs + b0 * csz, E.flm.as<double>(), nrad, nb, csz));
        }
        {
            StageScope sc(ctx, ST_EVAL_LEG);
            ZG_TRY(launch_ev_zt_leg(s, lm, tg, E.flm.as<double>(), E.G.as<double>(), L, nlat, nrad, nb));
        }
        {
            StageScope sc(ctx, ST_EVAL_LON);
            ZG_TRY(launch_ev_lon(s, tn, E.trig.as<double>(), E.G.as<double>(), values + (long long)b0 * nlon * npts,
                                 L, nlon, int(npts)));
        }
    }
    return ZEST_GPU_OK;
}

int st_evaluate_dev(zest_gpu_context* ctx, int sn, int sp, int L, int batch, const double* coeffs,
                    const std::vector<double>& z, const std::vector<double>& cs, double* values) {
    const int nlat = int(z.size()), nlon = int(cs.size() / 2);
    if (batch == 0 || nlat == 0 || nlon == 0) return ZEST_GPU_OK;
    cudaStream_t s = ctx->stream;
    if (L == 0) {
        ZG_CUDA_TRY(cudaMemsetAsync(values, 0, (size_t)batch * nlon * nlat * sizeof(double), s));
        return ZEST_GPU_OK;
    }
    EvalBufs& E = ctx->eval;
    LegMeta lm;
    {
        StageScope sc(ctx, ST_EVAL_TABLES);
        ZG_TRY(eval_leg_table(ctx, L, sn, sp, z, &lm));
        ZG_TRY(eval_trig_table(ctx, L, cs));
    }
    const long long csz = 2 * tri_size(L);
    const int per = eval_items_per_pass((size_t)L * nlat * 2 * sizeof(double), batch);
    ZG_TRY(E.G.ensure((size_t)L * nlat * per * 2 * sizeof(double)));
    int sbm, sbn, bm, bn;
    st_tile_shape(sbm, sbn);
    zt_tile_shape(0, bm, bn);
    int tiled_for = -1;
    TileList tg, tn;
    for (int b0 = 0; b0 < batch; b0 += per) {
        const int nb = std::min(per, batch - b0);
        if (nb != tiled_for) {
            std::vector<int4> v;
            for (int m = 0; m < L; ++m) add_tiles(v, m, nlat, 2LL * nb, sbm, sbn);
            ZG_TRY(upload_tiles(ctx, E.tiles[1], v, &tg));
            v.clear();
            for (int b = 0; b < nb; ++b) add_tiles(v, b, nlon, nlat, bm, bn);
            ZG_TRY(upload_tiles(ctx, E.tiles[2], v, &tn));
            tiled_for = nb;
        }
        {
            StageScope sc(ctx, ST_EVAL_LEG);
            ZG_TRY(launch_ev_st_leg(s, lm, tg, coeffs + b0 * csz, E.G.as<double>(), L, nlat, nb, csz));
        }
        {
            StageScope sc(ctx, ST_EVAL_LON);
            ZG_TRY(launch_ev_lon(s, tn, E.trig.as<double>(), E.G.as<double>(), values + (long long)b0 * nlon * nlat,
                                 L, nlon, nlat));
        }
    }
    return ZEST_GPU_OK;
}

int st_spectrum_dev(zest_gpu_context* ctx, int sn, int L, int batch, const double* a, const double* b, int nl,
                    long long out_stride, double* out) {
    if (batch == 0 || nl <= 0) return ZEST_GPU_OK;
    const double pi = 3.14159265358979323846264338327950288;
    const double norm = sn ? 1.0 : 1.0 / (4.0 * pi);
    const long long n = (long long)nl * batch;
    StageScope sc(ctx, ST_SPECTRUM);
    st_spectrum_kernel<<<unsigned((n + 255) / 256), 256, 0, ctx->stream>>>(nl, batch, a, b, 2 * tri_size(L), out,
                                                                          out_stride, norm);
    return launch_check("st_spectrum_kernel");
}

int zt_spectrum_dev(zest_gpu_context* ctx, int sn, int L, int batch, const double* c, double* out) {
    if (batch == 0 || L == 0) return ZEST_GPU_OK;
    const double pi = 3.14159265358979323846264338327950288;
    const double norm = sn ? 1.0 : 1.0 / (4.0 * pi);
    const long long nidx = ((long long)(L + 1) * (L + 1)) >> 2;
    const long long n = nidx * batch;
    StageScope sc(ctx, ST_SPECTRUM);
    zt_spectrum_kernel<<<unsigned((n + 255) / 256), 256, 0, ctx->stream>>>(L, batch, c, 2 * zsize(L), out, nidx,
                                                                          norm);
    return launch_check("zt_spectrum_kernel");
}

}  // namespace zgpu
