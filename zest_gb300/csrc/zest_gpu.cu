// C-ABI of the GB300 GLQ transform and rotation path (include/zest_gpu.h).
//
// A context owns one device + stream, the per-order tables (generated on the
// device, FP64), the FFT plans, the tile lists of the grouped contractions and
// the scratch buffers -- the GPU counterpart of the scratch a reference
// transformer holds (zernike_glq_transformer.hpp:951-964).  Tables are built
// once per (order, conventions) and cached, like the reference's resize().
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "context.cuh"
#include "evaluate.cuh"
#include "kernels.cuh"
#include "split.cuh"
#include "tables.cuh"
#include "zest_gpu.h"

namespace zgpu {

static thread_local std::string g_last_error;
static std::atomic<unsigned long long> g_launches{0};

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int launch_check(const char* what) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ZEST_GPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return ZEST_GPU_OK;
}

}  // namespace zgpu

using namespace zgpu;

namespace zgpu {

// ---------------------------------------------------------------------------
static int set_device(zest_gpu_context* ctx) {
    ZG_CUDA_TRY(cudaSetDevice(ctx->device));
    return ZEST_GPU_OK;
}

static void factorize(int N, FftPlan& p) {
    p.N = N;
    p.nst = 0;
    int n = N;
    while (n % 4 == 0) { p.radix[p.nst++] = 4; n /= 4; }
    while (n % 2 == 0) { p.radix[p.nst++] = 2; n /= 2; }
    for (int q = 3; n > 1; q += 2)
        while (n % q == 0) { p.radix[p.nst++] = q; n /= q; }
}

static int get_fft(zest_gpu_context* ctx, int N, const FftPlan** out) {
    auto it = ctx->ffts.find(N);
    if (it == ctx->ffts.end()) {
        auto e = std::make_unique<FftEntry>();
        factorize(N, e->plan);
        if (e->plan.nst > 24) return fail(ZEST_GPU_ERR_UNSUPPORTED, "FFT length has too many factors");
        if (fft_smem_bytes(N, 1) > 220 * 1024) return fail(ZEST_GPU_ERR_UNSUPPORTED, "FFT length too large");
        std::vector<double> tw(2 * (size_t)N);
        const double pi = 3.14159265358979323846264338327950288;
        for (int t = 0; t < N; ++t) {
            // W_t = exp(-2 pi i t/N), evaluated on the reduced angle for accuracy
            const double ang = 2.0 * pi * double(t) / double(N);
            tw[2 * t] = std::cos(ang);
            tw[2 * t + 1] = -std::sin(ang);
        }
        ZG_TRY(upload(e->tw, tw, ctx->stream));
        e->plan.tw = e->tw.as<double2>();
        it = ctx->ffts.emplace(N, std::move(e)).first;
    }
    *out = &it->second->plan;
    return ZEST_GPU_OK;
}

// Folded Legendre tables at nodes z (nnodes of them), scale_f per node.
static int build_leg(zest_gpu_context* ctx, LegTables& t, int L, int sh_norm, int sh_phase,
                     const std::vector<double>& z, const std::vector<double>& scale_f) {
    cudaStream_t s = ctx->stream;
    t.L = L;
    t.nnodes = int(z.size());
    t.off_h.assign(2 * (size_t)L + 1, 0);
    long long rows = 0;
    for (int m = 0; m < L; ++m)
        for (int p = 0; p < 2; ++p) {
            t.off_h[2 * m + p] = rows;
            const int cnt = (L - m - p > 0) ? (L - m - p + 1) / 2 : 0;
            rows += cnt;
        }
    t.off_h[2 * (size_t)L] = rows;
    ZG_TRY(upload(t.off, t.off_h, s));
    const size_t bytes = (size_t)rows * t.nnodes * sizeof(double);
    ZG_TRY(t.Pf.ensure(bytes));
    ZG_TRY(t.Pb.ensure(bytes));
    DevBuf dz, ds;
    ZG_TRY(upload(dz, z, s));
    ZG_TRY(upload(ds, scale_f, s));
    ZG_TRY(launch_plm_gemm(s, L, L, sh_norm, sh_phase, t.nnodes, dz.as<double>(), t.Pf.as<double>(),
                           t.off.as<long long>(), ds.as<double>(), t.nnodes, 1.0));
    ZG_TRY(launch_plm_gemm(s, L, L, sh_norm, sh_phase, t.nnodes, dz.as<double>(), t.Pb.as<double>(),
                           t.off.as<long long>(), nullptr, t.nnodes, 0.5));
    ZG_CUDA_TRY(cudaStreamSynchronize(s));
    return ZEST_GPU_OK;
}

static int leg_cnt(zest_gpu_context* ctx, LegTables& t, int Lm, const int** out) {
    auto it = t.cnt.find(Lm);
    if (it == t.cnt.end()) {
        std::vector<int> c(2 * (size_t)t.L, 0);
        for (int m = 0; m < t.L; ++m)
            for (int p = 0; p < 2; ++p) c[2 * m + p] = (Lm - m - p > 0) ? (Lm - m - p + 1) / 2 : 0;
        auto b = std::make_unique<DevBuf>();
        ZG_TRY(upload(*b, c, ctx->stream));
        it = t.cnt.emplace(Lm, std::move(b)).first;
    }
    *out = it->second->as<int>();
    return ZEST_GPU_OK;
}

static int rad_cnt(zest_gpu_context* ctx, RadTables& t, int Lm, const int** out) {
    auto it = t.cnt.find(Lm);
    if (it == t.cnt.end()) {
        std::vector<int> c((size_t)t.L, 0);
        for (int l = 0; l < t.L; ++l) c[l] = (Lm - l > 0) ? (Lm - l + 1) / 2 : 0;
        auto b = std::make_unique<DevBuf>();
        ZG_TRY(upload(*b, c, ctx->stream));
        it = t.cnt.emplace(Lm, std::move(b)).first;
    }
    *out = it->second->as<int>();
    return ZEST_GPU_OK;
}

static int get_zt_plan(zest_gpu_context* ctx, int L, int zn, int sn, int sp, ZtPlan** out) {
    auto key = std::make_tuple(L, zn, sn, sp);
    auto it = ctx->zt_plans.find(key);
    if (it != ctx->zt_plans.end()) {
        *out = it->second.get();
        return ZEST_GPU_OK;
    }
    auto p = std::make_unique<ZtPlan>();
    p->sh = zt_shape(L);
    const int nt = int(p->sh.nlat), nr = int(p->sh.nrad), np = int(p->sh.nlon);
    p->lat_nodes.resize(nt);
    p->lat_w.resize(nt);
    p->rad_nodes.resize(nr);
    p->rad_w.resize(nr);
    gl_nodes_weights(nt, false, p->lat_nodes.data(), p->lat_w.data());
    gl_nodes_weights(nr, false, p->rad_nodes.data(), p->rad_w.data());
    for (auto& x : p->rad_nodes) x = 0.5 * (1.0 + x);
    // folded latitude nodes: the non-negative half, ascending from the equator
    const int kh = (nt + 1) / 2;
    p->leg.j0u = nt - kh;
    p->leg.j0d = kh - 1;
    const double pi = 3.14159265358979323846264338327950288;
    // quadrature prefactor sh_norm * 1/2 * 2 pi / nlon (zernike_glq_transformer.hpp:710-720)
    const double shn = sn ? 1.0 : 1.0 / (4.0 * pi);
    const double pref = shn * 0.5 * ((2.0 * pi) / double(np));
    std::vector<double> z(kh), sc(kh);
    for (int j = 0; j < kh; ++j) {
        z[j] = p->lat_nodes[p->leg.j0u + j];
        sc[j] = p->lat_w[p->leg.j0u + j] * pref;
        if (p->leg.j0u + j == p->leg.j0d - j) sc[j] *= 0.5;  // equator node appears in both halves
    }
    ZG_TRY(build_leg(ctx, p->leg, L, sn, sp, z, sc));
    // radial tables: forward R_nl(r_k) r_k^2 u_k (2n+3 if unnormed), backward R_nl(r_k)
    RadTables& rt = p->rad;
    rt.L = L;
    rt.nr = nr;
    rt.off_h.assign((size_t)L + 1, 0);
    long long rows = 0;
    for (int l = 0; l < L; ++l) {
        rt.off_h[l] = rows;
        rows += (L - l + 1) / 2;
    }
    rt.off_h[L] = rows;
    ZG_TRY(upload(rt.off, rt.off_h, ctx->stream));
    ZG_TRY(rt.Rf.ensure((size_t)rows * nr * sizeof(double)));
    ZG_TRY(rt.Rb.ensure((size_t)rows * nr * sizeof(double)));
    std::vector<double> rw(nr);
    for (int k = 0; k < nr; ++k) rw[k] = p->rad_nodes[k] * p->rad_nodes[k] * p->rad_w[k];
    DevBuf dr, drw;
    ZG_TRY(upload(dr, p->rad_nodes, ctx->stream));
    ZG_TRY(upload(drw, rw, ctx->stream));
    ZG_TRY(launch_radial_gemm(ctx->stream, L, L, zn, nr, dr.as<double>(), rt.Rf.as<double>(), rt.off.as<long long>(),
                              drw.as<double>(), zn == ZEST_ZERNIKE_UNNORMED));
    ZG_TRY(launch_radial_gemm(ctx->stream, L, L, zn, nr, dr.as<double>(), rt.Rb.as<double>(), rt.off.as<long long>(),
                              nullptr, 0));
    ZG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *out = p.get();
    ctx->zt_plans.emplace(key, std::move(p));
    return ZEST_GPU_OK;
}

static int get_st_plan(zest_gpu_context* ctx, int L, int sn, int sp, int layout, StPlan** out) {
    auto key = std::make_tuple(L, sn, sp, layout);
    auto it = ctx->st_plans.find(key);
    if (it != ctx->st_plans.end()) {
        *out = it->second.get();
        return ZEST_GPU_OK;
    }
    auto p = std::make_unique<StPlan>();
    p->sh = st_shape(L, layout);
    const int nt = int(p->sh.nlat), np = int(p->sh.nlon);
    const int nu = (nt + 1) / 2;
    std::vector<double> pn(nu), pw(nu);
    gl_nodes_weights(nt, true, pn.data(), pw.data());
    p->leg.j0u = nt - nu;
    p->leg.j0d = nu - 1;
    const double pi = 3.14159265358979323846264338327950288;
    // prefactor sh_norm * 2 pi / nlon (sh_glq_transformer.hpp:757-765); the
    // reference folds the middle node of an odd grid twice -- kept as is.
    const double shn = sn ? 1.0 : 1.0 / (4.0 * pi);
    const double pref = shn * (2.0 * pi) / double(np);
    std::vector<double> sc(nu);
    for (int j = 0; j < nu; ++j) sc[j] = pw[j] * pref;
    ZG_TRY(build_leg(ctx, p->leg, L, sn, sp, pn, sc));
    *out = p.get();
    ctx->st_plans.emplace(key, std::move(p));
    return ZEST_GPU_OK;
}

// Tile lists of the grouped contractions, cached per (kind, L, Lm, batch).
// kinds: 0 zt_leg_fwd, 1 zt_leg_bwd, 2 zt_rad_fwd, 3 zt_rad_bwd, 4 st_leg_fwd, 5 st_leg_bwd
static int get_tiles(zest_gpu_context* ctx, int kind, int L, int Lm, int batch, int aux, TileList* tl,
                     int variant = 0) {
    if (kind > 3) variant = 0;
    auto key = std::make_tuple(kind, L, Lm, batch, aux, variant);
    auto it = ctx->tiles.find(key);
    if (it == ctx->tiles.end()) {
        int bm, bn;
        if (kind <= 3) zt_tile_shape(variant, bm, bn);
        else st_tile_shape(bm, bn);
        std::vector<int4> v;
        auto add = [&](int g, long long M, long long N) {
            for (long long r = 0; r < M; r += bm)
                for (long long c = 0; c < N; c += bn) v.push_back(make_int4(g, int(r), int(c), 0));
        };
        const ZtShape zs = zt_shape(L);
        const long long nr2 = 2 * zs.nrad;
        switch (kind) {
        case 0:
            for (int m = 0; m < Lm; ++m)
                for (int p = 0; p < 2; ++p) {
                    const int cnt = (Lm - m - p > 0) ? (Lm - m - p + 1) / 2 : 0;
                    if (cnt) add(2 * m + p, cnt, batch * nr2);
                }
            break;
        case 1:
            for (int m = 0; m < L; ++m) add(m, aux, batch * nr2);  // aux = folded node count
            break;
        case 2:
            for (int l = 0; l < Lm; ++l) add(l, (Lm - l + 1) / 2, (long long)(l + 1) * batch * 2);
            break;
        case 3:
            for (int l = 0; l < Lm; ++l) add(l, zs.nrad, (long long)(l + 1) * batch * 2);
            break;
        case 4:
            for (int m = 0; m < Lm; ++m)
                for (int p = 0; p < 2; ++p) {
                    const int cnt = (Lm - m - p > 0) ? (Lm - m - p + 1) / 2 : 0;
                    if (cnt) add(2 * m + p, cnt, 2LL * batch);
                }
            break;
        case 5:
            for (int m = 0; m < L; ++m) add(m, aux, 2LL * batch);
            break;
        }
        if (v.size() > 0x7fffffff) return fail(ZEST_GPU_ERR_UNSUPPORTED, "tile count overflow");
        auto e = std::make_unique<TileEntry>();
        e->count = int(v.size());
        ZG_TRY(upload(e->buf, v, ctx->stream));
        it = ctx->tiles.emplace(key, std::move(e)).first;
    }
    tl->variant = variant;
    tl->tiles = it->second->buf.as<int4>();
    tl->count = it->second->count;
    return ZEST_GPU_OK;
}

static bool valid01(int x) { return x == 0 || x == 1; }

// ---------------------------------------------------------------------------
// Autotuner of the tile shape of the Zernike FP64 sums.  When tuning is on,
// the first run of a stage (kind 0..3) at a size (L, Lm, batch) times each
// tile shape with CUDA events on the context stream (after one untimed run)
// and keeps the fastest; the stages overwrite their outputs, so the extra runs
// change nothing.  Without tuning, or while the stream is being captured, a
// size rule picks the shape: small orders have few rows per group.
template <class Run>
static int zt_tile_variant(zest_gpu_context* ctx, int kind, int L, int Lm, int batch, int aux, Run&& run,
                           int* variant) {
    auto key = std::make_tuple(kind, L, Lm, batch);
    auto it = ctx->tuned.find(key);
    if (it != ctx->tuned.end()) {
        *variant = it->second;
        return ZEST_GPU_OK;
    }
    *variant = Lm < 48 ? 2 : (Lm < 96 ? 1 : 0);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    ZG_CUDA_TRY(cudaStreamIsCapturing(ctx->stream, &cap));
    if (!ctx->autotune || cap != cudaStreamCaptureStatusNone) return ZEST_GPU_OK;
    cudaEvent_t e0, e1;
    ZG_CUDA_TRY(cudaEventCreate(&e0));
    ZG_CUDA_TRY(cudaEventCreate(&e1));
    float best = 0.0f;
    int rc = ZEST_GPU_OK;
    for (int v = 0; v < kZtTileVariants && rc == ZEST_GPU_OK; ++v) {
        TileList tl;
        rc = get_tiles(ctx, kind, L, Lm, batch, aux, &tl, v);
        if (rc == ZEST_GPU_OK) rc = run(tl);
        if (rc == ZEST_GPU_OK && cudaEventRecord(e0, ctx->stream) != cudaSuccess) rc = fail(ZEST_GPU_ERR_CUDA, "event");
        if (rc == ZEST_GPU_OK) rc = run(tl);
        if (rc == ZEST_GPU_OK && cudaEventRecord(e1, ctx->stream) != cudaSuccess) rc = fail(ZEST_GPU_ERR_CUDA, "event");
        float ms = 0.0f;
        if (rc == ZEST_GPU_OK && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
            rc = fail(ZEST_GPU_ERR_CUDA, "autotuner timing failed");
        if (rc == ZEST_GPU_OK && (v == 0 || ms < best)) {
            best = ms;
            *variant = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == ZEST_GPU_OK) ctx->tuned.emplace(key, *variant);
    return rc;
}

// Runs one Zernike FP64 stage with its tuned tile shape, profiled as `stage`.
template <class Run>
static int zt_stage(zest_gpu_context* ctx, int stage, int kind, int L, int Lm, int batch, int aux, Run&& run) {
    int v = 0;
    ZG_TRY(zt_tile_variant(ctx, kind, L, Lm, batch, aux, run, &v));
    TileList tl;
    ZG_TRY(get_tiles(ctx, kind, L, Lm, batch, aux, &tl, v));
    StageScope sc(ctx, stage);
    return run(tl);
}

// ---------------------------------------------------------------------------
// Zernike transforms on device pointers.
int zt_forward_dev(zest_gpu_context* ctx, int zn, int sn, int sp, int Lg, int Le, int batch, const double* grids,
                   double* coeffs) {
    cudaStream_t s = ctx->stream;
    const long long csz = 2 * zsize(Le);
    if (batch == 0 || Le == 0 || Lg == 0) return ZEST_GPU_OK;
    const int Lm = Lg < Le ? Lg : Le;
    // like the reference, only the coefficients of orders below min(Le, Lg) are
    // written; the rest of each expansion is left as it was
    ZG_CUDA_TRY(cudaMemset2DAsync(coeffs, (size_t)csz * sizeof(double), 0, (size_t)2 * zsize(Lm) * sizeof(double),
                                  batch, s));
    ZtPlan* plan;
    ZG_TRY(get_zt_plan(ctx, Lg, zn, sn, sp, &plan));
    if (ctx->precision == ZEST_PRECISION_SPLIT)
        return split_zt_forward(ctx, *plan, Lg, Le, Lm, batch, grids, coeffs);
    const ZtShape& sh = plan->sh;
    const FftPlan* fft;
    ZG_TRY(get_fft(ctx, int(sh.nlon), &fft));
    const long long cols = sh.nlat * sh.nrad;
    ZG_TRY(ctx->s0.ensure((size_t)batch * Lg * cols * 2 * sizeof(double)));
    ZG_TRY(ctx->s1.ensure((size_t)tri_size(Lm) * batch * 2 * sh.nrad * sizeof(double)));
    double* G = ctx->s0.as<double>();
    double* flm = ctx->s1.as<double>();
    {
        StageScope sc(ctx, ST_FFT_FWD);
        ZG_TRY(launch_rfft_fwd(s, *fft, grids, sh.size(), cols, 1, int(cols), Lg, batch, 0, G));
    }
    LegMeta lm;
    lm.P = plan->leg.Pf.as<double>();
    lm.off = plan->leg.off.as<long long>();
    ZG_TRY(leg_cnt(ctx, plan->leg, Lm, &lm.cnt));
    lm.ld = plan->leg.nnodes;
    lm.j0u = plan->leg.j0u;
    lm.j0d = plan->leg.j0d;
    ZG_TRY(zt_stage(ctx, ST_LEG_FWD, 0, Lg, Lm, batch, 0, [&](const TileList& tl) {
        return launch_zt_leg_fwd(s, lm, tl, G, flm, Lg, int(sh.nlat), int(sh.nrad), batch);
    }));
    RadMeta rm;
    rm.R = plan->rad.Rf.as<double>();
    rm.off = plan->rad.off.as<long long>();
    ZG_TRY(rad_cnt(ctx, plan->rad, Lm, &rm.cnt));
    return zt_stage(ctx, ST_RAD_FWD, 2, Lg, Lm, batch, 0, [&](const TileList& tl) {
        return launch_zt_rad_fwd(s, rm, tl, flm, coeffs, int(sh.nrad), batch, csz);
    });
}

int zt_backward_dev(zest_gpu_context* ctx, int zn, int sn, int sp, int Le, int Lg, int batch, const double* coeffs,
                    double* grids) {
    cudaStream_t s = ctx->stream;
    if (batch == 0 || Lg == 0) return ZEST_GPU_OK;
    const ZtShape shg = zt_shape(Lg);
    const int Lm = Lg < Le ? Lg : Le;
    if (Lm == 0) {
        ZG_CUDA_TRY(cudaMemsetAsync(grids, 0, (size_t)batch * shg.size() * sizeof(double), s));
        return ZEST_GPU_OK;
    }
    const long long csz = 2 * zsize(Le);
    ZtPlan* plan;
    ZG_TRY(get_zt_plan(ctx, Lg, zn, sn, sp, &plan));
    if (ctx->precision == ZEST_PRECISION_SPLIT)
        return split_zt_backward(ctx, *plan, Le, Lg, Lm, batch, coeffs, grids);
    const ZtShape& sh = plan->sh;
    const FftPlan* fft;
    ZG_TRY(get_fft(ctx, int(sh.nlon), &fft));
    const long long cols = sh.nlat * sh.nrad;
    ZG_TRY(ctx->s0.ensure((size_t)batch * Lg * cols * 2 * sizeof(double)));
    ZG_TRY(ctx->s1.ensure((size_t)tri_size(Lm) * batch * 2 * sh.nrad * sizeof(double)));
    double* G = ctx->s0.as<double>();
    double* flm = ctx->s1.as<double>();
    RadMeta rm;
    rm.R = plan->rad.Rb.as<double>();
    rm.off = plan->rad.off.as<long long>();
    ZG_TRY(rad_cnt(ctx, plan->rad, Lm, &rm.cnt));
    ZG_TRY(zt_stage(ctx, ST_RAD_BWD, 3, Lg, Lm, batch, 0, [&](const TileList& tl) {
        return launch_zt_rad_bwd(s, rm, tl, coeffs, flm, int(sh.nrad), batch, csz);
    }));
    LegMeta lm;
    lm.P = plan->leg.Pb.as<double>();
    lm.off = plan->leg.off.as<long long>();
    ZG_TRY(leg_cnt(ctx, plan->leg, Lm, &lm.cnt));
    lm.ld = plan->leg.nnodes;
    lm.j0u = plan->leg.j0u;
    lm.j0d = plan->leg.j0d;
    ZG_TRY(zt_stage(ctx, ST_LEG_BWD, 1, Lg, Lm, batch, lm.ld, [&](const TileList& tl) {
        return launch_zt_leg_bwd(s, lm, tl, flm, G, Lg, int(sh.nlat), int(sh.nrad), batch);
    }));
    StageScope sc(ctx, ST_FFT_INV);
    return launch_rfft_inv(s, *fft, G, int(cols), Lg, batch, 0, grids, sh.size(), cols, 1);
}

int st_forward_dev(zest_gpu_context* ctx, int sn, int sp, int layout, int Lg, int Le, int batch,
                   const double* grids, double* coeffs) {
    cudaStream_t s = ctx->stream;
    const long long csz = 2 * tri_size(Le);
    if (batch == 0 || Le == 0 || Lg == 0) return ZEST_GPU_OK;
    const int Lm = Lg < Le ? Lg : Le;
    // only the coefficients of orders below min(Le, Lg) are written, as in the reference
    ZG_CUDA_TRY(cudaMemset2DAsync(coeffs, (size_t)csz * sizeof(double), 0, (size_t)2 * tri_size(Lm) * sizeof(double),
                                  batch, s));
    StPlan* plan;
    ZG_TRY(get_st_plan(ctx, Lg, sn, sp, layout, &plan));
    const StShape& sh = plan->sh;
    const FftPlan* fft;
    ZG_TRY(get_fft(ctx, int(sh.nlon), &fft));
    ZG_TRY(ctx->s0.ensure((size_t)batch * Lg * sh.nlat * 2 * sizeof(double)));
    double* X = ctx->s0.as<double>();
    const bool split = ctx->precision == ZEST_PRECISION_SPLIT;
    if (!split || !split_st_tensor_dft(sh.latlon, Lg)) {
        StageScope sc(ctx, ST_FFT_FWD);
        if (layout == ZEST_LAYOUT_LATLON)
            ZG_TRY(launch_rfft_fwd(s, *fft, grids, sh.size(), 1, sh.nlon, int(sh.nlat), Lg, batch, 1, X));
        else
            ZG_TRY(launch_rfft_fwd(s, *fft, grids, sh.size(), sh.nlat, 1, int(sh.nlat), Lg, batch, 0, X));
    }
    if (split) return split_st_forward(ctx, *plan, Lg, Lm, batch, grids, X, coeffs, csz);
    LegMeta lm;
    lm.P = plan->leg.Pf.as<double>();
    lm.off = plan->leg.off.as<long long>();
    ZG_TRY(leg_cnt(ctx, plan->leg, Lm, &lm.cnt));
    lm.ld = plan->leg.nnodes;
    lm.j0u = plan->leg.j0u;
    lm.j0d = plan->leg.j0d;
    TileList tl;
    ZG_TRY(get_tiles(ctx, 4, Lg, Lm, batch, 0, &tl));
    StageScope sc(ctx, ST_LEG_FWD);
    return launch_st_leg_fwd(s, lm, tl, X, coeffs, Lg, int(sh.nlat), batch, csz);
}

int st_backward_dev(zest_gpu_context* ctx, int sn, int sp, int layout, int Le, int Lg, int batch,
                    const double* coeffs, double* grids) {
    cudaStream_t s = ctx->stream;
    if (batch == 0 || Lg == 0) return ZEST_GPU_OK;
    const StShape shg = st_shape(Lg, layout);
    const int Lm = Lg < Le ? Lg : Le;
    if (Lm == 0) {
        ZG_CUDA_TRY(cudaMemsetAsync(grids, 0, (size_t)batch * shg.size() * sizeof(double), s));
        return ZEST_GPU_OK;
    }
    const long long csz = 2 * tri_size(Le);
    StPlan* plan;
    ZG_TRY(get_st_plan(ctx, Lg, sn, sp, layout, &plan));
    const StShape& sh = plan->sh;
    const FftPlan* fft;
    ZG_TRY(get_fft(ctx, int(sh.nlon), &fft));
    ZG_TRY(ctx->s0.ensure((size_t)batch * Lg * sh.nlat * 2 * sizeof(double)));
    double* X = ctx->s0.as<double>();
    const bool split = ctx->precision == ZEST_PRECISION_SPLIT;
    if (split && split_st_tensor_dft(sh.latlon, Lg))  // grids written by the tensor-core DFT
        return split_st_backward(ctx, *plan, Lg, Lm, batch, coeffs, csz, X, grids);
    if (split) {
        ZG_TRY(split_st_backward(ctx, *plan, Lg, Lm, batch, coeffs, csz, X, grids));
        StageScope sc(ctx, ST_FFT_INV);
        if (layout == ZEST_LAYOUT_LATLON)
            return launch_rfft_inv(s, *fft, X, int(sh.nlat), Lg, batch, 1, grids, sh.size(), 1, sh.nlon);
        return launch_rfft_inv(s, *fft, X, int(sh.nlat), Lg, batch, 0, grids, sh.size(), sh.nlat, 1);
    }
    LegMeta lm;
    lm.P = plan->leg.Pb.as<double>();
    lm.off = plan->leg.off.as<long long>();
    ZG_TRY(leg_cnt(ctx, plan->leg, Lm, &lm.cnt));
    lm.ld = plan->leg.nnodes;
    lm.j0u = plan->leg.j0u;
    lm.j0d = plan->leg.j0d;
    TileList tl;
    ZG_TRY(get_tiles(ctx, 5, Lg, Lm, batch, lm.ld, &tl));
    {
        StageScope sc(ctx, ST_LEG_BWD);
        ZG_TRY(launch_st_leg_bwd(s, lm, tl, coeffs, X, Lg, int(sh.nlat), batch, csz));
    }
    StageScope sc(ctx, ST_FFT_INV);
    if (layout == ZEST_LAYOUT_LATLON)
        return launch_rfft_inv(s, *fft, X, int(sh.nlat), Lg, batch, 1, grids, sh.size(), 1, sh.nlon);
    return launch_rfft_inv(s, *fft, X, int(sh.nlat), Lg, batch, 0, grids, sh.size(), sh.nlat, 1);
}

// ---------------------------------------------------------------------------
static int get_wigner(zest_gpu_context* ctx, int L, const double** out) {
    auto it = ctx->wigner.find(L);
    if (it == ctx->wigner.end()) {
        auto b = std::make_unique<DevBuf>();
        ZG_TRY(b->ensure((size_t)wig_off(L) * sizeof(double)));
        ZG_TRY(launch_wignerd(ctx->stream, L, b->as<double>()));
        it = ctx->wigner.emplace(L, std::move(b)).first;
    }
    *out = it->second->as<double>();
    return ZEST_GPU_OK;
}

// coefficient pairs of one expansion of order L: Zernike, SH triangle, or the
// row-skipping triangle of one parity ((L + 1)^2 / 4, include/layout.hpp:356-362)
static long long coeff_pairs(int kind, long long L) {
    return kind == 0 ? zsize(L) : kind == 1 ? tri_size(L) : ((L + 1) * (L + 1)) >> 2;
}

// rotated (n, l) vectors of one expansion, grouped by l
static int get_vectors(zest_gpu_context* ctx, int kind, int L, const int2** out, int* nvec) {
    auto key = std::make_tuple(kind, L);
    auto it = ctx->vec_lists.find(key);
    if (it == ctx->vec_lists.end()) {
        std::vector<int2> v;
        for (int l = 0; l < L; ++l) {
            if (kind == 0) {
                for (int n = (l == 0 ? 2 : l); n < L; n += 2) v.push_back(make_int2(n, l));
            } else if (kind == 2) {  // rows l = (L - 1) mod 2, + 2, .. < L; l = 0 too, as the Zernike n-rows
                if ((l & 1) == ((L - 1) & 1)) v.push_back(make_int2(L - 1, l));
            } else if (l >= 1) {
                v.push_back(make_int2(l, l));
            }
        }
        auto b = std::make_unique<DevBuf>();
        ZG_TRY(upload(*b, v, ctx->stream));
        it = ctx->vec_lists.emplace(key, std::make_pair(std::move(b), int(v.size()))).first;
    }
    *out = it->second.first->as<int2>();
    *nvec = it->second.second;
    return ZEST_GPU_OK;
}

// The rotated vectors of `batch` expansions of one order, sorted by l, for
// the split-precision rotation (cached per kind, order and batch).
static int get_uniform_rotation(zest_gpu_context* ctx, int kind, int L, int batch, UniformRotation** out) {
    auto key = std::make_tuple(kind, L, batch);
    auto it = ctx->uniform_rot.find(key);
    if (it == ctx->uniform_rot.end()) {
        auto u = std::make_unique<UniformRotation>();
        std::vector<int4> v;
        u->voff.assign((size_t)L + 1, 0);
        for (int l = 0; l < L; ++l) {
            for (int b = 0; b < batch; ++b) {
                if (kind == 0) {
                    for (int n = (l == 0 ? 2 : l); n < L; n += 2) v.push_back(make_int4(b, n, l, int(zidx(n, l, 0))));
                } else if (kind == 2) {
                    if ((l & 1) == ((L - 1) & 1)) v.push_back(make_int4(b, L - 1, l, int(((long long)l * l) >> 2)));
                } else if (l >= 1) {
                    v.push_back(make_int4(b, l, l, int(tri_idx(l, 0))));
                }
            }
            u->voff[(size_t)l + 1] = (long long)v.size();
        }
        std::vector<long long> coff((size_t)batch);
        for (int b = 0; b < batch; ++b) coff[(size_t)b] = (long long)b * 2 * coeff_pairs(kind, L);
        u->nvec = (long long)v.size();
        ZG_TRY(upload(u->vecs, v, ctx->stream));
        ZG_TRY(upload(u->coff, coff, ctx->stream));
        it = ctx->uniform_rot.emplace(key, std::move(u)).first;
    }
    *out = it->second.get();
    return ZEST_GPU_OK;
}

int rotate_dev(zest_gpu_context* ctx, int kind, int L, int batch, double* coeffs, const double* euler, int type) {
    // a whole expansion of order 1 has nothing to rotate; the row span of
    // order 1 (n = 0) still rotates its l = 0 vector, as the reference does
    if (batch == 0 || L < 1 || (L == 1 && kind != 2)) return ZEST_GPU_OK;
    const double* wig;
    ZG_TRY(get_wigner(ctx, L, &wig));
    if (ctx->precision == ZEST_PRECISION_SPLIT && L <= 256 && L >= 2) {
        // the X(+-pi/2) products of all vectors of one l as split GEMMs
        UniformRotation* u;
        ZG_TRY(get_uniform_rotation(ctx, kind, L, batch, &u));
        ZG_TRY(ctx->phase.ensure((size_t)batch * 6 * L * sizeof(double)));
        ZG_TRY(split_rotate_ragged(ctx, L, batch, u->nvec, u->vecs.as<int4>(), u->voff, u->coff.as<long long>(),
                                   coeffs, wig, euler, type, ctx->phase.as<double>()));
        return split_finish(ctx);
    }
    const int2* vl;
    int nvec;
    ZG_TRY(get_vectors(ctx, kind, L, &vl, &nvec));
    ZG_TRY(ctx->phase.ensure((size_t)batch * 6 * L * sizeof(double)));
    const long long cstride = 2 * coeff_pairs(kind, L);
    StageScope sc(ctx, ST_ROTATE);
    return launch_rotate_vectors(ctx->stream, kind, L, batch, coeffs, cstride, vl, nvec, wig, euler, type,
                                 ctx->phase.as<double>());
}

int polar_dev(zest_gpu_context* ctx, int kind, int L, int batch, double* coeffs, const double* angles, int type) {
    if (batch == 0 || L <= 1) return ZEST_GPU_OK;
    const int2* vl;
    int nvec;
    ZG_TRY(get_vectors(ctx, kind, L, &vl, &nvec));
    const long long cstride = 2 * coeff_pairs(kind, L);
    StageScope sc(ctx, ST_ROTATE);
    return launch_polar_vectors(ctx->stream, kind, L, batch, coeffs, cstride, vl, nvec, angles, type);
}

// ---------------------------------------------------------------------------
// Adjoints (vector-Jacobian products); the identities are in adjoint.cu.

// Quadrature weights of one slab of the grid, cached: Zernike [lat][rad] of
// (2 pi / nlon) w_lat w_rad r^2 / 2; SH LonLat [lat] and LatLon [lat][lon] of
// (2 pi / nlon) w_lat, the middle latitude of an odd LatLon grid doubled.
static int get_adj_weights(zest_gpu_context* ctx, int kind, int L, int layout, const double** out, long long* slab) {
    const double pi = 3.14159265358979323846264338327950288;
    auto key = std::make_tuple(kind, L, kind == 0 ? 0 : layout);
    auto it = ctx->adj_w.find(key);
    std::vector<double> w;
    if (kind == 0) {
        const ZtShape sh = zt_shape(L);
        *slab = sh.nlat * sh.nrad;
        if (it == ctx->adj_w.end()) {
            std::vector<double> xl(sh.nlat), wl(sh.nlat), xr(sh.nrad), wr(sh.nrad);
            gl_nodes_weights(long(sh.nlat), false, xl.data(), wl.data());
            gl_nodes_weights(long(sh.nrad), false, xr.data(), wr.data());
            w.resize((size_t)*slab);
            const double cphi = 2.0 * pi / double(sh.nlon);
            for (long long j = 0; j < sh.nlat; ++j)
                for (long long k = 0; k < sh.nrad; ++k) {
                    const double r = 0.5 * (1.0 + xr[k]);
                    w[j * sh.nrad + k] = cphi * wl[j] * (wr[k] * r * r * 0.5);
                }
        }
    } else {
        const StShape sh = st_shape(L, layout);
        *slab = layout == ZEST_LAYOUT_LATLON ? sh.nlat * sh.nlon : sh.nlat;
        if (it == ctx->adj_w.end()) {
            std::vector<double> xl(sh.nlat), wl(sh.nlat);
            gl_nodes_weights(long(sh.nlat), false, xl.data(), wl.data());
            const double cphi = 2.0 * pi / double(sh.nlon);
            for (long long j = 0; j < sh.nlat; ++j) wl[j] *= cphi;
            if ((sh.nlat & 1) && layout == ZEST_LAYOUT_LATLON) wl[sh.nlat / 2] *= 2.0;
            if (layout == ZEST_LAYOUT_LATLON) {
                w.resize((size_t)*slab);
                for (long long j = 0; j < sh.nlat; ++j)
                    for (long long i = 0; i < sh.nlon; ++i) w[j * sh.nlon + i] = wl[j];
            } else {
                w = wl;
            }
        }
    }
    if (it == ctx->adj_w.end()) {
        auto buf = std::make_unique<DevBuf>();
        ZG_TRY(upload(*buf, w, ctx->stream));
        it = ctx->adj_w.emplace(key, std::move(buf)).first;
    }
    *out = it->second->as<double>();
    return ZEST_GPU_OK;
}

// grid cotangent of a forward transform: W B (G^+ cbar)
int zt_forward_vjp_dev(zest_gpu_context* ctx, int zn, int sn, int sp, int Lg, int Le, int batch, const double* cbar,
                       double* gbar) {
    if (batch == 0 || Lg == 0) return ZEST_GPU_OK;
    const long long csz = 2 * zsize(Le), gsz = zt_shape(Lg).size();
    ZG_TRY(ctx->adj0.ensure((size_t)batch * csz * sizeof(double) + 16));
    ZG_TRY(launch_zt_gram(ctx->stream, cbar, ctx->adj0.as<double>(), Le, batch, sn, zn, 1));
    ZG_TRY(zt_backward_dev(ctx, zn, sn, sp, Le, Lg, batch, ctx->adj0.as<double>(), gbar));
    const double* w;
    long long slab;
    ZG_TRY(get_adj_weights(ctx, 0, Lg, 0, &w, &slab));
    return launch_grid_weights(ctx->stream, gbar, gbar, (long long)batch * gsz, w, slab, 0);
}

// coefficient cotangent of a backward transform: G F (W^-1 gbar); orders not
// used by the backward transform get 0
int zt_backward_vjp_dev(zest_gpu_context* ctx, int zn, int sn, int sp, int Le, int Lg, int batch, const double* gbar,
                        double* cbar) {
    if (batch == 0 || Le == 0) return ZEST_GPU_OK;
    const long long csz = 2 * zsize(Le), gsz = zt_shape(Lg).size();
    ZG_CUDA_TRY(cudaMemsetAsync(cbar, 0, (size_t)batch * csz * sizeof(double), ctx->stream));
    if (Lg == 0) return ZEST_GPU_OK;
    const double* w;
    long long slab;
    ZG_TRY(get_adj_weights(ctx, 0, Lg, 0, &w, &slab));
    ZG_TRY(ctx->adj0.ensure((size_t)batch * gsz * sizeof(double) + 16));
    ZG_TRY(launch_grid_weights(ctx->stream, gbar, ctx->adj0.as<double>(), (long long)batch * gsz, w, slab, 1));
    ZG_TRY(zt_forward_dev(ctx, zn, sn, sp, Lg, Le, batch, ctx->adj0.as<double>(), cbar));
    return launch_zt_gram(ctx->stream, cbar, cbar, Le, batch, sn, zn, 0);
}

int st_forward_vjp_dev(zest_gpu_context* ctx, int sn, int sp, int layout, int Lg, int Le, int batch,
                       const double* cbar, double* gbar) {
    if (batch == 0 || Lg == 0) return ZEST_GPU_OK;
    const long long csz = 2 * tri_size(Le), gsz = st_shape(Lg, layout).size();
    ZG_TRY(ctx->adj0.ensure((size_t)batch * csz * sizeof(double) + 16));
    ZG_TRY(launch_st_gram(ctx->stream, cbar, ctx->adj0.as<double>(), Le, batch, sn, 1));
    ZG_TRY(st_backward_dev(ctx, sn, sp, layout, Le, Lg, batch, ctx->adj0.as<double>(), gbar));
    const double* w;
    long long slab;
    ZG_TRY(get_adj_weights(ctx, 1, Lg, layout, &w, &slab));
    return launch_grid_weights(ctx->stream, gbar, gbar, (long long)batch * gsz, w, slab, 0);
}

int st_backward_vjp_dev(zest_gpu_context* ctx, int sn, int sp, int layout, int Le, int Lg, int batch,
                        const double* gbar, double* cbar) {
    if (batch == 0 || Le == 0) return ZEST_GPU_OK;
    const long long csz = 2 * tri_size(Le), gsz = st_shape(Lg, layout).size();
    ZG_CUDA_TRY(cudaMemsetAsync(cbar, 0, (size_t)batch * csz * sizeof(double), ctx->stream));
    if (Lg == 0) return ZEST_GPU_OK;
    const double* w;
    long long slab;
    ZG_TRY(get_adj_weights(ctx, 1, Lg, layout, &w, &slab));
    ZG_TRY(ctx->adj0.ensure((size_t)batch * gsz * sizeof(double) + 16));
    ZG_TRY(launch_grid_weights(ctx->stream, gbar, ctx->adj0.as<double>(), (long long)batch * gsz, w, slab, 1));
    ZG_TRY(st_forward_dev(ctx, sn, sp, layout, Lg, Le, batch, ctx->adj0.as<double>(), cbar));
    return launch_st_gram(ctx->stream, cbar, cbar, Le, batch, sn, 0);
}

// y = rotate(x, euler): xbar = D^T ybar = rotate(ybar, inverse angles) (D is
// orthogonal on the real coefficients), ebar = (dy/d euler)^T ybar.
int rotate_vjp_dev(zest_gpu_context* ctx, int kind, int L, int batch, const double* x, const double* euler, int type,
                   const double* ybar, double* xbar, double* ebar) {
    if (batch == 0) return ZEST_GPU_OK;
    cudaStream_t s = ctx->stream;
    const long long cstride = kind == 0 ? 2 * zsize(L) : 2 * tri_size(L);
    if (xbar) {
        ZG_CUDA_TRY(cudaMemcpyAsync(xbar, ybar, (size_t)batch * cstride * sizeof(double), cudaMemcpyDeviceToDevice, s));
        ZG_TRY(ctx->adj1.ensure((size_t)batch * 3 * sizeof(double)));
        ZG_TRY(launch_invert_euler(s, batch, euler, ctx->adj1.as<double>()));
        ZG_TRY(rotate_dev(ctx, kind, L, batch, xbar, ctx->adj1.as<double>(), type));
    }
    if (ebar) {
        if (L <= 1) {
            ZG_CUDA_TRY(cudaMemsetAsync(ebar, 0, (size_t)batch * 3 * sizeof(double), s));
            return ZEST_GPU_OK;
        }
        const double* wig;
        ZG_TRY(get_wigner(ctx, L, &wig));
        const int2* vl;
        int nvec;
        ZG_TRY(get_vectors(ctx, kind, L, &vl, &nvec));
        ZG_TRY(ctx->phase.ensure((size_t)batch * 6 * L * sizeof(double)));
        ZG_TRY(ctx->adj2.ensure((size_t)batch * nvec * 3 * sizeof(double) + 16));
        StageScope sc(ctx, ST_ROTATE);
        ZG_TRY(launch_rotate_euler_grad(s, kind, L, batch, x, ybar, cstride, vl, nvec, wig, euler, type,
                                        ctx->phase.as<double>(), ctx->adj2.as<double>(), ebar));
    }
    return ZEST_GPU_OK;
}

// ---------------------------------------------------------------------------
// Batches of expansions of different orders: rotate every expansion (one
// launch over a ragged work list), then backward-transform each group of equal
// order as one batch.  The first call for a given (orders, buffers,
// conventions, precision) runs eagerly -- building tables, work lists and
// scratch, and autotuning tile shapes -- and then records the same sequence
// into a CUDA graph; later identical calls replay the graph (a single launch
// from the host).
static int ragged_sequence(zest_gpu_context* ctx, RaggedPlan& P, double* coeffs, const double* euler,
                           double* grids) {
    const double* wig;
    ZG_TRY(get_wigner(ctx, P.Lmax, &wig));
    if (P.precision == ZEST_PRECISION_SPLIT && P.Lmax <= 256) {
        // the X(+-pi/2) products of all vectors of one l as split GEMMs
        ZG_TRY(split_rotate_ragged(ctx, P.Lmax, int(P.orders.size()), P.nwork, P.vecl.as<int4>(), P.voff, P.coff.as<long long>(),
                                   coeffs, wig, euler, P.type, ctx->phase.as<double>()));
    } else {
        StageScope sc(ctx, ST_ROTATE);
        ZG_TRY(launch_rotate_ragged(ctx->stream, 0, P.Lmax, int(P.orders.size()), coeffs, P.coff.as<long long>(),
                                    P.work.as<int4>(), P.nwork, wig, euler, P.type, ctx->phase.as<double>()));
    }
    for (const auto& bk : P.buckets) {
        const int L = std::get<0>(bk), first = std::get<1>(bk), count = std::get<2>(bk);
        ZG_TRY(zt_backward_dev(ctx, P.zn, P.sn, P.sp, L, L, count, coeffs + P.coff_h[first], grids + P.goff_h[first]));
    }
    return ZEST_GPU_OK;
}

// Runs `body` on the context's own capture stream (created on first use; the
// legacy default stream cannot be captured), ordered after the work queued on
// the context stream and before the work queued on it later.
template <class F>
static int on_graph_stream(zest_gpu_context* ctx, F&& body) {
    if (!ctx->graph_stream) {
        ZG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->graph_stream, cudaStreamNonBlocking));
        ZG_CUDA_TRY(cudaEventCreateWithFlags(&ctx->graph_ev[0], cudaEventDisableTiming));
        ZG_CUDA_TRY(cudaEventCreateWithFlags(&ctx->graph_ev[1], cudaEventDisableTiming));
    }
    cudaStream_t user = ctx->stream;
    ZG_CUDA_TRY(cudaEventRecord(ctx->graph_ev[0], user));
    ZG_CUDA_TRY(cudaStreamWaitEvent(ctx->graph_stream, ctx->graph_ev[0], 0));
    ctx->stream = ctx->graph_stream;
    const int rc = body();
    ctx->stream = user;
    ZG_CUDA_TRY(cudaEventRecord(ctx->graph_ev[1], ctx->graph_stream));
    ZG_CUDA_TRY(cudaStreamWaitEvent(user, ctx->graph_ev[1], 0));
    return rc;
}

static int ragged_on_graph_stream(zest_gpu_context* ctx, int zn, int sn, int sp, const std::vector<int>& orders,
                                  double* coeffs, const double* euler, int type, double* grids);

int zt_rotate_backward_ragged_dev(zest_gpu_context* ctx, int zn, int sn, int sp, const std::vector<int>& orders,
                                  double* coeffs, const double* euler, int type, double* grids) {
    return on_graph_stream(ctx, [&] { return ragged_on_graph_stream(ctx, zn, sn, sp, orders, coeffs, euler, type, grids); });
}

static int ragged_on_graph_stream(zest_gpu_context* ctx, int zn, int sn, int sp, const std::vector<int>& orders,
                                  double* coeffs, const double* euler, int type, double* grids) {
    RaggedPlan* P = ctx->ragged.get();
    const bool same = P && P->orders == orders && P->coeffs == coeffs && P->euler == euler && P->grids == grids &&
                      P->zn == zn && P->sn == sn && P->sp == sp && P->type == type &&
                      P->precision == ctx->precision && P->slices == ctx->slices;
    // the graph's kernels hold pointers to scratch, tables and work lists: a
    // buffer freed or reallocated since it was recorded means recording anew
    if (same && P->exec && P->epoch == alloc_epoch().load(std::memory_order_relaxed)) {
        ZG_CUDA_TRY(cudaGraphLaunch(P->exec, ctx->stream));
        if (P->precision == ZEST_PRECISION_SPLIT) ZG_TRY(split_check_flag(ctx));
        return ZEST_GPU_OK;
    }
    // new plan: offsets, buckets and the rotation work list
    auto np = std::make_unique<RaggedPlan>();
    np->orders = orders;
    np->coeffs = coeffs;
    np->euler = euler;
    np->grids = grids;
    np->zn = zn;
    np->sn = sn;
    np->sp = sp;
    np->type = type;
    np->precision = ctx->precision;
    np->slices = ctx->slices;
    const int n = int(orders.size());
    np->coff_h.resize(n + 1);
    np->goff_h.resize(n + 1);
    std::vector<int4> work;
    long long co = 0, go = 0;
    for (int i = 0; i < n; ++i) {
        const int L = orders[i];
        np->coff_h[i] = co;
        np->goff_h[i] = go;
        co += 2 * zsize(L);
        go += zt_shape(L).size();
        np->Lmax = std::max(np->Lmax, L);
        if (np->buckets.empty() || std::get<0>(np->buckets.back()) != L) np->buckets.emplace_back(L, i, 0);
        ++std::get<2>(np->buckets.back());
        for (int l = 0; l < L; ++l)  // the rotated (n, l) vectors, as get_vectors, with their first coefficient
            for (int nn = (l == 0 ? 2 : l); nn < L; nn += 2) work.push_back(make_int4(i, nn, l, int(zidx(nn, l, 0))));
    }
    np->coff_h[n] = co;
    np->goff_h[n] = go;
    np->nwork = (long long)work.size();
    ZG_TRY(upload(np->coff, np->coff_h, ctx->stream));
    ZG_TRY(upload(np->work, work, ctx->stream));
    {
        // the same vectors grouped by l (stable: item, then n, within a group)
        std::vector<int4> byl(work.size());
        np->voff.assign((size_t)np->Lmax + 1, 0);
        for (const int4& w : work) ++np->voff[(size_t)w.z + 1];
        for (int l = 0; l < np->Lmax; ++l) np->voff[(size_t)l + 1] += np->voff[(size_t)l];
        std::vector<long long> fill(np->voff.begin(), np->voff.end() - 1);
        for (const int4& w : work) byl[(size_t)fill[(size_t)w.z]++] = w;
        ZG_TRY(upload(np->vecl, byl, ctx->stream));
    }
    ZG_TRY(ctx->phase.ensure((size_t)n * 6 * std::max(np->Lmax, 1) * sizeof(double)));
    ctx->ragged = std::move(np);
    P = ctx->ragged.get();
    // eager run: the result of this call, and every table, list and buffer the graph needs
    ZG_TRY(ragged_sequence(ctx, *P, coeffs, euler, grids));
    ZG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    // record the same sequence (nothing executes during capture)
    const bool prof = ctx->prof.on;
    ctx->prof.on = false;
    ZG_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
    const int rc = ragged_sequence(ctx, *P, coeffs, euler, grids);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(ctx->stream, &g);
    ctx->prof.on = prof;
    if (rc != ZEST_GPU_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ec != cudaSuccess) return fail(ZEST_GPU_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
    P->graph = g;
    ZG_CUDA_TRY(cudaGraphInstantiate(&P->exec, g, 0));
    P->epoch = alloc_epoch().load(std::memory_order_relaxed);
    return ZEST_GPU_OK;
}

}  // namespace zgpu

// ===========================================================================
// C ABI
// ===========================================================================
namespace {

constexpr size_t kMaxOrder = 4096;

int check_ctx(zest_gpu_context* ctx) {
    if (!ctx) return fail(ZEST_GPU_ERR_INVALID, "null context");
    return set_device(ctx);
}

// Runs `body(in_dev, out_dev)` on device pointers, staging host buffers.
// With out_pitch > 0 only the first out_width of every out_pitch output
// elements are written by `body` and copied back (the rest of a host output is
// left as it was).
template <class F>
int with_staging(zest_gpu_context* ctx, int mem, const double* in, size_t in_n, double* out, size_t out_n, F&& body,
                 size_t out_pitch = 0, size_t out_width = 0) {
    if (mem == ZEST_MEM_DEVICE) return body(in, out);
    if (mem != ZEST_MEM_HOST) return fail(ZEST_GPU_ERR_INVALID, "mem must be ZEST_MEM_HOST or ZEST_MEM_DEVICE");
    cudaStream_t s = ctx->stream;
    ZG_TRY(ctx->in_stage.ensure(in_n * sizeof(double)));
    ZG_TRY(ctx->out_stage.ensure(out_n * sizeof(double)));
    if (in_n) {
        StageScope sc(ctx, ST_COPY_H2D);
        ZG_CUDA_TRY(cudaMemcpyAsync(ctx->in_stage.p, in, in_n * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    ZG_TRY(body(ctx->in_stage.as<double>(), ctx->out_stage.as<double>()));
    if (out_n && out_pitch && out_width < out_pitch) {
        if (out_width) {
            StageScope sc(ctx, ST_COPY_D2H);
            ZG_CUDA_TRY(cudaMemcpy2DAsync(out, out_pitch * sizeof(double), ctx->out_stage.p, out_pitch * sizeof(double),
                                          out_width * sizeof(double), out_n / out_pitch, cudaMemcpyDeviceToHost, s));
        }
    } else if (out_n) {
        StageScope sc(ctx, ST_COPY_D2H);
        ZG_CUDA_TRY(cudaMemcpyAsync(out, ctx->out_stage.p, out_n * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    ZG_CUDA_TRY(cudaStreamSynchronize(s));
    return ZEST_GPU_OK;
}

// Host buffers of a batch larger than ctx->host_chunk_bytes of input: the
// batch is cut into chunks of about that size whose uploads, computation and
// downloads overlap -- uploads and downloads on two copy streams of the
// context, the computation on the context stream, two device slots per
// direction ordered by events.  `body(in_dev, out_dev, nb)` transforms nb
// items; item sizes are in doubles; with out_pitch > 0 only the first
// out_width of every out_pitch output doubles of an item are written and
// copied back.  Device buffers and smaller batches go through with_staging.
template <class F>
int with_staging_batched(zest_gpu_context* ctx, int mem, const double* in, size_t in_item, double* out,
                         size_t out_item, int batch, F&& body, size_t out_pitch = 0, size_t out_width = 0) {
    auto whole = [&](const double* i, double* o) { return body(i, o, batch); };
    const size_t item_bytes = std::max(in_item, out_item) * sizeof(double);
    const size_t chunk = ctx->host_chunk_bytes;
    if (mem != ZEST_MEM_HOST || batch < 2 || chunk == 0 || (size_t)batch * item_bytes <= chunk)
        return with_staging(ctx, mem, in, (size_t)batch * in_item, out, (size_t)batch * out_item, whole,
                            out_pitch, out_width);
    const int per = (int)std::max<size_t>(1, chunk / item_bytes);
    if (!ctx->copy_stream[0]) {
        for (int k = 0; k < 2; ++k) ZG_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->copy_stream[k], cudaStreamNonBlocking));
        for (auto& ev : ctx->pipe_ev)
            for (auto& e : ev) ZG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    const size_t in_slot = (size_t)per * in_item, out_slot = (size_t)per * out_item;
    ZG_TRY(ctx->in_stage.ensure(2 * in_slot * sizeof(double)));
    ZG_TRY(ctx->out_stage.ensure(2 * out_slot * sizeof(double)));
    cudaStream_t cs = ctx->stream, up = ctx->copy_stream[0], down = ctx->copy_stream[1];
    cudaEvent_t(&ev)[3][2] = ctx->pipe_ev;  // [0] uploaded, [1] computed, [2] downloaded
    const int nch = (batch + per - 1) / per;
    auto dev_in = [&](int c) { return ctx->in_stage.as<double>() + (size_t)(c & 1) * in_slot; };
    auto dev_out = [&](int c) { return ctx->out_stage.as<double>() + (size_t)(c & 1) * out_slot; };
    auto count = [&](int c) { return std::min(per, batch - c * per); };
    auto upload_chunk = [&](int c) -> int {
        if (c >= 2) ZG_CUDA_TRY(cudaStreamWaitEvent(up, ev[1][c & 1], 0));  // slot free: chunk c-2 computed
        StageScope sc(ctx, ST_COPY_H2D, up);
        ZG_CUDA_TRY(cudaMemcpyAsync(dev_in(c), in + (size_t)c * per * in_item,
                                    (size_t)count(c) * in_item * sizeof(double), cudaMemcpyHostToDevice, up));
        ZG_CUDA_TRY(cudaEventRecord(ev[0][c & 1], up));
        return ZEST_GPU_OK;
    };
    // the context stream must not run ahead of work queued on it before this call
    ZG_CUDA_TRY(cudaEventRecord(ev[2][0], cs));
    ZG_CUDA_TRY(cudaStreamWaitEvent(up, ev[2][0], 0));
    ZG_CUDA_TRY(cudaStreamWaitEvent(down, ev[2][0], 0));
    ZG_TRY(upload_chunk(0));
    for (int c = 0; c < nch; ++c) {
        if (c + 1 < nch) ZG_TRY(upload_chunk(c + 1));
        ZG_CUDA_TRY(cudaStreamWaitEvent(cs, ev[0][c & 1], 0));
        if (c >= 2) ZG_CUDA_TRY(cudaStreamWaitEvent(cs, ev[2][c & 1], 0));  // output slot downloaded
        ZG_TRY(body(dev_in(c), dev_out(c), count(c)));
        ZG_CUDA_TRY(cudaEventRecord(ev[1][c & 1], cs));
        ZG_CUDA_TRY(cudaStreamWaitEvent(down, ev[1][c & 1], 0));
        {
            StageScope sc(ctx, ST_COPY_D2H, down);
            double* h = out + (size_t)c * per * out_item;
            if (out_pitch && out_width < out_pitch) {
                if (out_width)
                    ZG_CUDA_TRY(cudaMemcpy2DAsync(h, out_pitch * sizeof(double), dev_out(c), out_pitch * sizeof(double),
                                                  out_width * sizeof(double), (size_t)count(c) * out_item / out_pitch,
                                                  cudaMemcpyDeviceToHost, down));
            } else {
                ZG_CUDA_TRY(cudaMemcpyAsync(h, dev_out(c), (size_t)count(c) * out_item * sizeof(double),
                                            cudaMemcpyDeviceToHost, down));
            }
        }
        ZG_CUDA_TRY(cudaEventRecord(ev[2][c & 1], down));
    }
    ZG_CUDA_TRY(cudaStreamSynchronize(down));
    ZG_CUDA_TRY(cudaStreamSynchronize(cs));
    return ZEST_GPU_OK;
}

}  // namespace

extern "C" {

int zest_gpu_ctx_create(zest_gpu_context** out, int device, void* stream) {
    if (!out) return fail(ZEST_GPU_ERR_INVALID, "null output pointer");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(ZEST_GPU_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    if (device < 0 || device >= n) return fail(ZEST_GPU_ERR_INVALID, "device index out of range");
    ZG_CUDA_TRY(cudaSetDevice(device));
    int major = 0, minor = 0;
    ZG_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device));
    ZG_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device));
    if (major != 10 || minor != 3)
        return fail(ZEST_GPU_ERR_UNSUPPORTED, "this library is built for sm_103a (GB300) only; device is sm_" +
                                                  std::to_string(major) + std::to_string(minor));
    auto* ctx = new zest_gpu_context();
    ctx->device = device;
    ctx->stream = static_cast<cudaStream_t>(stream);
    // ZEST_GPU_PRECISION=split starts every new context in the split-precision
    // form (six slices), so code written against the reference's classes,
    // which have no precision setting, runs on the tensor cores unchanged.
    const char* want = std::getenv("ZEST_GPU_PRECISION");
    if (want && std::string(want) == "split") {
        const int st = zest_gpu_set_precision(ctx, ZEST_PRECISION_SPLIT, 6);
        if (st != ZEST_GPU_OK) {
            delete ctx;
            return st;
        }
    } else if (want && *want && std::string(want) != "fp64") {
        delete ctx;
        return fail(ZEST_GPU_ERR_INVALID, std::string("ZEST_GPU_PRECISION must be split or fp64, not ") + want);
    }
    *out = ctx;
    return ZEST_GPU_OK;
}

int zest_gpu_ctx_destroy(zest_gpu_context* ctx) {
    if (!ctx) return ZEST_GPU_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->ragged.reset();
    if (ctx->graph_stream) {
        cudaStreamSynchronize(ctx->graph_stream);
        cudaStreamDestroy(ctx->graph_stream);
        for (cudaEvent_t e : ctx->graph_ev)
            if (e) cudaEventDestroy(e);
    }
    for (cudaStream_t st : ctx->copy_stream)
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    for (auto& ev : ctx->pipe_ev)
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    delete ctx;
    return ZEST_GPU_OK;
}

const char* zest_gpu_last_error(void) { return g_last_error.c_str(); }

int zest_gpu_set_precision(zest_gpu_context* ctx, int precision, int slices) {
    ZG_TRY(check_ctx(ctx));
    if (precision != ZEST_PRECISION_FP64 && precision != ZEST_PRECISION_SPLIT)
        return fail(ZEST_GPU_ERR_INVALID, "unknown precision");
    if (slices == 0) slices = 6;
    if (slices < 4 || slices > 6) return fail(ZEST_GPU_ERR_INVALID, "slices must be in 4..6");
    if (precision == ZEST_PRECISION_SPLIT) ZG_TRY(split_available());
    ctx->precision = precision;
    ctx->slices = slices;
    return ZEST_GPU_OK;
}

int zest_gpu_synchronize(zest_gpu_context* ctx) {
    ZG_TRY(check_ctx(ctx));
    ZG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return ZEST_GPU_OK;
}

int zest_gpu_trim(zest_gpu_context* ctx) {
    ZG_TRY(check_ctx(ctx));
    ZG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->zt_plans.clear();
    ctx->st_plans.clear();
    ctx->ffts.clear();
    ctx->wigner.clear();
    ctx->vec_lists.clear();
    ctx->tiles.clear();
    ctx->s0.release();
    ctx->s1.release();
    ctx->in_stage.release();
    ctx->out_stage.release();
    ctx->aux_stage.release();
    ctx->phase.release();
    ctx->split.reset();
    return ZEST_GPU_OK;
}

int zest_gpu_profile_enable(zest_gpu_context* ctx, int enable) {
    ZG_TRY(check_ctx(ctx));
    ctx->prof.on = enable != 0;
    return ZEST_GPU_OK;
}

int zest_gpu_profile_read(zest_gpu_context* ctx, int reset, double* ms, long long* count, int n) {
    ZG_TRY(check_ctx(ctx));
    ZG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    Profiler& p = ctx->prof;
    for (auto& t : p.pending) {
        float el = 0.f;
        ZG_CUDA_TRY(cudaEventElapsedTime(&el, std::get<1>(t), std::get<2>(t)));
        p.ms[std::get<0>(t)] += el;
        p.count[std::get<0>(t)] += 1;
        p.pool.push_back(std::get<1>(t));
        p.pool.push_back(std::get<2>(t));
    }
    p.pending.clear();
    for (int i = 0; i < n && i < ST_COUNT; ++i) {
        if (ms) ms[i] = p.ms[i];
        if (count) count[i] = p.count[i];
    }
    if (reset)
        for (int i = 0; i < ST_COUNT; ++i) {
            p.ms[i] = 0.0;
            p.count[i] = 0;
        }
    return ZEST_GPU_OK;
}

const char* zest_gpu_profile_stage_name(int stage) { return stage_name(stage); }

int zest_gpu_profile_flops(zest_gpu_context* ctx, int reset, double* useful, double* issued) {
    ZG_TRY(check_ctx(ctx));
    split_flops(ctx, reset != 0, useful, issued);
    return ZEST_GPU_OK;
}
int zest_gpu_profile_stage_count(void) { return ST_COUNT; }
unsigned long long zest_gpu_launch_count(void) { return g_launches.load(); }

size_t zest_gpu_zt_grid_size(size_t order) { return (size_t)zt_shape((long long)order).size(); }
size_t zest_gpu_zt_coeff_size(size_t order) { return (size_t)zsize((long long)order); }
size_t zest_gpu_st_grid_size(size_t order, int layout) {
    return (size_t)st_shape((long long)order, layout == ZEST_LAYOUT_LATLON).size();
}
size_t zest_gpu_st_coeff_size(size_t order) { return (size_t)tri_size((long long)order); }

int zest_gpu_zt_forward(zest_gpu_context* ctx, int zn, int sn, int sp, size_t grid_order, size_t exp_order,
                        size_t batch, const double* grids, double* coeffs, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(zn) || !valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (grid_order > kMaxOrder || exp_order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t gn = batch * zest_gpu_zt_grid_size(grid_order), cn = batch * 2 * zest_gpu_zt_coeff_size(exp_order);
    if ((gn && !grids) || (cn && !coeffs)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    const size_t lm = grid_order < exp_order ? grid_order : exp_order;
    return with_staging_batched(
        ctx, mem, grids, zest_gpu_zt_grid_size(grid_order), coeffs, 2 * zest_gpu_zt_coeff_size(exp_order), int(batch),
        [&](const double* in, double* out, int nb) {
            return zt_forward_dev(ctx, zn, sn, sp, int(grid_order), int(exp_order), nb, in, out);
        },
        2 * zest_gpu_zt_coeff_size(exp_order), 2 * zest_gpu_zt_coeff_size(lm));
}

int zest_gpu_zt_backward(zest_gpu_context* ctx, int zn, int sn, int sp, size_t exp_order, size_t grid_order,
                         size_t batch, const double* coeffs, double* grids, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(zn) || !valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (grid_order > kMaxOrder || exp_order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t gn = batch * zest_gpu_zt_grid_size(grid_order), cn = batch * 2 * zest_gpu_zt_coeff_size(exp_order);
    if ((gn && !grids) || (cn && !coeffs)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging_batched(ctx, mem, coeffs, 2 * zest_gpu_zt_coeff_size(exp_order), grids,
                                zest_gpu_zt_grid_size(grid_order), int(batch),
                                [&](const double* in, double* out, int nb) {
                                    return zt_backward_dev(ctx, zn, sn, sp, int(exp_order), int(grid_order), nb, in,
                                                           out);
                                });
}

int zest_gpu_st_forward(zest_gpu_context* ctx, int sn, int sp, int layout, size_t grid_order, size_t exp_order,
                        size_t batch, const double* grids, double* coeffs, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn) || !valid01(sp) || !valid01(layout)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention/layout");
    if (grid_order > kMaxOrder || exp_order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t gn = batch * zest_gpu_st_grid_size(grid_order, layout), cn = batch * 2 * zest_gpu_st_coeff_size(exp_order);
    if ((gn && !grids) || (cn && !coeffs)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    const size_t lm = grid_order < exp_order ? grid_order : exp_order;
    return with_staging(
        ctx, mem, grids, gn, coeffs, cn,
        [&](const double* in, double* out) {
            return st_forward_dev(ctx, sn, sp, layout, int(grid_order), int(exp_order), int(batch), in, out);
        },
        2 * zest_gpu_st_coeff_size(exp_order), 2 * zest_gpu_st_coeff_size(lm));
}

int zest_gpu_st_backward(zest_gpu_context* ctx, int sn, int sp, int layout, size_t exp_order, size_t grid_order,
                         size_t batch, const double* coeffs, double* grids, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn) || !valid01(sp) || !valid01(layout)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention/layout");
    if (grid_order > kMaxOrder || exp_order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t gn = batch * zest_gpu_st_grid_size(grid_order, layout), cn = batch * 2 * zest_gpu_st_coeff_size(exp_order);
    if ((gn && !grids) || (cn && !coeffs)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging(ctx, mem, coeffs, cn, grids, gn, [&](const double* in, double* out) {
        return st_backward_dev(ctx, sn, sp, layout, int(exp_order), int(grid_order), int(batch), in, out);
    });
}

// Row-skipping (single-parity) SH expansions of order exp_order, truncated to
// min(exp_order, grid_order) as the reference truncates its span (the rows
// then take the parity of the truncated order), expanded to the triangle
// layout and backward-transformed.
int zest_gpu_st_backward_rows(zest_gpu_context* ctx, int sn, int sp, int layout, size_t exp_order,
                              size_t grid_order, size_t batch, const double* coeffs, double* grids, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn) || !valid01(sp) || !valid01(layout)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention/layout");
    if (grid_order > kMaxOrder || exp_order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const long long rpairs = coeff_pairs(2, (long long)exp_order);
    const size_t gn = batch * zest_gpu_st_grid_size(grid_order, layout), cn = batch * 2 * size_t(rpairs);
    if ((gn && !grids) || (cn && !coeffs)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    const int Lm = int(std::min(exp_order, grid_order));
    return with_staging(ctx, mem, coeffs, cn, grids, gn, [&](const double* in, double* out) {
        ZG_TRY(ctx->adj0.ensure((size_t)batch * 2 * tri_size(Lm) * sizeof(double) + 16));
        ZG_TRY(launch_rows_to_triangle(ctx->stream, Lm, rpairs, int(batch), in, ctx->adj0.as<double>()));
        return st_backward_dev(ctx, sn, sp, layout, Lm, int(grid_order), int(batch), ctx->adj0.as<double>(), out);
    });
}

// The constants of the reference's conversions, computed as it computes
// them: st::conversion_const (include/sh_conventions.hpp:70-96) and the
// complex factor 1/sqrt(2) or sqrt(2) (include/real_sh_expansion.hpp:349, 400).
static double sh_conversion_const(int from, int to) {
    if (from == to) return 1.0;
    const double inv_sqrt_4pi = 0.5 * 0.564189583547756286948079451560772586;  // 0.5 / sqrt(pi)
    const double sqrt_4pi = 1.0 / inv_sqrt_4pi;
    double norm = from == ZEST_SH_QM ? 1.0 : sqrt_4pi;
    norm *= to == ZEST_SH_QM ? 1.0 : inv_sqrt_4pi;
    return norm;
}

int zest_gpu_convert_expansion(zest_gpu_context* ctx, int kind, size_t order, size_t batch, double* coeffs,
                               int src_zn, int src_sn, int src_sp, int dst_zn, int dst_sn, int dst_sp,
                               int to_complex, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (kind != ZEST_EXPANSION_ZERNIKE && kind != ZEST_EXPANSION_SH && kind != ZEST_EXPANSION_ZERNIKE_ROW)
        return fail(ZEST_GPU_ERR_INVALID, "invalid expansion kind");
    if (!valid01(src_zn) || !valid01(src_sn) || !valid01(src_sp) || !valid01(dst_zn) || !valid01(dst_sn) ||
        !valid01(dst_sp) || !valid01(to_complex))
        return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (kind != ZEST_EXPANSION_ZERNIKE && src_zn != dst_zn)
        return fail(ZEST_GPU_ERR_INVALID, "a Zernike normalisation change needs a whole Zernike expansion");
    if (order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    ConvertParams P;
    P.kind = kind == ZEST_EXPANSION_ZERNIKE ? CONVERT_ZERNIKE : kind == ZEST_EXPANSION_SH ? CONVERT_SH : CONVERT_ROWS;
    P.pairs = coeff_pairs(P.kind, (long long)order);
    P.parity = order ? int((order - 1) & 1) : 0;
    P.zconv = src_zn == dst_zn ? 0 : (dst_zn == ZEST_ZERNIKE_NORMED ? -1 : 1);
    P.phase_change = src_sp != dst_sp;
    P.shnorm = sh_conversion_const(src_sn, dst_sn);
    const double sqrt2 = 1.41421356237309504880168872420969808;
    const double cnorm = to_complex ? 1.0 / sqrt2 : sqrt2;
    P.norm = P.shnorm * cnorm;
    const size_t cn = batch * 2 * size_t(P.pairs);
    if (cn && !coeffs) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging(ctx, mem, coeffs, cn, coeffs, cn, [&](const double* in, double* out) {
        if (in != out && cn)
            ZG_CUDA_TRY(cudaMemcpyAsync(out, in, cn * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        return launch_convert(ctx->stream, P, int(batch), out);
    });
}

static int rotate_common(zest_gpu_context* ctx, int kind, size_t order, size_t batch, double* coeffs,
                         const double* angles, int nang, int type, int mem, bool polar) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(type)) return fail(ZEST_GPU_ERR_INVALID, "invalid rotation type");
    if (order > 2048) return fail(ZEST_GPU_ERR_INVALID, "rotation order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t cn = batch * 2 * size_t(coeff_pairs(kind, (long long)order));
    const size_t an = batch * nang;
    if ((cn && !coeffs) || (an && !angles)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    auto run = [&](double* c, const double* a) {
        return polar ? polar_dev(ctx, kind, int(order), int(batch), c, a, type)
                     : rotate_dev(ctx, kind, int(order), int(batch), c, a, type);
    };
    if (mem == ZEST_MEM_DEVICE) return run(coeffs, angles);
    if (mem != ZEST_MEM_HOST) return fail(ZEST_GPU_ERR_INVALID, "mem must be ZEST_MEM_HOST or ZEST_MEM_DEVICE");
    cudaStream_t s = ctx->stream;
    ZG_TRY(ctx->in_stage.ensure(cn * sizeof(double)));
    ZG_TRY(ctx->aux_stage.ensure(an * sizeof(double)));
    if (cn) ZG_CUDA_TRY(cudaMemcpyAsync(ctx->in_stage.p, coeffs, cn * sizeof(double), cudaMemcpyHostToDevice, s));
    if (an) ZG_CUDA_TRY(cudaMemcpyAsync(ctx->aux_stage.p, angles, an * sizeof(double), cudaMemcpyHostToDevice, s));
    ZG_TRY(run(ctx->in_stage.as<double>(), ctx->aux_stage.as<double>()));
    if (cn) ZG_CUDA_TRY(cudaMemcpyAsync(coeffs, ctx->in_stage.p, cn * sizeof(double), cudaMemcpyDeviceToHost, s));
    ZG_CUDA_TRY(cudaStreamSynchronize(s));
    return ZEST_GPU_OK;
}

int zest_gpu_zt_rotate(zest_gpu_context* ctx, size_t order, size_t batch, double* coeffs, const double* euler,
                       int rotation_type, int mem) {
    return rotate_common(ctx, 0, order, batch, coeffs, euler, 3, rotation_type, mem, false);
}
int zest_gpu_st_rotate(zest_gpu_context* ctx, size_t order, size_t batch, double* coeffs, const double* euler,
                       int rotation_type, int mem) {
    return rotate_common(ctx, 1, order, batch, coeffs, euler, 3, rotation_type, mem, false);
}
int zest_gpu_rows_rotate(zest_gpu_context* ctx, size_t order, size_t batch, double* coeffs, const double* euler,
                         int rotation_type, int mem) {
    return rotate_common(ctx, 2, order, batch, coeffs, euler, 3, rotation_type, mem, false);
}
int zest_gpu_zt_polar_rotate(zest_gpu_context* ctx, size_t order, size_t batch, double* coeffs, const double* angles,
                             int rotation_type, int mem) {
    return rotate_common(ctx, 0, order, batch, coeffs, angles, 1, rotation_type, mem, true);
}
int zest_gpu_st_polar_rotate(zest_gpu_context* ctx, size_t order, size_t batch, double* coeffs, const double* angles,
                             int rotation_type, int mem) {
    return rotate_common(ctx, 1, order, batch, coeffs, angles, 1, rotation_type, mem, true);
}

int zest_gpu_set_autotune(zest_gpu_context* ctx, int enable) {
    ZG_TRY(check_ctx(ctx));
    ctx->autotune = enable != 0;
    return ZEST_GPU_OK;
}

// ---- points of the quadrature grids ----------------------------------------------
// BallGLQGridPoints::resize (zernike_glq_transformer.hpp:472-495) and
// SphereGLQGridPoints::resize (sh_glq_transformer.hpp:483-500): longitudes
// dlon * i with dlon = 2 pi / nlon, colatitudes the GL nodes in angle style,
// radii (1 + x) / 2 of the cos-style nodes.  Counts from the layout's shape,
// padding included.
namespace {
void longitudes(size_t nlon, double* lon) {
    const double pi = 3.14159265358979323846264338327950288;
    const double dlon = (2.0 * pi) / double(nlon);
    for (size_t i = 0; i < nlon; ++i) lon[i] = dlon * double(i);
}
}  // namespace

int zest_gpu_zt_grid_points(size_t order, double* lon, double* colat, double* rad) {
    if (order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (order == 0) return ZEST_GPU_OK;
    if (!lon || !colat || !rad) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    const ZtShape sh = zt_shape(long(order));
    longitudes(size_t(sh.nlon), lon);
    gl_colatitudes(long(sh.nlat), colat);
    std::vector<double> w(size_t(sh.nrad));
    gl_nodes_weights(long(sh.nrad), false, rad, w.data());
    for (long k = 0; k < sh.nrad; ++k) rad[k] = 0.5 * (1.0 + rad[k]);
    return ZEST_GPU_OK;
}

int zest_gpu_st_grid_points(size_t order, int layout, double* lon, double* colat) {
    if (order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (layout != ZEST_LAYOUT_LONLAT && layout != ZEST_LAYOUT_LATLON) return fail(ZEST_GPU_ERR_INVALID, "bad layout");
    if (order == 0) return ZEST_GPU_OK;
    if (!lon || !colat) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    const StShape sh = st_shape(long(order), layout == ZEST_LAYOUT_LATLON);
    longitudes(size_t(sh.nlon), lon);
    gl_colatitudes(long(sh.nlat), colat);
    return ZEST_GPU_OK;
}

// ---- evaluation at arbitrary points, power spectra -------------------------------
namespace {

// points of an evaluation: host copies of the caller's arrays (device arrays are
// copied back), since cos/sin of the angles are taken on the host with std::cos
// and std::sin as in the reference (grid_evaluator.hpp:112-113, 251-252).
int points_to_host(int mem, const double* p, size_t n, std::vector<double>& out) {
    out.resize(n);
    if (!n) return ZEST_GPU_OK;
    if (!p) return fail(ZEST_GPU_ERR_INVALID, "null point array");
    if (mem == ZEST_MEM_DEVICE) {
        ZG_CUDA_TRY(cudaMemcpy(out.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
        std::copy(p, p + n, out.begin());
    }
    return ZEST_GPU_OK;
}

int eval_points(int mem, const double* lon, size_t nlon, const double* colat, size_t nlat, std::vector<double>& z,
                std::vector<double>& cs) {
    std::vector<double> a, c;
    ZG_TRY(points_to_host(mem, lon, nlon, a));
    ZG_TRY(points_to_host(mem, colat, nlat, c));
    z.resize(nlat);
    for (size_t j = 0; j < nlat; ++j) z[j] = std::cos(c[j]);
    cs.resize(2 * nlon);
    for (size_t i = 0; i < nlon; ++i) {
        cs[2 * i] = std::cos(a[i]);
        cs[2 * i + 1] = std::sin(a[i]);
    }
    return ZEST_GPU_OK;
}

}  // namespace

int zest_gpu_zt_evaluate(zest_gpu_context* ctx, int zn, int sn, int sp, size_t order, size_t batch,
                         const double* coeffs, size_t nlon, const double* lon, size_t nlat, const double* colat,
                         size_t nrad, const double* rad, double* values, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(zn) || !valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    if (nlon > 0x7fffffff || nlat > 0x7fffffff || nrad > 0x7fffffff || nlat * nrad > 0x7fffffff)
        return fail(ZEST_GPU_ERR_INVALID, "too many points");
    if (mem != ZEST_MEM_HOST && mem != ZEST_MEM_DEVICE)
        return fail(ZEST_GPU_ERR_INVALID, "mem must be ZEST_MEM_HOST or ZEST_MEM_DEVICE");
    const size_t cn = batch * 2 * zest_gpu_zt_coeff_size(order), vn = batch * nlon * nlat * nrad;
    if ((cn && !coeffs) || (vn && !values)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    if (vn == 0) return ZEST_GPU_OK;
    std::vector<double> z, cs, r;
    ZG_TRY(eval_points(mem, lon, nlon, colat, nlat, z, cs));
    ZG_TRY(points_to_host(mem, rad, nrad, r));
    return with_staging(ctx, mem, coeffs, cn, values, vn, [&](const double* in, double* out) {
        return zt_evaluate_dev(ctx, zn, sn, sp, int(order), int(batch), in, z, cs, r, out);
    });
}

int zest_gpu_st_evaluate(zest_gpu_context* ctx, int sn, int sp, size_t order, size_t batch, const double* coeffs,
                         size_t nlon, const double* lon, size_t nlat, const double* colat, double* values, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    if (nlon > 0x7fffffff || nlat > 0x7fffffff) return fail(ZEST_GPU_ERR_INVALID, "too many points");
    if (mem != ZEST_MEM_HOST && mem != ZEST_MEM_DEVICE)
        return fail(ZEST_GPU_ERR_INVALID, "mem must be ZEST_MEM_HOST or ZEST_MEM_DEVICE");
    const size_t cn = batch * 2 * zest_gpu_st_coeff_size(order), vn = batch * nlon * nlat;
    if ((cn && !coeffs) || (vn && !values)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    if (vn == 0) return ZEST_GPU_OK;
    std::vector<double> z, cs;
    ZG_TRY(eval_points(mem, lon, nlon, colat, nlat, z, cs));
    return with_staging(ctx, mem, coeffs, cn, values, vn, [&](const double* in, double* out) {
        return st_evaluate_dev(ctx, sn, sp, int(order), int(batch), in, z, cs, out);
    });
}

// st::LSQTransformer::transform (lsq_transformer.hpp:57-110): data at
// (latitude, longitude) points; zt::LSQTransformer::transform
// (lsq_transformer.hpp:119-187): data at (r, longitude, colatitude) points.
int zest_gpu_st_lsq(zest_gpu_context* ctx, int sn, int sp, size_t order, size_t npoints, size_t batch,
                    const double* data, const double* lat, const double* lon, double* coeffs, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (order > 4096) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535 || npoints > 0x7fffffff) return fail(ZEST_GPU_ERR_INVALID, "too many points or items");
    if (mem != ZEST_MEM_HOST && mem != ZEST_MEM_DEVICE)
        return fail(ZEST_GPU_ERR_INVALID, "mem must be ZEST_MEM_HOST or ZEST_MEM_DEVICE");
    const size_t dn = batch * npoints, cn = batch * 2 * zest_gpu_st_coeff_size(order);
    if ((dn && !data) || (cn && !coeffs)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    if (cn == 0) return ZEST_GPU_OK;
    std::vector<double> la, lo, z;
    ZG_TRY(points_to_host(mem, lat, npoints, la));
    ZG_TRY(points_to_host(mem, lon, npoints, lo));
    z.resize(npoints);
    for (size_t i = 0; i < npoints; ++i) z[i] = std::sin(la[i]);
    return with_staging(ctx, mem, data, dn, coeffs, cn, [&](const double* in, double* out) {
        return lsq_dev(ctx, 1, 0, sn, sp, int(order), int(npoints), int(batch), in, z, lo, std::vector<double>(), out);
    });
}

int zest_gpu_zt_lsq(zest_gpu_context* ctx, int zn, int sn, int sp, size_t order, size_t npoints, size_t batch,
                    const double* data, const double* r, const double* lon, const double* colat, double* coeffs,
                    int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(zn) || !valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (order > 1024) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535 || npoints > 0x7fffffff) return fail(ZEST_GPU_ERR_INVALID, "too many points or items");
    if (mem != ZEST_MEM_HOST && mem != ZEST_MEM_DEVICE)
        return fail(ZEST_GPU_ERR_INVALID, "mem must be ZEST_MEM_HOST or ZEST_MEM_DEVICE");
    const size_t dn = batch * npoints, cn = batch * 2 * zest_gpu_zt_coeff_size(order);
    if ((dn && !data) || (cn && !coeffs)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    if (cn == 0) return ZEST_GPU_OK;
    std::vector<double> rr, lo, co, z;
    ZG_TRY(points_to_host(mem, r, npoints, rr));
    ZG_TRY(points_to_host(mem, lon, npoints, lo));
    ZG_TRY(points_to_host(mem, colat, npoints, co));
    z.resize(npoints);
    for (size_t i = 0; i < npoints; ++i) z[i] = std::cos(co[i]);
    return with_staging(ctx, mem, data, dn, coeffs, cn, [&](const double* in, double* out) {
        return lsq_dev(ctx, 0, zn, sn, sp, int(order), int(npoints), int(batch), in, z, lo, rr, out);
    });
}

int zest_gpu_st_power_spectrum(zest_gpu_context* ctx, int sn, size_t order, size_t batch, const double* coeffs,
                               double* out, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t cn = batch * 2 * zest_gpu_st_coeff_size(order), on = batch * order;
    if ((cn && !coeffs) || (on && !out)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    if (on == 0) return ZEST_GPU_OK;
    return with_staging(ctx, mem, coeffs, cn, out, on, [&](const double* in, double* o) {
        return st_spectrum_dev(ctx, sn, int(order), int(batch), in, in, int(order), (long long)order, o);
    });
}

int zest_gpu_st_cross_power_spectrum(zest_gpu_context* ctx, int sn, size_t order, size_t batch, const double* a,
                                     const double* b, size_t out_len, double* out, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (order > kMaxOrder || out_len > kMaxOrder + 1) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t cn = batch * 2 * zest_gpu_st_coeff_size(order), on = batch * out_len;
    if ((cn && (!a || !b)) || (on && !out)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    // entries l < min(order, out_len - 1) are written (power_spectra.hpp:42-43)
    const size_t nl = out_len ? std::min(order, out_len - 1) : 0;
    if (on == 0 || nl == 0) return ZEST_GPU_OK;
    const double* bd = b;
    if (mem == ZEST_MEM_HOST) {
        ZG_TRY(ctx->aux_stage.ensure(cn * sizeof(double)));
        StageScope sc(ctx, ST_COPY_H2D);
        ZG_CUDA_TRY(cudaMemcpyAsync(ctx->aux_stage.p, b, cn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        bd = ctx->aux_stage.as<double>();
    }
    return with_staging(
        ctx, mem, a, cn, out, on,
        [&](const double* in, double* o) {
            return st_spectrum_dev(ctx, sn, int(order), int(batch), in, bd, int(nl), (long long)out_len, o);
        },
        out_len, nl);
}

int zest_gpu_zt_power_spectrum(zest_gpu_context* ctx, int sn, size_t order, size_t batch, const double* coeffs,
                               double* out, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t nidx = ((order + 1) * (order + 1)) >> 2;
    const size_t cn = batch * 2 * zest_gpu_zt_coeff_size(order), on = batch * nidx;
    if ((cn && !coeffs) || (on && !out)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    if (on == 0) return ZEST_GPU_OK;
    if (mem == ZEST_MEM_HOST) {
        // the entries the reference leaves alone (l = n) keep the caller's values
        ZG_TRY(ctx->out_stage.ensure(on * sizeof(double)));
        ZG_CUDA_TRY(cudaMemcpyAsync(ctx->out_stage.p, out, on * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    }
    return with_staging(ctx, mem, coeffs, cn, out, on, [&](const double* in, double* o) {
        return zt_spectrum_dev(ctx, sn, int(order), int(batch), in, o);
    });
}

int zest_gpu_selftest_wait_timeout(zest_gpu_context* ctx, double seconds) {
    ZG_TRY(check_ctx(ctx));
    if (!(seconds >= 1e-3 && seconds <= 2.0)) return fail(ZEST_GPU_ERR_INVALID, "wait limit outside [1 ms, 2 s]");
    return split_wait_selftest(ctx, (long long)(seconds * 1e9));
}

int zest_gpu_set_host_chunk_bytes(zest_gpu_context* ctx, size_t bytes) {
    ZG_TRY(check_ctx(ctx));
    ctx->host_chunk_bytes = bytes;
    return ZEST_GPU_OK;
}

int zest_gpu_host_register(void* ptr, size_t bytes) {
    if (!ptr || bytes == 0) return fail(ZEST_GPU_ERR_INVALID, "host register: null pointer or zero bytes");
    ZG_CUDA_TRY(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
    return ZEST_GPU_OK;
}

int zest_gpu_host_unregister(void* ptr) {
    if (!ptr) return fail(ZEST_GPU_ERR_INVALID, "host unregister: null pointer");
    ZG_CUDA_TRY(cudaHostUnregister(ptr));
    return ZEST_GPU_OK;
}

int zest_gpu_zt_rotate_backward_ragged(zest_gpu_context* ctx, int zn, int sn, int sp, size_t n_items,
                                       const int* orders, double* coeffs, const double* euler, int rotation_type,
                                       double* grids) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(zn) || !valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (!valid01(rotation_type)) return fail(ZEST_GPU_ERR_INVALID, "invalid rotation type");
    if (n_items == 0) return ZEST_GPU_OK;
    if (n_items > 65535) return fail(ZEST_GPU_ERR_INVALID, "too many expansions (max 65535)");
    if (!orders || !coeffs || !euler || !grids) return fail(ZEST_GPU_ERR_INVALID, "null pointer");
    std::vector<int> ord(orders, orders + n_items);
    for (size_t i = 0; i < n_items; ++i) {
        if (ord[i] < 1 || ord[i] > 2048) return fail(ZEST_GPU_ERR_INVALID, "orders must be in 1..2048");
        if (i && ord[i] < ord[i - 1]) return fail(ZEST_GPU_ERR_INVALID, "orders must be non-decreasing");
    }
    return zt_rotate_backward_ragged_dev(ctx, zn, sn, sp, ord, coeffs, euler, rotation_type, grids);
}

// ---- adjoints ----
int zest_gpu_zt_forward_vjp(zest_gpu_context* ctx, int zn, int sn, int sp, size_t grid_order, size_t exp_order,
                            size_t batch, const double* coeffs_cot, double* grids_cot, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(zn) || !valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (grid_order > kMaxOrder || exp_order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t gn = batch * zest_gpu_zt_grid_size(grid_order), cn = batch * 2 * zest_gpu_zt_coeff_size(exp_order);
    if ((gn && !grids_cot) || (cn && !coeffs_cot)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging(ctx, mem, coeffs_cot, cn, grids_cot, gn, [&](const double* in, double* out) {
        return zt_forward_vjp_dev(ctx, zn, sn, sp, int(grid_order), int(exp_order), int(batch), in, out);
    });
}

int zest_gpu_zt_backward_vjp(zest_gpu_context* ctx, int zn, int sn, int sp, size_t exp_order, size_t grid_order,
                             size_t batch, const double* grids_cot, double* coeffs_cot, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(zn) || !valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (grid_order > kMaxOrder || exp_order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t gn = batch * zest_gpu_zt_grid_size(grid_order), cn = batch * 2 * zest_gpu_zt_coeff_size(exp_order);
    if ((gn && !grids_cot) || (cn && !coeffs_cot)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging(ctx, mem, grids_cot, gn, coeffs_cot, cn, [&](const double* in, double* out) {
        return zt_backward_vjp_dev(ctx, zn, sn, sp, int(exp_order), int(grid_order), int(batch), in, out);
    });
}

int zest_gpu_st_forward_vjp(zest_gpu_context* ctx, int sn, int sp, int layout, size_t grid_order, size_t exp_order,
                            size_t batch, const double* coeffs_cot, double* grids_cot, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn) || !valid01(sp) || !valid01(layout)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention/layout");
    if (grid_order > kMaxOrder || exp_order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t gn = batch * zest_gpu_st_grid_size(grid_order, layout), cn = batch * 2 * zest_gpu_st_coeff_size(exp_order);
    if ((gn && !grids_cot) || (cn && !coeffs_cot)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging(ctx, mem, coeffs_cot, cn, grids_cot, gn, [&](const double* in, double* out) {
        return st_forward_vjp_dev(ctx, sn, sp, layout, int(grid_order), int(exp_order), int(batch), in, out);
    });
}

int zest_gpu_st_backward_vjp(zest_gpu_context* ctx, int sn, int sp, int layout, size_t exp_order, size_t grid_order,
                             size_t batch, const double* grids_cot, double* coeffs_cot, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn) || !valid01(sp) || !valid01(layout)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention/layout");
    if (grid_order > kMaxOrder || exp_order > kMaxOrder) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t gn = batch * zest_gpu_st_grid_size(grid_order, layout), cn = batch * 2 * zest_gpu_st_coeff_size(exp_order);
    if ((gn && !grids_cot) || (cn && !coeffs_cot)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging(ctx, mem, grids_cot, gn, coeffs_cot, cn, [&](const double* in, double* out) {
        return st_backward_vjp_dev(ctx, sn, sp, layout, int(exp_order), int(grid_order), int(batch), in, out);
    });
}

static int rotate_vjp_common(zest_gpu_context* ctx, int kind, size_t order, size_t batch, const double* coeffs,
                             const double* euler, int type, const double* out_cot, double* coeffs_cot,
                             double* euler_cot, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(type)) return fail(ZEST_GPU_ERR_INVALID, "invalid rotation type");
    if (order > 2048) return fail(ZEST_GPU_ERR_INVALID, "rotation order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const size_t cn = batch * 2 * (kind == 0 ? zest_gpu_zt_coeff_size(order) : zest_gpu_st_coeff_size(order));
    const size_t an = batch * 3;
    if (!coeffs_cot && !euler_cot) return ZEST_GPU_OK;
    if ((cn && !out_cot) || (an && !euler) || (euler_cot && cn && !coeffs))
        return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    auto run = [&](const double* x, const double* e, const double* yb, double* xb, double* eb) {
        return rotate_vjp_dev(ctx, kind, int(order), int(batch), x, e, type, yb, xb, eb);
    };
    if (mem == ZEST_MEM_DEVICE) return run(coeffs, euler, out_cot, coeffs_cot, euler_cot);
    if (mem != ZEST_MEM_HOST) return fail(ZEST_GPU_ERR_INVALID, "mem must be ZEST_MEM_HOST or ZEST_MEM_DEVICE");
    // staging: in_stage = [x | ybar], aux_stage = [euler | ebar], out_stage = xbar
    cudaStream_t s = ctx->stream;
    ZG_TRY(ctx->in_stage.ensure(2 * cn * sizeof(double) + 16));
    ZG_TRY(ctx->aux_stage.ensure(2 * an * sizeof(double) + 16));
    ZG_TRY(ctx->out_stage.ensure(cn * sizeof(double) + 16));
    double* dx = ctx->in_stage.as<double>();
    double* dy = dx + cn;
    double* de = ctx->aux_stage.as<double>();
    double* deb = de + an;
    double* dxb = ctx->out_stage.as<double>();
    if (cn && euler_cot) ZG_CUDA_TRY(cudaMemcpyAsync(dx, coeffs, cn * sizeof(double), cudaMemcpyHostToDevice, s));
    if (cn) ZG_CUDA_TRY(cudaMemcpyAsync(dy, out_cot, cn * sizeof(double), cudaMemcpyHostToDevice, s));
    if (an) ZG_CUDA_TRY(cudaMemcpyAsync(de, euler, an * sizeof(double), cudaMemcpyHostToDevice, s));
    ZG_TRY(run(dx, de, dy, coeffs_cot ? dxb : nullptr, euler_cot ? deb : nullptr));
    if (coeffs_cot && cn) ZG_CUDA_TRY(cudaMemcpyAsync(coeffs_cot, dxb, cn * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (euler_cot && an) ZG_CUDA_TRY(cudaMemcpyAsync(euler_cot, deb, an * sizeof(double), cudaMemcpyDeviceToHost, s));
    ZG_CUDA_TRY(cudaStreamSynchronize(s));
    return ZEST_GPU_OK;
}

int zest_gpu_zt_rotate_vjp(zest_gpu_context* ctx, size_t order, size_t batch, const double* coeffs,
                           const double* euler, int rotation_type, const double* out_cot, double* coeffs_cot,
                           double* euler_cot, int mem) {
    return rotate_vjp_common(ctx, 0, order, batch, coeffs, euler, rotation_type, out_cot, coeffs_cot, euler_cot, mem);
}

int zest_gpu_st_rotate_vjp(zest_gpu_context* ctx, size_t order, size_t batch, const double* coeffs,
                           const double* euler, int rotation_type, const double* out_cot, double* coeffs_cot,
                           double* euler_cot, int mem) {
    return rotate_vjp_common(ctx, 1, order, batch, coeffs, euler, rotation_type, out_cot, coeffs_cot, euler_cot, mem);
}

int zest_gpu_split_gemm(zest_gpu_context* ctx, size_t M, size_t N, size_t K, const double* A, const double* B,
                        double* C, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (M > (1u << 24) || N > (1u << 20) || K > 2048) return fail(ZEST_GPU_ERR_INVALID, "split GEMM size out of range");
    if ((M * K && !A) || (N * K && !B) || (M * N && !C)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    if (M == 0 || N == 0) return ZEST_GPU_OK;
    if (mem == ZEST_MEM_DEVICE) return split_dense_gemm(ctx, int(M), int(N), int(K), A, B, C);
    if (mem != ZEST_MEM_HOST) return fail(ZEST_GPU_ERR_INVALID, "mem must be ZEST_MEM_HOST or ZEST_MEM_DEVICE");
    cudaStream_t s = ctx->stream;
    ZG_TRY(ctx->in_stage.ensure(M * K * sizeof(double)));
    ZG_TRY(ctx->aux_stage.ensure(N * K * sizeof(double)));
    ZG_TRY(ctx->out_stage.ensure(M * N * sizeof(double)));
    ZG_CUDA_TRY(cudaMemcpyAsync(ctx->in_stage.p, A, M * K * sizeof(double), cudaMemcpyHostToDevice, s));
    ZG_CUDA_TRY(cudaMemcpyAsync(ctx->aux_stage.p, B, N * K * sizeof(double), cudaMemcpyHostToDevice, s));
    ZG_TRY(split_dense_gemm(ctx, int(M), int(N), int(K), ctx->in_stage.as<double>(), ctx->aux_stage.as<double>(),
                            ctx->out_stage.as<double>()));
    ZG_CUDA_TRY(cudaMemcpyAsync(C, ctx->out_stage.p, M * N * sizeof(double), cudaMemcpyDeviceToHost, s));
    ZG_CUDA_TRY(cudaStreamSynchronize(s));
    return ZEST_GPU_OK;
}

int zest_gpu_euler_from_matrix(const double* r, double* e) {
    if (!r || !e) return fail(ZEST_GPU_ERR_INVALID, "null pointer");
    // euler_angles_from_rotation_matrix, include/rotor.hpp:53-63 (as written there)
    const double r22sq = r[8] * r[8];
    const double by = std::sqrt((1.0 + r22sq) * (1.0 - r22sq));
    e[0] = std::atan2(r[5], r[2]);
    e[1] = std::atan2(by, r[8]);
    e[2] = std::atan2(r[7], -r[6]);
    return ZEST_GPU_OK;
}

int zest_gpu_gl_nodes_weights(size_t n, int packed, double* nodes, double* weights) {
    if (n > (1u << 20)) return fail(ZEST_GPU_ERR_INVALID, "too many nodes");
    if (n && (!nodes || !weights)) return fail(ZEST_GPU_ERR_INVALID, "null pointer");
    gl_nodes_weights(long(n), packed != 0, nodes, weights);
    return ZEST_GPU_OK;
}

int zest_gpu_plm_table(zest_gpu_context* ctx, size_t order, int sn, int sp, size_t nz, const double* z, double* out,
                       int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (order > kMaxOrder || nz > (1u << 20)) return fail(ZEST_GPU_ERR_INVALID, "size too large");
    const size_t on = (size_t)tri_size((long long)order) * nz;
    if ((nz && !z) || (on && !out)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging(ctx, mem, z, nz, out, on, [&](const double* zi, double* o) {
        return launch_plm_ref(ctx->stream, int(order), sn, sp, int(nz), zi, o);
    });
}

int zest_gpu_plm_complex_table(zest_gpu_context* ctx, size_t order, int sn, int sp, size_t nz, const double* z,
                               double* out, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(sn) || !valid01(sp)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (order > kMaxOrder || nz > (1u << 20)) return fail(ZEST_GPU_ERR_INVALID, "size too large");
    const size_t on = (size_t)tri_size((long long)order) * nz;
    if ((nz && !z) || (on && !out)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging(ctx, mem, z, nz, out, on, [&](const double* zi, double* o) {
        return launch_plm_ref(ctx->stream, int(order), sn, sp, int(nz), zi, o, true);
    });
}

int zest_gpu_radial_table(zest_gpu_context* ctx, size_t order, int zn, size_t nr, const double* r, double* out,
                          int mem) {
    ZG_TRY(check_ctx(ctx));
    if (!valid01(zn)) return fail(ZEST_GPU_ERR_INVALID, "invalid convention");
    if (order > kMaxOrder || nr > (1u << 20)) return fail(ZEST_GPU_ERR_INVALID, "size too large");
    const size_t on = (size_t)((((long long)order + 1) * ((long long)order + 1)) >> 2) * nr;
    if ((nr && !r) || (on && !out)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging(ctx, mem, r, nr, out, on, [&](const double* ri, double* o) {
        return launch_radial_ref(ctx->stream, int(order), zn, int(nr), ri, o);
    });
}

int zest_gpu_wignerd_table(zest_gpu_context* ctx, size_t order, double* out, int mem) {
    ZG_TRY(check_ctx(ctx));
    if (order > 2048) return fail(ZEST_GPU_ERR_INVALID, "order too large");
    const size_t on = (size_t)wig_off((long long)order);
    if (on && !out) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    return with_staging(ctx, mem, nullptr, 0, out, on, [&](const double*, double* o) {
        return launch_wignerd(ctx->stream, int(order), o);
    });
}

}  // extern "C"
