// FP64 tables of the GLQ path, generated on the device:
//   * normalised associated Legendre functions  P_lm(z)
//       (st::PlmRecursion::plm_real, include/plm_recursion.hpp:229-354,
//        coefficients src/plm_recursion.cpp:31-55)
//   * radial 3D Zernike polynomials R_nl(r)
//       (zt::RadialZernikeRecursion::zernike, include/radial_zernike_recursion.hpp:151-288,
//        coefficients src/radial_zernike_recursion.cpp:31-56)
//   * Wigner small-d matrices at pi/2
//       (WignerdPiHalfCollection, src/wignerd_collection.cpp:29-98)
// and the Gauss-Legendre nodes/weights, solved on the host in double-double.
//
// The recursions use explicitly rounded operations (__dmul_rn, __dadd_rn, ...)
// in the reference's order of evaluation, so the tables are bit-identical to
// the reference's (sqrt and division are correctly rounded on both sides).
#include <cmath>
#include <vector>

#include "common.cuh"
#include "tables.cuh"

namespace zgpu {

// ---------------------------------------------------------------------------
// Gauss-Legendre nodes/weights: Newton's method on the Legendre three-term
// recurrence, in double-double arithmetic (Dekker/Knuth error-free
// transformations), so nodes near +-1 keep full relative accuracy in their
// weights.  Layouts as include/gauss_legendre.hpp:32-66: unpacked ascending
// from -1; packed = the ceil(n/2) non-negative nodes ascending from 0.
namespace {
struct DD {
    double hi, lo;
};
inline DD two_sum(double a, double b) {
    volatile double s = a + b;
    volatile double bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
inline DD fast_two_sum(double a, double b) {
    volatile double s = a + b;
    return {s, b - (s - a)};
}
inline void split(double a, double& hi, double& lo) {
    volatile double c = 134217729.0 * a;
    volatile double t = c - a;
    hi = c - t;
    lo = a - hi;
}
inline DD two_prod(double a, double b) {
    volatile double p = a * b;
    double ah, al, bh, bl;
    split(a, ah, al);
    split(b, bh, bl);
    volatile double t1 = ah * bh - p;
    volatile double t2 = t1 + ah * bl;
    volatile double t3 = t2 + al * bh;
    return {p, t3 + al * bl};
}
inline DD add(DD x, DD y) {
    DD s = two_sum(x.hi, y.hi);
    return fast_two_sum(s.hi, s.lo + x.lo + y.lo);
}
inline DD neg(DD x) { return {-x.hi, -x.lo}; }
inline DD mul(DD x, DD y) {
    DD p = two_prod(x.hi, y.hi);
    return fast_two_sum(p.hi, p.lo + (x.hi * y.lo + x.lo * y.hi));
}
inline DD mul_d(DD x, double d) {
    DD p = two_prod(x.hi, d);
    return fast_two_sum(p.hi, p.lo + x.lo * d);
}
inline DD div(DD x, DD y) {
    double q1 = x.hi / y.hi;
    DD r = add(x, neg(mul_d(y, q1)));
    double q2 = r.hi / y.hi;
    r = add(r, neg(mul_d(y, q2)));
    double q3 = r.hi / y.hi;
    return add(fast_two_sum(q1, q2), DD{q3, 0.0});
}
inline DD dd(double a) { return {a, 0.0}; }

void legendre_pair(long n, DD x, DD& pn, DD& pnm1) {
    DD p0 = dd(1.0), p1 = x;
    if (n == 0) {
        pn = p0;
        pnm1 = dd(0.0);
        return;
    }
    for (long k = 2; k <= n; ++k) {
        DD t = add(mul_d(mul(x, p1), double(2 * k - 1)), neg(mul_d(p0, double(k - 1))));
        DD p2 = div(t, dd(double(k)));
        p0 = p1;
        p1 = p2;
    }
    pn = p1;
    pnm1 = p0;
}

// k-th node counted from +1 (k = 1 .. ceil(n/2)) in double-double
DD node_dd(long n, long k);

// k-th node counted from +1 (k = 1 .. ceil(n/2)) and its weight
void node_weight(long n, long k, double& node, double& weight) {
    const DD x = node_dd(n, k);
    DD pn, pnm1;
    legendre_pair(n, x, pn, pnm1);
    DD omx2 = mul(add(dd(1.0), neg(x)), add(dd(1.0), x));
    DD np = mul_d(pnm1, double(n));
    DD w = div(mul_d(omx2, 2.0), mul(np, np));
    node = x.hi + x.lo;
    weight = w.hi + w.lo;
}
DD node_dd(long n, long k) {
    const double pi = 3.14159265358979323846264338327950288;
    DD x;
    if ((n & 1) && k == (n + 1) / 2) return dd(0.0);
    const double theta = pi * (double(k) - 0.25) / (double(n) + 0.5);
    x = dd(std::cos(theta + 1.0 / (8.0 * double(n) * double(n) * std::tan(theta))));
    for (int it = 0; it < 60; ++it) {
        DD pn, pnm1;
        legendre_pair(n, x, pn, pnm1);
        DD omx2 = mul(add(dd(1.0), neg(x)), add(dd(1.0), x));
        DD dp = div(mul_d(add(pnm1, neg(mul(x, pn))), double(n)), omx2);
        DD dx = div(pn, dp);
        x = add(x, neg(dx));
        if (std::fabs(dx.hi) < 1e-30 * (std::fabs(x.hi) + 1e-300) || dx.hi == 0.0) break;
    }
    return x;
}

// arccos of a double-double cosine: acos(hi) corrected to first order in lo
double acos_dd(DD x) {
    if (x.hi == 0.0 && x.lo == 0.0) return std::acos(0.0);
    return std::acos(x.hi) - x.lo / std::sqrt((1.0 - x.hi) * (1.0 + x.hi));
}
}  // namespace

void gl_colatitudes(long n, double* theta) {
    const long nu = (n + 1) >> 1;
    for (long k = 1; k <= nu; ++k) {
        const DD x = node_dd(n, k);
        theta[k - 1] = acos_dd(neg(x));
        theta[n - k] = acos_dd(x);
    }
}

void gl_nodes_weights(long n, bool packed, double* nodes, double* weights) {
    const long nu = (n + 1) >> 1;
    for (long k = 1; k <= nu; ++k) {
        double x, w;
        node_weight(n, k, x, w);
        if (packed) {
            nodes[nu - k] = x;
            weights[nu - k] = w;
        } else {
            nodes[k - 1] = -x;
            weights[k - 1] = w;
            nodes[n - k] = x;  // the middle node of an odd rule stays +0
            weights[n - k] = w;
        }
    }
}

// ---------------------------------------------------------------------------
// P_lm recursion.  One thread per (m, node).  The writer decides where each
// P_lm(z_i) lands (reference vector layout, or a GEMM operand layout).
namespace {
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double sq(int l) { return __dsqrt_rn(double(l)); }

// cnorm: sqrt(2) for the real basis (plm_real), 1 for plm_complex
// (plm_recursion.hpp:96-139); it enters the recursion where the reference's
// complex_norm does (the m > 0 start value).
template <class Writer>
__global__ void plm_kernel(int L, int sh_norm, int sh_phase, int nz, const double* __restrict__ z, Writer w,
                           double cnorm = 1.41421356237309504880168872420969808) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y;
    if (i >= nz || m >= L) return;
    const double inv_sqrt_4pi = 0.28209479177387814347403972578038629;
    const double uc = 1.0e-280;
    const double phase = sh_phase ? 1.0 : -1.0;
    const double zi = z[i];
    if (m == 0) {
        const double p00 = sh_norm ? inv_sqrt_4pi : 1.0;
        w(0, 0, i, p00);
        if (L == 1) return;
        const double p10 = sh_norm ? mul(zi, mul(sq(3), inv_sqrt_4pi)) : mul(zi, sq(3));
        w(1, 0, i, p10);
        double p2 = p00, p1 = p10;
        for (int l = 2; l < L; ++l) {
            // a(l,0) = sqrt(2l-1) sqrt(2l+1) / l ; b(l,0) = (l-1) sqrt(2l+1) / (sqrt(2l-3) l)
            const double a = dv(mul(sq(2 * l - 1), sq(2 * l + 1)), double(l));
            const double b = dv(mul(double(l) - 1.0, sq(2 * l + 1)), mul(sq(2 * l - 3), double(l)));
            const double p = sub(mul(mul(a, zi), p1), mul(b, p2));
            w(l, 0, i, p);
            p2 = p1;
            p1 = p;
        }
        return;
    }
    const double u = __dsqrt_rn(mul(sub(1.0, zi), 1.0 + zi));
    double pmm = sh_norm ? mul(mul(uc, cnorm), inv_sqrt_4pi) : mul(uc, cnorm);
    double us = dv(1.0, uc);
    const int mlast = (m < L - 1) ? m : L - 2;
    for (int k = 1; k <= mlast; ++k) {
        us = mul(us, u);
        pmm = mul(pmm, dv(mul(phase, sq(2 * k + 1)), sq(2 * k)));
    }
    if (m == L - 1) {
        us = mul(us, u);
        const double v = mul(us, dv(mul(mul(phase, pmm), sq(2 * L - 1)), sq(2 * L - 2)));
        w(L - 1, L - 1, i, v);
        return;
    }
    // unscaled recursion, then multiplication by u^m (us = 1e280 u^m)
    w(m, m, i, mul(pmm, us));
    double p2 = pmm;
    double p1 = mul(zi, mul(sq(2 * m + 3), pmm));
    for (int l = m + 2; l < L; ++l) {
        // a(l,m) = sqrt(2l-1)sqrt(2l+1)/(sqrt(l-m)sqrt(l+m))
        // b(l,m) = sqrt(2l+1)sqrt(l+m-1)sqrt(l-m-1)/(sqrt(l-m)sqrt(l+m)sqrt(2l-3))
        const double a = dv(mul(sq(2 * l - 1), sq(2 * l + 1)), mul(sq(l - m), sq(l + m)));
        const double b = dv(mul(mul(sq(2 * l + 1), sq(l + m - 1)), sq(l - m - 1)),
                            mul(mul(sq(l - m), sq(l + m)), sq(2 * l - 3)));
        const double p = sub(mul(mul(zi, a), p1), mul(b, p2));
        w(l - 1, m, i, mul(p1, us));
        p2 = p1;
        p1 = p;
    }
    w(L - 1, m, i, mul(p1, us));
}

struct PlmRefWriter {  // out[idx(l,m) * nz + i]
    double* out;
    int nz;
    __device__ void operator()(int l, int m, int i, double v) const { out[tri_idx(l, m) * nz + i] = v; }
};

// GEMM operand layout of the folded Legendre tables: row (m, p = (l-m)&1,
// r = (l-m)>>1) at off[2m+p] + r, ld columns (one per folded node i); the
// value is P_lm(z_i) * scale[i] * (m>0 ? mscale : 1).
struct PlmGemmWriter {
    double* out;
    const long long* off;
    const double* scale;
    int ld;
    double mscale;
    int Lrows;  // only rows with l < Lrows are stored
    __device__ void operator()(int l, int m, int i, double v) const {
        if (l >= Lrows) return;
        const int p = (l - m) & 1;
        const long long row = off[2 * m + p] + ((l - m) >> 1);
        double s = scale ? scale[i] : 1.0;
        if (m > 0) s *= mscale;
        out[row * ld + i] = v * s;
    }
};

// ---------------------------------------------------------------------------
// Radial Zernike recursion.  One thread per (l, node): the sequence
// n = l, l+2, ... of the reference's recursion in n (the values it needs from
// other l -- r^n and R_22 = r^2 -- are recomputed in place).
template <class Writer>
__global__ void radial_kernel(int L, int zernike_norm, int nr, const double* __restrict__ r, Writer w) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int l = blockIdx.y;
    if (k >= nr || l >= L) return;
    const double rk = r[k];
    const double r22 = mul(rk, rk);
    auto emit = [&](int n, double v) {
        if (zernike_norm == 0) v = mul(v, __dsqrt_rn(2.0 * double(n) + 3.0));
        w(n, l, k, v);
    };
    // r^n by repeated multiplication: R_00 = 1, R_11 = r, R_22 = r r, R_nn = r R_{n-1,n-1}
    auto rpow = [&](int n) {
        if (n == 0) return 1.0;
        double p = rk;
        for (int j = 2; j <= n; ++j) p = (j == 2) ? r22 : mul(rk, p);
        return p;
    };
    double rll = rpow(l);
    emit(l, rll);
    if (l + 2 >= L) return;
    double rl2;  // R_{l+2, l}
    if (l == 0) rl2 = sub(mul(2.5, r22), 1.5);
    else if (l == 1) rl2 = mul(sub(mul(3.5, r22), 2.5), rk);
    else {
        const double rnn = (l + 2 == 3) ? mul(r22, rk) : mul(rk, mul(rk, rll));
        const double dn = double(l + 2);
        rl2 = sub(mul(dn + 0.5, rnn), mul(dn - 0.5, rll));
    }
    emit(l + 2, rl2);
    double rm4 = rll, rm2 = rl2;
    for (int n = l + 4; n < L; n += 2) {
        const double dn = double(n), dl = double(l);
        const double k0 = mul(mul(sub(dn, dl), dn + dl + 1.0), sub(2.0 * dn, 3.0));
        const double k1 = mul(mul(sub(2.0 * dn, 1.0), 2.0 * dn + 1), sub(2.0 * dn, 3.0));
        const double k2 = mul(mul(-0.5, sub(2.0 * dn, 1.0)),
                              __dadd_rn(mul(2 * dl + 1.0, 2.0 * dl + 1.0), mul(2.0 * dn + 1, sub(2.0 * dn, 3.0))));
        const double k3 = mul(-mul(sub(sub(dn, dl), 2.0), sub(dn + dl, 1.0)), 2.0 * dn + 1);
        const double k0i = dv(1.0, k0);
        const double c1 = mul(k1, k0i), c2 = mul(k2, k0i), c3 = mul(k3, k0i);
        const double v = __dadd_rn(mul(__dadd_rn(c2, mul(c1, r22)), rm2), mul(c3, rm4));
        emit(n, v);
        rm4 = rm2;
        rm2 = v;
    }
}

struct RadialRefWriter {  // out[(floor((n+1)^2/4) + l/2) * nr + k]
    double* out;
    int nr;
    __device__ void operator()(int n, int l, int k, double v) const {
        out[(long long)((((n + 1) * (n + 1)) >> 2) + (l >> 1)) * nr + k] = v;
    }
};

// GEMM operand layout of the radial tables: row (l, r = (n-l)/2) at off[l] + r,
// nr columns; value R_nl(r_k) * scale[k] * nscale(n).
struct RadialGemmWriter {
    double* out;
    const long long* off;
    const double* scale;
    int nr;
    int Lrows;
    int unnormed_factor;  // multiply by (2n+3) (unnormalised forward transform)
    __device__ void operator()(int n, int l, int k, double v) const {
        if (n >= Lrows) return;
        double s = scale ? scale[k] : 1.0;
        if (unnormed_factor) s *= double(2 * n + 3);
        out[(off[l] + ((n - l) >> 1)) * nr + k] = v * s;
    }
};

// ---------------------------------------------------------------------------
// Wigner d(pi/2): one block per l, one thread per column m1 of the lower
// triangle, then the (-1)^(m1+m2) symmetric fill.
__global__ void wignerd_kernel(int L, double* __restrict__ d) {
    const int l = blockIdx.x;
    if (l >= L) return;
    double* D = d + wig_off(l);
    const int ld = l + 1;
    const double sqrt2 = 1.41421356237309504880168872420969808;
    for (int e = threadIdx.x; e < ld * ld; e += blockDim.x) D[e] = 0.0;
    __syncthreads();
    if (l == 0) {
        if (threadIdx.x == 0) D[0] = 1.0;
        return;
    }
    if (l == 1) {
        if (threadIdx.x == 0) {
            D[0] = 0.0;
            D[2] = dv(-1.0, sqrt2);  // (1,0)
            D[1] = dv(1.0, sqrt2);   // (0,1)
            D[3] = 0.5;
        }
        return;
    }
    auto isq = [](int n) { return dv(1.0, __dsqrt_rn(double(n))); };
    // d_l0 chain: d^1_{10} = -1/sqrt2; d^l_{l0} = d^{l-1}_{l-1,0} * (-sqrt(2l-1)/sqrt(2l))
    double dl0 = dv(-1.0, sqrt2);
    for (int j = 2; j <= l; ++j) dl0 = mul(dl0, dv(-sq(2 * j - 1), sq(2 * j)));
    for (int m1 = threadIdx.x; m1 <= l; m1 += blockDim.x) {
        if (m1 == 0) {
            D[ld * l + 0] = dl0;
            D[ld * (l - 1) + 0] = 0.0;
            for (int i = 2; i <= l; i += 2) {
                const int m2 = l - i;
                D[ld * m2] = mul(mul(mul(mul(-D[ld * (m2 + 2)], sq(l - m2 - 1)), sq(l + m2 + 2)), isq(l - m2)),
                                 isq(l + m2 + 1));
            }
        } else if (m1 < l) {
            double dlm = dl0;
            for (int j = 1; j <= m1; ++j) dlm = mul(dlm, mul(-sq(l - j + 1), isq(l + j)));
            D[ld * l + m1] = dlm;
            D[ld * (l - 1) + m1] = mul(mul(mul(dlm, 2.0), double(m1)), isq(2 * l));
            for (int i = 2; i <= l - m1; ++i) {
                const int m2 = l - i;
                const double t = sub(mul(mul(2.0, double(m1)), D[ld * (m2 + 1) + m1]),
                                     mul(mul(sq(l - m2 - 1), sq(l + m2 + 2)), D[ld * (m2 + 2) + m1]));
                D[ld * m2 + m1] = mul(mul(t, isq(l - m2)), isq(l + m2 + 1));
            }
        } else {
            double dlm = dl0;
            for (int j = 1; j < l; ++j) dlm = mul(dlm, mul(-sq(l - j + 1), isq(l + j)));
            D[ld * l + l] = mul(-dlm, isq(2 * l));
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ld * ld; e += blockDim.x) {
        const int m1 = e / ld, m2 = e % ld;
        if (m2 > m1) D[e] = (((m1 ^ m2) & 1) ? -1.0 : 1.0) * D[ld * m2 + m1];
    }
}
}  // namespace

// ---------------------------------------------------------------------------
int launch_plm_ref(cudaStream_t s, int L, int sh_norm, int sh_phase, int nz, const double* z, double* out,
                   bool complex_basis) {
    if (L <= 0 || nz <= 0) return ZEST_GPU_OK;
    dim3 grid((nz + 127) / 128, L);
    const double cnorm = complex_basis ? 1.0 : 1.41421356237309504880168872420969808;
    plm_kernel<<<grid, 128, 0, s>>>(L, sh_norm, sh_phase, nz, z, PlmRefWriter{out, nz}, cnorm);
    return launch_check("plm_kernel");
}

int launch_plm_gemm(cudaStream_t s, int L, int Lrows, int sh_norm, int sh_phase, int nz, const double* z,
                    double* out, const long long* off, const double* scale, int ld, double mscale) {
    if (L <= 0 || nz <= 0) return ZEST_GPU_OK;
    dim3 grid((nz + 127) / 128, L);
    plm_kernel<<<grid, 128, 0, s>>>(L, sh_norm, sh_phase, nz, z, PlmGemmWriter{out, off, scale, ld, mscale, Lrows});
    return launch_check("plm_kernel");
}

int launch_radial_ref(cudaStream_t s, int L, int zernike_norm, int nr, const double* r, double* out) {
    if (L <= 0 || nr <= 0) return ZEST_GPU_OK;
    dim3 grid((nr + 127) / 128, L);
    radial_kernel<<<grid, 128, 0, s>>>(L, zernike_norm, nr, r, RadialRefWriter{out, nr});
    return launch_check("radial_kernel");
}

int launch_radial_gemm(cudaStream_t s, int L, int Lrows, int zernike_norm, int nr, const double* r, double* out,
                       const long long* off, const double* scale, int unnormed_factor) {
    if (L <= 0 || nr <= 0) return ZEST_GPU_OK;
    dim3 grid((nr + 127) / 128, L);
    radial_kernel<<<grid, 128, 0, s>>>(L, zernike_norm, nr, r,
                                       RadialGemmWriter{out, off, scale, nr, Lrows, unnormed_factor});
    return launch_check("radial_kernel");
}

int launch_wignerd(cudaStream_t s, int L, double* out) {
    if (L <= 0) return ZEST_GPU_OK;
    wignerd_kernel<<<L, 128, 0, s>>>(L, out);
    return launch_check("wignerd_kernel");
}

}  // namespace zgpu
