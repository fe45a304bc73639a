/*
 * zest_oracle.c -- CPU restatement of the reference (sebsassi/zest) algorithms
 * on the Gauss-Legendre-quadrature transform and rotation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests/, the
 * smoke check in __graft_entry__.py and the cpu_baseline leg of bench.py may
 * call it, to check results.  The product (zest_gb300/, include/) never links
 * or calls it, and the product path fails loudly rather than fall back here.
 *
 * Parity pin: checked against golden vectors produced by the compiled
 * reference (oracle/_ref, see oracle/build_ref.py and tests/golden/) and
 * against the closed-form known-answer cases of the reference's own tests.
 *
 * Everything is plain double arithmetic; build with -ffp-contract=off so that
 * x86 and aarch64 give identical bits.
 *
 * Index conventions (restated from the reference layouts):
 *   triangle   idx(l,m)   = l(l+1)/2 + m            include/layout.hpp:232-237
 *   radial     idx(n,l)   = floor((n+1)^2/4) + l/2  include/layout.hpp:279-281
 *   zernike    idx(n,l,m) = (n+1)(n+3)(2n+1)/24 + floor(l^2/4) + m
 *                                                   include/layout.hpp:414-417
 *   wigner d   idx(l,a,b) = l(l+1)(2l+1)/6 + (l+1)a + b
 *                                                   include/wignerd_collection.hpp:102-106
 *   Zernike grid [lon][lat][rad], (2L-1, L+1, pad8(L+1))
 *                                                   include/zernike_glq_transformer.hpp:50-131
 *   SH grid LonLat [lon][lat] (2L-1, pad8(L)); LatLon [lat][lon] (L, pad8(2L-1))
 *                                                   include/sh_glq_transformer.hpp:48-197
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#define PI 3.14159265358979323846264338327950288

typedef size_t sz;

static sz tri_idx(sz l, sz m) { return ((l * (l + 1)) >> 1) + m; }
static sz tri_size(sz L) { return (L * (L + 1)) >> 1; }
static sz rad_idx(sz n, sz l) { return (((n + 1) * (n + 1)) >> 2) + (l >> 1); }
static sz rad_size(sz L) { return ((L + 1) * (L + 1)) >> 2; }
static sz zidx(sz n, sz l, sz m) { return (n + 1) * (n + 3) * (2 * n + 1) / 24 + ((l * l) >> 2) + m; }
static sz zsize(sz L) { return (L + 1) * (L + 3) * (2 * L + 1) / 24; }
static sz pad8(sz n) { return (n + 7) & ~(sz)7; }

sz oracle_zt_lon_size(sz L) { return L ? 2 * L - 1 : 0; }
sz oracle_zt_lat_size(sz L) { return L + 1; }
sz oracle_zt_rad_size(sz L) { return pad8(L + 1); }
sz oracle_zt_coeff_size(sz L) { return zsize(L); }
sz oracle_tri_size(sz L) { return tri_size(L); }
sz oracle_rad_table_size(sz L) { return rad_size(L); }

/* ------------------------------------------------------------------------ */
/* Gauss-Legendre nodes and weights.
 * The reference uses tabulated values below 70 nodes and Bogaert's
 * asymptotic formulas above (include/gauss_legendre.hpp:1495-1565).  This
 * restatement solves P_n(x)=0 by Newton's method on the three-term
 * recurrence instead (standard, published method); nodes agree to a few ulp.
 * Unpacked layout: ascending in x, node 0 nearest -1
 * (include/gauss_legendre.hpp:368-412).  Packed layout: the ceil(n/2)
 * non-negative nodes, ascending from the centre (gauss_legendre.hpp:354-366).
 */
/* Double-double arithmetic (Dekker/Knuth error-free transformations).  The
 * Newton solve and the weight formula run in ~106-bit precision so that the
 * weights of nodes near +-1 keep full double accuracy. */
typedef struct { double hi, lo; } dd;
static dd dd_two_sum(double a, double b) {
    double s = a + b, bb = s - a;
    dd r = { s, (a - (s - bb)) + (b - bb) };
    return r;
}
static dd dd_fast(double a, double b) {
    double s = a + b;
    dd r = { s, b - (s - a) };
    return r;
}
static void dd_split(double a, double* hi, double* lo) {
    double c = 134217729.0 * a;
    *hi = c - (c - a);
    *lo = a - *hi;
}
static dd dd_two_prod(double a, double b) {
    double p = a * b, ah, al, bh, bl;
    dd_split(a, &ah, &al);
    dd_split(b, &bh, &bl);
    dd r = { p, ((ah * bh - p) + ah * bl + al * bh) + al * bl };
    return r;
}
static dd dd_add(dd x, dd y) {
    dd s = dd_two_sum(x.hi, y.hi);
    return dd_fast(s.hi, s.lo + x.lo + y.lo);
}
static dd dd_neg(dd x) { dd r = { -x.hi, -x.lo }; return r; }
static dd dd_mul(dd x, dd y) {
    dd p = dd_two_prod(x.hi, y.hi);
    return dd_fast(p.hi, p.lo + (x.hi * y.lo + x.lo * y.hi));
}
static dd dd_mul_d(dd x, double d) {
    dd p = dd_two_prod(x.hi, d);
    return dd_fast(p.hi, p.lo + x.lo * d);
}
static dd dd_div(dd x, dd y) {
    double q1 = x.hi / y.hi;
    dd r = dd_add(x, dd_neg(dd_mul_d(y, q1)));
    double q2 = r.hi / y.hi;
    r = dd_add(r, dd_neg(dd_mul_d(y, q2)));
    double q3 = r.hi / y.hi;
    return dd_add(dd_fast(q1, q2), (dd){ q3, 0.0 });
}
static dd dd_from(double a) { dd r = { a, 0.0 }; return r; }

/* P_n(x) and P_{n-1}(x) by the three-term recurrence, in double-double. */
static void legendre_pair_dd(sz n, dd x, dd* pn, dd* pnm1) {
    dd p0 = dd_from(1.0), p1 = x;
    if (n == 0) { *pn = p0; *pnm1 = dd_from(0.0); return; }
    for (sz k = 2; k <= n; ++k) {
        dd t = dd_add(dd_mul_d(dd_mul(x, p1), (double)(2 * k - 1)), dd_neg(dd_mul_d(p0, (double)(k - 1))));
        dd p2 = dd_div(t, dd_from((double)k));
        p0 = p1;
        p1 = p2;
    }
    *pn = p1;
    *pnm1 = p0;
}

/* k-th node from the top (k = 1 .. ceil(n/2)), i.e. the largest first. */
static void gl_node_weight(sz n, sz k, double* node, double* weight) {
    dd x;
    if ((n & 1) && k == (n + 1) / 2) {
        x = dd_from(0.0); /* middle node of an odd rule */
    } else {
        /* initial guess (Tricomi's asymptotic), then Newton in double-double */
        double theta = PI * ((double)k - 0.25) / ((double)n + 0.5);
        x = dd_from(cos(theta + 1.0 / (8.0 * (double)n * (double)n * tan(theta))));
        for (int it = 0; it < 60; ++it) {
            dd pn, pnm1;
            legendre_pair_dd(n, x, &pn, &pnm1);
            /* P'_n(x) = n (P_{n-1} - x P_n) / (1 - x^2) */
            dd omx2 = dd_mul(dd_add(dd_from(1.0), dd_neg(x)), dd_add(dd_from(1.0), x));
            dd dp = dd_div(dd_mul_d(dd_add(pnm1, dd_neg(dd_mul(x, pn))), (double)n), omx2);
            dd dx = dd_div(pn, dp);
            x = dd_add(x, dd_neg(dx));
            if (fabs(dx.hi) < 1e-30 * (fabs(x.hi) + 1e-300) || dx.hi == 0.0) break;
        }
    }
    dd pn, pnm1;
    legendre_pair_dd(n, x, &pn, &pnm1);
    /* w = 2 (1 - x^2) / (n P_{n-1}(x))^2 */
    dd omx2 = dd_mul(dd_add(dd_from(1.0), dd_neg(x)), dd_add(dd_from(1.0), x));
    dd np = dd_mul_d(pnm1, (double)n);
    dd w = dd_div(dd_mul_d(omx2, 2.0), dd_mul(np, np));
    *node = x.hi + x.lo;
    *weight = w.hi + w.lo;
}

void oracle_gl_nodes_weights(sz n, int packed, double* nodes, double* weights) {
    sz nu = (n + 1) >> 1;
    for (sz k = 1; k <= nu; ++k) {
        double x, w;
        gl_node_weight(n, k, &x, &w);
        if (packed) {
            nodes[nu - k] = x;
            weights[nu - k] = w;
        } else {
            nodes[k - 1] = -x;
            weights[k - 1] = w;
            nodes[n - k] = x; /* the middle node of an odd rule stays +0 */
            weights[n - k] = w;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Normalised associated Legendre functions, vector form.
 * Restates st::PlmRecursion::plm_impl(span z, ...) with complex_norm = sqrt2
 * (plm_real), include/plm_recursion.hpp:229-354, coefficients a(l,m), b(l,m)
 * from src/plm_recursion.cpp:31-55.  Output layout [idx(l,m)][i].
 *   sh_norm: 0 = geo (4pi), 1 = qm (orthonormal);  sh_phase: 0 = none (-1), 1 = cs (+1)
 */
void oracle_plm_real(sz L, int sh_norm, int sh_phase, sz nz, const double* z, double* out) {
    if (L == 0) return;
    const double inv_sqrt_4pi = 0.28209479177387814347403972578038629; /* 1/sqrt(4pi) */
    const double phase = sh_phase ? 1.0 : -1.0;
    double* sq = (double*)malloc(sizeof(double) * (2 * L + 2));
    for (sz l = 0; l < 2 * L + 2; ++l) sq[l] = sqrt((double)l);
    double* u = (double*)malloc(sizeof(double) * nz);
    double* us = (double*)malloc(sizeof(double) * nz);
    for (sz i = 0; i < nz; ++i) u[i] = sqrt((1.0 - z[i]) * (1.0 + z[i]));
#define P(l, m) (out + tri_idx((l), (m)) * nz)
    for (sz i = 0; i < nz; ++i) P(0, 0)[i] = sh_norm ? inv_sqrt_4pi : 1.0;
    if (L == 1) goto done;
    for (sz i = 0; i < nz; ++i) P(1, 0)[i] = sh_norm ? z[i] * (sq[3] * inv_sqrt_4pi) : z[i] * sq[3];
    for (sz l = 2; l < L; ++l) {
        /* a(l,0) = sqrt(2l-1)sqrt(2l+1)/l, b(l,0) = (l-1)sqrt(2l+1)/(sqrt(2l-3) l) */
        double a = sq[2 * l - 1] * sq[2 * l + 1] / (double)l;
        double b = ((double)l - 1.0) * sq[2 * l + 1] / (sq[2 * l - 3] * (double)l);
        for (sz i = 0; i < nz; ++i) P(l, 0)[i] = a * z[i] * P(l - 1, 0)[i] - b * P(l - 2, 0)[i];
    }
    {
        const double uc = 1.0e-280; /* underflow compensation, plm_recursion.hpp:295 */
        double pmm = sh_norm ? uc * 1.41421356237309504880168872420969808 * inv_sqrt_4pi
                             : uc * 1.41421356237309504880168872420969808;
        for (sz i = 0; i < nz; ++i) us[i] = 1.0 / uc;
        for (sz m = 1; m + 1 < L; ++m) {
            for (sz i = 0; i < nz; ++i) us[i] *= u[i];
            pmm *= phase * sq[2 * m + 1] / sq[2 * m];
            for (sz i = 0; i < nz; ++i) P(m, m)[i] = pmm;
            for (sz i = 0; i < nz; ++i) P(m + 1, m)[i] = z[i] * (sq[2 * m + 3] * pmm);
            for (sz l = m + 2; l < L; ++l) {
                /* a(l,m) = sqrt((2l-1)(2l+1)/((l-m)(l+m)))
                   b(l,m) = sqrt((2l+1)(l+m-1)(l-m-1)/((l-m)(l+m)(2l-3))) */
                double a = sq[2 * l - 1] * sq[2 * l + 1] / (sq[l - m] * sq[l + m]);
                double b = sq[2 * l + 1] * sq[l + m - 1] * sq[l - m - 1] / (sq[l - m] * sq[l + m] * sq[2 * l - 3]);
                double* pl = P(l, m);
                double* p1 = P(l - 1, m);
                double* p2 = P(l - 2, m);
                for (sz i = 0; i < nz; ++i) pl[i] = z[i] * a * p1[i] - b * p2[i];
                for (sz i = 0; i < nz; ++i) p2[i] *= us[i];
            }
            for (sz i = 0; i < nz; ++i) P(L - 1, m)[i] *= us[i];
            for (sz i = 0; i < nz; ++i) P(L - 2, m)[i] *= us[i];
        }
        for (sz i = 0; i < nz; ++i) us[i] *= u[i];
        for (sz i = 0; i < nz; ++i)
            P(L - 1, L - 1)[i] = us[i] * (phase * pmm * sq[2 * L - 1] / sq[2 * L - 2]);
    }
#undef P
done:
    free(sq);
    free(u);
    free(us);
}

/* ------------------------------------------------------------------------ */
/* Radial 3D Zernike polynomials R_nl(r), vector form.
 * Restates zt::RadialZernikeRecursion::zernike(span r, ...),
 * include/radial_zernike_recursion.hpp:151-288, coefficients k1,k2,k3 from
 * src/radial_zernike_recursion.cpp:31-56.  Output layout [idx(n,l)][k].
 * The normed form multiplies every entry by sqrt(2n+3); the recursion itself
 * always runs on unnormalised values, as in the reference.
 *   zernike_norm: 0 = normed, 1 = unnormed
 */
void oracle_radial_zernike(sz L, int zernike_norm, sz nr, const double* r, double* out) {
    if (L == 0) return;
#define R(n, l) (out + rad_idx((n), (l)) * nr)
    for (sz k = 0; k < nr; ++k) R(0, 0)[k] = 1.0;
    if (L > 1) for (sz k = 0; k < nr; ++k) R(1, 1)[k] = r[k];
    if (L > 2) {
        for (sz k = 0; k < nr; ++k) R(2, 2)[k] = r[k] * r[k];
        for (sz k = 0; k < nr; ++k) R(2, 0)[k] = 2.5 * R(2, 2)[k] - 1.5;
    }
    if (L > 3) {
        for (sz k = 0; k < nr; ++k) R(3, 1)[k] = (3.5 * R(2, 2)[k] - 2.5) * r[k];
        for (sz k = 0; k < nr; ++k) R(3, 3)[k] = R(2, 2)[k] * r[k];
    }
    for (sz n = 4; n < L; ++n) {
        const double dn = (double)n;
        for (sz l = n & 1; l + 4 <= n; l += 2) {
            const double dl = (double)l;
            const double k0 = (dn - dl) * (dn + dl + 1.0) * (2.0 * dn - 3.0);
            const double k1 = (2.0 * dn - 1.0) * (2.0 * dn + 1) * (2.0 * dn - 3.0);
            const double k2 = -0.5 * (2.0 * dn - 1.0) * ((2 * dl + 1.0) * (2.0 * dl + 1.0) + (2.0 * dn + 1) * (2.0 * dn - 3.0));
            const double k3 = -(dn - dl - 2.0) * (dn + dl - 1.0) * (2.0 * dn + 1);
            const double k0_inv = 1.0 / k0;
            const double c1 = k1 * k0_inv, c2 = k2 * k0_inv, c3 = k3 * k0_inv;
            double* rn = R(n, l);
            double* r2 = R(n - 2, l);
            double* r4 = R(n - 4, l);
            double* rsq = R(2, 2);
            for (sz k = 0; k < nr; ++k) rn[k] = (c2 + c1 * rsq[k]) * r2[k] + c3 * r4[k];
        }
        for (sz k = 0; k < nr; ++k) R(n, n)[k] = r[k] * R(n - 1, n - 1)[k];
        for (sz k = 0; k < nr; ++k) R(n, n - 2)[k] = (dn + 0.5) * R(n, n)[k] - (dn - 0.5) * R(n - 2, n - 2)[k];
    }
    if (zernike_norm == 0) {
        for (sz n = 0; n < L; ++n) {
            const double norm = sqrt(2.0 * (double)n + 3.0);
            for (sz l = n & 1; l <= n; l += 2)
                for (sz k = 0; k < nr; ++k) R(n, l)[k] *= norm;
        }
    }
#undef R
}

/* ------------------------------------------------------------------------ */
/* Real DFT helpers: forward X[m] = sum_i f_i exp(-2 pi i im/N), m < nm, with the
 * exact argument reduction (i*m mod N); and the Hermitian inverse with factor 1
 * (pocketfft r2c / c2r semantics, include/zernike_glq_transformer.hpp:710-720,
 * 943-949). */
static double* make_twiddles(sz N) {
    double* t = (double*)malloc(sizeof(double) * 2 * N);
    for (sz i = 0; i < N; ++i) {
        double ang = 2.0 * PI * (double)i / (double)N;
        t[2 * i] = cos(ang);
        t[2 * i + 1] = sin(ang);
    }
    return t;
}

/* ------------------------------------------------------------------------ */
/* Zernike GLQ forward transform (include/zernike_glq_transformer.hpp:640-655):
 * integrate_longitudinal (710-720), apply_weights (722-776),
 * integrate_latitudinal (778-817), integrate_radial (819-865).
 * grid: [lon][lat][rad] of order Lg; coeffs: idx(n,l,m) pairs of order Le;
 * coefficients are truncated to min(Lg, Le) and the rest left zero. */
void oracle_zt_forward(sz Lg, sz Le, int zernike_norm, int sh_norm, int sh_phase,
                       const double* grid, double* coeffs) {
    const sz Np = oracle_zt_lon_size(Lg), Nt = Lg + 1, Nr = pad8(Lg + 1);
    const sz Lm = Lg < Le ? Lg : Le;
    memset(coeffs, 0, sizeof(double) * 2 * zsize(Le));
    if (Lg == 0) return;
    double* latn = (double*)malloc(sizeof(double) * Nt);
    double* latw = (double*)malloc(sizeof(double) * Nt);
    double* radn = (double*)malloc(sizeof(double) * Nr);
    double* radw = (double*)malloc(sizeof(double) * Nr);
    oracle_gl_nodes_weights(Nt, 0, latn, latw);
    oracle_gl_nodes_weights(Nr, 0, radn, radw);
    for (sz k = 0; k < Nr; ++k) radn[k] = 0.5 * (1.0 + radn[k]);
    double* plm = (double*)malloc(sizeof(double) * tri_size(Lg) * Nt);
    oracle_plm_real(Lg, sh_norm, sh_phase, Nt, latn, plm);
    double* rz = (double*)malloc(sizeof(double) * rad_size(Lg) * Nr);
    oracle_radial_zernike(Lg, zernike_norm, Nr, radn, rz);

    /* longitudinal DFT + weights: G[m][j][k] (complex) */
    const double shn = sh_norm ? 1.0 : 1.0 / (4.0 * PI);
    const double pref = shn * 0.5 * ((2.0 * PI) / (double)Np);
    double* tw = make_twiddles(Np);
    double* G = (double*)calloc(2 * Lg * Nt * Nr, sizeof(double));
    for (sz m = 0; m < Lg; ++m) {
        for (sz j = 0; j < Nt; ++j) {
            for (sz k = 0; k < Nr; ++k) {
                double re = 0.0, im = 0.0;
                for (sz i = 0; i < Np; ++i) {
                    const double f = grid[(i * Nt + j) * Nr + k];
                    const sz t = (i * m) % Np;
                    re += f * tw[2 * t];
                    im -= f * tw[2 * t + 1];
                }
                if (m == 0) im = 0.0;
                const double r = radn[k];
                const double w = latw[j] * r * r * radw[k];
                double* g = G + 2 * ((m * Nt + j) * Nr + k);
                g[0] = w * (pref * re);
                g[1] = -w * (pref * im);
            }
        }
    }
    /* latitudinal integral: flm[idx(l,m)][k] */
    double* flm = (double*)calloc(2 * tri_size(Lm) * Nr, sizeof(double));
    for (sz l = 0; l < Lm; ++l)
        for (sz m = 0; m <= l; ++m) {
            double* f = flm + 2 * tri_idx(l, m) * Nr;
            const double* p = plm + tri_idx(l, m) * Nt;
            for (sz j = 0; j < Nt; ++j) {
                const double* g = G + 2 * ((m * Nt + j) * Nr);
                for (sz k = 0; k < Nr; ++k) {
                    f[2 * k] += p[j] * g[2 * k];
                    f[2 * k + 1] += p[j] * g[2 * k + 1];
                }
            }
        }
    /* radial integral */
    for (sz n = 0; n < Lm; ++n) {
        const double norm = zernike_norm ? (double)(2 * n + 3) : 1.0;
        for (sz l = n & 1; l <= n; l += 2) {
            const double* rr = rz + rad_idx(n, l) * Nr;
            for (sz m = 0; m <= l; ++m) {
                const double* f = flm + 2 * tri_idx(l, m) * Nr;
                double c0 = 0.0, c1 = 0.0;
                for (sz k = 0; k < Nr; ++k) {
                    c0 += rr[k] * f[2 * k];
                    c1 += rr[k] * f[2 * k + 1];
                }
                double* c = coeffs + 2 * zidx(n, l, m);
                c[0] = c0 * norm;
                c[1] = c1 * norm;
            }
        }
    }
    free(latn); free(latw); free(radn); free(radw); free(plm); free(rz); free(tw); free(G); free(flm);
}

/* Zernike GLQ backward transform (include/zernike_glq_transformer.hpp:663-679):
 * sum_n (867-899), sum_l (901-941, factor 1/2 for m>0 and conjugation),
 * sum_m (943-949, Hermitian c2r with factor 1). */
void oracle_zt_backward(sz Le, sz Lg, int zernike_norm, int sh_norm, int sh_phase,
                        const double* coeffs, double* grid) {
    const sz Np = oracle_zt_lon_size(Lg), Nt = Lg + 1, Nr = pad8(Lg + 1);
    const sz Lm = Lg < Le ? Lg : Le;
    memset(grid, 0, sizeof(double) * Np * Nt * Nr);
    if (Lg == 0) return;
    double* latn = (double*)malloc(sizeof(double) * Nt);
    double* latw = (double*)malloc(sizeof(double) * Nt);
    double* radn = (double*)malloc(sizeof(double) * Nr);
    double* radw = (double*)malloc(sizeof(double) * Nr);
    oracle_gl_nodes_weights(Nt, 0, latn, latw);
    oracle_gl_nodes_weights(Nr, 0, radn, radw);
    for (sz k = 0; k < Nr; ++k) radn[k] = 0.5 * (1.0 + radn[k]);
    double* plm = (double*)malloc(sizeof(double) * tri_size(Lg) * Nt);
    oracle_plm_real(Lg, sh_norm, sh_phase, Nt, latn, plm);
    double* rz = (double*)malloc(sizeof(double) * rad_size(Lg) * Nr);
    oracle_radial_zernike(Lg, zernike_norm, Nr, radn, rz);

    double* flm = (double*)calloc(2 * tri_size(Lm ? Lm : 1) * Nr, sizeof(double));
    for (sz n = 0; n < Lm; ++n)
        for (sz l = n & 1; l <= n; l += 2) {
            const double* rr = rz + rad_idx(n, l) * Nr;
            for (sz m = 0; m <= l; ++m) {
                const double* c = coeffs + 2 * zidx(n, l, m);
                double* f = flm + 2 * tri_idx(l, m) * Nr;
                for (sz k = 0; k < Nr; ++k) {
                    f[2 * k] += rr[k] * c[0];
                    f[2 * k + 1] += rr[k] * c[1];
                }
            }
        }
    double* F = (double*)calloc(2 * Lg * Nt * Nr, sizeof(double));
    for (sz l = 0; l < Lm; ++l)
        for (sz m = 0; m <= l; ++m) {
            const double mf = m > 0 ? 0.5 : 1.0;
            const double* p = plm + tri_idx(l, m) * Nt;
            const double* f = flm + 2 * tri_idx(l, m) * Nr;
            for (sz j = 0; j < Nt; ++j) {
                const double w = mf * p[j];
                double* g = F + 2 * ((m * Nt + j) * Nr);
                for (sz k = 0; k < Nr; ++k) {
                    g[2 * k] += w * f[2 * k];
                    g[2 * k + 1] += -w * f[2 * k + 1];
                }
            }
        }
    double* tw = make_twiddles(Np);
    for (sz j = 0; j < Nt; ++j)
        for (sz k = 0; k < Nr; ++k)
            for (sz i = 0; i < Np; ++i) {
                double s = F[2 * ((0 * Nt + j) * Nr + k)];
                for (sz m = 1; m < Lg; ++m) {
                    const double* g = F + 2 * ((m * Nt + j) * Nr + k);
                    const sz t = (i * m) % Np;
                    s += 2.0 * (g[0] * tw[2 * t] - g[1] * tw[2 * t + 1]);
                }
                grid[(i * Nt + j) * Nr + k] = s;
            }
    free(latn); free(latw); free(radn); free(radw); free(plm); free(rz); free(tw); free(F); free(flm);
}

/* ------------------------------------------------------------------------ */
/* SH GLQ transforms (include/sh_glq_transformer.hpp:632-668).
 * Grid layouts: latlon=0 -> LonLatLayout [lon][lat] with lat = pad8(L), lon = 2L-1
 *               latlon=1 -> LatLonLayout [lat][lon] with lat = L, lon = pad8(2L-1)
 *               (odd L: the reference's north/south fold visits the middle
 *               node twice; restated as is)
 * The forward path folds north/south node pairs with the packed GL weights
 * (fft_to_symm_asymm, :810-884) and sums even/odd l over the unique nodes
 * (integrate_latitudinal, :886-974); the backward path is the exact transpose
 * (sum_l :976-1051, symm_asymm_to_fft :1136-1193, sum_m :1195-1201). */
/* The LatLon layout pads the longitude axis to a multiple of 8 and the
 * reference transforms over the padded length, so its grid has pad8(2L-1)
 * equally spaced longitudes (sh_glq_transformer.hpp:98-108, 757-765). */
static void st_shape(sz L, int latlon, sz* nlon, sz* nlat, sz* lon_alloc) {
    if (latlon) { *nlat = L; *nlon = pad8(L ? 2 * L - 1 : 0); *lon_alloc = *nlon; }
    else { *nlat = pad8(L); *nlon = L ? 2 * L - 1 : 0; *lon_alloc = *nlon; }
}

sz oracle_st_grid_size(sz L, int latlon) {
    sz nlon, nlat, la;
    st_shape(L, latlon, &nlon, &nlat, &la);
    return la * nlat;
}

static sz st_off(int latlon, sz i_lon, sz j_lat, sz nlat, sz lon_alloc) {
    return latlon ? j_lat * lon_alloc + i_lon : i_lon * nlat + j_lat;
}

void oracle_st_forward(sz Lg, sz Le, int sh_norm, int sh_phase, int latlon,
                       const double* grid, double* coeffs) {
    sz Np, Nt, la;
    st_shape(Lg, latlon, &Np, &Nt, &la);
    const sz Lm = Lg < Le ? Lg : Le;
    memset(coeffs, 0, sizeof(double) * 2 * tri_size(Le));
    if (Lg == 0) return;
    const sz nu = (Nt + 1) >> 1;
    double* pn = (double*)malloc(sizeof(double) * nu);
    double* pw = (double*)malloc(sizeof(double) * nu);
    oracle_gl_nodes_weights(Nt, 1, pn, pw);
    double* plm = (double*)malloc(sizeof(double) * tri_size(Lg) * nu);
    oracle_plm_real(Lg, sh_norm, sh_phase, nu, pn, plm);
    const double shn = sh_norm ? 1.0 : 1.0 / (4.0 * PI);
    const double pref = shn * (2.0 * PI) / (double)Np;
    double* tw = make_twiddles(Np);
    /* X[m][lat] = pref * DFT */
    double* X = (double*)calloc(2 * Lg * Nt, sizeof(double));
    for (sz m = 0; m < Lg; ++m)
        for (sz j = 0; j < Nt; ++j) {
            double re = 0.0, im = 0.0;
            for (sz i = 0; i < Np; ++i) {
                const double f = grid[st_off(latlon, i, j, Nt, la)];
                const sz t = (i * m) % Np;
                re += f * tw[2 * t];
                im -= f * tw[2 * t + 1];
            }
            if (m == 0) im = 0.0;
            X[2 * (m * Nt + j)] = pref * re;
            X[2 * (m * Nt + j) + 1] = pref * im;
        }
    /* fold: S[par][m][i], par 0 = N + (-1)^m S, par 1 = N - (-1)^m S */
    const sz north = Nt >> 1, south = nu - 1;
    double* S = (double*)calloc(2 * 2 * Lg * nu, sizeof(double));
    for (sz m = 0; m < Lg; ++m) {
        const double sign = (m & 1) ? -1.0 : 1.0;
        for (sz i = 0; i < nu; ++i) {
            const double w = pw[i];
            const double* xs = X + 2 * (m * Nt + (south - i));
            const double* xn = X + 2 * (m * Nt + (north + i));
            const double sre = w * xs[0], sim = -w * xs[1];
            const double nre = w * xn[0], nim = -w * xn[1];
            double* s0 = S + 2 * ((0 * Lg + m) * nu + i);
            double* s1 = S + 2 * ((1 * Lg + m) * nu + i);
            s0[0] = nre + sign * sre; s0[1] = nim + sign * sim;
            s1[0] = nre - sign * sre; s1[1] = nim - sign * sim;
        }
    }
    for (sz l = 0; l < Lm; ++l)
        for (sz m = 0; m <= l; ++m) {
            const double* p = plm + tri_idx(l, m) * nu;
            const double* s = S + 2 * (((l & 1) * Lg + m) * nu);
            double c0 = 0.0, c1 = 0.0;
            for (sz i = 0; i < nu; ++i) {
                c0 += p[i] * s[2 * i];
                c1 += p[i] * s[2 * i + 1];
            }
            coeffs[2 * tri_idx(l, m)] = c0;
            coeffs[2 * tri_idx(l, m) + 1] = c1;
        }
    free(pn); free(pw); free(plm); free(tw); free(X); free(S);
}

void oracle_st_backward(sz Le, sz Lg, int sh_norm, int sh_phase, int latlon,
                        const double* coeffs, double* grid) {
    sz Np, Nt, la;
    st_shape(Lg, latlon, &Np, &Nt, &la);
    const sz Lm = Lg < Le ? Lg : Le;
    memset(grid, 0, sizeof(double) * la * Nt);
    if (Lg == 0) return;
    const sz nu = (Nt + 1) >> 1;
    double* pn = (double*)malloc(sizeof(double) * nu);
    double* pw = (double*)malloc(sizeof(double) * nu);
    oracle_gl_nodes_weights(Nt, 1, pn, pw);
    double* plm = (double*)malloc(sizeof(double) * tri_size(Lg) * nu);
    oracle_plm_real(Lg, sh_norm, sh_phase, nu, pn, plm);
    double* S = (double*)calloc(2 * 2 * Lg * nu, sizeof(double));
    for (sz l = 0; l < Lm; ++l)
        for (sz m = 0; m <= l; ++m) {
            const double* p = plm + tri_idx(l, m) * nu;
            double* s = S + 2 * (((l & 1) * Lg + m) * nu);
            const double c0 = coeffs[2 * tri_idx(l, m)], c1 = coeffs[2 * tri_idx(l, m) + 1];
            for (sz i = 0; i < nu; ++i) {
                const double w = m > 0 ? 0.5 * p[i] : p[i];
                s[2 * i] += w * c0;
                s[2 * i + 1] += -w * c1;
            }
        }
    const sz north = Nt >> 1, south = nu - 1;
    double* X = (double*)calloc(2 * Lg * Nt, sizeof(double));
    for (sz m = 0; m < Lg; ++m) {
        const double sign = (m & 1) ? -1.0 : 1.0;
        for (sz i = 0; i < nu; ++i) {
            const double* s0 = S + 2 * ((0 * Lg + m) * nu + i);
            const double* s1 = S + 2 * ((1 * Lg + m) * nu + i);
            double* xn = X + 2 * (m * Nt + (north + i));
            double* xs = X + 2 * (m * Nt + (south - i));
            xn[0] = s0[0] + s1[0]; xn[1] = s0[1] + s1[1];
            xs[0] = sign * (s0[0] - s1[0]); xs[1] = sign * (s0[1] - s1[1]);
        }
    }
    double* tw = make_twiddles(Np);
    for (sz j = 0; j < Nt; ++j)
        for (sz i = 0; i < Np; ++i) {
            double s = X[2 * (0 * Nt + j)];
            for (sz m = 1; m < Lg; ++m) {
                const double* g = X + 2 * (m * Nt + j);
                const sz t = (i * m) % Np;
                s += 2.0 * (g[0] * tw[2 * t] - g[1] * tw[2 * t + 1]);
            }
            grid[st_off(latlon, i, j, Nt, la)] = s;
        }
    free(pn); free(pw); free(plm); free(tw); free(X); free(S);
}

/* ------------------------------------------------------------------------ */
/* Wigner small-d matrices at pi/2 for 0 <= m1,m2 <= l < L.
 * Restates the recursion of WignerdPiHalfCollection's constructor,
 * src/wignerd_collection.cpp:29-98, layout wignerd_collection.hpp:102-106. */
sz oracle_wignerd_size(sz L) { return L * (L + 1) * (2 * L + 1) / 6; }

void oracle_wignerd(sz L, double* d) {
    if (L == 0) return;
    /* entries d^l_{m,0} with l+m odd are never written by the recursion: they are 0 */
    memset(d, 0, sizeof(double) * oracle_wignerd_size(L));
    double* sq = (double*)malloc(sizeof(double) * (2 * L + 2));
    double* isq = (double*)malloc(sizeof(double) * (2 * L + 2));
    for (sz l = 0; l < 2 * L + 2; ++l) { sq[l] = sqrt((double)l); isq[l] = 1.0 / sq[l]; }
#define D(l, a, b) d[(l) * ((l) + 1) * (2 * (l) + 1) / 6 + ((l) + 1) * (a) + (b)]
    D(0, 0, 0) = 1.0;
    if (L > 1) {
        const double s2 = 1.41421356237309504880168872420969808;
        D(1, 0, 0) = 0.0;
        D(1, 1, 0) = -1.0 / s2;
        D(1, 0, 1) = 1.0 / s2;
        D(1, 1, 1) = 0.5;
        double dl0 = -1.0 / s2;
        for (sz l = 2; l < L; ++l) {
            dl0 *= -sq[2 * l - 1] / sq[2 * l];
            D(l, l, 0) = dl0;
            D(l, l - 1, 0) = 0.0;
            for (sz i = 2; i <= l; i += 2) {
                const sz m2 = l - i;
                D(l, m2, 0) = -D(l, m2 + 2, 0) * sq[l - m2 - 1] * sq[l + m2 + 2] * isq[l - m2] * isq[l + m2 + 1];
            }
            double dlm = dl0;
            for (sz m1 = 1; m1 < l; ++m1) {
                dlm *= -sq[l - m1 + 1] * isq[l + m1];
                D(l, l, m1) = dlm;
                D(l, l - 1, m1) = D(l, l, m1) * 2.0 * (double)m1 * isq[2 * l];
                for (sz i = 2; i <= l - m1; ++i) {
                    const sz m2 = l - i;
                    D(l, m2, m1) = (2.0 * (double)m1 * D(l, m2 + 1, m1)
                                    - sq[l - m2 - 1] * sq[l + m2 + 2] * D(l, m2 + 2, m1))
                                   * isq[l - m2] * isq[l + m2 + 1];
                }
            }
            D(l, l, l) = -dlm * isq[2 * l];
            for (sz m1 = 0; m1 <= l; ++m1)
                for (sz m2 = m1 + 1; m2 <= l; ++m2) {
                    const double sign = ((m1 ^ m2) & 1) ? -1.0 : 1.0;
                    D(l, m1, m2) = sign * D(l, m2, m1);
                }
        }
    }
#undef D
    free(sq);
    free(isq);
}

/* ------------------------------------------------------------------------ */
/* Rotation of one complex vector of length l+1 (rotate_l,
 * include/wignerd_collection.hpp:122-296): gamma phase, X(pi/2) via the
 * even/odd sparsity of d(pi/2), beta phase, X(-pi/2), alpha phase.
 * v: interleaved complex; ea/eb/eg: e^{-i m angle} interleaved. */
static void rotate_l(sz l, double* v, const double* dl, const double* eg, const double* eb, const double* ea, double* tmp) {
#define W(a, b) dl[(l + 1) * (a) + (b)]
#define VR(m) v[2 * (m)]
#define VI(m) v[2 * (m) + 1]
    for (sz m = 0; m <= l; ++m) {
        const double cr = VR(m), ci = VI(m), rr = eg[2 * m], ri = eg[2 * m + 1];
        VR(m) = cr * rr - ci * ri;
        VI(m) = cr * ri + ci * rr;
    }
    if (l & 1) {
        for (sz m = 0; m < l; m += 2) {
            double s0 = 0.5 * W(m, 0) * VR(0), s1 = 0.0, s2 = 0.5 * W(m + 1, 0) * VR(0), s3 = 0.0;
            for (sz mp = 1; mp < l; mp += 2) {
                s0 += W(m, mp) * VR(mp);
                s1 += W(m + 1, mp) * VI(mp);
                s2 += W(m + 1, mp + 1) * VR(mp + 1);
                s3 += W(m, mp + 1) * VI(mp + 1);
            }
            s0 += W(m, l) * VR(l);
            s1 += W(m + 1, l) * VI(l);
            tmp[2 * m] = 2.0 * s0; tmp[2 * m + 1] = 2.0 * s3;
            tmp[2 * (m + 1)] = 2.0 * s2; tmp[2 * (m + 1) + 1] = 2.0 * s1;
        }
    } else {
        for (sz m = 0; m < l; m += 2) {
            double s0 = 0.5 * W(m + 1, 0) * VR(0), s1 = 0.0, s2 = 0.5 * W(m, 0) * VR(0), s3 = 0.0;
            for (sz mp = 1; mp < l; mp += 2) {
                s0 += W(m + 1, mp) * VR(mp);
                s1 += W(m, mp) * VI(mp);
                s2 += W(m, mp + 1) * VR(mp + 1);
                s3 += W(m + 1, mp + 1) * VI(mp + 1);
            }
            tmp[2 * m] = 2.0 * s2; tmp[2 * m + 1] = 2.0 * s1;
            tmp[2 * (m + 1)] = 2.0 * s0; tmp[2 * (m + 1) + 1] = 2.0 * s3;
        }
        double t0 = 0.0, t1 = 0.5 * W(l, 0) * VR(0);
        for (sz mp = 1; mp < l; mp += 2) {
            t1 += W(l, mp + 1) * VR(mp + 1);
            t0 += W(l, mp) * VI(mp);
        }
        tmp[2 * l] = 2.0 * t1; tmp[2 * l + 1] = 2.0 * t0;
    }
    for (sz m = 0; m <= l; ++m) {
        const double cr = tmp[2 * m], ci = tmp[2 * m + 1], rr = eb[2 * m], ri = eb[2 * m + 1];
        VR(m) = cr * rr - ci * ri;
        VI(m) = cr * ri + ci * rr;
    }
    if (l & 1) {
        for (sz m = 0; m < l; m += 2) {
            double s0 = 0.5 * W(0, m) * VR(0), s1 = 0.0, s2 = 0.5 * W(0, m + 1) * VR(0), s3 = 0.0;
            for (sz mp = 1; mp < l; mp += 2) {
                s0 += W(mp, m) * VR(mp);
                s1 += W(mp, m + 1) * VI(mp);
                s2 += W(mp + 1, m + 1) * VR(mp + 1);
                s3 += W(mp + 1, m) * VI(mp + 1);
            }
            s0 += W(l, m) * VR(l);
            s1 += W(l, m + 1) * VI(l);
            tmp[2 * m] = 2.0 * s0; tmp[2 * m + 1] = 2.0 * s3;
            tmp[2 * (m + 1)] = 2.0 * s2; tmp[2 * (m + 1) + 1] = 2.0 * s1;
        }
    } else {
        for (sz m = 0; m < l; m += 2) {
            double s0 = 0.5 * W(0, m + 1) * VR(0), s1 = 0.0, s2 = 0.5 * W(0, m) * VR(0), s3 = 0.0;
            for (sz mp = 1; mp < l; mp += 2) {
                s0 += W(mp, m + 1) * VR(mp);
                s1 += W(mp, m) * VI(mp);
                s2 += W(mp + 1, m) * VR(mp + 1);
                s3 += W(mp + 1, m + 1) * VI(mp + 1);
            }
            tmp[2 * m] = 2.0 * s2; tmp[2 * m + 1] = 2.0 * s1;
            tmp[2 * (m + 1)] = 2.0 * s0; tmp[2 * (m + 1) + 1] = 2.0 * s3;
        }
        double t0 = 0.0, t1 = 0.5 * W(l, 0) * VR(0);
        for (sz mp = 1; mp < l; mp += 2) {
            t1 += W(mp + 1, l) * VR(mp + 1);
            t0 += W(mp, l) * VI(mp);
        }
        tmp[2 * l] = 2.0 * t1; tmp[2 * l + 1] = 2.0 * t0;
    }
    for (sz m = 0; m <= l; ++m) {
        const double cr = tmp[2 * m], ci = tmp[2 * m + 1], rr = ea[2 * m], ri = ea[2 * m + 1];
        VR(m) = cr * rr - ci * ri;
        VI(m) = cr * ri + ci * rr;
    }
#undef W
#undef VR
#undef VI
}

/* Euler-angle convention change, detail::convert (include/rotor.hpp:68-81). */
static void convert_angles(const double* e, int type, double* out) {
    const double a = e[0] - 0.5 * PI, b = e[1], g = e[2] + 0.5 * PI;
    if (type == 0) { out[0] = a; out[1] = b; out[2] = g; }
    else { out[0] = -g; out[1] = -b; out[2] = -a; }
}

static void phases(sz L, double angle, double* e) {
    for (sz m = 0; m < L; ++m) {
        /* std::polar(1, -m*angle) = (cos, sin) of (-m*angle) */
        const double t = -(double)m * angle;
        e[2 * m] = cos(t);
        e[2 * m + 1] = sin(t);
    }
}

/* Rotor::rotate for a real Zernike expansion (include/rotor.hpp:210-243):
 * to_complex_expansion (zernike_expansion.hpp:484-575) -- m>0 pairs {a,b}
 * become {a/sqrt2, -b/sqrt2} -- then rotate_l for n >= 1 and l in indices(1)
 * of that n (for even n the parity range starts at l = 0, so l = 0 is also
 * "rotated", which zeroes its imaginary part), then to_real_expansion
 * (zernike_expansion.hpp:577-634).  Same-convention conversion only, as the
 * rotor uses. type: 0 = object, 1 = coordinate. */
void oracle_zt_rotate(sz L, double* c, const double* euler, int type) {
    if (L == 0) return;
    const double cn = 0.70710678118654752440084436210484903; /* 1/sqrt2 */
    const double rn = 1.41421356237309504880168872420969808;
    double* d = (double*)malloc(sizeof(double) * oracle_wignerd_size(L));
    oracle_wignerd(L, d);
    double ang[3];
    convert_angles(euler, type, ang);
    double* ea = (double*)malloc(sizeof(double) * 2 * L);
    double* eb = (double*)malloc(sizeof(double) * 2 * L);
    double* eg = (double*)malloc(sizeof(double) * 2 * L);
    double* tmp = (double*)malloc(sizeof(double) * 2 * L);
    phases(L, ang[0], ea);
    phases(L, ang[1], eb);
    phases(L, ang[2], eg);
    for (sz n = 0; n < L; ++n)
        for (sz l = n & 1; l <= n; l += 2)
            for (sz m = 1; m <= l; ++m) {
                c[2 * zidx(n, l, m)] *= cn;
                c[2 * zidx(n, l, m) + 1] *= -cn;
            }
    for (sz n = 1; n < L; ++n)
        for (sz l = n & 1; l <= n; l += 2)
            rotate_l(l, c + 2 * zidx(n, l, 0), d + l * (l + 1) * (2 * l + 1) / 6, eg, eb, ea, tmp);
    for (sz n = 0; n < L; ++n)
        for (sz l = n & 1; l <= n; l += 2)
            for (sz m = 1; m <= l; ++m) {
                c[2 * zidx(n, l, m)] *= rn;
                c[2 * zidx(n, l, m) + 1] *= -rn;
            }
    free(d); free(ea); free(eb); free(eg); free(tmp);
}

/* Rotor::rotate for a real SH expansion (include/rotor.hpp:121-141), the
 * SH conversions of include/real_sh_expansion.hpp:345-436. */
void oracle_st_rotate(sz L, double* c, const double* euler, int type) {
    if (L == 0) return;
    const double cn = 0.70710678118654752440084436210484903;
    const double rn = 1.41421356237309504880168872420969808;
    double* d = (double*)malloc(sizeof(double) * oracle_wignerd_size(L));
    oracle_wignerd(L, d);
    double ang[3];
    convert_angles(euler, type, ang);
    double* ea = (double*)malloc(sizeof(double) * 2 * L);
    double* eb = (double*)malloc(sizeof(double) * 2 * L);
    double* eg = (double*)malloc(sizeof(double) * 2 * L);
    double* tmp = (double*)malloc(sizeof(double) * 2 * L);
    phases(L, ang[0], ea);
    phases(L, ang[1], eb);
    phases(L, ang[2], eg);
    for (sz l = 0; l < L; ++l)
        for (sz m = 1; m <= l; ++m) { c[2 * tri_idx(l, m)] *= cn; c[2 * tri_idx(l, m) + 1] *= -cn; }
    for (sz l = 1; l < L; ++l)
        rotate_l(l, c + 2 * tri_idx(l, 0), d + l * (l + 1) * (2 * l + 1) / 6, eg, eb, ea, tmp);
    for (sz l = 0; l < L; ++l)
        for (sz m = 1; m <= l; ++m) { c[2 * tri_idx(l, m)] *= rn; c[2 * tri_idx(l, m) + 1] *= -rn; }
    free(d); free(ea); free(eb); free(eg); free(tmp);
}

/* Rotor::polar_rotate (include/rotor.hpp:310-378): a phase e^{-i m angle'}
 * per m on the complex form; angle' = angle (object) or -angle (coordinate). */
static void polar_vec(sz l, double* v, const double* e) {
    for (sz m = 0; m <= l; ++m) {
        const double cr = v[2 * m], ci = v[2 * m + 1], rr = e[2 * m], ri = e[2 * m + 1];
        v[2 * m] = cr * rr - ci * ri;
        v[2 * m + 1] = cr * ri + ci * rr;
    }
}

void oracle_zt_polar_rotate(sz L, double* c, double angle, int type) {
    if (L == 0) return;
    const double cn = 0.70710678118654752440084436210484903;
    const double rn = 1.41421356237309504880168872420969808;
    double* e = (double*)malloc(sizeof(double) * 2 * L);
    phases(L, type == 0 ? angle : -angle, e);
    for (sz n = 0; n < L; ++n)
        for (sz l = n & 1; l <= n; l += 2)
            for (sz m = 1; m <= l; ++m) { c[2 * zidx(n, l, m)] *= cn; c[2 * zidx(n, l, m) + 1] *= -cn; }
    for (sz n = 1; n < L; ++n)
        for (sz l = n & 1; l <= n; l += 2) polar_vec(l, c + 2 * zidx(n, l, 0), e);
    for (sz n = 0; n < L; ++n)
        for (sz l = n & 1; l <= n; l += 2)
            for (sz m = 1; m <= l; ++m) { c[2 * zidx(n, l, m)] *= rn; c[2 * zidx(n, l, m) + 1] *= -rn; }
    free(e);
}

void oracle_st_polar_rotate(sz L, double* c, double angle, int type) {
    if (L == 0) return;
    const double cn = 0.70710678118654752440084436210484903;
    const double rn = 1.41421356237309504880168872420969808;
    double* e = (double*)malloc(sizeof(double) * 2 * L);
    phases(L, type == 0 ? angle : -angle, e);
    for (sz l = 0; l < L; ++l)
        for (sz m = 1; m <= l; ++m) { c[2 * tri_idx(l, m)] *= cn; c[2 * tri_idx(l, m) + 1] *= -cn; }
    for (sz l = 1; l < L; ++l) polar_vec(l, c + 2 * tri_idx(l, 0), e);
    for (sz l = 0; l < L; ++l)
        for (sz m = 1; m <= l; ++m) { c[2 * tri_idx(l, m)] *= rn; c[2 * tri_idx(l, m) + 1] *= -rn; }
    free(e);
}

/* euler_angles_from_rotation_matrix (include/rotor.hpp:53-63); row-major 3x3. */
void oracle_euler_from_matrix(const double* r, double* e) {
    const double r22sq = r[8] * r[8];
    const double by = sqrt((1.0 + r22sq) * (1.0 - r22sq));
    e[0] = atan2(r[5], r[2]);
    e[1] = atan2(by, r[8]);
    e[2] = atan2(r[7], -r[6]);
}

/* ---------------------------------------------------------------------------
 * Evaluation at arbitrary points: zt::GridEvaluator::evaluate
 * (include/grid_evaluator.hpp:228-266; sum_n :275-306, sum_l and sum_m
 * src/grid_evaluator.cpp:195-257) and st::GridEvaluator::evaluate
 * (include/grid_evaluator.hpp:84-133; sum_m src/grid_evaluator.cpp:126-151),
 * with the reference's loop orders.  cos/sin(m lon) by the recurrence of
 * detail::recursive_trig (src/grid_evaluator.cpp:43-66).  Values are laid out
 * [lon][lat][rad] (Zernike) and [lon][lat] (SH), row-major.
 */
static double* eval_trig(sz L, sz nlon, const double* lon) {
    double* t = (double*)calloc(2 * L * nlon + 2, sizeof(double));
    for (sz i = 0; i < nlon; ++i) { t[2 * i] = 1.0; t[2 * i + 1] = 0.0; }
    if (L < 2) return t;
    double* t1 = t + 2 * nlon;
    for (sz i = 0; i < nlon; ++i) { t1[2 * i] = cos(lon[i]); t1[2 * i + 1] = sin(lon[i]); }
    for (sz m = 2; m < L; ++m) {
        const double* p = t + 2 * (m - 1) * nlon;
        double* q = t + 2 * m * nlon;
        for (sz i = 0; i < nlon; ++i) {
            q[2 * i] = p[2 * i] * t1[2 * i] - p[2 * i + 1] * t1[2 * i + 1];
            q[2 * i + 1] = p[2 * i] * t1[2 * i + 1] + p[2 * i + 1] * t1[2 * i];
        }
    }
    return t;
}

void oracle_zt_evaluate(sz L, int zernike_norm, int sh_norm, int sh_phase, const double* c, sz nlon,
                        const double* lon, sz nlat, const double* colat, sz nrad, const double* rad, double* out) {
    memset(out, 0, sizeof(double) * nlon * nlat * nrad);
    if (L == 0 || nlon == 0 || nlat == 0 || nrad == 0) return;
    double* R = (double*)calloc(rad_size(L) * nrad, sizeof(double));
    oracle_radial_zernike(L, zernike_norm, nrad, rad, R);
    double* z = (double*)malloc(sizeof(double) * nlat);
    for (sz j = 0; j < nlat; ++j) z[j] = cos(colat[j]);
    double* P = (double*)calloc(tri_size(L) * nlat, sizeof(double));
    oracle_plm_real(L, sh_norm, sh_phase, nlat, z, P);
    double* T = eval_trig(L, nlon, lon);
    /* sum_n: flm[tri(l,m)][k][2] */
    double* flm = (double*)calloc(tri_size(L) * nrad * 2, sizeof(double));
    for (sz n = 0; n < L; ++n)
        for (sz l = n & 1; l <= n; l += 2)
            for (sz m = 0; m <= l; ++m) {
                const double c0 = c[2 * zidx(n, l, m)], c1 = c[2 * zidx(n, l, m) + 1];
                const double* Rnl = R + rad_idx(n, l) * nrad;
                double* f = flm + tri_idx(l, m) * nrad * 2;
                for (sz k = 0; k < nrad; ++k) { f[2 * k] += Rnl[k] * c0; f[2 * k + 1] += Rnl[k] * c1; }
            }
    /* sum_l: fm[m][j][k][2] */
    double* fm = (double*)calloc(L * nlat * nrad * 2, sizeof(double));
    for (sz l = 0; l < L; ++l)
        for (sz m = 0; m <= l; ++m) {
            const double* f = flm + tri_idx(l, m) * nrad * 2;
            const double* Plm = P + tri_idx(l, m) * nlat;
            for (sz j = 0; j < nlat; ++j) {
                const double w = Plm[j];
                double* g = fm + (m * nlat + j) * nrad * 2;
                for (sz k = 0; k < nrad; ++k) { g[2 * k] += w * f[2 * k]; g[2 * k + 1] += w * f[2 * k + 1]; }
            }
        }
    /* sum_m */
    for (sz m = 0; m < L; ++m)
        for (sz i = 0; i < nlon; ++i) {
            const double cl = T[2 * (m * nlon + i)], sl = T[2 * (m * nlon + i) + 1];
            for (sz j = 0; j < nlat; ++j) {
                const double* g = fm + (m * nlat + j) * nrad * 2;
                double* v = out + (i * nlat + j) * nrad;
                for (sz k = 0; k < nrad; ++k) v[k] += g[2 * k] * cl + g[2 * k + 1] * sl;
            }
        }
    free(R); free(z); free(P); free(T); free(flm); free(fm);
}

void oracle_st_evaluate(sz L, int sh_norm, int sh_phase, const double* c, sz nlon, const double* lon, sz nlat,
                        const double* colat, double* out) {
    memset(out, 0, sizeof(double) * nlon * nlat);
    if (L == 0 || nlon == 0 || nlat == 0) return;
    double* z = (double*)malloc(sizeof(double) * nlat);
    for (sz j = 0; j < nlat; ++j) z[j] = cos(colat[j]);
    double* P = (double*)calloc(tri_size(L) * nlat, sizeof(double));
    oracle_plm_real(L, sh_norm, sh_phase, nlat, z, P);
    double* T = eval_trig(L, nlon, lon);
    double* fm = (double*)calloc(L * nlat * 2, sizeof(double));
    for (sz l = 0; l < L; ++l)
        for (sz m = 0; m <= l; ++m) {
            const double c0 = c[2 * tri_idx(l, m)], c1 = c[2 * tri_idx(l, m) + 1];
            const double* Plm = P + tri_idx(l, m) * nlat;
            for (sz j = 0; j < nlat; ++j) { fm[2 * (m * nlat + j)] += Plm[j] * c0; fm[2 * (m * nlat + j) + 1] += Plm[j] * c1; }
        }
    for (sz m = 0; m < L; ++m)
        for (sz i = 0; i < nlon; ++i) {
            const double cl = T[2 * (m * nlon + i)], sl = T[2 * (m * nlon + i) + 1];
            for (sz j = 0; j < nlat; ++j) out[i * nlat + j] += fm[2 * (m * nlat + j)] * cl + fm[2 * (m * nlat + j) + 1] * sl;
        }
    free(z); free(P); free(T); free(fm);
}

/* ---------------------------------------------------------------------------
 * Power spectra (include/power_spectra.hpp).  norm = 1/(4 pi) (geo) or 1 (qm),
 * st::normalization (include/sh_conventions.hpp).
 */
static double sh_norm_const(int sh_norm) { return sh_norm ? 1.0 : 0.07957747154594766788444188168625718; }

/* st::cross_power_spectrum (:38-52): l < min(L, out_len - 1); other entries untouched. */
void oracle_st_cross_power_spectrum(sz L, int sh_norm, const double* a, const double* b, sz out_len, double* out) {
    const double norm = sh_norm_const(sh_norm);
    const sz nl = out_len ? (L < out_len - 1 ? L : out_len - 1) : 0;
    for (sz l = 0; l < nl; ++l) {
        out[l] = a[2 * tri_idx(l, 0)] * b[2 * tri_idx(l, 0)];
        for (sz m = 1; m <= l; ++m)
            out[l] += a[2 * tri_idx(l, m)] * b[2 * tri_idx(l, m)] + a[2 * tri_idx(l, m) + 1] * b[2 * tri_idx(l, m) + 1];
        out[l] *= norm;
    }
}

/* st::power_spectrum (:88-104): l < L. */
void oracle_st_power_spectrum(sz L, int sh_norm, const double* a, double* out) {
    oracle_st_cross_power_spectrum(L, sh_norm, a, a, L + 1, out);
}

/* zt::power_spectrum (:124-146): out[floor((n+1)^2/4) + l/2], l = n&1, .. < n
 * (the reference's bound; the l = n entries are not written). */
void oracle_zt_power_spectrum(sz L, int sh_norm, const double* c, double* out) {
    const double norm = sh_norm_const(sh_norm);
    for (sz n = 0; n < L; ++n)
        for (sz l = n & 1; l < n; l += 2) {
            double* o = out + rad_idx(n, l);
            *o = c[2 * zidx(n, l, 0)] * c[2 * zidx(n, l, 0)];
            for (sz m = 1; m <= l; ++m)
                *o += c[2 * zidx(n, l, m)] * c[2 * zidx(n, l, m)] + c[2 * zidx(n, l, m) + 1] * c[2 * zidx(n, l, m) + 1];
            *o *= norm;
        }
}
