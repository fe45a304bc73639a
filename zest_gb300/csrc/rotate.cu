// Rotations of real Zernike and SH expansions, FP64 (Rotor::rotate and
// Rotor::polar_rotate, include/rotor.hpp:121-378).
//
// Per expansion and per (n, l) vector of l+1 complex coefficients:
//   real -> complex   m > 0: {a, b} -> {a/sqrt2, -b/sqrt2}    zernike_expansion.hpp:484-575
//   rotate_l          e^{-im g'} X(pi/2) e^{-im b'} X(-pi/2) e^{-im a'}
//                                                             wignerd_collection.hpp:122-296
//   complex -> real   m > 0: {a, b} -> {a sqrt2, -b sqrt2}    zernike_expansion.hpp:577-634
// with (a', b', g') = detail::convert(euler, type), rotor.hpp:68-81.
//
// X(pi/2) in the reference uses the parity structure of d^l(pi/2) and of the
// complex coefficients of a real function: output m with q = (l+m) & 1 takes
//   Re <- 1/2 d(m,0) Re v_0 + sum_{m' >= 1, m'+q even} d(m,m') Re v_m'
//   Im <-                     sum_{m' >= 1, m'+q odd } d(m,m') Im v_m'
// (times 2), and X(-pi/2) the same with d transposed.  One warp owns one
// vector; each lane computes whole outputs.  d(m,m') is read as
// (-1)^(m+m') d(m',m) so that consecutive lanes read consecutive addresses.
//
// Zernike vectors are n >= 1 and l in the parity range of n starting at 0
// for even n (the reference's indices(1) rounds down, so l = 0 is "rotated",
// which zeroes Im c_{n00}); SH vectors are l >= 1.
#include "common.cuh"
#include "kernels.cuh"

namespace zgpu {

namespace {

constexpr int MAXL = 2048;  // longest vector (order) supported

// warps per CTA: two shared buffers of L complex per warp within ~96 KB
inline int warps_for(int L) {
    int w = 8;
    while (w > 1 && (size_t)w * 2 * L * 16 > 96 * 1024) --w;
    return w;
}

__device__ __forceinline__ void convert_angles(const double* e, int type, double& a, double& b, double& g) {
    const double pi = 3.14159265358979323846264338327950288;
    const double ar = e[0] - 0.5 * pi, br = e[1], gr = e[2] + 0.5 * pi;
    if (type == 0) { a = ar; b = br; g = gr; }
    else { a = -gr; b = -br; g = -ar; }
}

// phases[b][k][m] = e^{-i m angle_k}, k = alpha, beta, gamma
__global__ void phase_kernel(int L, int batch, const double* __restrict__ euler, int type, double2* __restrict__ ph) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (m >= L || b >= batch) return;
    double ang[3];
    convert_angles(euler + 3 * b, type, ang[0], ang[1], ang[2]);
    for (int k = 0; k < 3; ++k) {
        double s, c;
        sincos(-double(m) * ang[k], &s, &c);
        ph[((long long)b * 3 + k) * L + m] = make_double2(c, s);
    }
}

__device__ __forceinline__ double2 cmul(double2 c, double2 r) {
    return make_double2(c.x * r.x - c.y * r.y, c.x * r.y + c.y * r.x);
}

// X(+-pi/2) output m of the vector v (length l+1) in shared memory.
// transpose = false: first rotation (d), true: second rotation (d^T).
__device__ __forceinline__ double2 xrot(const double2* v, const double* __restrict__ d, int l, int m, bool transpose) {
    const int ld = l + 1;
    const int q = (l + m) & 1;
    // d(m, m') = sgn d(m', m) for the first rotation; d(m', m) for the second
    auto D = [&](int mp) {
        const double x = d[ld * mp + m];
        return (!transpose && ((m + mp) & 1)) ? -x : x;
    };
    double re = 0.5 * D(0) * v[0].x;
    double im = 0.0;
    for (int mp = q ? 1 : 2; mp <= l; mp += 2) re = fma(D(mp), v[mp].x, re);
    for (int mp = q ? 2 : 1; mp <= l; mp += 2) im = fma(D(mp), v[mp].y, im);
    return make_double2(2.0 * re, 2.0 * im);
}

// First coefficient of vector (n, l): Zernike tetrahedral layout (kind 0),
// SH triangle (kind 1) or row-skipping triangle, floor(l^2 / 4) (kind 2).
__device__ __forceinline__ long long vec_base(int kind, int n, int l) {
    return kind == 0 ? zidx(n, l, 0) : kind == 1 ? tri_idx(l, 0) : ((long long)l * l) >> 2;
}

// vec_list[v] = {n, l} (Zernike) or {l, l} (SH); vectors of item b are v + b*nvec
__global__ void rotate_kernel(int L, int nvec, int batch, double* __restrict__ coeffs, long long cstride, int kind,
                              const int2* __restrict__ vec_list, const double* __restrict__ wig,
                              const double2* __restrict__ ph) {
    extern __shared__ double2 rbuf[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = blockDim.x >> 5;
    const long long vid = (long long)blockIdx.x * W + warp;
    if (vid >= (long long)nvec * batch) return;
    const int b = int(vid / nvec);
    const int2 nl = vec_list[vid - (long long)b * nvec];
    const int n = nl.x, l = nl.y;
    double* c = coeffs + b * cstride + 2 * vec_base(kind, n, l);
    const double2* pa = ph + ((long long)b * 3 + 0) * L;
    const double2* pb = ph + ((long long)b * 3 + 1) * L;
    const double2* pg = ph + ((long long)b * 3 + 2) * L;
    const double* d = wig + wig_off(l);
    double2* v = rbuf + (size_t)warp * 2 * L;
    double2* t = v + L;
    const double isq2 = 1.0 / 1.41421356237309504880168872420969808;
    const double sq2 = 1.41421356237309504880168872420969808;
    // real -> complex, gamma phase
    for (int m = lane; m <= l; m += 32) {
        double2 x = make_double2(c[2 * m], c[2 * m + 1]);
        if (m > 0) { x.x *= isq2; x.y *= -isq2; }
        v[m] = cmul(x, pg[m]);
    }
    __syncwarp();
    for (int m = lane; m <= l; m += 32) t[m] = xrot(v, d, l, m, false);
    __syncwarp();
    for (int m = lane; m <= l; m += 32) v[m] = cmul(t[m], pb[m]);
    __syncwarp();
    for (int m = lane; m <= l; m += 32) t[m] = xrot(v, d, l, m, true);
    __syncwarp();
    for (int m = lane; m <= l; m += 32) {
        double2 x = cmul(t[m], pa[m]);
        if (m > 0) { x.x *= sq2; x.y *= -sq2; }
        c[2 * m] = x.x;
        c[2 * m + 1] = x.y;
    }
}

// Rotations of many expansions of different orders in one launch: one warp
// per entry {item, n, l} of a ragged work list, coefficients of item i at
// coeffs + coff[i], phase tables of stride Lmax.
__global__ void rotate_ragged_kernel(int Lmax, long long nwork, double* __restrict__ coeffs,
                                     const long long* __restrict__ coff, const int4* __restrict__ work, int kind,
                                     const double* __restrict__ wig, const double2* __restrict__ ph) {
    extern __shared__ double2 rbuf2[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = blockDim.x >> 5;
    const long long wid = (long long)blockIdx.x * W + warp;
    if (wid >= nwork) return;
    const int4 w = work[wid];
    const int b = w.x, n = w.y, l = w.z;
    double* c = coeffs + coff[b] + 2 * vec_base(kind, n, l);
    const double2* pa = ph + ((long long)b * 3 + 0) * Lmax;
    const double2* pb = ph + ((long long)b * 3 + 1) * Lmax;
    const double2* pg = ph + ((long long)b * 3 + 2) * Lmax;
    const double* d = wig + wig_off(l);
    double2* v = rbuf2 + (size_t)warp * 2 * Lmax;
    double2* t = v + Lmax;
    const double isq2 = 1.0 / 1.41421356237309504880168872420969808;
    const double sq2 = 1.41421356237309504880168872420969808;
    for (int m = lane; m <= l; m += 32) {
        double2 x = make_double2(c[2 * m], c[2 * m + 1]);
        if (m > 0) { x.x *= isq2; x.y *= -isq2; }
        v[m] = cmul(x, pg[m]);
    }
    __syncwarp();
    for (int m = lane; m <= l; m += 32) t[m] = xrot(v, d, l, m, false);
    __syncwarp();
    for (int m = lane; m <= l; m += 32) v[m] = cmul(t[m], pb[m]);
    __syncwarp();
    for (int m = lane; m <= l; m += 32) t[m] = xrot(v, d, l, m, true);
    __syncwarp();
    for (int m = lane; m <= l; m += 32) {
        double2 x = cmul(t[m], pa[m]);
        if (m > 0) { x.x *= sq2; x.y *= -sq2; }
        c[2 * m] = x.x;
        c[2 * m + 1] = x.y;
    }
}

// Derivative of the rotated expansion with respect to the three converted
// angles (alpha', beta', gamma'), contracted with a cotangent ybar: per rotated
// vector, part[v][k] = <ybar, d rotate(x) / d angle_k> over the vector's real
// coefficients.  The rotation is E_a' X(-pi/2) E_b' X(pi/2) E_g' with
// E_t = diag(e^{-i m t}); d/dt of E_t is (-i m) E_t, carried forward through
// the remaining stages (five X applications instead of two).
__global__ void rotate_grad_kernel(int L, int nvec, int batch, const double* __restrict__ x,
                                   const double* __restrict__ ybar, long long cstride, int kind,
                                   const int2* __restrict__ vec_list, const double* __restrict__ wig,
                                   const double2* __restrict__ ph, double* __restrict__ part) {
    extern __shared__ double2 gbuf[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = blockDim.x >> 5;
    const long long vid = (long long)blockIdx.x * W + warp;
    if (vid >= (long long)nvec * batch) return;
    const int b = int(vid / nvec);
    const int2 nl = vec_list[vid - (long long)b * nvec];
    const int n = nl.x, l = nl.y;
    const long long off = b * cstride + 2 * vec_base(kind, n, l);
    const double* c = x + off;
    const double* yb = ybar + off;
    const double2* pa = ph + ((long long)b * 3 + 0) * L;
    const double2* pb = ph + ((long long)b * 3 + 1) * L;
    const double2* pg = ph + ((long long)b * 3 + 2) * L;
    const double* d = wig + wig_off(l);
    double2* A = gbuf + (size_t)warp * 4 * L;
    double2* B = A + L;
    double2* C = B + L;
    double2* D = C + L;
    const double isq2 = 1.0 / 1.41421356237309504880168872420969808;
    const double sq2 = 1.41421356237309504880168872420969808;
    // (-i m) z
    auto dphi = [](double2 z, int m) { return make_double2(double(m) * z.y, -double(m) * z.x); };
    for (int m = lane; m <= l; m += 32) {
        double2 v = make_double2(c[2 * m], c[2 * m + 1]);
        if (m > 0) { v.x *= isq2; v.y *= -isq2; }
        A[m] = cmul(v, pg[m]);
        B[m] = dphi(A[m], m);
    }
    __syncwarp();
    for (int m = lane; m <= l; m += 32) {
        C[m] = xrot(A, d, l, m, false);
        D[m] = xrot(B, d, l, m, false);
    }
    __syncwarp();
    for (int m = lane; m <= l; m += 32) {
        A[m] = cmul(C[m], pb[m]);
        B[m] = dphi(A[m], m);
        C[m] = cmul(D[m], pb[m]);
    }
    __syncwarp();
    double sa = 0.0, sb = 0.0, sg = 0.0;
    for (int m = lane; m <= l; m += 32) {
        const double2 w5 = cmul(xrot(A, d, l, m, true), pa[m]);
        const double2 ta = dphi(w5, m);
        const double2 tb = cmul(xrot(B, d, l, m, true), pa[m]);
        const double2 tg = cmul(xrot(C, d, l, m, true), pa[m]);
        // <ybar, real(t)>: real(t) = (Re t, Im t) at m = 0, sqrt2 (Re t, -Im t) above
        const double ya = yb[2 * m], yi = yb[2 * m + 1];
        if (m == 0) {
            sa += ya * ta.x + yi * ta.y;
            sb += ya * tb.x + yi * tb.y;
            sg += ya * tg.x + yi * tg.y;
        } else {
            sa += sq2 * (ya * ta.x - yi * ta.y);
            sb += sq2 * (ya * tb.x - yi * tb.y);
            sg += sq2 * (ya * tg.x - yi * tg.y);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        sa += __shfl_xor_sync(0xffffffffu, sa, o);
        sb += __shfl_xor_sync(0xffffffffu, sb, o);
        sg += __shfl_xor_sync(0xffffffffu, sg, o);
    }
    if (lane == 0) {
        double* pv = part + vid * 3;
        pv[0] = sa;
        pv[1] = sb;
        pv[2] = sg;
    }
}

// Per expansion: the sum over its vectors of the angle partials (fixed order,
// so the result does not depend on scheduling), mapped back from the
// converted angles to the Euler angles of the call (rotor.hpp:68-81):
// object (a', b', g') = (a - pi/2, b, g + pi/2); coordinate (-g - pi/2, -b, -a + pi/2).
__global__ void euler_grad_reduce_kernel(int nvec, const double* __restrict__ part, int type,
                                         double* __restrict__ grad) {
    __shared__ double red[3][256];
    const int b = blockIdx.x;
    double s[3] = {0.0, 0.0, 0.0};
    for (int v = threadIdx.x; v < nvec; v += blockDim.x)
        for (int k = 0; k < 3; ++k) s[k] += part[((long long)b * nvec + v) * 3 + k];
    for (int k = 0; k < 3; ++k) red[k][threadIdx.x] = s[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double da = red[0][0], db = red[1][0], dg = red[2][0];
        double* g = grad + 3 * (long long)b;
        if (type == 0) {
            g[0] = da;
            g[1] = db;
            g[2] = dg;
        } else {
            g[0] = -dg;
            g[1] = -db;
            g[2] = -da;
        }
    }
}

// Euler angles of the inverse rotation, for either convention: (-g, -b, -a).
__global__ void invert_euler_kernel(int batch, const double* __restrict__ e, double* __restrict__ out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= batch) return;
    const double a = e[3 * b], be = e[3 * b + 1], g = e[3 * b + 2];
    out[3 * b] = -g;
    out[3 * b + 1] = -be;
    out[3 * b + 2] = -a;
}

__global__ void polar_kernel(int L, int nvec, int batch, double* __restrict__ coeffs, long long cstride, int kind,
                             const int2* __restrict__ vec_list, const double* __restrict__ angles, int type) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long vid = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
    if (vid >= (long long)nvec * batch) return;
    const int b = int(vid / nvec);
    const int2 nl = vec_list[vid - (long long)b * nvec];
    const int n = nl.x, l = nl.y;
    double* c = coeffs + b * cstride + 2 * vec_base(kind, n, l);
    const double ang = type == 0 ? angles[b] : -angles[b];
    const double isq2 = 1.0 / 1.41421356237309504880168872420969808;
    const double sq2 = 1.41421356237309504880168872420969808;
    for (int m = lane; m <= l; m += 32) {
        double2 x = make_double2(c[2 * m], c[2 * m + 1]);
        if (m > 0) { x.x *= isq2; x.y *= -isq2; }
        double s, co;
        sincos(-double(m) * ang, &s, &co);
        x = cmul(x, make_double2(co, s));
        if (m > 0) { x.x *= sq2; x.y *= -sq2; }
        c[2 * m] = x.x;
        c[2 * m + 1] = x.y;
    }
}

}  // namespace

int launch_rotate_vectors(cudaStream_t s, int kind, int L, int batch, double* coeffs, long long cstride,
                          const int2* vec_list, int nvec, const double* wigner, const double* euler, int type,
                          double* phase_scratch) {
    if (batch <= 0 || nvec <= 0) return ZEST_GPU_OK;
    if (L > MAXL) return fail(ZEST_GPU_ERR_UNSUPPORTED, "rotation order above 2048");
    double2* ph = reinterpret_cast<double2*>(phase_scratch);
    phase_kernel<<<dim3((L + 127) / 128, batch), 128, 0, s>>>(L, batch, euler, type, ph);
    ZG_TRY(launch_check("phase_kernel"));
    const long long total = (long long)nvec * batch;
    const int W = warps_for(L);
    const size_t smem = (size_t)W * 2 * L * sizeof(double2);
    ZG_CUDA_TRY(cudaFuncSetAttribute(rotate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
    rotate_kernel<<<(unsigned)((total + W - 1) / W), W * 32, smem, s>>>(L, nvec, batch, coeffs, cstride, kind,
                                                                        vec_list, wigner, ph);
    return launch_check("rotate_kernel");
}

int launch_rotate_euler_grad(cudaStream_t s, int kind, int L, int batch, const double* x, const double* ybar,
                             long long cstride, const int2* vec_list, int nvec, const double* wigner,
                             const double* euler, int type, double* phase_scratch, double* part, double* grad) {
    if (batch <= 0) return ZEST_GPU_OK;
    if (L > 1024) return fail(ZEST_GPU_ERR_UNSUPPORTED, "rotation gradient: order above 1024");
    if (nvec <= 0) {
        ZG_CUDA_TRY(cudaMemsetAsync(grad, 0, (size_t)batch * 3 * sizeof(double), s));
        return ZEST_GPU_OK;
    }
    double2* ph = reinterpret_cast<double2*>(phase_scratch);
    phase_kernel<<<dim3((L + 127) / 128, batch), 128, 0, s>>>(L, batch, euler, type, ph);
    ZG_TRY(launch_check("phase_kernel"));
    // four vectors of L complex per warp within ~96 KB
    int W = 8;
    while (W > 1 && (size_t)W * 4 * L * 16 > 96 * 1024) --W;
    const size_t smem = (size_t)W * 4 * L * sizeof(double2);
    ZG_CUDA_TRY(cudaFuncSetAttribute(rotate_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
    const long long total = (long long)nvec * batch;
    rotate_grad_kernel<<<(unsigned)((total + W - 1) / W), W * 32, smem, s>>>(L, nvec, batch, x, ybar, cstride, kind,
                                                                            vec_list, wigner, ph, part);
    ZG_TRY(launch_check("rotate_grad_kernel"));
    euler_grad_reduce_kernel<<<batch, 256, 0, s>>>(nvec, part, type, grad);
    return launch_check("euler_grad_reduce_kernel");
}

int launch_rotate_ragged(cudaStream_t s, int kind, int Lmax, int items, double* coeffs, const long long* coff,
                         const int4* work, long long nwork, const double* wigner, const double* euler, int type,
                         double* phase_scratch) {
    if (items <= 0 || nwork <= 0) return ZEST_GPU_OK;
    if (Lmax > MAXL) return fail(ZEST_GPU_ERR_UNSUPPORTED, "rotation order above 2048");
    double2* ph = reinterpret_cast<double2*>(phase_scratch);
    phase_kernel<<<dim3((Lmax + 127) / 128, items), 128, 0, s>>>(Lmax, items, euler, type, ph);
    ZG_TRY(launch_check("phase_kernel"));
    const int W = warps_for(Lmax);
    const size_t smem = (size_t)W * 2 * Lmax * sizeof(double2);
    ZG_CUDA_TRY(cudaFuncSetAttribute(rotate_ragged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
    rotate_ragged_kernel<<<(unsigned)((nwork + W - 1) / W), W * 32, smem, s>>>(Lmax, nwork, coeffs, coff, work, kind,
                                                                              wigner, ph);
    return launch_check("rotate_ragged_kernel");
}

int launch_phases(cudaStream_t s, int Lmax, int items, const double* euler, int type, double* phase_scratch) {
    if (items <= 0 || Lmax <= 0) return ZEST_GPU_OK;
    phase_kernel<<<dim3((Lmax + 127) / 128, items), 128, 0, s>>>(Lmax, items, euler, type,
                                                                reinterpret_cast<double2*>(phase_scratch));
    return launch_check("phase_kernel");
}

int launch_invert_euler(cudaStream_t s, int batch, const double* euler, double* out) {
    if (batch <= 0) return ZEST_GPU_OK;
    invert_euler_kernel<<<(batch + 127) / 128, 128, 0, s>>>(batch, euler, out);
    return launch_check("invert_euler_kernel");
}

int launch_polar_vectors(cudaStream_t s, int kind, int L, int batch, double* coeffs, long long cstride,
                         const int2* vec_list, int nvec, const double* angles, int type) {
    if (batch <= 0 || nvec <= 0) return ZEST_GPU_OK;
    const long long total = (long long)nvec * batch;
    polar_kernel<<<(unsigned)((total + 7) / 8), 8 * 32, 0, s>>>(L, nvec, batch, coeffs, cstride, kind, vec_list,
                                                               angles, type);
    return launch_check("polar_kernel");
}

}  // namespace zgpu
