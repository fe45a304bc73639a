// Batched real DFT along the longitude axis, FP64, in shared memory.
//
// Replaces pocketfft::r2c / c2r as called by the reference transformers
// (zernike_glq_transformer.hpp:710-720 and 943-949, sh_glq_transformer.hpp:
// 757-765 and 1195-1201).  The longitude count is odd (2L-1: 39, 399, 2047,
// ...) or a multiple of 8 (LatLon layout), so the kernel is a mixed-radix
// Stockham FFT with a generic radix-R stage: every thread computes whole
// outputs of a stage, out = sum_r in[j + r N/R] W^(r (j%Ns + q Ns) N/(Ns R)),
// which reads its R inputs from shared memory and needs no bit reversal.
//
// Each CTA transforms 2*NC real columns packed as NC complex columns
// (z = x_a + i x_b); the real spectra are separated at the end.  Columns are
// the contiguous (lat, rad) points of one longitude row, so every global load
// and store is coalesced.
//
// Forward output  F[b][m][col][2] = conj(X_m(col)), m < nm (no scaling; the
//                 quadrature prefactor lives in the Legendre tables).
// Inverse input   F[b][m][col][2] = Hermitian coefficients of m < nm; output
//                 x_i = Re F_0 + 2 sum_{m>0} Re(F_m e^{+2 pi i im/N}) -- the
//                 c2r semantics with factor 1.
#include "common.cuh"
#include "kernels.cuh"

namespace zgpu {

namespace {

__device__ __forceinline__ double2 cmul_tw(double2 a, double2 w, bool conj) {
    if (conj) w.y = -w.y;
    return make_double2(fma(a.x, w.x, -a.y * w.y), fma(a.x, w.y, a.y * w.x));
}

// One Stockham pass for all NC columns: src -> dst, twiddle table tw (size N,
// W_t = e^{-2 pi i t/N}; conjugated for the inverse transform).  Butterfly
// (j, column) of radix R takes x_r = src[j + r N/R], twiddles it,
// t_r = x_r W^{r jm step}, and forms the R-point DFT
//     y_q = sum_r t_r W_R^{r q} -> dst[(j/Ns) Ns R + jm + q Ns].
// Radix 2 and 4 are done per butterfly.  An odd radix pairs the outputs q and
// R - q: with s_r = t_r + t_{R-r}, d_r = t_r - t_{R-r} (r = 1..(R-1)/2),
//     y_q = a -+ i b,  y_{R-q} = a +- i b,  a = t_0 + sum_r s_r cos(2 pi r q/R),
//     b = sum_r d_r sin(2 pi r q/R)
// (upper signs forward): R - 1 multiply-adds per output instead of 4 R.
// Phase A (per butterfly) twiddles and writes s_r, d_r back in place --
// every src element belongs to exactly one butterfly -- and stores y_0;
// phase B computes the output pairs, one (butterfly, q) per thread.
__device__ __forceinline__ void stockham_stage(double2* __restrict__ src, double2* __restrict__ dst,
                                               const double2* __restrict__ tw, int N, int R, int Ns, int NC,
                                               bool inverse) {
    const int NR = N / R;
    const int step = N / (Ns * R);
    const int wR = N / R;  // W_R^m = tw[wR m]
    const size_t xs = (size_t)NR * NC;
    const int nb = NR * NC;
    for (int o = threadIdx.x; o < nb; o += blockDim.x) {
        const int cp = o % NC;
        const int j = o / NC;
        const int jm = j % Ns;
        const int obase = (j / Ns) * Ns * R + jm;
        double2* x = src + (size_t)j * NC + cp;
        const int tstep = jm * step;
        int t = tstep;
        for (int r = 1; r < R; ++r) {
            x[r * xs] = cmul_tw(x[r * xs], tw[t], inverse);
            t += tstep;
            if (t >= N) t -= N;
        }
        if (R == 2) {
            const double2 a = x[0], b = x[xs];
            dst[(size_t)obase * NC + cp] = make_double2(a.x + b.x, a.y + b.y);
            dst[(size_t)(obase + Ns) * NC + cp] = make_double2(a.x - b.x, a.y - b.y);
        } else if (R == 4) {
            const double2 a = x[0], b = x[xs], c = x[2 * xs], d = x[3 * xs];
            const double2 s0 = make_double2(a.x + c.x, a.y + c.y), d0 = make_double2(a.x - c.x, a.y - c.y);
            const double2 s1 = make_double2(b.x + d.x, b.y + d.y), d1 = make_double2(b.x - d.x, b.y - d.y);
            // forward: y1 = d0 - i d1, y3 = d0 + i d1 (signs of i swapped for the inverse)
            const double2 md1 = inverse ? make_double2(-d1.y, d1.x) : make_double2(d1.y, -d1.x);  // -+ i d1
            dst[(size_t)obase * NC + cp] = make_double2(s0.x + s1.x, s0.y + s1.y);
            dst[(size_t)(obase + Ns) * NC + cp] = make_double2(d0.x + md1.x, d0.y + md1.y);
            dst[(size_t)(obase + 2 * Ns) * NC + cp] = make_double2(s0.x - s1.x, s0.y - s1.y);
            dst[(size_t)(obase + 3 * Ns) * NC + cp] = make_double2(d0.x - md1.x, d0.y - md1.y);
        } else {
            const int h = R >> 1;
            double2 y0 = x[0];
            for (int r = 1; r <= h; ++r) {
                const double2 a = x[r * xs], b = x[(R - r) * xs];
                const double2 sr = make_double2(a.x + b.x, a.y + b.y);
                x[r * xs] = sr;
                x[(R - r) * xs] = make_double2(a.x - b.x, a.y - b.y);
                y0.x += sr.x;
                y0.y += sr.y;
            }
            dst[(size_t)obase * NC + cp] = y0;
        }
    }
    if (R == 2 || R == 4) return;
    __syncthreads();
    const int h = R >> 1;
    const int np = nb * h;
    for (int o = threadIdx.x; o < np; o += blockDim.x) {
        const int bq = o / h;
        const int q = o - bq * h + 1;
        const int cp = bq % NC;
        const int j = bq / NC;
        const int jm = j % Ns;
        const int obase = (j / Ns) * Ns * R + jm;
        const double2* x = src + (size_t)j * NC + cp;
        double2 a = x[0], b = make_double2(0.0, 0.0);
        int m = q;
        for (int r = 1; r <= h; ++r) {
            const double2 w = tw[wR * m];  // cos(2 pi m/R), -sin(2 pi m/R)
            const double2 sr = x[r * xs], dr = x[(R - r) * xs];
            a.x = fma(sr.x, w.x, a.x);
            a.y = fma(sr.y, w.x, a.y);
            b.x = fma(dr.x, -w.y, b.x);
            b.y = fma(dr.y, -w.y, b.y);
            m += q;
            if (m >= R) m -= R;
        }
        // forward: y_q = a - i b, y_{R-q} = a + i b; inverse: the other way round
        const double2 mib = inverse ? make_double2(-b.y, b.x) : make_double2(b.y, -b.x);  // -+ i b
        dst[(size_t)(obase + q * Ns) * NC + cp] = make_double2(a.x + mib.x, a.y + mib.y);
        dst[(size_t)(obase + (R - q) * Ns) * NC + cp] = make_double2(a.x - mib.x, a.y - mib.y);
    }
}

__device__ __forceinline__ double2* run_stages(double2* a, double2* b, const double2* tw, const FftPlan& plan, int NC,
                                               bool inverse) {
    int Ns = 1;
    for (int s = 0; s < plan.nst; ++s) {
        const int R = plan.radix[s];
        stockham_stage(a, b, tw, plan.N, R, Ns, NC, inverse);
        __syncthreads();
        double2* t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// x(b, i, col) = x + b*xb + i*si + col*sc ; lon_fast: i is the contiguous axis
__global__ void rfft_fwd_kernel(FftPlan plan, const double* __restrict__ x, long long xb, long long si,
                                long long sc, int C, int nm, int NC, int lon_fast, double* __restrict__ F) {
    extern __shared__ double2 smem[];
    const int N = plan.N;
    double2* tw = smem;
    double2* A = smem + N;
    double2* Bf = A + (size_t)N * NC;
    const int b = blockIdx.y;
    const int col0 = blockIdx.x * 2 * NC;
    for (int t = threadIdx.x; t < N; t += blockDim.x) tw[t] = plan.tw[t];
    const double* xbp = x + (long long)b * xb;
    double* Ad = reinterpret_cast<double*>(A);
    const int W = 2 * NC;
    for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
        int i, cl;
        if (lon_fast) { i = e % N; cl = e / N; }
        else { cl = e % W; i = e / W; }
        const int col = col0 + cl;
        const double v = (col < C) ? xbp[(long long)i * si + (long long)col * sc] : 0.0;
        Ad[(i * NC + (cl >> 1)) * 2 + (cl & 1)] = v;
    }
    __syncthreads();
    const double2* Z = run_stages(A, Bf, tw, plan, NC, false);
    // separate the two real spectra and store conj(X_m), m < nm
    for (int e = threadIdx.x; e < nm * NC; e += blockDim.x) {
        const int cp = e % NC;
        const int m = e / NC;
        const double2 z = Z[m * NC + cp];
        const double2 zn = Z[((N - m) % N) * NC + cp];
        // X_a = (Z_m + conj Z_{N-m}) / 2,  X_b = (Z_m - conj Z_{N-m}) / (2i)
        const double2 xa = make_double2(0.5 * (z.x + zn.x), 0.5 * (z.y - zn.y));
        const double2 xbv = make_double2(0.5 * (z.y + zn.y), 0.5 * (zn.x - z.x));
        const int col = col0 + 2 * cp;
        double* out = F + (((long long)b * nm + m) * C + col) * 2;
        if (col < C) { out[0] = xa.x; out[1] = -xa.y; }
        if (col + 1 < C) { out[2] = xbv.x; out[3] = -xbv.y; }
    }
}

__global__ void rfft_inv_kernel(FftPlan plan, const double* __restrict__ F, int C, int nm, int NC, int lon_fast,
                                double* __restrict__ x, long long xb, long long si, long long sc) {
    extern __shared__ double2 smem[];
    const int N = plan.N;
    double2* tw = smem;
    double2* A = smem + N;
    double2* Bf = A + (size_t)N * NC;
    const int b = blockIdx.y;
    const int col0 = blockIdx.x * 2 * NC;
    for (int t = threadIdx.x; t < N; t += blockDim.x) tw[t] = plan.tw[t];
    // Hermitian completion of the two packed spectra
    for (int e = threadIdx.x; e < N * NC; e += blockDim.x) A[e] = make_double2(0.0, 0.0);
    __syncthreads();
    for (int e = threadIdx.x; e < nm * NC; e += blockDim.x) {
        const int cp = e % NC;
        const int m = e / NC;
        const int col = col0 + 2 * cp;
        const double* in = F + (((long long)b * nm + m) * C + col) * 2;
        const double2 fa = (col < C) ? make_double2(in[0], in[1]) : make_double2(0.0, 0.0);
        const double2 fb = (col + 1 < C) ? make_double2(in[2], in[3]) : make_double2(0.0, 0.0);
        if (m == 0) {
            A[cp] = make_double2(fa.x, fb.x);
        } else {
            A[m * NC + cp] = make_double2(fa.x - fb.y, fa.y + fb.x);
            A[(N - m) * NC + cp] = make_double2(fa.x + fb.y, fb.x - fa.y);
        }
    }
    __syncthreads();
    const double2* Z = run_stages(A, Bf, tw, plan, NC, true);
    const double* Zd = reinterpret_cast<const double*>(Z);
    double* xbp = x + (long long)b * xb;
    const int W = 2 * NC;
    for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
        int i, cl;
        if (lon_fast) { i = e % N; cl = e / N; }
        else { cl = e % W; i = e / W; }
        const int col = col0 + cl;
        if (col < C) xbp[(long long)i * si + (long long)col * sc] = Zd[(i * NC + (cl >> 1)) * 2 + (cl & 1)];
    }
}

int choose_nc(int N) {
    // two ping-pong buffers + twiddles within ~110 KB keeps 2 CTAs per SM
    int nc = 8;
    while (nc > 1 && (size_t)N * 16 * (1 + 2 * nc) > 110 * 1024) --nc;
    return nc;
}

}  // namespace

size_t fft_smem_bytes(int N, int NC) { return (size_t)N * 16 * (1 + 2 * (size_t)NC); }

int launch_rfft_fwd(cudaStream_t s, const FftPlan& plan, const double* x, long long xb, long long si, long long sc,
                    int C, int nm, int batch, int lon_fast, double* F) {
    if (batch <= 0 || C <= 0 || nm <= 0) return ZEST_GPU_OK;
    const int NC = choose_nc(plan.N);
    const size_t smem = fft_smem_bytes(plan.N, NC);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(rfft_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        cudaFuncSetAttribute(rfft_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        attr = true;
    }
    dim3 grid((C + 2 * NC - 1) / (2 * NC), batch);
    rfft_fwd_kernel<<<grid, 256, smem, s>>>(plan, x, xb, si, sc, C, nm, NC, lon_fast, F);
    return launch_check("rfft_fwd_kernel");
}

int launch_rfft_inv(cudaStream_t s, const FftPlan& plan, const double* F, int C, int nm, int batch, int lon_fast,
                    double* x, long long xb, long long si, long long sc) {
    if (batch <= 0 || C <= 0) return ZEST_GPU_OK;
    const int NC = choose_nc(plan.N);
    const size_t smem = fft_smem_bytes(plan.N, NC);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(rfft_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        cudaFuncSetAttribute(rfft_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        attr = true;
    }
    dim3 grid((C + 2 * NC - 1) / (2 * NC), batch);
    rfft_inv_kernel<<<grid, 256, smem, s>>>(plan, F, C, nm, NC, lon_fast, x, xb, si, sc);
    return launch_check("rfft_inv_kernel");
}

}  // namespace zgpu
