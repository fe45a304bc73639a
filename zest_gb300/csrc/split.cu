// Split-precision form of the GLQ contractions on tcgen05 tensor cores: every
// Zernike contraction and the SH Legendre sums.
//
// Every dense contraction -- the longitude DFT of the Zernike path (as a
// matrix product with the cos/sin table, folded over x_i +- x_{N-i}), the
// folded Legendre sums and the radial sums -- is evaluated as
//     C[r, n] = sum_k A[r, k] B[n, k]
// with FP64 operands represented in BF16 fixed-point slices:
//   * each operand row gets an exponent e (|x| < 2^(e-1) over the row) and
//     its values are rounded to v = round(x 2^{8S - e}) (ties away from zero);
//   * v is cut into S balanced base-256 digits d_s in [-128, 127] (the
//     leading one in [-128, 128]), each exact in BF16;
//   * the products d_s(A) d_t(B) with s + t = level <= S - 1 (21 products at
//     S = 6) accumulate in FP32 TMEM accumulators, one per level.  A product
//     is at most 2^14, so a level with p products is exact while
//     p K 2^14 <= 2^24: levels 0..3 are exact for sums of up to 256 terms;
//     levels 4 and 5 (2^-32 and 2^-40 of level 0) hold integers rounded to
//     their FP32 spacing once they pass 2^24.  Longer sums run as K-chunks of
//     at most 256 terms; every chunk after the first adds its FP64 result
//     through the accumulating form of the stage's epilogue;
//   * the epilogue recombines the S accumulators by integer Horner into an
//     int64 T and builds the FP64 result 2^{eA + eB - 8 (S + 1)} T with
//     integer operations only.
// Only the tables (P_lm, R_nl, cos/sin) are prepared in FP64.
//
// Kernel: warp-specialised, persistent, one CTA per SM.  Warp 0 issues TMA
// loads (SWIZZLE_32B, one 16-wide K block of the S slices of both operands
// per pipeline stage, the B slices back to back), warp 1 issues tcgen05.mma
// (M = 128 operand rows; the products of one A slice with consecutive B
// slices go to consecutive accumulators, so up to 256 / NT of them form one
// MMA of N = g NT: 9 MMAs per K block at NT = 80), warps 2..17 read the
// accumulators back (tcgen05.ld, four warps per TMEM lane quarter),
// recombine and store through a stage-specific epilogue.  Six accumulators
// of NT = 80 columns fill the 512 TMEM columns; with NT = 32 (or 16) two sets
// fit, so that the next tile's MMAs overlap the drain.  For the SH sums the
// table is the 128-row operand and the 2 x batch data rows are the columns.
// Every wait is bounded (about 2 s); on timeout the kernel records an error
// code and winds down instead of hanging.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>
#include <set>
#include <type_traits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "context.cuh"
#include "split.cuh"

namespace zgpu {

// ===========================================================================
// Device helpers (inline PTX)
// ===========================================================================
namespace {

constexpr int SP_EPI_WARPS = 16;                  // epilogue warps: four per TMEM lane quarter
constexpr int SP_THREADS = 32 * (2 + SP_EPI_WARPS);  // + TMA producer + MMA issuer
constexpr int SP_M = 128;
constexpr int SP_MIXED = 1;      // narrow threshold value that selects mixed 80/32-column launches
constexpr int SP_KB = 16;        // K elements per pipeline stage (32 bytes of bf16)
constexpr long long SP_TIMEOUT_NS = 2000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long gtime() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
        "r"(bytes)
        : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
        : "memory");
}
// One test of an mbarrier phase.  A thread whose phase is not complete is
// suspended until it completes or for at most 20 us, so that waiting warps
// take no issue slots from the working ones.
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(20000u)
        : "memory");
    return ok != 0;
}
// Bounded wait on an mbarrier phase; false (and the error flag set) on timeout
// or when another role already gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code,
                                          long long limit_ns = SP_TIMEOUT_NS) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = gtime();
    for (unsigned it = 1;; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 255) == 0) {
            if (*(volatile int*)err) return false;
            if (gtime() - t0 > (unsigned long long)limit_ns) {
                atomicCAS(err, 0, code);
                return false;
            }
        }
    }
}
// One box of a [slice][row][k] slice array: all S slices of a tile, planes
// of `rows` rows one after the other in shared memory.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void umma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, uint32_t (&r)[4]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// a * b + c with a 32 x 32 -> 64-bit signed product
__device__ __forceinline__ long long mad_wide_s32(int a, int b, long long c) {
    long long r;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(r) : "r"(a), "r"(b), "l"(c));
    return r;
}

// K-major operand tile, SWIZZLE_32B: rows of 32 bytes, 8-row groups 256 bytes apart.
__device__ __forceinline__ uint64_t desc_sw32(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
    d |= (uint64_t)(16u >> 4) << 16;           // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(256u >> 4) << 32;          // stride byte offset: 8 rows x 32 B
    d |= (uint64_t)1 << 46;                    // descriptor version for tcgen05
    d |= (uint64_t)6 << 61;                    // SWIZZLE_32B
    return d;
}
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4)                       // D format F32
           | (1u << 7)                     // A format BF16
           | (1u << 10)                    // B format BF16
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

// (-1)^neg 2^E a for a 64-bit magnitude a, assembled with integer operations
// (round to nearest even to 53 bits; results below the normal range flush to 0).
__device__ __forceinline__ double u64_ldexp(unsigned long long a, bool neg, int E) {
    if (a == 0) return 0.0;
    const unsigned long long sgn = neg ? (1ull << 63) : 0ull;
    int lz = __clzll((long long)a);
    unsigned long long n = a << lz;
    unsigned long long mant = n >> 11;
    const unsigned long long rest = n & 0x7FFull;
    if (rest > 0x400ull || (rest == 0x400ull && (mant & 1ull))) {
        ++mant;
        if (mant >> 53) {
            mant >>= 1;
            --lz;
        }
    }
    const int biased = (63 - lz) + E + 1023;
    if (biased <= 0) return 0.0;
    if (biased >= 2047) return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ull));
    return __longlong_as_double((long long)(sgn | ((unsigned long long)biased << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}


// The same for a signed 64-bit T, without branches (so that the epilogue's
// independent elements interleave), in 32-bit halves: |T| below 2^32 is moved
// up by 32 bits first, so that one 32-bit leading-zero count and two funnel
// shifts normalise it; the rounding carry runs into the exponent field through
// the bit pattern; zero, results below the normal range and overflow are
// selected at the end.  Bit-identical to u64_ldexp.
__device__ __forceinline__ double i64_ldexp(long long T, int E) {
    const unsigned long long sm = (unsigned long long)(T >> 63);  // all ones for T < 0
    const unsigned long long a = ((unsigned long long)T ^ sm) - sm;
    const bool small = (a >> 32) == 0;
    const unsigned ah = small ? (unsigned)a : (unsigned)(a >> 32);
    const unsigned al = small ? 0u : (unsigned)a;
    const int lz = __clz(ah);                           // 32 only for T = 0
    const unsigned nh = __funnelshift_l(al, ah, lz);    // leading one at bit 31
    const unsigned nl = al << (lz & 31);
    const unsigned mh = nh >> 11;                       // mantissa bits 52..32 (the leading one at bit 20)
    const unsigned ml = __funnelshift_r(nl, nh, 11);    // mantissa bits 31..0
    const unsigned inc = ((nl & 0x7FFu) + (ml & 1u) + 0x3FFu) >> 11;  // round half to even
    const int e = E + 1023 + 63 - (small ? 32 : 0) - lz;  // exponent field of the leading one
    const unsigned lo = ml + inc;
    const unsigned mc = mh + (lo < ml ? 1u : 0u);
    const int eff = e + int(mc >> 21);                  // after a rounding carry
    const unsigned hi = (eff >= 2047 ? 0x7FF00000u : ((unsigned)(e - 1) << 20) + mc) |
                        ((unsigned)(sm >> 32) & 0x80000000u);
    const double v = __hiloint2double((int)hi, eff >= 2047 ? 0 : (int)lo);
    return (a == 0 || eff <= 0) ? 0.0 : v;
}

}  // namespace

// ===========================================================================
// Slicing kernel: FP64 operand rows -> S BF16 digit slices + row exponents
// ===========================================================================
namespace {

constexpr int SL_KMAX = 2048;  // longest operand row the slicing stages (and longest sum)
constexpr int SL_K8MAX = 256;  // K bound of exact level sums with balanced 8-bit digits
constexpr int SL_UNROLL = 8;   // independent loads per thread in the staging loops (halved for 4 inputs)

// Digits are 8 bits wide at any length: sums longer than SL_K8MAX terms run
// as K-chunks of at most SL_K8MAX whose FP64 results are added.
inline int digit_bits(int) { return 8; }
constexpr int KCHUNK = SL_K8MAX;
inline int nchunks(int K) { return (K + KCHUNK - 1) / KCHUNK; }

// Sets a kernel's launch attributes once per (kernel, device), not at every
// launch (setting them is a CUDA runtime call).
template <class Kern, class Set>
int set_attributes_once(Kern kern, Set&& set) {
    static std::mutex mu;
    static std::set<std::pair<const void*, int>> done;
    int dev = 0;
    ZG_CUDA_TRY(cudaGetDevice(&dev));
    const auto key = std::make_pair(reinterpret_cast<const void*>(kern), dev);
    std::lock_guard<std::mutex> lock(mu);
    if (done.count(key)) return ZEST_GPU_OK;
    ZG_TRY(set(kern));
    done.insert(key);
    return ZEST_GPU_OK;
}

// Rows per slicing block: a power of two (so that in row-fast loops every
// thread stays on one row), up to 32 rows (longer contiguous runs in the
// row-fast loads), with the staged FP64 rows (row_bytes each) within 96 KB.
inline int slice_rows_per_block(int row_bytes) {
    // ZEST_GPU_SLICE_ROWS (a power of two up to 32) caps the rows per block,
    // to measure the trade between longer row-fast reads and blocks per SM
    static const int cap = [] {
        const char* e = std::getenv("ZEST_GPU_SLICE_ROWS");
        const int v = e ? std::atoi(e) : 32;
        return (v >= 1 && v <= 32 && (v & (v - 1)) == 0) ? v : 32;
    }();
    int r = cap;
    while (r > 1 && r * row_bytes > 96 * 1024) r >>= 1;
    return r;
}

enum { SL_ONE = 0, SL_FOLD = 1, SL_PAIR = 2, SL_PFOLD = 3 };

// Loaders give the pair (up, dn) of operand element (row, k) through a per-row
// handle computed once per block row.  ROW_FAST loaders read consecutive rows
// at one k contiguously; the others read consecutive k of one row.  TWO
// loaders produce both members of the pair (a fold or two interleaved
// operands), the others only `up`.
struct RowMajorLoader {  // tables and dense operands: p[r*ld + k]
    static constexpr bool ROW_FAST = false, TWO = false;
    static constexpr int MODE = SL_ONE, SHIFT = 0;
    const double* p;
    long long ld;
    struct Row { const double* p; };
    __device__ Row row(long long r) const { return Row{p + r * ld}; }
    __device__ void get(const Row& R, int k, double& up, double&) const { up = R.p[k]; }
};

// row i of two row-major tables of one shape: (P[i][k], Q[i][k])
struct TablePairLoader {
    static constexpr bool ROW_FAST = false, TWO = true;
    static constexpr int MODE = SL_PAIR, SHIFT = 1;
    const double* P;
    const double* Q;
    long long ld;
    struct Row { const double* p; const double* q; };
    __device__ Row row(long long r) const { return Row{P + r * ld, Q + r * ld}; }
    __device__ void get(const Row& R, int k, double& up, double& dn) const {
        up = R.p[k];
        dn = R.q[k];
    }
};

// rows (b, col) of the ball grids; k = longitude: (x_k, x_{N-k}), x_0 alone.
// Folded: cos operand x_k + x_{N-k} (k < L), sin operand x_k - x_{N-k} at k - 1.
struct DftFwdLoader {
    static constexpr bool ROW_FAST = true, TWO = true;
    static constexpr int MODE = SL_FOLD, SHIFT = 1;
    const double* grid;
    long long gsz;
    int C, N;
    struct Row { const double* x; };
    __device__ Row row(long long r) const {
        const long long b = r / C;
        return Row{grid + b * gsz + (r - b * C)};
    }
    __device__ void get(const Row& R, int k, double& up, double& dn) const {
        up = R.x[(long long)k * C];
        dn = k ? R.x[(long long)(N - k) * C] : 0.0;
    }
};

// rows (m, b, kc) of the spectra; k = folded latitude node (north, south).
struct LegFwdLoader {
    static constexpr bool ROW_FAST = true, TWO = true;
    static constexpr int MODE = SL_FOLD, SHIFT = 0;
    const double* G;
    int B, L, Nt, nr2, j0u, j0d;
    struct Row { const double* base; };
    __device__ Row row(long long r) const {
        const long long mb = r / nr2;
        const int kc = int(r - mb * nr2);
        const int m = int(mb / B), b = int(mb - (long long)m * B);
        return Row{G + ((long long)b * L + m) * Nt * nr2 + kc};
    }
    __device__ void get(const Row& R, int k, double& up, double& dn) const {
        up = R.base[(long long)(j0u + k) * nr2];
        dn = R.base[(long long)(j0d - k) * nr2];
    }
};

// Rows of the radial sums, grouped by degree l: row 2 (tri(l,0) B + b (l+1) + m) + c
// is (l, b, m, c), so that neighbouring rows are neighbouring (m, c) of one
// (l, b), whose Zernike coefficients zidx(n, l, m) + c are contiguous.
struct RadRow {
    int l, b, m, c;
};
__device__ __forceinline__ RadRow rad_row(long long r, int B) {
    const long long q = (r >> 1) / B;  // in [tri(l,0), tri(l+1,0))
    int l = int((sqrtf(8.0f * float(q) + 1.0f) - 1.0f) * 0.5f);
    while ((long long)(l + 1) * (l + 2) / 2 <= q) ++l;
    while ((long long)l * (l + 1) / 2 > q) --l;
    const long long local = (r >> 1) - (long long)l * (l + 1) / 2 * B;  // b (l + 1) + m
    const int b = int(local / (l + 1));
    return RadRow{l, b, int(local - (long long)b * (l + 1)), int(r & 1)};
}
// the same decoding for a row of the known group l
__device__ __forceinline__ RadRow rad_row_of(long long r, int l, int B) {
    const long long local = (r >> 1) - (long long)l * (l + 1) / 2 * B;
    const int b = int(local / (l + 1));
    return RadRow{l, b, int(local - (long long)b * (l + 1)), int(r & 1)};
}

struct RadFwdLoader {  // rows (l, b, m, c) as rad_row; k = radial node: flm[(tri(l,m) B + b)][k][c]
    static constexpr bool ROW_FAST = false, TWO = false;
    static constexpr int MODE = SL_ONE, SHIFT = 0;
    const double* flm;
    int nr, B;
    struct Row { const double* p; };
    __device__ Row row(long long r) const {
        const RadRow w = rad_row(r, B);
        return Row{flm + ((long long)tri_idx(w.l, w.m) * B + w.b) * nr * 2 + w.c};
    }
    __device__ void get(const Row& R, int k, double& up, double&) const { up = R.p[(long long)k * 2]; }
};

struct RadBwdLoader {  // rows (l, b, m, c) as rad_row; k = i, n = l + 2i
    // row-fast: neighbouring rows read neighbouring coefficients
    static constexpr bool ROW_FAST = true, TWO = false;
    static constexpr int MODE = SL_ONE, SHIFT = 0;
    const double* coeffs;
    long long cs;
    int B, Lm;
    struct Row { const double* base; int l, m; };
    __device__ Row row(long long r) const {
        const RadRow w = rad_row(r, B);
        return Row{coeffs + w.b * cs + w.c, w.l, w.m};
    }
    __device__ void get(const Row& R, int k, double& up, double&) const {
        const int n = R.l + 2 * k;
        up = (n < Lm) ? R.base[zidx(n, R.l, R.m) * 2] : 0.0;
    }
    __device__ int kvalid(const Row& R) const { return (Lm - R.l + 1) / 2; }  // n = l + 2k < Lm
};

// rows (m, b, kc) of flm; k = i: up = flm(l = m + 2i), dn = flm(l = m + 1 + 2i)
struct LegBwdLoader {
    static constexpr bool ROW_FAST = true, TWO = true;
    static constexpr int MODE = SL_PAIR, SHIFT = 0;
    const double* flm;
    int B, nr2, Lm;
    struct Row { const double* base; int m; };
    __device__ Row row(long long r) const {
        const long long mb = r / nr2;
        const int kc = int(r - mb * nr2);
        const int m = int(mb / B), b = int(mb - (long long)m * B);
        return Row{flm + (long long)b * nr2 + kc, m};
    }
    __device__ void get(const Row& R, int k, double& up, double& dn) const {
        const int l = R.m + 2 * k;
        const long long st = (long long)B * nr2;
        up = (l < Lm) ? R.base[tri_idx(l, R.m) * st] : 0.0;
        dn = (l + 1 < Lm) ? R.base[tri_idx(l + 1, R.m) * st] : 0.0;
    }
    __device__ int kvalid(const Row& R) const { return (Lm - R.m + 1) / 2; }  // l = m + 2k < Lm
};

// SH coefficients [b][tri(l,m)][c], rows (m, b, c); k = i: the pair
// (l = m + 2i, l + 1), zero from Lm on (the two parity operands).
// rows (m, b, kc) of flm; k = q: flm(l = m + q), zero from Lm on (the data of
// the unfolded backward Legendre sums, all l of one m in one operand)
struct LegBwdULoader {
    static constexpr bool ROW_FAST = true, TWO = false;
    static constexpr int MODE = SL_ONE, SHIFT = 0;
    const double* flm;
    int B, nr2, Lm;
    struct Row { const double* base; int m; };
    __device__ Row row(long long r) const {
        const long long mb = r / nr2;
        const int kc = int(r - mb * nr2);
        const int m = int(mb / B), b = int(mb - (long long)m * B);
        return Row{flm + (long long)b * nr2 + kc, m};
    }
    __device__ void get(const Row& R, int k, double& up, double&) const {
        const int l = R.m + k;
        up = (l < Lm) ? R.base[tri_idx(l, R.m) * ((long long)B * nr2)] : 0.0;
    }
    __device__ int kvalid(const Row& R) const { return Lm - R.m; }  // l = m + k < Lm
};

struct StLegBwdLoader {
    static constexpr bool ROW_FAST = true, TWO = true;
    static constexpr int MODE = SL_PAIR, SHIFT = 0;
    const double* c;
    long long cs;
    int B, Lm;
    struct Row { const double* base; int m; };
    __device__ Row row(long long r) const {
        const long long mb = r >> 1;
        const int m = int(mb / B), b = int(mb - (long long)m * B);
        return Row{c + b * cs + (r & 1), m};
    }
    __device__ void get(const Row& R, int k, double& up, double& dn) const {
        const int l = R.m + 2 * k;
        up = (l < Lm) ? R.base[2 * tri_idx(l, R.m)] : 0.0;
        dn = (l + 1 < Lm) ? R.base[2 * tri_idx(l + 1, R.m)] : 0.0;
    }
    __device__ int kvalid(const Row& R) const { return (Lm - R.m + 1) / 2; }  // l = m + 2k < Lm
};

// rows (b, col = (lat, rad)); k = m: the spectrum (Re F_m, Im F_m) at
// latitude lat (the sin operand takes Im F_k at k - 1), formed from the two
// parity sums E_p[b][m][j'][2 rad + {re, im}] of the Legendre stage: E_0 + E_1
// at the north node lat = j0u + j', E_0 - E_1 at the south node lat = j0d - j'
// (the equator, j0u = j0d, is north).  The sums are formed exactly in
// integers by the slicing (SL_PFOLD): the loader gives (Re E_0, Im E_0,
// Re E_1, Im E_1), E_1 negated for a south row by a sign-bit flip.
struct DftBwdLoader {
    static constexpr bool ROW_FAST = true, TWO = true;
    static constexpr int MODE = SL_PFOLD, SHIFT = 1;
    const double* E;
    int L, C, nrad, kh, j0u, j0d, B;
    struct Row { const double* e0; int neg; };  // neg: the sign bit of E_1's high word
    __device__ Row row(long long r) const {
        const long long b = r / C;
        const int col = int(r - b * C);
        const int lat = col / nrad, rad = col - lat * nrad;
        const bool north = lat >= j0u;
        const int jf = north ? lat - j0u : j0d - lat;
        return Row{E + ((b * L) * kh + jf) * (2LL * nrad) + 2 * rad, north ? 0 : int(0x80000000u)};
    }
    __device__ void get4(const Row& R, int k, double* v) const {
        const long long mo = (long long)k * kh * 2 * nrad;
        const double2 a = *reinterpret_cast<const double2*>(R.e0 + mo);
        const double2 c = *reinterpret_cast<const double2*>(R.e0 + mo + (long long)B * L * kh * 2 * nrad);
        v[0] = a.x;
        v[1] = a.y;
        v[2] = __hiloint2double(__double2hiint(c.x) ^ R.neg, __double2loint(c.x));
        v[3] = __hiloint2double(__double2hiint(c.y) ^ R.neg, __double2loint(c.y));
    }
};

// rows (b, col = (lat, rad)); k = m: the spectrum (Re F_m, Im F_m) at
// latitude lat, E[b][m][lat][2 rad + {re, im}] of the unfolded backward
// Legendre sums (the sin operand takes Im F_k at k - 1)
struct DftBwdGridLoader {
    static constexpr bool ROW_FAST = true, TWO = true;
    static constexpr int MODE = SL_PAIR, SHIFT = 1;
    const double* E;
    int L, C, nrad, nlat;
    struct Row { const double* e; };
    __device__ Row row(long long r) const {
        const long long b = r / C;
        const int col = int(r - b * C);
        const int lat = col / nrad, rad = col - lat * nrad;
        return Row{E + ((b * L) * nlat + lat) * (2LL * nrad) + 2 * rad};
    }
    __device__ void get(const Row& R, int k, double& up, double& dn) const {
        const double2 a = *reinterpret_cast<const double2*>(R.e + (long long)k * nlat * 2 * nrad);
        up = a.x;
        dn = a.y;
    }
};

// One slicing job: one operand array (SL_ONE) or two from one read of the
// input (SL_FOLD: up + dn and up - dn; SL_PAIR: up and dn; SL_PFOLD: the
// sums of two pairs), the second at index k - shift.  Both share the row
// exponents.  Each loader fixes its mode and shift (Loader::MODE,
// Loader::SHIFT), so the kernel is specialised.
struct SliceJob {
    long long rows;
    int K;            // longest valid k of any staged input (loads stop there)
    int Ku, Kd;       // inputs of the first array are zero from Ku on, of the second from Kd on
    int KS;           // staged k range: max(Kp0, Kp1) + shift, the rest zero
    int Ks;           // shared-memory row stride in doubles (padded layout, below)
    int S, bits, R, lr;  // lr = log2(R)
    int K0, Kp0, K1, Kp1;
    __nv_bfloat16* out0;
    __nv_bfloat16* out1;
    long long stride0, stride1;  // elements between slices
    int* ex0;
    int* ex1;
};

// Staged inputs per operand row: 1 (SL_ONE), 2 (SL_FOLD, SL_PAIR) or 4 (SL_PFOLD).
template <class Loader>
__host__ __device__ constexpr int staged_arrays() {
    return Loader::MODE == SL_ONE ? 1 : (Loader::MODE == SL_PFOLD ? 4 : 2);
}

// Ragged loaders (a member kvalid(row): the row's inputs are zero from that k
// on) feed triangular sums whose GEMM work lists read, for the rows of one
// group, only the K blocks up to their valid length rounded up to 16.  A
// slicing block then stages and writes only up to the largest such length of
// its rows (rounded up to 16; the zeros in between are written), not the whole
// row: the slices beyond are never read.
template <class L, class = void>
struct ragged_loader : std::false_type {};
template <class L>
struct ragged_loader<L, std::void_t<decltype(std::declval<const L&>().kvalid(std::declval<const typename L::Row&>()))>>
    : std::true_type {};

// Shared-memory position of element k of a staged row: one double of padding
// after every 8, so that the lanes of a warp reading 8 consecutive elements
// each at neighbouring chunks (stride 9 doubles) hit distinct banks.
__device__ __forceinline__ int sl_pos(int k) { return k + (k >> 3); }

// Row stride of the staged rows: room for KS padded elements, and 2 mod 4
// doubles, so that the row-fast staging (16 rows x 2 k per warp) stores
// conflict-free.
inline int sl_row_stride(int KS) {
    const int p = KS + (KS >> 3) + 1;
    return p + ((6 - p % 4) % 4);
}

// fixed point: round(x 2^{nbits-e}) as int64 (|x| < 2^(e-1)), ties away from
// zero, with Cr = 1074 + e - nbits.  q = |x| 2^{nbits-e+1} truncated (one bit
// more than kept), then ((q ^ s) + 1) >> 1 with s the sign mask is
// floor(q/2 + 1/2) for x >= 0 and its negative for x < 0.  The shift
// Cr - E(x) is at least 5 for every element of a row (the row exponent keeps
// a bit of headroom); PTX shifts of 64 or more give 0, so a zero or an element
// far below the row's largest rounds to 0 without a branch.
__device__ __forceinline__ long long to_fixed_c(double x, int Cr) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const unsigned E = unsigned(bits >> 52) & 0x7FFu;
    const unsigned long long M = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    unsigned long long q;
    asm("shr.b64 %0, %1, %2;" : "=l"(q) : "l"(M), "r"(unsigned(Cr) - E));
    const long long sg = (long long)bits >> 63;  // 0 or -1
    return (((long long)q ^ sg) + 1) >> 1;
}

// Balanced 8-bit digits of 8 neighbouring elements (slice 0 most
// significant), written as 8 BF16 per slice with one 16-byte store.  Adding
// 128 sum_{i<S-1} 256^i turns the lower balanced digits into the plain bytes
// of the sum (digit = byte - 128) and leaves the leading digit as the sum
// shifted down.  A lower digit's float is built by one byte permute,
// 0x4B4000bb = 2^23 + 2^22 + byte, and one subtraction of 2^23 + 2^22 + 128;
// the float is exact with at most 8 significant bits, so its upper half is the
// BF16.
template <int S>
__device__ __forceinline__ void store_digits8(const long long (&w)[8], __nv_bfloat16* out, long long stride) {
    constexpr long long OFF = (long long)((0x8080808080808080ull) >> (8 * (9 - S)));  // 128 per lower byte
    uint32_t lo[8], hi[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const unsigned long long u = (unsigned long long)(w[q] + OFF);
        lo[q] = uint32_t(u);
        hi[q] = uint32_t(u >> 32);
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
        uint32_t o[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            float f[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int q = 2 * p + h;
                if (s == 0) {
                    const long long u = (long long)(((unsigned long long)hi[q] << 32) | lo[q]);
                    f[h] = __int_as_float(0x4B400000 + int(u >> (8 * (S - 1)))) - 12582912.0f;
                } else {
                    const int b = S - 1 - s;  // byte of the sum holding digit s
                    f[h] = __int_as_float(int(__byte_perm(b < 4 ? lo[q] : hi[q], 0x4B400000u, 0x7650u | (b & 3)))) -
                           12583040.0f;
                }
            }
            o[p] = __byte_perm(__float_as_uint(f[0]), __float_as_uint(f[1]), 0x7632);
        }
        *reinterpret_cast<uint4*>(out + s * stride) = make_uint4(o[0], o[1], o[2], o[3]);
    }
}

template <class Loader>
__device__ __forceinline__ void load_staged(const Loader& ld, const typename Loader::Row& R, int k, double* v) {
    if constexpr (Loader::MODE == SL_PFOLD) {
        ld.get4(R, k, v);
    } else {
        double dn = 0.0;
        ld.get(R, k, v[0], dn);
        if constexpr (Loader::TWO) v[1] = dn;
    }
}

// One CTA converts R rows (R a power of two, <= 32) of staged values.
// Phase 1 stages the FP64 inputs in shared memory (zero beyond each input's
// valid range, up to KS) and finds each row's largest exponent: for row-fast
// operands lane l of a warp reads row l mod R (so a warp reads R consecutive
// rows at 32/R neighbouring k), otherwise one warp walks one row along k.
// Phase 2 cuts the rows into chunks of 8 neighbouring k and gives each thread
// one chunk of one row at a time: the chunk's values (and, for a shifted
// second array, the next one) are rounded to the row's fixed-point grid once,
// folded exactly in integers where requested, split into balanced 8-bit
// digits and written as S BF16 slices, 16 bytes per slice and array.
template <class Loader, int S>
__global__ void __launch_bounds__(256) slice_kernel(Loader ld, SliceJob J) {
    constexpr int MODE = Loader::MODE, SHIFT = Loader::SHIFT, NA = staged_arrays<Loader>();
    constexpr int fold_bit = (MODE == SL_FOLD || MODE == SL_PFOLD) ? 1 : 0;
    constexpr int UNR = NA == 4 ? SL_UNROLL / 2 : SL_UNROLL;  // loads in flight per thread and input
    static_assert((NA > 1) == Loader::TWO && (SHIFT == 0 || (NA > 1 && SHIFT == 1)), "loader mode");
    extern __shared__ double sl_smem[];
    constexpr bool RAGGED = ragged_loader<Loader>::value;
    static_assert(!RAGGED || SHIFT == 0, "ragged loaders stage unshifted arrays");
    const int R = J.R, lr = J.lr, Ks = J.Ks;
    const int astride = R * Ks;  // between the staged arrays
    __shared__ unsigned emax[32];  // largest |x| high word per row (sign cleared)
    __shared__ typename Loader::Row rowh[32];
    __shared__ int kv_s;           // ragged loaders: the largest valid length of the block's rows
    const long long row0 = (long long)blockIdx.x * R;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if constexpr (RAGGED) {
        if (threadIdx.x == 0) kv_s = 0;
        __syncthreads();
    }
    if (threadIdx.x < 32) emax[threadIdx.x] = 0;
    if (threadIdx.x < R && row0 + threadIdx.x < J.rows) {
        rowh[threadIdx.x] = ld.row(row0 + threadIdx.x);
        if constexpr (RAGGED) atomicMax(&kv_s, ld.kvalid(rowh[threadIdx.x]));
    }
    __syncthreads();
    // staged (and written) k range of this block
    int KS = J.KS;
    if constexpr (RAGGED) KS = min(KS, (max(kv_s, 0) + 15) & ~15);
    // input a feeds the first array (a even) or the second (a odd): zero from Ku / Kd
    auto lim = [&](int a) { return (NA == 1 || (a & 1) == 0 || MODE == SL_FOLD) ? J.Ku : J.Kd; };
    if (Loader::ROW_FAST) {
        const int r = lane & (R - 1), kl = lane >> lr, kstep = 32 >> lr;
        const bool rv = row0 + r < J.rows;
        unsigned tmax = 0;
        const int kst = nw * kstep;
        double* srow = sl_smem + r * Ks;
        for (int k0 = warp * kstep + kl; k0 < KS; k0 += UNR * kst) {
            double v[UNR][NA];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
#pragma unroll
                for (int a = 0; a < NA; ++a) v[u][a] = 0.0;
                const int k = k0 + u * kst;
                if (rv && k < J.K) load_staged(ld, rowh[r], k, v[u]);
            }
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int k = k0 + u * kst;
                if (k < KS) {
#pragma unroll
                    for (int a = 0; a < NA; ++a) {
                        const double x = k < lim(a) ? v[u][a] : 0.0;
                        srow[a * astride + sl_pos(k)] = x;
                        tmax = max(tmax, unsigned(__double2hiint(x)) & 0x7FFFFFFFu);
                    }
                }
            }
        }
        for (int o = R; o < 32; o <<= 1) tmax = max(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
        if (lane < R && tmax) atomicMax(&emax[lane], tmax);
    } else {
        for (int r = warp; r < R; r += nw) {
            unsigned tmax = 0;
            const bool rv = row0 + r < J.rows;
            double* srow = sl_smem + r * Ks;
            for (int k0 = lane; k0 < KS; k0 += 32 * UNR) {
                double v[UNR][NA];
#pragma unroll
                for (int u = 0; u < UNR; ++u) {
#pragma unroll
                    for (int a = 0; a < NA; ++a) v[u][a] = 0.0;
                    const int k = k0 + 32 * u;
                    if (rv && k < J.K) load_staged(ld, rowh[r], k, v[u]);
                }
#pragma unroll
                for (int u = 0; u < UNR; ++u) {
                    const int k = k0 + 32 * u;
                    if (k < KS) {
#pragma unroll
                        for (int a = 0; a < NA; ++a) {
                            const double x = k < lim(a) ? v[u][a] : 0.0;
                            srow[a * astride + sl_pos(k)] = x;
                            tmax = max(tmax, unsigned(__double2hiint(x)) & 0x7FFFFFFFu);
                        }
                    }
                }
            }
            for (int o = 16; o > 0; o >>= 1) tmax = max(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
            if (lane == 0) emax[r] = tmax;
        }
    }
    __syncthreads();
    const int nbits = 8 * S;
    // row exponents: |x| < 2^(E_max - 1022), at least 64 - 1022 (below that
    // every value rounds to 0); one more bit of headroom for the balanced
    // leading digit, and one for a folded sum
    if (threadIdx.x < R && row0 + threadIdx.x < J.rows) {
        const int er = max(int(emax[threadIdx.x] >> 20), 64) - 1022 + 1 + fold_bit;
        J.ex0[row0 + threadIdx.x] = er;
        if (NA > 1) J.ex1[row0 + threadIdx.x] = er;
    }
    const int nch0 = min(J.Kp0, KS) >> 3, nch1 = NA > 1 ? min(J.Kp1, KS) >> 3 : 0;
    const int nch = max(nch0, nch1);
    if (nch == 0) return;  // a ragged block of rows with no valid k: exponents only
    const int items = R * nch;
    int r = threadIdx.x / nch, c = threadIdx.x - r * nch;
    const int dr = blockDim.x / nch, dc = blockDim.x - dr * nch;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const long long row = row0 + r;
        if (row < J.rows) {
            const int Cr = 1074 + (max(int(emax[r] >> 20), 64) - 1022 + 1 + fold_bit) - nbits;
            const double* base = sl_smem + r * Ks + 9 * c;  // element 8c
            constexpr int NJ = 8 + SHIFT;
            auto at = [&](int a, int j) { return base[a * astride + j + (j >> 3)]; };
            if constexpr (MODE == SL_ONE) {
                long long w[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) w[q] = to_fixed_c(at(0, q), Cr);
                store_digits8<S>(w, J.out0 + row * J.Kp0 + 8 * c, J.stride0);
            } else if constexpr (MODE == SL_FOLD) {
                long long fu[NJ], fd[NJ];
#pragma unroll
                for (int j = 0; j < NJ; ++j) {
                    fu[j] = to_fixed_c(at(0, j), Cr);
                    fd[j] = to_fixed_c(at(1, j), Cr);
                }
                long long w[8];
                if (c < nch0) {
#pragma unroll
                    for (int q = 0; q < 8; ++q) w[q] = fu[q] + fd[q];
                    store_digits8<S>(w, J.out0 + row * J.Kp0 + 8 * c, J.stride0);
                }
                if (c < nch1) {
#pragma unroll
                    for (int q = 0; q < 8; ++q) w[q] = fu[q + SHIFT] - fd[q + SHIFT];
                    store_digits8<S>(w, J.out1 + row * J.Kp1 + 8 * c, J.stride1);
                }
            } else {
                // SL_PAIR: up | dn; SL_PFOLD: up + up2 | dn + dn2 (inputs 0, 2 | 1, 3)
                long long w[8];
                if (c < nch0) {
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        w[q] = to_fixed_c(at(0, q), Cr);
                        if constexpr (MODE == SL_PFOLD) w[q] += to_fixed_c(at(2, q), Cr);
                    }
                    store_digits8<S>(w, J.out0 + row * J.Kp0 + 8 * c, J.stride0);
                }
                if (c < nch1) {
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        w[q] = to_fixed_c(at(1, q + SHIFT), Cr);
                        if constexpr (MODE == SL_PFOLD) w[q] += to_fixed_c(at(3, q + SHIFT), Cr);
                    }
                    store_digits8<S>(w, J.out1 + row * J.Kp1 + 8 * c, J.stride1);
                }
            }
        }
        c += dc;
        r += dr;
        if (c >= nch) {
            c -= nch;
            ++r;
        }
    }
}

}  // namespace

// ===========================================================================
// GEMM kernel
// ===========================================================================
struct SplitUnit {
    int a_row0;   // first operand row of the tile (row index inside the slice array)
    int a_rows;   // valid rows (<= 128)
    int b_row0;   // first table row
    int n;        // valid table rows (<= NT)
    int ksteps;   // 16-wide K blocks
    int flags;    // bit 0: A map, bit 1: B map, bit 2: parity / RMW
    int g;        // group (m or l)
    int aux;      // group-relative index of the first table row
    int k0;       // first 16-wide K block (sums split into chunks of at most 256)
};

namespace {

// Epilogues map (operand row, table row) of a tile to an output location.
// row(u, r) is evaluated once per row and tile; store() once per element.
// ACC = true: a later K-chunk of the sum, whose value is added to what the
// earlier chunks stored (load() reads it back; every epilogue is linear in v).
// RMW epilogues expose load() so that the old values are fetched before the
// accumulators are read (hiding the memory latency).
template <bool ACC = false>
struct EpiDense {  // C[row][b_row0 + n] (utility GEMM)
    static constexpr bool RMW = ACC;
    static constexpr bool CHUNK = ACC;
    double* C;
    long long ldc;
    struct Row { double* p; };
    __device__ Row row(const SplitUnit& u, int r) const { return Row{C + (long long)r * ldc + u.b_row0}; }
    __device__ void load(const Row& R, int n, double* old) const { old[0] = R.p[n]; }
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double* old) const {
        R.p[n] = ACC ? old[0] + v : v;
    }
};
template <bool ACC = false>
struct EpiDftFwd {  // rows (b, col): conj X_m -> G[b][m][col][re, im]
    static constexpr bool RMW = ACC;
    static constexpr bool CHUNK = ACC;
    double* G;
    int C, L;
    struct Row { double* p; };  // &G[b][m0][col][re or im]
    __device__ Row row(const SplitUnit& u, int r) const {
        const int b = r / C, col = r - b * C;
        const int sin = (u.flags >> 1) & 1;
        const int m0 = u.aux + sin;
        return Row{G + (((long long)b * L + m0) * C + col) * 2 + sin};
    }
    __device__ void load(const Row& R, int n, double* old) const { old[0] = R.p[(long long)n * C * 2]; }
    __device__ void store(const Row& R, const SplitUnit& u, int n, double v, const double* old) const {
        double* g = R.p + (long long)n * C * 2;
        g[0] = ACC ? old[0] + v : v;
        if (!ACC && ((u.flags >> 1) & 1) == 0 && u.aux + n == 0) g[1] = 0.0;  // Im X_0 = 0
    }
};
template <bool ACC = false>
struct EpiLegFwd {  // rows (m, b, kc) -> flm[tri(l,m)][b][kc], l = m + p + 2 (aux + n)
    static constexpr bool RMW = ACC;
    static constexpr bool CHUNK = ACC;
    double* flm;
    int B, nr2;
    struct Row { double* p; int l0; };
    __device__ Row row(const SplitUnit& u, int r) const {
        const int m = u.g, p = (u.flags >> 2) & 1;
        const long long local = r - (long long)m * B * nr2;
        const int l0 = m + p + 2 * u.aux;
        return Row{flm + (tri_idx(l0, m) * B) * nr2 + local, l0};
    }
    // tri(l0 + 2n, m) - tri(l0, m) = n (2 l0 + 2 n + 1)
    __device__ double* at(const Row& R, int n) const {
        return R.p + (long long)n * (2LL * R.l0 + 2 * n + 1) * B * nr2;
    }
    __device__ void load(const Row& R, int n, double* old) const { old[0] = *at(R, n); }
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double* old) const {
        *at(R, n) = ACC ? old[0] + v : v;
    }
};
template <bool ACC = false>
struct EpiRadFwd {  // rows (l, b, m, c) as rad_row -> coeffs[b][zidx(n,l,m)][c]
    static constexpr bool RMW = ACC;
    static constexpr bool CHUNK = ACC;
    double* coeffs;
    int B;
    long long cs;
    struct Row { double* p; long long zl0; int l; };
    __device__ Row row(const SplitUnit& u, int r) const {
        const RadRow w = rad_row_of(r, u.g, B);
        const long long n0 = w.l + 2 * u.aux;
        return Row{coeffs + w.b * cs + 2 * w.m + w.c, n0, w.l};
    }
    __device__ double* at(const Row& R, int n) const {
        const long long nn = R.zl0 + 2 * n;
        return R.p + 2 * ((nn + 1) * (nn + 3) * (2 * nn + 1) / 24 + ((R.l * R.l) >> 2));
    }
    __device__ void load(const Row& R, int n, double* old) const { old[0] = *at(R, n); }
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double* old) const {
        *at(R, n) = ACC ? old[0] + v : v;
    }
};
template <bool ACC = false>
struct EpiRadBwd {  // rows (l, b, m, c) as rad_row -> flm[(tri(l,m) B + b)][k][c]
    static constexpr bool RMW = ACC;
    static constexpr bool CHUNK = ACC;
    static constexpr bool PAIR_ROWS = !ACC;  // rows c = 0, 1 of one (l, b, m): (re, im) at each k
    double* flm;
    int nr, B;
    struct Row { double* p; };
    __device__ Row row(const SplitUnit& u, int r) const {
        const RadRow w = rad_row_of(r, u.g, B);
        return Row{flm + ((tri_idx(w.l, w.m) * B + w.b) * nr + u.aux) * 2 + w.c};
    }
    __device__ void load(const Row& R, int n, double* old) const { old[0] = R.p[2 * n]; }
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double* old) const {
        R.p[2 * n] = ACC ? old[0] + v : v;
    }
    // (re, im) of column n, from the row of part c (the pair starts c doubles before R.p)
    __device__ void store_pair(const Row& R, int n, double2 v, int c) const {
        *reinterpret_cast<double2*>(R.p - c + 2 * n) = v;
    }
};
// rows (m, b, kc) -> E_p[b][m][j'][kc] (conjugated): the parity-p Legendre
// sum at folded node j'; the north node j0u + j' of the spectrum is E_0 + E_1
// and the south node j0d - j' is E_0 - E_1, formed by the DFT slicing that
// reads them (no read-modify-write here).
template <bool ACC = false>
struct EpiLegBwdE {
    static constexpr bool RMW = ACC;
    static constexpr bool CHUNK = ACC;
    double* E;
    int B, L, kh, nr2;
    struct Row { double* p; unsigned long long sgn; };  // sgn: the sign bit flipped for imaginary parts
    __device__ Row row(const SplitUnit& u, int r) const {
        const int m = u.g, par = (u.flags >> 2) & 1;
        const long long local = r - (long long)m * B * nr2;
        const int b = int(local / nr2), kc = int(local - (long long)b * nr2);
        return Row{E + ((((long long)par * B + b) * L + m) * kh + u.aux) * nr2 + kc,
                   (kc & 1) ? (1ull << 63) : 0ull};
    }
    __device__ void load(const Row& R, int n, double* old) const { old[0] = R.p[(long long)n * nr2]; }
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double* old) const {
        // the conjugate by a sign-bit flip (an integer operation, not an FP64 multiply)
        const double w = __longlong_as_double(__double_as_longlong(v) ^ (long long)R.sgn);
        R.p[(long long)n * nr2] = ACC ? old[0] + w : w;
    }
};

// Unfolded backward Legendre sums: rows (m, b, kc), table rows (m, lat) for
// every latitude node -> E[b][m][lat][kc], the imaginary parts conjugated.
template <bool ACC>
struct EpiLegBwdU {
    static constexpr bool RMW = ACC;
    static constexpr bool CHUNK = ACC;
    double* E;
    int B, L, nlat, nr2;
    struct Row { double* p; unsigned long long sgn; };
    __device__ Row row(const SplitUnit& u, int r) const {
        const int m = u.g;
        const long long local = r - (long long)m * B * nr2;
        const int b = int(local / nr2), kc = int(local - (long long)b * nr2);
        return Row{E + (((long long)b * L + m) * nlat + u.aux) * nr2 + kc, (kc & 1) ? (1ull << 63) : 0ull};
    }
    __device__ void load(const Row& R, int n, double* old) const { old[0] = R.p[(long long)n * nr2]; }
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double* old) const {
        const double w = __longlong_as_double(__double_as_longlong(v) ^ (long long)R.sgn);
        R.p[(long long)n * nr2] = ACC ? old[0] + w : w;
    }
};

// SH sums: the table is the 128-row operand (rows = table rows of a group), the
// 2 x batch data rows (b, c) are the columns.
// Forward: table row r of group (m, p) holds l = m + p + 2 (r - off(m, p)),
// off(m, 0) = m L - m (m - 1) / 2 and off(m, 1) = off(m, 0) + (L - m + 1) / 2
// (the group offsets of the Legendre tables of order L); column n -> (b, c).
// ACC: a later K-chunk of the sum, added to the earlier chunks' result.
template <bool ACC>
struct EpiStLegFwd {
    static constexpr bool RMW = ACC;
    static constexpr bool CHUNK = ACC;
    double* coeffs;
    long long cs;
    int L;
    struct Row { double* p; };
    __device__ Row row(const SplitUnit& u, int r) const {
        const int m = u.g, p = (u.flags >> 2) & 1;
        const long long off = (long long)m * L - (long long)m * (m - 1) / 2 + (p ? (L - m + 1) / 2 : 0);
        const long long l = m + p + 2 * (r - off);
        return Row{coeffs + 2 * tri_idx(l, m) + (u.aux >> 1) * cs};  // the unit's first column (b, c) = (aux/2, 0)
    }
    __device__ void load(const Row& R, int n, double* old) const { old[0] = R.p[(n >> 1) * cs + (n & 1)]; }
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double* old) const {
        R.p[(n >> 1) * cs + (n & 1)] = ACC ? old[0] + v : v;
    }
};
// Backward: table row r of group (m, p) is folded node j = r - (2m + p) kh;
// the parity sums go to E[p][b][m][j][c], the imaginary parts with the sign bit
// flipped (flip_im: conjugated, as the inverse longitude DFT reads them).
template <bool ACC>
struct EpiStLegBwdE {
    static constexpr bool RMW = ACC;
    static constexpr bool CHUNK = ACC;
    double* E;
    int B, L, kh;
    unsigned long long flip_im;  // 1 << 63: the imaginary parts conjugated (a sign-bit flip), else 0
    struct Row { double* p; };
    __device__ Row row(const SplitUnit& u, int r) const {
        const int m = u.g, par = (u.flags >> 2) & 1;
        const long long j = r - (long long)(2 * m + par) * kh;
        return Row{E + (((long long)par * B * L + m) * kh + j) * 2 + (long long)(u.aux >> 1) * L * kh * 2};
    }
    __device__ void load(const Row& R, int n, double* old) const {
        old[0] = R.p[(long long)(n >> 1) * L * kh * 2 + (n & 1)];
    }
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double* old) const {
        const double w = __longlong_as_double(__double_as_longlong(v) ^ (long long)((n & 1) ? flip_im : 0ull));
        R.p[(long long)(n >> 1) * L * kh * 2 + (n & 1)] = ACC ? old[0] + w : w;
    }
};

// Inverse DFT, rows (b, col).  The cos pass writes x_0 = C_0 to the grid and
// C_i (i >= 1) to the scratch Cs[b][i][col]; the sin pass reads C_i once and
// writes x_i = C_i + S_i and x_{N-i} = C_i - S_i.
template <bool ACC = false>
struct EpiDftBwdCos {
    static constexpr bool RMW = ACC;
    static constexpr bool CHUNK = ACC;
    double* grid;
    double* Cs;
    int C, N, L;
    long long gsz;
    struct Row { double* x; double* c; int aux; };
    __device__ Row row(const SplitUnit& u, int r) const {
        const long long b = r / C, col = r - b * C;
        return Row{grid + b * gsz + col, Cs + (b * L + u.aux) * C + col, u.aux};
    }
    __device__ double* at(const Row& R, int n) const { return R.aux + n == 0 ? R.x : R.c + (long long)n * C; }
    __device__ void load(const Row& R, int n, double* old) const { old[0] = *at(R, n); }
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double* old) const {
        *at(R, n) = ACC ? old[0] + v : v;
    }
};
// The first chunk reads the finished cos sums C_i and writes x_i = C_i + S_i,
// x_{N-i} = C_i - S_i; later chunks add their S_i to x_i and subtract it from x_{N-i}.
template <bool ACC = false>
struct EpiDftBwdSin {
    static constexpr bool RMW = true;
    static constexpr bool CHUNK = ACC;
    double* grid;
    const double* Cs;
    int C, N, L;
    long long gsz;
    struct Row { double* x; const double* c; int i0; };
    __device__ Row row(const SplitUnit& u, int r) const {
        const long long b = r / C, col = r - b * C;
        return Row{grid + b * gsz + col, Cs + (b * L + u.aux + 1) * C + col, u.aux + 1};
    }
    __device__ void load(const Row& R, int n, double* old) const {
        if (ACC) {
            const int i = R.i0 + n;
            old[0] = R.x[(long long)i * C];
            old[1] = R.x[(long long)(N - i) * C];
        } else {
            old[0] = old[1] = R.c[(long long)n * C];
        }
    }
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double* old) const {
        const int i = R.i0 + n;
        R.x[(long long)i * C] = old[0] + v;
        R.x[(long long)(N - i) * C] = old[1] - v;
    }
};

// The same inverse DFT for sums of at most 256 terms, combined in integers:
// the cos and sin tables are sliced together, so that row i of both shares
// one exponent, and the data operands share theirs (one slicing job), so
// C_i and S_i are exact integers T_c, T_s on the same scale 2^e.  The cos
// pass writes x_0 = C_0 and the raw T_c (int64) of i >= 1 to the scratch; the
// sin pass forms x_i = 2^e (T_c + T_s) and x_{N-i} = 2^e (T_c - T_s) exactly
// before one rounding each, with integer operations only (no FP64 adds).
// The table digits are at most 64 in magnitude (|2 cos|, |2 sin| <= 2), so
// |T| < 2^61 and the sums cannot overflow.
// Epilogues whose rows 2i and 2i + 1 are the two halves of one 16-byte pair
// at each column (PAIR_ROWS; store_pair writes both)
template <class E, class = void>
struct pair_rows_epi : std::false_type {};
template <class E>
struct pair_rows_epi<E, std::void_t<decltype(E::PAIR_ROWS)>> : std::integral_constant<bool, E::PAIR_ROWS> {};

template <class E, class = void>
struct raw_epi : std::false_type {};
template <class E>
struct raw_epi<E, std::void_t<decltype(E::RAW)>> : std::integral_constant<bool, E::RAW> {};

struct EpiDftBwdCosRaw {
    static constexpr bool RMW = false;
    static constexpr bool CHUNK = false;
    static constexpr bool RAW = true;
    double* grid;
    long long* Ts;
    int C, N, L;
    long long gsz;
    struct Row { double* x; long long* t; int aux; };
    __device__ Row row(const SplitUnit& u, int r) const {
        const long long b = r / C, col = r - b * C;
        return Row{grid + b * gsz + col, Ts + (b * L + u.aux) * C + col, u.aux};
    }
    __device__ void load_raw(const Row&, int, long long*) const {}
    __device__ void store_raw(const Row& R, const SplitUnit&, int n, long long T, int e, long long) const {
        if (R.aux + n == 0) *R.x = i64_ldexp(T, e);
        else R.t[(long long)n * C] = T;
    }
};
struct EpiDftBwdSinRaw {
    static constexpr bool RMW = true;
    static constexpr bool CHUNK = false;
    static constexpr bool RAW = true;
    double* grid;
    const long long* Ts;
    int C, N, L;
    long long gsz;
    struct Row { double* x; const long long* t; int i0; };
    __device__ Row row(const SplitUnit& u, int r) const {
        const long long b = r / C, col = r - b * C;
        return Row{grid + b * gsz + col, Ts + (b * L + u.aux + 1) * C + col, u.aux + 1};
    }
    __device__ void load_raw(const Row& R, int n, long long* old) const { *old = R.t[(long long)n * C]; }
    __device__ void store_raw(const Row& R, const SplitUnit&, int n, long long T, int e, long long old) const {
        const int i = R.i0 + n;
        R.x[(long long)i * C] = i64_ldexp(old + T, e);
        R.x[(long long)(N - i) * C] = i64_ldexp(old - T, e);
    }
};

struct SplitParams {
    const SplitUnit* units;
    int nunits;
    const int* ea[2];
    const int* eb[2];
    int narrow;               // units of at most this many valid table rows run one MMA per product
    int* err;
    int* host_err;            // mapped host word: each CTA copies a set flag there as it exits
    unsigned long long* dbg;  // optional cycle counters (null in normal use)
};

// Product schedule of S slices of 8-bit digits.  The products
// d_s(A) d_t(B) of level d = s + t <= S - 1 are kept (21 at S = 6) and each
// level has its own FP32 accumulator in TMEM, so every accumulator holds an
// integer: a product is at most 2^14, levels 0..3 stay exact (below 2^24)
// for sums of up to 256 terms, and levels 4 and 5, which may pass 2^24, are
// rounded to integers of their own weight (2^-32 and 2^-40 of level 0).  No
// operand needs pre-scaled copies of its slices.
//
// The products of one A slice s with the B slices t, t + 1, .. go to the
// accumulators s + t, s + t + 1, ..: with the B slices of a stage stored one
// after the other (NT rows each) and the accumulators NT columns apart, up to
// 256 / NT of them are one MMA of N = g NT (9 MMAs per K block at S = 6,
// NT = 80, instead of 21 of N = NT).  Each MMA reads its A tile once for g
// products, which is what keeps the shared-memory reads per MAC low enough
// for the tensor pipe.
template <int S>
struct Sched {
    static constexpr int NACC = S;                      // accumulators: levels 0..S-1
    static constexpr int NB = S;                        // B tiles per stage: the S slices
    static constexpr int PRODUCTS = S * (S + 1) / 2;    // slice products per K block
};
static_assert(Sched<6>::PRODUCTS == 21 && Sched<4>::PRODUCTS == 10, "schedules");

template <int S, int BITS, int NT>
__host__ __device__ constexpr int stage_count() {
    constexpr int st = S * 128 * 32 + Sched<S>::NB * NT * 32;
    constexpr int n = (220 * 1024) / st;
    return n > 6 ? 6 : n;
}

template <int S, int BITS, int NT, class Epi>  // S slices of BITS-bit digits, NT table rows per tile
__global__ void __launch_bounds__(SP_THREADS, 1)
    split_gemm_kernel(const __grid_constant__ CUtensorMap mapA0, const __grid_constant__ CUtensorMap mapA1,
                      const __grid_constant__ CUtensorMap mapB0, const __grid_constant__ CUtensorMap mapB1,
                      const SplitParams P, const Epi epi) {
    using SC = Sched<S>;
    static_assert(BITS == 8, "8-bit digits");
    constexpr int NST = stage_count<S, BITS, NT>();
    constexpr int A_TILE = SP_M * 32;  // one slice, 16 K elements
    constexpr int B_TILE = NT * 32;    // one slice of NT table rows: the B slices are contiguous
    constexpr int STAGE = S * A_TILE + SC::NB * B_TILE;
    constexpr uint32_t TX = S * (SP_M * 32) + SC::NB * (NT * 32);
    constexpr int GMAX = 256 / NT;     // products of one A slice per MMA (N = g NT <= 256)
    // every B tile is loaded whole; a unit of at most 32 valid table rows runs
    // its 21 products as MMAs of N = its rows rounded up to 16, the others as
    // grouped MMAs of full tiles
    static_assert(SC::NACC * NT <= 512, "accumulators must fit in TMEM");
    static_assert(NT % 16 == 0 && NT >= 16 && NT <= 128, "the MMA's N and the epilogue's 4-column loads");
    static_assert(STAGE % 1024 == 0 && B_TILE % 256 == 0, "stage and tile alignment of the 32-byte swizzle");
    // Two accumulator sets when they fit in TMEM (NT = 48): the MMAs of the
    // next unit then run while the epilogue drains the previous one.
    constexpr int NBUF = 2 * SC::NACC * NT <= 512 ? 2 : 1;

    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * STAGE);
    uint64_t* empty = full + NST;
    uint64_t* tfull = empty + NST;  // [NBUF]
    uint64_t* tempty = tfull + 2;   // [NBUF]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + 2);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long t_start = clock64();
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < NBUF; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], SP_EPI_WARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            int it = 0;
            bool ok = true;
            for (int ui = blockIdx.x; ui < P.nunits && ok; ui += gridDim.x) {
                const SplitUnit u = P.units[ui];
                const CUtensorMap* ma = (u.flags & 1) ? &mapA1 : &mapA0;
                const CUtensorMap* mb = (u.flags & 2) ? &mapB1 : &mapB0;
                for (int kb = 0; kb < u.ksteps; ++kb, ++it) {
                    const int st = it % NST;
                    const uint32_t ph = (it / NST) & 1;
                    const long long w0 = clock64();
                    if (!mbar_wait(&empty[st], ph ^ 1, P.err, 1)) { ok = false; break; }
                    if (P.dbg) atomicAdd(&P.dbg[0], (unsigned long long)(clock64() - w0));
                    mbar_expect_tx(&full[st], TX);
                    unsigned char* sa = smem + st * STAGE;
                    unsigned char* sb = sa + S * A_TILE;
                    // one box per operand: the S slices of 128 rows (A) and of NT rows (B)
                    tma_load_3d(sa, ma, &full[st], (u.k0 + kb) * SP_KB, u.a_row0, 0);
                    tma_load_3d(sb, mb, &full[st], (u.k0 + kb) * SP_KB, u.b_row0, 0);
                }
            }
            // drain: wait (bounded) for the copies this thread issued
            for (int q = 0; q < NST && it > 0; ++q) {
                const int j = it - 1 - q;
                if (j < 0) break;
                mbar_wait(&full[j % NST], (j / NST) & 1, P.err, 5);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            int it = 0, tile = 0;
            bool ok = true;
            for (int ui = blockIdx.x; ui < P.nunits && ok; ui += gridDim.x, ++tile) {
                const SplitUnit u = P.units[ui];
                // narrow units: one MMA per product, N = valid rows rounded up to 16
                const bool narrow = u.n <= P.narrow && NT > 32;
                const uint32_t idesc1 = idesc_bf16_f32(SP_M, narrow ? ((u.n + 15) & ~15) : NT);
                // accumulator set of this unit: the k-th use of set b is unit tile = k NBUF + b
                const int buf = NBUF == 2 ? (tile & 1) : 0;
                const uint32_t tacc = tmem + (uint32_t)(buf * 256);
                const long long w0 = clock64();
                if (!mbar_wait(&tempty[buf], ((tile / NBUF) & 1) ^ 1, P.err, 2)) { ok = false; break; }
                if (P.dbg) atomicAdd(&P.dbg[1], (unsigned long long)(clock64() - w0));
                tc_fence_after();
                for (int kb = 0; kb < u.ksteps; ++kb, ++it) {
                    const int st = it % NST;
                    const uint32_t ph = (it / NST) & 1;
                    const long long w1 = clock64();
                    if (!mbar_wait(&full[st], ph, P.err, 3)) { ok = false; break; }
                    if (P.dbg) atomicAdd(&P.dbg[2], (unsigned long long)(clock64() - w1));
                    tc_fence_after();
                    // descriptors differ only in the start-address field (address >> 4)
                    const uint64_t da = desc_sw32(smem_u32(smem + st * STAGE));
                    const uint64_t db = da + (uint64_t)((S * A_TILE) >> 4);
                    // A slice 0 comes first: its products start every accumulator
                    // (levels 0..S-1) in the first K block, all later ones add
#pragma unroll
                    for (int s = 0; s < S; ++s) {
                        const uint32_t acc = (kb > 0 || s > 0) ? 1u : 0u;
                        const uint64_t as = da + (uint64_t)((s * A_TILE) >> 4);
                        if (narrow) {
#pragma unroll
                            for (int t = 0; t < S - s; ++t)
                                umma_bf16(tacc + (uint32_t)((s + t) * NT), as, db + (uint64_t)((t * B_TILE) >> 4),
                                          idesc1, acc);
                        } else {
#pragma unroll
                            for (int t = 0; t < S - s; t += GMAX) {
                                const int g = (S - s - t) < GMAX ? (S - s - t) : GMAX;
                                umma_bf16(tacc + (uint32_t)((s + t) * NT), as, db + (uint64_t)((t * B_TILE) >> 4),
                                          idesc_bf16_f32(SP_M, g * NT), acc);
                            }
                        }
                    }
                    umma_commit(&empty[st]);
                }
                if (ok) umma_commit(&tfull[buf]);
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue ----------------
        const int q = warp & 3;              // TMEM lane quarter of this warp
        constexpr int CW = NT / (SP_EPI_WARPS / 4);  // columns per epilogue warp
        static_assert(CW % 4 == 0 && CW <= 64, "epilogue column split");
        const int part = (warp - 2) >> 2;    // which column part
        const int col0 = part * CW;
        int tile = 0;
        for (int ui = blockIdx.x; ui < P.nunits; ui += gridDim.x, ++tile) {
            const SplitUnit u = P.units[ui];
            const int r = 32 * q + lane;
            const bool rv = r < u.a_rows;
            const int row = u.a_row0 + (rv ? r : 0);
            const int amap = u.flags & 1, bmap = (u.flags >> 1) & 1;
            // exponents: the row's, and this warp's columns (one per lane, read by shuffles)
            const int* __restrict__ eav = amap ? P.ea[1] : P.ea[0];
            const int* __restrict__ ebv = bmap ? P.eb[1] : P.eb[0];
            const int ea = eav[row];
            // NT/2 <= 64 columns per warp: lane l holds the exponents of columns col0 + l and col0 + 32 + l
            const int ca = col0 + lane, cb = col0 + 32 + lane;
            const int eb_a = (ca < col0 + CW && ca < u.n) ? ebv[u.b_row0 + ca] : 0;
            const int eb_b = (CW > 32 && cb < col0 + CW && cb < u.n) ? ebv[u.b_row0 + cb] : 0;
            const typename Epi::Row R = epi.row(u, row);
            const int buf = NBUF == 2 ? (tile & 1) : 0;
            const uint32_t tacc = tmem + (uint32_t)(buf * 256);
            const long long w0 = clock64();
            const bool got = mbar_wait(&tfull[buf], (tile / NBUF) & 1, P.err, 4);
            const long long w1 = clock64();
            if (!__all_sync(0xffffffffu, got)) break;
            tc_fence_after();
            // phase 1: drain the accumulators of this warp's columns into exact
            // integers, then hand TMEM back to the MMA issuer.  Every
            // accumulator holds an integer: acc_0 (|acc_0| <= 256 2^14 = 2^22)
            // by an exact FP32 offset, the others by conversion; levels 0 and 1
            // combine in 32 bits (|acc_0| 2^8 + |acc_1| < 2^31), the rest by
            // 32 x 32 -> 64-bit multiply-adds (six slices) or Horner in 64 bits:
            // T = sum_d acc_d 2^{8 (S-1-d)}  (|T| < 2^63), and the product is
            // T 2^{eA + eB - 8 (S + 1)}.
            constexpr int TEXP = -8 * (S + 1);
            static_assert(SC::NACC == S && S >= 2, "one accumulator per level");
            long long T[CW];
            // warps whose columns are all past the unit's valid rows skip the work
            const bool active = col0 < u.n;
            if (active) {
#pragma unroll
            for (int c = 0; c < CW / 4; ++c) {
                uint32_t v[SC::NACC][4];
#pragma unroll
                for (int a = 0; a < SC::NACC; ++a)
                    tmem_ld4(tacc + ((uint32_t)(32 * q) << 16) + (uint32_t)(a * NT + col0 + 4 * c), v[a]);
                tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int i0 = __float_as_int(__uint_as_float(v[0][j]) + 12582912.0f) - 0x4B400000;
                    const int i01 = i0 * 256 + __float2int_rn(__uint_as_float(v[1][j]));
                    long long t;
                    if constexpr (S == 6) {
                        // levels 4 and 5 combined in FP32 at level 4's unit (2^8 of T):
                        // one rounding of the sum and one of the conversion, at most
                        // 1.5 units of level 4 (384 of T), against up to K 2^7 of T
                        // from the rounding of the operands to 48 bits
                        const int i45 = __float2int_rn(__fmaf_rn(__uint_as_float(v[5][j]), 0.00390625f,
                                                                 __uint_as_float(v[4][j])));
                        t = (long long)i01 * 4294967296LL;
                        t = mad_wide_s32(__float2int_rn(__uint_as_float(v[2][j])), 1 << 24, t);
                        t = mad_wide_s32(__float2int_rn(__uint_as_float(v[3][j])), 1 << 16, t);
                        t = mad_wide_s32(i45, 1 << 8, t);
                    } else {
                        t = i01;
#pragma unroll
                        for (int a = 2; a < SC::NACC; ++a) t = t * 256 + __float2int_rn(__uint_as_float(v[a][j]));
                    }
                    T[4 * c + j] = t;
                }
            }
            }
            tc_fence_before();
            __syncwarp();
            const long long w2 = clock64();
            if (lane == 0) mbar_arrive(&tempty[buf]);
            // phase 2 (overlaps the next tile's MMAs): FP64 results and stores
            if constexpr (raw_epi<Epi>::value) {
            if (active) {
#pragma unroll
            for (int c = 0; c < CW / 4; ++c) {
                long long oldr[4] = {0, 0, 0, 0};
                if constexpr (Epi::RMW) {
                    if (rv) {
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            if (col0 + 4 * c + j < u.n) epi.load_raw(R, col0 + 4 * c + j, &oldr[j]);
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int n = col0 + 4 * c + j;
                    const int idx = 4 * c + j;
                    int eb;
                    if constexpr (CW <= 32) {
                        eb = __shfl_sync(0xffffffffu, eb_a, idx);
                    } else {
                        const int e1 = __shfl_sync(0xffffffffu, eb_a, idx & 31);
                        const int e2 = __shfl_sync(0xffffffffu, eb_b, idx & 31);
                        eb = idx < 32 ? e1 : e2;
                    }
                    if (rv && n < u.n) epi.store_raw(R, u, n, T[4 * c + j], ea + eb + TEXP, oldr[j]);
                }
            }
            }
            } else {
            if (active) {
#pragma unroll
            for (int c = 0; c < CW / 4; ++c) {
                double old[4][2];
                double vv[4];  // pair-row epilogues: this row's values of the four columns
                if constexpr (Epi::RMW) {
                    if (rv) {
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            if (col0 + 4 * c + j < u.n) epi.load(R, col0 + 4 * c + j, old[j]);
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int n = col0 + 4 * c + j;
                    const int idx = 4 * c + j;
                    int eb;
                    if constexpr (CW <= 32) {
                        eb = __shfl_sync(0xffffffffu, eb_a, idx);
                    } else {
                        const int e1 = __shfl_sync(0xffffffffu, eb_a, idx & 31);
                        const int e2 = __shfl_sync(0xffffffffu, eb_b, idx & 31);
                        eb = idx < 32 ? e1 : e2;
                    }
                    if constexpr (pair_rows_epi<Epi>::value) {
                        // rows 2i and 2i + 1 are the two halves of one 16-byte
                        // pair at every column: neighbouring lanes swap one
                        // value, and each stores a whole pair, the even lane at
                        // the even column of the two and the odd lane at the
                        // odd one
                        vv[j] = i64_ldexp(T[4 * c + j], ea + eb + TEXP);
                        if (j & 1) {
                            const bool odd = lane & 1;
                            const double got = __shfl_xor_sync(0xffffffffu, odd ? vv[j - 1] : vv[j], 1);
                            const int np = odd ? n : n - 1;
                            if (rv && np < u.n)
                                epi.store_pair(R, np, odd ? make_double2(got, vv[j]) : make_double2(vv[j - 1], got),
                                               odd);
                        }
                    } else if (rv && n < u.n) {
                        const double v = i64_ldexp(T[4 * c + j], ea + eb + TEXP);
                        epi.store(R, u, n, v, old[j]);
                    }
                }
            }
            }
            }
            if (P.dbg && warp == 2 && lane == 0) {
                atomicAdd(&P.dbg[3], (unsigned long long)(w1 - w0));
                atomicAdd(&P.dbg[4], (unsigned long long)(w2 - w1));
                atomicAdd(&P.dbg[6], (unsigned long long)(clock64() - w2));
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (P.dbg && threadIdx.x == 0) atomicAdd(&P.dbg[5], (unsigned long long)(clock64() - t_start));
    if (threadIdx.x == 0) {  // the host reads this word instead of copying the device flag back
        const int e = *(volatile int*)P.err;
        if (e) *(volatile int*)P.host_err = e;
    }
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
}

// Self-test of the failure path: warp 0 waits, with a limit of limit_ns, on an
// mbarrier that nothing arrives on; warp 1 waits on another one with the
// GEMMs' own limit and must give up as soon as warp 0 has set the flag.  The
// flag reaches the host as in split_gemm_kernel.
__global__ void wait_expiry_kernel(int* err, int* host_err, long long limit_ns) {
    __shared__ __align__(8) uint64_t bar[2];
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        const int w = threadIdx.x >> 5;
        if (w == 0) mbar_wait(&bar[0], 0, err, 6, limit_ns);
        else mbar_wait(&bar[1], 0, err, 7);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int e = *(volatile int*)err;
        if (e) *(volatile int*)host_err = e;
    }
}

template <int S, int BITS, int NT>
constexpr size_t split_smem_bytes() {
    constexpr int NST = stage_count<S, BITS, NT>();
    return (size_t)NST * (S * SP_M * 32 + Sched<S>::NB * NT * 32) + 1024 + 256;
}

}  // namespace

// ===========================================================================
// Host side
// ===========================================================================
namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// [S][rows][Kp] bf16 slice array -> 3D map (Kp, rows, S), box (16, box_rows,
// S), 32B swizzle: one copy brings a tile of every slice, the slices one
// after the other in shared memory (rows past the array's end read as 0)
int make_map(CUtensorMap* map, const void* base, long long rows, int Kp, int S, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return fail(ZEST_GPU_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    if (rows >= (1ll << 31)) return fail(ZEST_GPU_ERR_UNSUPPORTED, "slice array too tall for TMA");
    cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)S};
    cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)rows * Kp * 2};
    cuuint32_t box[3] = {16, (cuuint32_t)box_rows, (cuuint32_t)S};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(ZEST_GPU_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ")");
    return ZEST_GPU_OK;
}

inline int r16(int k) { return (k + 15) & ~15; }

// table rows per tile: S accumulators of NT columns within the 512 TMEM columns
// (6 x 80, 5 x 96, 4 x 64 with two accumulator sets)
int n_tile(int S) { return S == 6 ? 80 : S == 5 ? 96 : 64; }

}  // namespace

// Slice arrays of one operand: [copies * S][rows][Kp] bf16 + per-row exponents
// (the GEMMs read one copy: every level has its own accumulator).
struct SliceArray {
    DevBuf data, ex;
    long long rows = 0;
    int Kp = 0;
    int S = 0;
    int copies = 1;
    int bits = 7;  // digit width of the slices
    int ensure(long long r, int kp, int s, int c = 1) {
        rows = r;
        Kp = kp;
        S = s;
        copies = c;
        ZG_TRY(data.ensure((size_t)c * s * r * kp * 2 + 256));
        ZG_TRY(ex.ensure((size_t)r * 4 + 16));
        return ZEST_GPU_OK;
    }
    __nv_bfloat16* ptr() const { return data.as<__nv_bfloat16>(); }
};

// Sliced tables of one Zernike plan for one slice count.
// work-list keys: (stage, Lg, Lm, batch, S, pass)
enum {
    WK_DFT_F = 0, WK_LEG_F, WK_RAD_F, WK_RAD_B, WK_LEG_B, WK_DFT_B, WK_DENSE, WK_ST_LEG_F, WK_ST_LEG_B,
    WK_ST_DFT_F, WK_ST_DFT_B, WK_ROT
};

// Sliced longitude DFT tables of one (order L, longitude count N): shared by
// the Zernike grids and the SH LonLat grids of the same order.
struct DftTables {
    SliceArray cos_f, sin_f, cos_b, sin_b;
    // the inverse tables sliced together (orders up to 256): row i of both
    // (sin row 0 = 0) shares one exponent; the sin slices hold m >= 1 at m - 1
    SliceArray cos_bj, sin_bj;
};

// Sliced tables of the two X(+-pi/2) products of a rotation, all l < Lmax:
// rows tri(l) + m, K = m' (see rot_table_kernel).
struct RotTables {
    SliceArray re1, im1, re2, im2;
};

struct ZtSplitTables {
    int S = 0;
    const DftTables* dft = nullptr;
    SliceArray leg_f, rad_f, rad_bT, leg_bT;
    // orders up to 256: the backward Legendre table at every latitude node,
    // rows (m, lat), K = l - m (no fold over the equator)
    SliceArray leg_bU;
};

// Sliced Legendre tables of one SH plan (the 128-row operand: no scaled copies).
struct StSplitTables {
    int S = 0;
    SliceArray leg_f, leg_bT;
};

// Work list of one GEMM launch, with its tensor-core work.
struct UnitList {
    std::vector<SplitUnit> v;
    int max_ksteps = 0;   // longest sum of a unit, in 16-wide K blocks
    double useful = 0.0;  // 2 * rows * table rows * K * products, valid tiles only
    double issued = 0.0;  // the same for full 128 x NT x 16k tiles
    DevBuf dev;
    std::vector<long long> rows;  // exact row offsets a hashed key stands for (ragged rotation)
    // mixed launches: the units of more than 32 valid table rows (80-column
    // tiles) and the others (32-column tiles), split on first use
    std::unique_ptr<UnitList> wide, narrow;
};

struct SplitState {
    DevBuf err;                 // device error flag of the GEMM kernels
    int* host_err = nullptr;    // its mirror in mapped, pinned host memory
    int* host_err_dev = nullptr;
    ~SplitState() {
        if (host_err) cudaFreeHost(host_err);
    }
    SliceArray op[2];           // data operands of the current stage
    std::map<std::tuple<const void*, int>, std::unique_ptr<ZtSplitTables>> zt_tables;  // per (plan, S)
    std::map<std::tuple<const void*, int>, std::unique_ptr<StSplitTables>> st_tables;  // per (plan, S)
    std::map<std::tuple<int, int, int>, std::unique_ptr<DftTables>> dft_tables;        // per (L, N, S)
    std::map<std::tuple<int, int>, std::unique_ptr<RotTables>> rot_tables;             // per (Lmax, S)
    std::map<std::tuple<int, int, int, int, int, int>, std::unique_ptr<UnitList>> units;  // cached work lists
    DevBuf tmp;                 // FP64 staging of generated tables
    DevBuf cycles;              // role wait counters, kept when ZEST_GPU_SPLIT_CYCLES is set
    bool cycles_on = false;
    int narrow = 32;            // widest unit (valid table rows) run as one MMA per product
    bool narrow_fixed = false;  // set by the tuning override: the autotuner keeps it
    // timed choice per (stage, Lg, Lm, batch): column tile | narrow threshold << 8
    std::map<std::tuple<int, int, int, int>, int> tuned;
    int nt[16];                 // column tile of each work-list stage: 0 = chosen per launch, or 32 / 80
    SplitState();
    double useful_flops = 0.0, issued_flops = 0.0;  // accumulated while profiling
};

// Column tiles are chosen per launch (stage_nt) unless pinned by the tuning
// override: 0 = automatic.
SplitState::SplitState() {
    for (int& v : nt) v = 0;
}

void destroy_split(SplitState* s) { delete s; }

// Bounded-wait error flag of the split GEMMs launched so far (0 if none); clears
// it.  Waits for the context stream, then reads the flag's host mirror: no
// device-to-host copy, which would queue behind the copies of a pipelined call.
int split_check_flag(zest_gpu_context* ctx) {
    SplitState* st = ctx->split.get();
    if (!st || !st->host_err) return ZEST_GPU_OK;
    ZG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    const int herr = *(volatile int*)st->host_err;
    if (herr) {
        *(volatile int*)st->host_err = 0;
        ZG_CUDA_TRY(cudaMemsetAsync(st->err.p, 0, sizeof(int), ctx->stream));
        ZG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        return fail(ZEST_GPU_ERR_TIMEOUT, "split GEMM: bounded wait expired (code " + std::to_string(herr) + ")");
    }
    return ZEST_GPU_OK;
}

namespace {

template <class Loader>
int run_slice(cudaStream_t s, const Loader& ld, SliceJob J) {
    if (J.rows <= 0) return ZEST_GPU_OK;
    if (J.K > SL_KMAX) return fail(ZEST_GPU_ERR_UNSUPPORTED, "split path: K above 2048");
    if (J.bits != 8) return fail(ZEST_GPU_ERR_INVALID, "split path: digit width");
    constexpr int NA = staged_arrays<Loader>();
    if ((J.Kp0 & 7) || (NA > 1 && (J.Kp1 & 7)) || J.Kp0 < J.K0 || (NA > 1 && J.Kp1 < J.K1))
        return fail(ZEST_GPU_ERR_INVALID, "split path: slice row length");
    if (std::max(J.Kp0, NA > 1 ? J.Kp1 : 0) == 0) return ZEST_GPU_OK;  // nothing to write
    J.KS = std::max(J.Kp0, NA > 1 ? J.Kp1 : 0) + Loader::SHIFT;
    if (J.K > J.KS) return fail(ZEST_GPU_ERR_INVALID, "split path: staged range");
    J.Ks = sl_row_stride(J.KS);
    J.R = slice_rows_per_block(NA * J.Ks * (int)sizeof(double));
    J.lr = 0;
    while ((1 << J.lr) < J.R) ++J.lr;
    const size_t smem = (size_t)NA * J.R * J.Ks * sizeof(double);
    if (smem > 100 * 1024) return fail(ZEST_GPU_ERR_UNSUPPORTED, "split path: slicing rows exceed shared memory");
    const long long blocks = (J.rows + J.R - 1) / J.R;
    auto go = [&](auto kern) -> int {
        ZG_TRY(set_attributes_once(kern, [](auto k) -> int {
            ZG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
            ZG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             cudaSharedmemCarveoutMaxShared));
            return ZEST_GPU_OK;
        }));
        kern<<<(unsigned)blocks, 256, smem, s>>>(ld, J);
        return launch_check("slice_kernel");
    };
    switch (J.S) {
    case 4: return go(slice_kernel<Loader, 4>);
    case 5: return go(slice_kernel<Loader, 5>);
    case 6: return go(slice_kernel<Loader, 6>);
    }
    return fail(ZEST_GPU_ERR_UNSUPPORTED, "split path supports 4..6 slices");
}

// One operand array from `up`.
template <class Loader>
int launch_slice(cudaStream_t s, const Loader& ld, long long rows, int K, int S, int bits, SliceArray& out) {
    static_assert(Loader::MODE == SL_ONE, "one-array loader");
    if (out.copies != 1) return fail(ZEST_GPU_ERR_INVALID, "split path: slice copies");
    out.bits = bits;
    SliceJob J{};
    J.rows = rows;
    J.K = J.K0 = J.Ku = K;
    J.Kp0 = out.Kp;
    J.S = S;
    J.bits = bits;
    J.out0 = out.ptr();
    J.stride0 = out.rows * out.Kp;
    J.ex0 = out.ex.as<int>();
    return run_slice(s, ld, J);
}

// Two operand arrays from one read: SL_FOLD (up + dn, up - dn), SL_PAIR
// (up, dn) or SL_PFOLD (up + up2, dn + dn2); the second holds k in
// [shift, shift + K1) at k - shift.  A fold needs K0 = K1 + shift (both sums
// end at the same input).
template <class Loader>
int launch_slice2(cudaStream_t s, const Loader& ld, long long rows, int K0, int K1, int shift, int S, int bits,
                  int mode, SliceArray& out0, SliceArray& out1) {
    out0.bits = out1.bits = bits;
    SliceJob J{};
    J.rows = rows;
    if (mode != Loader::MODE || shift != Loader::SHIFT)
        return fail(ZEST_GPU_ERR_INVALID, "split path: slicing mode of the loader");
    if (mode == SL_FOLD && K0 != K1 + shift) return fail(ZEST_GPU_ERR_INVALID, "split path: fold ranges");
    if (out0.copies != 1 || out1.copies != 1) return fail(ZEST_GPU_ERR_INVALID, "split path: slice copies");
    J.K0 = K0;
    J.K1 = K1;
    J.K = std::max(K0, K1 + shift);
    J.Ku = mode == SL_FOLD ? J.K : K0;
    J.Kd = mode == SL_FOLD ? J.K : K1 + shift;
    J.Kp0 = out0.Kp;
    J.Kp1 = out1.Kp;
    J.S = S;
    J.bits = bits;
    J.out0 = out0.ptr();
    J.out1 = out1.ptr();
    J.stride0 = out0.rows * out0.Kp;
    J.stride1 = out1.rows * out1.Kp;
    J.ex0 = out0.ex.as<int>();
    J.ex1 = out1.ex.as<int>();
    return run_slice(s, ld, J);
}

int get_state(zest_gpu_context* ctx, SplitState** out) {
    if (!ctx->split) {
        ctx->split.reset(new SplitState());
        ctx->split->cycles_on = std::getenv("ZEST_GPU_SPLIT_CYCLES") != nullptr;
        // tuning override: units of at most this many valid table rows (16..64)
        // issue one MMA per product instead of grouped full-width MMAs
        if (const char* e = std::getenv("ZEST_GPU_SPLIT_NARROW")) {
            // "mixed": units of up to 32 rows in a second launch of 32-column tiles
            const int v = std::string(e) == "mixed" ? SP_MIXED : std::atoi(e);
            if (v == SP_MIXED) {
                ctx->split->narrow = SP_MIXED;
                ctx->split->narrow_fixed = true;
            }
            if (v >= 16 && v <= 64) {
                ctx->split->narrow = v;
                ctx->split->narrow_fixed = true;
            }
        }
        // tuning override of the column tiles, "stage=nt,..." with stage one of
        // dft_f leg_f rad_f rad_b leg_b dft_b st_dft_f st_dft_b and nt 32 or 80
        if (const char* e = std::getenv("ZEST_GPU_SPLIT_NT")) {
            static const char* names[] = {"dft_f", "leg_f", "rad_f", "rad_b", "leg_b", "dft_b", "dense",
                                          "st_leg_f", "st_leg_b", "st_dft_f", "st_dft_b"};
            std::string spec(e);
            size_t pos = 0;
            while (pos < spec.size()) {
                size_t end = spec.find(',', pos);
                if (end == std::string::npos) end = spec.size();
                const std::string item = spec.substr(pos, end - pos);
                const size_t eq = item.find('=');
                if (eq != std::string::npos) {
                    const std::string key = item.substr(0, eq);
                    const int v = std::atoi(item.c_str() + eq + 1);
                    for (int i = 0; i < int(sizeof(names) / sizeof(names[0])); ++i)
                        if (key == names[i] && (v == 32 || v == 80)) ctx->split->nt[i] = v;
                }
                pos = end + 1;
            }
        }
        ZG_TRY(ctx->split->err.ensure(16));
        ZG_CUDA_TRY(cudaMemsetAsync(ctx->split->err.p, 0, 16, ctx->stream));
        ZG_CUDA_TRY(cudaHostAlloc((void**)&ctx->split->host_err, sizeof(int), cudaHostAllocMapped));
        *(volatile int*)ctx->split->host_err = 0;
        ZG_CUDA_TRY(cudaHostGetDevicePointer((void**)&ctx->split->host_err_dev, ctx->split->host_err, 0));
    }
    *out = ctx->split.get();
    return ZEST_GPU_OK;
}

// SH backward: the parity sums E[p][b][m][j][c] (groups with no degree below Lm
// read as 0) unfolded to X[b][m][lat][c], conjugated as the reference's sum_l
// writes them: north lat = j0u + j gets E_0 + E_1, south lat = j0d - j gets
// E_0 - E_1 (the equator of an odd grid, j0u = j0d, where E_1 = 0, is written
// twice with the same value).
__global__ void st_unfold_kernel(const double* __restrict__ E, double* __restrict__ X, int B, int L, int Lm, int kh,
                                 int nlat, int j0u, int j0d) {
    const long long n = (long long)B * L * kh * 2;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int c = int(t & 1);
    const long long q = t >> 1;
    const int j = int(q % kh);
    const long long bm = q / kh;
    const int m = int(bm % L), b = int(bm / L);
    const double e0 = (Lm - m > 0) ? E[(((long long)b * L + m) * kh + j) * 2 + c] : 0.0;
    const double e1 = (Lm - m - 1 > 0) ? E[((((long long)B + b) * L + m) * kh + j) * 2 + c] : 0.0;
    const double sg = c ? -1.0 : 1.0;
    double* x = X + (((long long)b * L + m) * nlat) * 2 + c;
    x[(long long)(j0u + j) * 2] = sg * (e0 + e1);
    x[(long long)(j0d - j) * 2] = sg * (e0 - e1);
}

// FP64 table generators
__global__ void dft_table_kernel(double* __restrict__ out, int rows, int K, int ld, int N, int row_off, int col_off,
                                 int mode) {
    // mode 0: cos(2 pi r c / N); 1: sin(2 pi r c / N); 2: (c>0 ? 2 : 1) cos; 3: -2 sin
    // r = row + row_off, c = col + col_off ; laid out [row][col] with stride ld
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (r >= rows || c >= ld) return;
    double v = 0.0;
    if (c < K) {
        const long long rr = r + row_off, cc = c + col_off;
        const long long t = (rr * cc) % N;
        double sn, cs;
        sincospi(2.0 * double(t) / double(N), &sn, &cs);
        if (mode == 0) v = cs;
        else if (mode == 1) v = sn;
        else if (mode == 2) v = (cc > 0 ? 2.0 : 1.0) * cs;
        else v = -2.0 * sn;
    }
    out[(long long)r * ld + c] = v;
}

// out[(blk*nrow + k) * ld + i] = in[(off[blk] + i) * nrow + k] for i < cnt[blk] else 0
__global__ void transpose_blocks_kernel(const double* __restrict__ in, const long long* __restrict__ off,
                                        const int* __restrict__ cnt, int nrow, int ld, double* __restrict__ out) {
    const int blk = blockIdx.y;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nrow * ld) return;
    const int k = e / ld, i = e - k * ld;
    out[((long long)blk * nrow + k) * ld + i] = (i < cnt[blk]) ? in[(off[blk] + i) * nrow + k] : 0.0;
}

// out[(m nlat + lat) ld + q] = P_{m+q}^m at latitude node lat, from the folded
// backward blocks Pb[(off[2m + p] + i) kh + j] (l = m + p + 2i at folded node
// j): north nodes lat = j0u + j as they are, south nodes lat = j0d - j with
// the sign (-1)^(l - m); zero from q = L - m on.
__global__ void unfold_leg_table_kernel(const double* __restrict__ Pb, const long long* __restrict__ off, int L,
                                        int kh, int nlat, int j0u, int j0d, int ld, double* __restrict__ out) {
    const long long rowi = blockIdx.y;  // m nlat + lat
    const int m = int(rowi / nlat), lat = int(rowi - (long long)m * nlat);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ld) return;
    double v = 0.0;
    if (q < L - m) {
        const int p = q & 1, i = q >> 1;
        const bool north = lat >= j0u;
        const int j = north ? lat - j0u : j0d - lat;
        v = Pb[(off[2 * m + p] + i) * kh + j];
        if (!north && p) v = -v;
    }
    out[rowi * ld + q] = v;
}

int slice_table(zest_gpu_context* ctx, const double* src, long long rows, int K, int ld, int S, int bits,
                SliceArray& dst, int copies = 1) {
    ZG_TRY(dst.ensure(rows, r16(K), S, copies));
    return launch_slice(ctx->stream, RowMajorLoader{src, ld}, rows, K, S, bits, dst);
}

// The longitude DFT tables of order L over N longitudes, sliced (cached).
int build_dft_tables(zest_gpu_context* ctx, SplitState* st, int L, int N, int S, const DftTables** out) {
    auto key = std::make_tuple(L, N, S);
    auto it = st->dft_tables.find(key);
    if (it != st->dft_tables.end()) {
        *out = it->second.get();
        return ZEST_GPU_OK;
    }
    cudaStream_t s = ctx->stream;
    auto t = std::make_unique<DftTables>();
    const int ld = r16(L);
    // room for the two inverse tables sliced together (below), so that no
    // queued slicing job reads a buffer that was reallocated
    ZG_TRY(st->tmp.ensure((size_t)2 * L * ld * sizeof(double)));
    double* tmp = st->tmp.as<double>();
    auto gen = [&](int rows, int K, int row_off, int col_off, int mode, SliceArray& dst) -> int {
        dim3 grid((ld + 127) / 128, rows);
        dft_table_kernel<<<grid, 128, 0, s>>>(tmp, rows, K, ld, N, row_off, col_off, mode);
        ZG_TRY(launch_check("dft_table_kernel"));
        return slice_table(ctx, tmp, rows, K, ld, S, digit_bits(L), dst);
    };
    // forward: cos rows m in [0,L), cols i in [0,L); sin rows m in [1,L), cols i in [1,L)
    ZG_TRY(gen(L, L, 0, 0, 0, t->cos_f));
    if (L > 1) ZG_TRY(gen(L - 1, L - 1, 1, 1, 1, t->sin_f));
    // backward: cos rows i in [0,L), cols m in [0,L); sin rows i in [1,L), cols m in [1,L)
    // (K-chunked sums, orders above 256; single sums use the joint tables below)
    if (L > KCHUNK || L == 1) ZG_TRY(gen(L, L, 0, 0, 2, t->cos_b));
    if (L > KCHUNK) ZG_TRY(gen(L - 1, L - 1, 1, 1, 3, t->sin_b));
    if (L > 1 && L <= KCHUNK) {
        // both inverse tables over all rows i and m, sliced in one job with shared row
        // exponents (the earlier tables' slicing jobs are queued before these writes)
        ZG_CUDA_TRY(cudaStreamSynchronize(s));
        double* P = tmp;
        double* Q = P + (size_t)L * ld;
        dim3 grid((ld + 127) / 128, L);
        dft_table_kernel<<<grid, 128, 0, s>>>(P, L, L, ld, N, 0, 0, 2);
        ZG_TRY(launch_check("dft_table_kernel"));
        dft_table_kernel<<<grid, 128, 0, s>>>(Q, L, L, ld, N, 0, 0, 3);
        ZG_TRY(launch_check("dft_table_kernel"));
        ZG_TRY(t->cos_bj.ensure(L, r16(L), S));
        ZG_TRY(t->sin_bj.ensure(L, r16(L), S));
        ZG_TRY(launch_slice2(s, TablePairLoader{P, Q, ld}, L, L, L - 1, 1, S, 8, SL_PAIR, t->cos_bj, t->sin_bj));
    }
    ZG_CUDA_TRY(cudaStreamSynchronize(s));
    *out = t.get();
    st->dft_tables.emplace(key, std::move(t));
    return ZEST_GPU_OK;
}

int build_zt_tables(zest_gpu_context* ctx, SplitState* st, ZtPlan& plan, int S, ZtSplitTables** out) {
    auto key = std::make_tuple((const void*)&plan, S);
    auto it = st->zt_tables.find(key);
    if (it != st->zt_tables.end()) {
        *out = it->second.get();
        return ZEST_GPU_OK;
    }
    cudaStream_t s = ctx->stream;
    auto t = std::make_unique<ZtSplitTables>();
    t->S = S;
    const int L = int(plan.sh.L), N = int(plan.sh.nlon), nr = int(plan.sh.nrad), kh = plan.leg.nnodes;
    ZG_TRY(build_dft_tables(ctx, st, L, N, S, &t->dft));
    // forward Legendre and radial tables (FP64 tables of the plain form)
    ZG_TRY(slice_table(ctx, plan.leg.Pf.as<double>(), plan.leg.off_h[2 * (size_t)L], kh, kh, S, digit_bits(kh),
                       t->leg_f));
    ZG_TRY(slice_table(ctx, plan.rad.Rf.as<double>(), plan.rad.off_h[L], nr, nr, S, digit_bits(nr), t->rad_f));
    // backward tables: transposed blocks
    {
        const int kl = r16((L + 1) / 2);
        // Legendre: per (m,p) block [kh][cnt] from Pb
        std::vector<int> cnt(2 * (size_t)L);
        for (int m = 0; m < L; ++m)
            for (int p = 0; p < 2; ++p) cnt[2 * m + p] = (L - m - p > 0) ? (L - m - p + 1) / 2 : 0;
        DevBuf dcnt;
        ZG_TRY(upload(dcnt, cnt, s));
        ZG_TRY(st->tmp.ensure((size_t)2 * L * kh * kl * sizeof(double)));
        dim3 g1((kh * kl + 255) / 256, 2 * L);
        transpose_blocks_kernel<<<g1, 256, 0, s>>>(plan.leg.Pb.as<double>(), plan.leg.off.as<long long>(),
                                                   dcnt.as<int>(), kh, kl, st->tmp.as<double>());
        ZG_TRY(launch_check("transpose_blocks_kernel"));
        ZG_TRY(slice_table(ctx, st->tmp.as<double>(), (long long)2 * L * kh, kl, kl, S, digit_bits((L + 1) / 2),
                           t->leg_bT));
        ZG_CUDA_TRY(cudaStreamSynchronize(s));
        // radial: per l block [nr][cnt(l)] from Rb
        std::vector<int> rc((size_t)L);
        for (int l = 0; l < L; ++l) rc[l] = (L - l + 1) / 2;
        DevBuf drc;
        ZG_TRY(upload(drc, rc, s));
        ZG_TRY(st->tmp.ensure((size_t)L * nr * kl * sizeof(double)));
        dim3 g2((nr * kl + 255) / 256, L);
        transpose_blocks_kernel<<<g2, 256, 0, s>>>(plan.rad.Rb.as<double>(), plan.rad.off.as<long long>(),
                                                   drc.as<int>(), nr, kl, st->tmp.as<double>());
        ZG_TRY(launch_check("transpose_blocks_kernel"));
        ZG_TRY(slice_table(ctx, st->tmp.as<double>(), (long long)L * nr, kl, kl, S, digit_bits((L + 1) / 2),
                           t->rad_bT));
        ZG_CUDA_TRY(cudaStreamSynchronize(s));
        if (L <= KCHUNK) {
            const int nlat = int(plan.sh.nlat), ku = r16(L);
            ZG_TRY(st->tmp.ensure((size_t)L * nlat * ku * sizeof(double)));
            dim3 g3((ku + 127) / 128, (unsigned)((long long)L * nlat));
            unfold_leg_table_kernel<<<g3, 128, 0, s>>>(plan.leg.Pb.as<double>(), plan.leg.off.as<long long>(), L,
                                                       kh, nlat, plan.leg.j0u, plan.leg.j0d, ku,
                                                       st->tmp.as<double>());
            ZG_TRY(launch_check("unfold_leg_table_kernel"));
            ZG_TRY(slice_table(ctx, st->tmp.as<double>(), (long long)L * nlat, L, ku, S, 8, t->leg_bU));
            ZG_CUDA_TRY(cudaStreamSynchronize(s));
        }
    }
    *out = t.get();
    st->zt_tables.emplace(key, std::move(t));
    return ZEST_GPU_OK;
}

template <int S, int BITS, int NT, class Epi>
int run_gemm_t(zest_gpu_context* ctx, UnitList& ul, const SliceArray& A0, const SliceArray& A1, const SliceArray& B0,
               const SliceArray& B1, const Epi& epi) {
    const std::vector<SplitUnit>& units = ul.v;
    if (units.empty()) return ZEST_GPU_OK;
    SplitState* st;
    ZG_TRY(get_state(ctx, &st));
    cudaStream_t s = ctx->stream;
    CUtensorMap ma0, ma1, mb0, mb1;
    if (A0.copies != 1 || A1.copies != 1 || B0.copies != 1 || B1.copies != 1)
        return fail(ZEST_GPU_ERR_INVALID, "split GEMM: operands must hold one copy of their slices");
    // the FP32 level sums stay exact only up to these lengths
    if (ul.max_ksteps * SP_KB > (BITS == 8 ? SL_K8MAX : SL_KMAX))
        return fail(ZEST_GPU_ERR_INVALID, "split GEMM: sum too long for exact level sums");
    if (A0.S != S || A1.S != S || B0.S != S || B1.S != S)
        return fail(ZEST_GPU_ERR_INVALID, "split GEMM: operands sliced with another slice count");
    ZG_TRY(make_map(&ma0, A0.ptr(), A0.rows, A0.Kp, S, SP_M));
    ZG_TRY(make_map(&ma1, A1.ptr(), A1.rows, A1.Kp, S, SP_M));
    ZG_TRY(make_map(&mb0, B0.ptr(), B0.rows, B0.Kp, S, NT));
    ZG_TRY(make_map(&mb1, B1.ptr(), B1.rows, B1.Kp, S, NT));
    if (!ul.dev.p) {  // work lists are uploaded once and cached with their key
        ZG_TRY(ul.dev.ensure(units.size() * sizeof(SplitUnit)));
        ZG_CUDA_TRY(cudaMemcpyAsync(ul.dev.p, units.data(), units.size() * sizeof(SplitUnit),
                                    cudaMemcpyHostToDevice, s));
    }
    if (ctx->prof.on) {
        st->useful_flops += ul.useful;
        st->issued_flops += ul.issued;
    }
    SplitParams P;
    P.units = ul.dev.as<SplitUnit>();
    P.nunits = int(units.size());
    P.ea[0] = A0.ex.as<int>();
    P.ea[1] = A1.ex.as<int>();
    P.eb[0] = B0.ex.as<int>();
    P.eb[1] = B1.ex.as<int>();
    P.err = st->err.as<int>();
    P.host_err = st->host_err_dev;
    P.narrow = st->narrow;
    P.dbg = nullptr;
    if (st->cycles_on) {
        ZG_TRY(st->cycles.ensure(8 * sizeof(unsigned long long)));
        ZG_CUDA_TRY(cudaMemsetAsync(st->cycles.p, 0, 8 * sizeof(unsigned long long), s));
        P.dbg = st->cycles.as<unsigned long long>();
    }
    const size_t smem = split_smem_bytes<S, BITS, NT>();
    ZG_TRY(set_attributes_once(split_gemm_kernel<S, BITS, NT, Epi>, [smem](auto k) -> int {
        ZG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return ZEST_GPU_OK;
    }));
    int nsm = 0;
    ZG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    const int grid = std::min<int>(int(units.size()), nsm);
    {
        StageScope sc(ctx, ST_SPLIT_GEMM);
        split_gemm_kernel<S, BITS, NT, Epi><<<grid, SP_THREADS, smem, s>>>(ma0, ma1, mb0, mb1, P, epi);
        ZG_TRY(launch_check("split_gemm_kernel"));
    }
    // A bounded-wait timeout reaches the caller through split_finish at the end
    // of the transform; the launches after a timed-out one see the device flag
    // and return at their first wait.
    if (P.dbg) {  // mean cycles per CTA in each wait, and in the epilogue's own work
        ZG_CUDA_TRY(cudaStreamSynchronize(s));
        unsigned long long c[8];
        ZG_CUDA_TRY(cudaMemcpy(c, P.dbg, sizeof(c), cudaMemcpyDeviceToHost));
        const char* fn = __PRETTY_FUNCTION__;
        const char* tag = std::strstr(fn, "Epi = ");
        std::fprintf(stderr,
                     "split_gemm S=%d NT=%d %.40s units=%zu grid=%d: total %.0f | producer waits %.0f | mma waits "
                     "tmem %.0f, smem %.0f | epilogue waits %.0f, drains %.0f, stores %.0f (cycles per CTA)\n",
                     S, NT, tag ? tag + 6 : "", units.size(), grid, double(c[5]) / grid, double(c[0]) / grid,
                     double(c[1]) / grid,
                     double(c[2]) / grid, double(c[3]) / grid, double(c[4]) / grid, double(c[6]) / grid);
    }
    return ZEST_GPU_OK;
}

// slice products per K block: pairs (s, t) of S slices with s + t <= the kept top level
inline int products(int S, int bits) {
    const int dmax = bits == 8 ? S - 1 : S;
    int n = 0;
    for (int a = 0; a < S; ++a)
        for (int b = 0; b < S; ++b) n += (a + b <= dmax);
    return n;
}

// Returns the cached work list of `key`, built by `build` on first use.
template <class Build>
int get_units(zest_gpu_context* ctx, std::tuple<int, int, int, int, int, int> key, Build&& build, UnitList** out) {
    SplitState* st;
    ZG_TRY(get_state(ctx, &st));
    auto it = st->units.find(key);
    if (it == st->units.end()) {
        auto ul = std::make_unique<UnitList>();
        build(*ul);
        it = st->units.emplace(key, std::move(ul)).first;
    }
    *out = it->second.get();
    return ZEST_GPU_OK;
}

// The split GEMM of a work list, its column tile NT chosen at run time: with
// six slices 80 (one accumulator set) or 32 (two sets, so that the next
// unit's MMAs overlap the epilogue's drain); five slices use 96 and four 64.
// Later K-chunks of long sums need six slices.
template <class Epi>
int run_gemm_nt(zest_gpu_context* ctx, int nt, int S, UnitList& ul, const SliceArray& A0, const SliceArray& A1,
                const SliceArray& B0, const SliceArray& B1, const Epi& epi) {
    const int bits = A0.bits;
    if (A1.bits != bits || B0.bits != bits || B1.bits != bits)
        return fail(ZEST_GPU_ERR_INVALID, "split GEMM: operands sliced with different digit widths");
    if (bits != 8) return fail(ZEST_GPU_ERR_INVALID, "split GEMM: operands need 8-bit digits");
    if (Epi::CHUNK && S != 6)
        return fail(ZEST_GPU_ERR_UNSUPPORTED, "split path: sums longer than 256 terms need 6 slices");
    SplitState* st;
    ZG_TRY(get_state(ctx, &st));
    if (S == 6 && nt == 80 && st->narrow == SP_MIXED) {
        // mixed: units of at most 32 valid table rows run in a second launch of
        // 32-column tiles (one MMA per A slice over all levels), the others in
        // 80-column tiles; the two launches write disjoint outputs
        if (!ul.wide) {
            ul.wide.reset(new UnitList());
            ul.narrow.reset(new UnitList());
            for (const SplitUnit& u : ul.v) (u.n <= 32 ? ul.narrow : ul.wide)->v.push_back(u);
            ul.wide->max_ksteps = ul.narrow->max_ksteps = ul.max_ksteps;
        }
        if (ctx->prof.on) {  // the halves carry no flop counts of their own
            st->useful_flops += ul.useful;
            st->issued_flops += ul.issued;
        }
        const int rc = run_gemm_t<6, 8, 80>(ctx, *ul.wide, A0, A1, B0, B1, epi);
        if (rc != ZEST_GPU_OK) return rc;
        return run_gemm_t<6, 8, 32>(ctx, *ul.narrow, A0, A1, B0, B1, epi);
    }
    switch (S) {
    case 6: return nt == 32 ? run_gemm_t<6, 8, 32>(ctx, ul, A0, A1, B0, B1, epi)
                            : run_gemm_t<6, 8, 80>(ctx, ul, A0, A1, B0, B1, epi);
    case 5: return run_gemm_t<5, 8, 96>(ctx, ul, A0, A1, B0, B1, epi);
    case 4: return run_gemm_t<4, 8, 64>(ctx, ul, A0, A1, B0, B1, epi);
    }
    return fail(ZEST_GPU_ERR_UNSUPPORTED, "split path supports 4..6 slices");
}

// tiles of a group: operand rows [a0, a0 + arows) x table rows [b0, b0 + nrows), K = kk
void add_units(UnitList& ul, int S, int bits, long long a0, long long arows, int b0, int nrows, int NT, int kk,
               int flags, int g, int k0 = 0) {
    if (arows <= 0 || nrows <= 0 || kk <= 0) return;
    const int ksteps = r16(kk) / 16;
    ul.max_ksteps = std::max(ul.max_ksteps, ksteps);
    const double P = products(S, bits);
    for (long long r = 0; r < arows; r += SP_M)
        for (int c = 0; c < nrows; c += NT) {
            SplitUnit u;
            u.a_row0 = int(a0 + r);
            u.a_rows = int(std::min<long long>(SP_M, arows - r));
            u.b_row0 = b0 + c;
            u.n = std::min(NT, nrows - c);
            u.ksteps = ksteps;
            // a unit of at most 32 valid rows runs N = its rows rounded up to 16
            const int ncols = (u.n <= 32 && NT > 32) ? r16(u.n) : NT;
            u.flags = flags;
            u.g = g;
            u.aux = c;
            u.k0 = k0 / 16;
            ul.v.push_back(u);
            ul.useful += 2.0 * u.a_rows * u.n * kk * P;
            ul.issued += 2.0 * SP_M * ncols * 16.0 * ksteps * P;
        }
}


// Column tile of a stage's launches with six slices, also part of the
// work-list key; ncols = the most table rows a group of the stage has.
//   * 32 where no group has more than 32 columns (the small orders of a
//     ragged batch): two accumulator sets, and an 80-wide tile would be at
//     least 60% empty;
//   * 80 otherwise: one set of six 80-column accumulators, MMAs of up to
//     three products (N = 240).
// A tuning override (ZEST_GPU_SPLIT_NT) can pin a stage to 32 or 80.
inline int stage_nt(const SplitState* st, int wk, int S, int ncols) {
    if (S != 6) return n_tile(S);
    if (st->nt[wk]) return st->nt[wk];
    return ncols <= 32 ? 32 : 80;
}
inline int nt_pass(int nt) { return nt == 32 ? 1 << 16 : 0; }

// Runs one split GEMM stage, `launch(nt)`, with its column tile and narrow
// threshold: a tuning override (ZEST_GPU_SPLIT_NT) if set; else, with the
// context's autotuner on, outside graph capture and for a stage whose
// launches overwrite their outputs (single sums), the fastest of the
// candidates (80 columns with units of up to 32, 48 or 64 valid table rows
// issued as one MMA per product; 80 columns with the units of up to 32 rows
// in a second launch of 32-column tiles; or 32 columns), timed with CUDA events on
// the context stream at the stage's first run at this size (each candidate
// once untimed, then once timed; neither choice changes a result); else the
// rule of stage_nt.
template <class Launch>
int tuned_stage(zest_gpu_context* ctx, SplitState* st, int wk, int S, int Lg, int Lm, int batch, int ncols,
                bool idempotent, Launch&& launch) {
    int nt = stage_nt(st, wk, S, ncols);
    if (S != 6 || st->nt[wk] || !ctx->autotune || !idempotent) return launch(nt);
    const int narrow0 = st->narrow;
    // runs candidate (t, w): tile t, narrow threshold w
    auto run = [&](int t, int w) -> int {
        st->narrow = w;
        const int rc = launch(t);
        st->narrow = narrow0;
        return rc;
    };
    const auto key = std::make_tuple(wk, Lg, Lm, batch);
    auto it = st->tuned.find(key);
    if (it != st->tuned.end()) return run(it->second & 0xFF, it->second >> 8);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    ZG_CUDA_TRY(cudaStreamIsCapturing(ctx->stream, &cap));
    if (cap != cudaStreamCaptureStatusNone) return launch(nt);
    cudaEvent_t e0, e1;
    ZG_CUDA_TRY(cudaEventCreate(&e0));
    ZG_CUDA_TRY(cudaEventCreate(&e1));
    const bool prof = ctx->prof.on;  // the timing runs stay out of the stage profile
    ctx->prof.on = false;
    const int cand[5][2] = {{80, 32}, {80, 48}, {80, 64}, {80, SP_MIXED}, {32, 32}};
    float best = 0.0f;
    int choice = nt | (narrow0 << 8);
    int rc = ZEST_GPU_OK;
    for (int i = 0; i < 5 && rc == ZEST_GPU_OK; ++i) {
        // one tile of at most 32 columns: the thresholds agree; a fixed threshold is kept
        if (i > 0 && i < 4 && (ncols <= 32 || st->narrow_fixed)) continue;
        const int w = st->narrow_fixed ? narrow0 : cand[i][1];
        rc = run(cand[i][0], w);
        if (rc == ZEST_GPU_OK && cudaEventRecord(e0, ctx->stream) != cudaSuccess) rc = fail(ZEST_GPU_ERR_CUDA, "event");
        if (rc == ZEST_GPU_OK) rc = run(cand[i][0], w);
        if (rc == ZEST_GPU_OK && cudaEventRecord(e1, ctx->stream) != cudaSuccess) rc = fail(ZEST_GPU_ERR_CUDA, "event");
        float ms = 0.0f;
        if (rc == ZEST_GPU_OK &&
            (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
            rc = fail(ZEST_GPU_ERR_CUDA, "split tile autotuner: timing failed");
        if (rc == ZEST_GPU_OK && (i == 0 || ms < best)) {
            best = ms;
            choice = cand[i][0] | (w << 8);
        }
    }
    ctx->prof.on = prof;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != ZEST_GPU_OK) return rc;
    st->tuned.emplace(key, choice);
    return run(choice & 0xFF, choice >> 8);
}

// Longitude DFT of `batch` grids x[b][lon][col] (C columns, item stride gsz)
// to the spectra G[b][m][col][re, im], m < Lm (L = Lg orders per item):
// folded cos/sin products (x_k + x_{N-k} against cos, x_k - x_{N-k} against
// sin), K-chunked.  `wk` keys the work lists of the caller's grid family.
int dft_forward_stage(zest_gpu_context* ctx, SplitState* st, const DftTables& t, int S, int wk, const double* grids,
                      long long gsz, int C, int N, int Lg, int Lm, int batch, double* G) {
    const int bits = digit_bits(Lg);
    const long long rows = (long long)batch * C;
    ZG_TRY(st->op[0].ensure(rows, r16(Lg), S));
    ZG_TRY(st->op[1].ensure(rows, r16(Lg), S));
    {
        StageScope sc(ctx, ST_SPLIT_SLICE);
        ZG_TRY(launch_slice2(ctx->stream, DftFwdLoader{grids, gsz, C, N}, rows, Lg, Lg - 1, 1, S, bits, SL_FOLD,
                             st->op[0], st->op[1]));
    }
    return tuned_stage(ctx, st, wk, S, Lg, Lm, batch, Lm, nchunks(Lg) == 1, [&](int NT) -> int {
        for (int ch = 0; ch < nchunks(Lg); ++ch) {
            const int k0 = ch * KCHUNK;
            UnitList* u;
            ZG_TRY(get_units(ctx, std::make_tuple(wk, Lg, Lm, batch, S, 8 * ch + nt_pass(NT)), [&](UnitList& ul) {
                for (long long r = 0; r < rows; r += SP_M) {
                    const long long rr = std::min<long long>(SP_M, rows - r);
                    add_units(ul, S, bits, r, rr, 0, Lm, NT, std::min(KCHUNK, Lg - k0), 0, 0, k0);
                    if (Lm > 1)
                        add_units(ul, S, bits, r, rr, 0, Lm - 1, NT, std::min(KCHUNK, Lg - 1 - k0), 1 | 2, 0, k0);
                }
            }, &u));
            if (ch == 0)
                ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], t.cos_f, t.sin_f,
                                   EpiDftFwd<false>{G, C, Lg}));
            else
                ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], t.cos_f, t.sin_f,
                                   EpiDftFwd<true>{G, C, Lg}));
        }
        return ZEST_GPU_OK;
    });
}

// The parity sums E_p[b][m][j][kc] (kc < nr2) a Legendre stage leaves
// unwritten, which the inverse DFT reads as 0: E_0 for m >= Lm, E_1 for
// m >= Lm - 1 (its last group is empty).
int zero_parity_tails(zest_gpu_context* ctx, double* E, int batch, int Lg, int Lm, int kh, int nr2) {
    StageScope sc(ctx, ST_MEMSET);
    const long long eblock = (long long)Lg * kh * nr2;  // one (p, b)
    const size_t row = (size_t)kh * nr2 * sizeof(double);
    if (Lm < Lg)
        ZG_CUDA_TRY(cudaMemset2DAsync(E + (size_t)Lm * kh * nr2, eblock * sizeof(double), 0, (size_t)(Lg - Lm) * row,
                                      batch, ctx->stream));
    ZG_CUDA_TRY(cudaMemset2DAsync(E + (size_t)batch * eblock + (size_t)(Lm - 1) * kh * nr2, eblock * sizeof(double), 0,
                                  (size_t)(Lg - Lm + 1) * row, batch, ctx->stream));
    return ZEST_GPU_OK;
}

// Inverse longitude DFT of the spectra the loader forms (rows (b, col), C
// columns) to the grids x[b][lon][col] (item stride gsz): a cos pass writing
// x_0 and the cos sums C_i (to Cs, batch * Lg * C doubles), then a sin pass
// reading them and writing x_i = C_i + S_i, x_{N-i} = C_i - S_i; both K-chunked.
template <class Loader>
int dft_backward_stage(zest_gpu_context* ctx, SplitState* st, const DftTables& t, int S, int wk,
                       const Loader& ld, int C, int N, int Lg, int Lm, int batch, double* grids, long long gsz,
                       double* Cs) {
    const int bits = digit_bits(Lg);
    const long long rows = (long long)batch * C;
    ZG_TRY(st->op[0].ensure(rows, r16(Lg), S));
    ZG_TRY(st->op[1].ensure(rows, r16(Lg), S));
    {
        StageScope sc(ctx, ST_SPLIT_SLICE);
        ZG_TRY(launch_slice2(ctx->stream, ld, rows, Lg, Lg - 1, 1, S, bits, Loader::MODE, st->op[0], st->op[1]));
    }
    if (Lg > 1 && Lg <= KCHUNK && t.cos_bj.rows) {
      // single sums: the cos and sin results combined in integers (the pair of
      // launches overwrites its outputs: tuned)
      return tuned_stage(ctx, st, wk, S, Lg, Lm, batch, Lg, true, [&](int NT) -> int {
        long long* Ts = reinterpret_cast<long long*>(Cs);
        UnitList* u;
        ZG_TRY(get_units(ctx, std::make_tuple(wk, Lg, Lm, batch, S, 4 + nt_pass(NT)), [&](UnitList& ul) {
            for (long long r = 0; r < rows; r += SP_M)
                add_units(ul, S, bits, r, std::min<long long>(SP_M, rows - r), 0, Lg, NT, Lg, 0, 0, 0);
        }, &u));
        ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], t.cos_bj, t.sin_bj,
                           EpiDftBwdCosRaw{grids, Ts, C, N, Lg, gsz}));
        UnitList* v;
        ZG_TRY(get_units(ctx, std::make_tuple(wk, Lg, Lm, batch, S, 5 + nt_pass(NT)), [&](UnitList& ul) {
            for (long long r = 0; r < rows; r += SP_M)  // sin rows i = 1 + (0 .. Lg - 2) of the joint table
                add_units(ul, S, bits, r, std::min<long long>(SP_M, rows - r), 1, Lg - 1, NT, Lg - 1, 1 | 2 | 4, 0,
                          0);
        }, &v));
        return run_gemm_nt(ctx, NT, S, *v, st->op[0], st->op[1], t.cos_bj, t.sin_bj,
                           EpiDftBwdSinRaw{grids, Ts, C, N, Lg, gsz});
      });
    }
    const int NT = stage_nt(st, wk, S, Lg);
    for (int ch = 0; ch < nchunks(Lg); ++ch) {
        const int k0 = ch * KCHUNK;
        UnitList* u;
        ZG_TRY(get_units(ctx, std::make_tuple(wk, Lg, Lm, batch, S, 8 * ch + nt_pass(NT)), [&](UnitList& ul) {
            for (long long r = 0; r < rows; r += SP_M)
                add_units(ul, S, bits, r, std::min<long long>(SP_M, rows - r), 0, Lg, NT, std::min(KCHUNK, Lg - k0),
                          0, 0, k0);
        }, &u));
        if (ch == 0)
            ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], t.cos_b, t.sin_b,
                            EpiDftBwdCos<false>{grids, Cs, C, N, Lg, gsz}));
        else
            ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], t.cos_b, t.sin_b,
                            EpiDftBwdCos<true>{grids, Cs, C, N, Lg, gsz}));
    }
    // the sin pass after every cos chunk: its first chunk reads the finished C_i
    for (int ch = 0; Lg > 1 && ch < nchunks(Lg - 1); ++ch) {
        const int k0 = ch * KCHUNK;
        UnitList* v;
        ZG_TRY(get_units(ctx, std::make_tuple(wk, Lg, Lm, batch, S, 1 + 8 * ch + nt_pass(NT)), [&](UnitList& ul) {
            for (long long r = 0; r < rows; r += SP_M)
                add_units(ul, S, bits, r, std::min<long long>(SP_M, rows - r), 0, Lg - 1, NT,
                          std::min(KCHUNK, Lg - 1 - k0), 1 | 2 | 4, 0, k0);
        }, &v));
        if (ch == 0)
            ZG_TRY(run_gemm_nt(ctx, NT, S, *v, st->op[0], st->op[1], t.cos_b, t.sin_b,
                            EpiDftBwdSin<false>{grids, Cs, C, N, Lg, gsz}));
        else
            ZG_TRY(run_gemm_nt(ctx, NT, S, *v, st->op[0], st->op[1], t.cos_b, t.sin_b,
                            EpiDftBwdSin<true>{grids, Cs, C, N, Lg, gsz}));
    }
    return ZEST_GPU_OK;
}

// SH Legendre tables in digit slices: the forward table (weights and the
// quadrature prefactor folded in, rows (m, p, l), K = folded nodes) and the
// backward table transposed per group (m, p) to rows = folded nodes,
// K = degrees l = m + p + 2i.
int build_st_tables(zest_gpu_context* ctx, SplitState* st, StPlan& plan, int S, StSplitTables** out) {
    auto key = std::make_tuple((const void*)&plan, S);
    auto it = st->st_tables.find(key);
    if (it != st->st_tables.end()) {
        *out = it->second.get();
        return ZEST_GPU_OK;
    }
    cudaStream_t s = ctx->stream;
    auto t = std::make_unique<StSplitTables>();
    t->S = S;
    LegTables& lg = plan.leg;
    const int L = lg.L, kh = lg.nnodes, kl = r16((L + 1) / 2);
    // 8-bit digits at any length: the sums are cut into K-chunks of at most 256
    ZG_TRY(slice_table(ctx, lg.Pf.as<double>(), lg.off_h[2 * (size_t)L], kh, kh, S, 8, t->leg_f, 1));
    std::vector<int> cnt(2 * (size_t)L);
    for (int m = 0; m < L; ++m)
        for (int p = 0; p < 2; ++p) cnt[2 * m + p] = (L - m - p > 0) ? (L - m - p + 1) / 2 : 0;
    DevBuf dcnt;
    ZG_TRY(upload(dcnt, cnt, s));
    ZG_TRY(st->tmp.ensure((size_t)2 * L * kh * kl * sizeof(double)));
    dim3 g1((kh * kl + 255) / 256, 2 * L);
    transpose_blocks_kernel<<<g1, 256, 0, s>>>(lg.Pb.as<double>(), lg.off.as<long long>(), dcnt.as<int>(), kh, kl,
                                               st->tmp.as<double>());
    ZG_TRY(launch_check("transpose_blocks_kernel"));
    ZG_TRY(slice_table(ctx, st->tmp.as<double>(), (long long)2 * L * kh, kl, kl, S, 8, t->leg_bT, 1));
    ZG_CUDA_TRY(cudaStreamSynchronize(s));
    st->tmp.release();  // several GB at high orders; rebuilt on demand
    *out = t.get();
    st->st_tables.emplace(key, std::move(t));
    return ZEST_GPU_OK;
}

}  // namespace

// ===========================================================================
// Split-precision Zernike transforms
// ===========================================================================
// End of a split-path call: check the bounded-wait flag, unless the stream is
// being captured into a graph (whose caller checks it after each replay).
int split_finish(zest_gpu_context* ctx) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    ZG_CUDA_TRY(cudaStreamIsCapturing(ctx->stream, &cap));
    if (cap != cudaStreamCaptureStatusNone) return ZEST_GPU_OK;
    return split_check_flag(ctx);
}

int split_available() {
    int dev = 0, major = 0, minor = 0;
    ZG_CUDA_TRY(cudaGetDevice(&dev));
    ZG_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    ZG_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10 || minor != 3) return fail(ZEST_GPU_ERR_UNSUPPORTED, "split path needs sm_103a");
    if (!encode_fn()) return fail(ZEST_GPU_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    return ZEST_GPU_OK;
}

int split_zt_forward(zest_gpu_context* ctx, ZtPlan& plan, int Lg, int Le, int Lm, int batch, const double* grids,
                     double* coeffs) {
    (void)Le;
    const int S = ctx->slices;
    cudaStream_t s = ctx->stream;
    SplitState* st;
    ZG_TRY(get_state(ctx, &st));
    if (Lg < 2 || Lg > SL_KMAX || plan.sh.nrad > SL_KMAX)
        return fail(ZEST_GPU_ERR_UNSUPPORTED, "split path: orders 2..2047");
    ZtSplitTables* tb;
    ZG_TRY(build_zt_tables(ctx, st, plan, S, &tb));
    const ZtShape& sh = plan.sh;
    const int C = int(sh.nlat * sh.nrad), N = int(sh.nlon), nt = int(sh.nlat), nr = int(sh.nrad), nr2 = 2 * nr;
    const int kh = plan.leg.nnodes;
    const long long csz = 2 * zsize(Le);
    // scratch: G (FP64 spectra) and flm
    ZG_TRY(ctx->s0.ensure((size_t)batch * Lg * C * 2 * sizeof(double)));
    ZG_TRY(ctx->s1.ensure((size_t)tri_size(Lm) * batch * nr2 * sizeof(double)));
    double* G = ctx->s0.as<double>();
    double* flm = ctx->s1.as<double>();

    // ---- longitude DFT: folded cos/sin products ----
    ZG_TRY(dft_forward_stage(ctx, st, *tb->dft, S, WK_DFT_F, grids, sh.size(), C, N, Lg, Lm, batch, G));
    // ---- Legendre (folded over the equator) ----
    {
        const int bits = digit_bits(kh);
        const long long per_m = (long long)batch * nr2;
        const long long rows = (long long)Lm * per_m;
        ZG_TRY(st->op[0].ensure(rows, r16(kh), S));
        ZG_TRY(st->op[1].ensure(rows, r16(kh), S));
        {
            StageScope sc(ctx, ST_SPLIT_SLICE);
            LegFwdLoader ld{G, batch, Lg, nt, nr2, plan.leg.j0u, plan.leg.j0d};
            ZG_TRY(launch_slice2(s, ld, rows, kh, kh, 0, S, bits, SL_FOLD, st->op[0], st->op[1]));
        }
        ZG_TRY(tuned_stage(ctx, st, WK_LEG_F, S, Lg, Lm, batch, (Lm + 1) / 2, nchunks(kh) == 1, [&](int NT) -> int {
        for (int ch = 0; ch < nchunks(kh); ++ch) {
            const int k0 = ch * KCHUNK;
            UnitList* u;
            ZG_TRY(get_units(ctx, std::make_tuple(int(WK_LEG_F), Lg, Lm, batch, S, 8 * ch + nt_pass(NT)), [&](UnitList& ul) {
                for (int m = 0; m < Lm; ++m)
                    for (int p = 0; p < 2; ++p) {
                        const int cnt = (Lm - m - p > 0) ? (Lm - m - p + 1) / 2 : 0;
                        add_units(ul, S, bits, (long long)m * per_m, per_m, int(plan.leg.off_h[2 * m + p]), cnt, NT,
                                  std::min(KCHUNK, kh - k0), p | (p << 2), m, k0);
                    }
            }, &u));
            if (ch == 0)
                ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], tb->leg_f, tb->leg_f, EpiLegFwd<false>{flm, batch, nr2}));
            else
                ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], tb->leg_f, tb->leg_f, EpiLegFwd<true>{flm, batch, nr2}));
        }
        return ZEST_GPU_OK;
        }));
    }
    // ---- radial ----
    {
        const int bits = digit_bits(nr);
        const long long rows = tri_size(Lm) * batch * 2;
        ZG_TRY(st->op[0].ensure(rows, r16(nr), S));
        {
            StageScope sc(ctx, ST_SPLIT_SLICE);
            ZG_TRY(launch_slice(s, RadFwdLoader{flm, nr, batch}, rows, nr, S, bits, st->op[0]));
        }
        ZG_TRY(tuned_stage(ctx, st, WK_RAD_F, S, Lg, Lm, batch, (Lm + 1) / 2, nchunks(nr) == 1, [&](int NT) -> int {
        for (int ch = 0; ch < nchunks(nr); ++ch) {
            const int k0 = ch * KCHUNK;
            UnitList* u;
            ZG_TRY(get_units(ctx, std::make_tuple(int(WK_RAD_F), Lg, Lm, batch, S, 8 * ch + nt_pass(NT)), [&](UnitList& ul) {
                for (int l = 0; l < Lm; ++l)
                    add_units(ul, S, bits, tri_idx(l, 0) * batch * 2, (long long)(l + 1) * batch * 2,
                              int(plan.rad.off_h[l]), (Lm - l + 1) / 2, NT, std::min(KCHUNK, nr - k0), 0, l, k0);
            }, &u));
            if (ch == 0)
                ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[0], tb->rad_f, tb->rad_f, EpiRadFwd<false>{coeffs, batch, csz}));
            else
                ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[0], tb->rad_f, tb->rad_f, EpiRadFwd<true>{coeffs, batch, csz}));
        }
        return ZEST_GPU_OK;
        }));
    }
    return split_finish(ctx);
}

int split_zt_backward(zest_gpu_context* ctx, ZtPlan& plan, int Le, int Lg, int Lm, int batch, const double* coeffs,
                      double* grids) {
    const int S = ctx->slices;
    cudaStream_t s = ctx->stream;
    SplitState* st;
    ZG_TRY(get_state(ctx, &st));
    if (Lg < 2 || Lg > SL_KMAX || plan.sh.nrad > SL_KMAX)
        return fail(ZEST_GPU_ERR_UNSUPPORTED, "split path: orders 2..2047");
    ZtSplitTables* tb;
    ZG_TRY(build_zt_tables(ctx, st, plan, S, &tb));
    const ZtShape& sh = plan.sh;
    const int C = int(sh.nlat * sh.nrad), N = int(sh.nlon), nr = int(sh.nrad), nr2 = 2 * nr;
    const int kh = plan.leg.nnodes;
    const int kl = r16((Lg + 1) / 2);
    const long long csz = 2 * zsize(Le);
    // the two parity sums E_p[b][m][folded node][kc] of the Legendre stage
    const long long eblock = (long long)Lg * kh * nr2;  // one (p, b)
    ZG_TRY(ctx->s0.ensure((size_t)2 * batch * eblock * sizeof(double)));
    ZG_TRY(ctx->s1.ensure((size_t)tri_size(Lm) * batch * nr2 * sizeof(double)));
    double* E = ctx->s0.as<double>();
    double* flm = ctx->s1.as<double>();

    // ---- radial: coefficients -> flm ----
    {
        const int bits = digit_bits((Lg + 1) / 2);
        const long long rows = tri_size(Lm) * batch * 2;
        ZG_TRY(st->op[0].ensure(rows, kl, S));
        {
            StageScope sc(ctx, ST_SPLIT_SLICE);
            ZG_TRY(launch_slice(s, RadBwdLoader{coeffs, csz, batch, Lm}, rows, (Lm + 1) / 2, S, bits,
                                st->op[0]));
        }
        ZG_TRY(tuned_stage(ctx, st, WK_RAD_B, S, Lg, Lm, batch, nr, nchunks((Lm + 1) / 2) == 1, [&](int NT) -> int {
        for (int ch = 0; ch < nchunks((Lm + 1) / 2); ++ch) {
            const int k0 = ch * KCHUNK;
            UnitList* u;
            ZG_TRY(get_units(ctx, std::make_tuple(int(WK_RAD_B), Lg, Lm, batch, S, 8 * ch + nt_pass(NT)), [&](UnitList& ul) {
                for (int l = 0; l < Lm; ++l)
                    add_units(ul, S, bits, tri_idx(l, 0) * batch * 2, (long long)(l + 1) * batch * 2, l * nr, nr, NT,
                              std::min(KCHUNK, (Lm - l + 1) / 2 - k0), 0, l, k0);
            }, &u));
            if (ch == 0)
                ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[0], tb->rad_bT, tb->rad_bT, EpiRadBwd<false>{flm, nr, batch}));
            else
                ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[0], tb->rad_bT, tb->rad_bT, EpiRadBwd<true>{flm, nr, batch}));
        }
        return ZEST_GPU_OK;
        }));
    }
    if (tb->leg_bU.rows > 0) {
        // ---- Legendre, orders up to 256: flm -> E[b][m][lat][kc] at every
        // latitude node, all l of one m in one sum (no fold over the equator) ----
        const int nlat = int(sh.nlat);
        const long long per_m = (long long)batch * nr2;
        const long long rows = (long long)Lm * per_m;
        ZG_TRY(st->op[0].ensure(rows, r16(Lm), S));
        {
            StageScope sc(ctx, ST_SPLIT_SLICE);
            ZG_TRY(launch_slice(s, LegBwdULoader{flm, batch, nr2, Lm}, rows, Lm, S, 8, st->op[0]));
        }
        if (Lm < Lg) {  // orders m >= Lm of the spectra are zero
            StageScope sc(ctx, ST_MEMSET);
            const long long eb = (long long)Lg * nlat * nr2;  // one b
            ZG_CUDA_TRY(cudaMemset2DAsync(E + (size_t)Lm * nlat * nr2, eb * sizeof(double), 0,
                                          (size_t)(Lg - Lm) * nlat * nr2 * sizeof(double), batch, s));
        }
        ZG_TRY(tuned_stage(ctx, st, WK_LEG_B, S, Lg, Lm, batch, nlat, true, [&](int NT) -> int {
            UnitList* u;
            ZG_TRY(get_units(ctx, std::make_tuple(int(WK_LEG_B), Lg, Lm, batch, S, 4 + nt_pass(NT)), [&](UnitList& ul) {
                for (int m = 0; m < Lm; ++m)
                    add_units(ul, S, 8, (long long)m * per_m, per_m, (long long)m * nlat, nlat, NT, Lm - m, 0, m, 0);
                // the algorithmic work is that of the sums folded over the equator
                // (half the products); the unfolded form spends the other half to
                // spare the inverse DFT's input a second array
                ul.useful *= 0.5;
            }, &u));
            return run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[0], tb->leg_bU, tb->leg_bU,
                               EpiLegBwdU<false>{E, batch, Lg, nlat, nr2});
        }));
        // ---- longitude: inverse real DFT of the spectra at every latitude ----
        // (the cos sums C_i go to the scratch of the spectra, consumed by the slicing)
        ZG_TRY(dft_backward_stage(ctx, st, *tb->dft, S, WK_DFT_B, DftBwdGridLoader{E, Lg, C, nr, nlat}, C, N, Lg,
                                  Lm, batch, grids, sh.size(), E));
        return split_finish(ctx);
    }
    // ---- Legendre: flm -> G (north/south unfold; parity 1 read-modify-write) ----
    {
        const int bits = digit_bits((Lg + 1) / 2);
        const long long per_m = (long long)batch * nr2;
        const long long rows = (long long)Lm * per_m;
        ZG_TRY(st->op[0].ensure(rows, kl, S));
        ZG_TRY(st->op[1].ensure(rows, kl, S));
        {
            StageScope sc(ctx, ST_SPLIT_SLICE);
            ZG_TRY(launch_slice2(s, LegBwdLoader{flm, batch, nr2, Lm}, rows, (Lm + 1) / 2, Lm / 2, 0, S, bits,
                                 SL_PAIR, st->op[0], st->op[1]));
        }
        ZG_TRY(zero_parity_tails(ctx, E, batch, Lg, Lm, kh, nr2));
        ZG_TRY(tuned_stage(ctx, st, WK_LEG_B, S, Lg, Lm, batch, kh, nchunks((Lm + 1) / 2) == 1, [&](int NT) -> int {
        for (int p = 0; p < 2; ++p)
            for (int ch = 0; ch < nchunks((Lm + 1) / 2); ++ch) {
            const int k0 = ch * KCHUNK;
            UnitList* u;
            ZG_TRY(get_units(ctx, std::make_tuple(int(WK_LEG_B), Lg, Lm, batch, S, p + 8 * ch + nt_pass(NT)), [&](UnitList& ul) {
                for (int m = 0; m < Lm; ++m) {
                    const int cnt = (Lm - m - p > 0) ? (Lm - m - p + 1) / 2 : 0;
                    if (cnt == 0) continue;
                    add_units(ul, S, bits, (long long)m * per_m, per_m, (2 * m + p) * kh, kh, NT,
                              std::min(KCHUNK, cnt - k0), p | (p << 2), m, k0);
                }
            }, &u));
            if (ch == 0)
                ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], tb->leg_bT, tb->leg_bT,
                                EpiLegBwdE<false>{E, batch, Lg, kh, nr2}));
            else
                ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], tb->leg_bT, tb->leg_bT,
                                EpiLegBwdE<true>{E, batch, Lg, kh, nr2}));
        }
        return ZEST_GPU_OK;
        }));
    }
    // ---- longitude: inverse real DFT, cos pass then sin read-modify-write pass ----
    // (the cos sums C_i go to the scratch of the parity sums, consumed by the slicing)
    ZG_TRY(dft_backward_stage(ctx, st, *tb->dft, S, WK_DFT_B,
                              DftBwdLoader{E, Lg, C, nr, kh, plan.leg.j0u, plan.leg.j0d, batch}, C, N,
                              Lg, Lm, batch, grids, sh.size(), E));
    return split_finish(ctx);
}

// ===========================================================================
// Split-precision SH Legendre sums.  The table is the 128-row operand: with
// 2 x batch data rows per order m the data could not fill a row tile.  The
// data (the folded spectra, or the coefficients) is the scaled-copy operand,
// sliced per call; its 2 x batch rows are the columns, in tiles of 16 (batches
// up to 8: a tile loads no unused data rows), 32 (up to 16) or 80.
// ===========================================================================
namespace {
template <class F>
int st_with_nt(int batch, F&& f) {
    if (2 * batch <= 16) return f(std::integral_constant<int, 16>{});
    return 2 * batch <= 32 ? f(std::integral_constant<int, 32>{}) : f(std::integral_constant<int, 80>{});
}
// SH sums always use 8-bit digits and 6 slices; sums longer than 256 run as
// K-chunks of at most 256 whose FP64 results are added (the later chunks
// through the read-modify-write epilogues).
constexpr int ST_KCHUNK = SL_K8MAX;
template <int NT, class Epi>
int run_gemm_st(zest_gpu_context* ctx, UnitList& ul, const SliceArray& A, const SliceArray& B0, const SliceArray& B1,
                const Epi& epi) {
    if (A.bits != 8 || B0.bits != 8 || B1.bits != 8)
        return fail(ZEST_GPU_ERR_INVALID, "split SH sums: operands must have 8-bit digits");
    return run_gemm_t<6, 8, NT>(ctx, ul, A, A, B0, B1, epi);
}
}  // namespace

int split_st_forward(zest_gpu_context* ctx, StPlan& plan, int Lg, int Lm, int batch, const double* grids, double* X,
                     double* coeffs, long long csz) {
    const int S = ctx->slices;
    if (S != 6) return fail(ZEST_GPU_ERR_UNSUPPORTED, "split SH transforms need 6 slices");
    cudaStream_t s = ctx->stream;
    SplitState* st;
    ZG_TRY(get_state(ctx, &st));
    const int kh = plan.leg.nnodes, nlat = int(plan.sh.nlat);
    if (Lg > SL_KMAX || kh > SL_KMAX) return fail(ZEST_GPU_ERR_UNSUPPORTED, "split SH path: orders up to 2048");
    StSplitTables* tb;
    ZG_TRY(build_st_tables(ctx, st, plan, S, &tb));
    if (split_st_tensor_dft(plan.sh.latlon, Lg)) {
        // LonLat grids [lon][lat]: the longitude DFT on the tensor cores, to X[b][m][lat][re, im]
        const DftTables* dt;
        ZG_TRY(build_dft_tables(ctx, st, Lg, int(plan.sh.nlon), S, &dt));
        ZG_TRY(dft_forward_stage(ctx, st, *dt, S, WK_ST_DFT_F, grids, plan.sh.size(), nlat, int(plan.sh.nlon), Lg, Lm,
                                 batch, X));
    }
    const int bits = 8;
    const long long per_m = 2LL * batch, rows = (long long)Lm * per_m;
    ZG_TRY(st->op[0].ensure(rows, r16(kh), S));
    ZG_TRY(st->op[1].ensure(rows, r16(kh), S));
    {
        StageScope sc(ctx, ST_SPLIT_SLICE);
        LegFwdLoader ld{X, batch, Lg, nlat, 2, plan.leg.j0u, plan.leg.j0d};
        ZG_TRY(launch_slice2(s, ld, rows, kh, kh, 0, S, bits, SL_FOLD, st->op[0], st->op[1]));
    }
    const int nchunk = (kh + ST_KCHUNK - 1) / ST_KCHUNK;
    for (int ch = 0; ch < nchunk; ++ch) {
        const int k0 = ch * ST_KCHUNK, kk = std::min(ST_KCHUNK, kh - k0);
        ZG_TRY(st_with_nt(batch, [&](auto nt) -> int {
            constexpr int NT = decltype(nt)::value;
            UnitList* u;
            ZG_TRY(get_units(ctx, std::make_tuple(int(WK_ST_LEG_F), Lg, Lm, batch, S, int(plan.sh.latlon) + 2 * ch),
                             [&](UnitList& ul) {
                                 for (int m = 0; m < Lm; ++m)
                                     for (int p = 0; p < 2; ++p) {
                                         const int cnt = (Lm - m - p > 0) ? (Lm - m - p + 1) / 2 : 0;
                                         add_units(ul, S, bits, plan.leg.off_h[2 * m + p], cnt, int(m * per_m),
                                                   int(per_m), NT, kk, (p << 1) | (p << 2), m, k0);
                                     }
                             },
                             &u));
            if (ch == 0)
                return run_gemm_st<NT>(ctx, *u, tb->leg_f, st->op[0], st->op[1],
                                       EpiStLegFwd<false>{coeffs, csz, plan.leg.L});
            return run_gemm_st<NT>(ctx, *u, tb->leg_f, st->op[0], st->op[1],
                                   EpiStLegFwd<true>{coeffs, csz, plan.leg.L});
        }));
    }
    return split_finish(ctx);
}

int split_st_backward(zest_gpu_context* ctx, StPlan& plan, int Lg, int Lm, int batch, const double* coeffs,
                      long long csz, double* X, double* grids) {
    const int S = ctx->slices;
    if (S != 6) return fail(ZEST_GPU_ERR_UNSUPPORTED, "split SH transforms need 6 slices");
    cudaStream_t s = ctx->stream;
    SplitState* st;
    ZG_TRY(get_state(ctx, &st));
    const int kh = plan.leg.nnodes, nlat = int(plan.sh.nlat), kl = r16((Lg + 1) / 2);
    if (Lg > SL_KMAX || kh > SL_KMAX) return fail(ZEST_GPU_ERR_UNSUPPORTED, "split SH path: orders up to 2048");
    const bool lonlat = split_st_tensor_dft(plan.sh.latlon, Lg);
    StSplitTables* tb;
    ZG_TRY(build_st_tables(ctx, st, plan, S, &tb));
    const int bits = 8;
    const long long per_m = 2LL * batch, rows = (long long)Lm * per_m;
    ZG_TRY(st->op[0].ensure(rows, kl, S));
    ZG_TRY(st->op[1].ensure(rows, kl, S));
    {
        StageScope sc(ctx, ST_SPLIT_SLICE);
        ZG_TRY(launch_slice2(s, StLegBwdLoader{coeffs, csz, batch, Lm}, rows, (Lm + 1) / 2, Lm / 2, 0, S, bits,
                             SL_PAIR, st->op[0], st->op[1]));
    }
    // parity sums E[p][b][m][j][c]; groups with no degree below Lm are not
    // written and the unfolding reads them as 0
    ZG_TRY(ctx->s1.ensure((size_t)2 * batch * Lg * kh * 2 * sizeof(double)));
    double* E = ctx->s1.as<double>();
    const int nchunk = ((Lm + 1) / 2 + ST_KCHUNK - 1) / ST_KCHUNK;
    for (int ch = 0; ch < nchunk; ++ch) {
        const int k0 = ch * ST_KCHUNK;
        ZG_TRY(st_with_nt(batch, [&](auto nt) -> int {
            constexpr int NT = decltype(nt)::value;
            UnitList* u;
            ZG_TRY(get_units(ctx, std::make_tuple(int(WK_ST_LEG_B), Lg, Lm, batch, S, int(plan.sh.latlon) + 2 * ch),
                             [&](UnitList& ul) {
                                 for (int m = 0; m < Lm; ++m)
                                     for (int p = 0; p < 2; ++p) {
                                         const int cnt = (Lm - m - p > 0) ? (Lm - m - p + 1) / 2 : 0;
                                         // the degrees of this chunk: i in [k0, min(cnt, k0 + 256))
                                         const int kk = std::min(cnt - k0, ST_KCHUNK);
                                         add_units(ul, S, bits, (long long)(2 * m + p) * kh, kh, int(m * per_m),
                                                   int(per_m), NT, kk, (p << 1) | (p << 2), m, k0);
                                     }
                             },
                             &u));
            // conjugated for the inverse DFT of a LonLat grid; the unfolding conjugates
            const unsigned long long sgi = lonlat ? (1ull << 63) : 0ull;
            if (ch == 0)
                return run_gemm_st<NT>(ctx, *u, tb->leg_bT, st->op[0], st->op[1],
                                       EpiStLegBwdE<false>{E, batch, Lg, kh, sgi});
            return run_gemm_st<NT>(ctx, *u, tb->leg_bT, st->op[0], st->op[1],
                                   EpiStLegBwdE<true>{E, batch, Lg, kh, sgi});
        }));
    }
    if (lonlat) {
        // LonLat grids [lon][lat]: the inverse longitude DFT on the tensor cores,
        // straight from the parity sums; X holds the cos sums
        ZG_TRY(zero_parity_tails(ctx, E, batch, Lg, Lm, kh, 2));
        const DftTables* dt;
        ZG_TRY(build_dft_tables(ctx, st, Lg, int(plan.sh.nlon), S, &dt));
        ZG_TRY(dft_backward_stage(ctx, st, *dt, S, WK_ST_DFT_B,
                                  DftBwdLoader{E, Lg, nlat, 1, kh, plan.leg.j0u, plan.leg.j0d, batch}, nlat,
                                  int(plan.sh.nlon), Lg, Lm, batch, grids, plan.sh.size(), X));
        return split_finish(ctx);
    }
    {
        StageScope sc(ctx, ST_SPLIT_SLICE);
        const long long n = (long long)batch * Lg * kh * 2;
        st_unfold_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(E, X, batch, Lg, Lm, kh, nlat, plan.leg.j0u,
                                                                  plan.leg.j0d);
        ZG_TRY(launch_check("st_unfold_kernel"));
    }
    return split_finish(ctx);
}

// ===========================================================================
// Split-precision rotation of ragged Zernike batches (Rotor::rotate,
// rotor.hpp:210-243; rotate_l, wignerd_collection.hpp:122-296).  Every rotated
// (n, l) vector of every item is one operand row, the rows sorted by l.  The
// two X(+-pi/2) products of rotate_l are, per l, real matrices applied to the
// real and the imaginary parts apart (the parity structure of d^l(pi/2) and
// of a real function's complex coefficients):
//   Re t_m = sum_m' Re1[m][m'] Re v_m',   Im t_m = sum_m' Im1[m][m'] Im v_m'
// with Re1[m][0] = D(m, 0), Re1[m][m'] = 2 D(m, m') for m' >= 1 of the
// parity of l + m, Im1[m][m'] = 2 D(m, m') for m' >= 1 of the other parity;
// D(m, m') = (-1)^{m+m'} d(m', m) for X(pi/2) and d(m', m) for X(-pi/2)
// (d(m', m) at wig[wig_off(l) + (l+1) m' + m]).  So each product is a split
// GEMM per l-group with the table as the scaled-copy operand.  The phases and
// the real/complex conversions are applied where the operands are sliced
// (gamma', beta') and by a last elementwise pass (alpha').
// ===========================================================================
namespace {

__global__ void rot_table_kernel(const double* __restrict__ wig, int Kp, int which, double* __restrict__ out) {
    const long long t = blockIdx.y;  // tri(l) + m
    int l = int((sqrtf(8.0f * float(t) + 1.0f) - 1.0f) * 0.5f);
    while ((long long)(l + 1) * (l + 2) / 2 <= t) ++l;
    while ((long long)l * (l + 1) / 2 > t) --l;
    const int m = int(t - (long long)l * (l + 1) / 2);
    const int mp = blockIdx.x * blockDim.x + threadIdx.x;
    if (mp >= Kp) return;
    double v = 0.0;
    if (mp <= l) {
        const double x = wig[wig_off(l) + (long long)(l + 1) * mp + m];
        const double D = (which < 2 && ((m + mp) & 1)) ? -x : x;
        const int q = (l + m) & 1;
        if ((which & 1) == 0) v = mp == 0 ? D : (((mp & 1) == q) ? 2.0 * D : 0.0);
        else v = (mp >= 1 && (mp & 1) != q) ? 2.0 * D : 0.0;
    }
    out[t * Kp + mp] = v;
}

int build_rot_tables(zest_gpu_context* ctx, SplitState* st, const double* wig, int Lmax, int S, const RotTables** out) {
    auto key = std::make_tuple(Lmax, S);
    auto it = st->rot_tables.find(key);
    if (it != st->rot_tables.end()) {
        *out = it->second.get();
        return ZEST_GPU_OK;
    }
    auto t = std::make_unique<RotTables>();
    const int Kp = r16(Lmax);
    const long long rows = tri_size(Lmax);
    ZG_TRY(st->tmp.ensure((size_t)rows * Kp * sizeof(double)));
    SliceArray* dst[4] = {&t->re1, &t->im1, &t->re2, &t->im2};
    for (int w = 0; w < 4; ++w) {
        rot_table_kernel<<<dim3((Kp + 127) / 128, (unsigned)rows), 128, 0, ctx->stream>>>(wig, Kp, w,
                                                                                          st->tmp.as<double>());
        ZG_TRY(launch_check("rot_table_kernel"));
        ZG_TRY(slice_table(ctx, st->tmp.as<double>(), rows, Lmax, Kp, S, 8, *dst[w]));
    }
    ZG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *out = t.get();
    st->rot_tables.emplace(key, std::move(t));
    return ZEST_GPU_OK;
}

// row v = vecs[v] = {item, n, l, base}: k = m: r2c(c_m) e^{-i m gamma'} (Re, Im)
struct RotInLoader {
    static constexpr bool ROW_FAST = false, TWO = true;
    static constexpr int MODE = SL_PAIR, SHIFT = 0;
    const int4* vecs;
    const long long* coff;
    const double* coeffs;
    const double2* ph;
    int Lmax;
    struct Row { const double* c; const double2* pg; int l; };
    __device__ Row row(long long r) const {
        const int4 w = vecs[r];
        return Row{coeffs + coff[w.x] + 2 * (long long)w.w, ph + ((long long)w.x * 3 + 2) * Lmax, w.z};
    }
    __device__ void get(const Row& R, int k, double& up, double& dn) const {
        if (k > R.l) {
            up = dn = 0.0;
            return;
        }
        const double isq2 = 1.0 / 1.41421356237309504880168872420969808;
        double xr = R.c[2 * k], xi = R.c[2 * k + 1];
        if (k > 0) {
            xr *= isq2;
            xi *= -isq2;
        }
        const double2 p = R.pg[k];
        up = xr * p.x - xi * p.y;
        dn = xr * p.y + xi * p.x;
    }
    __device__ int kvalid(const Row& R) const { return R.l + 1; }  // m <= l
};

// row v: k = m: t_m e^{-i m beta'} (Re, Im), t = T[v][m][re, im]
struct RotMidLoader {
    static constexpr bool ROW_FAST = false, TWO = true;
    static constexpr int MODE = SL_PAIR, SHIFT = 0;
    const int4* vecs;
    const double* T;
    const double2* ph;
    int Lmax;
    struct Row { const double* t; const double2* pb; int l; };
    __device__ Row row(long long r) const {
        const int4 w = vecs[r];
        return Row{T + r * 2LL * Lmax, ph + ((long long)w.x * 3 + 1) * Lmax, w.z};
    }
    __device__ void get(const Row& R, int k, double& up, double& dn) const {
        if (k > R.l) {
            up = dn = 0.0;
            return;
        }
        const double tr = R.t[2 * k], ti = R.t[2 * k + 1];
        const double2 p = R.pb[k];
        up = tr * p.x - ti * p.y;
        dn = tr * p.y + ti * p.x;
    }
    __device__ int kvalid(const Row& R) const { return R.l + 1; }  // m <= l
};

// rows v, columns m = aux + n: T[v][m][part], part = 0 (real) for the units
// of the first operand pair, 1 (imaginary) for the second
struct EpiRot {
    static constexpr bool RMW = false;
    static constexpr bool CHUNK = false;
    double* T;
    int Lmax;
    struct Row { double* p; };
    __device__ Row row(const SplitUnit& u, int r) const {
        return Row{T + ((long long)r * Lmax + u.aux) * 2 + (u.flags & 1)};
    }
    __device__ void load(const Row&, int, double*) const {}
    __device__ void store(const Row& R, const SplitUnit&, int n, double v, const double*) const { R.p[2 * n] = v; }
};

// coefficients of vector v, m <= l: c2r(u_m e^{-i m alpha'}), u = U[v][m]
__global__ void rot_out_kernel(long long nvec, const int4* __restrict__ vecs, const long long* __restrict__ coff,
                               double* __restrict__ coeffs, const double* __restrict__ U, int Lmax,
                               const double2* __restrict__ ph) {
    const long long v = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (v >= nvec) return;
    const int lane = threadIdx.x & 31;
    const int4 w = vecs[v];
    double* c = coeffs + coff[w.x] + 2 * (long long)w.w;
    const double2* pa = ph + ((long long)w.x * 3 + 0) * Lmax;
    const double* u = U + v * 2LL * Lmax;
    const double sq2 = 1.41421356237309504880168872420969808;
    for (int m = lane; m <= w.z; m += 32) {
        const double2 p = pa[m];
        double xr = u[2 * m] * p.x - u[2 * m + 1] * p.y;
        double xi = u[2 * m] * p.y + u[2 * m + 1] * p.x;
        if (m > 0) {
            xr *= sq2;
            xi *= -sq2;
        }
        c[2 * m] = xr;
        c[2 * m + 1] = xi;
    }
}

}  // namespace

int split_rotate_ragged(zest_gpu_context* ctx, int Lmax, int items, long long nvec, const int4* vecs,
                        const std::vector<long long>& voff, const long long* coff, double* coeffs, const double* wig,
                        const double* euler, int type, double* phase) {
    if (nvec <= 0) return ZEST_GPU_OK;
    if (Lmax > SL_K8MAX) return fail(ZEST_GPU_ERR_UNSUPPORTED, "split rotation: orders up to 256");
    const int S = ctx->slices;
    cudaStream_t s = ctx->stream;
    SplitState* st;
    ZG_TRY(get_state(ctx, &st));
    const RotTables* tb;
    ZG_TRY(build_rot_tables(ctx, st, wig, Lmax, S, &tb));
    ZG_TRY(launch_phases(s, Lmax, items, euler, type, phase));
    const double2* ph = reinterpret_cast<const double2*>(phase);
    const int Kp = r16(Lmax);
    ZG_TRY(ctx->s0.ensure((size_t)nvec * 2 * Lmax * sizeof(double)));
    double* T = ctx->s0.as<double>();
    ZG_TRY(st->op[0].ensure(nvec, Kp, S));
    ZG_TRY(st->op[1].ensure(nvec, Kp, S));
    // one work list for both products: per l, the rows of its vectors against
    // its l + 1 table rows, real parts (operands 0) and imaginary parts (1)
    // the list's key: two independent hashes of the row offsets (FNV-1a and
    // a weighted sum), with the order, the vector count and the tile
    unsigned h1 = 2166136261u;
    unsigned long long h2 = 0;
    for (size_t l = 0; l < voff.size(); ++l) {
        h1 = (h1 ^ unsigned(voff[l])) * 16777619u;
        h2 = h2 * 1000003ull + (unsigned long long)voff[l] * (2 * l + 1);
    }
    const int NT = stage_nt(st, WK_ROT, S, Lmax);
    auto fill = [&](UnitList& ul) {
        for (int l = 0; l < Lmax; ++l) {
            const long long cnt = voff[l + 1] - voff[l];
            add_units(ul, S, 8, voff[l], cnt, int(tri_size(l)), l + 1, NT, l + 1, 0, l);
            add_units(ul, S, 8, voff[l], cnt, int(tri_size(l)), l + 1, NT, l + 1, 1 | 2, l);
        }
        ul.rows = voff;
    };
    UnitList* u;
    ZG_TRY(get_units(ctx, std::make_tuple(int(WK_ROT), Lmax + nt_pass(NT), int(nvec), int(h1 & 0x7fffffff), S,
                                          int((h2 ^ (h2 >> 31)) & 0x7fffffff)),
                     fill, &u));
    if (u->rows != voff) {
        // two batches whose row offsets share both hashes: the cached list
        // belongs to the other one, so it is rebuilt for this batch
        ZG_CUDA_TRY(cudaStreamSynchronize(s));  // the old list may still be read by a queued launch
        u->v.clear();
        u->max_ksteps = 0;
        u->useful = u->issued = 0.0;
        u->dev.release();
        fill(*u);
    }
    {
        StageScope sc(ctx, ST_SPLIT_SLICE);
        ZG_TRY(launch_slice2(s, RotInLoader{vecs, coff, coeffs, ph, Lmax}, nvec, Lmax, Lmax, 0, S, 8, SL_PAIR,
                             st->op[0], st->op[1]));
    }
    ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], tb->re1, tb->im1, EpiRot{T, Lmax}));
    {
        StageScope sc(ctx, ST_SPLIT_SLICE);
        ZG_TRY(launch_slice2(s, RotMidLoader{vecs, T, ph, Lmax}, nvec, Lmax, Lmax, 0, S, 8, SL_PAIR, st->op[0],
                             st->op[1]));
    }
    ZG_TRY(run_gemm_nt(ctx, NT, S, *u, st->op[0], st->op[1], tb->re2, tb->im2, EpiRot{T, Lmax}));
    {
        StageScope sc(ctx, ST_ROTATE);
        const int W = 8;
        rot_out_kernel<<<(unsigned)((nvec + W - 1) / W), W * 32, 0, s>>>(nvec, vecs, coff, coeffs, T, Lmax, ph);
        ZG_TRY(launch_check("rot_out_kernel"));
    }
    return ZEST_GPU_OK;
}

// Dense FP64 product C = A B^T through the split path (A: M x K, B: N x K,
// row-major, device pointers); used to test the emulation itself.
int split_dense_gemm(zest_gpu_context* ctx, int M, int N, int K, const double* A, const double* B, double* C) {
    const int S = ctx->slices;
    const int NT = n_tile(S);
    if (K > SL_KMAX) return fail(ZEST_GPU_ERR_UNSUPPORTED, "split GEMM: K above 2048");
    SplitState* st;
    ZG_TRY(get_state(ctx, &st));
    SliceArray a, b;
    ZG_TRY(a.ensure(M, r16(K), S));
    ZG_TRY(b.ensure(N, r16(K), S));
    const int bits = digit_bits(K);
    ZG_TRY(launch_slice(ctx->stream, RowMajorLoader{A, K}, M, K, S, bits, a));
    ZG_TRY(launch_slice(ctx->stream, RowMajorLoader{B, K}, N, K, S, bits, b));
    for (int ch = 0; ch < nchunks(K); ++ch) {
        const int k0 = ch * KCHUNK;
        UnitList u;
        add_units(u, S, bits, 0, M, 0, N, NT, std::min(KCHUNK, K - k0), 0, 0, k0);
        if (ch == 0) ZG_TRY(run_gemm_nt(ctx, NT, S, u, a, a, b, b, EpiDense<false>{C, N}));
        else ZG_TRY(run_gemm_nt(ctx, NT, S, u, a, a, b, b, EpiDense<true>{C, N}));
        ZG_TRY(split_finish(ctx));  // the local work list must outlive its launch
    }
    return ZEST_GPU_OK;  // the local operands outlive the launches (split_finish synchronizes)
}

int split_wait_selftest(zest_gpu_context* ctx, long long limit_ns) {
    SplitState* st;
    ZG_TRY(get_state(ctx, &st));
    wait_expiry_kernel<<<1, 64, 0, ctx->stream>>>(st->err.as<int>(), st->host_err_dev, limit_ns);
    ZG_TRY(launch_check("wait_expiry_kernel"));
    return split_finish(ctx);
}

void split_flops(zest_gpu_context* ctx, bool reset, double* useful, double* issued) {
    SplitState* st = ctx->split.get();
    if (useful) *useful = st ? st->useful_flops : 0.0;
    if (issued) *issued = st ? st->issued_flops : 0.0;
    if (reset && st) st->useful_flops = st->issued_flops = 0.0;
}

}  // namespace zgpu
