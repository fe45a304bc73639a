// Rotation of real Zernike expansions that allocates no device memory.
//
// zest_gpu_zt_rotate_noalloc runs the kernels of zest_gpu_zt_rotate
// (Rotor::rotate, include/rotor.hpp:214-243) on caller-owned device buffers.
// The two scratch buffers that path keeps in the context -- the list of
// rotated (n, l) vectors and the per-item phase tables e^{-i m angle} -- live
// here in one fixed array compiled into the library's device image, so a call
// makes no cudaMalloc, cudaFree or other allocating call.  The Wigner d(pi/2)
// table is the caller's (zest_gpu_wignerd_table fills one).
//
// Layout of the array for a call of order L and batch B:
//   [0, vec_bytes)            int2 vectors {n, l}, grouped by l, n ascending
//                             (the order of the context path), vec_bytes =
//                             8 * nvec(L) rounded up to 256
//   [vec_bytes, + 48 L B)     phases, 3 tables of L double2 per batch item
// Every byte a call reads is written earlier in the same call, so nothing in
// the array has to start at zero.
#include <cuda.h>

#include <mutex>
#include <string>

#include "common.cuh"
#include "kernels.cuh"

#define ZEST_GPU_NOALLOC_MAX_DEVICES 64

namespace {

static __device__ __align__(256) unsigned char zt_rotate_scratch[ZEST_GPU_NOALLOC_SCRATCH_BYTES];

// The array's device address, cached per device together with the id of the
// CUDA context it was looked up in.  A context that is destroyed and created
// anew (cudaDeviceReset, or the primary context released and retained again)
// gets a new id, and the address is looked up again in it: an address from an
// earlier context is never passed to a kernel.
struct ScratchSlot {
    unsigned long long ctx_id = 0;
    void* addr = nullptr;
};
std::mutex g_scratch_mu;
ScratchSlot g_scratch[ZEST_GPU_NOALLOC_MAX_DEVICES];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// cuCtxGetCurrent and cuCtxGetId through the runtime's driver entry points
// (the library links only the CUDA runtime); resolved once per process.
bool context_fns(CtxGetCurrentFn* get_current, CtxGetIdFn* get_id) {
    static CtxGetCurrentFn cur = nullptr;
    static CtxGetIdFn id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            cur = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            id = reinterpret_cast<CtxGetIdFn>(p);
        cudaGetLastError();
    });
    *get_current = cur;
    *get_id = id;
    return cur && id;
}

// rotated vectors of order L with the given l: n = n0, n0 + 2, .. < L
__host__ __device__ inline long long vec_count(int L, int l) {
    const int n0 = l == 0 ? 2 : l;
    return n0 < L ? (L - 1 - n0) / 2 + 1 : 0;
}

long long vec_total(int L) {
    long long t = 0;
    for (int l = 0; l < L; ++l) t += vec_count(L, l);
    return t;
}

// one thread per l writes its run of vectors at the run's offset
__global__ void zt_vector_list_kernel(int L, int2* __restrict__ out) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= L) return;
    long long off = 0;
    for (int lp = 0; lp < l; ++lp) off += vec_count(L, lp);
    const int n0 = l == 0 ? 2 : l;
    const long long c = vec_count(L, l);
    for (long long i = 0; i < c; ++i) out[off + i] = make_int2(n0 + 2 * int(i), l);
}

// Address of the array in the current device's current context.  The first
// call per device (and the first after that device's context was replaced)
// looks it up with cudaGetSymbolAddress, which also loads the library's
// kernels into the context; later calls only compare the context id.
int scratch_of_current_device(unsigned char** out) {
    int dev = -1;
    ZG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= ZEST_GPU_NOALLOC_MAX_DEVICES)
        return zgpu::fail(ZEST_GPU_ERR_UNSUPPORTED, "zt_rotate_noalloc: device index above 63");
    CtxGetCurrentFn get_current = nullptr;
    CtxGetIdFn get_id = nullptr;
    if (!context_fns(&get_current, &get_id))
        return zgpu::fail(ZEST_GPU_ERR_CUDA, "zt_rotate_noalloc: cuCtxGetCurrent/cuCtxGetId are unavailable");
    auto lookup = [](void** p) -> int {
        const cudaError_t e = cudaGetSymbolAddress(p, zt_rotate_scratch);
        if (e != cudaSuccess || !*p)
            return zgpu::fail(ZEST_GPU_ERR_CUDA, std::string("zt_rotate_noalloc: cudaGetSymbolAddress of the scratch "
                                                             "array failed: ") + cudaGetErrorString(e));
        return ZEST_GPU_OK;
    };
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    CUcontext cu_ctx = nullptr;
    void* fresh = nullptr;
    if (get_current(&cu_ctx) != CUDA_SUCCESS) cu_ctx = nullptr;
    if (!cu_ctx) {  // no context yet on this thread: the lookup creates the device's primary context
        ZG_TRY(lookup(&fresh));
        if (get_current(&cu_ctx) != CUDA_SUCCESS) cu_ctx = nullptr;
    }
    unsigned long long ctx_id = 0;
    if (!cu_ctx || get_id(cu_ctx, &ctx_id) != CUDA_SUCCESS)
        return zgpu::fail(ZEST_GPU_ERR_CUDA, "zt_rotate_noalloc: no current CUDA context on the device");
    ScratchSlot& slot = g_scratch[dev];
    if (!slot.addr || slot.ctx_id != ctx_id) {
        if (!fresh) ZG_TRY(lookup(&fresh));
        slot.addr = fresh;
        slot.ctx_id = ctx_id;
    }
    *out = static_cast<unsigned char*>(slot.addr);
    return ZEST_GPU_OK;
}

}  // namespace

extern "C" int zest_gpu_zt_rotate_noalloc(void* stream, size_t order, size_t batch, double* coeffs,
                                          const double* euler, int rotation_type, const double* wignerd,
                                          size_t wignerd_order) {
    using namespace zgpu;
    if (rotation_type != 0 && rotation_type != 1) return fail(ZEST_GPU_ERR_INVALID, "invalid rotation type");
    if (order > 2048) return fail(ZEST_GPU_ERR_INVALID, "rotation order too large");
    if (batch > 65535) return fail(ZEST_GPU_ERR_INVALID, "batch too large (max 65535)");
    const int L = int(order), B = int(batch);
    const long long nvec = vec_total(L);
    const size_t vec_bytes = ((size_t)nvec * sizeof(int2) + 255) & ~size_t(255);
    const size_t need = vec_bytes + (size_t)6 * L * B * sizeof(double);
    if (need > ZEST_GPU_NOALLOC_SCRATCH_BYTES)
        return fail(ZEST_GPU_ERR_UNSUPPORTED,
                    "zt_rotate_noalloc: order " + std::to_string(order) + " and batch " + std::to_string(batch) +
                        " need " + std::to_string(need) + " bytes of scratch, above the fixed " +
                        std::to_string((size_t)ZEST_GPU_NOALLOC_SCRATCH_BYTES));
    if (batch && order && (!coeffs || !euler)) return fail(ZEST_GPU_ERR_INVALID, "null data pointer");
    unsigned char* scratch = nullptr;
    ZG_TRY(scratch_of_current_device(&scratch));  // set-up on the first call per device
    if (nvec == 0 || batch == 0) return ZEST_GPU_OK;
    if (!wignerd) return fail(ZEST_GPU_ERR_INVALID, "null Wigner d table");
    if (wignerd_order < order)
        return fail(ZEST_GPU_ERR_INVALID, "Wigner d table of order " + std::to_string(wignerd_order) +
                                              " is smaller than the expansion order " + std::to_string(order));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int2* vecs = reinterpret_cast<int2*>(scratch);
    double* phases = reinterpret_cast<double*>(scratch + vec_bytes);
    zt_vector_list_kernel<<<(L + 127) / 128, 128, 0, s>>>(L, vecs);
    ZG_TRY(launch_check("zt_vector_list_kernel"));
    return launch_rotate_vectors(s, 0, L, B, coeffs, 2 * zsize(L), vecs, int(nvec), wignerd, euler, rotation_type,
                                 phases);
}
