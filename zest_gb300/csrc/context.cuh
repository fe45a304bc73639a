// Context and per-order plan structures of the GLQ path, shared by the FP64
// host code (zest_gpu.cu) and the split-precision host code (split.cu).
#pragma once

#include <atomic>

#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "split.cuh"
#include "lsq.cuh"

namespace zgpu {

// ---------------------------------------------------------------------------
// Number of device buffers freed so far (process-wide).  A captured CUDA
// graph holds raw device pointers: it may be replayed only while this count is
// what it was at capture, i.e. while no buffer it might use has been freed or
// moved by a reallocation.
inline std::atomic<unsigned long long>& alloc_epoch() {
    static std::atomic<unsigned long long> epoch{0};
    return epoch;
}

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) {
            cudaFree(p);
            alloc_epoch().fetch_add(1, std::memory_order_relaxed);
        }
        p = nullptr;
        bytes = 0;
    }
    int ensure(size_t n) {
        if (n <= bytes && p) return ZEST_GPU_OK;
        release();
        if (n == 0) n = 16;
        if (cudaMalloc(&p, n) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return fail(ZEST_GPU_ERR_OOM, "device allocation of " + std::to_string(n) + " bytes failed");
        }
        bytes = n;
        return ZEST_GPU_OK;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

template <class T>
inline int upload(DevBuf& buf, const std::vector<T>& v, cudaStream_t s) {
    ZG_TRY(buf.ensure(v.size() * sizeof(T)));
    if (!v.empty()) ZG_CUDA_TRY(cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    ZG_CUDA_TRY(cudaStreamSynchronize(s));  // host vector may die after return
    return ZEST_GPU_OK;
}

// Device buffers of the evaluation at arbitrary points (evaluate.cu).
struct EvalBufs {
    DevBuf z, r, cs, trig;            // points: cos(colat), radii, (cos, sin)(lon), trig table
    DevBuf P, offP, cntP;             // Legendre table at the colatitudes, groups (m, parity)
    DevBuf R, offR, cntR;             // radial table at the radii, groups l
    DevBuf flm, G;                    // radial and Legendre sums
    DevBuf tiles[3];                  // tile lists of the three sums
};

struct FftEntry {
    FftPlan plan;
    DevBuf tw;
};

// Folded Legendre tables (forward: weights * quadrature prefactor folded in;
// backward: 1/2 for m > 0) with their group offsets.
struct LegTables {
    int L = 0, nnodes = 0;  // nnodes = folded node count (ld)
    int j0u = 0, j0d = 0;
    DevBuf Pf, Pb, off;
    std::vector<long long> off_h;
    std::map<int, std::unique_ptr<DevBuf>> cnt;  // per truncation order Lm
};

struct RadTables {
    int L = 0, nr = 0;
    DevBuf Rf, Rb, off;
    std::vector<long long> off_h;
    std::map<int, std::unique_ptr<DevBuf>> cnt;
};

struct ZtPlan {
    ZtShape sh{};
    LegTables leg;
    RadTables rad;
    std::vector<double> lat_nodes, lat_w, rad_nodes, rad_w;  // host copies (r = (1+x)/2)
};

struct StPlan {
    StShape sh{};
    LegTables leg;
};

// A batch of expansions of different orders (rotate, then backward
// transform), its device work lists and the CUDA graph that replays it.
struct RaggedPlan {
    std::vector<int> orders;
    const void* coeffs = nullptr;
    const void* euler = nullptr;
    const void* grids = nullptr;
    int zn = 0, sn = 0, sp = 0, type = 0, precision = 0, slices = 0;
    int Lmax = 0;
    long long nwork = 0;
    DevBuf coff, work;                                         // per-item coefficient offsets, {item, n, l}
    DevBuf vecl;                                               // the {item, n, l} vectors sorted by l
    std::vector<long long> voff;                               // vecl rows of order l: [voff[l], voff[l+1])
    std::vector<long long> coff_h, goff_h;
    std::vector<std::tuple<int, int, int>> buckets;            // {order, first item, count}
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long epoch = 0;  // alloc_epoch() when the graph was recorded
    ~RaggedPlan() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

// The rotated vectors of a batch of expansions of one order, sorted by l
// ({item, n, l, first coefficient}), and each item's coefficient offset.
struct UniformRotation {
    DevBuf vecs, coff;
    std::vector<long long> voff;
    long long nvec = 0;
};

struct TileEntry {
    DevBuf buf;
    int count = 0;
};

// CUDA-event timing of pipeline stages on the context stream.
struct Profiler {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    std::vector<std::tuple<int, cudaEvent_t, cudaEvent_t>> pending;
    double ms[ST_COUNT] = {};
    long long count[ST_COUNT] = {};
    cudaEvent_t get() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    ~Profiler() {
        for (auto& t : pending) {
            cudaEventDestroy(std::get<1>(t));
            cudaEventDestroy(std::get<2>(t));
        }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

}  // namespace zgpu

using namespace zgpu;

struct zest_gpu_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    int precision = ZEST_PRECISION_FP64;
    int slices = 6;
    std::map<std::tuple<int, int, int, int>, std::unique_ptr<ZtPlan>> zt_plans;
    std::map<std::tuple<int, int, int, int>, std::unique_ptr<StPlan>> st_plans;
    std::map<int, std::unique_ptr<FftEntry>> ffts;
    std::map<int, std::unique_ptr<DevBuf>> wigner;
    std::map<std::tuple<int, int>, std::pair<std::unique_ptr<DevBuf>, int>> vec_lists;
    std::map<std::tuple<int, int, int>, std::unique_ptr<UniformRotation>> uniform_rot;  // split rotations
    std::map<std::tuple<int, int, int, int, int, int>, std::unique_ptr<TileEntry>> tiles;
    bool autotune = true;                                     // time the tile shapes on first use
    size_t host_chunk_bytes = size_t(1) << 28;                // pipelined host calls: input bytes per chunk
    std::unique_ptr<RaggedPlan> ragged;                       // last batch of uneven orders, with its graph
    cudaStream_t graph_stream = nullptr;                      // own stream for graph capture and replay
    cudaStream_t copy_stream[2] = {nullptr, nullptr};         // host->device, device->host of pipelined calls
    cudaEvent_t pipe_ev[3][2] = {};                           // uploaded, computed, downloaded per slot
    cudaEvent_t graph_ev[2] = {nullptr, nullptr};             // ordering with the context stream
    std::map<std::tuple<int, int, int, int>, int> tuned;      // chosen shape per (stage, L, Lm, batch)
    DevBuf s0, s1;          // transform scratch (spectra, flm)
    DevBuf in_stage, out_stage, aux_stage;  // host <-> device staging
    DevBuf phase;           // rotation phases
    DevBuf adj0, adj1, adj2;  // adjoint scratch (scaled operands, inverse angles, angle partials)
    std::map<std::tuple<int, int, int>, std::unique_ptr<DevBuf>> adj_w;  // quadrature weight slabs
    std::unique_ptr<SplitState, SplitDeleter> split;
    EvalBufs eval;          // evaluation at arbitrary points
    std::unique_ptr<LsqState, LsqDeleter> lsq;  // least-squares fits
    Profiler prof;
};

namespace zgpu {
// Brackets one pipeline stage with events when profiling is on.
struct StageScope {
    zest_gpu_context* ctx;
    int stage;
    cudaStream_t stream;
    cudaEvent_t e0 = nullptr;
    StageScope(zest_gpu_context* c, int st, cudaStream_t s = nullptr) : ctx(c), stage(st), stream(s ? s : c->stream) {
        if (ctx->prof.on) {
            e0 = ctx->prof.get();
            cudaEventRecord(e0, stream);
        }
    }
    ~StageScope() {
        if (e0) {
            cudaEvent_t e1 = ctx->prof.get();
            cudaEventRecord(e1, stream);
            ctx->prof.pending.emplace_back(stage, e0, e1);
        }
    }
};
}  // namespace zgpu


