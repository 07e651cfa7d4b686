// deac_engine.cu -- host side of the GB300 DEAC engine and its C-ABI
// (include/deac_gb300.h).
//
// A batch holds any number of independent runs (seeds, temperatures, grids,
// models).  Set-up builds each run's constant terms on the host in FP64
// (deac_model.cpp), draws its initial population and per-gene PRNG table
// exactly as the reference does (deac.cpp:418-458, 1114-1135), uploads
// everything once and evaluates the initial fitness on the device.  Each
// generation of all runs is then two kernel launches (deac_kernels.cu);
// blocks of generations are captured once into a CUDA graph and replayed.
// The stop test runs on the device, so the host never synchronises inside
// a block -- the reference does a D2H copy and ~10 stream syncs per
// generation (deac.cpp:1140-1147 and the deac_wait calls of 1168-1574).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <atomic>
#include <thread>
#include <vector>

#include "deac_gb300.h"
#include "deac_kernels.cuh"
#include "deac_model.hpp"
#include "deac_rng.cuh"
#include "deac_split.cuh"

namespace {

thread_local std::string g_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_error = buf;
    return code;
}

}  // namespace

namespace deac {
// The last-error message of this thread, for the C-ABI entry points that
// live in other translation units.
__attribute__((visibility("hidden"))) int set_error(int code, const char* msg) { return fail(code, "%s", msg); }
}  // namespace deac

namespace {

#define CUDA_TRY(call)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return fail(DEAC_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                               \
    } while (0)

constexpr uint64_t kGraphBlock = 16;             // generations per captured graph
constexpr uint64_t kTrialSmemCapDoubles = 25600;  // 200 KB: trial genes + one row of weights
constexpr uint64_t kTailSlotsBytes = 4 * 1024 * 8;  // reduction slots of the finishing CTA

uint64_t align256(uint64_t x) { return (x + 255) & ~uint64_t(255); }

// Raise a kernel's dynamic shared-memory limit to at least `bytes`, never
// lower it: batches set up in other host threads (and the allocation-free
// fitness entry point) launch the same kernels with their own needs.
template <typename Kernel>
cudaError_t raise_smem_limit(Kernel kernel, size_t bytes) {
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    if ((size_t)fa.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

struct Arena {
    uint64_t size = 0;
    uint64_t take(uint64_t bytes) {
        const uint64_t off = size;
        size = align256(size + bytes);
        return off;
    }
};

// Device copy of a kernel matrix, shared by runs with identical inputs,
// with its BF16 digit planes for the split engine.
struct KernelMatrix {
    double* k_pos = nullptr;
    double* k_neg = nullptr;
    uint16_t* kdig = nullptr;   // tiled digit planes (rows = timeslices)
    bool nonneg = false;        // every entry >= 0
    int16_t* kexp = nullptr;    // [Nt][split_chunks(M)]
    int16_t* kexp_max = nullptr;  // [Nt]
    uint32_t group = 0;         // index of the runs sharing it (split tiles)
};

struct RunHost {
    deac_config cfg;
    std::vector<double> tau, isf, err, freq;
    uint64_t Nt = 0, M = 0, P = 0;
    int S = 2;
    deac::Model model;
    uint64_t rng_start[4] = {0, 0, 0, 0};  // generator state after the initial draws
    uint64_t n_states = 0;
    uint64_t trace_cap = 0;
    char* arena = nullptr;               // device allocation of this run
    uint64_t arena_bytes = 0;            // its size
    char* split_arena = nullptr;         // split-engine buffers of this run
    deac::RunDev dev{};                  // host copy of the descriptor
    deac::SplitRun split{};              // host copy of the split descriptor
    uint32_t kgroup = 0;                 // kernel-matrix group (split tiles)
    // results
    bool finished = false;
};

}  // namespace

struct deac_batch {
    int device = 0;
    cudaStream_t stream = nullptr;     // launch stream (caller's or own)
    bool own_stream = false;
    cudaStream_t capture_stream = nullptr;
    int32_t engine = DEAC_ENGINE_PLAIN_FP64;
    int32_t streams = DEAC_STREAMS_REFERENCE;
    std::vector<std::unique_ptr<RunHost>> runs;
    std::map<std::string, KernelMatrix> kcache;
    deac::RunDev* d_runs = nullptr;
    deac::Work* d_trial_work = nullptr;
    deac::Work* d_contract_work = nullptr;
    uint32_t n_trial_ctas = 0, n_contract_ctas = 0;
    int smem_doubles = 0;
    size_t trial_smem_bytes = 0;
    size_t contract_smem_bytes = 0;
    bool set_up = false;
    // snapshot of every run's status, parent fitness and parent buffers,
    // taken after the last launch (finalised: split-engine parents exact)
    bool snapped = false;
    bool snapped_all = false;  // every parent's fitness exact in the snapshot
    std::vector<deac::RunDev> snap;
    std::vector<std::vector<double>> snap_fit;
    std::vector<std::vector<uint8_t>> snap_cur;
    cudaGraphExec_t graph = nullptr;
    std::vector<deac::RunDev> status;  // host mirror of d_runs
    // split engine
    deac::SplitRun* d_split = nullptr;
    deac::SplitTile* d_tiles = nullptr;
    deac::SplitWork* d_split_work = nullptr;
    std::vector<uint16_t*> group_xdig;      // trial digit planes per kernel-matrix group
    CUtensorMap* d_maps = nullptr;          // per group: K planes, trial planes
    deac::SplitRow* d_rows = nullptr;
    float4* d_partial = nullptr;       // partial sums of the split contraction CTAs
    uint32_t n_tiles = 0, n_split_ctas = 0;
    int sms = 0;                             // the device's multiprocessors
    // split engine launch shapes (what deac_batch_autotune varies): trial
    // parts per CTA, and the contraction split so that its CTAs number about
    // split_waves x the SMs it has; the tiles before splitting kept to rebuild
    uint32_t parts_per_cta = deac::kPartsPerCta;
    uint32_t split_waves = 1;
    std::vector<deac::SplitTile> tiles_host;
    std::vector<uint32_t> tile_chunks;
    uint64_t free_sms = 1;
    uint32_t* d_final_members = nullptr;     // split engine: the final evaluations' member lists,
    uint64_t* d_final_items = nullptr;       // their items and its length
    uint32_t* d_final_count = nullptr;
    uint32_t final_capacity = 0;
    bool combine_wide = false;               // split_combine_wide_kernel sums the partials
    uint64_t* d_exact_list = nullptr;        // split engine: the exact pass's items
    uint32_t* d_exact_count = nullptr;
    uint32_t n_combine_tiles = 0;            // tiles split over several contraction CTAs
    uint32_t* d_combine_tiles = nullptr;     // their indices
    int* d_status = nullptr;            // set when a bounded wait gave up
    uint64_t* d_jpow = nullptr;         // jump_powers on the device
    uint64_t* d_jstep = nullptr;        // step_powers on the device (initial populations)
    bool any_defer = false;             // a run normalises raw trials in the selection (kDeferNorm)
    char* run_pool = nullptr;           // every run's arena, one allocation
    char* split_pool = nullptr;         // every run's split-engine buffers, one allocation
    uint32_t* d_fit_off = nullptr;      // snapshot_kernel: each run's first fitness slot (and the total)
    uint64_t* d_gene_off = nullptr;     // snapshot_kernel: each run's first gene slot
    std::vector<uint64_t> gene_off;     // its host copy
    uint64_t* d_snap = nullptr;         // snapshot_kernel output
    uint64_t* h_snap = nullptr;         // its pinned host copy
    size_t snap_bytes = 0;
    // timing: kernel kinds 0 trial, 1 contract (plain generation or exact
    // passes), 2 normalisation row sums, 3 split contraction, 4 combine + decisions (+ scaling)
    bool timing = false;
    cudaEvent_t ev[8] = {};
    // split engine, --normalize runs: the normalisation row sums run on a
    // second stream beside the tensor-core contraction (forked and joined
    // with events, also inside the captured graphs)
    cudaStream_t side_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    deac::Work* d_norm_work = nullptr;
    uint32_t n_norm_ctas = 0;
    // split engine: the raw trials in parts (trial_part_kernel)
    deac::PartWork* d_part_work = nullptr;
    uint32_t n_part_ctas = 0;
    size_t part_smem_bytes = 0;
    // split engine on counter streams: the trial slices (trial_slice_kernel)
    // of the runs with at most kSliceRows members, segments of items per
    // persistent CTA
    deac::SliceSeg* d_slice_segs = nullptr;
    uint32_t* d_slice_start = nullptr;
    uint32_t n_slice_ctas = 0;
    double kernel_ms[5] = {};
    uint64_t kernel_launches[5] = {};
    // bytes copied between host and device by this batch's calls
    uint64_t h2d_bytes = 0, d2h_bytes = 0;
};

namespace {

// cudaMemcpy / cudaMemcpyAsync that count the bytes crossing the bus
cudaError_t copy(deac_batch* b, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    const cudaError_t e = cudaMemcpy(dst, src, bytes, kind);
    if (e == cudaSuccess) {
        if (kind == cudaMemcpyHostToDevice) b->h2d_bytes += bytes;
        if (kind == cudaMemcpyDeviceToHost) b->d2h_bytes += bytes;
    }
    return e;
}
cudaError_t copy_async(deac_batch* b, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind,
                       cudaStream_t s) {
    const cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, s);
    if (e == cudaSuccess) {
        if (kind == cudaMemcpyHostToDevice) b->h2d_bytes += bytes;
        if (kind == cudaMemcpyDeviceToHost) b->d2h_bytes += bytes;
    }
    return e;
}

// A launch that may start while the previous kernel on the stream is still
// running (`early`: programmatic stream serialisation); the kernel's first
// statement, grid_dependency_wait(), holds it until that kernel is done.
template <typename... Params, typename... Args>
void launch(void (*kernel)(Params...), uint32_t grid, uint32_t block, size_t smem, cudaStream_t s, bool early,
            Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = early ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<Params>(args)...);
}

// The partial sums of the split tiles: a thread per output when no tile is
// split over more than kCombineWideSplits CTAs, else warps sharing the splits.
void launch_combine(deac_batch* b, cudaStream_t s, bool early) {
    const deac::SplitTile* tiles = b->d_tiles;
    const uint32_t* ct = b->d_combine_tiles;
    const deac::SplitRow* rows = b->d_rows;
    const float4* partial = b->d_partial;
    if (b->combine_wide)
        launch(deac::split_combine_wide_kernel, b->n_combine_tiles * deac::kCombineWideCtasPerTile, 256, 0, s, early,
               b->d_runs, b->d_split, tiles, ct, rows, partial);
    else
        launch(deac::split_combine_kernel, b->n_combine_tiles * deac::kCombineCtasPerTile, 256, 0, s, early,
               b->d_runs, b->d_split, tiles, ct, rows, partial);
}

void launch_contract(deac_batch* b, cudaStream_t s, int mode, bool early = false) {
    if (mode == deac::kModeRecheck) {
        // the listed items, over at most one CTA per SM (one fits per SM)
        const uint32_t grid = std::min<uint32_t>(2 * b->n_contract_ctas, (uint32_t)b->sms);
        // (a packed tile stages within kFinalSmemBytes)
        const size_t smem = std::max<size_t>(b->contract_smem_bytes, deac::kFinalSmemBytes);
        launch(deac::exact_pass_kernel, grid, deac::kContractThreads, smem, s, early, b->d_runs,
               static_cast<const uint64_t*>(b->d_exact_list), static_cast<const uint32_t*>(b->d_exact_count));
        return;
    }
    launch(deac::contract_kernel, b->n_contract_ctas, deac::kContractThreads, b->contract_smem_bytes, s, early,
           b->d_runs, static_cast<const deac::Work*>(b->d_contract_work), mode);
}

// One generation of every run: two launches for the plain engine; for the
// split engine trial, digits, tensor-core estimate, interval decisions and
// the exact passes for what the intervals left open.  With `timed`, events
// bracket every launch and their device times are accumulated per kind.
int launch_generation(deac_batch* b, cudaStream_t s, int init_mode, bool timed = false) {
    int e = 0;
    auto mark = [&](int kind) -> int {
        if (!timed) return DEAC_OK;
        CUDA_TRY(cudaEventRecord(b->ev[e + 1], s));
        CUDA_TRY(cudaEventSynchronize(b->ev[e + 1]));
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, b->ev[e], b->ev[e + 1]));
        b->kernel_ms[kind] += ms;
        b->kernel_launches[kind] += 1;
        ++e;
        return DEAC_OK;
    };
    if (timed) CUDA_TRY(cudaEventRecord(b->ev[0], s));
    // split engine generations: kernels whose only predecessor is the
    // previous launch on `s` are scheduled early (not when timed one by one)
    const bool early = !timed;
    int rc;
    if (b->engine == DEAC_ENGINE_PLAIN_FP64 || init_mode) {
        deac::trial_kernel<<<b->n_trial_ctas, deac::kTrialThreads, b->trial_smem_bytes, s>>>(
            b->d_runs, b->d_trial_work, init_mode, b->smem_doubles);
    } else {
        if (b->n_part_ctas)
            launch(b->streams == DEAC_STREAMS_COUNTER ? deac::trial_part_counter_kernel : deac::trial_part_kernel,
                   b->n_part_ctas, deac::kTrialPartThreads, b->part_smem_bytes, s, early, b->d_runs,
                   static_cast<const deac::PartWork*>(b->d_part_work));
        if (b->n_slice_ctas)
            launch(deac::trial_slice_kernel, b->n_slice_ctas, deac::kSliceThreads, deac::kSliceSmemBytes, s, early,
                   b->d_runs, static_cast<const deac::SliceSeg*>(b->d_slice_segs),
                   static_cast<const uint32_t*>(b->d_slice_start), b->d_status);
    }
    if ((rc = mark(0))) return rc;
    if (b->engine == DEAC_ENGINE_PLAIN_FP64 || init_mode) {
        launch_contract(b, s, init_mode ? deac::kModeInit : deac::kModeGeneration);
        if (init_mode && b->engine != DEAC_ENGINE_PLAIN_FP64)
            deac::jde_kernel<<<(b->n_trial_ctas + 127) / 128, 128, 0, s>>>(
                b->d_runs, static_cast<const deac::Work*>(b->d_trial_work), b->n_trial_ctas);
        return mark(1);
    }
    // the normalisation row sums of --normalize runs: forked beside the
    // tensor-core contraction (in line when timing kernels one by one)
    const bool fork = b->n_norm_ctas && !timed;
    if (b->n_norm_ctas) {
        cudaStream_t ns = s;
        if (fork) {
            CUDA_TRY(cudaEventRecord(b->ev_fork, s));
            CUDA_TRY(cudaStreamWaitEvent(b->side_stream, b->ev_fork, 0));
            ns = b->side_stream;
        }
        deac::norm_kernel<<<b->n_norm_ctas, deac::kNormThreads, deac::kNormSmemBytes, ns>>>(b->d_runs,
                                                                                         b->d_norm_work);
        if (fork) CUDA_TRY(cudaEventRecord(b->ev_join, b->side_stream));
        if ((rc = mark(2))) return rc;
    }
    launch(deac::split_contract_kernel, b->n_split_ctas, deac::kSplitThreads, deac::split_smem_bytes(2), s, early,
           b->d_runs, b->d_split, static_cast<const deac::SplitTile*>(b->d_tiles),
           static_cast<const deac::SplitWork*>(b->d_split_work), static_cast<const deac::SplitRow*>(b->d_rows),
           static_cast<const CUtensorMap*>(b->d_maps), b->d_partial, b->d_status);
    if ((rc = mark(3))) return rc;
    // not scheduled early: its waiting CTAs would hold the SMs that the
    // normalisation row sums need
    if (b->n_combine_tiles) launch_combine(b, s, early && !fork);
    if (fork) CUDA_TRY(cudaStreamWaitEvent(s, b->ev_join, 0));
    // (scheduled early behind the contraction or the combine: the selection
    // waits for them in its first instruction)
    const deac::Work* tw = static_cast<const deac::Work*>(b->d_trial_work);
    if (b->any_defer)
        launch(deac::split_select_kernel, b->n_trial_ctas, deac::kSelectThreads, 0, s, early && !fork, b->d_runs,
               b->d_split, tw);
    else
        launch(deac::split_select_lean_kernel, b->n_trial_ctas, deac::kSelectLeanThreads, 0, s, early && !fork,
               b->d_runs, b->d_split, tw);
    if ((rc = mark(4))) return rc;
    launch_contract(b, s, deac::kModeRecheck, early);
    return mark(1);
}

int launch_generation_timed(deac_batch* b) { return launch_generation(b, b->stream, 0, true); }

// Split engine, generation 0: the initial population's moments and
// normalisation (trial_kernel's initial pass), its digit slices, the
// tensor-core estimate of every parent and its fitness interval
// (split_init_kernel), the exact FP64 fitness of the members the intervals
// leave open and generation 0's bookkeeping (contract_kernel's initial pass,
// which skips every other member), then the first generation's jDE.
int launch_split_init(deac_batch* b) {
    cudaStream_t s = b->stream;
    std::vector<deac::PartWork> pw;
    uint32_t smax = 1;
    for (uint32_t ri = 0; ri < b->runs.size(); ++ri) {
        const RunHost& r = *b->runs[ri];
        const uint32_t parts = (uint32_t)((r.M + deac::kTrialPart - 1) / deac::kTrialPart);
        smax = std::max<uint32_t>(smax, (uint32_t)r.S);
        for (uint32_t i = 0; i < r.dev.P; ++i)
            for (uint32_t q = 0; q < parts; q += 8) pw.push_back({ri, i, q, std::min<uint32_t>(8, parts - q)});
    }
    deac::PartWork* d_pw = nullptr;
    CUDA_TRY(cudaMalloc(&d_pw, pw.size() * sizeof(deac::PartWork)));
    struct Free {
        void* p;
        ~Free() { cudaFree(p); }
    } free_pw{d_pw};
    CUDA_TRY(copy(b, d_pw, pw.data(), pw.size() * sizeof(deac::PartWork), cudaMemcpyHostToDevice));
    deac::trial_kernel<<<b->n_trial_ctas, deac::kTrialThreads, b->trial_smem_bytes, s>>>(b->d_runs, b->d_trial_work,
                                                                                          1, b->smem_doubles);
    deac::parent_digits_kernel<<<(uint32_t)pw.size(), deac::kTrialPartThreads,
                                 (size_t)smax * deac::kTrialPart * sizeof(double), s>>>(
        b->d_runs, static_cast<const deac::PartWork*>(d_pw));
    launch(deac::split_contract_kernel, b->n_split_ctas, deac::kSplitThreads, deac::split_smem_bytes(2), s, false,
           b->d_runs, b->d_split, static_cast<const deac::SplitTile*>(b->d_tiles),
           static_cast<const deac::SplitWork*>(b->d_split_work), static_cast<const deac::SplitRow*>(b->d_rows),
           static_cast<const CUtensorMap*>(b->d_maps), b->d_partial, b->d_status);
    if (b->n_combine_tiles) launch_combine(b, s, false);
    deac::split_init_kernel<<<b->n_trial_ctas, deac::kInitThreads, 0, s>>>(b->d_runs, b->d_split, b->d_trial_work);
    launch_contract(b, s, deac::kModeInit);
    deac::jde_kernel<<<(b->n_trial_ctas + 127) / 128, 128, 0, s>>>(
        b->d_runs, static_cast<const deac::Work*>(b->d_trial_work), b->n_trial_ctas);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(s));  // before the work list is freed
    return DEAC_OK;
}

// Take the snapshot the result and fetch calls read; nothing is done again
// until the next launch.  Split engine: first make exact the fitness of the
// parents that may hold each run's minimum (the best member, the reported
// minimum and spectrum), or with `all` of every parent (state fetches,
// checkpoints).  A parent whose interval starts above another's upper end
// cannot hold the minimum, so its midpoint stays in the snapshot: above the
// exact minimum, it changes neither the argmin nor the minimum.
int finalize_split(deac_batch* b, bool all = false) {
    if (b->snapped && (b->snapped_all || !all)) return DEAC_OK;
    if (b->engine == DEAC_ENGINE_SPLIT_BF16) {
        // the parents to evaluate listed per run, then only their tiles
        // (two CTAs of 96 KB per SM)
        const int mode = all ? deac::kModeFinal : deac::kModeFinalBest;
        CUDA_TRY(cudaMemsetAsync(b->d_final_count, 0, sizeof(uint32_t), b->stream));
        deac::final_list_kernel<<<(unsigned)b->runs.size(), 32, 0, b->stream>>>(
            b->d_runs, mode, b->d_final_items, b->d_final_count, b->final_capacity, b->d_status);
        CUDA_TRY(cudaGetLastError());
        const uint32_t grid = std::max<uint32_t>(1, std::min<uint32_t>(b->final_capacity, 2 * (uint32_t)b->sms));
        deac::final_exact_kernel<<<grid, deac::kContractThreads, deac::kFinalSmemBytes, b->stream>>>(
            b->d_runs, b->d_final_items, b->d_final_count, mode);
        CUDA_TRY(cudaGetLastError());
    }
    b->snapped_all = all || b->engine != DEAC_ENGINE_SPLIT_BF16;
    // every run's descriptor, parent fitness and parent buffers packed on
    // the device and read back in one copy
    const size_t n = b->runs.size();
    if (!b->d_snap) {
        std::vector<uint32_t> off(n + 1, 0);
        for (size_t r = 0; r < n; ++r) off[r + 1] = off[r] + b->runs[r]->dev.P;
        b->gene_off.assign(n + 1, 0);
        for (size_t r = 0; r < n; ++r) b->gene_off[r + 1] = b->gene_off[r] + (uint64_t)b->runs[r]->S * b->runs[r]->M;
        b->snap_bytes = n * sizeof(deac::RunDev) + (size_t)off[n] * 8 + ((size_t)off[n] + 7) / 8 * 8 +
                        (size_t)b->gene_off[n] * 8;
        CUDA_TRY(cudaMalloc(&b->d_fit_off, off.size() * 4));
        CUDA_TRY(copy(b, b->d_fit_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMalloc(&b->d_gene_off, b->gene_off.size() * 8));
        CUDA_TRY(copy(b, b->d_gene_off, b->gene_off.data(), b->gene_off.size() * 8, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMalloc(&b->d_snap, b->snap_bytes));
        CUDA_TRY(cudaMallocHost(&b->h_snap, b->snap_bytes));
    }
    deac::snapshot_kernel<<<(unsigned)n, 128, 0, b->stream>>>(b->d_runs, (uint32_t)n, b->d_fit_off, b->d_gene_off,
                                                              b->d_snap);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(copy_async(b, b->h_snap, b->d_snap, b->snap_bytes, cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    if (b->engine == DEAC_ENGINE_SPLIT_BF16) {
        int st = 0;
        CUDA_TRY(copy(b, &st, b->d_status, sizeof st, cudaMemcpyDeviceToHost));
        if (st) return fail(DEAC_E_CUDA, "the final exact evaluations failed (status %d)", st);
    }
    b->snap.resize(n);
    b->snap_fit.resize(n);
    b->snap_cur.resize(n);
    std::memcpy(b->snap.data(), b->h_snap, n * sizeof(deac::RunDev));
    const double* fit = reinterpret_cast<const double*>(reinterpret_cast<const char*>(b->h_snap) +
                                                        n * sizeof(deac::RunDev));
    size_t total = 0;
    for (size_t r = 0; r < n; ++r) total += b->runs[r]->dev.P;
    const uint8_t* cur = reinterpret_cast<const uint8_t*>(fit + total);
    size_t o = 0;
    for (size_t r = 0; r < n; ++r) {
        const uint32_t P = b->runs[r]->dev.P;
        b->snap_fit[r].assign(fit + o, fit + o + P);
        b->snap_cur[r].assign(cur + o, cur + o + P);
        o += P;
    }
    b->snapped = true;
    return DEAC_OK;
}

std::string kernel_key(const RunHost& r) {
    std::string k;
    auto put = [&k](const void* p, size_t n) { k.append(static_cast<const char*>(p), n); };
    put(&r.cfg.model, sizeof r.cfg.model);
    put(&r.cfg.zero_temperature, sizeof r.cfg.zero_temperature);
    put(&r.cfg.bosonic, sizeof r.cfg.bosonic);
    put(&r.model.beta, sizeof r.model.beta);
    put(&r.model.periodicity, sizeof r.model.periodicity);
    put(r.tau.data(), r.tau.size() * sizeof(double));
    put(r.freq.data(), r.freq.size() * sizeof(double));
    return k;
}

// Bits of the largest jump count below n (at least one).
uint32_t jump_bits(uint64_t n) {
    uint32_t b = 1;
    while (b < 64 && (1ull << b) < n) ++b;
    return b;
}

// The matrices J^(2^b), b < bits, of the PRNG jump over GF(2) (1024 words
// each), grown on demand and kept for the process: the same for every run.
const std::vector<uint64_t>& jump_powers(uint32_t bits) {
    static std::mutex mu;
    static std::vector<uint64_t> tab;
    std::lock_guard<std::mutex> lock(mu);
    if (tab.empty()) {
        tab.resize(1024);
        deac::jump_matrix(tab.data());
    }
    while (tab.size() < (size_t)bits * 1024) {
        const size_t k = tab.size();
        tab.resize(k + 1024);
        deac::gf2_matmul(tab.data() + k - 1024, tab.data() + k - 1024, tab.data() + k);
    }
    return tab;
}

// The matrices J^(2^b), b < bits, of one generator step over GF(2), grown
// on demand and kept for the process.
const std::vector<uint64_t>& step_powers(uint32_t bits) {
    static std::mutex mu;
    static std::vector<uint64_t> tab;
    std::lock_guard<std::mutex> lock(mu);
    if (tab.empty()) {
        tab.resize(1024);
        deac::step_matrix(tab.data());
    }
    while (tab.size() < (size_t)bits * 1024) {
        const size_t k = tab.size();
        tab.resize(k + 1024);
        deac::gf2_matmul(tab.data() + k - 1024, tab.data() + k - 1024, tab.data() + k);
    }
    return tab;
}

// Host part of one run's set-up: its constants (the kernel matrix is formed
// once per distinct one, after this).
void prepare_model(RunHost& r) {
    deac::build_model(r.cfg, r.tau.data(), r.isf.data(), r.err.data(), r.Nt, r.freq.data(), r.M, r.model, false);
}

// Byte offsets of a run's arena (one device allocation).
struct ArenaLayout {
    uint64_t o_isf, o_err, o_tw, o_np, o_nn, o_fp, o_fn, o_tp, o_tn, o_pop, o_cur, o_rng, o_cr, o_fw, o_fo, o_fnw,
        o_E, o_E2, o_mom, o_stats, o_trace, size;
    uint64_t pop_bytes;  // bytes of one population buffer (S P M doubles)
};

ArenaLayout arena_layout(const RunHost& r) {
    const uint64_t P = r.P, M = r.M, Nt = r.Nt, N = r.cfg.number_of_generations;
    const int S = r.S;
    Arena a;
    ArenaLayout L;
    L.o_isf = a.take(Nt * 8), L.o_err = a.take(Nt * 8), L.o_tw = a.take(Nt * 8);
    L.o_np = a.take(M * 8), L.o_nn = a.take(M * 8), L.o_fp = a.take(M * 8), L.o_fn = a.take(M * 8);
    L.o_tp = a.take(M * 8), L.o_tn = a.take(M * 8);
    L.o_pop = a.take(2ull * S * P * M * 8);
    L.o_cur = a.take(P);
    L.o_rng = a.take(4 * r.n_states * 8);
    L.o_cr = a.take(2ull * S * P * 8), L.o_fw = a.take(2ull * S * P * 8);
    L.o_fo = a.take(P * 8), L.o_fnw = a.take(P * 8);
    L.o_E = a.take(P * Nt * 8), L.o_E2 = a.take(P * Nt * 8), L.o_mom = a.take(2 * P * 8);
    L.o_stats = a.take(r.cfg.track_stats ? 3 * N * 8 : 8);
    L.o_trace = a.take(std::max<uint64_t>(r.trace_cap * P * 8, 8));
    L.size = a.size;
    L.pop_bytes = (uint64_t)S * P * M * 8;
    return L;
}

// Byte offsets of a run's split-engine buffers (one region of the batch's
// split pool).
struct SplitLayout {
    uint64_t o_xe, o_xm, o_mu, o_em, o_eb, o_ch, o_rc, o_fl, o_fh, o_tl, o_th, o_cnt, o_rcp, o_ie, o_pm, size;
};

SplitLayout split_layout(const RunHost& r) {
    const uint64_t P = r.P, Nt = r.Nt, C = deac::split_chunks(r.M);
    Arena sa;
    SplitLayout L;
    L.o_xe = sa.take(P * C * 2), L.o_xm = sa.take(P * 4), L.o_mu = sa.take(P * 3 * 4);
    L.o_em = sa.take(P * Nt * 8), L.o_eb = sa.take(P * Nt * 8);
    L.o_ch = sa.take(P), L.o_rc = sa.take(P);
    L.o_fl = sa.take(P * 8), L.o_fh = sa.take(P * 8), L.o_tl = sa.take(P * 8), L.o_th = sa.take(P * 8);
    L.o_cnt = sa.take(3 * 8);
    L.o_rcp = sa.take(P * 8), L.o_ie = sa.take(Nt * 8);
    L.o_pm = sa.take(2 * P * 8);
    L.size = sa.size;
    return L;
}

// Host part of one run's set-up: the PRNG start state.  The initial
// population (population_kernel, on the device) takes P*M*S draws of the
// stream seeded with 1407513600 + seed (deac.cpp:2089-2091); with reference
// streams the per-gene states start from the generator after them
// (deac.cpp:1114-1126): J^(PMS) s0, a product of the step matrices J^(2^b)
// of PMS's set bits.  With counter streams one slot per member (its jDE
// step count, from 0).
void prepare_start(RunHost& r, int32_t streams) {
    const uint64_t P = r.P, M = r.M, S = (uint64_t)r.S;
    r.n_states = streams == DEAC_STREAMS_COUNTER ? P : P * (1 + S * M);
    const deac::Xoshiro g = deac::Xoshiro::seeded(1407513600ULL + r.cfg.seed);
    uint64_t v[4] = {g.s[0], g.s[1], g.s[2], g.s[3]};
    if (streams != DEAC_STREAMS_COUNTER) {
        const uint64_t n = P * M * S;
        const uint32_t bits = jump_bits(n) + 1;
        const std::vector<uint64_t>& J = step_powers(bits);
        for (uint32_t b2 = 0; b2 < bits; ++b2)
            if ((n >> b2) & 1u) {
                uint64_t o[4];
                deac::gf2_matvec(J.data() + (uint64_t)b2 * 1024, v, o);
                for (int w = 0; w < 4; ++w) v[w] = o[w];
            }
    }
    for (int w = 0; w < 4; ++w) r.rng_start[w] = v[w];
}

// A run's host image, what crosses the bus at set-up (the arena is zeroed on
// the device): the ISF, its errors and the tau weights at their arena
// offsets ([0, o_np)), then packed: each weight row the run has, the
// initial CR / F and 1/sigma.
struct ImageLayout {
    uint64_t rows[6];  // norm +/-, first moment +/-, third moment +/- (~0: absent)
    uint64_t crfw, ie, size;
};

const std::vector<double>* weight_rows(const RunHost& r, int k) {
    const deac::Model& m = r.model;
    const std::vector<double>* v[6] = {&m.norm_pos, &m.norm_neg, &m.first_pos, &m.first_neg, &m.third_pos,
                                       &m.third_neg};
    return v[k];
}

ImageLayout image_layout(const RunHost& r, const ArenaLayout& L) {
    ImageLayout I;
    uint64_t o = L.o_np;
    for (int k = 0; k < 6; ++k) {
        const std::vector<double>& v = *weight_rows(r, k);
        I.rows[k] = v.empty() ? ~0ull : o;
        if (!v.empty()) o += (v.size() * 8 + 15) / 16 * 16;
    }
    I.crfw = o;
    o += 2ull * r.S * r.P * 8;
    I.ie = o;
    o += r.Nt * 8;
    I.size = (o + 255) / 256 * 256;
    return I;
}

void fill_image(RunHost& r, const ArenaLayout& L, const ImageLayout& I, int32_t streams, char* img) {
    const uint64_t P = r.P, S = (uint64_t)r.S;
    const deac::Model& m = r.model;
    std::memset(img, 0, L.o_np);
    auto put = [&](uint64_t off, const std::vector<double>& v) {
        if (!v.empty()) std::memcpy(img + off, v.data(), v.size() * 8);
    };
    put(L.o_isf, r.isf);
    put(L.o_err, r.err);
    put(L.o_tw, m.tau_weight);
    for (int k = 0; k < 6; ++k)
        if (I.rows[k] != ~0ull) put(I.rows[k], *weight_rows(r, k));
    prepare_start(r, streams);
    double* crfw = reinterpret_cast<double*>(img + I.crfw);
    for (uint64_t k = 0; k < S * P; ++k) {
        crfw[k] = r.cfg.crossover_probability;
        crfw[S * P + k] = r.cfg.differential_weight;
    }
    // 1/sigma as the split engine's decisions use it (one rounding each)
    double* ie = reinterpret_cast<double*>(img + I.ie);
    for (uint64_t t = 0; t < r.Nt; ++t) ie[t] = 1.0 / r.err[t];
}

// Device part of one run's set-up from its host image `img` (pinned; the
// copies are asynchronous on the batch stream: the image stays untouched
// until the stream has been synchronised).
int upload_run(deac_batch* b, RunHost& r, const char* img) {
    const ImageLayout I = image_layout(r, arena_layout(r));
    const uint64_t P = r.P, M = r.M, Nt = r.Nt, N = r.cfg.number_of_generations;
    const int S = r.S;
    const deac::Model& m = r.model;
    (void)N;
    // constant kernel matrix, shared between runs with the same inputs
    const std::string key = kernel_key(r);
    auto it = b->kcache.find(key);
    if (it == b->kcache.end()) {
        KernelMatrix km;
        CUDA_TRY(cudaMalloc(&km.k_pos, Nt * M * sizeof(double)));
        CUDA_TRY(copy(b, km.k_pos, m.k_pos.data(), Nt * M * sizeof(double), cudaMemcpyHostToDevice));
        if (S == 2) {
            CUDA_TRY(cudaMalloc(&km.k_neg, Nt * M * sizeof(double)));
            CUDA_TRY(copy(b, km.k_neg, m.k_neg.data(), Nt * M * sizeof(double), cudaMemcpyHostToDevice));
        }
        km.nonneg = true;
        for (double v : m.k_pos) km.nonneg = km.nonneg && v >= 0.0;
        if (S == 2)
            for (double v : m.k_neg) km.nonneg = km.nonneg && v >= 0.0;
        if (b->engine == DEAC_ENGINE_SPLIT_BF16) {
            // digit planes of K: one scale per (timeslice, 64-gene chunk)
            // shared by both sides, seven 7-bit digits per value, tiled as
            // [plane][unit of 8 genes][timeslice][8]
            const uint64_t C = deac::split_chunks(M);
            CUDA_TRY(cudaMalloc(&km.kdig, (uint64_t)deac::kDigits * S * Nt * M * 2));
            CUDA_TRY(cudaMalloc(&km.kexp, Nt * C * 2));
            CUDA_TRY(cudaMalloc(&km.kexp_max, Nt * 2));
            deac::k_digits_kernel<<<(unsigned)Nt, 256>>>(km.k_pos, S == 2 ? km.k_neg : nullptr, (uint32_t)Nt,
                                                         (uint32_t)M, km.kdig, km.kexp, km.kexp_max);
            CUDA_TRY(cudaGetLastError());
        }
        km.group = (uint32_t)b->kcache.size();
        it = b->kcache.emplace(key, km).first;
    }
    r.kgroup = it->second.group;

    const ArenaLayout L = arena_layout(r);
    const uint64_t o_isf = L.o_isf, o_err = L.o_err, o_tw = L.o_tw, o_np = L.o_np, o_nn = L.o_nn, o_fp = L.o_fp,
                   o_fn = L.o_fn, o_tp = L.o_tp, o_tn = L.o_tn, o_pop = L.o_pop, o_cur = L.o_cur, o_rng = L.o_rng,
                   o_cr = L.o_cr, o_fw = L.o_fw, o_fo = L.o_fo, o_fnw = L.o_fnw, o_E = L.o_E, o_E2 = L.o_E2,
                   o_mom = L.o_mom, o_stats = L.o_stats, o_trace = L.o_trace;
    // the run's region of the batch's pool, zeroed on the device already
    // (the initial parents, buffer 0, are drawn there by population_kernel
    // once every run is in place): only the inputs, the initial CR / F and
    // 1/sigma cross the bus
    r.arena_bytes = L.size;
    char* base = r.arena;
    const bool counter = b->streams == DEAC_STREAMS_COUNTER;
    // the ISF, its errors and the tau weights, then each weight row the run
    // has (an absent one stays zero: the pool was zeroed on the device)
    CUDA_TRY(copy_async(b, base, img, o_np, cudaMemcpyHostToDevice, b->stream));
    const uint64_t row_offsets[6] = {o_np, o_nn, o_fp, o_fn, o_tp, o_tn};
    for (int k = 0; k < 6; ++k)
        if (I.rows[k] != ~0ull)
            CUDA_TRY(copy_async(b, base + row_offsets[k], img + I.rows[k], weight_rows(r, k)->size() * 8,
                                cudaMemcpyHostToDevice, b->stream));
    const char* crfw = img + I.crfw;
    CUDA_TRY(copy_async(b, base + o_cr, crfw, (uint64_t)S * P * 8, cudaMemcpyHostToDevice, b->stream));
    CUDA_TRY(copy_async(b, base + o_fw, crfw + (uint64_t)S * P * 8, (uint64_t)S * P * 8, cudaMemcpyHostToDevice,
                        b->stream));
    if (!counter) {
        const uint32_t bits = jump_bits(r.n_states);
        // on the batch's stream: the host's set-up goes on meanwhile (the
        // device is synchronised before the initial generation)
        const uint64_t blocks = std::min<uint64_t>((r.n_states / 8 + 128) / 128, 4096);
        deac::rng_table_kernel<<<(unsigned)blocks, 128, 0, b->stream>>>(reinterpret_cast<uint64_t*>(base + o_rng), r.n_states,
                                                          b->d_jpow, bits, r.rng_start[0], r.rng_start[1],
                                                          r.rng_start[2], r.rng_start[3], (uint32_t)P, (uint32_t)M,
                                                          (uint32_t)S);
        CUDA_TRY(cudaGetLastError());
    }

    deac::RunDev& d = r.dev;
    d = deac::RunDev{};
    d.P = (uint32_t)P;
    d.M = (uint32_t)M;
    d.Nt = (uint32_t)Nt;
    d.S = (uint32_t)S;
    d.flags = (r.cfg.normalize ? deac::kNormalize : 0) | (m.use_first_moment ? deac::kFirstMoment : 0) |
              (m.use_third_moment ? deac::kThirdMoment : 0) |
              (m.use_negative_first_moment ? deac::kNegativeFirstMoment : 0) |
              (r.cfg.allow_negative_weight ? deac::kSignedWeights : 0) |
              (r.cfg.track_stats ? deac::kTrackStats : 0) | (r.trace_cap ? deac::kTrace : 0) |
              (counter ? deac::kCounterStreams : 0) |
              (m.use_first_moment && r.cfg.first_moment_formula == DEAC_FIRST_MOMENT_CPU ? deac::kFirstMomentCpu : 0);
    if (counter) deac::stream_keys(1407513600ULL + r.cfg.seed, d.key_crossover, d.key_jde);
    // contraction tile: a power-of-two number of members times timeslices
    // filling the CTA's 64 (two-sided) or 128 (one-sided) chain pairs, and a
    // staging chunk that keeps two stages within 96 KB of shared memory
    const uint32_t pairs = deac::contract_pairs((uint32_t)S);
    uint32_t mt = 1;
    while (mt * 2 <= std::min<uint64_t>(P, pairs)) mt *= 2;
    d.member_tile = mt;
    d.tau_tile = pairs / mt;
    const uint64_t rows = (uint64_t)S * (d.member_tile + d.tau_tile);
    uint64_t chunk = (96 * 1024 / 8) / (2 * rows) - 2;
    chunk = std::min<uint64_t>(chunk, 128) & ~uint64_t(1);
    d.chunk = (uint32_t)std::max<uint64_t>(chunk, 8);
    const uint32_t member_tiles = (d.P + d.member_tile - 1) / d.member_tile;
    const uint32_t tau_tiles = (d.Nt + d.tau_tile - 1) / d.tau_tile;
    d.contract_ctas = member_tiles * tau_tiles;
    d.N = N;
    d.tau_cr = r.cfg.self_adapting_crossover_probability;
    d.p_magic = ~0ull / P;
    d.tau_f = r.cfg.self_adapting_differential_weight_probability;
    auto thr = [](double tau) -> uint64_t {  // m < thr  <=>  m 2^-53 < tau for m < 2^53
        if (!(tau > 0.0)) return 0;
        if (tau >= 1.0) return 1ull << 53;
        return (uint64_t)std::ceil(tau * 0x1.0p53);
    };
    d.tau_cr_thr = thr(d.tau_cr);
    d.tau_f_thr = thr(d.tau_f);
    d.alpha = 1.0 / m.zeroth_moment;
    d.stop = r.cfg.stop_minimum_fitness;
    d.first_target = r.cfg.first_moment;
    d.third_target = r.cfg.third_moment;
    d.third_error = r.cfg.third_moment_error;
    d.negfirst_target = m.negative_first_moment;
    d.negfirst_error = m.negative_first_moment_error;
    d.k_pos = it->second.k_pos;
    d.k_neg = it->second.k_neg;
    auto ptr = [&](uint64_t off) { return reinterpret_cast<double*>(base + off); };
    d.isf = ptr(o_isf);
    d.err = ptr(o_err);
    d.tau_w = ptr(o_tw);
    d.norm_pos = ptr(o_np);
    d.norm_neg = ptr(o_nn);
    d.first_pos = ptr(o_fp);
    d.first_neg = ptr(o_fn);
    d.third_pos = ptr(o_tp);
    d.third_neg = ptr(o_tn);
    d.pop = ptr(o_pop);
    d.cur = reinterpret_cast<uint8_t*>(base + o_cur);
    d.rng = reinterpret_cast<uint64_t*>(base + o_rng);
    d.n_states = r.n_states;
    d.cr = ptr(o_cr);
    d.fw = ptr(o_fw);
    d.fit_old = ptr(o_fo);
    d.fit_new = ptr(o_fnw);
    d.model_isf = ptr(o_E);
    d.model_isf2 = ptr(o_E2);
    d.moments = ptr(o_mom);
    d.stats = ptr(o_stats);
    d.trace = ptr(o_trace);
    d.trace_cap = r.trace_cap;
    if (b->engine == DEAC_ENGINE_SPLIT_BF16) {
        const uint64_t C = deac::split_chunks(M);
        // the run's region of the batch's split pool (zeroed on the device)
        const SplitLayout SL = split_layout(r);
        const uint64_t o_xe = SL.o_xe, o_xm = SL.o_xm, o_mu = SL.o_mu, o_em = SL.o_em, o_eb = SL.o_eb,
                       o_ch = SL.o_ch, o_rc = SL.o_rc, o_fl = SL.o_fl, o_fh = SL.o_fh, o_tl = SL.o_tl,
                       o_th = SL.o_th, o_cnt = SL.o_cnt, o_rcp = SL.o_rcp, o_ie = SL.o_ie, o_pm = SL.o_pm;
        char* sb = r.split_arena;
        deac::SplitRun& x = r.split;
        x.sel_min_bits = ~0ull;  // no member tallied yet
        x.xexp = reinterpret_cast<int16_t*>(sb + o_xe);
        x.xexp_max = reinterpret_cast<int32_t*>(sb + o_xm);
        // below every exponent: no trial sliced yet
        CUDA_TRY(cudaMemsetAsync(x.xexp_max, 0x80, P * 4, b->stream));
        x.kdig = it->second.kdig;
        x.kexp = it->second.kexp;
        x.kexp_max = it->second.kexp_max;
        x.e_mp = reinterpret_cast<double*>(sb + o_em);
        x.e_bound = reinterpret_cast<double*>(sb + o_eb);
        x.changed = reinterpret_cast<uint8_t*>(sb + o_ch);
        x.recheck = reinterpret_cast<uint8_t*>(sb + o_rc);
        x.f_lo = reinterpret_cast<double*>(sb + o_fl);
        x.f_hi = reinterpret_cast<double*>(sb + o_fh);
        x.t_lo = reinterpret_cast<double*>(sb + o_tl);
        x.t_hi = reinterpret_cast<double*>(sb + o_th);
        x.counts = reinterpret_cast<unsigned long long*>(sb + o_cnt);
        // 1/sigma as the decisions use it, from the image
        CUDA_TRY(copy_async(b, sb + o_ie, img + I.ie, Nt * 8, cudaMemcpyHostToDevice, b->stream));
        x.inv_err = reinterpret_cast<const double*>(sb + o_ie);
        x.inv_nt = 1.0 / (double)Nt;
        d.changed = x.changed;
        d.xexp = x.xexp;
        d.xexp_max = x.xexp_max;
        d.mutants = reinterpret_cast<uint32_t*>(sb + o_mu);
        d.recheck = x.recheck;
        d.f_lo = x.f_lo;
        d.f_hi = x.f_hi;
        d.recip = reinterpret_cast<double*>(sb + o_rcp);
        d.pmoments = reinterpret_cast<double*>(sb + o_pm);
        // with --normalize the trials stay raw until the decisions
        if (r.cfg.normalize) d.flags |= deac::kDeferNorm;
        if (it->second.nonneg && !r.cfg.allow_negative_weight) d.flags |= deac::kNonNegProducts;
    }
    // host copies are no longer needed
    return DEAC_OK;
}

// Counter streams address draws by (generation, member, side, gene): every
// position of a run must stay below 2^63.  Null when they fit, else why not.
const char* counter_streams_unfit(const RunHost& r) {
    const long double n = (long double)r.cfg.number_of_generations, p = (long double)r.P;
    if (n * p * (long double)r.S * (long double)r.M >= 0x1p62L || n * p * (long double)deac::kJdeSpan >= 0x1p62L)
        return "number_of_generations x population_size x genome is too large for counter streams";
    return nullptr;
}

int refresh_status(deac_batch* b) {
    b->status.resize(b->runs.size());
    CUDA_TRY(copy_async(b, b->status.data(), b->d_runs, b->runs.size() * sizeof(deac::RunDev),
                             cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    return DEAC_OK;
}

int build_graph(deac_batch* b) {
    if (b->graph) return DEAC_OK;
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal));
    for (uint64_t k = 0; k < kGraphBlock; ++k) launch_generation(b, b->capture_stream, 0);
    CUDA_TRY(cudaStreamEndCapture(b->capture_stream, &g));
    cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(DEAC_E_CUDA, "cudaGraphInstantiate failed: %s", cudaGetErrorString(e));
    return DEAC_OK;
}

}  // namespace

namespace {

// Split engine: the trial digit planes of every group of runs that share a
// kernel matrix, one tiled buffer per group with the members of its runs as
// consecutive rows (the row order of the split tiles), and the two TMA
// tensor maps per group that split_contract_kernel loads its chunks with.
int make_group_planes(deac_batch* b) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return fail(DEAC_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const uint32_t ng = (uint32_t)b->kcache.size();
    std::vector<const KernelMatrix*> kms(ng, nullptr);
    for (auto& kv : b->kcache) kms[kv.second.group] = &kv.second;
    std::vector<CUtensorMap> maps(2 * ng);
    b->group_xdig.assign(ng, nullptr);
    for (uint32_t g = 0; g < ng; ++g) {
        uint64_t R = 0, M = 0, Nt = 0;
        int S = 1;
        for (auto& rp : b->runs)
            if (rp->kgroup == g) {
                R += rp->P;
                M = rp->M;
                Nt = rp->Nt;
                S = rp->S;
            }
        if (R == 0) continue;
        const uint64_t units = M / 8;
        // trial planes [side][unit][64-row tile, half][digit][32 rows][8]
        const uint64_t halves = 2 * ((R + deac::kRowTile - 1) / deac::kRowTile);
        const uint64_t unit_elems = halves * deac::kDigits * deac::kHalfRows * 8;
        const uint64_t elems = (uint64_t)S * units * unit_elems;
        CUDA_TRY(cudaMalloc(&b->group_xdig[g], elems * 2));
        CUDA_TRY(cudaMemset(b->group_xdig[g], 0, elems * 2));
        uint64_t row = 0;
        for (auto& rp : b->runs)
            if (rp->kgroup == g) {
                rp->dev.xdig = b->group_xdig[g];
                rp->dev.xdig_unit = unit_elems;
                rp->dev.xdig_side = units * unit_elems;
                rp->dev.xdig_row0 = (uint32_t)row;
                row += rp->P;
            }
        auto encode_map = [&](CUtensorMap* m, void* base, uint32_t rank, const cuuint64_t* dims,
                              const cuuint64_t* strides, const cuuint32_t* box) -> int {
            const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
            const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, rank, base, dims, strides, box, estr,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return fail(DEAC_E_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
            return DEAC_OK;
        };
        // K: a unit's timeslices are consecutive; the innermost dimension is
        // all of them (two 8-byte elements per 16-byte row): dims Nt*2,
        // units, planes; box one tile of 128 timeslices, the two units of a
        // 16-gene MMA step (one operand stage), every plane (2 KB lines)
        {
            const uint64_t planes = (uint64_t)deac::kDigits * S;
            const cuuint64_t dims[3] = {Nt * 2, units, planes};
            const cuuint64_t strides[2] = {Nt * 16, units * Nt * 16};
            const cuuint32_t box[3] = {2 * deac::kTauTile, 2, (cuuint32_t)planes};
            int rc = encode_map(&maps[2 * g], kms[g]->kdig, 3, dims, strides, box);
            if (rc) return rc;
        }
        // trials: dims 32 rows * 2, digits, (tile, half), units, sides; box
        // one tile's two halves of one 16-gene MMA step, every digit and side
        // (512-byte lines)
        {
            const cuuint64_t dims[5] = {deac::kHalfRows * 2, deac::kDigits, halves, units, (cuuint64_t)S};
            const cuuint64_t strides[4] = {deac::kHalfRows * 16, deac::kDigits * deac::kHalfRows * 16,
                                           unit_elems * 2, units * unit_elems * 2};
            const cuuint32_t box[5] = {2 * deac::kHalfRows, deac::kDigits, 2, 2, (cuuint32_t)S};
            int rc = encode_map(&maps[2 * g + 1], b->group_xdig[g], 5, dims, strides, box);
            if (rc) return rc;
        }
    }
    CUDA_TRY(cudaMalloc(&b->d_maps, maps.size() * sizeof(CUtensorMap)));
    CUDA_TRY(copy(b, b->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
    return DEAC_OK;
}

// Split engine: the trial work lists.  On counter streams the runs with at
// most kSliceRows members go to trial_slice_kernel: their items, in run
// order, spread over its persistent CTAs (one per SM) in contiguous ranges
// of about equal gene counts, as segments of consecutive items of one run.  Every other run goes to trial_part_kernel, up to
// b->parts_per_cta consecutive 512-gene parts of one member per CTA.
int build_part_work(deac_batch* b) {
    std::vector<deac::PartWork> pw;
    std::vector<uint32_t> slice_runs;
    uint64_t slice_genes = 0, slice_items = 0;
    uint32_t smax = 1;
    for (uint32_t ri = 0; ri < b->runs.size(); ++ri) {
        const RunHost& r = *b->runs[ri];
        if (b->streams == DEAC_STREAMS_COUNTER && r.dev.P <= deac::kSliceRows) {
            const uint64_t len = (uint64_t)deac::slice_chunks(r.dev.P, (uint32_t)r.S) * deac::kChunk;
            slice_runs.push_back(ri);
            slice_genes += (uint64_t)r.dev.P * r.S * r.M;
            slice_items += (r.M + len - 1) / len;
            continue;
        }
        const uint32_t parts = (uint32_t)((r.M + deac::kTrialPart - 1) / deac::kTrialPart);
        smax = std::max<uint32_t>(smax, (uint32_t)r.S);
        for (uint32_t i = 0; i < r.dev.P; ++i)
            for (uint32_t q = 0; q < parts; q += b->parts_per_cta)
                pw.push_back({ri, i, q, std::min<uint32_t>(b->parts_per_cta, parts - q)});
    }
    cudaFree(b->d_part_work);
    b->d_part_work = nullptr;
    b->n_part_ctas = (uint32_t)pw.size();
    b->part_smem_bytes = (size_t)smax * deac::kTrialPart * sizeof(double);
    if (!pw.empty()) {
        CUDA_TRY(cudaMalloc(&b->d_part_work, pw.size() * sizeof(deac::PartWork)));
        CUDA_TRY(copy(b, b->d_part_work, pw.data(), pw.size() * sizeof(deac::PartWork), cudaMemcpyHostToDevice));
    }
    cudaFree(b->d_slice_segs);
    cudaFree(b->d_slice_start);
    b->d_slice_segs = nullptr;
    b->d_slice_start = nullptr;
    b->n_slice_ctas = 0;
    if (slice_runs.empty()) return DEAC_OK;
    CUDA_TRY(raise_smem_limit(deac::trial_slice_kernel, deac::kSliceSmemBytes));
    int per_sm = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, deac::trial_slice_kernel, deac::kSliceThreads,
                                                           deac::kSliceSmemBytes));
    const uint32_t G = (uint32_t)std::min<uint64_t>(slice_items, (uint64_t)std::max(per_sm, 1) * b->sms);
    std::vector<deac::SliceSeg> segs;
    std::vector<uint32_t> start(G + 1, 0);
    uint64_t acc = 0;
    int64_t last = -1;  // CTA of the last segment
    for (uint32_t ri : slice_runs) {
        const RunHost& r = *b->runs[ri];
        const uint32_t P = r.dev.P, S = (uint32_t)r.S, M = (uint32_t)r.M;
        const uint32_t len = deac::slice_chunks(P, S) * deac::kChunk;
        const uint32_t items = (M + len - 1) / len;
        for (uint32_t it = 0; it < items; ++it) {
            const uint64_t w = (uint64_t)P * S * std::min(len, M - it * len);
            // the CTA whose share of the genes holds this item's middle
            const int64_t cta = (int64_t)std::min<uint64_t>(G - 1, (acc + w / 2) * G / slice_genes);
            acc += w;
            if (segs.empty() || cta != last || segs.back().run != ri) {
                for (int64_t q = last + 1; q <= cta; ++q) start[q] = (uint32_t)segs.size();
                segs.push_back({ri, it, it + 1});
                last = cta;
            } else {
                segs.back().item1 = it + 1;
            }
        }
    }
    for (int64_t q = last + 1; q <= (int64_t)G; ++q) start[q] = (uint32_t)segs.size();
    CUDA_TRY(cudaMalloc(&b->d_slice_segs, segs.size() * sizeof(deac::SliceSeg)));
    CUDA_TRY(cudaMalloc(&b->d_slice_start, start.size() * sizeof(uint32_t)));
    CUDA_TRY(copy(b, b->d_slice_segs, segs.data(), segs.size() * sizeof(deac::SliceSeg), cudaMemcpyHostToDevice));
    CUDA_TRY(copy(b, b->d_slice_start, start.data(), start.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    b->n_slice_ctas = G;
    return DEAC_OK;
}

// Split engine: the batch's chunks (summed over its tiles) shared out so that
// no CTA takes more than total / (split_waves x the SMs the row sums leave
// free) of them (one CTA per SM: the kernel uses ~214 KB of shared memory and
// all of TMEM); a tile is split in proportion to its chunk count, so long
// tiles (large M) no longer set the launch's tail. Partial-sum blocks only for
// tiles split over several CTAs (a tile with one CTA has its estimates formed
// by that CTA).
int build_split_work(deac_batch* b) {
    std::vector<deac::SplitTile> tiles = b->tiles_host;
    const std::vector<uint32_t>& tile_chunks = b->tile_chunks;
    uint64_t total = 0;
    for (uint32_t C : tile_chunks) total += C;
    const uint64_t ctas = std::max<uint64_t>(1, b->split_waves * b->free_sms);
    const uint64_t target = std::max<uint64_t>(1, (total + ctas - 1) / ctas);
    std::vector<deac::SplitWork> work;
    std::vector<uint32_t> combine_tiles;
    uint32_t blocks = 0, max_split = 1;
    for (uint32_t t = 0; t < tiles.size(); ++t) {
        const uint32_t C = tile_chunks[t];
        const uint32_t want = (uint32_t)std::min<uint64_t>(C, (C + target - 1) / target);
        const uint32_t per = (C + want - 1) / want;
        const uint32_t nsplit = (C + per - 1) / per;
        tiles[t].block0 = nsplit > 1 ? blocks : ~0u;
        tiles[t].nsplit = nsplit;
        tiles[t].per = per;
        for (uint32_t c0 = 0; c0 < C; c0 += per)
            work.push_back({t, c0, std::min(C, c0 + per), nsplit > 1 ? blocks++ : ~0u});
        if (nsplit > 1) combine_tiles.push_back(t);
        max_split = std::max(max_split, nsplit);
    }
    b->combine_wide = max_split <= deac::kCombineWideSplits;
    // longest pieces first: the block scheduler hands CTAs out in index
    // order, so this is longest-processing-time-first over the SMs
    std::stable_sort(work.begin(), work.end(), [](const deac::SplitWork& a, const deac::SplitWork& b2) {
        return a.c1 - a.c0 > b2.c1 - b2.c0;
    });
    for (void* p : {(void*)b->d_combine_tiles, (void*)b->d_tiles, (void*)b->d_split_work, (void*)b->d_partial})
        cudaFree(p);
    b->d_combine_tiles = nullptr;
    b->d_tiles = nullptr;
    b->d_split_work = nullptr;
    b->d_partial = nullptr;
    b->n_tiles = (uint32_t)tiles.size();
    b->n_combine_tiles = (uint32_t)combine_tiles.size();
    b->n_split_ctas = (uint32_t)work.size();
    if (!combine_tiles.empty()) {
        CUDA_TRY(cudaMalloc(&b->d_combine_tiles, combine_tiles.size() * sizeof(uint32_t)));
        CUDA_TRY(copy(b, b->d_combine_tiles, combine_tiles.data(), combine_tiles.size() * sizeof(uint32_t),
                      cudaMemcpyHostToDevice));
    }
    CUDA_TRY(cudaMalloc(&b->d_tiles, tiles.size() * sizeof(deac::SplitTile)));
    CUDA_TRY(copy(b, b->d_tiles, tiles.data(), tiles.size() * sizeof(deac::SplitTile), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMalloc(&b->d_split_work, work.size() * sizeof(deac::SplitWork)));
    CUDA_TRY(copy(b, b->d_split_work, work.data(), work.size() * sizeof(deac::SplitWork), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMalloc(&b->d_partial, std::max<uint64_t>(blocks, 1) * deac::kPartialBlock * sizeof(float4)));
    return DEAC_OK;
}

// The shapes autotuning chose for batches of the same mix (sizes, sides and
// row sums of their runs), for this process.
std::mutex g_tune_mutex;
std::map<std::string, std::pair<uint32_t, uint32_t>> g_tune_cache;

std::string tune_key(const deac_batch* b) {
    std::vector<std::string> parts;
    for (auto& r : b->runs) {
        char buf[96];
        snprintf(buf, sizeof buf, "%d/%llu/%llu/%llu/%u;", r->S, (unsigned long long)r->M, (unsigned long long)r->Nt,
                 (unsigned long long)r->P,
                 (unsigned)(r->dev.flags & (deac::kDeferNorm | deac::kFirstMoment | deac::kThirdMoment)));
        parts.emplace_back(buf);
    }
    std::sort(parts.begin(), parts.end());
    std::string k = std::to_string(b->kcache.size()) + "|" + std::to_string(b->streams) + "|";
    for (auto& p : parts) k += p;
    return k;
}

}  // namespace

extern "C" {

const char* deac_last_error(void) { return g_error.c_str(); }

const char* deac_version(void) { return "deac-gb300 0.1.0 (sm_103a)"; }

void deac_config_default(deac_config* c) {
    std::memset(c, 0, sizeof *c);
    c->model = DEAC_MODEL_STANDARD;
    c->spectra_type = DEAC_SPECTRA_SPFSF;
    c->temperature = 0.0;
    c->first_moment = -1.0;
    c->third_moment = -1.0;
    c->third_moment_error = 0.0;
    c->crossover_probability = 0.9;
    c->self_adapting_crossover_probability = 0.1;
    c->differential_weight = 0.9;
    c->self_adapting_differential_weight_probability = 0.1;
    c->self_adapting_differential_weight_shift = 0.1;
    c->self_adapting_differential_weight = 0.9;
    c->stop_minimum_fitness = 1.0;
    c->number_of_generations = 100000;
    c->population_size = 512;
    c->seed = 0;
}

int deac_config_check(const deac_config* c) {
    if (!c) return fail(DEAC_E_INVALID, "null configuration");
    const std::string msg = deac::check_config(*c);
    if (!msg.empty()) return fail(DEAC_E_INVALID, "%s", msg.c_str());
    return DEAC_OK;
}

int deac_batch_create(int device, void* cuda_stream, int32_t engine, deac_batch** out) {
    if (!out) return fail(DEAC_E_INVALID, "null output pointer");
    *out = nullptr;
    if (engine != DEAC_ENGINE_PLAIN_FP64 && engine != DEAC_ENGINE_SPLIT_BF16)
        return fail(DEAC_E_INVALID, "unknown engine %d", engine);
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0)
        return fail(DEAC_E_NODEVICE, "no CUDA device %d", device);
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10 || prop.minor != 3)
        return fail(DEAC_E_NODEVICE, "device %d is sm_%d%d; this library is built for sm_103a (GB300)", device,
                    prop.major, prop.minor);
    CUDA_TRY(cudaSetDevice(device));
    auto b = std::make_unique<deac_batch>();
    b->device = device;
    b->engine = engine;
    if (cuda_stream) {
        b->stream = static_cast<cudaStream_t>(cuda_stream);
    } else {
        CUDA_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        b->own_stream = true;
    }
    CUDA_TRY(cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&b->side_stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming));
    for (auto& e : b->ev) CUDA_TRY(cudaEventCreate(&e));
    *out = b.release();
    return DEAC_OK;
}

int deac_batch_add_run(deac_batch* b, const deac_config* cfg, const double* tau, const double* isf,
                       const double* err, uint64_t nt, const double* freq, uint64_t m, uint32_t* run_index) {
    if (!b || !cfg || !tau || !isf || !err || !freq) return fail(DEAC_E_INVALID, "null argument");
    if (b->set_up) return fail(DEAC_E_STATE, "runs must be added before deac_batch_setup");
    int rc = deac_config_check(cfg);
    if (rc) return rc;
    if (nt < 2) return fail(DEAC_E_INVALID, "ISF input file must contain at least two timeslices");
    if (m < 2) return fail(DEAC_E_INVALID, "genome_size must be at least 2");
    if (cfg->population_size > (1u << 20) || m > (1u << 26) || nt > (1u << 20))
        return fail(DEAC_E_INVALID, "problem size beyond the engine's limits");
    if (isf[0] == 0.0 && cfg->normalize) return fail(DEAC_E_INVALID, "--normalize needs a nonzero F(0)");
    if (b->engine == DEAC_ENGINE_SPLIT_BF16 && m % deac::kGeneStep != 0)
        return fail(DEAC_E_INVALID, "the split engine needs genome_size a multiple of %d", deac::kGeneStep);
    auto r = std::make_unique<RunHost>();
    r->cfg = *cfg;
    r->P = cfg->population_size;
    r->M = m;
    r->S = cfg->bosonic ? 1 : 2;
    if (b->streams == DEAC_STREAMS_COUNTER) {
        const char* why = counter_streams_unfit(*r);
        if (why) return fail(DEAC_E_INVALID, "%s", why);
    }
    r->tau.assign(tau, tau + nt);
    r->isf.assign(isf, isf + nt);
    r->err.assign(err, err + nt);
    r->freq.assign(freq, freq + m);
    r->Nt = nt;
    r->M = m;
    r->P = cfg->population_size;
    r->S = cfg->bosonic ? 1 : 2;
    if (run_index) *run_index = (uint32_t)b->runs.size();
    b->runs.push_back(std::move(r));
    return DEAC_OK;
}

int deac_batch_set_streams(deac_batch* b, int32_t layout) {
    if (!b) return fail(DEAC_E_INVALID, "null batch");
    if (b->set_up) return fail(DEAC_E_STATE, "choose the stream layout before deac_batch_setup");
    if (layout != DEAC_STREAMS_REFERENCE && layout != DEAC_STREAMS_COUNTER)
        return fail(DEAC_E_INVALID, "unknown stream layout %d", layout);
    if (layout == DEAC_STREAMS_COUNTER)
        for (auto& r : b->runs) {
            const char* why = counter_streams_unfit(*r);
            if (why) return fail(DEAC_E_INVALID, "%s", why);
        }
    b->streams = layout;
    return DEAC_OK;
}

int deac_batch_enable_trace(deac_batch* b, uint32_t run, uint64_t max_generations) {
    if (!b || run >= b->runs.size()) return fail(DEAC_E_INVALID, "bad run index");
    if (b->set_up) return fail(DEAC_E_STATE, "enable the trace before deac_batch_setup");
    b->runs[run]->trace_cap = max_generations;
    return DEAC_OK;
}

int deac_batch_setup(deac_batch* b) {
    if (!b) return fail(DEAC_E_INVALID, "null batch");
    if (b->set_up) return DEAC_OK;
    if (b->runs.empty()) return fail(DEAC_E_STATE, "empty batch");
    CUDA_TRY(cudaSetDevice(b->device));
    // host preparation of the runs' constants, spread over the host's threads
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    {
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < hw && t < b->runs.size(); ++t)
            pool.emplace_back([b, t, hw] {
                for (size_t k = t; k < b->runs.size(); k += hw) prepare_model(*b->runs[k]);
            });
        for (auto& th : pool) th.join();
        pool.clear();
        // the kernel matrix of each distinct (model, T, tau and omega grid),
        // in the first run that has it (the one upload_run takes it from),
        // its rows spread over the host's threads
        std::map<std::string, RunHost*> owners;
        for (auto& rp : b->runs) owners.emplace(kernel_key(*rp), rp.get());
        // blocks of 8 rows of every matrix, taken from one list by all the
        // host's threads
        std::vector<std::pair<RunHost*, uint64_t>> blocks;
        for (auto& kv : owners) {
            RunHost& r = *kv.second;
            r.model.k_pos.assign(r.Nt * r.M, 0.0);
            if (r.S == 2) r.model.k_neg.assign(r.Nt * r.M, 0.0);
            for (uint64_t i0 = 0; i0 < r.Nt; i0 += 8) blocks.emplace_back(&r, i0);
        }
        std::atomic<size_t> next{0};
        pool.clear();
        for (unsigned t = 0; t < hw && t < blocks.size(); ++t)
            pool.emplace_back([&blocks, &next] {
                for (size_t k; (k = next.fetch_add(1)) < blocks.size();) {
                    RunHost& r = *blocks[k].first;
                    const uint64_t i0 = blocks[k].second;
                    deac::kernel_rows(r.cfg, r.model, r.tau.data(), r.freq.data(), r.M, i0, std::min(r.Nt, i0 + 8));
                }
            });
        for (auto& th : pool) th.join();
    }
    for (auto& r : b->runs)
        r->n_states = b->streams == DEAC_STREAMS_COUNTER ? r->P : r->P * (1 + (uint64_t)r->S * r->M);
    if (b->streams == DEAC_STREAMS_REFERENCE) {
        uint32_t bits = 1;
        for (auto& r : b->runs) bits = std::max(bits, jump_bits(r->n_states));
        const std::vector<uint64_t>& jp = jump_powers(bits);
        CUDA_TRY(cudaMalloc(&b->d_jpow, (size_t)bits * 1024 * 8));
        CUDA_TRY(copy(b, b->d_jpow, jp.data(), (size_t)bits * 1024 * 8, cudaMemcpyHostToDevice));
    }
    {
        // the step matrices the initial populations' threads jump with
        uint32_t bits = 1;
        for (auto& r : b->runs) bits = std::max(bits, jump_bits((uint64_t)r->P * r->M * r->S) + 1);
        const std::vector<uint64_t>& J = step_powers(bits);
        CUDA_TRY(cudaMalloc(&b->d_jstep, (size_t)bits * 1024 * 8));
        CUDA_TRY(copy(b, b->d_jstep, J.data(), (size_t)bits * 1024 * 8, cudaMemcpyHostToDevice));
    }
    {
        // every run's arena (and split-engine buffers) in one allocation,
        // zeroed on the device
        uint64_t run_bytes = 0, split_bytes = 0;
        for (auto& r : b->runs) {
            run_bytes += arena_layout(*r).size;
            if (b->engine == DEAC_ENGINE_SPLIT_BF16) split_bytes += split_layout(*r).size;
        }
        CUDA_TRY(cudaMalloc(&b->run_pool, run_bytes));
        CUDA_TRY(cudaMemsetAsync(b->run_pool, 0, run_bytes, b->stream));
        if (split_bytes) {
            CUDA_TRY(cudaMalloc(&b->split_pool, split_bytes));
            CUDA_TRY(cudaMemsetAsync(b->split_pool, 0, split_bytes, b->stream));
        }
        uint64_t ro = 0, so = 0;
        for (auto& r : b->runs) {
            r->arena = b->run_pool + ro;
            ro += arena_layout(*r).size;
            if (split_bytes) {
                r->split_arena = b->split_pool + so;
                so += split_layout(*r).size;
            }
        }
    }
    uint64_t trial_doubles = 0, contract_bytes = std::max<uint64_t>(kTailSlotsBytes, deac::kContractMinSmemBytes);
    std::vector<deac::Work> tw, cw;
    // every run's host image in one pinned buffer, filled by all the host's
    // threads, then copied asynchronously run by run
    std::vector<uint64_t> image_off(b->runs.size() + 1, 0);
    for (size_t k = 0; k < b->runs.size(); ++k)
        image_off[k + 1] = image_off[k] + image_layout(*b->runs[k], arena_layout(*b->runs[k])).size;
    char* images = nullptr;
    struct PinnedFree {
        char** p;
        ~PinnedFree() {
            if (*p) cudaFreeHost(*p);
        }
    } pinned_free{&images};
    CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&images), std::max<uint64_t>(image_off.back(), 256)));
    {
        std::atomic<size_t> next{0};
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < hw && t < b->runs.size(); ++t)
            pool.emplace_back([b, &next, &image_off, images] {
                for (size_t k; (k = next.fetch_add(1)) < b->runs.size();) {
                    RunHost& rk = *b->runs[k];
                    const ArenaLayout L = arena_layout(rk);
                    fill_image(rk, L, image_layout(rk, L), b->streams, images + image_off[k]);
                }
            });
        for (auto& th : pool) th.join();
    }
    for (uint32_t ri = 0; ri < b->runs.size(); ++ri) {
        RunHost& r = *b->runs[ri];
        int rc = upload_run(b, r, images + image_off[ri]);
        if (rc) return rc;
        for (uint32_t i = 0; i < r.dev.P; ++i) tw.push_back({ri, i});
        for (uint32_t k = 0; k < r.dev.contract_ctas; ++k) cw.push_back({ri, k});
        // trial genes, plus one row of weights when a row sum is formed
        const uint64_t genes = (uint64_t)r.S * r.M;
        const bool sums = (r.dev.flags & (deac::kNormalize | deac::kFirstMoment | deac::kThirdMoment)) != 0;
        if (sums && 2 * genes <= kTrialSmemCapDoubles) trial_doubles = std::max(trial_doubles, 2 * genes);
        else if (genes <= kTrialSmemCapDoubles) trial_doubles = std::max(trial_doubles, genes);
        const uint64_t stage =
            deac::stage_doubles(r.dev.S, r.dev.member_tile, r.dev.tau_tile, r.dev.chunk) * 2 * sizeof(double);
        contract_bytes = std::max<uint64_t>(contract_bytes, stage);
    }
    {
        // every run's initial population, one launch
        std::vector<deac::PopRun> pr;
        std::vector<deac::PopWork> pwk;
        for (uint32_t ri = 0; ri < b->runs.size(); ++ri) {
            const RunHost& r = *b->runs[ri];
            const deac::Xoshiro g = deac::Xoshiro::seeded(1407513600ULL + r.cfg.seed);
            pr.push_back({reinterpret_cast<double*>(r.arena + arena_layout(r).o_pop),
                          {g.s[0], g.s[1], g.s[2], g.s[3]}, (uint32_t)r.P, (uint32_t)r.M, (uint32_t)r.S,
                          r.cfg.allow_negative_weight ? 1u : 0u});
            const uint64_t threads =
                ((uint64_t)r.P * r.M * r.S + (1ull << deac::kPopBlockLog2) - 1) >> deac::kPopBlockLog2;
            for (uint64_t t0 = 0; t0 < threads; t0 += deac::kPopThreads) pwk.push_back({ri, (uint32_t)t0});
        }
        deac::PopRun* d_pr = nullptr;
        deac::PopWork* d_pw = nullptr;
        CUDA_TRY(cudaMalloc(&d_pr, pr.size() * sizeof(deac::PopRun)));
        CUDA_TRY(cudaMalloc(&d_pw, pwk.size() * sizeof(deac::PopWork)));
        struct Free {
            void* a;
            void* b;
            ~Free() {
                cudaFree(a);
                cudaFree(b);
            }
        } free_pop{d_pr, d_pw};
        CUDA_TRY(copy(b, d_pr, pr.data(), pr.size() * sizeof(deac::PopRun), cudaMemcpyHostToDevice));
        CUDA_TRY(copy(b, d_pw, pwk.data(), pwk.size() * sizeof(deac::PopWork), cudaMemcpyHostToDevice));
        deac::population_kernel<<<(unsigned)pwk.size(), deac::kPopThreads, 0, b->stream>>>(d_pr, d_pw, b->d_jstep);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamSynchronize(b->stream));  // before the lists are freed
    }
    b->smem_doubles = (int)trial_doubles;
    b->trial_smem_bytes = trial_doubles * sizeof(double);
    b->contract_smem_bytes = contract_bytes;
    CUDA_TRY(raise_smem_limit(deac::trial_kernel, std::max<size_t>(b->trial_smem_bytes, 1024)));
    CUDA_TRY(raise_smem_limit(deac::contract_kernel, b->contract_smem_bytes));
    CUDA_TRY(raise_smem_limit(deac::exact_pass_kernel,
                              std::max<size_t>(b->contract_smem_bytes, deac::kFinalSmemBytes)));
    CUDA_TRY(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device));
    b->n_trial_ctas = (uint32_t)tw.size();
    b->n_contract_ctas = (uint32_t)cw.size();
    if (b->engine == DEAC_ENGINE_SPLIT_BF16) {
        // one CTA per trial of every run that normalises or has moment
        // terms (their exact row sums)
        std::vector<deac::Work> nw;
        for (uint32_t ri = 0; ri < b->runs.size(); ++ri) {
            const RunHost& r = *b->runs[ri];
            if (r.dev.flags & deac::kDeferNorm) b->any_defer = true;
            if (!(r.dev.flags & (deac::kDeferNorm | deac::kFirstMoment | deac::kThirdMoment))) continue;
            for (uint32_t i = 0; i < r.dev.P; ++i) nw.push_back({ri, i});
        }
        int rc = build_part_work(b);
        if (rc) return rc;
        b->n_norm_ctas = (uint32_t)nw.size();
        if (!nw.empty()) {
            CUDA_TRY(raise_smem_limit(deac::norm_kernel, deac::kNormSmemBytes));
            CUDA_TRY(cudaMalloc(&b->d_norm_work, nw.size() * sizeof(deac::Work)));
            CUDA_TRY(copy(b, b->d_norm_work, nw.data(), nw.size() * sizeof(deac::Work), cudaMemcpyHostToDevice));
        }
    }
    CUDA_TRY(cudaMalloc(&b->d_trial_work, tw.size() * sizeof(deac::Work)));
    CUDA_TRY(cudaMalloc(&b->d_contract_work, cw.size() * sizeof(deac::Work)));
    CUDA_TRY(copy(b, b->d_trial_work, tw.data(), tw.size() * sizeof(deac::Work), cudaMemcpyHostToDevice));
    CUDA_TRY(copy(b, b->d_contract_work, cw.data(), cw.size() * sizeof(deac::Work), cudaMemcpyHostToDevice));
    if (b->engine == DEAC_ENGINE_SPLIT_BF16) {
        int rc = make_group_planes(b);
        if (rc) return rc;
    }
    if (b->engine == DEAC_ENGINE_SPLIT_BF16) {
        // the exact pass lists both passes of a run, in the run's own tiles
        // or packed with its open members (at most the largest packed tiling)
        uint64_t exact_cap = 0;
        for (auto& r : b->runs) {
            uint32_t most = r->dev.contract_ctas;
            for (uint32_t n = 1; n <= r->dev.P; ++n) {
                uint32_t mt, tt, chunk, ctas;
                deac::final_tiling(n, r->dev.S, r->dev.Nt, mt, tt, chunk, ctas, deac::kExactMinMembers);
                most = std::max(most, ctas);
            }
            exact_cap += 2ull * most;
        }
        CUDA_TRY(cudaMalloc(&b->d_exact_list, std::max<uint64_t>(exact_cap, 1) * sizeof(uint64_t)));
        CUDA_TRY(cudaMalloc(&b->d_exact_count, sizeof(uint32_t)));
        CUDA_TRY(cudaMemset(b->d_exact_count, 0, sizeof(uint32_t)));
        for (auto& r : b->runs) {
            r->dev.exact_list = b->d_exact_list;
            r->dev.exact_count = b->d_exact_count;
        }
        // the final exact evaluations: every run's member list, and room
        // for the item list of the largest tiling of every run
        uint64_t members = 0, cap = 0;
        for (auto& r : b->runs) {
            members += r->dev.P;
            uint32_t most = 0;
            for (uint32_t n = 1; n <= r->dev.P; ++n) {
                uint32_t mt, tt, chunk, ctas;
                deac::final_tiling(n, r->dev.S, r->dev.Nt, mt, tt, chunk, ctas);
                most = std::max(most, ctas);
            }
            cap += most;
        }
        b->final_capacity = (uint32_t)cap;
        CUDA_TRY(cudaMalloc(&b->d_final_members, members * sizeof(uint32_t)));
        CUDA_TRY(cudaMalloc(&b->d_final_items, std::max<uint64_t>(cap, 1) * sizeof(uint64_t)));
        CUDA_TRY(cudaMalloc(&b->d_final_count, sizeof(uint32_t)));
        uint64_t off = 0;
        for (auto& r : b->runs) {
            r->dev.final_members = b->d_final_members + off;
            off += r->dev.P;
        }
        CUDA_TRY(raise_smem_limit(deac::final_exact_kernel, deac::kFinalSmemBytes));
    }
    std::vector<deac::RunDev> descs;
    for (auto& r : b->runs) descs.push_back(r->dev);
    CUDA_TRY(cudaMalloc(&b->d_runs, descs.size() * sizeof(deac::RunDev)));
    CUDA_TRY(copy(b, b->d_runs, descs.data(), descs.size() * sizeof(deac::RunDev), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMalloc(&b->d_status, sizeof(int)));
    CUDA_TRY(cudaMemset(b->d_status, 0, sizeof(int)));
    if (b->engine == DEAC_ENGINE_SPLIT_BF16) {
        std::vector<deac::SplitRun> xs;
        for (auto& r : b->runs) xs.push_back(r->split);
        CUDA_TRY(cudaMalloc(&b->d_split, xs.size() * sizeof(deac::SplitRun)));
        CUDA_TRY(copy(b, b->d_split, xs.data(), xs.size() * sizeof(deac::SplitRun), cudaMemcpyHostToDevice));
        // output tiles: the members of all runs that share a kernel matrix,
        // 64 rows at a time, times 128 timeslices
        std::vector<deac::SplitRow> rows;
        std::vector<deac::SplitTile> tiles;
        std::vector<uint32_t> tile_chunks;
        for (uint32_t g = 0; g < b->kcache.size(); ++g) {
            std::vector<deac::SplitRow> grp;
            uint32_t nt = 0, chunks = 0;
            for (uint32_t ri = 0; ri < b->runs.size(); ++ri) {
                if (b->runs[ri]->kgroup != g) continue;
                nt = (uint32_t)b->runs[ri]->Nt;
                chunks = deac::split_chunks(b->runs[ri]->M);
                for (uint32_t m = 0; m < b->runs[ri]->P; ++m) grp.push_back({ri, m});
            }
            for (size_t r0 = 0; r0 < grp.size(); r0 += deac::kRowTile) {
                const uint32_t nrow = (uint32_t)std::min<size_t>(deac::kRowTile, grp.size() - r0);
                for (uint32_t t0 = 0; t0 < nt; t0 += deac::kTauTile) {
                    tiles.push_back({t0, (uint32_t)(rows.size() + r0), nrow, grp[r0].run, 0, 0, 0, g, (uint32_t)r0});
                    tile_chunks.push_back(chunks);
                }
            }
            rows.insert(rows.end(), grp.begin(), grp.end());
        }
        // the normalisation and moment row sums run beside the contraction:
        // leave them their SMs (up to half)
        uint64_t norm_ctas = 0;
        for (auto& r : b->runs)
            if (r->dev.flags & (deac::kDeferNorm | deac::kFirstMoment | deac::kThirdMoment)) norm_ctas += r->P;
        b->free_sms = (uint64_t)b->sms - std::min<uint64_t>(norm_ctas, (uint64_t)b->sms / 2);
        b->tiles_host = tiles;
        b->tile_chunks = tile_chunks;
        int rc = build_split_work(b);
        if (rc) return rc;
        CUDA_TRY(cudaMalloc(&b->d_rows, rows.size() * sizeof(deac::SplitRow)));
        CUDA_TRY(copy(b, b->d_rows, rows.data(), rows.size() * sizeof(deac::SplitRow), cudaMemcpyHostToDevice));
        CUDA_TRY(raise_smem_limit(deac::split_contract_kernel, deac::split_smem_bytes(2)));
    }
    CUDA_TRY(cudaDeviceSynchronize());
    // initial fitness, statistics of generation 0 and the first stop test
    if (b->engine == DEAC_ENGINE_SPLIT_BF16) {
        int rc = launch_split_init(b);
        if (rc) return rc;
    } else {
        launch_generation(b, b->stream, 1);
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->set_up = true;
    return refresh_status(b);
}

int deac_batch_launch(deac_batch* b, uint64_t generations) {
    if (!b) return fail(DEAC_E_INVALID, "null batch");
    if (!b->set_up) return fail(DEAC_E_STATE, "deac_batch_setup has not run");
    if (b->timing) {
        b->snapped = false;
        for (uint64_t g = 0; g < generations; ++g) {
            int rc = launch_generation_timed(b);
            if (rc) return rc;
        }
        CUDA_TRY(cudaGetLastError());
        return DEAC_OK;
    }
    // whole blocks as the captured graph, the remainder launched directly
    const uint64_t blocks = generations / kGraphBlock, rest = generations % kGraphBlock;
    if (blocks) {
        int rc = build_graph(b);
        if (rc) return rc;
    }
    b->snapped = false;
    for (uint64_t g = 0; g < blocks; ++g) CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
    for (uint64_t g = 0; g < rest; ++g) {
        int rc = launch_generation(b, b->stream, 0);
        if (rc) return rc;
    }
    CUDA_TRY(cudaGetLastError());
    return DEAC_OK;
}

int deac_batch_sync(deac_batch* b, uint32_t* runs_finished) {
    if (!b) return fail(DEAC_E_INVALID, "null batch");
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    CUDA_TRY(cudaGetLastError());
    if (b->d_status) {
        int st = 0;
        CUDA_TRY(copy(b, &st, b->d_status, sizeof st, cudaMemcpyDeviceToHost));
        if (st) return fail(DEAC_E_CUDA, "a tensor-core wait gave up (status %d)", st);
    }
    int rc = refresh_status(b);
    if (rc) return rc;
    uint32_t n = 0;
    for (auto& s : b->status) n += s.done ? 1 : 0;
    if (runs_finished) *runs_finished = n;
    return DEAC_OK;
}

int deac_batch_run(deac_batch* b) {
    if (!b) return fail(DEAC_E_INVALID, "null batch");
    int rc = deac_batch_setup(b);
    if (rc) return rc;
    uint32_t done = 0;
    if ((rc = deac_batch_sync(b, &done))) return rc;
    // a run needs at most N-1 generations; poll every few graph blocks
    uint64_t block = kGraphBlock * 4;
    while (done < b->runs.size()) {
        if ((rc = deac_batch_launch(b, block))) return rc;
        if ((rc = deac_batch_sync(b, &done))) return rc;
        block = std::min<uint64_t>(block * 2, kGraphBlock * 256);
    }
    return DEAC_OK;
}

int deac_batch_size(const deac_batch* b, uint32_t* runs) {
    if (!b || !runs) return fail(DEAC_E_INVALID, "null argument");
    *runs = (uint32_t)b->runs.size();
    return DEAC_OK;
}

// Copy a run's parents and fitness back and locate the best member.
static int gather(deac_batch* b, uint32_t run, std::vector<double>& pop, std::vector<double>& fit,
                  std::vector<double>* crfw, deac::RunDev& st) {
    RunHost& r = *b->runs[run];
    int rc = finalize_split(b, true);
    if (rc) return rc;
    CUDA_TRY(copy(b, &st, b->d_runs + run, sizeof st, cudaMemcpyDeviceToHost));
    const uint64_t P = r.P, M = r.M, S = r.S;
    std::vector<uint8_t> cur(P);
    std::vector<double> both(2 * S * P * M);
    fit.assign(P, 0.0);
    CUDA_TRY(copy(b, cur.data(), st.cur, P, cudaMemcpyDeviceToHost));
    CUDA_TRY(copy(b, both.data(), st.pop, both.size() * 8, cudaMemcpyDeviceToHost));
    CUDA_TRY(copy(b, fit.data(), st.fit_old, P * 8, cudaMemcpyDeviceToHost));
    pop.assign(S * P * M, 0.0);
    for (uint64_t s = 0; s < S; ++s)
        for (uint64_t i = 0; i < P; ++i)
            std::memcpy(&pop[(s * P + i) * M], &both[((uint64_t)cur[i] * S * P + s * P + i) * M], M * 8);
    if (crfw) {
        crfw->assign(4 * S * P, 0.0);
        CUDA_TRY(copy(b, crfw->data(), st.cr, S * P * 8, cudaMemcpyDeviceToHost));
        CUDA_TRY(copy(b, crfw->data() + 2 * S * P, st.fw, S * P * 8, cudaMemcpyDeviceToHost));
    }
    return DEAC_OK;
}

static void summarize(const RunHost& r, const deac::RunDev& st, const std::vector<double>& fit,
                      deac_run_result* out) {
    // argmin_and_min: first index of the strict minimum (deac.cpp:146-158)
    uint64_t best = 0;
    double mn = fit[0];
    for (uint64_t i = 0; i < fit.size(); ++i)
        if (fit[i] < mn) {
            mn = fit[i];
            best = i;
        }
    uint64_t gen = st.generation;
    if (st.done && gen == r.cfg.number_of_generations - 2) gen += 1;  // deac.cpp:1677-1679
    std::memset(out, 0, sizeof *out);
    out->generation = gen;
    out->minimum_fitness = mn;
    out->best_index = best;
    out->spectrum_length = r.S == 2 ? 2 * r.M - 1 : r.M;
    out->stats_length = r.cfg.track_stats ? gen + 1 : 0;
    out->population_size = r.P;
    out->genome_size = r.M;
    out->number_of_timeslices = r.Nt;
    out->sides = r.S;
    out->finished = st.done ? 1 : 0;
}

int deac_batch_result(deac_batch* b, uint32_t run, deac_run_result* out) {
    if (!b || !out || run >= b->runs.size()) return fail(DEAC_E_INVALID, "bad argument");
    if (!b->set_up) return fail(DEAC_E_STATE, "deac_batch_setup has not run");
    RunHost& r = *b->runs[run];
    int rc = finalize_split(b);
    if (rc) return rc;
    summarize(r, b->snap[run], b->snap_fit[run], out);
    return DEAC_OK;
}

int deac_batch_fetch(deac_batch* b, uint32_t run, double* best_dsf, double* best_frequency,
                     double* stats_mean, double* stats_minimum, double* stats_squared_mean) {
    if (!b || run >= b->runs.size()) return fail(DEAC_E_INVALID, "bad argument");
    if (!b->set_up) return fail(DEAC_E_STATE, "deac_batch_setup has not run");
    RunHost& r = *b->runs[run];
    const uint64_t P = r.P, M = r.M, S = r.S;
    // only the fitness, the buffer indices and the best member's genes cross
    // the bus (the reference copies the whole population, deac.cpp:1577-1590)
    int rc0 = finalize_split(b);
    if (rc0) return rc0;
    const deac::RunDev& st = b->snap[run];
    const std::vector<double>& fit = b->snap_fit[run];
    deac_run_result res;
    summarize(r, st, fit, &res);
    // the best parent's genes (res.best_index, found by snapshot_kernel
    // in the same values) are in the snapshot
    size_t total = 0;
    for (auto& rp : b->runs) total += rp->dev.P;
    const double* const genes =
        reinterpret_cast<const double*>(reinterpret_cast<const char*>(b->h_snap) + b->runs.size() * sizeof(deac::RunDev) +
                                        total * 8 + (total + 7) / 8 * 8) +
        b->gene_off[run];
    const uint64_t L = res.spectrum_length;
    if (best_dsf && best_frequency) {
        deac::best_spectrum(r.cfg, r.model, r.freq.data(), M, genes, S == 2 ? &genes[M] : nullptr, best_dsf,
                            best_frequency);
    } else if (best_dsf || best_frequency) {
        std::vector<double> dsf(L), fr(L);
        deac::best_spectrum(r.cfg, r.model, r.freq.data(), M, genes, S == 2 ? &genes[M] : nullptr, dsf.data(),
                            fr.data());
        if (best_dsf) std::memcpy(best_dsf, dsf.data(), L * 8);
        if (best_frequency) std::memcpy(best_frequency, fr.data(), L * 8);
    }
    if (r.cfg.track_stats && (stats_mean || stats_minimum || stats_squared_mean)) {
        const uint64_t N = r.cfg.number_of_generations, n = res.stats_length;
        std::vector<double> stats(3 * n);
        for (int k = 0; k < 3; ++k)
            if (n) CUDA_TRY(copy(b, &stats[k * n], st.stats + k * N, n * 8, cudaMemcpyDeviceToHost));
        if (st.done && st.generation == N - 2) {
            // last entry from the host, with the sequential mean
            // (deac.cpp:1677-1685)
            stats[n - 1] = deac::sequential_mean(fit.data(), P);
            stats[2 * n - 1] = res.minimum_fitness;
            stats[3 * n - 1] = deac::sequential_squared_mean(fit.data(), P);
        }
        if (stats_mean) std::memcpy(stats_mean, stats.data(), n * 8);
        if (stats_minimum) std::memcpy(stats_minimum, stats.data() + n, n * 8);
        if (stats_squared_mean) std::memcpy(stats_squared_mean, stats.data() + 2 * n, n * 8);
    }
    return DEAC_OK;
}

int deac_batch_spectra_length(deac_batch* b, uint64_t* doubles) {
    if (!b || !doubles) return fail(DEAC_E_INVALID, "bad argument");
    uint64_t n = 0;
    for (auto& r : b->runs) n += r->S == 2 ? 2 * r->M - 1 : r->M;
    *doubles = n;
    return DEAC_OK;
}

int deac_batch_fetch_all(deac_batch* b, deac_run_result* results, double* best_dsf, double* best_frequency) {
    if (!b) return fail(DEAC_E_INVALID, "bad argument");
    if (!b->set_up) return fail(DEAC_E_STATE, "deac_batch_setup has not run");
    int rc0 = finalize_split(b);
    if (rc0) return rc0;
    const size_t n = b->runs.size();
    size_t total = 0;
    for (auto& rp : b->runs) total += rp->dev.P;
    const double* const genes0 = reinterpret_cast<const double*>(
        reinterpret_cast<const char*>(b->h_snap) + n * sizeof(deac::RunDev) + total * 8 + (total + 7) / 8 * 8);
    std::vector<deac_run_result> res(n);
    std::vector<uint64_t> off(n + 1, 0);
    for (size_t r = 0; r < n; ++r) {
        summarize(*b->runs[r], b->snap[r], b->snap_fit[r], &res[r]);
        off[r + 1] = off[r] + res[r].spectrum_length;
    }
    if (results) std::memcpy(results, res.data(), n * sizeof(deac_run_result));
    if (best_dsf || best_frequency) {
        // runs shared out over host threads, by their spectrum lengths
        const unsigned threads = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 32u));
        std::atomic<size_t> next{0};
        auto work = [&]() {
            std::vector<double> scratch;
            for (size_t r; (r = next.fetch_add(1)) < n;) {
                const RunHost& rh = *b->runs[r];
                const uint64_t M = rh.M, L = res[r].spectrum_length;
                const double* genes = genes0 + b->gene_off[r];
                double* d = best_dsf ? best_dsf + off[r] : nullptr;
                double* f = best_frequency ? best_frequency + off[r] : nullptr;
                if (!d || !f) {
                    scratch.resize(L);
                    if (!d) d = scratch.data();
                    if (!f) f = scratch.data();
                }
                deac::best_spectrum(rh.cfg, rh.model, rh.freq.data(), M, genes, rh.S == 2 ? &genes[M] : nullptr, d,
                                    f);
            }
        };
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < threads; ++t) pool.emplace_back(work);
        work();
        for (auto& th : pool) th.join();
    }
    return DEAC_OK;
}

int deac_batch_fetch_state(deac_batch* b, uint32_t run, double* population, double* fitness,
                           double* crossover_rates, double* differential_weights) {
    if (!b || run >= b->runs.size()) return fail(DEAC_E_INVALID, "bad argument");
    if (!b->set_up) return fail(DEAC_E_STATE, "deac_batch_setup has not run");
    RunHost& r = *b->runs[run];
    std::vector<double> pop, fit, crfw;
    deac::RunDev st;
    int rc = gather(b, run, pop, fit, &crfw, st);
    if (rc) return rc;
    const uint64_t SP = (uint64_t)r.S * r.P;
    if (population) std::memcpy(population, pop.data(), pop.size() * 8);
    if (fitness) std::memcpy(fitness, fit.data(), fit.size() * 8);
    if (crossover_rates) std::memcpy(crossover_rates, crfw.data(), SP * 8);
    if (differential_weights) std::memcpy(differential_weights, crfw.data() + 2 * SP, SP * 8);
    return DEAC_OK;
}

namespace {

// A checkpoint: this header, then the run's evolving state as it lies in its
// arena (both parent buffers, the parent selectors, the PRNG table, CR and F,
// fitness, model ISF, moments, statistics and trace), from the population to
// the end.  The constant inputs before it are not saved: a restore takes
// them from the run it restores into.
struct CheckpointHeader {
    char magic[8];  // "DEACCKP2"
    uint32_t P, M, Nt, S;
    uint64_t N;
    uint64_t state_bytes;
    uint64_t ii, generation;
    int32_t done;
    uint32_t flags;
    uint64_t inputs;  // input_hash of the run
    int32_t kind;     // kCheckpointPlain or kCheckpointSplit
    uint32_t reserved;
};
// A plain-engine block is taken at a generation boundary before the next
// jDE step; a split-engine block after it, with the next generation's mutant
// indices ([P][3] uint32) and the run's decision counts (3 uint64) appended.
constexpr int32_t kCheckpointPlain = 0, kCheckpointSplit = 1;
uint64_t split_extra_bytes(const RunHost& r) { return r.P * 3 * sizeof(uint32_t) + 3 * sizeof(uint64_t); }

uint64_t state_offset(const RunHost& r) { return (uint64_t)(reinterpret_cast<char*>(r.dev.pop) - r.arena); }

// FNV-1a over the run's whole configuration (seed, temperature, model,
// spectra type, moment targets, jDE parameters, stop fitness ...) and its
// input arrays (tau, F, sigma, frequency grid): a checkpoint continues only
// a run with the same inputs, not merely the same sizes.
uint64_t input_hash(const RunHost& r) {
    uint64_t h = 1469598103934665603ull;
    auto put = [&h](const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        for (size_t k = 0; k < n; ++k) h = (h ^ c[k]) * 1099511628211ull;
    };
    put(&r.cfg, sizeof r.cfg);
    for (const std::vector<double>* v : {&r.tau, &r.isf, &r.err, &r.freq}) {
        const uint64_t n = v->size();
        put(&n, sizeof n);
        put(v->data(), n * sizeof(double));
    }
    return h;
}

}  // namespace

int deac_batch_checkpoint(deac_batch* b, uint32_t run, void* out, uint64_t capacity, uint64_t* bytes) {
    if (!b || run >= b->runs.size() || !bytes) return fail(DEAC_E_INVALID, "bad argument");
    if (!b->set_up) return fail(DEAC_E_STATE, "deac_batch_setup has not run");
    RunHost& r = *b->runs[run];
    const bool split = b->engine == DEAC_ENGINE_SPLIT_BF16;
    const uint64_t off = state_offset(r), state = r.arena_bytes - off;
    *bytes = sizeof(CheckpointHeader) + state + (split ? split_extra_bytes(r) : 0);
    if (!out) return DEAC_OK;
    if (capacity < *bytes) return fail(DEAC_E_INVALID, "checkpoint buffer too small (%llu < %llu bytes)",
                                       (unsigned long long)capacity, (unsigned long long)*bytes);
    if (split) {
        // every parent's fitness exact (the checkpoint holds no intervals)
        int rc = finalize_split(b, true);
        if (rc) return rc;
    }
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    deac::RunDev st;
    CUDA_TRY(copy(b, &st, b->d_runs + run, sizeof st, cudaMemcpyDeviceToHost));
    CheckpointHeader h{};
    std::memcpy(h.magic, "DEACCKP2", 8);
    h.P = st.P;
    h.M = st.M;
    h.Nt = st.Nt;
    h.S = st.S;
    h.N = st.N;
    h.state_bytes = state;
    h.ii = st.ii;
    h.generation = st.generation;
    h.done = st.done;
    h.flags = st.flags & ~(deac::kDeferNorm | deac::kNonNegProducts);  // engine-specific flags
    h.inputs = input_hash(r);
    h.kind = split ? kCheckpointSplit : kCheckpointPlain;
    char* dst = static_cast<char*>(out);
    std::memcpy(dst, &h, sizeof h);
    CUDA_TRY(copy(b, dst + sizeof h, r.arena + off, state, cudaMemcpyDeviceToHost));
    if (split) {
        char* extra = dst + sizeof h + state;
        CUDA_TRY(copy(b, extra, r.dev.mutants, r.P * 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        CUDA_TRY(copy(b, extra + r.P * 3 * sizeof(uint32_t), r.split.counts, 3 * sizeof(uint64_t),
                      cudaMemcpyDeviceToHost));
    }
    return DEAC_OK;
}

int deac_batch_restore(deac_batch* b, uint32_t run, const void* in, uint64_t bytes) {
    if (!b || run >= b->runs.size() || !in) return fail(DEAC_E_INVALID, "bad argument");
    if (!b->set_up) return fail(DEAC_E_STATE, "deac_batch_setup has not run");
    RunHost& r = *b->runs[run];
    const bool split = b->engine == DEAC_ENGINE_SPLIT_BF16;
    const uint64_t off = state_offset(r), state = r.arena_bytes - off;
    CheckpointHeader h;
    if (bytes < sizeof h) return fail(DEAC_E_INVALID, "checkpoint too short");
    std::memcpy(&h, in, sizeof h);
    const deac::RunDev& d = r.dev;
    if (std::memcmp(h.magic, "DEACCKP2", 8) != 0) return fail(DEAC_E_INVALID, "not a checkpoint");
    if (h.kind != kCheckpointPlain && h.kind != kCheckpointSplit) return fail(DEAC_E_INVALID, "not a checkpoint");
    const uint64_t want = sizeof h + state + (h.kind == kCheckpointSplit ? split_extra_bytes(r) : 0);
    const uint32_t flags = d.flags & ~(deac::kDeferNorm | deac::kNonNegProducts);
    if (h.P != d.P || h.M != d.M || h.Nt != d.Nt || h.S != d.S || h.N != d.N || h.flags != flags ||
        h.state_bytes != state || bytes != want)
        return fail(DEAC_E_INVALID, "checkpoint of a different configuration");
    if (h.inputs != input_hash(r))
        return fail(DEAC_E_INVALID, "checkpoint of a run with other inputs (seed, temperature, model, data or grid)");
    if (h.kind == kCheckpointSplit && !split)
        return fail(DEAC_E_INVALID,
                    "a split-engine checkpoint (its next jDE step already drawn) continues only in the split engine");
    // the values the kernels index with must lie in range
    if (h.ii > h.N || h.generation > h.N || (h.done != 0 && h.done != 1))
        return fail(DEAC_E_INVALID, "checkpoint counters out of range");
    const char* body = static_cast<const char*>(in) + sizeof h;
    const uint64_t cur_off = (uint64_t)(reinterpret_cast<char*>(d.cur) - r.arena) - off;
    for (uint64_t i = 0; i < d.P; ++i)
        if ((uint8_t)body[cur_off + i] > 1) return fail(DEAC_E_INVALID, "checkpoint parent selector out of range");
    if (h.kind == kCheckpointSplit) {
        const uint32_t* mut = reinterpret_cast<const uint32_t*>(body + state);
        for (uint64_t k = 0; k < 3 * d.P; ++k)
            if (mut[k] >= d.P) return fail(DEAC_E_INVALID, "checkpoint mutant index out of range");
    }
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    CUDA_TRY(copy(b, r.arena + off, body, state, cudaMemcpyHostToDevice));
    deac::RunDev st;
    CUDA_TRY(copy(b, &st, b->d_runs + run, sizeof st, cudaMemcpyDeviceToHost));
    st.ii = h.ii;
    st.generation = h.generation;
    st.done = h.done;
    st.ticket = 0;
    CUDA_TRY(copy(b, b->d_runs + run, &st, sizeof st, cudaMemcpyHostToDevice));
    if (split) {
        // the split state of a generation boundary: exact parents (their
        // intervals are points), no trial sliced or pending, the selection
        // tallies cleared
        const uint64_t P = r.P;
        const double* fit = reinterpret_cast<const double*>(body + ((reinterpret_cast<char*>(d.fit_old) - r.arena) - off));
        CUDA_TRY(copy(b, r.split.f_lo, fit, P * 8, cudaMemcpyHostToDevice));
        CUDA_TRY(copy(b, r.split.f_hi, fit, P * 8, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemset(r.split.changed, 0, P));
        CUDA_TRY(cudaMemset(r.split.recheck, 0, P));
        CUDA_TRY(cudaMemset(r.split.xexp_max, 0x80, P * 4));
        CUDA_TRY(copy(b, b->d_split + run, &r.split, sizeof r.split, cudaMemcpyHostToDevice));
        if (h.kind == kCheckpointSplit) {
            CUDA_TRY(copy(b, d.mutants, body + state, P * 3 * sizeof(uint32_t), cudaMemcpyHostToDevice));
            CUDA_TRY(copy(b, r.split.counts, body + state + P * 3 * sizeof(uint32_t), 3 * sizeof(uint64_t),
                          cudaMemcpyHostToDevice));
        } else {
            CUDA_TRY(cudaMemset(r.split.counts, 0, 3 * sizeof(uint64_t)));
            // a plain block stops before the next jDE step: draw it for this
            // run's members (its slice of the trial work list), as after set-up
            uint64_t first = 0;
            for (uint32_t k = 0; k < run; ++k) first += b->runs[k]->P;
            deac::jde_kernel<<<(unsigned)((P + 127) / 128), 128, 0, b->stream>>>(
                b->d_runs, static_cast<const deac::Work*>(b->d_trial_work) + first, (uint32_t)P);
            CUDA_TRY(cudaGetLastError());
            CUDA_TRY(cudaStreamSynchronize(b->stream));
        }
    }
    b->snapped = false;
    return refresh_status(b);
}

int deac_batch_fetch_trace(deac_batch* b, uint32_t run, double* trial_fitness, uint64_t capacity) {
    if (!b || run >= b->runs.size() || !trial_fitness) return fail(DEAC_E_INVALID, "bad argument");
    RunHost& r = *b->runs[run];
    if (!b->set_up || !r.trace_cap) return fail(DEAC_E_STATE, "no trace recorded");
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    deac::RunDev st;
    CUDA_TRY(copy(b, &st, b->d_runs + run, sizeof st, cudaMemcpyDeviceToHost));
    const uint64_t rows = std::min(std::min(st.ii, r.trace_cap), capacity);
    if (rows) CUDA_TRY(copy(b, trial_fitness, st.trace, rows * r.P * 8, cudaMemcpyDeviceToHost));
    return DEAC_OK;
}

int deac_batch_split_counts(deac_batch* b, uint32_t run, uint64_t counts[3]) {
    if (!b || run >= b->runs.size() || !counts) return fail(DEAC_E_INVALID, "bad argument");
    if (b->engine != DEAC_ENGINE_SPLIT_BF16 || !b->set_up) return fail(DEAC_E_STATE, "not a set-up split batch");
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    CUDA_TRY(copy(b, counts, b->runs[run]->split.counts, 3 * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    return DEAC_OK;
}

int deac_batch_autotune(deac_batch* b, uint64_t generations, deac_tune_report* out) {
    if (!b || !out) return fail(DEAC_E_INVALID, "null argument");
    if (!b->set_up) return fail(DEAC_E_STATE, "deac_batch_setup has not run");
    std::memset(out, 0, sizeof *out);
    if (b->engine != DEAC_ENGINE_SPLIT_BF16) return DEAC_OK;  // the plain engine's shapes are fixed
    if (b->timing) return fail(DEAC_E_STATE, "disable kernel timing before autotuning");
    CUDA_TRY(cudaSetDevice(b->device));
    const std::string key = tune_key(b);
    auto apply = [&](uint32_t parts, uint32_t waves) -> int {
        if (parts == b->parts_per_cta && waves == b->split_waves) return DEAC_OK;
        CUDA_TRY(cudaStreamSynchronize(b->stream));
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        b->parts_per_cta = parts;
        b->split_waves = waves;
        int rc = build_part_work(b);
        if (rc) return rc;
        return build_split_work(b);
    };
    // time `generations` real generations of the batch in the current
    // shapes (the shapes change no result)
    auto time_it = [&](double& ms) -> int {
        cudaEvent_t e0 = b->ev[6], e1 = b->ev[7];
        CUDA_TRY(cudaEventRecord(e0, b->stream));
        int rc = deac_batch_launch(b, generations);
        if (rc) return rc;
        CUDA_TRY(cudaEventRecord(e1, b->stream));
        CUDA_TRY(cudaEventSynchronize(e1));
        float f = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&f, e0, e1));
        ms = (double)f / (double)generations;
        return DEAC_OK;
    };
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end() || generations == 0) {
            const uint32_t parts = it != g_tune_cache.end() ? it->second.first : b->parts_per_cta;
            const uint32_t waves = it != g_tune_cache.end() ? it->second.second : b->split_waves;
            int rc = apply(parts, waves);
            if (rc) return rc;
            out->parts_per_cta = parts;
            out->split_waves = waves;
            out->from_cache = it != g_tune_cache.end() ? 1 : 0;
            return DEAC_OK;
        }
    }
    static const uint32_t kParts[] = {1, 2, 4, 8};
    static const uint32_t kWaves[] = {1, 2, 4};
    double best_ms = 0.0;
    uint32_t best_parts = b->parts_per_cta, best_waves = b->split_waves;
    // the defaults first (also warms the caches), then every other candidate
    std::vector<std::pair<uint32_t, uint32_t>> cands{{b->parts_per_cta, b->split_waves}};
    // (parts per CTA only shape trial_part_kernel: no choice when every run
    // goes to trial_slice_kernel)
    for (uint32_t p : kParts)
        for (uint32_t w : kWaves)
            if ((p != b->parts_per_cta || w != b->split_waves) && (b->n_part_ctas || p == b->parts_per_cta))
                cands.emplace_back(p, w);
    for (size_t k = 0; k < cands.size(); ++k) {
        int rc = apply(cands[k].first, cands[k].second);
        if (rc) return rc;
        double ms = 0.0;
        if ((rc = time_it(ms))) return rc;
        if (k == 0) out->ms_per_generation_default = ms;
        if (k == 0 || ms < best_ms) {
            best_ms = ms;
            best_parts = cands[k].first;
            best_waves = cands[k].second;
        }
        out->candidates += 1;
    }
    int rc = apply(best_parts, best_waves);
    if (rc) return rc;
    out->parts_per_cta = best_parts;
    out->split_waves = best_waves;
    out->ms_per_generation = best_ms;
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = {best_parts, best_waves};
    return DEAC_OK;
}

int deac_batch_generation_launches(const deac_batch* b, uint32_t* launches) {
    if (!b || !launches) return fail(DEAC_E_INVALID, "null argument");
    if (!b->set_up) return fail(DEAC_E_STATE, "deac_batch_setup has not run");
    // as launch_generation issues them
    if (b->engine == DEAC_ENGINE_PLAIN_FP64) {
        *launches = 2;  // trial_kernel, contract_kernel
    } else {
        *launches = (b->n_part_ctas ? 1u : 0u) + (b->n_slice_ctas ? 1u : 0u) + (b->n_norm_ctas ? 1u : 0u) +
                    1u /* split_contract_kernel */ + (b->n_combine_tiles ? 1u : 0u) +
                    1u /* split_select_kernel */ + 1u /* exact_pass_kernel */;
    }
    return DEAC_OK;
}

int deac_batch_transfer_bytes(const deac_batch* b, uint64_t* host_to_device, uint64_t* device_to_host) {
    if (!b) return fail(DEAC_E_INVALID, "null batch");
    if (host_to_device) *host_to_device = b->h2d_bytes;
    if (device_to_host) *device_to_host = b->d2h_bytes;
    return DEAC_OK;
}

int deac_batch_enable_timing(deac_batch* b, int32_t enable) {
    if (!b) return fail(DEAC_E_INVALID, "null batch");
    b->timing = enable != 0;
    for (int k = 0; k < 5; ++k) {
        b->kernel_ms[k] = 0.0;
        b->kernel_launches[k] = 0;
    }
    return DEAC_OK;
}

int deac_batch_kernel_time(deac_batch* b, int32_t kind, double* ms, uint64_t* launches) {
    if (!b || kind < 0 || kind > 4) return fail(DEAC_E_INVALID, "bad argument");
    if (ms) *ms = b->kernel_ms[kind];
    if (launches) *launches = b->kernel_launches[kind];
    return DEAC_OK;
}

int deac_batch_destroy(deac_batch* b) {
    if (!b) return DEAC_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    cudaFree(b->run_pool);
    cudaFree(b->split_pool);
    for (auto& kv : b->kcache) {
        cudaFree(kv.second.k_pos);
        if (kv.second.k_neg) cudaFree(kv.second.k_neg);
        if (kv.second.kdig) cudaFree(kv.second.kdig);
        if (kv.second.kexp) cudaFree(kv.second.kexp);
        if (kv.second.kexp_max) cudaFree(kv.second.kexp_max);
    }
    cudaFree(b->d_split);
    cudaFree(b->d_tiles);
    cudaFree(b->d_split_work);
    for (uint16_t* x : b->group_xdig) cudaFree(x);
    cudaFree(b->d_maps);
    cudaFree(b->d_partial);
    cudaFree(b->d_combine_tiles);
    cudaFree(b->d_exact_list);
    cudaFree(b->d_final_members);
    cudaFree(b->d_final_items);
    cudaFree(b->d_final_count);
    cudaFree(b->d_exact_count);
    cudaFree(b->d_rows);
    cudaFree(b->d_status);
    cudaFree(b->d_jpow);
    cudaFree(b->d_jstep);
    cudaFree(b->d_fit_off);
    cudaFree(b->d_gene_off);
    cudaFree(b->d_snap);
    if (b->h_snap) cudaFreeHost(b->h_snap);
    cudaFree(b->d_runs);
    cudaFree(b->d_trial_work);
    cudaFree(b->d_contract_work);
    for (auto& e : b->ev)
        if (e) cudaEventDestroy(e);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    cudaFree(b->d_norm_work);
    cudaFree(b->d_part_work);
    cudaFree(b->d_slice_segs);
    cudaFree(b->d_slice_start);
    if (b->side_stream) cudaStreamDestroy(b->side_stream);
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
    return DEAC_OK;
}

int deac_reconstruct(const deac_config* cfg, const double* tau, const double* isf, const double* err,
                     uint64_t nt, const double* freq, uint64_t m, deac_run_result* result, double* best_dsf,
                     double* best_frequency, double* stats_mean, double* stats_minimum,
                     double* stats_squared_mean) {
    deac_batch* b = nullptr;
    int rc = deac_batch_create(0, nullptr, DEAC_ENGINE_PLAIN_FP64, &b);
    if (rc) return rc;
    std::unique_ptr<deac_batch, int (*)(deac_batch*)> guard(b, deac_batch_destroy);
    if ((rc = deac_batch_add_run(b, cfg, tau, isf, err, nt, freq, m, nullptr))) return rc;
    if ((rc = deac_batch_run(b))) return rc;
    if (result && (rc = deac_batch_result(b, 0, result))) return rc;
    return deac_batch_fetch(b, 0, best_dsf, best_frequency, stats_mean, stats_minimum, stats_squared_mean);
}

}  // extern "C"
