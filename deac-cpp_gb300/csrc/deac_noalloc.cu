// deac_noalloc.cu -- deac_population_fitness_noalloc: the fitness pass of
// contract_kernel for a population that the caller already holds in device
// memory, with the kernel's scratch in a fixed static device array instead of
// memory allocated per call.
//
// Who needs it: callers that cannot allocate device memory at the moment they
// want fitness values.  A framework that reserves most of the GPU when it
// starts (or a pool allocator that owns every buffer) leaves a cudaMalloc from
// this library failing even though the caller holds every input and output;
// and cudaFree waits for the whole device, which stalls the caller's other
// streams.  Such callers pass their own device buffers for the inputs and the
// output; everything else the kernel needs lives in `g_fitness_scratch`.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>

#include "deac_gb300.h"
#include "deac_kernels.cuh"

// Scratch of every call on a device: the run descriptor, the CTA work list,
// the members' buffer indices and the member x timeslice model-ISF matrix.
// Reserved when a GPU loads this library and held until the process exits.
static __device__ __align__(256) unsigned char g_fitness_scratch[DEAC_NOALLOC_SCRATCH_BYTES];

namespace deac {
__attribute__((visibility("hidden"))) int set_error(int code, const char* msg);
}

namespace {

int error(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int error(int code, const char* fmt, ...) {
    char buf[384];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return deac::set_error(code, buf);
}

#define NOALLOC_TRY(call)                                                                              \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return error(DEAC_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

uint64_t round256(uint64_t x) { return (x + 255) & ~uint64_t(255); }

// Offsets of the scratch parts for one call.
struct ScratchLayout {
    uint64_t work, cur, model_isf, total;
};
ScratchLayout layout(uint64_t P, uint64_t Nt, uint64_t ctas) {
    ScratchLayout l;
    l.work = round256(sizeof(deac::RunDev));
    l.cur = l.work + round256(ctas * sizeof(deac::Work));
    l.model_isf = l.cur + round256(P);
    l.total = l.model_isf + P * Nt * sizeof(double);
    return l;
}

// Writes the run descriptor and the work list and clears the buffer indices:
// everything contract_kernel expects to find at zero or freshly set, since
// the scratch keeps whatever the previous call left in it.
__global__ void noalloc_prepare_kernel(deac::RunDev desc, deac::RunDev* run, deac::Work* work, uint32_t n_work,
                                       uint8_t* cur, uint32_t P) {
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *run = desc;
    for (uint32_t k = i; k < n_work; k += stride) work[k] = deac::Work{0u, k};
    for (uint32_t m = i; m < P; m += stride) cur[m] = 0;
}

// With the target device current: the device address of the scratch array
// in the current context (its host-side name is only a stand-in).  Looked up
// on every call rather than cached, so that a context torn down and made
// again (cudaDeviceReset, a new primary context) never leaves a stale
// address behind; the lookup is cheap beside the launch.
int scratch_address(int device, void** scratch) {
    void* p = nullptr;
    NOALLOC_TRY(cudaGetSymbolAddress(&p, g_fitness_scratch));
    if (!p) return error(DEAC_E_CUDA, "no device address for the fitness scratch on device %d", device);
    *scratch = p;
    return DEAC_OK;
}

bool aligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

}  // namespace

extern "C" int deac_population_fitness_noalloc(int device, void* cuda_stream, int32_t sides,
                                               const double* population, uint64_t population_size,
                                               uint64_t genome_size, const double* kernel_pos,
                                               const double* kernel_neg, const double* isf,
                                               const double* isf_error, uint64_t number_of_timeslices,
                                               double* fitness) {
    const uint64_t P = population_size, M = genome_size, Nt = number_of_timeslices;
    // --- arguments (checked before any CUDA call)
    if (sides != 1 && sides != 2) return error(DEAC_E_INVALID, "sides must be 1 or 2, not %d", sides);
    if (P == 0 || M == 0 || Nt == 0) return error(DEAC_E_INVALID, "population, genome and timeslice counts must be positive");
    if (P > UINT32_MAX || M > UINT32_MAX || Nt > UINT32_MAX)
        return error(DEAC_E_INVALID, "population, genome and timeslice counts must fit in 32 bits");
    if (!population || !kernel_pos || (sides == 2 && !kernel_neg) || !isf || !isf_error || !fitness)
        return error(DEAC_E_INVALID, "null device pointer");
    if (!aligned(population, 16) || !aligned(kernel_pos, 16) || (sides == 2 && !aligned(kernel_neg, 16)))
        return error(DEAC_E_INVALID, "population and kernel matrices must be 16-byte aligned");
    if (!aligned(isf, 8) || !aligned(isf_error, 8) || !aligned(fitness, 8))
        return error(DEAC_E_INVALID, "isf, isf_error and fitness must be 8-byte aligned");

    if (P > DEAC_NOALLOC_SCRATCH_BYTES / sizeof(double) / Nt)
        return error(DEAC_E_INVALID,
                     "population_size %llu x number_of_timeslices %llu exceeds the static scratch of %llu bytes",
                     (unsigned long long)P, (unsigned long long)Nt, (unsigned long long)DEAC_NOALLOC_SCRATCH_BYTES);

    // contraction tile as the batch engine chooses it: a power-of-two number
    // of members times timeslices filling the CTA's chain pairs, and a staging
    // chunk that keeps two stages within 96 KB of shared memory
    const uint32_t S = (uint32_t)sides;
    const uint32_t pairs = deac::contract_pairs(S);
    uint32_t mt = 1;
    while (mt * 2 <= (P < pairs ? P : pairs)) mt *= 2;
    const uint32_t tt = pairs / mt;
    const uint64_t rows = (uint64_t)S * (mt + tt);
    uint64_t chunk = (96 * 1024 / 8) / (2 * rows) - 2;
    chunk = (chunk < 128 ? chunk : 128) & ~uint64_t(1);
    if (chunk < 8) chunk = 8;
    const uint64_t ctas = ((P + mt - 1) / mt) * ((Nt + tt - 1) / tt);
    const ScratchLayout lay = layout(P, Nt, ctas);
    if (lay.total > DEAC_NOALLOC_SCRATCH_BYTES)
        return error(DEAC_E_INVALID,
                     "population_size %llu x number_of_timeslices %llu needs %llu bytes of scratch; the static "
                     "scratch holds %llu bytes",
                     (unsigned long long)P, (unsigned long long)Nt, (unsigned long long)lay.total,
                     (unsigned long long)DEAC_NOALLOC_SCRATCH_BYTES);
    uint64_t smem = deac::stage_doubles(S, mt, tt, (uint32_t)chunk) * 2 * sizeof(double);
    if (smem < 4 * 1024 * sizeof(double)) smem = 4 * 1024 * sizeof(double);  // the finishing CTA's tree slots
    if (smem < deac::kContractMinSmemBytes) smem = deac::kContractMinSmemBytes;  // one CTA per SM

    // --- device
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || device < 0 || device >= n_dev) {
        cudaGetLastError();
        return error(DEAC_E_NODEVICE, "no CUDA device %d", device);
    }
    cudaDeviceProp prop;
    NOALLOC_TRY(cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10 || prop.minor != 3)
        return error(DEAC_E_NODEVICE, "device %d is sm_%d%d; this library is built for sm_103a (GB300)", device,
                     prop.major, prop.minor);
    int previous = 0;
    NOALLOC_TRY(cudaGetDevice(&previous));
    NOALLOC_TRY(cudaSetDevice(device));
    int rc = DEAC_OK;
    do {
        void* scratch = nullptr;
        if ((rc = scratch_address(device, &scratch))) break;
        cudaFuncAttributes fa;
        cudaError_t e = cudaFuncGetAttributes(&fa, deac::contract_kernel);
        if (e == cudaSuccess && (uint64_t)fa.maxDynamicSharedSizeBytes < smem)
            e = cudaFuncSetAttribute(deac::contract_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) {
            rc = error(DEAC_E_CUDA, "contract_kernel attributes: %s", cudaGetErrorString(e));
            break;
        }
        unsigned char* base = static_cast<unsigned char*>(scratch);
        deac::RunDev* run = reinterpret_cast<deac::RunDev*>(base);
        deac::Work* work = reinterpret_cast<deac::Work*>(base + lay.work);
        uint8_t* cur = base + lay.cur;

        deac::RunDev d{};
        d.P = (uint32_t)P;
        d.M = (uint32_t)M;
        d.Nt = (uint32_t)Nt;
        d.S = S;
        d.flags = 0;  // reduced chi^2 only: no moment terms
        d.contract_ctas = (uint32_t)ctas;
        d.member_tile = mt;
        d.tau_tile = tt;
        d.chunk = (uint32_t)chunk;
        d.N = 2;  // the pass's generation bookkeeping stays within the scratch descriptor
        d.stop = -HUGE_VAL;
        d.k_pos = kernel_pos;
        d.k_neg = sides == 2 ? kernel_neg : nullptr;
        d.isf = isf;
        d.err = isf_error;
        d.pop = const_cast<double*>(population);  // read only: buffer 0 of every member
        d.cur = cur;
        d.fit_old = fitness;
        d.model_isf = reinterpret_cast<double*>(base + lay.model_isf);
        // ii, ticket and done start at zero (value-initialised descriptor)

        cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
        const uint64_t items = ctas > P ? ctas : P;
        const uint32_t blocks = (uint32_t)((items + 255) / 256 < 1024 ? (items + 255) / 256 : 1024);
        noalloc_prepare_kernel<<<blocks, 256, 0, st>>>(d, run, work, (uint32_t)ctas, cur, (uint32_t)P);
        deac::contract_kernel<<<(uint32_t)ctas, deac::kContractThreads, smem, st>>>(run, work, deac::kModeInit);
        e = cudaGetLastError();
        if (e != cudaSuccess) rc = error(DEAC_E_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    } while (0);
    cudaSetDevice(previous);
    return rc;
}
