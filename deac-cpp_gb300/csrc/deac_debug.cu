// deac_debug.cu -- test aids (include/deac_gb300_debug.h), built into their
// own library (lib/libdeac_gb300_debug.so), not into the engine's.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "deac_chain.cuh"
#include "deac_gb300.h"
#include "deac_gb300_debug.h"
#include "deac_kernels.cuh"

namespace deac {
namespace {
thread_local std::string g_debug_error;
int set_error(int code, const char* msg) {
    g_debug_error = msg;
    return code;
}
}  // namespace
}  // namespace deac

extern "C" const char* deac_debug_last_error(void) { return deac::g_debug_error.c_str(); }

namespace {

// warps 0-7: the exact parallel chain in the configuration of trial_kernel;
// warp 8, lane 0: the plain chain
__global__ void fma_chains_kernel(const double* x, const double* w, uint64_t n, const double* start, double* fast,
                                  double* plain) {
    __shared__ deac::ChainScratch sc;
    const uint64_t c = blockIdx.x;
    const double* xc = x + c * n;
    const double* wc = w + c * n;
    if (threadIdx.x < 32 * deac::kChainWarps) {
        const double r = deac::group_fma_chain<deac::kChainWarps, deac::kChainSteps>(xc, wc, (uint32_t)n, start[c],
                                                                                      0, 1, sc);
        if (threadIdx.x == 0) fast[c] = r;
    } else if (threadIdx.x == 32 * deac::kChainWarps) {
        double acc = start[c];
        for (uint64_t k = 0; k < n; ++k) acc = fma(xc[k], wc[k], acc);
        plain[c] = acc;
    }
}

int cuda_fail(cudaError_t e, const char* what) {
    char buf[256];
    std::snprintf(buf, sizeof buf, "%s failed: %s", what, cudaGetErrorString(e));
    return deac::set_error(DEAC_E_CUDA, buf);
}

}  // namespace

extern "C" int deac_debug_fma_chains(const double* x, const double* w, uint64_t n, const double* start,
                                     uint32_t count, double* fast_out, double* plain_out) {
    if (!x || !w || !start || !fast_out || !plain_out || n == 0 || n > 0xFFFFFFFFull || count == 0)
        return deac::set_error(DEAC_E_INVALID, "bad arguments");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return deac::set_error(DEAC_E_NODEVICE, "no CUDA device 0");
    }
    double *dx = nullptr, *dw = nullptr, *ds = nullptr, *df = nullptr, *dp = nullptr;
    const size_t bytes = (size_t)count * n * sizeof(double);
    cudaError_t e = cudaSuccess;
    int rc = DEAC_OK;
    do {
        if ((e = cudaMalloc(&dx, bytes)) || (e = cudaMalloc(&dw, bytes)) ||
            (e = cudaMalloc(&ds, count * sizeof(double))) || (e = cudaMalloc(&df, count * sizeof(double))) ||
            (e = cudaMalloc(&dp, count * sizeof(double)))) {
            rc = cuda_fail(e, "cudaMalloc");
            break;
        }
        if ((e = cudaMemcpy(dx, x, bytes, cudaMemcpyHostToDevice)) ||
            (e = cudaMemcpy(dw, w, bytes, cudaMemcpyHostToDevice)) ||
            (e = cudaMemcpy(ds, start, count * sizeof(double), cudaMemcpyHostToDevice))) {
            rc = cuda_fail(e, "cudaMemcpy");
            break;
        }
        fma_chains_kernel<<<count, 32 * deac::kChainWarps + 32>>>(dx, dw, n, ds, df, dp);
        if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize())) {
            rc = cuda_fail(e, "fma_chains_kernel");
            break;
        }
        if ((e = cudaMemcpy(fast_out, df, count * sizeof(double), cudaMemcpyDeviceToHost)) ||
            (e = cudaMemcpy(plain_out, dp, count * sizeof(double), cudaMemcpyDeviceToHost))) {
            rc = cuda_fail(e, "cudaMemcpy");
            break;
        }
    } while (0);
    cudaFree(dx);
    cudaFree(dw);
    cudaFree(ds);
    cudaFree(df);
    cudaFree(dp);
    return rc;
}
