// Device-vector dot product that allocates nothing.
//
// qkrylov_vector_dot_device_f64 reduces into scratch that the library
// allocates with cudaMalloc on first use.  Some callers cannot let a library
// allocate device memory: applications that reserve the GPU's memory up front
// in their own pool and forbid allocations outside it (a serving process that
// takes nearly all HBM at start-up, or one that runs under a hard memory cap),
// and latency-critical loops that cannot afford cudaMalloc's implicit device
// synchronisation.  This variant keeps its scratch in a fixed array compiled
// into the library instead.
//
// Limits and sharing:
//  * the scratch is kNoAllocMaxBlocks partial sums plus one result slot,
//    (16384 + 1) x 16 bytes = 256 KiB + 16 B, held by every GPU that loads the
//    library until the process exits;
//  * one block reduces kNoAllocPerBlock = 8192 elements, so n is limited to
//    8192 * 16384 = 134,217,728 complex elements; larger n is rejected;
//  * every call shares the one array: calls that overlap on the GPU (from
//    different threads or on different streams of one GPU) race and must be
//    serialised by the caller;
//  * nothing in the array has to start at zero: each call writes every
//    partial slot it reads and the result slot before reading them.
//
// The first call on a GPU looks up the array's device address there
// (cudaGetSymbolAddress, with that GPU current), caches it, and makes sure both
// kernels are loaded on that GPU.  With CUDA's lazy module loading that first
// call is when the array and the kernels' code take their device memory, so a
// call with n = 0 serves as the warm-up a caller makes before it reserves the
// GPU's memory for itself.  The call waits for its stream (it reads the result
// back to the host), so it cannot be used inside a stream capture.
#include "../../include/qkrylov_c_api.h"
#include "qkg.hpp"

#include <mutex>
#include <string>

namespace {

constexpr int kNoAllocThreads = 256;
constexpr uint64_t kNoAllocPerBlock = 8192;
constexpr int kNoAllocMaxBlocks = 16384;
constexpr uint64_t kNoAllocMaxElements = kNoAllocPerBlock * (uint64_t)kNoAllocMaxBlocks;
constexpr int kMaxDevices = 256;

// Partial sums in [0, kNoAllocMaxBlocks), the result in [kNoAllocMaxBlocks].
__device__ __align__(256) double2 g_noalloc_dot_scratch[kNoAllocMaxBlocks + 1];

__device__ __forceinline__ double2 na_block_sum(double re, double im) {
    __shared__ double2 sh[kNoAllocThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_down_sync(0xffffffffu, re, o);
        im += __shfl_down_sync(0xffffffffu, im, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = make_double2(re, im);
    __syncthreads();
    double2 v = make_double2(0.0, 0.0);
    if (wid == 0) {
        v = lane < (int)(blockDim.x >> 5) ? sh[lane] : make_double2(0.0, 0.0);
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_down_sync(0xffffffffu, v.x, o);
            v.y += __shfl_down_sync(0xffffffffu, v.y, o);
        }
    }
    return v;
}

// Block b reduces conj(x_i) y_i over [b * 8192, min((b + 1) * 8192, n)).
__global__ void __launch_bounds__(kNoAllocThreads) na_partial_kernel(const double2* __restrict__ x,
                                                                     const double2* __restrict__ y, uint64_t n,
                                                                     double2* __restrict__ scratch) {
    const uint64_t base = (uint64_t)blockIdx.x * kNoAllocPerBlock;
    const uint64_t end = base + kNoAllocPerBlock < n ? base + kNoAllocPerBlock : n;
    double re = 0.0, im = 0.0;
    for (uint64_t i = base + threadIdx.x; i < end; i += blockDim.x) {
        const double2 a = x[i], b = y[i];
        re = fma(a.x, b.x, re);
        re = fma(a.y, b.y, re);
        im = fma(a.x, b.y, im);
        im = fma(-a.y, b.x, im);
    }
    const double2 s = na_block_sum(re, im);
    if (threadIdx.x == 0) scratch[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kNoAllocThreads) na_finish_kernel(double2* __restrict__ scratch, int nblocks) {
    double re = 0.0, im = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        re += scratch[i].x;
        im += scratch[i].y;
    }
    const double2 s = na_block_sum(re, im);
    if (threadIdx.x == 0) scratch[kNoAllocMaxBlocks] = s;
}

std::mutex g_na_mu;
double2* g_na_addr[kMaxDevices] = {};

// Device address of the scratch array on the current GPU (looked up once per
// GPU, when both kernels are also loaded there).
double2* na_scratch_on_current_device() {
    int dev = -1;
    QKG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw qkg::Error(qkg::INVALID_ARG, "device id out of range");
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_dot_scratch);
        if (e != cudaSuccess || !p)
            throw qkg::Error(qkg::CUDA_ERR, std::string("cudaGetSymbolAddress(g_noalloc_dot_scratch): ") +
                                                 cudaGetErrorString(e));
        cudaFuncAttributes fa;
        QKG_CUDA(cudaFuncGetAttributes(&fa, na_partial_kernel));
        QKG_CUDA(cudaFuncGetAttributes(&fa, na_finish_kernel));
        g_na_addr[dev] = static_cast<double2*>(p);
    }
    return g_na_addr[dev];
}

}  // namespace

extern "C" int qkrylov_vector_dot_device_f64_noalloc(const void* d_x, const void* d_y, uint64_t n, double* result,
                                                     void* stream) {
    if (!result || (n && (!d_x || !d_y))) return QKRYLOV_ERROR_INVALID_ARG;
    // whole complex FP64 elements (16-byte loads): a pointer off that grid is refused
    if (n && ((reinterpret_cast<uintptr_t>(d_x) | reinterpret_cast<uintptr_t>(d_y)) & 15u)) return QKRYLOV_ERROR_INVALID_ARG;
    if (n > kNoAllocMaxElements) {
        qkg::set_last_error("qkrylov_vector_dot_device_f64_noalloc: n = " + std::to_string(n) +
                            " exceeds the fixed scratch limit of " + std::to_string(kNoAllocMaxElements) +
                            " complex elements");
        return QKRYLOV_ERROR_INVALID_ARG;
    }
    try {
        qkg::set_last_error("");
        result[0] = result[1] = 0.0;
        double2* scratch = na_scratch_on_current_device();  // n = 0: the warm-up only
        if (!n) return QKRYLOV_SUCCESS;
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const int nblocks = (int)((n + kNoAllocPerBlock - 1) / kNoAllocPerBlock);
        na_partial_kernel<<<nblocks, kNoAllocThreads, 0, s>>>(static_cast<const double2*>(d_x),
                                                              static_cast<const double2*>(d_y), n, scratch);
        QKG_LAUNCHED();
        na_finish_kernel<<<1, kNoAllocThreads, 0, s>>>(scratch, nblocks);
        QKG_LAUNCHED();
        double2 r;
        QKG_CUDA(cudaMemcpyAsync(&r, scratch + kNoAllocMaxBlocks, sizeof(double2), cudaMemcpyDeviceToHost, s));
        QKG_CUDA(cudaStreamSynchronize(s));
        result[0] = r.x;
        result[1] = r.y;
        return QKRYLOV_SUCCESS;
    } catch (const qkg::Error& e) {
        qkg::set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        qkg::set_last_error(e.what());
        return QKRYLOV_ERROR_EXCEPTION;
    }
}
