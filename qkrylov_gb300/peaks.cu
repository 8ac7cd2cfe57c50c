// Throughput probes for the roofline denominators the SpMV and Krylov kernels
// are measured against: FP64 and FP32 FMA rates, L2 and DRAM read bandwidth,
// and the rate of scattered 8-byte reads from shared memory and from
// L1-resident global memory (the access pattern of the SpMV's inner gathers).
//
//     nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o peaks peaks.cu && ./peaks
//
// (python -m qkrylov_gb300.timing --peaks builds and runs it.)  Prints one JSON
// line; every figure is the best of several CUDA-event timed launches.  Every
// index is masked into its buffer, so no probe reads out of bounds.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#define CK(x)                                                                              \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess) {                                                           \
            std::fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
            std::exit(1);                                                                  \
        }                                                                                  \
    } while (0)

constexpr int kChains = 8;

template <class T>
__global__ void fma_kernel(T* out, int iters, T b, T c) {
    T a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = (T)(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == (T)-1.2345) out[0] = s;  // keeps the chains live
}

// Reads `reps` times over n float4 (grid-stride), XOR-folding the bits.
__global__ void read_kernel(const float4* __restrict__ p, size_t n, int reps, unsigned* out) {
    unsigned acc = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int r = 0; r < reps; ++r)
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const float4 v = __ldcg(p + i);
            acc ^= __float_as_uint(v.x) ^ __float_as_uint(v.y) ^ __float_as_uint(v.z) ^ __float_as_uint(v.w);
        }
    if (acc == 0x12345678u) out[0] = acc;
}

// Scattered 8-byte reads: each thread follows `iters` pseudo-random indices into
// a table of `mask + 1` float2 (a power of two), from shared memory (SMEM) or
// from a per-CTA global region small enough to stay in L1.
template <bool SMEM>
__global__ void gather_kernel(const float2* __restrict__ g, unsigned mask, int iters, float* out) {
    extern __shared__ float2 tab[];
    if (SMEM) {
        for (unsigned i = threadIdx.x; i <= mask; i += blockDim.x) tab[i] = g[i];
        __syncthreads();
    }
    unsigned h = threadIdx.x * 2654435761u + blockIdx.x;
    float sx = 0.f, sy = 0.f;
    for (int i = 0; i < iters; ++i) {
        float2 v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const unsigned idx = (h + k * 0x9E3779B9u) & mask;
            v[k] = SMEM ? tab[idx] : __ldg(g + idx);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            sx += v[k].x;
            sy += v[k].y;
        }
        h = h * 1664525u + 1013904223u;
    }
    if (sx == -1.f && sy == -2.f) out[0] = sx;
}

struct Timer {
    cudaEvent_t a, b;
    Timer() {
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
    }
    template <class F>
    float best_ms(F f, int reps = 5) {
        f();
        CK(cudaDeviceSynchronize());
        float best = 1e30f;
        for (int r = 0; r < reps; ++r) {
            CK(cudaEventRecord(a));
            f();
            CK(cudaEventRecord(b));
            CK(cudaEventSynchronize(b));
            float ms;
            CK(cudaEventElapsedTime(&ms, a, b));
            if (ms < best) best = ms;
        }
        CK(cudaGetLastError());
        return best;
    }
};

int main() {
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, 0));
    const int sms = prop.multiProcessorCount;
    Timer t;
    double* d64;
    float* d32;
    unsigned* du;
    CK(cudaMalloc(&d64, 64));
    CK(cudaMalloc(&d32, 64));
    CK(cudaMalloc(&du, 64));

    // FMA rates: 8 independent chains per thread, 4 x 256-thread CTAs per SM
    const int fma_iters = 1 << 14;
    const int fgrid = sms * 8, fblk = 256;
    const double nfma = (double)fgrid * fblk * kChains * fma_iters;
    const float ms64 = t.best_ms([&] { fma_kernel<double><<<fgrid, fblk>>>(d64, fma_iters, 1.0000001, 1e-9); });
    const float ms32 = t.best_ms([&] { fma_kernel<float><<<fgrid, fblk>>>(d32, fma_iters, 1.0000001f, 1e-9f); });

    // L2: a 48 MiB buffer read 20 times after a warming pass; DRAM: 4 GiB read once
    const size_t l2_bytes = 48ull << 20, dram_bytes = 4ull << 30;
    float4 *bl2, *bdr;
    CK(cudaMalloc(&bl2, l2_bytes));
    CK(cudaMalloc(&bdr, dram_bytes));
    CK(cudaMemset(bl2, 1, l2_bytes));
    CK(cudaMemset(bdr, 1, dram_bytes));
    const int rgrid = sms * 4, rblk = 512, l2_reps = 20;
    const float ms_l2 = t.best_ms([&] { read_kernel<<<rgrid, rblk>>>(bl2, l2_bytes / 16, l2_reps, du); });
    const float ms_dr = t.best_ms([&] { read_kernel<<<rgrid, rblk>>>(bdr, dram_bytes / 16, 1, du); });

    // scattered 8-byte reads from a 32 KiB table (the size of one outer block's
    // FP32 slice at L=28): shared memory vs L1-resident global
    const unsigned tab_n = 4096;  // float2
    const int g_iters = 1 << 12, ggrid = sms * 4, gblk = 256;
    const float ms_gs = t.best_ms([&] {
        gather_kernel<true><<<ggrid, gblk, tab_n * sizeof(float2)>>>(reinterpret_cast<const float2*>(bl2), tab_n - 1,
                                                                    g_iters, d32);
    });
    const float ms_gl = t.best_ms([&] {
        gather_kernel<false><<<ggrid, gblk, 0>>>(reinterpret_cast<const float2*>(bl2), tab_n - 1, g_iters, d32);
    });
    const double ngather = (double)ggrid * gblk * g_iters * 4;

    int clk_khz = 0;
    CK(cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, 0));
    std::printf(
        "{\"gpu\": \"%s\", \"sms\": %d, \"clock_max_mhz\": %.0f, "
        "\"fp64_fma_tflops\": %.3f, \"fp32_fma_tflops\": %.3f, "
        "\"l2_read_gbs\": %.1f, \"dram_read_gbs\": %.1f, "
        "\"smem_gather8_g_per_s\": %.1f, \"l1_gather8_g_per_s\": %.1f, "
        "\"ms\": {\"fp64\": %.4f, \"fp32\": %.4f, \"l2\": %.4f, \"dram\": %.4f, \"smem_gather\": %.4f, "
        "\"l1_gather\": %.4f}}\n",
        prop.name, sms, clk_khz / 1e3, 2.0 * nfma / ms64 / 1e9, 2.0 * nfma / ms32 / 1e9,
        (double)l2_bytes * l2_reps / ms_l2 / 1e6, (double)dram_bytes / ms_dr / 1e6, ngather / ms_gs / 1e6,
        ngather / ms_gl / 1e6, ms64, ms32, ms_l2, ms_dr, ms_gs, ms_gl);
    CK(cudaFree(bl2));
    CK(cudaFree(bdr));
    return 0;
}
