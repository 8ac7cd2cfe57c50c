// Tall-skinny projections out[o k + j] = <V_j, W_o> (j < k <= 128, o < nw <= 4)
// of FP32 complex vectors on the tensor cores (tcgen05, TF32 inputs, FP32
// accumulation in tensor memory).
//
// This is the product the Davidson solver forms for its projected matrix and
// its Gram-Schmidt passes (src/solvers/davidson.cpp:143-150 and :213-223 do it
// as m(m+1)/2 and k*m separate dots).  As a real GEMM over the interleaved
// (re, im) components:
//     D[c][j] = sum_t A[c][t] B[j][t],   B[j] = V_j as (re, im, re, im, ...),
//     A[2o] = W_o as (re, im, ...),  A[2o+1] = (im, -re, im, -re, ...),
// so Re<V_j, W_o> = D[2o][j] and Im<V_j, W_o> = D[2o+1][j].  The MMA is
// M = 128 (A: the 8 rows of the right-hand vectors; the 16 eight-row groups of
// the operand all alias the same 1 KB atom, so rows 8..127 repeat rows 0..7
// and are never read), N = np = 16 ceil(k / 16) (B: the basis vectors, rows
// k..np-1 zero), K = 8 per instruction.
//
// Precision: each FP32 operand x is split into hi = x with its 13 low mantissa
// bits cleared (exact in TF32) and lo = x - hi (exact in FP32), and the MMA
// accumulates hi*hi + hi*lo + lo*hi (the "3xTF32" scheme; the dropped lo*lo is
// below 2^-22 of the product).  The FP32 accumulator in tensor memory holds at
// most kTcChunkStages * kTcKc * 32 real products per entry before it is read out
// (tcgen05.ld) and added to FP64 sums in shared memory, so the result carries
// the rounding of FP32 sums of about a thousand terms, against the FP64-level
// error of the compensated CUDA-core kernel (mdot32_multi_kernel).
//
// Data movement: every thread loads 16-byte chunks of V and W, splits them and
// stores hi and lo into the operands' 128-byte-swizzled K-major layout (row r's
// 16-byte chunk c at byte 128 (r mod 8) + 16 (c ^ (r mod 8)) of its 1 KB
// atom), then fences the shared-memory writes for the tensor core's async
// proxy.  Two stages alternate: while the tensor core works on one, the CTA
// fills the other.  One thread issues the MMAs and commits them to the stage's
// mbarrier.  Every wait is bounded by the global timer; a give-up is counted,
// the CTA waits once more (bounded) for its MMAs, frees its tensor memory and
// returns, and the host reports the call as failed.
#include "fast_common.cuh"

#include <algorithm>
#include <mutex>
#include <map>
#include <array>

namespace qkg {

namespace {

constexpr int kTcThreads = 256;
constexpr int kTcKc = 2;            // 128-byte K chunks (32 floats, 16 complex elements) per stage
constexpr int kTcChunkStages = 16;  // stages accumulated in tensor memory before the FP64 read-out
constexpr int kTcMaxK = 128;
constexpr uint32_t kAtom = 1024;    // 8 rows x 128 bytes
constexpr unsigned long long kTcWaitNs = 2000000000ull;
constexpr size_t kTcSmemLimit = 200 * 1024;

__device__ unsigned int g_tc_errors;

__device__ __forceinline__ unsigned long long tc_now() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool tc_test(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __noinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
    const unsigned long long t0 = tc_now();
    while (!tc_test(bar, parity))
        if (tc_now() - t0 > kTcWaitNs) return false;
    return true;
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms of
// 1 KB (stride byte offset sbo between eight-row groups; 0 aliases them all).
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)(16u >> 4) << 16;         // leading byte offset (not used by swizzled K-major)
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;                  // descriptor version
    d |= (uint64_t)2 << 61;                  // 128-byte swizzle
    return d;
}
// Instruction descriptor: D FP32, A and B TF32, both K-major, M = 128, N = np.
__device__ __forceinline__ uint32_t tc_idesc(uint32_t np) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((np >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }
__device__ __forceinline__ float4 hi4(float4 v) { return make_float4(tf32_hi(v.x), tf32_hi(v.y), tf32_hi(v.z), tf32_hi(v.w)); }
__device__ __forceinline__ float4 lo4(float4 v, float4 h) { return make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w); }

// Byte offset of 16-byte chunk c (0..7) of row r in a K-major 128-byte-swizzled operand.
__device__ __forceinline__ uint32_t sw_off(uint32_t r, uint32_t c) {
    return (r >> 3) * kAtom + (r & 7u) * 128u + ((c ^ (r & 7u)) << 4);
}

// 16 bytes of a complex FP32 vector from element e on (two elements), zero past n.
__device__ __forceinline__ float4 load2(const float2* __restrict__ p, uint64_t e, uint64_t n) {
    if (e + 1 < n) return __ldg(reinterpret_cast<const float4*>(p + e));
    if (e < n) {
        const float2 a = __ldg(p + e);
        return make_float4(a.x, a.y, 0.f, 0.f);
    }
    return make_float4(0.f, 0.f, 0.f, 0.f);
}

// Stage layout (bytes from the 1 KB-aligned stage base), per K chunk q < kTcKc:
//   A_hi[q] 1 KB, A_lo[q] 1 KB, then B_hi[q] np*128, B_lo[q] np*128.
struct StageMap {
    uint32_t bsz;  // np * 128
    __host__ __device__ uint32_t a_hi(int q) const { return (uint32_t)q * 2u * kAtom; }
    __host__ __device__ uint32_t a_lo(int q) const { return (uint32_t)q * 2u * kAtom + kAtom; }
    __host__ __device__ uint32_t b_hi(int q) const { return (uint32_t)kTcKc * 2u * kAtom + (uint32_t)q * 2u * bsz; }
    __host__ __device__ uint32_t b_lo(int q) const { return (uint32_t)kTcKc * 2u * kAtom + (uint32_t)q * 2u * bsz + bsz; }
    __host__ __device__ uint32_t bytes() const { return (uint32_t)kTcKc * 2u * (kAtom + bsz); }
};

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

// LPT: B chunks one thread loads per stage (16 k / 256 rounded up: 2, 4 or 8).
template <int NW, int LPT>
__global__ void __launch_bounds__(kTcThreads) mdot_tc_kernel(const float2* const* __restrict__ V, int k,
                                                             const float2* const* __restrict__ W, uint64_t n,
                                                             uint32_t np, uint32_t tcols,
                                                             double2* __restrict__ part, int stride,
                                                             unsigned int* __restrict__ fail) {
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    // 1 KB alignment for the swizzle atoms
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023u) & ~(uintptr_t)1023u);
    StageMap sm;
    sm.bsz = np * 128u;
    const uint32_t sbytes = (sm.bytes() + 1023u) & ~1023u;
    unsigned char* stage[2] = {base, base + sbytes};
    double* acc = reinterpret_cast<double*>(base + 2 * sbytes);  // [2 NW][np] FP64 sums
    __shared__ unsigned long long s_bar[2];
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail;

    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const uint32_t bar[2] = {(uint32_t)__cvta_generic_to_shared(&s_bar[0]),
                             (uint32_t)__cvta_generic_to_shared(&s_bar[1])};
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(&s_tmem)),
                     "r"(tcols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar[0]) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar[1]) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
    }
    // zero both stages (rows of B at and beyond k, rows of A beyond 2 NW stay zero) and the FP64 sums
    for (uint32_t i = tid; i < 2 * sbytes / 16; i += kTcThreads)
        reinterpret_cast<float4*>(base)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint32_t i = tid; i < 2u * NW * np; i += kTcThreads) acc[i] = 0.0;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s_tmem;

    // Stages are dealt out round robin (stage s to CTA s mod gridDim.x), so the
    // grid sweeps every vector front to back together: the pages in use at once
    // stay few (a contiguous range per CTA touches a page per CTA and vector).
    const uint64_t total_stages = (n + 16ull * kTcKc - 1) / (16ull * kTcKc);
    const uint64_t g = gridDim.x;
    const uint32_t n_it = blockIdx.x < total_stages ? (uint32_t)((total_stages - blockIdx.x + g - 1) / g) : 0u;
    const uint32_t idesc = tc_idesc(np);
    bool ok = true;  // uniform: every thread reads s_fail after a barrier
    uint32_t chunk_fill = 0;
    uint32_t commits[2] = {0u, 0u};  // thread 0: MMA commits per stage

    const uint32_t nbj = (uint32_t)k * 8u * kTcKc;  // 16-byte chunks of B per stage
    const bool has_a = tid < (uint32_t)NW * 8u * kTcKc;
    // This thread's loads of one stage (B: rows j < k, chunk c of K chunk q; A:
    // the right-hand vectors).  The next stage's loads are issued before this
    // stage waits and synchronises, so a DRAM round trip overlaps each stage.
    float4 vb[LPT], wa = make_float4(0.f, 0.f, 0.f, 0.f);
    auto load_stage = [&](uint64_t st, float4* out_b, float4& out_a) {
        const uint64_t f0 = st * 16ull * kTcKc;
#pragma unroll
        for (int u = 0; u < LPT; ++u) {
            const uint32_t i = tid + (uint32_t)u * kTcThreads;
            if (i < nbj) {
                const uint32_t j = i / (8u * kTcKc), rem = i % (8u * kTcKc);
                out_b[u] = load2(V[j], f0 + 16ull * (rem >> 3) + 2ull * (rem & 7u), n);
            }
        }
        if (has_a) {
            const uint32_t o = tid / (8u * kTcKc), rem = tid % (8u * kTcKc);
            out_a = load2(W[o], f0 + 16ull * (rem >> 3) + 2ull * (rem & 7u), n);
        }
    };
    if (n_it > 0) load_stage(blockIdx.x, vb, wa);
    for (uint32_t it = 0; it < n_it && ok; ++it) {
        const uint32_t b = it & 1u;
        unsigned char* sb = stage[b];
        float4 nb[LPT], na = make_float4(0.f, 0.f, 0.f, 0.f);
        if (it + 1 < n_it) load_stage(blockIdx.x + (uint64_t)(it + 1) * g, nb, na);
        // the MMAs that read this stage two iterations ago are complete
        if (it >= 2 && !tc_wait(bar[b], ((it - 2) >> 1) & 1u)) {
            if (lane == 0) {
                atomicAdd(&g_tc_errors, 1u);
                atomicAdd(fail, 1u);
            }
            s_fail = 1;
        }
#pragma unroll
        for (int u = 0; u < LPT; ++u) {
            const uint32_t i = tid + (uint32_t)u * kTcThreads;
            if (i < nbj) {
                const uint32_t j = i / (8u * kTcKc), rem = i % (8u * kTcKc), q = rem >> 3, c = rem & 7u;
                const float4 h = hi4(vb[u]);
                *reinterpret_cast<float4*>(sb + sm.b_hi(q) + sw_off(j, c)) = h;
                *reinterpret_cast<float4*>(sb + sm.b_lo(q) + sw_off(j, c)) = lo4(vb[u], h);
            }
        }
        // A: rows 2o (W_o) and 2o + 1 (W_o rotated)
        if (has_a) {
            const uint32_t o = tid / (8u * kTcKc), rem = tid % (8u * kTcKc), q = rem >> 3, c = rem & 7u;
            const float4 w = wa;
            const float4 wr = make_float4(w.y, -w.x, w.w, -w.z);
            const float4 h = hi4(w), hr = hi4(wr);
            *reinterpret_cast<float4*>(sb + sm.a_hi(q) + sw_off(2 * o, c)) = h;
            *reinterpret_cast<float4*>(sb + sm.a_lo(q) + sw_off(2 * o, c)) = lo4(w, h);
            *reinterpret_cast<float4*>(sb + sm.a_hi(q) + sw_off(2 * o + 1, c)) = hr;
            *reinterpret_cast<float4*>(sb + sm.a_lo(q) + sw_off(2 * o + 1, c)) = lo4(wr, hr);
        }
#pragma unroll
        for (int u = 0; u < LPT; ++u) vb[u] = nb[u];
        wa = na;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        ok = s_fail == 0;
        if (!ok) break;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = (uint32_t)__cvta_generic_to_shared(sb);
#pragma unroll
            for (int q = 0; q < kTcKc; ++q) {
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {  // K = 8 TF32 (32 bytes) per instruction
                    const uint32_t ko = 32u * kk;
                    const uint64_t ah = tc_desc(sa + sm.a_hi(q) + ko, 0u), al = tc_desc(sa + sm.a_lo(q) + ko, 0u);
                    const uint64_t bh = tc_desc(sa + sm.b_hi(q) + ko, kAtom), bl = tc_desc(sa + sm.b_lo(q) + ko, kAtom);
                    const uint32_t first = (chunk_fill == 0 && q == 0 && kk == 0) ? 0u : 1u;
                    tc_mma(tmem, ah, bh, idesc, first);
                    tc_mma(tmem, ah, bl, idesc, 1u);
                    tc_mma(tmem, al, bh, idesc, 1u);
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar[b])
                         : "memory");
            ++commits[b];
        }
        ++chunk_fill;
        // read the accumulator out every kTcChunkStages stages and at the end
        if (chunk_fill == (uint32_t)kTcChunkStages || it + 1 == n_it) {
            if (!tc_wait(bar[b], (it >> 1) & 1u)) {
                if (lane == 0) {
                atomicAdd(&g_tc_errors, 1u);
                atomicAdd(fail, 1u);
            }
                s_fail = 1;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (warp == 0) {
                for (uint32_t c0 = 0; c0 < np; c0 += 8) {
                    uint32_t r[8];
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                          "=r"(r[7])
                        : "r"(tmem + c0)
                        : "memory");
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (lane < 2u * NW)
#pragma unroll
                        for (int t = 0; t < 8; ++t) acc[lane * np + c0 + t] += (double)__uint_as_float(r[t]);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            ok = s_fail == 0;
            chunk_fill = 0;
        }
    }
    if (!ok && tid == 0) {
        // MMAs may still be running: wait (bounded) for the last commit on each stage
        for (uint32_t b = 0; b < 2; ++b)
            if (commits[b]) tc_wait(bar[b], (commits[b] - 1u) & 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcols) : "memory");
    }
    // per-CTA partials of <V_j, W_o>
    for (uint32_t i = tid; i < (uint32_t)k * NW; i += kTcThreads) {
        const uint32_t j = i / NW, o = i % NW;
        part[(size_t)i * stride + blockIdx.x] =
            ok ? make_double2(acc[(2 * o) * np + j], acc[(2 * o + 1) * np + j]) : make_double2(0.0, 0.0);
    }
}

__global__ void tc_finish_kernel(const double2* __restrict__ part, int nparts, int stride, double2* __restrict__ out) {
    double r = 0.0, i = 0.0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) {
        const double2 v = part[(size_t)blockIdx.x * stride + b];
        r += v.x;
        i += v.y;
    }
    __shared__ double sr[32], si[32];
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_down_sync(0xffffffffu, r, o);
        i += __shfl_down_sync(0xffffffffu, i, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sr[wid] = r;
        si[wid] = i;
    }
    __syncthreads();
    if (wid == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sr[lane] : 0.0;
        i = lane < (int)(blockDim.x >> 5) ? si[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            r += __shfl_down_sync(0xffffffffu, r, o);
            i += __shfl_down_sync(0xffffffffu, i, o);
        }
        if (lane == 0) out[blockIdx.x] = make_double2(r, i);
    }
}

template <int LPT>
void allow_tc(int lim) {
    QKG_CUDA(cudaFuncSetAttribute(mdot_tc_kernel<1, LPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    QKG_CUDA(cudaFuncSetAttribute(mdot_tc_kernel<2, LPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    QKG_CUDA(cudaFuncSetAttribute(mdot_tc_kernel<3, LPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    QKG_CUDA(cudaFuncSetAttribute(mdot_tc_kernel<4, LPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
}
template <int LPT>
void launch_tc(int nw, int g, size_t smem, cudaStream_t s, const float2* const* V, int k, float2* const* dw, uint64_t n,
               uint32_t np, uint32_t tcols, double2* part, unsigned int* fail) {
    switch (nw) {
        case 1: mdot_tc_kernel<1, LPT><<<g, kTcThreads, smem, s>>>(V, k, dw, n, np, tcols, part, g, fail); break;
        case 2: mdot_tc_kernel<2, LPT><<<g, kTcThreads, smem, s>>>(V, k, dw, n, np, tcols, part, g, fail); break;
        case 3: mdot_tc_kernel<3, LPT><<<g, kTcThreads, smem, s>>>(V, k, dw, n, np, tcols, part, g, fail); break;
        default: mdot_tc_kernel<4, LPT><<<g, kTcThreads, smem, s>>>(V, k, dw, n, np, tcols, part, g, fail); break;
    }
}

// CTAs of the kernel for (nw, lpt) resident on the whole GPU at this shared
// memory and tensor-memory width, from the kernel's registers, the SM's shared
// memory (1 KB reserved per CTA) and the 512 tensor-memory columns of an SM
// (the caller caches it).
int tc_resident(int dev, int nw, int lpt, size_t smem, uint32_t tcols) {
    int sms = 0, smem_sm = 0;
    QKG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    QKG_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    const void* f = nullptr;
    auto pick = [&](auto k1, auto k2, auto k3, auto k4) {
        f = nw == 1 ? (const void*)k1 : nw == 2 ? (const void*)k2 : nw == 3 ? (const void*)k3 : (const void*)k4;
    };
    if (lpt == 2) pick(mdot_tc_kernel<1, 2>, mdot_tc_kernel<2, 2>, mdot_tc_kernel<3, 2>, mdot_tc_kernel<4, 2>);
    else if (lpt == 4) pick(mdot_tc_kernel<1, 4>, mdot_tc_kernel<2, 4>, mdot_tc_kernel<3, 4>, mdot_tc_kernel<4, 4>);
    else pick(mdot_tc_kernel<1, 8>, mdot_tc_kernel<2, 8>, mdot_tc_kernel<3, 8>, mdot_tc_kernel<4, 8>);
    cudaFuncAttributes fa{};
    QKG_CUDA(cudaFuncGetAttributes(&fa, f));
    const int warp_regs = ((std::max(fa.numRegs, 1) * 32 + 255) / 256) * 256;  // allocated per warp in 256s
    const int by_regs = 65536 / (warp_regs * (kTcThreads / 32));
    const int by_smem = smem_sm / (int)(smem + fa.sharedSizeBytes + 1024);
    const int by_tmem = 512 / (int)tcols;
    const int by_threads = 2048 / kTcThreads;
    const int per = std::max(1, std::min(std::min(by_regs, by_smem), std::min(by_tmem, by_threads)));
    return per * std::max(1, sms);
}

}  // namespace

uint32_t tc_wait_timeouts() {
    uint32_t c = 0;
    QKG_CUDA(cudaMemcpyFromSymbol(&c, g_tc_errors, sizeof(c)));
    return c;
}

size_t mdot_tc_smem(int k, int nw) {
    const uint32_t np = (uint32_t)(((k + 15) / 16) * 16);
    const uint32_t stage = ((uint32_t)kTcKc * 2u * (kAtom + np * 128u) + 1023u) & ~1023u;
    return 1024 + 2 * (size_t)stage + (size_t)2 * nw * np * sizeof(double);
}

bool mdot_tc_supported(int k, int nw) {
    return k >= 1 && k <= kTcMaxK && nw >= 1 && nw <= 4 && mdot_tc_smem(k, nw) <= kTcSmemLimit;
}

void mdot_multi_f32_tc(const float2* const* V, int k, float2* const* W, int nw, uint64_t n, std::complex<double>* out,
                       Workspace& ws, cudaStream_t s) {
    if (k <= 0 || nw <= 0) return;
    QKG_REQUIRE(mdot_tc_supported(k, nw), "tensor-core projections: 1 <= k <= 128 basis vectors, 1..4 right-hand vectors");
    const uint32_t np = (uint32_t)(((k + 15) / 16) * 16);
    uint32_t tcols = 32;
    while (tcols < np) tcols <<= 1;
    const size_t smem = mdot_tc_smem(k, nw);
    const int lpt = k <= 32 ? 2 : k <= 64 ? 4 : 8;
    int dev = 0;
    QKG_CUDA(cudaGetDevice(&dev));
    int resident = 0;
    {
        // per device: the shared-memory opt-in once, and the resident CTAs per
        // (nw, k rounded up to 16)
        static std::mutex mu;
        static std::map<int, std::array<int, 33>> cache;  // [0]: opt-in done; [1 + 8 (nw-1) + np/16 - 1]
        std::lock_guard<std::mutex> lk(mu);
        auto& c = cache[dev];
        if (!c[0]) {
            const int lim = (int)kTcSmemLimit;
            allow_tc<2>(lim);
            allow_tc<4>(lim);
            allow_tc<8>(lim);
            c[0] = 1;
        }
        int& r = c[1 + 8 * (nw - 1) + (int)(np / 16) - 1];
        if (!r) r = tc_resident(dev, nw, lpt, smem, tcols);
        resident = r;
    }
    // Host-side scratch in the pinned result slots: the W pointer table (copied in
    // without staging) and the failure count of this call.
    double2* hslot = reinterpret_cast<double2*>(ws.host);
    double2* dslot = ws.result.as<double2>();
    float2** hw = reinterpret_cast<float2**>(hslot + 4096 - 8);
    for (int o = 0; o < nw; ++o) hw[o] = W[o];
    float2** dw = reinterpret_cast<float2**>(dslot + 4096 - 8);
    unsigned int* dfail = reinterpret_cast<unsigned int*>(dslot + 4096 - 16);
    unsigned int* hfail = reinterpret_cast<unsigned int*>(hslot + 4096 - 16);
    QKG_CUDA(cudaMemcpyAsync(dw, hw, (size_t)nw * sizeof(float2*), cudaMemcpyHostToDevice, s));
    QKG_CUDA(cudaMemsetAsync(dfail, 0, sizeof(unsigned int), s));
    const uint64_t total = (n + 16ull * kTcKc - 1) / (16ull * kTcKc);
    // one wave: as many CTAs as can be resident at once
    const uint64_t want =
        std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)resident, ws.cap_partials / ((size_t)k * nw)));
    const int g = (int)std::max<uint64_t>(1, std::min<uint64_t>(want, total));
    QKG_REQUIRE((size_t)g * k * nw <= ws.cap_partials, "tensor-core projections: workspace too small");
    double2* part = ws.partial.as<double2>();
    if (lpt == 2) launch_tc<2>(nw, g, smem, s, V, k, dw, n, np, tcols, part, dfail);
    else if (lpt == 4) launch_tc<4>(nw, g, smem, s, V, k, dw, n, np, tcols, part, dfail);
    else launch_tc<8>(nw, g, smem, s, V, k, dw, n, np, tcols, part, dfail);
    QKG_LAUNCHED();
    tc_finish_kernel<<<k * nw, 256, 0, s>>>(part, g, g, ws.result.as<double2>());
    QKG_LAUNCHED();
    QKG_CUDA(cudaMemcpyAsync(ws.host, ws.result.p, (size_t)k * nw * sizeof(double2), cudaMemcpyDeviceToHost, s));
    QKG_CUDA(cudaMemcpyAsync(hfail, dfail, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    QKG_CUDA(cudaStreamSynchronize(s));
    if (*hfail != 0) throw Error(DEVICE_TIMEOUT, "tensor-core projection: a bounded wait gave up");
    const double2* r = reinterpret_cast<const double2*>(ws.host);
    for (int j = 0; j < k; ++j)
        for (int o = 0; o < nw; ++o) out[(size_t)o * k + j] = {r[(size_t)j * nw + o].x, r[(size_t)j * nw + o].y};
}

}  // namespace qkg
