// Krylov vector algebra on device-resident complex vectors.
//
// The reference runs every BLAS-1 call as its own Kokkos kernel and returns
// each reduction to the host (include/qkrylov/linalg/vector_ops.hpp:14-137);
// its full reorthogonalisation is k sequential dot+axpy pairs
// (src/solvers/lanczos.cpp:148-151).  Here the Lanczos three-term update and
// the norm are one fused pass, the projections against k stored vectors are
// one pass over w (classical Gram-Schmidt), and reductions finish on the
// device with one host read.
//
// FP32 reductions use error-free transformations (Ogita, Rump & Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005), Dot2):
// each product a*b is split exactly into p + e with one fma, p is added with
// Knuth's TwoSum and the rounding errors are carried in a second float, so a
// thread's partial sum is as accurate as if computed in twice the working
// precision.  Partials are then combined in FP64.  This keeps the reductions
// off GB300's low-rate FP64 pipe.
#include "fast_common.cuh"

#include <algorithm>
#include <atomic>

namespace qkg {

namespace {
constexpr int kThreads = 256;

inline int stream_grid(uint64_t n) {
    const uint64_t g = (n + kThreads - 1) / kThreads;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, 152ull * 8));
}

// ---- compensated FP32 accumulation ----------------------------------------
struct FF {  // unevaluated sum hi + lo
    float hi, lo;
};
__device__ __forceinline__ void ff_add_prod(FF& acc, float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);  // exact: a*b = p + e
    const float t = acc.hi + p;      // TwoSum(acc.hi, p)
    const float z = t - acc.hi;
    const float err = (acc.hi - (t - z)) + (p - z);
    acc.hi = t;
    acc.lo += err + e;
}
__device__ __forceinline__ double ff_value(const FF& a) { return (double)a.hi + (double)a.lo; }
// a += b in float-float arithmetic
__device__ __forceinline__ void ff_add_ff(FF& a, FF b) {
    const float t = a.hi + b.hi;
    const float z = t - a.hi;
    a.lo += ((a.hi - (t - z)) + (b.hi - z)) + b.lo;
    a.hi = t;
}
// Block sum of a complex float-float value, all in FP32 arithmetic (GB300's
// FP64 pipe is narrow: a double reduction per output and CTA costs more than
// the pass it finishes); thread 0 writes the result, rounded to double, to *dst.
__device__ __forceinline__ void block_sum_cff(FF re, FF im, double2* dst) {
    __shared__ FF sre[32], sim[32];
    for (int o = 16; o > 0; o >>= 1) {
        FF r2{__shfl_down_sync(0xffffffffu, re.hi, o), __shfl_down_sync(0xffffffffu, re.lo, o)};
        FF i2{__shfl_down_sync(0xffffffffu, im.hi, o), __shfl_down_sync(0xffffffffu, im.lo, o)};
        ff_add_ff(re, r2);
        ff_add_ff(im, i2);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();  // the arrays may still be read from the previous call
    if (lane == 0) {
        sre[wid] = re;
        sim[wid] = im;
    }
    __syncthreads();
    if (wid == 0) {
        const bool on = threadIdx.x < (blockDim.x >> 5);
        re = on ? sre[lane] : FF{0.f, 0.f};
        im = on ? sim[lane] : FF{0.f, 0.f};
        for (int o = 16; o > 0; o >>= 1) {
            FF r2{__shfl_down_sync(0xffffffffu, re.hi, o), __shfl_down_sync(0xffffffffu, re.lo, o)};
            FF i2{__shfl_down_sync(0xffffffffu, im.hi, o), __shfl_down_sync(0xffffffffu, im.lo, o)};
            ff_add_ff(re, r2);
            ff_add_ff(im, i2);
        }
    }
    if (threadIdx.x == 0) *dst = make_double2(ff_value(re), ff_value(im));
}

// ---- block reduction of double pairs ---------------------------------------
__device__ __forceinline__ double2 warp_sum(double2 v) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, o);
        v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    return v;
}
__device__ __forceinline__ double2 block_sum(double2 v) {
    __shared__ double2 sh[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = (threadIdx.x < (blockDim.x >> 5)) ? sh[lane] : make_double2(0.0, 0.0);
    if (wid == 0) v = warp_sum(v);
    return v;
}

// dot: sum conj(x_i) y_i
__global__ void dot64_kernel(const double2* __restrict__ x, const double2* __restrict__ y, uint64_t n, double2* part) {
    double re = 0.0, im = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double2 a = x[i], b = y[i];
        re = fma(a.x, b.x, re);
        re = fma(a.y, b.y, re);
        im = fma(a.x, b.y, im);
        im = fma(-a.y, b.x, im);
    }
    const double2 s = block_sum(make_double2(re, im));
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void dot32_kernel(const float2* __restrict__ x, const float2* __restrict__ y, uint64_t n, double2* part) {
    FF re{0.f, 0.f}, im{0.f, 0.f};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float2 a = x[i], b = y[i];
        ff_add_prod(re, a.x, b.x);
        ff_add_prod(re, a.y, b.y);
        ff_add_prod(im, a.x, b.y);
        ff_add_prod(im, -a.y, b.x);
    }
    const double2 s = block_sum(make_double2(ff_value(re), ff_value(im)));
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void nrm64_kernel(const double2* __restrict__ x, uint64_t n, double2* part) {
    double acc = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double2 a = x[i];
        acc = fma(a.x, a.x, acc);
        acc = fma(a.y, a.y, acc);
    }
    const double2 s = block_sum(make_double2(acc, 0.0));
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void nrm32_kernel(const float2* __restrict__ x, uint64_t n, double2* part) {
    FF acc{0.f, 0.f};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float2 a = x[i];
        ff_add_prod(acc, a.x, a.x);
        ff_add_prod(acc, a.y, a.y);
    }
    const double2 s = block_sum(make_double2(ff_value(acc), 0.0));
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Sum `nparts` partials for each of `k` columns (column j at part[j*stride ...]).
__global__ void finish_kernel(const double2* __restrict__ part, int nparts, int stride, double2* out) {
    const int j = blockIdx.x;
    double re = 0.0, im = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        const double2 v = part[(size_t)j * stride + i];
        re += v.x;
        im += v.y;
    }
    const double2 s = block_sum(make_double2(re, im));
    if (threadIdx.x == 0) out[j] = s;
}

__global__ void axpy64_kernel(double ar, double ai, const double2* __restrict__ x, double2* __restrict__ y, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double2 a = x[i];
        double2 b = y[i];
        b.x = fma(ar, a.x, fma(-ai, a.y, b.x));
        b.y = fma(ar, a.y, fma(ai, a.x, b.y));
        y[i] = b;
    }
}
__global__ void axpy32_kernel(float ar, float ai, const float2* __restrict__ x, float2* __restrict__ y, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float2 a = x[i];
        float2 b = y[i];
        b.x = fmaf(ar, a.x, fmaf(-ai, a.y, b.x));
        b.y = fmaf(ar, a.y, fmaf(ai, a.x, b.y));
        y[i] = b;
    }
}
__global__ void scal64_kernel(double a, double2* __restrict__ x, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        double2 v = x[i];
        v.x *= a;
        v.y *= a;
        x[i] = v;
    }
}
__global__ void scal32_kernel(float a, float2* __restrict__ x, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float2 v = x[i];
        v.x *= a;
        v.y *= a;
        x[i] = v;
    }
}
__global__ void d2f_kernel2(const double2* __restrict__ a, float2* __restrict__ b, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        b[i] = make_float2((float)a[i].x, (float)a[i].y);
}
__global__ void f2d_kernel(const float2* __restrict__ a, double2* __restrict__ b, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        b[i] = make_double2((double)a[i].x, (double)a[i].y);
}

// w <- w - alpha v - beta vprev, and ||w||^2 of the result (one pass).
__global__ void lupd64_kernel(double2* __restrict__ w, const double2* __restrict__ v, const double2* __restrict__ vp,
                              double alpha, double beta, uint64_t n, double2* part) {
    double acc = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        double2 a = w[i];
        const double2 b = v[i];
        a.x = fma(-alpha, b.x, a.x);
        a.y = fma(-alpha, b.y, a.y);
        if (vp) {
            const double2 c = vp[i];
            a.x = fma(-beta, c.x, a.x);
            a.y = fma(-beta, c.y, a.y);
        }
        w[i] = a;
        acc = fma(a.x, a.x, acc);
        acc = fma(a.y, a.y, acc);
    }
    const double2 s = block_sum(make_double2(acc, 0.0));
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void lupd32_kernel(float2* __restrict__ w, const float2* __restrict__ v, const float2* __restrict__ vp,
                              float alpha, float beta, uint64_t n, double2* part) {
    FF acc{0.f, 0.f};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float2 a = w[i];
        const float2 b = v[i];
        a.x = fmaf(-alpha, b.x, a.x);
        a.y = fmaf(-alpha, b.y, a.y);
        if (vp) {
            const float2 c = vp[i];
            a.x = fmaf(-beta, c.x, a.x);
            a.y = fmaf(-beta, c.y, a.y);
        }
        w[i] = a;
        ff_add_prod(acc, a.x, a.x);
        ff_add_prod(acc, a.y, a.y);
    }
    const double2 s = block_sum(make_double2(ff_value(acc), 0.0));
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Projections <V_j, w> for a group of up to KB vectors per block column.
// Grid of all projection kernels: x = column (group of vectors), y = row chunk
// (grid-stride over the elements).  x varies fastest in launch order, so the
// columns of one row chunk run side by side on the same elements and w (or W)
// comes from DRAM once and from L2 for the other columns.
constexpr int KB = 8;
template <class T2, bool F32>
__global__ void mdot_kernel(const T2* const* __restrict__ V, int k, const T2* __restrict__ w, uint64_t n, double2* part,
                            int stride) {
    const int j0 = blockIdx.x * KB;
    const int kk = min(KB, k - j0);
    double re[KB], im[KB];
    FF fre[KB], fim[KB];
#pragma unroll
    for (int q = 0; q < KB; ++q) { re[q] = im[q] = 0.0; fre[q] = fim[q] = FF{0.f, 0.f}; }
    const T2* vp[KB];
#pragma unroll
    for (int q = 0; q < KB; ++q) vp[q] = (q < kk) ? V[j0 + q] : nullptr;
    for (uint64_t i = blockIdx.y * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.y * blockDim.x) {
        const T2 b = w[i];
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            if (q < kk) {
                const T2 a = vp[q][i];
                if (F32) {
                    ff_add_prod(fre[q], (float)a.x, (float)b.x);
                    ff_add_prod(fre[q], (float)a.y, (float)b.y);
                    ff_add_prod(fim[q], (float)a.x, (float)b.y);
                    ff_add_prod(fim[q], -(float)a.y, (float)b.x);
                } else {
                    re[q] = fma((double)a.x, (double)b.x, re[q]);
                    re[q] = fma((double)a.y, (double)b.y, re[q]);
                    im[q] = fma((double)a.x, (double)b.y, im[q]);
                    im[q] = fma(-(double)a.y, (double)b.x, im[q]);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < KB; ++q) {
        if (q < kk) {
            const double2 v = F32 ? make_double2(ff_value(fre[q]), ff_value(fim[q])) : make_double2(re[q], im[q]);
            const double2 s = block_sum(v);
            if (threadIdx.x == 0) part[(size_t)(j0 + q) * stride + blockIdx.y] = s;
        }
    }
}

// FP32 projections <V_j, w> (compensated) for a group of up to KB32 vectors per
// block column, two consecutive elements per thread and iteration (16-byte
// loads when every vector of the group and w are 16-byte aligned).
constexpr int KB32 = 8;
__device__ __forceinline__ void ff_cmac(FF& re, FF& im, float ax, float ay, float bx, float by) {
    ff_add_prod(re, ax, bx);
    ff_add_prod(re, ay, by);
    ff_add_prod(im, ax, by);
    ff_add_prod(im, -ay, bx);
}
__global__ void __launch_bounds__(kThreads) mdot32_kernel(const float2* const* __restrict__ V, int k,
                                                          const float2* __restrict__ w, uint64_t n, double2* part,
                                                          int stride) {
    const int j0 = blockIdx.x * KB32;
    const int kk = min(KB32, k - j0);
    FF re[KB32], im[KB32];
    const float2* vp[KB32];
    bool al = (reinterpret_cast<uintptr_t>(w) & 15u) == 0;
#pragma unroll
    for (int q = 0; q < KB32; ++q) {
        re[q] = im[q] = FF{0.f, 0.f};
        vp[q] = V[j0 + (q < kk ? q : 0)];
        al = al && (reinterpret_cast<uintptr_t>(vp[q]) & 15u) == 0;
    }
    const uint64_t step = (uint64_t)gridDim.y * blockDim.x;
    const uint64_t t0 = blockIdx.y * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t done = 0;
    if (al) {
        const uint64_t n2 = n / 2;
        const float4* w4 = reinterpret_cast<const float4*>(w);
        for (uint64_t i = t0; i < n2; i += step) {
            const float4 b = w4[i];
#pragma unroll
            for (int q = 0; q < KB32; ++q) {
                if (q < kk) {
                    const float4 a = reinterpret_cast<const float4*>(vp[q])[i];
                    ff_cmac(re[q], im[q], a.x, a.y, b.x, b.y);
                    ff_cmac(re[q], im[q], a.z, a.w, b.z, b.w);
                }
            }
        }
        done = 2 * n2;
    }
    for (uint64_t i = done + t0; i < n; i += step) {
        const float2 b = w[i];
#pragma unroll
        for (int q = 0; q < KB32; ++q)
            if (q < kk) {
                const float2 a = vp[q][i];
                ff_cmac(re[q], im[q], a.x, a.y, b.x, b.y);
            }
    }
#pragma unroll
    for (int q = 0; q < KB32; ++q) {
        if (q < kk) block_sum_cff(re[q], im[q], part + (size_t)(j0 + q) * stride + blockIdx.y);
    }
}

// FP32 projections <V_j, W_o> (compensated) for a column of up to KBM vectors
// V_j and NW vectors W_o: every V_j is read once and every W_o once per
// column, where NW separate projections would read every V_j NW times.
constexpr int KBM = 4;
template <int NW>
__global__ void __launch_bounds__(kThreads) mdot32_multi_kernel(const float2* const* __restrict__ V, int k,
                                                                const float2* const* __restrict__ W, uint64_t n,
                                                                double2* part, int stride) {
    const int j0 = blockIdx.x * KBM;
    const int kk = min(KBM, k - j0);
    FF re[KBM][NW], im[KBM][NW];
    const float2* vp[KBM];
    const float2* wp[NW];
    bool al = true;
#pragma unroll
    for (int q = 0; q < KBM; ++q) {
        vp[q] = V[j0 + (q < kk ? q : 0)];
        al = al && (reinterpret_cast<uintptr_t>(vp[q]) & 15u) == 0;
#pragma unroll
        for (int o = 0; o < NW; ++o) re[q][o] = im[q][o] = FF{0.f, 0.f};
    }
#pragma unroll
    for (int o = 0; o < NW; ++o) {
        wp[o] = W[o];
        al = al && (reinterpret_cast<uintptr_t>(wp[o]) & 15u) == 0;
    }
    const uint64_t step = (uint64_t)gridDim.y * blockDim.x;
    const uint64_t t0 = blockIdx.y * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t done = 0;
    if (al) {
        const uint64_t n2 = n / 2;
        for (uint64_t i = t0; i < n2; i += step) {
            float4 b[NW];
#pragma unroll
            for (int o = 0; o < NW; ++o) b[o] = reinterpret_cast<const float4*>(wp[o])[i];
#pragma unroll
            for (int q = 0; q < KBM; ++q) {
                if (q < kk) {
                    const float4 a = reinterpret_cast<const float4*>(vp[q])[i];
#pragma unroll
                    for (int o = 0; o < NW; ++o) {
                        ff_cmac(re[q][o], im[q][o], a.x, a.y, b[o].x, b[o].y);
                        ff_cmac(re[q][o], im[q][o], a.z, a.w, b[o].z, b[o].w);
                    }
                }
            }
        }
        done = 2 * n2;
    }
    for (uint64_t i = done + t0; i < n; i += step) {
#pragma unroll
        for (int q = 0; q < KBM; ++q)
            if (q < kk) {
                const float2 a = vp[q][i];
#pragma unroll
                for (int o = 0; o < NW; ++o) {
                    const float2 b = wp[o][i];
                    ff_cmac(re[q][o], im[q][o], a.x, a.y, b.x, b.y);
                }
            }
    }
#pragma unroll
    for (int q = 0; q < KBM; ++q)
#pragma unroll
        for (int o = 0; o < NW; ++o)
            if (q < kk) block_sum_cff(re[q][o], im[q][o], part + ((size_t)(j0 + q) * NW + o) * stride + blockIdx.y);
}

// The same projections with FP32 sums over short runs: every thread adds its
// products with plain FP32 FMAs over kFastRun consecutive elements (16 pairs of
// elements) and folds each run into a float-float sum (one TwoSum per run), so
// the error is the FP32 rounding of sums of at most 2 kFastRun products, about
// u sqrt(2 kFastRun) of their magnitude (u = 2^-24), instead of the compensated
// kernel's FP64 level, at about a ninth of its FP32 operations.  KC basis
// vectors per column (CTA).
constexpr int kFastRun = 16;  // grid-stride iterations (two elements each) per run
__device__ __forceinline__ void ff_add_f(FF& a, float t) {
    const float s = a.hi + t;
    const float z = s - a.hi;
    a.lo += (a.hi - (s - z)) + (t - z);
    a.hi = s;
}
template <int NW, int KC>
__global__ void __launch_bounds__(kThreads, KC == 4 ? 2 : 3) mdot32_multi_fast_kernel(const float2* const* __restrict__ V, int k,
                                                                     const float2* const* __restrict__ W, uint64_t n,
                                                                     double2* part, int stride) {
    const int j0 = blockIdx.x * KC;
    const int kk = min(KC, k - j0);
    FF re[KC][NW], im[KC][NW];
    float tr[KC][NW], ti[KC][NW];
    const float2* vp[KC];
    const float2* wp[NW];
    bool al = true;
#pragma unroll
    for (int q = 0; q < KC; ++q) {
        vp[q] = V[j0 + (q < kk ? q : 0)];
        al = al && (reinterpret_cast<uintptr_t>(vp[q]) & 15u) == 0;
#pragma unroll
        for (int o = 0; o < NW; ++o) {
            re[q][o] = im[q][o] = FF{0.f, 0.f};
            tr[q][o] = ti[q][o] = 0.f;
        }
    }
#pragma unroll
    for (int o = 0; o < NW; ++o) {
        wp[o] = W[o];
        al = al && (reinterpret_cast<uintptr_t>(wp[o]) & 15u) == 0;
    }
    auto fold = [&]() {
#pragma unroll
        for (int q = 0; q < KC; ++q)
#pragma unroll
            for (int o = 0; o < NW; ++o) {
                ff_add_f(re[q][o], tr[q][o]);
                ff_add_f(im[q][o], ti[q][o]);
                tr[q][o] = ti[q][o] = 0.f;
            }
    };
    const uint64_t step = (uint64_t)gridDim.y * blockDim.x;
    const uint64_t t0 = blockIdx.y * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t done = 0;
    int run = 0;
    if (al) {
        const uint64_t n2 = n / 2;
        for (uint64_t i = t0; i < n2; i += step) {
            float4 b[NW];
#pragma unroll
            for (int o = 0; o < NW; ++o) b[o] = reinterpret_cast<const float4*>(wp[o])[i];
#pragma unroll
            for (int q = 0; q < KC; ++q) {
                if (q < kk) {
                    const float4 a = reinterpret_cast<const float4*>(vp[q])[i];
#pragma unroll
                    for (int o = 0; o < NW; ++o) {
                        float r = tr[q][o], m = ti[q][o];
                        r = fmaf(a.x, b[o].x, r);
                        r = fmaf(a.y, b[o].y, r);
                        m = fmaf(a.x, b[o].y, m);
                        m = fmaf(-a.y, b[o].x, m);
                        r = fmaf(a.z, b[o].z, r);
                        r = fmaf(a.w, b[o].w, r);
                        m = fmaf(a.z, b[o].w, m);
                        m = fmaf(-a.w, b[o].z, m);
                        tr[q][o] = r;
                        ti[q][o] = m;
                    }
                }
            }
            if (++run == kFastRun) {
                fold();
                run = 0;
            }
        }
        done = 2 * n2;
    }
    for (uint64_t i = done + t0; i < n; i += step) {
#pragma unroll
        for (int q = 0; q < KC; ++q)
            if (q < kk) {
                const float2 a = vp[q][i];
#pragma unroll
                for (int o = 0; o < NW; ++o) {
                    const float2 b = wp[o][i];
                    tr[q][o] = fmaf(a.y, b.y, fmaf(a.x, b.x, tr[q][o]));
                    ti[q][o] = fmaf(-a.y, b.x, fmaf(a.x, b.y, ti[q][o]));
                }
            }
        if (++run == kFastRun) {
            fold();
            run = 0;
        }
    }
    fold();
#pragma unroll
    for (int q = 0; q < KC; ++q)
#pragma unroll
        for (int o = 0; o < NW; ++o)
            if (q < kk) block_sum_cff(re[q][o], im[q][o], part + ((size_t)(j0 + q) * NW + o) * stride + blockIdx.y);
}

// w += sum_j c_j V_j ; coefficients (complex double) in global memory.
template <class T2, class A>
__global__ void mcomb_kernel(const T2* const* __restrict__ V, int k, const double2* __restrict__ c, T2* __restrict__ w,
                             uint64_t n) {
    // coefficients converted to the working type once (a double-to-float
    // conversion per element would run on the FP64 pipe)
    extern __shared__ double2 sc_raw[];
    A* sc = reinterpret_cast<A*>(sc_raw);
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
        sc[2 * j] = (A)c[j].x;
        sc[2 * j + 1] = (A)c[j].y;
    }
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        T2 o = w[i];
        A re = (A)o.x, im = (A)o.y;
        for (int j = 0; j < k; ++j) {
            const T2 a = V[j][i];
            const A cr = sc[2 * j], ci = sc[2 * j + 1];
            re = fma(cr, (A)a.x, fma(-ci, (A)a.y, re));
            im = fma(cr, (A)a.y, fma(ci, (A)a.x, im));
        }
        o.x = re;
        o.y = im;
        w[i] = o;
    }
}

// W_o = (accumulate ? W_o : 0) + sum_j C[o * k + j] V_j for o < nout: each
// V_j is read once for all outputs.
template <class T2, class A, int NOUT>
__global__ void mcomb_multi_kernel(const T2* const* __restrict__ V, int k, const double2* __restrict__ c,
                                   T2* const* __restrict__ W, uint64_t n, int accumulate) {
    extern __shared__ double2 sc_raw[];
    A* sc = reinterpret_cast<A*>(sc_raw);
    for (int j = threadIdx.x; j < NOUT * k; j += blockDim.x) {
        sc[2 * j] = (A)c[j].x;
        sc[2 * j + 1] = (A)c[j].y;
    }
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        A re[NOUT], im[NOUT];
#pragma unroll
        for (int o = 0; o < NOUT; ++o) {
            re[o] = 0;
            im[o] = 0;
            if (accumulate) {
                const T2 w = W[o][i];
                re[o] = (A)w.x;
                im[o] = (A)w.y;
            }
        }
        for (int j = 0; j < k; ++j) {
            const T2 a = V[j][i];
#pragma unroll
            for (int o = 0; o < NOUT; ++o) {
                const A cr = sc[2 * (o * k + j)], ci = sc[2 * (o * k + j) + 1];
                re[o] = fma(cr, (A)a.x, fma(-ci, (A)a.y, re[o]));
                im[o] = fma(cr, (A)a.y, fma(ci, (A)a.x, im[o]));
            }
        }
#pragma unroll
        for (int o = 0; o < NOUT; ++o) {
            T2 w;
            w.x = re[o];
            w.y = im[o];
            W[o][i] = w;
        }
    }
}

// The Davidson preconditioner for FP32 vectors (difference taken in FP64).
__global__ void precond32_kernel(const float2* __restrict__ r, const double2* __restrict__ d, double lambda,
                                 float2* __restrict__ t, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float fr = (float)(d[i].x - lambda), fi = (float)d[i].y;
        if (sqrtf(fr * fr + fi * fi) < 1e-10f) { fr = (fr >= 0.f) ? 1e-10f : -1e-10f; fi = 0.f; }
        const float2 a = r[i];
        const float den = fr * fr + fi * fi;
        t[i] = make_float2((a.x * fr + a.y * fi) / den, (a.y * fr - a.x * fi) / den);
    }
}

__global__ void precond_kernel(const double2* __restrict__ r, const double2* __restrict__ d, double lambda,
                               double2* __restrict__ t, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        // src/solvers/davidson.cpp:171-175: diff = d_i - lambda, clamped to +-1e-10.
        double dr = d[i].x - lambda, di = d[i].y;
        if (sqrt(dr * dr + di * di) < 1e-10) { dr = (dr >= 0) ? 1e-10 : -1e-10; di = 0.0; }
        const double2 a = r[i];
        const double den = dr * dr + di * di;
        t[i] = make_double2((a.x * dr + a.y * di) / den, (a.y * dr - a.x * di) / den);
    }
}

// Element i gets one Philox block; Box-Muller turns its words into a complex
// standard normal (real and imaginary parts independent N(0,1)).
template <class T2, bool F64>
__global__ void philox_normal_kernel(uint64_t seed, uint64_t stream, T2* out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = fastk::philox_cnormal<T2, F64>(seed, stream, i);
}

double2* finish(Workspace& ws, int nparts, int stride, int k, cudaStream_t s) {
    finish_kernel<<<k, kThreads, 0, s>>>(ws.partial.as<double2>(), nparts, stride, ws.result.as<double2>());
    QKG_LAUNCHED();
    QKG_CUDA(cudaMemcpyAsync(ws.host, ws.result.p, (size_t)k * sizeof(double2), cudaMemcpyDeviceToHost, s));
    QKG_CUDA(cudaStreamSynchronize(s));
    return reinterpret_cast<double2*>(ws.host);
}

}  // namespace

Workspace::Workspace(size_t cap) : cap_partials(cap) {
    partial.alloc(cap * sizeof(double2));
    result.alloc(4096 * sizeof(double2));
    QKG_CUDA(cudaMallocHost(&host, 4096 * sizeof(double2)));
}
Workspace::~Workspace() {
    if (host) cudaFreeHost(host);
}

std::complex<double> dot_f64(const double2* x, const double2* y, uint64_t n, Workspace& ws, cudaStream_t s) {
    const int g = stream_grid(n);
    dot64_kernel<<<g, kThreads, 0, s>>>(x, y, n, ws.partial.as<double2>());
    QKG_LAUNCHED();
    const double2 r = finish(ws, g, g, 1, s)[0];
    return {r.x, r.y};
}
std::complex<double> dot_f32(const float2* x, const float2* y, uint64_t n, Workspace& ws, cudaStream_t s) {
    const int g = stream_grid(n);
    dot32_kernel<<<g, kThreads, 0, s>>>(x, y, n, ws.partial.as<double2>());
    QKG_LAUNCHED();
    const double2 r = finish(ws, g, g, 1, s)[0];
    return {r.x, r.y};
}
double nrm2sq_f64(const double2* x, uint64_t n, Workspace& ws, cudaStream_t s) {
    const int g = stream_grid(n);
    nrm64_kernel<<<g, kThreads, 0, s>>>(x, n, ws.partial.as<double2>());
    QKG_LAUNCHED();
    return finish(ws, g, g, 1, s)[0].x;
}
double nrm2sq_f32(const float2* x, uint64_t n, Workspace& ws, cudaStream_t s) {
    const int g = stream_grid(n);
    nrm32_kernel<<<g, kThreads, 0, s>>>(x, n, ws.partial.as<double2>());
    QKG_LAUNCHED();
    return finish(ws, g, g, 1, s)[0].x;
}
void axpy_f64(std::complex<double> a, const double2* x, double2* y, uint64_t n, cudaStream_t s) {
    axpy64_kernel<<<stream_grid(n), kThreads, 0, s>>>(a.real(), a.imag(), x, y, n);
    QKG_LAUNCHED();
}
void axpy_f32(std::complex<double> a, const float2* x, float2* y, uint64_t n, cudaStream_t s) {
    axpy32_kernel<<<stream_grid(n), kThreads, 0, s>>>((float)a.real(), (float)a.imag(), x, y, n);
    QKG_LAUNCHED();
}
void scal_f64(double a, double2* x, uint64_t n, cudaStream_t s) {
    scal64_kernel<<<stream_grid(n), kThreads, 0, s>>>(a, x, n);
    QKG_LAUNCHED();
}
void scal_f32(double a, float2* x, uint64_t n, cudaStream_t s) {
    scal32_kernel<<<stream_grid(n), kThreads, 0, s>>>((float)a, x, n);
    QKG_LAUNCHED();
}
void f64_to_f32(const double2* x, float2* y, uint64_t n, cudaStream_t s) {
    d2f_kernel2<<<stream_grid(n), kThreads, 0, s>>>(x, y, n);
    QKG_LAUNCHED();
}
void f32_to_f64(const float2* x, double2* y, uint64_t n, cudaStream_t s) {
    f2d_kernel<<<stream_grid(n), kThreads, 0, s>>>(x, y, n);
    QKG_LAUNCHED();
}
double lanczos_update_f64(double2* w, const double2* v, const double2* vp, double alpha, double beta, uint64_t n,
                          Workspace& ws, cudaStream_t s) {
    const int g = stream_grid(n);
    lupd64_kernel<<<g, kThreads, 0, s>>>(w, v, vp, alpha, beta, n, ws.partial.as<double2>());
    QKG_LAUNCHED();
    return finish(ws, g, g, 1, s)[0].x;
}
double lanczos_update_f32(float2* w, const float2* v, const float2* vp, double alpha, double beta, uint64_t n,
                          Workspace& ws, cudaStream_t s) {
    const int g = stream_grid(n);
    lupd32_kernel<<<g, kThreads, 0, s>>>(w, v, vp, (float)alpha, (float)beta, n, ws.partial.as<double2>());
    QKG_LAUNCHED();
    return finish(ws, g, g, 1, s)[0].x;
}

template <class T2, bool F32>
static void mdot_impl(const T2* const* V, int k, const T2* w, uint64_t n, std::complex<double>* out, Workspace& ws,
                      cudaStream_t s) {
    if (k <= 0) return;
    QKG_REQUIRE(k <= 4096, "mdot: too many vectors");
    int g = stream_grid(n);
    g = (int)std::min<size_t>((size_t)g, ws.cap_partials / (size_t)k);
    g = std::max(1, g);
    if (F32) {
        dim3 grid((k + KB32 - 1) / KB32, g);
        mdot32_kernel<<<grid, kThreads, 0, s>>>(reinterpret_cast<const float2* const*>(V), k,
                                                reinterpret_cast<const float2*>(w), n, ws.partial.as<double2>(), g);
    } else {
        dim3 grid((k + KB - 1) / KB, g);
        mdot_kernel<T2, F32><<<grid, kThreads, 0, s>>>(V, k, w, n, ws.partial.as<double2>(), g);
    }
    QKG_LAUNCHED();
    const double2* r = finish(ws, g, g, k, s);
    for (int j = 0; j < k; ++j) out[j] = {r[j].x, r[j].y};
}
void mdot_f64(const double2* const* V, int k, const double2* w, uint64_t n, std::complex<double>* out, Workspace& ws,
              cudaStream_t s) {
    mdot_impl<double2, false>(V, k, w, n, out, ws, s);
}
void mdot_f32(const float2* const* V, int k, const float2* w, uint64_t n, std::complex<double>* out, Workspace& ws,
              cudaStream_t s) {
    mdot_impl<float2, true>(V, k, w, n, out, ws, s);
}
namespace {
// the run-summed kernel: at the mixed Davidson's accuracy (FP32 vectors) it
// gives the compensated kernel's eigenvalues and residuals at about half the time
std::atomic<int> g_projection_mode{2};
}
void set_projection_mode(int mode) { g_projection_mode.store(mode); }
int projection_mode() { return g_projection_mode.load(); }

void mdot_multi_f32(const float2* const* V, int k, float2* const* W, int nw, uint64_t n, std::complex<double>* out,
                    Workspace& ws, cudaStream_t s) {
    if (k <= 0 || nw <= 0) return;
    const int mode = g_projection_mode.load();
    if (mode == 1 && mdot_tc_supported(k, nw)) {
        mdot_multi_f32_tc(V, k, W, nw, n, out, ws, s);
        return;
    }
    if (mode == 2) {
        mdot_multi_f32_fast(V, k, W, nw, n, out, ws, s);
        return;
    }
    mdot_multi_f32_cuda(V, k, W, nw, n, out, ws, s);
}

// Row chunks for a grid of ncol columns on `slots` resident CTAs: the fewest
// waves (from two) whose last wave is at least 90% full, at most g_max chunks
// (every chunk a whole grid-stride sweep, so a nearly empty last wave costs a
// full CTA time).
static int balanced_chunks(int ncol, int slots, int g_max) {
    for (int waves = 2; waves <= 16; ++waves) {
        const int g = std::max(1, waves * slots / ncol);
        if (g > g_max) break;
        const long long total = (long long)g * ncol, full = (total + slots - 1) / slots;
        if ((double)total >= 0.9 * (double)(full * slots)) return g;
    }
    return g_max;
}

void mdot_multi_f32_fast(const float2* const* V, int k, float2* const* W, int nw, uint64_t n, std::complex<double>* out,
                         Workspace& ws, cudaStream_t s) {
    if (k <= 0 || nw <= 0) return;
    QKG_REQUIRE(nw <= 4 && (size_t)k * nw <= 4088, "mdot_multi: at most 4 right-hand vectors and 4088 products");
    float2** dw = reinterpret_cast<float2**>(ws.result.as<double2>() + 4096 - 8);
    QKG_CUDA(cudaMemcpyAsync(dw, W, (size_t)nw * sizeof(float2*), cudaMemcpyHostToDevice, s));
    int g = stream_grid(n);
    g = (int)std::min<size_t>((size_t)g, ws.cap_partials / ((size_t)k * nw));
    g = std::max(1, g);
    // Columns of 2 basis vectors for 3-4 right-hand vectors (80 registers, 3
    // CTAs per SM; W's re-reads come from L2), of 4 for 1-2 (at k = 32, n = 11.8 M:
    // nw = 4 1.00 against 1.42 ms, nw = 1 0.18 against 0.16 ms).  Row chunks for
    // two resident waves of CTAs in all, rounded down (a last, nearly empty wave
    // of whole chunks would double the time): at k = 32, nw = 4, n = 11.8 M
    // 0.93 ms, against 1.02 ms for 512 chunks and 1.71 ms for one wave rounded up.
    double2* part = ws.partial.as<double2>();
    auto launch = [&](auto kern, int kc) {
        const int ncol = (k + kc - 1) / kc;
        int per_sm = 1;
        QKG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, 0));
        g = balanced_chunks(ncol, 152 * std::max(1, per_sm), g);
        kern<<<dim3(ncol, g), kThreads, 0, s>>>(V, k, dw, n, part, g);
    };
    switch (nw) {
        case 1: launch(mdot32_multi_fast_kernel<1, KBM>, KBM); break;
        case 2: launch(mdot32_multi_fast_kernel<2, KBM>, KBM); break;
        case 3: launch(mdot32_multi_fast_kernel<3, 2>, 2); break;
        default: launch(mdot32_multi_fast_kernel<4, 2>, 2); break;
    }
    QKG_LAUNCHED();
    const double2* r = finish(ws, g, g, k * nw, s);
    for (int j = 0; j < k; ++j)
        for (int o = 0; o < nw; ++o) out[(size_t)o * k + j] = {r[(size_t)j * nw + o].x, r[(size_t)j * nw + o].y};
}

void mdot_multi_f32_cuda(const float2* const* V, int k, float2* const* W, int nw, uint64_t n, std::complex<double>* out,
                         Workspace& ws, cudaStream_t s) {
    if (k <= 0 || nw <= 0) return;
    QKG_REQUIRE(nw <= 4 && (size_t)k * nw <= 4088, "mdot_multi: at most 4 right-hand vectors and 4088 products");
    // the W pointer table goes through the result slots (read by the kernel before finish overwrites them)
    float2** dw = reinterpret_cast<float2**>(ws.result.as<double2>() + 4096 - 8);
    QKG_CUDA(cudaMemcpyAsync(dw, W, (size_t)nw * sizeof(float2*), cudaMemcpyHostToDevice, s));
    int g = stream_grid(n);
    g = (int)std::min<size_t>((size_t)g, ws.cap_partials / ((size_t)k * nw));
    g = std::max(1, g);
    const dim3 grid((k + KBM - 1) / KBM, g);
    double2* part = ws.partial.as<double2>();
    switch (nw) {
        case 1: mdot32_multi_kernel<1><<<grid, kThreads, 0, s>>>(V, k, dw, n, part, g); break;
        case 2: mdot32_multi_kernel<2><<<grid, kThreads, 0, s>>>(V, k, dw, n, part, g); break;
        case 3: mdot32_multi_kernel<3><<<grid, kThreads, 0, s>>>(V, k, dw, n, part, g); break;
        default: mdot32_multi_kernel<4><<<grid, kThreads, 0, s>>>(V, k, dw, n, part, g); break;
    }
    QKG_LAUNCHED();
    const double2* r = finish(ws, g, g, k * nw, s);
    for (int j = 0; j < k; ++j)
        for (int o = 0; o < nw; ++o) out[(size_t)o * k + j] = {r[(size_t)j * nw + o].x, r[(size_t)j * nw + o].y};
}

template <class T2, class A>
static void mcomb_impl(const T2* const* V, int k, const std::complex<double>* c, T2* w, uint64_t n, Workspace& ws,
                       cudaStream_t s) {
    // Chunks of at most 1024 vectors (16 KB of coefficients in shared memory).
    for (int j0 = 0; j0 < k; j0 += 1024) {
        const int kk = std::min(1024, k - j0);
        QKG_CUDA(cudaMemcpyAsync(ws.result.p, c + j0, (size_t)kk * sizeof(double2), cudaMemcpyHostToDevice, s));
        mcomb_kernel<T2, A><<<stream_grid(n), kThreads, (size_t)kk * sizeof(double2), s>>>(V + j0, kk,
                                                                                              ws.result.as<double2>(), w, n);
        QKG_LAUNCHED();
        QKG_CUDA(cudaStreamSynchronize(s));  // the coefficient slot is reused by the next chunk
    }
}
void mcombine_f64(const double2* const* V, int k, const std::complex<double>* c, double2* w, uint64_t n, Workspace& ws,
                  cudaStream_t s) {
    mcomb_impl<double2, double>(V, k, c, w, n, ws, s);
}
void mcombine_f32(const float2* const* V, int k, const std::complex<double>* c, float2* w, uint64_t n, Workspace& ws,
                  cudaStream_t s) {
    mcomb_impl<float2, float>(V, k, c, w, n, ws, s);
}
void philox_normal_f64(uint64_t seed, uint64_t stream, double2* out, uint64_t n, cudaStream_t s) {
    philox_normal_kernel<double2, true><<<stream_grid(n), kThreads, 0, s>>>(seed, stream, out, n);
    QKG_LAUNCHED();
}
void philox_normal_f32(uint64_t seed, uint64_t stream, float2* out, uint64_t n, cudaStream_t s) {
    philox_normal_kernel<float2, false><<<stream_grid(n), kThreads, 0, s>>>(seed, stream, out, n);
    QKG_LAUNCHED();
}
template <class T2, class A>
static void mcomb_multi_impl(const T2* const* V, int k, const std::complex<double>* c, T2* const* W, int nout,
                             uint64_t n, bool accumulate, Workspace& ws, cudaStream_t s) {
    QKG_REQUIRE(nout >= 1 && nout <= 8, "mcombine_multi: 1..8 outputs");
    QKG_REQUIRE(k >= 0 && nout * k <= 1024, "mcombine_multi: at most 1024 coefficients");
    if (!n) return;
    // coefficients and the output pointer table go through the workspace result slots
    double2* dc = ws.result.as<double2>();
    QKG_CUDA(cudaMemcpyAsync(dc, c, (size_t)nout * k * sizeof(double2), cudaMemcpyHostToDevice, s));
    T2** dw = reinterpret_cast<T2**>(dc + 1024);
    QKG_CUDA(cudaMemcpyAsync(dw, W, (size_t)nout * sizeof(T2*), cudaMemcpyHostToDevice, s));
    const size_t sm = (size_t)nout * k * sizeof(double2);
    const int g = stream_grid(n);
    const int acc = accumulate ? 1 : 0;
    switch (nout) {
        case 1: mcomb_multi_kernel<T2, A, 1><<<g, kThreads, sm, s>>>(V, k, dc, dw, n, acc); break;
        case 2: mcomb_multi_kernel<T2, A, 2><<<g, kThreads, sm, s>>>(V, k, dc, dw, n, acc); break;
        case 3: mcomb_multi_kernel<T2, A, 3><<<g, kThreads, sm, s>>>(V, k, dc, dw, n, acc); break;
        case 4: mcomb_multi_kernel<T2, A, 4><<<g, kThreads, sm, s>>>(V, k, dc, dw, n, acc); break;
        case 5: mcomb_multi_kernel<T2, A, 5><<<g, kThreads, sm, s>>>(V, k, dc, dw, n, acc); break;
        case 6: mcomb_multi_kernel<T2, A, 6><<<g, kThreads, sm, s>>>(V, k, dc, dw, n, acc); break;
        case 7: mcomb_multi_kernel<T2, A, 7><<<g, kThreads, sm, s>>>(V, k, dc, dw, n, acc); break;
        default: mcomb_multi_kernel<T2, A, 8><<<g, kThreads, sm, s>>>(V, k, dc, dw, n, acc); break;
    }
    QKG_LAUNCHED();
    // the host arrays may be reused once the copies have been consumed
    QKG_CUDA(cudaStreamSynchronize(s));
}
void mcombine_multi_f64(const double2* const* V, int k, const std::complex<double>* c, double2* const* W, int nout,
                        uint64_t n, bool accumulate, Workspace& ws, cudaStream_t s) {
    mcomb_multi_impl<double2, double>(V, k, c, W, nout, n, accumulate, ws, s);
}
void mcombine_multi_f32(const float2* const* V, int k, const std::complex<double>* c, float2* const* W, int nout,
                        uint64_t n, bool accumulate, Workspace& ws, cudaStream_t s) {
    mcomb_multi_impl<float2, float>(V, k, c, W, nout, n, accumulate, ws, s);
}
void davidson_precond_f32(const float2* r, const double2* d, double lambda, float2* t, uint64_t n, cudaStream_t s) {
    precond32_kernel<<<stream_grid(n), kThreads, 0, s>>>(r, d, lambda, t, n);
    QKG_LAUNCHED();
}
void davidson_precond_f64(const double2* r, const double2* d, double lambda, double2* t, uint64_t n, cudaStream_t s) {
    precond_kernel<<<stream_grid(n), kThreads, 0, s>>>(r, d, lambda, t, n);
    QKG_LAUNCHED();
}

}  // namespace qkg
