// Device-side types and helpers shared by the SpMV kernels (hamiltonian.cu)
// and the block-vector kernels (block.cu).
#pragma once

#include "ham.hpp"

namespace qkg {
namespace fastk {

constexpr int kBlock = 256;
constexpr uint32_t kChunk = 1024;
constexpr int kMaxOuter = 256;
constexpr int kMaxInnerTable = 512;  // inner terms a table may reference
constexpr uint32_t kEllEmpty = 0xFFFFFFFFu;

template <class S, class A>
struct alignas(16) KTerm {
    S C, V, X, J;
    A ar, ai;
    uint32_t flags, var0;
};
template <class A>
struct alignas(16) KVar {
    uint64_t sm, pf;
    A a0r, a0i, a1r, a1i;
};

template <class T> struct V2;
template <> struct V2<double> { using t = double2; };
template <> struct V2<float> { using t = float2; };

template <class S> __device__ __forceinline__ int popcnt(S x);
template <> __device__ __forceinline__ int popcnt<uint32_t>(uint32_t x) { return __popc(x); }
template <> __device__ __forceinline__ int popcnt<uint64_t>(uint64_t x) { return __popcll(x); }

template <class S, class A>
__device__ __forceinline__ void term_amp(const KTerm<S, A>& t, S s, const KVar<A>* __restrict__ vars, A& ar, A& ai) {
    ar = t.ar;
    ai = t.ai;
    const uint32_t nv = (t.flags >> 8) & 0xffu;
    for (uint32_t k = 0; k < nv; ++k) {
        const KVar<A> v = vars[t.var0 + k];
        const bool sel = (((uint64_t)s ^ v.pf) & v.sm) == v.sm;
        const A cr = sel ? v.a1r : v.a0r, ci = sel ? v.a1i : v.a0i;
        const A nr = ar * cr - ai * ci;
        ai = ar * ci + ai * cr;
        ar = nr;
    }
    if (popcnt<S>(s & t.J) & 1) {
        ar = -ar;
        ai = -ai;
    }
}

template <class A, class X2>
__device__ __forceinline__ void cmac(A& r, A& i, A ar, A ai, const X2& x, bool real) {
    r = fma(ar, (A)x.x, r);
    i = fma(ar, (A)x.y, i);
    if (!real) {
        r = fma(-ai, (A)x.y, r);
        i = fma(ai, (A)x.x, i);
    }
}

template <class A>
struct alignas(16) OutEnt {
    int32_t delta;
    uint32_t J;
    A ar, ai;
};

template <class A>
struct FastParams {
    int n_in;
    uint32_t in_mask;
    int ngroups, no_double, N;
    uint32_t gmask0, gmask1;
    int gpop0, gpop1;
    const uint32_t* outer_off;
    const uint32_t* inner_rank;   // null: inner rank = inner bits
    const uint32_t* inner_state;  // null: inner configuration = table index
    const WorkItem* items;
    const uint32_t* iptr;         // table rows
    const uint32_t* ient;         // entries: rank | inner sign << rbits | term << (rbits + 1)
    int rbits;
    const KTerm<uint32_t, A>* inner;  // per term: amplitude, J (its outer part signs per block)
    int n_inner;
    A u_ar, u_ai;                 // UNIF: the one amplitude (no signs)
    const KTerm<uint32_t, A>* outer;
    int n_outer, outer_has_j;
    const KTerm<uint32_t, A>* mixed;
    const KVar<A>* vars;
    int n_mixed;
    // per outer configuration a: its valid outer entries oent[optr[a] ..
    // optr[a+1]) and the straddling terms whose outer-bit condition holds,
    // ment[mptr[a] .. mptr[a+1]) = (term index, target block offset)
    const uint32_t* optr;
    const OutEnt<A>* oent;
    const uint32_t* mptr;
    const uint2* ment;
    int diag_mode;
    int n_dtab;
    const void* dcode;
    const A* dtab;
    // Lanczos mode (null otherwise): x, y, scale and the previous-vector term
    // from *lz (y = scale H x - bprev vprev); each block writes Re sum conj(x) y
    // to apart.
    const LzOperands* lz;
    double2* apart;
};

// Compensated accumulation of a*b into (hi, lo) (TwoProduct + TwoSum).
__device__ __forceinline__ void ffma_acc(float& hi, float& lo, float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    const float t = hi + p;
    const float z = t - hi;
    lo += ((hi - (t - z)) + (p - z)) + e;
    hi = t;
}
__device__ __forceinline__ void ffma_acc(double& hi, double& lo, double a, double b) { hi = fma(a, b, hi); }

// (hi, lo) += (bh, bl) in float-float arithmetic (TwoSum on the high parts).
__device__ __forceinline__ void ff_add(float& hi, float& lo, float bh, float bl) {
    const float t = hi + bh;
    const float z = t - hi;
    lo += ((hi - (t - z)) + (bh - z)) + bl;
    hi = t;
}
// Block sum of float-float values, entirely in FP32 arithmetic (the FP64 pipe
// is narrow: a double-precision block reduction in every small CTA costs more
// than the reduction is worth).  The result is valid in thread 0.
__device__ __forceinline__ float2 block_sum_ff(float hi, float lo) {
    __shared__ float2 shf[32];
    for (int o = 16; o > 0; o >>= 1) {
        const float bh = __shfl_down_sync(0xffffffffu, hi, o), bl = __shfl_down_sync(0xffffffffu, lo, o);
        ff_add(hi, lo, bh, bl);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) shf[wid] = make_float2(hi, lo);
    __syncthreads();
    if (wid == 0) {
        const float2 v = (threadIdx.x < (blockDim.x >> 5)) ? shf[lane] : make_float2(0.f, 0.f);
        hi = v.x;
        lo = v.y;
        for (int o = 16; o > 0; o >>= 1) {
            const float bh = __shfl_down_sync(0xffffffffu, hi, o), bl = __shfl_down_sync(0xffffffffu, lo, o);
            ff_add(hi, lo, bh, bl);
        }
    }
    return make_float2(hi, lo);
}

__device__ __forceinline__ double block_sum_d(double v) {
    __shared__ double sh[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = (threadIdx.x < (blockDim.x >> 5)) ? sh[lane] : 0.0;
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ bool in_basis_fast(int ng, uint32_t g0, uint32_t g1, int p0, int p1, int no_double, int N,
                                              uint32_t s) {
    if (ng > 0 && __popc(s & g0) != p0) return false;
    if (ng > 1 && __popc(s & g1) != p1) return false;
    if (no_double && (s & (s >> N) & ((1u << N) - 1u))) return false;
    return true;
}

constexpr int kMaxMixedSmem = 64;

// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror & Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64-bit
// multiplies with the round keys bumped by the Weyl constants.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += W0;
        k.y += W1;
    }
    return c;
}

// Complex standard normal (real and imaginary parts independent N(0,1)) from
// the Philox block (counter i, stream) by Box-Muller.
template <class T2, bool F64>
__device__ __forceinline__ T2 philox_cnormal(uint64_t seed, uint64_t stream, uint64_t i) {
    const uint4 r = philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)),
                                  make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    T2 o;
    if (F64) {
        const double u1 = ((double)r.x + 1.0) * 2.3283064365386963e-10;  // (0, 1]
        const double u2 = (double)r.y * 2.3283064365386963e-10;
        const double rad = sqrt(-2.0 * log(u1));
        double sn, cs;
        sincospi(2.0 * u2, &sn, &cs);
        o.x = rad * cs;
        o.y = rad * sn;
    } else {
        const float u1 = ((float)r.x + 1.0f) * 2.3283064e-10f;
        const float u2 = (float)r.y * 2.3283064e-10f;
        const float rad = sqrtf(-2.0f * logf(u1));
        float sn, cs;
        sincospif(2.0f * u2, &sn, &cs);
        o.x = rad * cs;
        o.y = rad * sn;
    }
    return o;
}

}  // namespace fastk
}  // namespace qkg
