// Block SpMV and the batched three-term Lanczos recurrence.
//
// A block vector holds Rp complex vectors interleaved by row, X[row * Rp + r],
// so one gather of a row reads Rp * sizeof(T2) contiguous bytes (Rp = 32 in
// FP32: 256 B) and the index work of a row (its state, the walk of its inner
// ELL table row, the ranks of straddling terms) is shared by its Rp values.
// Several Hamiltonians share one block vector: Hamiltonian h owns rows
// [base_h, base_h + dim_h).  The SpMV grid is the concatenation of every
// Hamiltonian's work items, each tagged with its Hamiltonian; a CTA first
// copies that Hamiltonian's kernel parameters into shared memory, so sectors
// of very different sizes (1 to 2.7 M rows for an L = 24 chain) share one
// launch.  Thread mapping: G = Rp / VPL lanes per row, each lane holding VPL
// vectors (VPL complex values per gather), 32 / G rows per warp; VPL is picked
// by timing (the autotuner below).
//
// The recurrence is the reference's compute_tridiag / continued_fraction_coeffs
// loop (src/solvers/ftlm.cpp:24-53, src/solvers/dynamics.cpp:13-59) run for all
// vectors at once, with every scalar kept on the device: vector v at step k is
// q_k = c_k u_k with u_k the stored (unnormalised) vector and c_k its scale, so
//   y = c_k H u_k                (SpMV, scale applied in its epilogue)
//   alpha_k = c_k Re<u_k, y>     (SpMV epilogue partials + finish kernel)
//   w = y - alpha_k c_k u_k - beta_{k-1} c_{k-1} u_{k-1}   (update, in place on y)
//   beta_k = ||w||, u_{k+1} = w, c_{k+1} = 1 / beta_k
// and a vector whose beta falls below 1e-15 stops recording (its scale becomes
// 0, so its later values are zero).  Three buffers rotate; the steps after the
// first three are one CUDA graph of three steps (a full rotation) replayed,
// with the step index in device memory.
#include "block.hpp"
#include "fast_common.cuh"
#include "solvers.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>

namespace qkg {
using namespace fastk;
namespace {

struct BItem {
    WorkItem w;     // the Hamiltonian's own work item (row0 relative to it)
    uint64_t base;  // first row of the Hamiltonian in the block vector
    uint32_t ham;
    uint32_t unused;
};

template <class T, int VPL>
__device__ __forceinline__ void vload(const typename V2<T>::t* p, typename V2<T>::t (&v)[VPL]) {
    if constexpr (sizeof(T) == 4 && VPL % 2 == 0) {
#pragma unroll
        for (int j = 0; j < VPL; j += 2) {
            const float4 q = reinterpret_cast<const float4*>(p)[j / 2];
            v[j].x = q.x;
            v[j].y = q.y;
            v[j + 1].x = q.z;
            v[j + 1].y = q.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < VPL; ++j) v[j] = p[j];
    }
}

// y is written once per step and next read by the update pass: stored
// evict-first (cache-streaming), so the gathered x keeps more of L2
template <class T, int VPL>
__device__ __forceinline__ void vstore(typename V2<T>::t* p, const typename V2<T>::t (&v)[VPL]) {
    if constexpr (sizeof(T) == 4 && VPL % 2 == 0) {
#pragma unroll
        for (int j = 0; j < VPL; j += 2)
            __stcs(reinterpret_cast<float4*>(p) + j / 2, make_float4(v[j].x, v[j].y, v[j + 1].x, v[j + 1].y));
    } else {
#pragma unroll
        for (int j = 0; j < VPL; ++j) __stcs(p + j, v[j]);
    }
}

// y = diag(scale) H x for the Rp vectors of every Hamiltonian; with apart,
// CTA c writes Re sum conj(x_v) y_v over its rows to apart[c * Rp + v].
// Resident CTAs per SM the register allocation is held to (FP32 / FP64).
#ifndef QKG_BLOCK_MINB
#define QKG_BLOCK_MINB 4
#endif
#ifndef QKG_BLOCK_MINB64
#define QKG_BLOCK_MINB64 2
#endif
#ifndef QKG_BLOCK_PREFETCH
#define QKG_BLOCK_PREFETCH 1
#endif
template <class T, class A, bool REAL, bool UNIF, bool OJ, int VPL>
__global__ void __launch_bounds__(kBlock, sizeof(T) == 4 ? QKG_BLOCK_MINB : QKG_BLOCK_MINB64) spmv_block_kernel(const FastParams<A>* __restrict__ P,
                                                            const BItem* __restrict__ items, int Rp,
                                                            const typename V2<T>::t* __restrict__ X,
                                                            typename V2<T>::t* __restrict__ Y,
                                                            const double* __restrict__ scale,
                                                            double* __restrict__ apart) {
    using T2 = typename V2<T>::t;
    __shared__ FastParams<A> sp;
    __shared__ OutEnt<A> s_out[kMaxOuter];
    __shared__ A s_iamp[2 * kMaxInnerTable];
    __shared__ KTerm<uint32_t, A> s_mixed[kMaxMixedSmem];
    __shared__ A s_dtab[512];
    __shared__ double s_red[kBlock * VPL];
    __shared__ int s_n;
    const BItem bi = items[blockIdx.x];
    if (threadIdx.x == 0) sp = P[bi.ham];
    __syncthreads();
    const WorkItem it = bi.w;
    const int n_mixed = sp.n_mixed;
    const bool mixed_smem = n_mixed <= kMaxMixedSmem;
    if (mixed_smem)
        for (int t = threadIdx.x; t < n_mixed; t += blockDim.x) s_mixed[t] = sp.mixed[t];
    const int diag_mode = sp.diag_mode;
    if (diag_mode == DIAG_U8)
        for (int t = threadIdx.x; t < 2 * sp.n_dtab; t += blockDim.x) s_dtab[t] = sp.dtab[t];
    const int n_in = sp.n_in;
    const uint32_t* __restrict__ outer_off = sp.outer_off;
    const uint32_t* __restrict__ inner_state = sp.inner_state;
    const uint32_t block_off = __ldg(outer_off + it.a);
    if (!UNIF) {
        const uint32_t sa = it.a << n_in;
        for (int t = threadIdx.x; t < sp.n_inner; t += blockDim.x) {
            const KTerm<uint32_t, A> k = sp.inner[t];
            const bool neg = __popc(sa & k.J) & 1;
            s_iamp[2 * t] = neg ? -k.ar : k.ar;
            s_iamp[2 * t + 1] = neg ? -k.ai : k.ai;
        }
    }
    if (threadIdx.x < 32) {
        const uint32_t b0 = inner_state ? __ldg(inner_state + it.inner_base) : it.inner_base;
        const uint32_t s0 = (it.a << n_in) | b0;
        int base = 0;
        for (int t0 = 0; t0 < sp.n_outer; t0 += 32) {
            const int ti = t0 + (int)threadIdx.x;
            bool ok = false;
            OutEnt<A> e;
            if (ti < sp.n_outer) {
                const KTerm<uint32_t, A> t = sp.outer[ti];
                if ((s0 & t.C) == t.V) {
                    const uint32_t s2 = s0 ^ t.X;
                    if (!(t.flags & 1u) ||
                        in_basis_fast(sp.ngroups, sp.gmask0, sp.gmask1, sp.gpop0, sp.gpop1, sp.no_double, sp.N, s2)) {
                        ok = true;
                        e.delta = (int32_t)(__ldg(outer_off + (s2 >> n_in)) - block_off);
                        e.J = t.J;
                        e.ar = t.ar;
                        e.ai = t.ai;
                    }
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (ok) s_out[base + __popc(m & ((1u << threadIdx.x) - 1u))] = e;
            base += __popc(m);
        }
        if (threadIdx.x == 0) s_n = base;
    }
    __syncthreads();
    const int nout = s_n;
    const uint32_t* __restrict__ iptr = sp.iptr;
    const uint32_t* __restrict__ ient = sp.ient;
    const uint32_t* __restrict__ inner_rank = sp.inner_rank;
    const void* dcode = sp.dcode;
    const A* __restrict__ dtab = sp.dtab;
    const KTerm<uint32_t, A>* mixed = mixed_smem ? s_mixed : sp.mixed;
    const KVar<A>* vars = sp.vars;
    const int rbits = sp.rbits;
    const uint32_t rmask = (1u << rbits) - 1u;
    const uint32_t in_mask = sp.in_mask;
    const A u_ar = sp.u_ar, u_ai = sp.u_ai;
    const int ngroups = sp.ngroups, no_double = sp.no_double, N = sp.N, gpop0 = sp.gpop0, gpop1 = sp.gpop1;
    const uint32_t gmask0 = sp.gmask0, gmask1 = sp.gmask1;

    const int G = Rp / VPL;
    const int lr = threadIdx.x % G;
    const int rs = threadIdx.x / G;
    const int rpp = kBlock / G;
    const T2* __restrict__ Xh = X + bi.base * Rp + lr * VPL;  // row i of this Hamiltonian: Xh[i * Rp]
    T2* __restrict__ Yh = Y + bi.base * Rp + lr * VPL;
    A sc[VPL], dhi[VPL], dlo[VPL];
#pragma unroll
    for (int j = 0; j < VPL; ++j) {
        sc[j] = scale ? (A)scale[(size_t)bi.ham * Rp + lr * VPL + j] : (A)1;
        dhi[j] = 0;
        dlo[j] = 0;
    }
    for (uint32_t r = rs; r < it.count; r += rpp) {
        const uint32_t row = (uint32_t)it.row0 + r;
        const uint32_t pidx = it.inner_base + r;
        const uint32_t b = inner_state ? __ldg(inner_state + pidx) : pidx;
        const uint32_t s = (it.a << n_in) | b;
        A ar[VPL], ai[VPL];
#pragma unroll
        for (int j = 0; j < VPL; ++j) ar[j] = ai[j] = 0;
        T2 xv[VPL];
        for (int k = 0; k < nout; ++k) {
            const OutEnt<A> e = s_out[k];
            vload<T, VPL>(Xh + (size_t)(int64_t)((int64_t)row + e.delta) * Rp, xv);
            A cr = e.ar, ci = e.ai;
            if (OJ && (__popc(s & e.J) & 1)) {
                cr = -cr;
                ci = -ci;
            }
#pragma unroll
            for (int j = 0; j < VPL; ++j) cmac<A>(ar[j], ai[j], cr, ci, xv[j], REAL);
        }
        const uint32_t grp = it.pad + (r >> 5);
        const uint32_t e0 = __ldg(iptr + grp) + (r & 31u), e1 = __ldg(iptr + grp + 1);
#if QKG_BLOCK_PREFETCH
        // the next entry is loaded while this entry's gather is in flight
        uint32_t nxt = e0 < e1 ? __ldg(ient + e0) : kEllEmpty;
        for (uint32_t e = e0; nxt != kEllEmpty;) {
            const uint32_t ent = nxt;
            e += 32;
            nxt = e < e1 ? __ldg(ient + e) : kEllEmpty;
            vload<T, VPL>(Xh + (size_t)(block_off + (ent & rmask)) * Rp, xv);
#else
        for (uint32_t e = e0; e < e1; e += 32) {
            const uint32_t ent = __ldg(ient + e);
            if (ent == kEllEmpty) break;
            vload<T, VPL>(Xh + (size_t)(block_off + (ent & rmask)) * Rp, xv);
#endif
            A cr, ci;
            if (UNIF) {
                cr = u_ar;
                ci = u_ai;
            } else {
                const uint32_t t = ent >> (rbits + 1);
                cr = s_iamp[2 * t];
                ci = s_iamp[2 * t + 1];
                if ((ent >> rbits) & 1u) {
                    cr = -cr;
                    ci = -ci;
                }
            }
#pragma unroll
            for (int j = 0; j < VPL; ++j) cmac<A>(ar[j], ai[j], cr, ci, xv[j], REAL);
        }
        for (int k = 0; k < n_mixed; ++k) {
            const KTerm<uint32_t, A> t = mixed[k];
            if ((s & t.C) != t.V) continue;
            const uint32_t s2 = s ^ t.X;
            if ((t.flags & 1u) && !in_basis_fast(ngroups, gmask0, gmask1, gpop0, gpop1, no_double, N, s2)) continue;
            const uint32_t b2 = s2 & in_mask;
            const uint32_t idx = __ldg(outer_off + (s2 >> n_in)) + (inner_rank ? __ldg(inner_rank + b2) : b2);
            A cr, ci;
            term_amp<uint32_t, A>(t, s, vars, cr, ci);
            vload<T, VPL>(Xh + (size_t)idx * Rp, xv);
#pragma unroll
            for (int j = 0; j < VPL; ++j) cmac<A>(ar[j], ai[j], cr, ci, xv[j], REAL);
        }
        const uint32_t dc = diag_mode == DIAG_U8 ? (uint32_t)__ldg(static_cast<const uint8_t*>(dcode) + row)
                                                 : (uint32_t)__ldg(static_cast<const uint16_t*>(dcode) + row);
        const A dr = diag_mode == DIAG_U8 ? s_dtab[2 * dc] : __ldg(dtab + 2 * dc);
        const A di = REAL ? (A)0 : (diag_mode == DIAG_U8 ? s_dtab[2 * dc + 1] : __ldg(dtab + 2 * dc + 1));
        vload<T, VPL>(Xh + (size_t)row * Rp, xv);
        T2 out[VPL];
#pragma unroll
        for (int j = 0; j < VPL; ++j) {
            A accr = fma(dr, (A)xv[j].x, ar[j]);
            A acci = fma(dr, (A)xv[j].y, ai[j]);
            if (!REAL) {
                accr = fma(-di, (A)xv[j].y, accr);
                acci = fma(di, (A)xv[j].x, acci);
            }
            out[j].x = (T)(accr * sc[j]);
            out[j].y = (T)(acci * sc[j]);
            if (apart) {
                ffma_acc(dhi[j], dlo[j], (A)xv[j].x, (A)out[j].x);
                ffma_acc(dhi[j], dlo[j], (A)xv[j].y, (A)out[j].y);
            }
        }
        vstore<T, VPL>(Yh + (size_t)row * Rp, out);
    }
    if (apart) {
#pragma unroll
        for (int j = 0; j < VPL; ++j) s_red[threadIdx.x * VPL + j] = (double)dhi[j] + (double)dlo[j];
        __syncthreads();
        if ((int)threadIdx.x < Rp) {
            const int v = threadIdx.x, g = v / VPL, j = v % VPL;
            double acc = 0.0;
            for (int q = 0; q < rpp; ++q) acc += s_red[(q * G + g) * VPL + j];
            apart[(size_t)blockIdx.x * Rp + v] = acc;
        }
    }
}

// w = y - ca u - cb up in place on y, and per CTA the partial ||w_v||^2
// (u == nullptr: only the norms of y).  Rp divides kBlock, so each thread
// always touches the same vector v = threadIdx.x % Rp.
template <class T, class A>
__global__ void __launch_bounds__(kBlock) block_update_kernel(const BItem* __restrict__ items, int Rp,
                                                              typename V2<T>::t* __restrict__ Y,
                                                              const typename V2<T>::t* __restrict__ U,
                                                              const typename V2<T>::t* __restrict__ Up,
                                                              const double* __restrict__ ca,
                                                              const double* __restrict__ cb, double* __restrict__ part) {
    using T2 = typename V2<T>::t;
    __shared__ double s_red[kBlock];
    const BItem bi = items[blockIdx.x];
    const size_t e0 = (bi.base + bi.w.row0) * (size_t)Rp;
    const uint32_t ne = bi.w.count * (uint32_t)Rp;
    const int v = threadIdx.x % Rp;
    const size_t vid = (size_t)bi.ham * Rp + v;
    const A a = U ? (A)ca[vid] : (A)0, b = U ? (A)cb[vid] : (A)0;
    A hi = 0, lo = 0;
    for (uint32_t e = threadIdx.x; e < ne; e += kBlock) {
        const T2 y = Y[e0 + e];
        A wx = (A)y.x, wy = (A)y.y;
        if (U) {
            const T2 u = U[e0 + e], up = Up[e0 + e];
            wx = fma(-a, (A)u.x, wx);
            wy = fma(-a, (A)u.y, wy);
            wx = fma(-b, (A)up.x, wx);
            wy = fma(-b, (A)up.y, wy);
            T2 w;
            w.x = (T)wx;
            w.y = (T)wy;
            Y[e0 + e] = w;
        }
        ffma_acc(hi, lo, wx, wx);
        ffma_acc(hi, lo, wy, wy);
    }
    s_red[threadIdx.x] = (double)hi + (double)lo;
    __syncthreads();
    if ((int)threadIdx.x < Rp) {
        double acc = 0.0;
        for (int q = threadIdx.x; q < kBlock; q += Rp) acc += s_red[q];
        part[(size_t)blockIdx.x * Rp + threadIdx.x] = acc;
    }
}

struct BState {
    double *c_cur, *c_prev, *beta_prev, *ca, *cb, *norm2;
    double *alpha, *beta;  // [k * V + vid]
    int *active, *n_alpha, *n_beta, *kstep;
    int V, Rp, Ruser;
};

enum { FIN_INIT = 0, FIN_ALPHA = 1, FIN_BETA = 2 };

// Per vector (one CTA each): the sum of its CTA partials over its
// Hamiltonian's CTA range (fixed order), then the scalar bookkeeping.
__global__ void __launch_bounds__(kBlock) block_finish_kernel(const double* __restrict__ part,
                                                              const uint32_t* __restrict__ cta_range, int mode,
                                                              BState st) {
    const int vid = blockIdx.x, h = vid / st.Rp, v = vid % st.Rp;
    double acc = 0.0;
    for (uint32_t c = cta_range[h] + threadIdx.x; c < cta_range[h + 1]; c += blockDim.x) acc += part[(size_t)c * st.Rp + v];
    acc = block_sum_d(acc);
    if (threadIdx.x) return;
    if (mode == FIN_INIT) {
        st.norm2[vid] = acc;
        const double nr = sqrt(acc);
        const bool on = v < st.Ruser && nr >= 1e-15;  // dynamics.cpp:27
        st.active[vid] = on;
        st.c_cur[vid] = on ? 1.0 / nr : 0.0;
        st.c_prev[vid] = 0.0;
        st.beta_prev[vid] = 0.0;
        st.n_alpha[vid] = 0;
        st.n_beta[vid] = 0;
        return;
    }
    const int k = *st.kstep;
    if (mode == FIN_ALPHA) {
        if (st.active[vid]) {
            const double a = st.c_cur[vid] * acc;
            st.alpha[(size_t)k * st.V + vid] = a;
            st.n_alpha[vid] = k + 1;
            st.ca[vid] = a * st.c_cur[vid];
            st.cb[vid] = st.beta_prev[vid] * st.c_prev[vid];
        } else {
            st.ca[vid] = 0.0;
            st.cb[vid] = 0.0;
        }
        return;
    }
    if (!st.active[vid]) return;
    const double b = sqrt(acc);
    st.c_prev[vid] = st.c_cur[vid];
    if (b < 1e-15) {  // ftlm.cpp:45, dynamics.cpp:52
        st.active[vid] = 0;
        st.c_cur[vid] = 0.0;
        return;
    }
    st.beta[(size_t)k * st.V + vid] = b;
    st.n_beta[vid] = k + 1;
    st.c_cur[vid] = 1.0 / b;
    st.beta_prev[vid] = b;
}

__global__ void block_advance_kernel(int* k) { ++*k; }

// Seeded Philox Gaussian start vectors: vector v of Hamiltonian h, row i gets
// the Philox block (counter i, stream h * Rp + v); padding vectors are zero.
template <class T2, bool F64>
__global__ void __launch_bounds__(kBlock) block_philox_kernel(const BItem* __restrict__ items, int Rp, int Ruser,
                                                              uint64_t seed, T2* __restrict__ U) {
    const BItem bi = items[blockIdx.x];
    const size_t e0 = (bi.base + bi.w.row0) * (size_t)Rp;
    const uint32_t ne = bi.w.count * (uint32_t)Rp;
    for (uint32_t e = threadIdx.x; e < ne; e += kBlock) {
        const uint32_t v = e % Rp;
        const uint64_t row = bi.w.row0 + e / Rp;
        T2 o;
        o.x = 0;
        o.y = 0;
        if ((int)v < Ruser) o = philox_cnormal<T2, F64>(seed, (uint64_t)bi.ham * Rp + v, row);
        U[e0 + e] = o;
    }
}

// Column v of a block vector from a contiguous FP64 vector (internal order).
template <class T2>
__global__ void block_column_kernel(const double2* __restrict__ src, uint64_t n, int Rp, T2* __restrict__ dst) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        T2 o;
        o.x = src[i].x;
        o.y = src[i].y;
        dst[i * Rp] = o;
    }
}

template <class T, class A, int VPL>
void launch_block_vpl(const FastParams<A>* P, const BItem* items, unsigned n_items, int Rp, bool real, bool unif,
                      bool oj, const typename V2<T>::t* X, typename V2<T>::t* Y, const double* scale, double* apart,
                      cudaStream_t s) {
    const int key = (real ? 4 : 0) | (unif ? 2 : 0) | (oj ? 1 : 0);
    switch (key) {
        case 0: spmv_block_kernel<T, A, false, false, false, VPL><<<n_items, kBlock, 0, s>>>(P, items, Rp, X, Y, scale, apart); break;
        case 1: spmv_block_kernel<T, A, false, false, true, VPL><<<n_items, kBlock, 0, s>>>(P, items, Rp, X, Y, scale, apart); break;
        case 2: spmv_block_kernel<T, A, false, true, false, VPL><<<n_items, kBlock, 0, s>>>(P, items, Rp, X, Y, scale, apart); break;
        case 3: spmv_block_kernel<T, A, false, true, true, VPL><<<n_items, kBlock, 0, s>>>(P, items, Rp, X, Y, scale, apart); break;
        case 4: spmv_block_kernel<T, A, true, false, false, VPL><<<n_items, kBlock, 0, s>>>(P, items, Rp, X, Y, scale, apart); break;
        case 5: spmv_block_kernel<T, A, true, false, true, VPL><<<n_items, kBlock, 0, s>>>(P, items, Rp, X, Y, scale, apart); break;
        case 6: spmv_block_kernel<T, A, true, true, false, VPL><<<n_items, kBlock, 0, s>>>(P, items, Rp, X, Y, scale, apart); break;
        default: spmv_block_kernel<T, A, true, true, true, VPL><<<n_items, kBlock, 0, s>>>(P, items, Rp, X, Y, scale, apart); break;
    }
    QKG_LAUNCHED();
}

// The block engine for one arithmetic type.
template <class T, class A>
class BlockEngine {
public:
    using T2 = typename V2<T>::t;
    BlockEngine(const std::vector<Hamiltonian*>& hs, int Rp, int Ruser)
        : hs_(hs), Rp_(Rp), Ruser_(Ruser), ws_lock_(hs[0]->workspace_lock()) {
        s_ = hs[0]->stream();
        std::vector<FastParams<A>> P(hs.size());
        std::vector<BItem> items;
        std::vector<uint32_t> range(1, 0);
        real_ = unif_ = true;
        oj_ = false;
        for (size_t h = 0; h < hs.size(); ++h) {
            Hamiltonian& H = *hs[h];
            QKG_REQUIRE(H.fast(), "batched Lanczos needs every Hamiltonian on the fast SpMV kernel");
            QKG_REQUIRE(H.device() == hs[0]->device(), "batched Lanczos needs every Hamiltonian on one device");
            QKG_CUDA(cudaStreamSynchronize(H.stream()));
            H.fast_params(P[h]);
            real_ = real_ && H.all_real();
            unif_ = unif_ && H.uniform_inner();
            oj_ = oj_ || P[h].outer_has_j;
            for (const WorkItem& w : H.items_host()) items.push_back({w, rows_, (uint32_t)h, 0u});
            range.push_back((uint32_t)items.size());
            dims_.push_back(H.dim());
            bases_.push_back(rows_);
            rows_ += H.dim();
        }
        n_items_ = items.size();
        params_.alloc(P.size() * sizeof(FastParams<A>));
        QKG_CUDA(cudaMemcpy(params_.p, P.data(), P.size() * sizeof(FastParams<A>), cudaMemcpyHostToDevice));
        items_.alloc(std::max<size_t>(1, items.size()) * sizeof(BItem));
        if (!items.empty()) QKG_CUDA(cudaMemcpy(items_.p, items.data(), items.size() * sizeof(BItem), cudaMemcpyHostToDevice));
        range_.alloc(range.size() * sizeof(uint32_t));
        QKG_CUDA(cudaMemcpy(range_.p, range.data(), range.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
        // the three rotating block vectors live in the first Hamiltonian's
        // Krylov workspace, kept between calls (freeing 13 GB costs milliseconds
        // and fresh pages slow the first steps)
        const size_t vbytes = (std::max<uint64_t>(1, rows_) * Rp * sizeof(T2) + 255) / 256 * 256;
        char* ws = static_cast<char*>(hs[0]->krylov_workspace(3 * vbytes).p);
        for (int i = 0; i < 3; ++i) {
            buf_[i] = ws + (size_t)i * vbytes;
            QKG_CUDA(cudaMemsetAsync(buf_[i], 0, vbytes, s_));
        }
        apart_.alloc(std::max<size_t>(1, n_items_) * Rp * sizeof(double));
        bpart_.alloc(std::max<size_t>(1, n_items_) * Rp * sizeof(double));
    }

    uint64_t rows() const { return rows_; }
    size_t n_items() const { return n_items_; }
    T2* buf(int i) { return static_cast<T2*>(buf_[i]); }

    void spmv(int vpl, const T2* x, T2* y, const double* scale, double* apart) {
        const auto* P = params_.as<FastParams<A>>();
        const auto* it = items_.as<BItem>();
        const unsigned g = (unsigned)n_items_;
        if (!g) return;
        if (vpl == 4) launch_block_vpl<T, A, 4>(P, it, g, Rp_, real_, unif_, oj_, x, y, scale, apart, s_);
        else if (vpl == 2) launch_block_vpl<T, A, 2>(P, it, g, Rp_, real_, unif_, oj_, x, y, scale, apart, s_);
        else launch_block_vpl<T, A, 1>(P, it, g, Rp_, real_, unif_, oj_, x, y, scale, apart, s_);
    }

    // Autotuner: time the block SpMV for each vectors-per-lane choice that
    // divides Rp (at most 32 lanes per row) and keep the fastest.
    int autotune(std::vector<double>& rec) {
        rec.assign(3, 0.0);
        int best = 0;
        double best_ms = 0.0;
        const bool big = rows_ * (uint64_t)Rp_ >= (1ull << 22);
        if (!big) return std::min(Rp_, 4);  // small blocks: widest loads
        for (int vi = 0; vi < 3; ++vi) {
            const int vpl = 1 << vi;
            if (Rp_ % vpl || Rp_ / vpl > 32) continue;
            LaunchTimer tm(s_);
            spmv(vpl, buf(0), buf(1), nullptr, nullptr);
            tm.start();
            for (int r = 0; r < 2; ++r) spmv(vpl, buf(0), buf(1), nullptr, nullptr);
            tm.stop();
            QKG_CUDA(cudaStreamSynchronize(s_));
            rec[vi] = tm.collect() * 1e3 / 2.0;
            if (!best || rec[vi] < best_ms) {
                best = vpl;
                best_ms = rec[vi];
            }
        }
        return best;
    }

    void update(const T2* u, const T2* up, T2* y, const double* ca, const double* cb, double* part) {
        if (!n_items_) return;
        block_update_kernel<T, A><<<(unsigned)n_items_, kBlock, 0, s_>>>(items_.as<BItem>(), Rp_, y, u, up, ca, cb, part);
        QKG_LAUNCHED();
    }
    void finish(const double* part, int mode, const BState& st) {
        block_finish_kernel<<<(unsigned)(hs_.size() * Rp_), kBlock, 0, s_>>>(part, range_.as<uint32_t>(), mode, st);
        QKG_LAUNCHED();
    }
    void philox(uint64_t seed, T2* u) {
        if (!n_items_) return;
        block_philox_kernel<T2, sizeof(T) == 8><<<(unsigned)n_items_, kBlock, 0, s_>>>(items_.as<BItem>(), Rp_, Ruser_, seed, u);
        QKG_LAUNCHED();
    }
    // column v of Hamiltonian h from a reference-order host vector
    void set_column(size_t h, int v, const cd* host_ref, DBuf& tmp, DBuf& tmp2, T2* u) {
        Hamiltonian& H = *hs_[h];
        const uint64_t n = dims_[h];
        if (!n) return;
        if (tmp.bytes < n * sizeof(double2)) tmp.alloc(n * sizeof(double2));
        QKG_CUDA(cudaMemcpyAsync(tmp.p, host_ref, n * sizeof(double2), cudaMemcpyHostToDevice, s_));
        const double2* src = tmp.as<double2>();
        if (H.permuted()) {
            if (tmp2.bytes < n * sizeof(double2)) tmp2.alloc(n * sizeof(double2));
            H.to_internal_f64(tmp.as<double2>(), tmp2.as<double2>(), s_);
            src = tmp2.as<double2>();
        }
        const int g = (int)std::min<uint64_t>((n + 255) / 256, 152ull * 16);
        block_column_kernel<T2><<<g, 256, 0, s_>>>(src, n, Rp_, u + (bases_[h]) * Rp_ + v);
        QKG_LAUNCHED();
        QKG_CUDA(cudaStreamSynchronize(s_));  // host_ref may be reused by the caller
    }
    cudaStream_t stream() const { return s_; }

private:
    std::vector<Hamiltonian*> hs_;
    int Rp_, Ruser_;
    std::unique_lock<std::mutex> ws_lock_;  // the first Hamiltonian's workspace, held for the engine's life
    cudaStream_t s_ = nullptr;
    bool real_ = true, unif_ = true, oj_ = false;
    uint64_t rows_ = 0;
    size_t n_items_ = 0;
    std::vector<uint64_t> dims_, bases_;
    DBuf params_, items_, range_, apart_, bpart_;
    void* buf_[3] = {nullptr, nullptr, nullptr};

public:
    double* apart() { return apart_.as<double>(); }
    double* bpart() { return bpart_.as<double>(); }
};

template <class T, class A>
BlockTridiag run_block(const std::vector<Hamiltonian*>& hs, const BlockOpts& o, int Rp) {
    using T2 = typename V2<T>::t;
    BlockTridiag out;
    out.n_ham = (int)hs.size();
    out.R = o.R;
    out.steps = o.steps;
    out.rp = Rp;
    BlockEngine<T, A> E(hs, Rp, o.R);
    cudaStream_t s = E.stream();
    out.rows = E.rows();
    const int V = out.n_ham * Rp;
    const int M = std::max(0, o.steps);
    // device state
    DBuf scal(9 * (size_t)V * sizeof(double)), ab(2 * std::max<size_t>(1, (size_t)M * V) * sizeof(double)),
        ints((3 * (size_t)V + 1) * sizeof(int));
    QKG_CUDA(cudaMemsetAsync(scal.p, 0, scal.bytes, s));
    QKG_CUDA(cudaMemsetAsync(ab.p, 0, ab.bytes, s));
    QKG_CUDA(cudaMemsetAsync(ints.p, 0, ints.bytes, s));
    BState st;
    double* d = scal.as<double>();
    st.c_cur = d;
    st.c_prev = d + V;
    st.beta_prev = d + 2 * V;
    st.ca = d + 3 * V;
    st.cb = d + 4 * V;
    st.norm2 = d + 5 * V;
    st.alpha = ab.as<double>();
    st.beta = ab.as<double>() + std::max<size_t>(1, (size_t)M * V);
    int* ip = ints.as<int>();
    st.active = ip;
    st.n_alpha = ip + V;
    st.n_beta = ip + 2 * V;
    st.kstep = ip + 3 * V;
    st.V = V;
    st.Rp = Rp;
    st.Ruser = o.R;

    // start vectors into buffer 0
    T2* U0 = E.buf(0);
    if (o.start == BlockStart::Philox) {
        E.philox(o.seed, U0);
    } else {
        DBuf tmp, tmp2;
        std::vector<cd> h;
        for (size_t hh = 0; hh < hs.size(); ++hh) {
            const uint64_t n = hs[hh]->dim();
            NormalStream ns(o.f32_stream);  // restarted per Hamiltonian, as one ftlm() call per sector
            for (int v = 0; v < o.R; ++v) {
                const cd* src = nullptr;
                if (o.start == BlockStart::Given) {
                    src = o.given.at(hh * o.R + v);
                } else {
                    h.resize(n);
                    ns.fill(n, h.data());
                    src = h.data();
                }
                if (src) E.set_column(hh, v, src, tmp, tmp2, U0);
            }
        }
    }
    // tile shape: autotuned once per batch of Hamiltonians, vector width and precision
    int vpl = o.vpl;
    if (vpl <= 0) {
        static std::mutex mu;
        static std::map<std::vector<uintptr_t>, std::pair<int, std::vector<double>>> cache;
        std::vector<uintptr_t> key;
        for (auto* h : hs) {
            key.push_back(reinterpret_cast<uintptr_t>(h));
            key.push_back((uintptr_t)h->dim());
        }
        key.push_back((uintptr_t)Rp);
        key.push_back((uintptr_t)sizeof(T));
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it == cache.end()) {
            vpl = E.autotune(out.tune_ms);
            cache[key] = {vpl, out.tune_ms};
        } else {
            vpl = it->second.first;
            out.tune_ms = it->second.second;
        }
    }
    QKG_REQUIRE(Rp % vpl == 0 && Rp / vpl <= 32, "vectors per lane must divide the padded block width");
    out.vpl = vpl;
    // the autotuner wrote into buffer 1: clear it again (it is u_{-1} at step 0)
    QKG_CUDA(cudaMemsetAsync(E.buf(1), 0, std::max<uint64_t>(1, E.rows()) * Rp * sizeof(T2), s));
    QKG_CUDA(cudaMemsetAsync(E.buf(2), 0, std::max<uint64_t>(1, E.rows()) * Rp * sizeof(T2), s));

    LaunchTimer total(s), tsp(s);
    total.start();
    E.update(nullptr, nullptr, U0, nullptr, nullptr, E.bpart());  // ||u_0||^2 partials
    E.finish(E.bpart(), FIN_INIT, st);
    // step k: u_k = buf[k % 3], u_{k-1} = buf[(k + 2) % 3], y = buf[(k + 1) % 3]
    auto step = [&](int k, LaunchTimer* t) {
        T2* u = E.buf(k % 3);
        T2* up = E.buf((k + 2) % 3);
        T2* y = E.buf((k + 1) % 3);
        if (t) t->start();
        E.spmv(vpl, u, y, st.c_cur, E.apart());
        if (t) t->stop();
        E.finish(E.apart(), FIN_ALPHA, st);
        E.update(u, up, y, st.ca, st.cb, E.bpart());
        E.finish(E.bpart(), FIN_BETA, st);
        block_advance_kernel<<<1, 1, 0, s>>>(st.kstep);
        QKG_LAUNCHED();
    };
    constexpr int kStepKernels = 5;  // SpMV, alpha finish, update, beta finish, step counter
    const int eager = std::min(M, 3);
    double sp_sum = 0.0;
    for (int k = 0; k < eager; ++k) {
        step(k, &tsp);
        QKG_CUDA(cudaStreamSynchronize(s));
        sp_sum += tsp.collect();
    }
    out.spmv_ms = eager ? sp_sum * 1e3 / eager : 0.0;
    const int rest = M - eager, q = rest / 3, rem = rest % 3;
    auto capture = [&](int nsteps) {
        cudaGraph_t g;
        cudaGraphExec_t ge;
        const uint64_t c0 = launch_count();
        QKG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < nsteps; ++k) step(3 + k, nullptr);  // rotation of steps 3, 4, 5 = 0, 1, 2
        QKG_CUDA(cudaStreamEndCapture(s, &g));
        add_launches(-(int64_t)(launch_count() - c0));
        QKG_CUDA(cudaGraphInstantiate(&ge, g, 0));
        cudaGraphDestroy(g);
        return ge;
    };
    if (q > 0) {
        cudaGraphExec_t g3 = capture(3);
        for (int i = 0; i < q; ++i) {
            QKG_CUDA(cudaGraphLaunch(g3, s));
            add_launches(3 * kStepKernels);
        }
        QKG_CUDA(cudaStreamSynchronize(s));
        cudaGraphExecDestroy(g3);
    }
    if (rem > 0) {
        cudaGraphExec_t gr = capture(rem);
        QKG_CUDA(cudaGraphLaunch(gr, s));
        add_launches(rem * kStepKernels);
        QKG_CUDA(cudaStreamSynchronize(s));
        cudaGraphExecDestroy(gr);
    }
    total.stop();
    QKG_CUDA(cudaStreamSynchronize(s));
    out.seconds = total.collect();

    // results
    std::vector<double> ha((size_t)M * V), hb((size_t)M * V), hn(V);
    std::vector<int> na(V), nb(V);
    if (M) {
        QKG_CUDA(cudaMemcpy(ha.data(), st.alpha, ha.size() * sizeof(double), cudaMemcpyDeviceToHost));
        QKG_CUDA(cudaMemcpy(hb.data(), st.beta, hb.size() * sizeof(double), cudaMemcpyDeviceToHost));
    }
    QKG_CUDA(cudaMemcpy(hn.data(), st.norm2, V * sizeof(double), cudaMemcpyDeviceToHost));
    QKG_CUDA(cudaMemcpy(na.data(), st.n_alpha, V * sizeof(int), cudaMemcpyDeviceToHost));
    QKG_CUDA(cudaMemcpy(nb.data(), st.n_beta, V * sizeof(int), cudaMemcpyDeviceToHost));
    const int nv = out.n_ham * o.R;
    out.alpha.resize(nv);
    out.beta.resize(nv);
    out.norm2.resize(nv);
    for (int h = 0; h < out.n_ham; ++h)
        for (int v = 0; v < o.R; ++v) {
            const int vid = h * Rp + v, oi = h * o.R + v;
            out.norm2[oi] = hn[vid];
            for (int k = 0; k < na[vid]; ++k) out.alpha[oi].push_back(ha[(size_t)k * V + vid]);
            for (int k = 0; k < nb[vid]; ++k) out.beta[oi].push_back(hb[(size_t)k * V + vid]);
        }
    return out;
}

}  // namespace

BlockTridiag block_lanczos(const std::vector<Hamiltonian*>& hs, const BlockOpts& o) {
    QKG_REQUIRE(!hs.empty(), "no Hamiltonians");
    QKG_REQUIRE(o.R >= 1 && o.R <= 32, "vectors per Hamiltonian must be 1..32");
    QKG_REQUIRE(o.steps >= 0, "negative step count");
    QKG_REQUIRE(o.start != BlockStart::Given || o.given.size() == hs.size() * (size_t)o.R, "start vector count");
    QKG_REQUIRE(o.vpl == 0 || o.vpl == 1 || o.vpl == 2 || o.vpl == 4, "vectors per lane must be 1, 2 or 4");
    int Rp = 1;
    while (Rp < o.R) Rp *= 2;
    int dev = 0;
    QKG_CUDA(cudaGetDevice(&dev));
    QKG_REQUIRE(dev == hs[0]->device(), "current device differs from the Hamiltonians' device");
    return o.mixed ? run_block<float, float>(hs, o, Rp) : run_block<double, double>(hs, o, Rp);
}

void ftlm_observables_block(const BlockTridiag& t, const double* betas, int nb, double* Zo, double* Eo, double* Co,
                            bool shifted, double* log_zmax) {
    // per vector: eigenvalues and squared first components (ftlm.cpp:61-119)
    // (independent per vector: spread over the host cores)
    std::vector<FTLMTri> tri(t.alpha.size());
#pragma omp parallel for schedule(dynamic, 4)
    for (long long v = 0; v < (long long)t.alpha.size(); ++v) {
        FTLMTri& x = tri[v];
        x.norm2 = t.norm2[v];
        const auto& a = t.alpha[v];
        if (!a.empty()) {
            std::vector<double> b = t.beta[v];
            b.resize(a.size(), 0.0);
            std::vector<double> z;
            tridiag_eig(a.data(), b.data(), (int)a.size(), x.evals, {0}, z);
            x.w0.resize(x.evals.size());
            for (size_t j = 0; j < x.evals.size(); ++j) x.w0[j] = z[j] * z[j];
        }
    }
    // Z_h carries 1/R (ftlm.cpp:160-162): the sum over Hamiltonians of the
    // per-Hamiltonian estimates is the plain sum over all vectors divided by R.
    ftlm_observables(tri, betas, nb, Zo, Eo, Co, shifted, log_zmax);
    if (t.n_ham > 1)
        for (int k = 0; k < nb; ++k) {
            // ftlm_observables divided by the vector count n_ham * R; undo the n_ham
            Zo[k] *= t.n_ham;
        }
}

}  // namespace qkg
