// Tiled SpMV: y = Hx for the fast path (32-bit states, table ranks), one CTA
// per group of G outer blocks that share an inner class.
//
// The rows of block a are the inner configurations b of its class, so a
// block's slice of x is a row of the matrix X[a, b].  The CTA copies the G
// slices into shared memory with asynchronous bulk copies (TMA engine,
// completing on one mbarrier) and walks the columns b with one thread each:
//   inner terms   - the inner table row of b (rank of the target inner
//                   configuration, sign, term) is read once and applied to
//                   all G blocks, the gathered x read from shared memory
//                   (scattered 8-byte reads from shared memory run about five
//                   times faster on GB300 than the same reads from L1);
//   outer terms   - the block's precomputed list (delta, J, amplitude): a
//                   coalesced read of the neighbouring block's row;
//   straddling    - the terms listed for the block, ranked per row;
//   diagonal      - coded per row, times the staged x.
// The sum per row runs outer, straddling, inner, diagonal (the fast kernels'
// class order within each class is the reference's term order; the row sum
// is complete to rounding, matrix_free_hamiltonian.cpp:156-167).
//
// A wait on the bulk copies is bounded by the global timer; if it gives up the
// warp counts it (tile_wait_timeouts) and reads x from global memory instead,
// so the results stay valid, and before exiting waits once more (bounded) for
// the copies still in flight.
#include "tile.hpp"

#include <algorithm>
#include <mutex>

namespace qkg {
namespace tilek {

using namespace fastk;

namespace {

__device__ unsigned int g_tile_wait_timeouts;
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s of global time

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool mbar_test0(uint32_t bar) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar)
        : "memory");
    return done != 0;
}
// Wait for phase 0 of the mbarrier at shared address bar; false after limit_ns.
__device__ __noinline__ bool mbar_wait0_ns(uint32_t bar, unsigned long long limit_ns) {
    const unsigned long long t0 = global_ns();
    while (!mbar_test0(bar))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}
// The same for the phase of the given parity.
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __noinline__ bool mbar_wait_ns(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
    const unsigned long long t0 = global_ns();
    while (!mbar_test(bar, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}

template <class T, int G> struct MinB;
template <> struct MinB<float, 1> { static constexpr int v = 5; };
template <> struct MinB<float, 2> { static constexpr int v = 4; };
template <> struct MinB<float, 4> { static constexpr int v = 2; };
template <> struct MinB<double, 1> { static constexpr int v = 3; };
template <> struct MinB<double, 2> { static constexpr int v = 2; };
template <> struct MinB<double, 4> { static constexpr int v = 1; };

// Per-block constants of a CTA, kept in shared memory.
struct BlkInfo {
    uint32_t off, sa, o0, o1, m0, m1;
};

template <class T, class A, bool REAL, bool UNIF, bool OJ, int G>
__global__ void __launch_bounds__(kTileThreads, MinB<T, G>::v)
    spmv_tile_kernel(const FastParams<A> p, const TileItem* __restrict__ items, const typename V2<T>::t* __restrict__ x_in,
                     typename V2<T>::t* __restrict__ y_in, uint32_t slot) {
    using T2 = typename V2<T>::t;
    constexpr uint32_t E16 = 16 / sizeof(T2);  // elements per 16-byte unit
    extern __shared__ __align__(16) unsigned char tile_smem_raw[];
    T2* xs = reinterpret_cast<T2*>(tile_smem_raw);
    A* s_iamp = reinterpret_cast<A*>(tile_smem_raw + (size_t)G * slot * sizeof(T2));  // !UNIF: [G][2 n_inner]
    __shared__ unsigned long long s_bar;
    __shared__ BlkInfo s_blk[G];

    const T2* __restrict__ x = x_in;
    T2* __restrict__ y = y_in;
    A scale = (A)1, bprev = (A)0;
    const T2* __restrict__ vprev = nullptr;
    if (p.lz) {
        const LzOperands o = *p.lz;
        x = static_cast<const T2*>(o.x);
        y = static_cast<T2*>(o.y);
        vprev = static_cast<const T2*>(o.vprev);
        scale = sizeof(A) == 4 ? (A)o.scale32 : (A)o.scale;
        bprev = sizeof(A) == 4 ? (A)o.bprev32 : (A)o.bprev;
    }
    const TileItem it = items[blockIdx.x];
    const uint32_t W = it.width, tid = threadIdx.x, lane = tid & 31u;
    const bool aligned = (reinterpret_cast<uintptr_t>(x) & 15u) == 0;

    // Slot g holds x[st0 .. off + W) of block g from xs[g * slot] on, st0 the
    // 16-byte boundary at or below off; base[g] is the slot index of row 0.
    uint32_t base[G];
    bool need_wait = false;
    uint32_t bytes = 0;
#pragma unroll
    for (int g = 0; g < G; ++g) {
        const bool has = g < (int)it.nblk;
        const uint32_t a = has ? it.a[g] : it.a[0];
        const uint32_t off = __ldg(p.outer_off + a);
        const uint32_t st0 = off & ~(E16 - 1u), end = (off + W) & ~(E16 - 1u);
        base[g] = (uint32_t)g * slot + (off - st0);
        const bool bulk = has && aligned && end > st0;
        if (bulk) {
            need_wait = true;
            bytes += (end - st0) * (uint32_t)sizeof(T2);
            for (uint32_t i = end + tid; i < off + W; i += kTileThreads) xs[(uint32_t)g * slot + (i - st0)] = x[i];
        } else if (has) {
            for (uint32_t i = tid; i < W; i += kTileThreads) xs[base[g] + i] = x[off + i];
        }
        if (tid == 0) {
            BlkInfo bi;
            bi.off = off;
            bi.sa = a << p.n_in;
            bi.o0 = has ? __ldg(p.optr + a) : 0u;
            bi.o1 = has ? __ldg(p.optr + a + 1) : 0u;
            bi.m0 = has ? __ldg(p.mptr + a) : 0u;
            bi.m1 = has ? __ldg(p.mptr + a + 1) : 0u;
            s_blk[g] = bi;
        }
        if (!UNIF && has) {
            const uint32_t sa = a << p.n_in;
            for (int t = tid; t < p.n_inner; t += kTileThreads) {
                const KTerm<uint32_t, A> k = p.inner[t];
                const bool neg = __popc(sa & k.J) & 1;
                s_iamp[(2 * g) * p.n_inner + 2 * t] = neg ? -k.ar : k.ar;
                s_iamp[(2 * g) * p.n_inner + 2 * t + 1] = neg ? -k.ai : k.ai;
            }
        }
    }
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&s_bar);
    if (tid == 0 && need_wait) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0 && need_wait) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
#pragma unroll
        for (int g = 0; g < G; ++g) {
            if (g >= (int)it.nblk) break;
            const uint32_t off = s_blk[g].off;
            const uint32_t st0 = off & ~(E16 - 1u), end = (off + W) & ~(E16 - 1u);
            if (!(end > st0)) continue;
            const uint32_t dst = (uint32_t)__cvta_generic_to_shared(xs + (uint32_t)g * slot);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                "l"(x + st0), "r"((end - st0) * (uint32_t)sizeof(T2)), "r"(bar)
                : "memory");
        }
    }

    const uint32_t rmask = (1u << p.rbits) - 1u;
    bool staged = true;          // slices read from shared memory
    bool waited = !need_wait;
    A dot_hi = 0, dot_lo = 0;

    for (uint32_t j0 = 0; j0 < W; j0 += kTileThreads) {
        const uint32_t j = j0 + tid;
        const bool live = j < W;
        const uint32_t jl = live ? j : 0u;
        const uint32_t b = p.inner_state ? __ldg(p.inner_state + it.inner_base + jl) : it.inner_base + jl;
        A ar[G], ai[G];
#pragma unroll
        for (int g = 0; g < G; ++g) ar[g] = ai[g] = (A)0;
        if (live) {
            // outer terms: coalesced rows of the neighbouring blocks
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (g >= (int)it.nblk) break;
                const uint32_t o0 = s_blk[g].o0, o1 = s_blk[g].o1, off = s_blk[g].off, s = s_blk[g].sa | b;
                for (uint32_t k = o0; k < o1; ++k) {
                    const OutEnt<A> e = p.oent[k];
                    const T2 xv = x[(uint32_t)((int32_t)(off + j) + e.delta)];
                    A cr = e.ar, ci = e.ai;
                    if (OJ && (__popc(s & e.J) & 1)) {
                        cr = -cr;
                        ci = -ci;
                    }
                    cmac<A>(ar[g], ai[g], cr, ci, xv, REAL);
                }
            }
            // straddling terms listed for the block, ranked per row
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (g >= (int)it.nblk) break;
                const uint32_t m0 = s_blk[g].m0, m1 = s_blk[g].m1, s = s_blk[g].sa | b;
                for (uint32_t m = m0; m < m1; ++m) {
                    const uint2 mk = __ldg(p.ment + m);
                    const KTerm<uint32_t, A> t = p.mixed[mk.x];
                    bool ok = (s & t.C) == t.V;
                    const uint32_t s2 = s ^ t.X;
                    if (ok && (t.flags & 1u))
                        ok = in_basis_fast(p.ngroups, p.gmask0, p.gmask1, p.gpop0, p.gpop1, p.no_double, p.N, s2);
                    if (!ok) continue;
                    const uint32_t b2 = s2 & p.in_mask;
                    const T2 xv = x[mk.y + (p.inner_rank ? __ldg(p.inner_rank + b2) : b2)];
                    A cr, ci;
                    term_amp<uint32_t, A>(t, s, p.vars, cr, ci);
                    cmac<A>(ar[g], ai[g], cr, ci, xv, REAL);
                }
            }
        }
        if (!waited) {
            // one lane per warp polls; the warp follows its verdict
            bool ok = true;
            if (lane == 0) ok = mbar_wait0_ns(bar, kWaitLimitNs);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            // every lane observes the completed phase itself (its own acquire)
            if (ok) mbar_test0(bar);
            if (!ok) {
                staged = false;
                if (lane == 0) atomicAdd(&g_tile_wait_timeouts, 1u);
            }
            waited = true;
        }
        if (live) {
            // inner terms: one table walk for the G blocks, gathers from shared memory
            const uint32_t grp = it.grp + (j >> 5);
            uint32_t e0 = __ldg(p.iptr + grp) + lane;
            const uint32_t e1 = __ldg(p.iptr + grp + 1);
            uint32_t cur = e0 < e1 ? __ldg(p.ient + e0) : kEllEmpty;
            while (cur != kEllEmpty) {
                e0 += 32;
                const uint32_t nxt = e0 < e1 ? __ldg(p.ient + e0) : kEllEmpty;
                const uint32_t r = cur & rmask;
                T2 xv[G];
#pragma unroll
                for (int g = 0; g < G; ++g)
                    if (g < (int)it.nblk) xv[g] = staged ? xs[base[g] + r] : x[s_blk[g].off + r];
                const bool neg = (cur >> p.rbits) & 1u;
                const uint32_t t = cur >> (p.rbits + 1);
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if (g >= (int)it.nblk) break;
                    if (UNIF) {
                        cmac<A>(ar[g], ai[g], p.u_ar, p.u_ai, xv[g], REAL);
                    } else {
                        A cr = s_iamp[(2 * g) * p.n_inner + 2 * t], ci = s_iamp[(2 * g) * p.n_inner + 2 * t + 1];
                        if (neg) {
                            cr = -cr;
                            ci = -ci;
                        }
                        cmac<A>(ar[g], ai[g], cr, ci, xv[g], REAL);
                    }
                }
                cur = nxt;
            }
            // diagonal, scale, previous-vector term, store
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (g >= (int)it.nblk) break;
                const uint32_t row = s_blk[g].off + j;
                const uint32_t dc = p.diag_mode == DIAG_U8 ? (uint32_t)__ldg(static_cast<const uint8_t*>(p.dcode) + row)
                                                           : (uint32_t)__ldg(static_cast<const uint16_t*>(p.dcode) + row);
                const T2 xd = staged ? xs[base[g] + j] : x[row];
                const A dr = __ldg(p.dtab + 2 * dc);
                A accr = fma(dr, (A)xd.x, ar[g]);
                A acci = fma(dr, (A)xd.y, ai[g]);
                if (!REAL) {
                    const A di = __ldg(p.dtab + 2 * dc + 1);
                    accr = fma(-di, (A)xd.y, accr);
                    acci = fma(di, (A)xd.x, acci);
                }
                A o_r = accr * scale, o_i = acci * scale;
                if (vprev) {
                    const T2 pv = vprev[row];
                    o_r = fma(-bprev, (A)pv.x, o_r);
                    o_i = fma(-bprev, (A)pv.y, o_i);
                }
                T2 out;
                out.x = (T)o_r;
                out.y = (T)o_i;
                y[row] = out;
                if (p.apart) {
                    ffma_acc(dot_hi, dot_lo, (A)xd.x, (A)out.x);
                    ffma_acc(dot_hi, dot_lo, (A)xd.y, (A)out.y);
                }
            }
        }
    }
    if (!waited) {  // no pass ran (W == 0 cannot happen for a listed block; kept for safety)
        if (lane == 0 && !mbar_wait0_ns(bar, kWaitLimitNs)) atomicAdd(&g_tile_wait_timeouts, 1u);
    } else if (!staged && lane == 0) {
        // the copies may still be writing this CTA's shared memory: wait for them before exiting
        if (!mbar_wait0_ns(bar, kWaitLimitNs)) atomicAdd(&g_tile_wait_timeouts, 1u);
    }
    if (p.apart) {
        if (sizeof(A) == 4) {
            const float2 t = block_sum_ff((float)dot_hi, (float)dot_lo);
            if (tid == 0) p.apart[blockIdx.x] = make_double2((double)t.x + (double)t.y, 0.0);
        } else {
            const double t = block_sum_d((double)dot_hi + (double)dot_lo);
            if (tid == 0) p.apart[blockIdx.x] = make_double2(t, 0.0);
        }
    }
}

// Thread 0 of a class CTA: block bi's slice of x into buffer b, the part below
// a whole 16-byte unit by plain stores first, then the arrival that releases
// them (expecting the bulk copy's bytes when there is one).
template <class T2>
__device__ __noinline__ void class_issue(const uint32_t* __restrict__ outer_off, const ClassPlan plan,
                                         const T2* __restrict__ x, T2* xs, const uint32_t* bar, uint32_t bi, int b,
                                         uint32_t* issued) {
    constexpr uint32_t E16 = 16 / sizeof(T2);
    const CBlock cb = plan.blocks[bi];
    const uint32_t W = plan.classes[cb.cls].W;
    const uint32_t off = __ldg(outer_off + cb.a);
    const uint32_t st0 = off & ~(E16 - 1u), end = (off + W) & ~(E16 - 1u);
    T2* dst = xs + (uint32_t)b * plan.slot;
    for (uint32_t i = (end > st0 ? end : off); i < off + W; ++i) dst[i - st0] = x[i];
    if (end > st0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar[b]),
                     "r"((end - st0) * (uint32_t)sizeof(T2))
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                (uint32_t)__cvta_generic_to_shared(dst)),
            "l"(x + st0), "r"((end - st0) * (uint32_t)sizeof(T2)), "r"(bar[b])
            : "memory");
    } else {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar[b]) : "memory");
    }
    ++issued[b];
}

// ------------------------------------------------------------ class-persistent
// One 1024-thread CTA per SM.  CTA k walks blocks k, k + grid, k + 2 grid, ...
// of a list sorted by inner class, so all SMs sweep the list together and the
// neighbouring blocks the outer terms read stay in L2 while a class runs.
// Per class the CTA copies the class's rows of the inner table (and its group
// offsets) into shared memory and keeps, per thread, the inner configurations
// and table positions of its four columns (j = 128 warp + lane + 32 q).  Per
// block, thread 0 first issues the bulk copy of the NEXT block's slice into the
// other buffer, then the CTA sums the outer and straddling terms from global
// memory, waits (bounded) for this block's slice and walks the inner table with
// both the table and x in shared memory.  A wait that gives up is counted, the
// CTA reads x from global memory from then on, and before exiting waits
// (bounded) for the copies still in flight.
template <class T, class A, bool REAL, bool UNIF, bool OJ>
__global__ void __launch_bounds__(kClassThreads, 1)
    spmv_class_kernel(const FastParams<A> p, const ClassPlan plan, const typename V2<T>::t* __restrict__ x_in,
                      typename V2<T>::t* __restrict__ y_in) {
    using T2 = typename V2<T>::t;
    constexpr uint32_t E16 = 16 / sizeof(T2);
    constexpr int RT = kClassCols;
    extern __shared__ __align__(16) unsigned char cls_smem_raw[];
    T2* xs = reinterpret_cast<T2*>(cls_smem_raw);  // two slices of plan.slot elements
    uint32_t* ell = reinterpret_cast<uint32_t*>(cls_smem_raw + 2 * (size_t)plan.slot * sizeof(T2));
    uint32_t* gp = ell + plan.ell_cap;  // plan.gcap + 1 group offsets (relative to ell)
    A* s_iamp = reinterpret_cast<A*>(cls_smem_raw + 2 * (size_t)plan.slot * sizeof(T2) +
                                     ((((size_t)plan.ell_cap + plan.gcap + 1) * 4 + 15) / 16) * 16);
    __shared__ unsigned long long s_bar[2];

    const T2* __restrict__ x = x_in;
    T2* __restrict__ y = y_in;
    A scale = (A)1, bprev = (A)0;
    const T2* __restrict__ vprev = nullptr;
    if (p.lz) {
        const LzOperands o = *p.lz;
        x = static_cast<const T2*>(o.x);
        y = static_cast<T2*>(o.y);
        vprev = static_cast<const T2*>(o.vprev);
        scale = sizeof(A) == 4 ? (A)o.scale32 : (A)o.scale;
        bprev = sizeof(A) == 4 ? (A)o.bprev32 : (A)o.bprev;
    }
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t nb = plan.nblocks, G = gridDim.x;
    const uint32_t bar[2] = {(uint32_t)__cvta_generic_to_shared(&s_bar[0]),
                             (uint32_t)__cvta_generic_to_shared(&s_bar[1])};
    bool use_smem = (reinterpret_cast<uintptr_t>(x) & 15u) == 0;  // uniform
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar[0]) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar[1]) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    uint32_t issued[2] = {0u, 0u};  // thread 0: copies issued per buffer
    if (tid == 0 && use_smem && blockIdx.x < nb)
        class_issue<T2>(p.outer_off, plan, x, xs, bar, blockIdx.x, 0, issued);

    const uint32_t rmask = (1u << p.rbits) - 1u;
    A dot_hi = 0, dot_lo = 0;
    int loaded = -1;
    uint32_t bcol[RT];
    uint32_t it = 0;
    for (uint32_t bi = blockIdx.x; bi < nb; bi += G, ++it) {
        const int buf = (int)(it & 1u);
        const CBlock cb = plan.blocks[bi];
        const CClass cc = plan.classes[cb.cls];
        const uint32_t W = cc.W, off = __ldg(p.outer_off + cb.a);
        if ((int)cb.cls != loaded) {
            // the previous block is finished (barrier at the end of each block)
            for (uint32_t k = tid; k < cc.ell1 - cc.ell0; k += kClassThreads) ell[k] = __ldg(p.ient + cc.ell0 + k);
            for (uint32_t k = tid; k <= cc.ngroups; k += kClassThreads) gp[k] = __ldg(p.iptr + cc.gbase + k) - cc.ell0;
            __syncthreads();
#pragma unroll
            for (int q = 0; q < RT; ++q) {
                const uint32_t j = warp * (32u * RT) + lane + 32u * q;
                const uint32_t jl = j < W ? j : 0u;
                bcol[q] = p.inner_state ? __ldg(p.inner_state + cc.inner_base + jl) : cc.inner_base + jl;
            }
            loaded = (int)cb.cls;
        }
        const uint32_t sa = cb.a << p.n_in;
        if (!UNIF) {
            for (int t = tid; t < p.n_inner; t += kClassThreads) {
                const KTerm<uint32_t, A> k = p.inner[t];
                const bool neg = __popc(sa & k.J) & 1;
                s_iamp[2 * t] = neg ? -k.ar : k.ar;
                s_iamp[2 * t + 1] = neg ? -k.ai : k.ai;
            }
            __syncthreads();
        }
        // the next block's slice goes into the other buffer while this one runs
        if (tid == 0 && use_smem && bi + G < nb) class_issue<T2>(p.outer_off, plan, x, xs, bar, bi + G, buf ^ 1, issued);

        A ar_[RT], ai_[RT];
        bool live[RT];
#pragma unroll
        for (int q = 0; q < RT; ++q) {
            ar_[q] = ai_[q] = (A)0;
            live[q] = warp * (32u * RT) + lane + 32u * q < W;
        }
        const T2* xr = x + off + warp * (32u * RT) + lane;  // column q of this thread: xr[32 q]
        // outer terms: the block's list, a coalesced row of the neighbouring block per entry
        {
            const uint32_t o1 = __ldg(p.optr + cb.a + 1);
            for (uint32_t k = __ldg(p.optr + cb.a); k < o1; ++k) {
                const OutEnt<A> e = p.oent[k];
                T2 xv[RT];
#pragma unroll
                for (int q = 0; q < RT; ++q)
                    if (live[q]) xv[q] = xr[32 * q + e.delta];
#pragma unroll
                for (int q = 0; q < RT; ++q) {
                    if (!live[q]) continue;
                    A cr = e.ar, ci = e.ai;
                    if (OJ && (__popc((sa | bcol[q]) & e.J) & 1)) {
                        cr = -cr;
                        ci = -ci;
                    }
                    cmac<A>(ar_[q], ai_[q], cr, ci, xv[q], REAL);
                }
            }
        }
        // straddling terms listed for the block, ranked per column
        {
            const uint32_t m1 = __ldg(p.mptr + cb.a + 1);
            for (uint32_t m = __ldg(p.mptr + cb.a); m < m1; ++m) {
                const uint2 mk = __ldg(p.ment + m);
                const KTerm<uint32_t, A> t = p.mixed[mk.x];
                uint32_t idx[RT];
                bool ok[RT];
#pragma unroll
                for (int q = 0; q < RT; ++q) {
                    const uint32_t s = sa | bcol[q];
                    ok[q] = live[q] && (s & t.C) == t.V;
                    const uint32_t s2 = s ^ t.X;
                    if (ok[q] && (t.flags & 1u))
                        ok[q] = in_basis_fast(p.ngroups, p.gmask0, p.gmask1, p.gpop0, p.gpop1, p.no_double, p.N, s2);
                    const uint32_t b2 = s2 & p.in_mask;
                    idx[q] = ok[q] ? mk.y + (p.inner_rank ? __ldg(p.inner_rank + b2) : b2) : 0u;
                }
                T2 xv[RT];
#pragma unroll
                for (int q = 0; q < RT; ++q)
                    if (ok[q]) xv[q] = x[idx[q]];
#pragma unroll
                for (int q = 0; q < RT; ++q) {
                    if (!ok[q]) continue;
                    A cr, ci;
                    term_amp<uint32_t, A>(t, sa | bcol[q], p.vars, cr, ci);
                    cmac<A>(ar_[q], ai_[q], cr, ci, xv[q], REAL);
                }
            }
        }
        // this block's slice: bounded wait, one lane per warp polls
        bool staged = use_smem;
        if (use_smem) {
            const uint32_t parity = (it >> 1) & 1u;
            bool ok = true;
            if (lane == 0) ok = mbar_wait_ns(bar[buf], parity, kWaitLimitNs);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (ok) mbar_test(bar[buf], parity);  // each lane's own acquire of the completed phase
            else if (lane == 0) atomicAdd(&g_tile_wait_timeouts, 1u);
            staged = ok;
        }
        const T2* xsb = xs + (uint32_t)buf * plan.slot + (off - (off & ~(E16 - 1u)));  // row 0 of the block
        const T2* xg = x + off;
        // inner terms: the class's table and the slice in shared memory.
        // Column q of this thread lies in group 4 warp + q of the class, whose
        // slot count is the same for the whole warp.
#pragma unroll
        for (int q = 0; q < RT; ++q) {
            const uint32_t g = warp * RT + q;
            if (g * 32u >= W) break;  // warp-uniform: groups past the class end
            const uint32_t e0 = gp[g], ns = (gp[g + 1] - e0) >> 5;
            const uint32_t* __restrict__ ep = ell + e0 + lane;
            for (uint32_t k = 0; k < ns; ++k) {
                const uint32_t ent = ep[32u * k];
                if (ent == kEllEmpty) continue;
                const T2 xv = staged ? xsb[ent & rmask] : xg[ent & rmask];
                if (UNIF) {
                    cmac<A>(ar_[q], ai_[q], p.u_ar, p.u_ai, xv, REAL);
                } else {
                    const uint32_t t = ent >> (p.rbits + 1);
                    A cr = s_iamp[2 * t], ci = s_iamp[2 * t + 1];
                    if ((ent >> p.rbits) & 1u) {
                        cr = -cr;
                        ci = -ci;
                    }
                    cmac<A>(ar_[q], ai_[q], cr, ci, xv, REAL);
                }
            }
        }
        // diagonal, scale, previous-vector term, store
#pragma unroll
        for (int q = 0; q < RT; ++q) {
            if (!live[q]) continue;
            const uint32_t j = warp * (32u * RT) + lane + 32u * q;
            const uint32_t row = off + j;
            const uint32_t dc = p.diag_mode == DIAG_U8 ? (uint32_t)__ldg(static_cast<const uint8_t*>(p.dcode) + row)
                                                       : (uint32_t)__ldg(static_cast<const uint16_t*>(p.dcode) + row);
            const T2 xd = staged ? xsb[j] : xg[j];
            const A dr = __ldg(p.dtab + 2 * dc);
            A accr = fma(dr, (A)xd.x, ar_[q]);
            A acci = fma(dr, (A)xd.y, ai_[q]);
            if (!REAL) {
                const A di = __ldg(p.dtab + 2 * dc + 1);
                accr = fma(-di, (A)xd.y, accr);
                acci = fma(di, (A)xd.x, acci);
            }
            A o_r = accr * scale, o_i = acci * scale;
            if (vprev) {
                const T2 pv = vprev[row];
                o_r = fma(-bprev, (A)pv.x, o_r);
                o_i = fma(-bprev, (A)pv.y, o_i);
            }
            T2 out;
            out.x = (T)o_r;
            out.y = (T)o_i;
            y[row] = out;
            if (p.apart) {
                ffma_acc(dot_hi, dot_lo, (A)xd.x, (A)out.x);
                ffma_acc(dot_hi, dot_lo, (A)xd.y, (A)out.y);
            }
        }
        // every thread is done with this buffer (and, at a class change, the
        // table); a wait that gave up anywhere stops the use of shared memory
        const int gave_up = __syncthreads_or(use_smem && !staged);
        if (gave_up) use_smem = false;
    }
    // copies still in flight into this CTA's shared memory finish before it exits
    if (tid == 0)
        for (int b = 0; b < 2; ++b)
            if (issued[b] && !mbar_wait_ns(bar[b], (issued[b] - 1u) & 1u, kWaitLimitNs))
                atomicAdd(&g_tile_wait_timeouts, 1u);
    if (p.apart) {
        if (sizeof(A) == 4) {
            const float2 t = block_sum_ff((float)dot_hi, (float)dot_lo);
            if (tid == 0) p.apart[blockIdx.x] = make_double2((double)t.x + (double)t.y, 0.0);
        } else {
            const double t = block_sum_d((double)dot_hi + (double)dot_lo);
            if (tid == 0) p.apart[blockIdx.x] = make_double2(t, 0.0);
        }
    }
}

template <class T, class A>
void launch_class_key(const FastParams<A>& p, const ClassPlan& plan, unsigned grid, int key,
                      const typename V2<T>::t* x, typename V2<T>::t* y, size_t smem, cudaStream_t s) {
    switch (key) {
        case 0: spmv_class_kernel<T, A, false, false, false><<<grid, kClassThreads, smem, s>>>(p, plan, x, y); break;
        case 1: spmv_class_kernel<T, A, false, false, true><<<grid, kClassThreads, smem, s>>>(p, plan, x, y); break;
        case 2: spmv_class_kernel<T, A, false, true, false><<<grid, kClassThreads, smem, s>>>(p, plan, x, y); break;
        case 3: spmv_class_kernel<T, A, false, true, true><<<grid, kClassThreads, smem, s>>>(p, plan, x, y); break;
        case 4: spmv_class_kernel<T, A, true, false, false><<<grid, kClassThreads, smem, s>>>(p, plan, x, y); break;
        case 5: spmv_class_kernel<T, A, true, false, true><<<grid, kClassThreads, smem, s>>>(p, plan, x, y); break;
        case 6: spmv_class_kernel<T, A, true, true, false><<<grid, kClassThreads, smem, s>>>(p, plan, x, y); break;
        default: spmv_class_kernel<T, A, true, true, true><<<grid, kClassThreads, smem, s>>>(p, plan, x, y); break;
    }
}

template <class T, class A>
void allow_class(int bytes) {
    QKG_CUDA(cudaFuncSetAttribute(spmv_class_kernel<T, A, false, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_class_kernel<T, A, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_class_kernel<T, A, false, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_class_kernel<T, A, false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_class_kernel<T, A, true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_class_kernel<T, A, true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_class_kernel<T, A, true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_class_kernel<T, A, true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

template <class T, class A, int G>
void launch_g(const FastParams<A>& p, const TileItem* items, unsigned n, int key, const typename V2<T>::t* x,
              typename V2<T>::t* y, uint32_t slot, size_t smem, cudaStream_t s) {
    switch (key) {
        case 0: spmv_tile_kernel<T, A, false, false, false, G><<<n, kTileThreads, smem, s>>>(p, items, x, y, slot); break;
        case 1: spmv_tile_kernel<T, A, false, false, true, G><<<n, kTileThreads, smem, s>>>(p, items, x, y, slot); break;
        case 2: spmv_tile_kernel<T, A, false, true, false, G><<<n, kTileThreads, smem, s>>>(p, items, x, y, slot); break;
        case 3: spmv_tile_kernel<T, A, false, true, true, G><<<n, kTileThreads, smem, s>>>(p, items, x, y, slot); break;
        case 4: spmv_tile_kernel<T, A, true, false, false, G><<<n, kTileThreads, smem, s>>>(p, items, x, y, slot); break;
        case 5: spmv_tile_kernel<T, A, true, false, true, G><<<n, kTileThreads, smem, s>>>(p, items, x, y, slot); break;
        case 6: spmv_tile_kernel<T, A, true, true, false, G><<<n, kTileThreads, smem, s>>>(p, items, x, y, slot); break;
        default: spmv_tile_kernel<T, A, true, true, true, G><<<n, kTileThreads, smem, s>>>(p, items, x, y, slot); break;
    }
}

template <class T, class A, int G>
void allow_g(int bytes) {
    QKG_CUDA(cudaFuncSetAttribute(spmv_tile_kernel<T, A, false, false, false, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_tile_kernel<T, A, false, false, true, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_tile_kernel<T, A, false, true, false, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_tile_kernel<T, A, false, true, true, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_tile_kernel<T, A, true, false, false, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_tile_kernel<T, A, true, false, true, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_tile_kernel<T, A, true, true, false, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    QKG_CUDA(cudaFuncSetAttribute(spmv_tile_kernel<T, A, true, true, true, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

}  // namespace

template <class T, class A>
void launch_tile(const FastParams<A>& p, const TileItem* items, size_t n_items, int G, bool real, bool unif,
                 const typename V2<T>::t* x, typename V2<T>::t* y, uint32_t slot, size_t smem, cudaStream_t s) {
    if (!n_items) return;
    QKG_REQUIRE(smem <= kTileSmemLimit, "tile SpMV: shared memory above the limit");
    const unsigned n = (unsigned)n_items;
    const int key = (real ? 4 : 0) | (unif ? 2 : 0) | (p.outer_has_j ? 1 : 0);
    if (G == 1) launch_g<T, A, 1>(p, items, n, key, x, y, slot, smem, s);
    else if (G == 2) launch_g<T, A, 2>(p, items, n, key, x, y, slot, smem, s);
    else launch_g<T, A, 4>(p, items, n, key, x, y, slot, smem, s);
    QKG_LAUNCHED();
}

template <class T, class A>
void launch_class(const FastParams<A>& p, const ClassPlan& plan, unsigned grid, bool real, bool unif,
                  const typename V2<T>::t* x, typename V2<T>::t* y, size_t smem, cudaStream_t s) {
    if (!plan.nblocks || !grid) return;
    QKG_REQUIRE(smem <= kTileSmemLimit, "class SpMV: shared memory above the limit");
    {
        static std::mutex mu;
        static uint64_t done = 0;
        int dev = 0;
        QKG_CUDA(cudaGetDevice(&dev));
        std::lock_guard<std::mutex> lk(mu);
        const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
        if (!(bit && (done & bit))) {
            allow_class<T, A>((int)kTileSmemLimit);
            done |= bit;
        }
    }
    const int key = (real ? 4 : 0) | (unif ? 2 : 0) | (p.outer_has_j ? 1 : 0);
    launch_class_key<T, A>(p, plan, grid, key, x, y, smem, s);
    QKG_LAUNCHED();
}

template <class T, class A>
void tile_allow_smem(size_t bytes) {
    // The attribute belongs to the kernel on the current device, not to a
    // Hamiltonian: it is raised once per device to the limit every tile launch
    // stays under, so no Hamiltonian's setting can shrink another's.
    static std::mutex mu;
    static uint64_t done = 0;  // devices already raised (bit per device id < 64)
    if (bytes == 0) return;
    int dev = 0;
    QKG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
    if (bit && (done & bit)) return;
    const int b = (int)kTileSmemLimit;
    allow_g<T, A, 1>(b);
    allow_g<T, A, 2>(b);
    allow_g<T, A, 4>(b);
    done |= bit;
}

namespace {
// One thread waits on an mbarrier that nothing will complete (no copy is ever
// issued on it) for limit_ns of global time, counts the give-up like a tile
// kernel's, then arrives on the barrier itself so no phase is left pending.
__global__ void wait_probe_kernel(unsigned long long limit_ns) {
    __shared__ unsigned long long bar;
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
    if (threadIdx.x != 0) return;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    if (!mbar_wait0_ns(b, limit_ns)) atomicAdd(&g_tile_wait_timeouts, 1u);
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(b) : "memory");
}
}  // namespace

void wait_probe(long long limit_ns) {
    const unsigned long long lim = (unsigned long long)std::min<long long>(std::max<long long>(limit_ns, 1000), 1000000000);
    wait_probe_kernel<<<1, 32>>>(lim);
    QKG_LAUNCHED();
    QKG_CUDA(cudaDeviceSynchronize());
}

uint32_t tile_wait_timeouts() {
    QKG_CUDA(cudaDeviceSynchronize());
    uint32_t c = 0;
    QKG_CUDA(cudaMemcpyFromSymbol(&c, g_tile_wait_timeouts, sizeof(c)));
    return c;
}

template void launch_tile<float, float>(const FastParams<float>&, const TileItem*, size_t, int, bool, bool,
                                        const float2*, float2*, uint32_t, size_t, cudaStream_t);
template void launch_tile<double, double>(const FastParams<double>&, const TileItem*, size_t, int, bool, bool,
                                          const double2*, double2*, uint32_t, size_t, cudaStream_t);
template void launch_class<float, float>(const FastParams<float>&, const ClassPlan&, unsigned, bool, bool,
                                          const float2*, float2*, size_t, cudaStream_t);
template void launch_class<double, double>(const FastParams<double>&, const ClassPlan&, unsigned, bool, bool,
                                            const double2*, double2*, size_t, cudaStream_t);
template void tile_allow_smem<float, float>(size_t);
template void tile_allow_smem<double, double>(size_t);

}  // namespace tilek
}  // namespace qkg
