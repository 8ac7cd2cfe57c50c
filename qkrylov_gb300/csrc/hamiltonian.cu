// Matrix-free y = Hx on the GPU.
//
// The reference builds a host CSR once (src/hamiltonian/matrix_free_hamiltonian.cpp:45-92)
// and applies it with one thread per row (:156-167), which costs 20 bytes of
// matrix stream per nonzero and int32 offsets that overflow beyond 2^31
// nonzeros.  Here nothing but the diagonal (as a 1- or 2-byte code per row) is
// stored: every off-diagonal entry is regenerated in the kernel from the
// compiled term masks (compile.cpp) and ranked with the basis tables
// (basis.cpp).  The row sum is
//     y[a] = d[a] x[a] + sum_t conj(amp_t(s_a)) x[rank(s_a ^ X_t)]
// which is the reference's y[alpha] = sum_j vals[j] x[cols[j]] with the
// diagonal entries of one row pre-summed in term order (the reference's own
// diagonal accumulation, :86-89).
//
// Work decomposition: rows are grouped into work items that lie inside one
// outer block (constant high bits a).  Terms are classified at construction:
//   outer  - flips and conditions only on outer bits: validity and the target
//            block are the same for every row of the item, so they are
//            evaluated once per block (by one warp in the generic kernel, at
//            construction for the fast kernels) and each row only adds
//            x[row+delta] (a coalesced, contiguous stream from the
//            neighbouring block);
//   inner  - flips and conditions only on inner bits: the target lies in the
//            same block, rank = block offset + inner_rank[b'];
//   mixed  - everything else: full rank of the target.
#include "fast_common.cuh"
#include "tile.hpp"

#include <algorithm>
#include <mutex>
#include <atomic>
#include <string>
#include <cstring>
#include <set>
#include <utility>

namespace qkg {

namespace {
std::atomic<int64_t> g_live_allocs{0};
std::atomic<int64_t> g_fail_after{-1};  // allocations left before an injected failure (-1: none)
}  // namespace

void device_alloc(void** p, size_t bytes) {
    *p = nullptr;
    int64_t left = g_fail_after.load();
    while (left >= 0 && !g_fail_after.compare_exchange_weak(left, left - 1)) {
    }
    if (left == 0)
        throw Error(CUDA_ERR, "cudaMalloc(" + std::to_string(bytes) + " bytes): out of memory (injected failure)");
    QKG_CUDA(cudaMalloc(p, std::max<size_t>(bytes, 1)));
    ++g_live_allocs;
}
void device_free(void* p) {
    if (!p) return;
    cudaFree(p);
    --g_live_allocs;
}
int64_t live_device_allocs() { return g_live_allocs.load(); }
void inject_alloc_failure(int64_t after_n) { g_fail_after.store(after_n < 0 ? -1 : after_n); }

void DBuf::alloc(size_t n) {
    reset();
    if (n) {
        device_alloc(&p, n);
        bytes = n;
    }
}
void DBuf::reset() {
    device_free(p);
    p = nullptr;
    bytes = 0;
}

namespace {

using namespace fastk;

constexpr size_t kSmemTermBudget = 40 * 1024;

template <class S>
__device__ __forceinline__ bool in_basis(const DevBasis& b, S s) {
    if (b.ngroups > 0 && popcnt<S>(s & (S)b.gmask[0]) != b.gpop[0]) return false;
    if (b.ngroups > 1 && popcnt<S>(s & (S)b.gmask[1]) != b.gpop[1]) return false;
    if (b.no_double && (s & (s >> b.N) & (S)((1ULL << b.N) - 1))) return false;
    return true;
}

__device__ __forceinline__ uint64_t outer_off(const DevBasis& b, uint64_t a) {
    return b.idx32 ? (uint64_t)__ldg(static_cast<const uint32_t*>(b.outer_off) + a)
                   : (uint64_t)__ldg(static_cast<const unsigned long long*>(b.outer_off) + a);
}

template <class S>
__device__ __forceinline__ uint64_t rank_table(const DevBasis& b, S s) {
    const uint64_t a = (uint64_t)(s >> b.n_in);
    const S bb = s & (S)b.in_mask;
    return outer_off(b, a) + (b.inner_all ? (uint64_t)bb : (uint64_t)__ldg(b.inner_rank + bb));
}

template <class S>
__device__ __forceinline__ uint64_t rank_search(const DevBasis& b, S s) {
    const uint64_t a = b.n_out ? (uint64_t)((uint64_t)s >> b.n_in) : 0;
    uint64_t lo = outer_off(b, a), hi = outer_off(b, a + 1);
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (__ldg(reinterpret_cast<const unsigned long long*>(b.states_int) + mid) < (uint64_t)s) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

template <class S, int RANK>
__device__ __forceinline__ uint64_t rank_of(const DevBasis& b, S s) {
    return RANK == RANK_TABLE ? rank_table<S>(b, s) : rank_search<S>(b, s);
}

// Row state of row r of a work item.
template <class S, int RANK>
__device__ __forceinline__ S row_state(const DevBasis& b, const WorkItem& it, uint32_t r) {
    if (RANK == RANK_TABLE) {
        const S bb = b.inner_all ? (S)(it.inner_base + r) : (S)__ldg(b.inner_state + it.inner_base + r);
        return (S)(((uint64_t)it.a << b.n_in) | (uint64_t)bb);
    }
    return (S)__ldg(reinterpret_cast<const unsigned long long*>(b.states_int) + it.row0 + r);
}

template <class S, class A>
struct SpmvParams {
    DevBasis b;
    const WorkItem* items;
    const KTerm<S, A>* outer;
    const KTerm<S, A>* inner;
    const KTerm<S, A>* mixed;
    const KVar<A>* vars;
    int n_outer, n_inner, n_mixed, n_vars;
    int terms_in_smem;
    int real;
    int diag_mode;
    const void* dcode;
    const void* dtab;   // A pairs
    const void* dfull;  // T pairs per row (DIAG_FULL)
};

template <class S, class T, class A, int RANK>
__global__ void __launch_bounds__(kBlock) spmv_kernel(const SpmvParams<S, A> p, const typename V2<T>::t* __restrict__ x,
                                                      typename V2<T>::t* __restrict__ y) {
    using T2 = typename V2<T>::t;
    using Term = KTerm<S, A>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_nvalid;
    __shared__ int s_ti[kMaxOuter];
    __shared__ long long s_delta[kMaxOuter];

    const Term* outer = p.outer;
    const Term* inner = p.inner;
    const Term* mixed = p.mixed;
    const KVar<A>* vars = p.vars;
    if (p.terms_in_smem) {
        // Stage the term lists (read by every row) in shared memory.
        Term* st = reinterpret_cast<Term*>(smem_raw);
        const int nt = p.n_outer + p.n_inner + p.n_mixed;
        for (int i = threadIdx.x; i < nt; i += blockDim.x) {
            st[i] = i < p.n_outer ? p.outer[i] : (i < p.n_outer + p.n_inner ? p.inner[i - p.n_outer] : p.mixed[i - p.n_outer - p.n_inner]);
        }
        KVar<A>* sv = reinterpret_cast<KVar<A>*>(st + nt);
        for (int i = threadIdx.x; i < p.n_vars; i += blockDim.x) sv[i] = p.vars[i];
        outer = st;
        inner = st + p.n_outer;
        mixed = st + p.n_outer + p.n_inner;
        vars = sv;
        __syncthreads();
    }
    const DevBasis& b = p.b;
    const bool real = p.real;

    const WorkItem it = p.items[blockIdx.x];
    uint64_t block_off = 0;
    int nvalid = 0;
    if (RANK == RANK_TABLE) {
        block_off = outer_off(b, it.a);
        if (p.n_outer > 0) {
            if (threadIdx.x < 32) {
                // One warp finds the outer terms valid for this block, in term order.
                const S s0 = row_state<S, RANK>(b, it, 0);
                int base = 0;
                for (int t0 = 0; t0 < p.n_outer; t0 += 32) {
                    const int ti = t0 + (int)threadIdx.x;
                    bool ok = false;
                    long long delta = 0;
                    if (ti < p.n_outer) {
                        const Term t = outer[ti];
                        if ((s0 & t.C) == t.V) {
                            const S s2 = s0 ^ t.X;
                            if (!(t.flags & 1u) || in_basis<S>(b, s2)) {
                                ok = true;
                                delta = (long long)outer_off(b, (uint64_t)(s2 >> b.n_in)) - (long long)block_off;
                            }
                        }
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, ok);
                    if (ok) {
                        const int pos = base + __popc(m & ((1u << threadIdx.x) - 1u));
                        s_ti[pos] = ti;
                        s_delta[pos] = delta;
                    }
                    base += __popc(m);
                }
                if (threadIdx.x == 0) s_nvalid = base;
            }
            __syncthreads();
            nvalid = s_nvalid;
        }
    }

    for (uint32_t r = threadIdx.x; r < it.count; r += blockDim.x) {
        const uint64_t row = it.row0 + r;
        const S s = row_state<S, RANK>(b, it, r);
        A accr, acci;
        {
            A dr, di;
            if (p.diag_mode == DIAG_U8) {
                const uint32_t c = __ldg(static_cast<const uint8_t*>(p.dcode) + row);
                const A* tab = static_cast<const A*>(p.dtab);
                dr = tab[2 * c];
                di = tab[2 * c + 1];
            } else if (p.diag_mode == DIAG_U16) {
                const uint32_t c = __ldg(static_cast<const uint16_t*>(p.dcode) + row);
                const A* tab = static_cast<const A*>(p.dtab);
                dr = tab[2 * c];
                di = tab[2 * c + 1];
            } else {
                const T2 d = static_cast<const T2*>(p.dfull)[row];
                dr = (A)d.x;
                di = (A)d.y;
            }
            const T2 xv = x[row];
            accr = dr * (A)xv.x;
            acci = dr * (A)xv.y;
            if (!real) {
                accr = fma(-di, (A)xv.y, accr);
                acci = fma(di, (A)xv.x, acci);
            }
        }
        for (int k = 0; k < nvalid; ++k) {
            const Term t = outer[s_ti[k]];
            A ar, ai;
            term_amp<S, A>(t, s, vars, ar, ai);
            const T2 xv = x[row + s_delta[k]];
            cmac<A>(accr, acci, ar, ai, xv, real);
        }
        for (int k = 0; k < p.n_inner; ++k) {
            const Term t = inner[k];
            if ((s & t.C) != t.V) continue;
            const S s2 = s ^ t.X;
            if ((t.flags & 1u) && !in_basis<S>(b, s2)) continue;
            const S b2 = s2 & (S)b.in_mask;
            const uint64_t idx = block_off + (b.inner_all ? (uint64_t)b2 : (uint64_t)__ldg(b.inner_rank + b2));
            A ar, ai;
            term_amp<S, A>(t, s, vars, ar, ai);
            const T2 xv = x[idx];
            cmac<A>(accr, acci, ar, ai, xv, real);
        }
        for (int k = 0; k < p.n_mixed; ++k) {
            const Term t = mixed[k];
            if ((s & t.C) != t.V) continue;
            const S s2 = s ^ t.X;
            if ((t.flags & 1u) && !in_basis<S>(b, s2)) continue;
            const uint64_t idx = rank_of<S, RANK>(b, s2);
            A ar, ai;
            term_amp<S, A>(t, s, vars, ar, ai);
            const T2 xv = x[idx];
            cmac<A>(accr, acci, ar, ai, xv, real);
        }
        T2 out;
        out.x = (T)accr;
        out.y = (T)acci;
        y[row] = out;
    }
}

// ---------------------------------------------------------------------------
// Fast path (32-bit states, table ranks, 32-bit indices, coded diagonal).
//
// Inner terms are replaced by a table built once per Hamiltonian: for every
// inner configuration b (indexed like inner_state, so consecutive rows of a
// work item read consecutive table rows) the list of (target inner rank,
// amplitude index) of the inner terms valid on b, in term order, with their
// Jordan-Wigner sign folded in.  The table depends only on b, so one copy
// serves every block.  Outer terms come from a per-block list built at
// construction (optr/oent); of the remaining (straddling) terms, those whose
// outer-bit condition holds on the block are listed per block with their
// target block offset (mptr/ment) and evaluated per row.
// STAGE: the work item is a whole outer block and its x slice is staged in
// shared memory, so inner-table gathers read shared memory.
template <class T, class A, bool REAL, bool UNIF, bool OJ, bool STAGE>
__global__ void __launch_bounds__(kBlock) spmv_fast_kernel(const FastParams<A> p, const typename V2<T>::t* __restrict__ x_in,
                                                           typename V2<T>::t* __restrict__ y_in) {
    using T2 = typename V2<T>::t;
    extern __shared__ __align__(16) unsigned char fast_smem[];
    T2* xs = reinterpret_cast<T2*>(fast_smem);
    const T2* __restrict__ x = x_in;
    T2* __restrict__ y = y_in;
    A scale = (A)1, bprev = (A)0;
    const T2* __restrict__ vprev = nullptr;
    if (p.lz) {
        const LzOperands o = *p.lz;
        x = static_cast<const T2*>(o.x);
        y = static_cast<T2*>(o.y);
        vprev = static_cast<const T2*>(o.vprev);
        scale = sizeof(A) == 4 ? (A)o.scale32 : (A)o.scale;  // no per-thread FP64 conversion for FP32
        bprev = sizeof(A) == 4 ? (A)o.bprev32 : (A)o.bprev;
    }
    A dot_hi = 0, dot_lo = 0;  // Re sum conj(x) y over this thread's rows (Lanczos mode)
    __shared__ A s_iamp[2 * kMaxInnerTable];
    const WorkItem it = p.items[blockIdx.x];
    const uint32_t block_off = __ldg(p.outer_off + it.a);
    if (STAGE)  // the item is the whole block: rows [block_off, block_off + count)
        for (uint32_t i = threadIdx.x; i < it.count; i += blockDim.x) xs[i] = x[block_off + i];
    if (!UNIF) {
        // inner-term amplitudes with the sign their JW mask takes on this block's outer bits
        const uint32_t sa = it.a << p.n_in;
        for (int t = threadIdx.x; t < p.n_inner; t += blockDim.x) {
            const KTerm<uint32_t, A> k = p.inner[t];
            const bool neg = __popc(sa & k.J) & 1;
            s_iamp[2 * t] = neg ? -k.ar : k.ar;
            s_iamp[2 * t + 1] = neg ? -k.ai : k.ai;
        }
    }
    if (STAGE || !UNIF) __syncthreads();
    // this block's outer entries and straddling terms, listed per outer configuration
    const uint32_t o0 = __ldg(p.optr + it.a), o1 = __ldg(p.optr + it.a + 1);
    const uint32_t m0 = __ldg(p.mptr + it.a), m1 = __ldg(p.mptr + it.a + 1);
    const uint32_t rmask = (1u << p.rbits) - 1u;
    for (uint32_t r = threadIdx.x; r < it.count; r += blockDim.x) {
        const uint32_t row = (uint32_t)it.row0 + r;
        const uint32_t pidx = it.inner_base + r;
        const uint32_t b = p.inner_state ? __ldg(p.inner_state + pidx) : pidx;
        const uint32_t s = (it.a << p.n_in) | b;
        // ELL group of this row (32 rows per group, lane = r % 32)
        const uint32_t grp = it.pad + (r >> 5);
        const uint32_t e0 = __ldg(p.iptr + grp) + (r & 31u), e1 = __ldg(p.iptr + grp + 1);
        const uint32_t dc = p.diag_mode == DIAG_U8 ? (uint32_t)__ldg(static_cast<const uint8_t*>(p.dcode) + row)
                                                   : (uint32_t)__ldg(static_cast<const uint16_t*>(p.dcode) + row);
        const T2 xd = STAGE ? xs[r] : x[row];
        A accr = 0, acci = 0;
#pragma unroll 2
        for (uint32_t k = o0; k < o1; ++k) {
            const OutEnt<A> e = p.oent[k];
            const T2 xv = x[row + e.delta];
            A ar = e.ar, ai = e.ai;
            if (OJ && (__popc(s & e.J) & 1)) {
                ar = -ar;
                ai = -ai;
            }
            cmac<A>(accr, acci, ar, ai, xv, REAL);
        }
#pragma unroll 2
        for (uint32_t e = e0; e < e1; e += 32) {
            const uint32_t ent = __ldg(p.ient + e);
            if (ent == kEllEmpty) break;  // a row's entries fill its first slots
            const T2 xv = STAGE ? xs[ent & rmask] : x[block_off + (ent & rmask)];
            if (UNIF) {
                cmac<A>(accr, acci, p.u_ar, p.u_ai, xv, REAL);
            } else {
                const uint32_t t = ent >> (p.rbits + 1);
                A ar = s_iamp[2 * t], ai = s_iamp[2 * t + 1];
                if ((ent >> p.rbits) & 1u) {
                    ar = -ar;
                    ai = -ai;
                }
                cmac<A>(accr, acci, ar, ai, xv, REAL);
            }
        }
        for (uint32_t j = m0; j < m1; ++j) {
            const uint2 mk = __ldg(p.ment + j);
            const KTerm<uint32_t, A> t = p.mixed[mk.x];
            if ((s & t.C) != t.V) continue;
            const uint32_t s2 = s ^ t.X;
            if ((t.flags & 1u) && !in_basis_fast(p.ngroups, p.gmask0, p.gmask1, p.gpop0, p.gpop1, p.no_double, p.N, s2))
                continue;
            const uint32_t b2 = s2 & p.in_mask;
            const uint32_t idx = mk.y + (p.inner_rank ? __ldg(p.inner_rank + b2) : b2);
            A ar, ai;
            term_amp<uint32_t, A>(t, s, p.vars, ar, ai);
            cmac<A>(accr, acci, ar, ai, x[idx], REAL);
        }
        {
            const A dr = __ldg(p.dtab + 2 * dc);
            accr = fma(dr, (A)xd.x, accr);
            acci = fma(dr, (A)xd.y, acci);
            if (!REAL) {
                const A di = __ldg(p.dtab + 2 * dc + 1);
                accr = fma(-di, (A)xd.y, accr);
                acci = fma(di, (A)xd.x, acci);
            }
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
    if (p.apart) {
        if (sizeof(A) == 4) {
            const float2 t = block_sum_ff((float)dot_hi, (float)dot_lo);
            if (threadIdx.x == 0) p.apart[blockIdx.x] = make_double2((double)t.x + (double)t.y, 0.0);
        } else {
            const double t = block_sum_d((double)dot_hi + (double)dot_lo);
            if (threadIdx.x == 0) p.apart[blockIdx.x] = make_double2(t, 0.0);
        }
    }
}

// Unstaged fast kernel, four rows per thread: in a 1024-row work item warp w
// covers rows 128w .. 128w+127, lane l taking rows 128w + l + 32q (q < 4), so
// row q of every lane lies in one 32-row ELL group.  Every outer entry and
// every straddling term is read once per thread and applied to its four rows,
// which also gives four independent gathers in flight per entry; the four
// rows' ELL walks advance together.
constexpr int kRowsPerThread = 4;
static_assert(kRowsPerThread * kBlock == kChunk, "work items hold kRowsPerThread rows per thread");

// Resident CTAs per SM the register allocation is held to (FP32 / FP64).
#ifndef QKG_ROWS_MINB
#define QKG_ROWS_MINB 5
#endif
#ifndef QKG_ROWS_MINB64
#define QKG_ROWS_MINB64 2
#endif
#ifndef QKG_ELL_PREFETCH
#define QKG_ELL_PREFETCH 1
#endif
#ifndef QKG_STAGE_BULK
#define QKG_STAGE_BULK 1
#endif
// Waits on an mbarrier that gave up (bounded by the global timer): counted
// here, read by the host through spmv_wait_timeouts().  A thread whose wait
// gave up reads x from global memory instead of the staged copy (its results
// stay valid) and, before the CTA exits, waits once more (bounded) for the copy
// still in flight into its shared memory.
__device__ unsigned int g_spmv_wait_timeouts;
constexpr unsigned long long kMbarWaitNs = 2000000000ull;  // 2 s of global time

// One-shot bulk copy of `bytes` (a multiple of 16, both addresses 16-byte
// aligned) from global to shared memory, completing on the mbarrier `bar`.
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(bar), d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(d),
                 "l"(src), "r"(bytes), "r"(b)
                 : "memory");
}
// Bounded wait for phase 0 of `bar`; false once limit_ns of global time passed.
__device__ __noinline__ bool mbar_wait0(unsigned long long* bar, unsigned long long limit_ns) {
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(bar);
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(b)
            : "memory");
        if (done) return true;
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > limit_ns) return false;
    }
}

#ifndef QKG_ROWS_MINB_WIDE
#define QKG_ROWS_MINB_WIDE 4
#endif
// WIDE: a larger register budget (4 instead of 5 resident CTAs per SM), which
// pays where straddling terms keep more state live.
template <class T, class A, bool REAL, bool UNIF, bool OJ, bool STAGE, bool WIDE = false, int RT = kRowsPerThread>
__global__ void __launch_bounds__(kBlock, sizeof(T) == 4 ? (WIDE ? QKG_ROWS_MINB_WIDE : (STAGE ? QKG_ROWS_MINB - 1 : QKG_ROWS_MINB)) : QKG_ROWS_MINB64) spmv_rows_kernel(const FastParams<A> p, const typename V2<T>::t* __restrict__ x_in,
                                                           typename V2<T>::t* __restrict__ y_in) {
    using T2 = typename V2<T>::t;
    extern __shared__ __align__(16) unsigned char rows_smem[];
    T2* xs = reinterpret_cast<T2*>(rows_smem);  // STAGE: the outer block's slice of x
    const T2* __restrict__ x = x_in;
    T2* __restrict__ y = y_in;
    A scale = (A)1, bprev = (A)0;
    const T2* __restrict__ vprev = nullptr;
    if (p.lz) {
        const LzOperands o = *p.lz;
        x = static_cast<const T2*>(o.x);
        y = static_cast<T2*>(o.y);
        vprev = static_cast<const T2*>(o.vprev);
        scale = sizeof(A) == 4 ? (A)o.scale32 : (A)o.scale;  // no per-thread FP64 conversion for FP32
        bprev = sizeof(A) == 4 ? (A)o.bprev32 : (A)o.bprev;
    }
    __shared__ A s_iamp[2 * kMaxInnerTable];
    const WorkItem it = p.items[blockIdx.x];
    const uint32_t block_off = __ldg(p.outer_off + it.a);
    // STAGE: the item is the whole outer block, rows [block_off, block_off +
    // count); xs holds x from the even index st0 = block_off & ~1 on, so row i
    // of the block is xst[i] = xs[(block_off & 1) + i]
    const T2* xst = xs + (block_off & 1u);
#if QKG_STAGE_BULK
    // the slice arrives by one asynchronous bulk copy (TMA engine) issued
    // before the outer terms are summed and waited for before the inner walk
    __shared__ unsigned long long s_bar;
    bool bulk = false;
    if (STAGE) {
        const uint32_t st0 = block_off & ~1u, end = (block_off + it.count) & ~1u;  // [st0, end): whole 16-byte pairs
        bulk = end > st0 && (reinterpret_cast<uintptr_t>(x) & 15u) == 0;
        if (bulk) {
            if (threadIdx.x == 0) mbar_init(&s_bar);
            if (threadIdx.x == 32 && end < block_off + it.count) xs[end - st0] = x[end];  // odd last row
        } else {
            for (uint32_t i = threadIdx.x; i < it.count; i += blockDim.x) xs[(block_off & 1u) + i] = x[block_off + i];
        }
    }
#else
    if (STAGE)
        for (uint32_t i = threadIdx.x; i < it.count; i += blockDim.x) xs[(block_off & 1u) + i] = x[block_off + i];
#endif
    if (!UNIF) {
        const uint32_t sa = it.a << p.n_in;
        for (int t = threadIdx.x; t < p.n_inner; t += blockDim.x) {
            const KTerm<uint32_t, A> k = p.inner[t];
            const bool neg = __popc(sa & k.J) & 1;
            s_iamp[2 * t] = neg ? -k.ar : k.ar;
            s_iamp[2 * t + 1] = neg ? -k.ai : k.ai;
        }
    }
    if (STAGE || !UNIF) __syncthreads();
#if QKG_STAGE_BULK
    if (STAGE && bulk && threadIdx.x == 0) {
        const uint32_t st0 = block_off & ~1u, end = (block_off + it.count) & ~1u;
        bulk_g2s(xs, x + st0, (end - st0) * (uint32_t)sizeof(T2), &s_bar);
    }
#endif
    // this block's outer entries and straddling terms (with their target block
    // offsets), listed per outer configuration at construction
    const uint32_t o0 = __ldg(p.optr + it.a), o1 = __ldg(p.optr + it.a + 1);
    const uint32_t m0 = __ldg(p.mptr + it.a), m1 = __ldg(p.mptr + it.a + 1);
    const uint32_t rmask = (1u << p.rbits) - 1u;

    A dot_hi = 0, dot_lo = 0;
    bool staged_ok = true;  // STAGE: the slice is read from shared memory
    // a warp covers RT * 32 consecutive rows: row q of this thread is tbase + 32 q
    const uint32_t tbase = (threadIdx.x & ~31u) * RT + (threadIdx.x & 31u);
    // passes of kChunk rows (one pass unless a whole outer block is staged)
    for (uint32_t pass = 0; pass < (STAGE ? it.count : 1u); pass += RT * kBlock) {
    uint32_t s[RT], e0[RT], e1[RT];
    A ar_[RT], ai_[RT];
    bool live[RT];
    const T2* xr = x + (uint32_t)it.row0 + pass + tbase;  // row q of this thread is xr[q * 32]
#pragma unroll
    for (int q = 0; q < RT; ++q) {
        const uint32_t r = pass + tbase + q * 32u;
        live[q] = r < it.count;
        const uint32_t rr = live[q] ? r : 0;
        const uint32_t pidx = it.inner_base + rr;
        const uint32_t b = p.inner_state ? __ldg(p.inner_state + pidx) : pidx;
        s[q] = (it.a << p.n_in) | b;
        const uint32_t grp = it.pad + (rr >> 5);
        e0[q] = __ldg(p.iptr + grp) + (rr & 31u);
        e1[q] = live[q] ? __ldg(p.iptr + grp + 1) : 0u;
        ar_[q] = 0;
        ai_[q] = 0;
    }
    for (uint32_t k = o0; k < o1; ++k) {
        const OutEnt<A> e = p.oent[k];
        T2 xv[RT];
#pragma unroll
        for (int q = 0; q < RT; ++q)
            if (live[q]) xv[q] = xr[q * 32 + e.delta];
#pragma unroll
        for (int q = 0; q < RT; ++q) {
            if (!live[q]) continue;
            A cr = e.ar, ci = e.ai;
            if (OJ && (__popc(s[q] & e.J) & 1)) {
                cr = -cr;
                ci = -ci;
            }
            cmac<A>(ar_[q], ai_[q], cr, ci, xv[q], REAL);
        }
    }
    // the four rows' ELL walks, slot by slot
#if QKG_STAGE_BULK
    if (STAGE && bulk && pass == 0 && !mbar_wait0(&s_bar, kMbarWaitNs)) {
        atomicAdd(&g_spmv_wait_timeouts, 1u);
        staged_ok = false;
    }
#endif
#if QKG_ELL_PREFETCH
    // the next slot's entries are loaded while this slot's gathers are in flight
    uint32_t cur[RT];
#pragma unroll
    for (int q = 0; q < RT; ++q) cur[q] = e0[q] < e1[q] ? __ldg(p.ient + e0[q]) : kEllEmpty;
    bool more = true;
    while (more) {
        uint32_t nxt[RT];
        T2 xv[RT];
#pragma unroll
        for (int q = 0; q < RT; ++q) {
            e0[q] += 32;
            nxt[q] = (cur[q] != kEllEmpty && e0[q] < e1[q]) ? __ldg(p.ient + e0[q]) : kEllEmpty;
            if (cur[q] != kEllEmpty)
                xv[q] = (STAGE && staged_ok) ? xst[cur[q] & rmask] : x[block_off + (cur[q] & rmask)];
        }
        more = false;
#pragma unroll
        for (int q = 0; q < RT; ++q) {
            if (cur[q] != kEllEmpty) {
                if (UNIF) {
                    cmac<A>(ar_[q], ai_[q], p.u_ar, p.u_ai, xv[q], REAL);
                } else {
                    const uint32_t t = cur[q] >> (p.rbits + 1);
                    A cr = s_iamp[2 * t], ci = s_iamp[2 * t + 1];
                    if ((cur[q] >> p.rbits) & 1u) {
                        cr = -cr;
                        ci = -ci;
                    }
                    cmac<A>(ar_[q], ai_[q], cr, ci, xv[q], REAL);
                }
            }
            cur[q] = nxt[q];
            more = more || (nxt[q] != kEllEmpty);
        }
    }
#else
    bool more = true;
    while (more) {
        more = false;
        uint32_t ent[RT];
#pragma unroll
        for (int q = 0; q < RT; ++q) {
            ent[q] = kEllEmpty;
            if (e0[q] < e1[q]) ent[q] = __ldg(p.ient + e0[q]);
        }
        T2 xv[RT];
#pragma unroll
        for (int q = 0; q < RT; ++q)
            if (ent[q] != kEllEmpty)
                xv[q] = (STAGE && staged_ok) ? xst[ent[q] & rmask] : x[block_off + (ent[q] & rmask)];
#pragma unroll
        for (int q = 0; q < RT; ++q) {
            if (ent[q] == kEllEmpty) {
                e0[q] = e1[q];
                continue;
            }
            if (UNIF) {
                cmac<A>(ar_[q], ai_[q], p.u_ar, p.u_ai, xv[q], REAL);
            } else {
                const uint32_t t = ent[q] >> (p.rbits + 1);
                A cr = s_iamp[2 * t], ci = s_iamp[2 * t + 1];
                if ((ent[q] >> p.rbits) & 1u) {
                    cr = -cr;
                    ci = -ci;
                }
                cmac<A>(ar_[q], ai_[q], cr, ci, xv[q], REAL);
            }
            e0[q] += 32;
            more = more || (e0[q] < e1[q]);
        }
    }
#endif
    for (uint32_t j = m0; j < m1; ++j) {
        // the four rows' targets first (their rank lookups in flight together),
        // then the gathers, then the sums
        const uint2 mk = __ldg(p.ment + j);
        const KTerm<uint32_t, A> t = p.mixed[mk.x];
        uint32_t idx[RT];
        bool ok[RT];
#pragma unroll
        for (int q = 0; q < RT; ++q) {
            ok[q] = live[q] && (s[q] & t.C) == t.V;
            const uint32_t s2 = s[q] ^ t.X;
            if (ok[q] && (t.flags & 1u))
                ok[q] = in_basis_fast(p.ngroups, p.gmask0, p.gmask1, p.gpop0, p.gpop1, p.no_double, p.N, s2);
            idx[q] = 0;
            if (ok[q]) {
                const uint32_t b2 = s2 & p.in_mask;
                idx[q] = mk.y + (p.inner_rank ? __ldg(p.inner_rank + b2) : b2);
            }
        }
        T2 xv[RT];
#pragma unroll
        for (int q = 0; q < RT; ++q)
            if (ok[q]) xv[q] = x[idx[q]];
#pragma unroll
        for (int q = 0; q < RT; ++q) {
            if (!ok[q]) continue;
            A cr, ci;
            term_amp<uint32_t, A>(t, s[q], p.vars, cr, ci);
            cmac<A>(ar_[q], ai_[q], cr, ci, xv[q], REAL);
        }
    }
    T2 xd[RT], pv[RT];
    uint32_t dc[RT];
#pragma unroll
    for (int q = 0; q < RT; ++q) {
        const uint32_t rl = live[q] ? pass + tbase + q * 32u : 0u;
        const uint32_t row = (uint32_t)it.row0 + rl;
        dc[q] = p.diag_mode == DIAG_U8 ? (uint32_t)__ldg(static_cast<const uint8_t*>(p.dcode) + row)
                                       : (uint32_t)__ldg(static_cast<const uint16_t*>(p.dcode) + row);
        xd[q] = (STAGE && staged_ok) ? xst[rl] : x[row];
        // v_{k-1} and y are touched once per step: loaded and stored evict-first
        // (cache-streaming), so the gathered x keeps more of L2
        if (vprev) pv[q] = __ldcs(vprev + row);
    }
#pragma unroll
    for (int q = 0; q < RT; ++q) {
        if (!live[q]) continue;
        const A dr = __ldg(p.dtab + 2 * dc[q]);
        A accr = fma(dr, (A)xd[q].x, ar_[q]);
        A acci = fma(dr, (A)xd[q].y, ai_[q]);
        if (!REAL) {
            const A di = __ldg(p.dtab + 2 * dc[q] + 1);
            accr = fma(-di, (A)xd[q].y, accr);
            acci = fma(di, (A)xd[q].x, acci);
        }
        A o_r = accr * scale, o_i = acci * scale;
        if (vprev) {
            o_r = fma(-bprev, (A)pv[q].x, o_r);
            o_i = fma(-bprev, (A)pv[q].y, o_i);
        }
        T2 out;
        out.x = (T)o_r;
        out.y = (T)o_i;
        __stcs(y + ((uint32_t)it.row0 + pass + tbase + q * 32u), out);
        if (p.apart) {
            ffma_acc(dot_hi, dot_lo, (A)xd[q].x, (A)out.x);
            ffma_acc(dot_hi, dot_lo, (A)xd[q].y, (A)out.y);
        }
    }
    }
#if QKG_STAGE_BULK
    // a copy that outlived this thread's wait is still writing shared memory:
    // wait for it (bounded) before the CTA exits
    if (STAGE && bulk && !staged_ok && !mbar_wait0(&s_bar, kMbarWaitNs)) atomicAdd(&g_spmv_wait_timeouts, 1u);
#endif
    if (p.apart) {
        if (sizeof(A) == 4) {
            const float2 t = block_sum_ff((float)dot_hi, (float)dot_lo);
            if (threadIdx.x == 0) p.apart[blockIdx.x] = make_double2((double)t.x + (double)t.y, 0.0);
        } else {
            const double t = block_sum_d((double)dot_hi + (double)dot_lo);
            if (threadIdx.x == 0) p.apart[blockIdx.x] = make_double2(t, 0.0);
        }
    }
}

// Diagonal of H, summed in OpSum term order like the reference
// (matrix_free_hamiltonian.cpp:86-89).
template <class S, int RANK>
__global__ void __launch_bounds__(kBlock) diag_kernel(const DevBasis b, const WorkItem* __restrict__ items,
                                                      const KTerm<S, double>* __restrict__ diag, int n_diag,
                                                      const KVar<double>* __restrict__ vars, double2* __restrict__ out) {
    const WorkItem it = items[blockIdx.x];
    for (uint32_t r = threadIdx.x; r < it.count; r += blockDim.x) {
        const S s = row_state<S, RANK>(b, it, r);
        double sr = 0.0, si = 0.0;
        for (int k = 0; k < n_diag; ++k) {
            const KTerm<S, double> t = diag[k];
            if ((s & t.C) != t.V) continue;
            double ar, ai;
            term_amp<S, double>(t, s, vars, ar, ai);
            sr += ar;
            si += ai;
        }
        out[it.row0 + r] = make_double2(sr, si);
    }
}

// Code each diagonal value by binary search in a sorted table of bit patterns;
// values not in the table are collected (bounded) for the next round.
__global__ void diag_code_kernel(const double2* __restrict__ d, uint64_t n, const ulonglong2* __restrict__ tab, int ntab,
                                 void* codes, int code_bytes, ulonglong2* missing, unsigned long long* n_missing,
                                 unsigned long long cap) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double2 v = d[i];
        const unsigned long long kx = (unsigned long long)__double_as_longlong(v.x);
        const unsigned long long ky = (unsigned long long)__double_as_longlong(v.y);
        int lo = 0, hi = ntab;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            const ulonglong2 t = tab[mid];
            if (t.x < kx || (t.x == kx && t.y < ky)) lo = mid + 1;
            else hi = mid;
        }
        int code = 0;
        if (lo < ntab && tab[lo].x == kx && tab[lo].y == ky) {
            code = lo;
        } else {
            const unsigned long long slot = atomicAdd(n_missing, 1ULL);
            if (slot < cap) missing[slot] = make_ulonglong2(kx, ky);
        }
        if (code_bytes == 1) static_cast<uint8_t*>(codes)[i] = (uint8_t)code;
        else static_cast<uint16_t*>(codes)[i] = (uint16_t)code;
    }
}

template <class A>
__global__ void diag_expand_kernel(const void* codes, int code_bytes, const A* tab, uint64_t n, typename V2<A>::t* out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = code_bytes == 1 ? static_cast<const uint8_t*>(codes)[i] : static_cast<const uint16_t*>(codes)[i];
        typename V2<A>::t o;
        o.x = tab[2 * c];
        o.y = tab[2 * c + 1];
        out[i] = o;
    }
}

__global__ void d2f_kernel(const double2* __restrict__ a, float2* __restrict__ b, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

template <class V, class I>
__global__ void gather_kernel(const V* __restrict__ src, V* __restrict__ dst, const I* __restrict__ perm, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[perm[i]];
}
template <class V, class I>
__global__ void scatter_kernel(const V* __restrict__ src, V* __restrict__ dst, const I* __restrict__ perm, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        dst[perm[i]] = src[i];
}

// Debug emitter: every entry of every row in term order (count pass, then fill).
template <class S, int RANK>
__global__ void emit_kernel(const DevBasis b, const WorkItem* __restrict__ items, const KTerm<S, double>* __restrict__ all,
                            int n_all, const KVar<double>* __restrict__ vars, const unsigned long long* __restrict__ offs,
                            unsigned long long* __restrict__ counts, unsigned long long* __restrict__ cols,
                            double2* __restrict__ vals) {
    const WorkItem it = items[blockIdx.x];
    for (uint32_t r = threadIdx.x; r < it.count; r += blockDim.x) {
        const uint64_t row = it.row0 + r;
        const S s = row_state<S, RANK>(b, it, r);
        unsigned long long k = 0;
        for (int q = 0; q < n_all; ++q) {
            const KTerm<S, double> t = all[q];
            if ((s & t.C) != t.V) continue;
            const S s2 = s ^ t.X;
            if ((t.flags & 1u) && !in_basis<S>(b, s2)) continue;
            if (offs) {
                double ar, ai;
                term_amp<S, double>(t, s, vars, ar, ai);
                cols[offs[row] + k] = rank_of<S, RANK>(b, s2);
                vals[offs[row] + k] = make_double2(ar, ai);
            }
            ++k;
        }
        if (!offs) counts[row] = k;
    }
}

inline int grid_for(uint64_t n) {
    uint64_t g = (n + kBlock - 1) / kBlock;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, 152ull * 32));
}

template <class S, class A>
KTerm<S, A> to_kterm(const HostTerm& h, uint32_t var0) {
    KTerm<S, A> k;
    k.C = (S)h.C; k.V = (S)h.V; k.X = (S)h.X; k.J = (S)h.J;
    k.ar = (A)h.amp.real(); k.ai = (A)h.amp.imag();
    k.flags = (h.check ? 1u : 0u) | ((uint32_t)h.vars.size() << 8);
    k.var0 = var0;
    return k;
}

template <class T>
void upload_vec(DBuf& buf, const std::vector<T>& v) {
    buf.alloc(std::max<size_t>(1, v.size()) * sizeof(T));
    if (!v.empty()) QKG_CUDA(cudaMemcpy(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
}

}  // namespace

// ------------------------------------------------------------------------ host
template <class S>
void Hamiltonian::upload_terms(const std::vector<HostTerm>& ht) {
    // Classification (see top of file).
    std::vector<const HostTerm*> outer, inner, mixed, diag;
    const uint64_t inm = basis_->rank_kind == RANK_TABLE ? db_->in_mask : 0;
    for (const auto& h : ht) {
        if (h.X == 0) { diag.push_back(&h); continue; }
        if (basis_->rank_kind == RANK_TABLE && ((h.X | h.C) & inm) == 0) outer.push_back(&h);
        else if (basis_->rank_kind == RANK_TABLE && ((h.X | h.C) & ~inm) == 0) inner.push_back(&h);
        else mixed.push_back(&h);
    }
    if ((int)outer.size() > kMaxOuter) {
        mixed.insert(mixed.end(), outer.begin(), outer.end());
        outer.clear();
    }
    auto build = [&](auto tag, TermSet& ts) {
        using A = decltype(tag);
        std::vector<KVar<A>> vars;
        auto conv = [&](const std::vector<const HostTerm*>& lst) {
            std::vector<KTerm<S, A>> out;
            for (const HostTerm* h : lst) {
                out.push_back(to_kterm<S, A>(*h, (uint32_t)vars.size()));
                for (const DVar& v : h->vars)
                    vars.push_back({v.sm, v.pf, (A)v.a0r, (A)v.a0i, (A)v.a1r, (A)v.a1i});
            }
            return out;
        };
        std::vector<const HostTerm*> allp;
        for (const auto& h : ht) allp.push_back(&h);
        auto ko = conv(outer), ki = conv(inner), km = conv(mixed), kd = conv(diag), ka = conv(allp);
        upload_vec(ts.outer, ko); upload_vec(ts.inner, ki); upload_vec(ts.mixed, km);
        upload_vec(ts.diag, kd); upload_vec(ts.all, ka); upload_vec(ts.vars, vars);
        ts.n_outer = (int)ko.size(); ts.n_inner = (int)ki.size(); ts.n_mixed = (int)km.size();
        ts.n_diag = (int)kd.size(); ts.n_all = (int)ka.size();
    };
    build(double(), t64_);
    build(float(), t32_);
}

Hamiltonian::Hamiltonian(std::shared_ptr<Basis> basis, SiteKind site, const std::vector<Term>& terms)
    : basis_(std::move(basis)), site_(site) {
    QKG_CUDA(cudaGetDevice(&dev_));
    hterms_ = compile_terms(*basis_, site, terms);
    db_ = &basis_->device(dev_);
    wide_ = basis_->nbits > 32;
    for (const auto& h : hterms_) {
        if (h.amp.imag() != 0.0) all_real_ = false;
        for (const auto& v : h.vars) if (v.a0i != 0.0 || v.a1i != 0.0) all_real_ = false;
    }
    if (wide_) upload_terms<uint64_t>(hterms_);
    else upload_terms<uint32_t>(hterms_);
    auto items = basis_->work_items(kChunk);
    n_items_ = items.size();
    upload_vec(items_, items);
    QKG_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    build_diagonal();
    build_fast();
}

namespace {
template <class S, class A>
void pack(const std::vector<const HostTerm*>& lst, std::vector<KTerm<S, A>>& out, std::vector<KVar<A>>& vars) {
    for (const HostTerm* h : lst) {
        out.push_back(to_kterm<S, A>(*h, (uint32_t)vars.size()));
        for (const DVar& v : h->vars) vars.push_back({v.sm, v.pf, (A)v.a0r, (A)v.a0i, (A)v.a1r, (A)v.a1i});
    }
}
}  // namespace

template <class T, class A>
static void allow_stage_smem(size_t bytes);

void Hamiltonian::build_fast() {
    const Basis& B = *basis_;
    fast_ = false;
    if (B.rank_kind != RANK_TABLE || wide_ || dim() == 0 || dim() >= (1ull << 31) || diag_mode_ == DIAG_FULL) return;
    const uint64_t inm = db_->in_mask;
    std::vector<const HostTerm*> outer, inner, mixed;
    for (const auto& h : hterms_) {
        if (h.X == 0) continue;
        if (((h.X | h.C) & ~inm) == 0 && h.vars.empty()) inner.push_back(&h);
        else if (((h.X | h.C) & inm) == 0 && h.vars.empty()) outer.push_back(&h);
        else mixed.push_back(&h);
    }
    if ((int)outer.size() > kMaxOuter) { mixed.insert(mixed.end(), outer.begin(), outer.end()); outer.clear(); }
    if ((int)inner.size() > kMaxInnerTable) { mixed.insert(mixed.end(), inner.begin(), inner.end()); inner.clear(); }
    // Inner table over all inner configurations of the classes that occur.
    const uint32_t P = 1u << B.n_in;
    std::vector<char> present(B.n_in + 2, B.inner_all ? 1 : 0);
    if (!B.inner_all)
        for (uint64_t a = 0; a < (1ull << B.n_out); ++a)
            if (B.outer_off[a + 1] > B.outer_off[a]) present[B.inner_class_of((uint32_t)a)] = 1;
    rbits_ = std::max(1, B.n_in);
    const int tbits = 32 - rbits_ - 1;
    if (tbits < 1 || (inner.size() > (1ull << tbits))) return;
    unif_ = true;
    const std::complex<double> amp0 = inner.empty() ? std::complex<double>(0.0) : inner[0]->amp;
    for (const HostTerm* h : inner)
        if (h->amp != amp0 || (h->J != 0)) unif_ = false;
    // Entries of one inner configuration, in term order.
    auto row_entries = [&](uint32_t b, std::vector<uint32_t>& out) {
        out.clear();
        for (size_t t = 0; t < inner.size(); ++t) {
            const HostTerm& h = *inner[t];
            if ((b & h.C) != h.V) continue;
            const uint32_t b2 = b ^ (uint32_t)h.X;
            // an inner flip stays in the sector iff the inner popcount class is kept
            if (h.check && !B.inner_all && __builtin_popcount(b2) != __builtin_popcount(b)) continue;
            const uint32_t r2 = B.inner_all ? b2 : B.inner_rank[b2];
            const uint32_t sg = __builtin_popcountll((uint64_t)b & h.J & inm) & 1u;
            out.push_back(r2 | (sg << rbits_) | ((uint32_t)t << (rbits_ + 1)));
        }
    };
    // Warp-aligned ELL layout: the rows of a class are grouped by 32 (a work
    // item starts at a multiple of 32 inside its class, so lane = row % 32);
    // group g holds W_g slots per row, slot j of the 32 rows stored
    // contiguously, unused slots = kEllEmpty.  gptr[g] is the group's first slot.
    std::vector<uint32_t> gptr(1, 0), ent, class_gbase(B.n_in + 2, 0), rowbuf;
    std::vector<std::vector<uint32_t>> grp(32);
    const int nclass = B.inner_all ? 1 : B.n_in + 1;
    for (int m = 0; m < nclass; ++m) {
        class_gbase[m] = (uint32_t)(gptr.size() - 1);
        const uint32_t cbase = B.inner_all ? 0u : B.class_base[m];
        const uint32_t csize = B.inner_all ? P : (uint32_t)(B.class_base[m + 1] - B.class_base[m]);
        const bool use = B.inner_all || present[m];
        for (uint32_t g0 = 0; g0 < csize; g0 += 32) {
            size_t w = 0;
            for (uint32_t l = 0; l < 32; ++l) {
                grp[l].clear();
                if (use && g0 + l < csize) {
                    const uint32_t pi = cbase + g0 + l;
                    row_entries(B.inner_all ? pi : B.inner_state[pi], grp[l]);
                }
                w = std::max(w, grp[l].size());
            }
            for (size_t j = 0; j < w; ++j)
                for (uint32_t l = 0; l < 32; ++l) ent.push_back(j < grp[l].size() ? grp[l][j] : kEllEmpty);
            gptr.push_back((uint32_t)ent.size());
            if (ent.size() > (1ull << 31)) return;
        }
    }
    n_ient_ = ent.size();
    upload_vec(iptr_, gptr);
    upload_vec(ient_, ent);
    // each work item records the ELL group of its first row
    auto set_groups = [&](std::vector<WorkItem>& items) {
        for (auto& w : items) {
            const int m = B.inner_all ? 0 : B.inner_class_of(w.a);
            const uint32_t r_loc = w.inner_base - (B.inner_all ? 0u : B.class_base[m]);
            w.pad = class_gbase[m] + r_loc / 32;
        }
    };
    // Launch order of the work items.  A straddling term that flips a high
    // outer bit (the periodic bond of a chain) gathers from the block half a
    // vector away, at scattered rows; ordering the items so that the two blocks
    // of each such pair run side by side keeps those rows in L2.
    int pair_bit = -1;
    for (const HostTerm* h : mixed) {
        const uint64_t xo = (h->X & ~inm) >> B.n_in;
        if ((h->X & inm) && xo) pair_bit = std::max(pair_bit, 63 - __builtin_clzll(xo));
    }
    auto pair_order = [&](std::vector<WorkItem>& v) {
        if (pair_bit < 0) return;
        const uint32_t m = 1u << pair_bit;
        auto key = [&](const WorkItem& w) { return ((uint64_t)(w.a & ~m) << 1) | ((w.a & m) ? 1u : 0u); };
        std::stable_sort(v.begin(), v.end(), [&](const WorkItem& x, const WorkItem& y) { return key(x) < key(y); });
    };
    {
        auto items = B.work_items(kChunk);
        set_groups(items);
        pair_order(items);
        upload_vec(items_, items);
    }
    u_ar_ = amp0.real();
    u_ai_ = amp0.imag();
    // Per outer configuration a (every row of block a shares its outer bits):
    // the outer terms whose condition holds, with the offset of their target
    // block, and the straddling terms whose outer-bit condition holds, with
    // their (uniform) target block.  Built once here instead of by every CTA.
    const uint64_t n_a = 1ull << B.n_out;
    std::vector<uint32_t> optr(n_a + 1, 0), mptr(n_a + 1, 0);
    std::vector<std::pair<uint32_t, int32_t>> oraw;  // (outer term, delta)
    std::vector<uint2> ment;
    for (uint64_t a = 0; a < n_a; ++a) {
        optr[a] = (uint32_t)oraw.size();
        mptr[a] = (uint32_t)ment.size();
        if (B.outer_off[a + 1] == B.outer_off[a]) continue;
        const int c = B.inner_class_of((uint32_t)a);
        const uint64_t b0 = B.inner_all ? 0 : B.inner_state[B.class_base[c]];
        const uint64_t s0 = (a << B.n_in) | b0;
        for (size_t t = 0; t < outer.size(); ++t) {
            const HostTerm& h = *outer[t];
            if ((s0 & h.C) != h.V) continue;
            const uint64_t s2 = s0 ^ h.X;
            if (h.check && !B.contains_int(s2)) continue;
            oraw.push_back({(uint32_t)t, (int32_t)((int64_t)B.outer_off[s2 >> B.n_in] - (int64_t)B.outer_off[a])});
        }
        const uint64_t sa = a << B.n_in;
        for (size_t t = 0; t < mixed.size(); ++t) {
            const HostTerm& h = *mixed[t];
            if ((sa & h.C & ~inm) != (h.V & ~inm)) continue;
            ment.push_back(make_uint2((uint32_t)t, (uint32_t)B.outer_off[(sa ^ h.X) >> B.n_in]));
        }
        if (oraw.size() > 0xFFFFFFF0ull || ment.size() > 0xFFFFFFF0ull) return;
    }
    optr[n_a] = (uint32_t)oraw.size();
    mptr[n_a] = (uint32_t)ment.size();
    upload_vec(optr_, optr);
    upload_vec(mptr_, mptr);
    upload_vec(ment_, ment);
    auto build = [&](auto tag, FastSet& fs) {
        using A = decltype(tag);
        std::vector<KTerm<uint32_t, A>> ko, ki, km;
        std::vector<KVar<A>> vars, dummy;
        pack<uint32_t, A>(outer, ko, dummy);
        pack<uint32_t, A>(inner, ki, dummy);
        pack<uint32_t, A>(mixed, km, vars);
        std::vector<OutEnt<A>> oe(oraw.size());
        for (size_t i = 0; i < oraw.size(); ++i) {
            const KTerm<uint32_t, A>& k = ko[oraw[i].first];
            oe[i].delta = oraw[i].second;
            oe[i].J = k.J;
            oe[i].ar = k.ar;
            oe[i].ai = k.ai;
        }
        upload_vec(fs.oent, oe);
        upload_vec(fs.outer, ko);
        upload_vec(fs.inner, ki);
        upload_vec(fs.mixed, km);
        upload_vec(fs.vars, vars);
        fs.n_outer = (int)ko.size();
        fs.n_inner = (int)ki.size();
        fs.n_mixed = (int)km.size();
        fs.outer_has_j = 0;
        for (const auto* h : outer) if (h->J) fs.outer_has_j = 1;
    };
    build(double(), f64s_);
    build(float(), f32s_);
    // one item per outer block for the staged kernel
    auto bitems = B.work_items(0xFFFFFFFFu);
    set_groups(bitems);
    pair_order(bitems);
    max_block_ = 0;
    for (const auto& w : bitems) max_block_ = std::max<size_t>(max_block_, w.count);
    n_items_blk_ = bitems.size();
    upload_vec(items_blk_, bitems);
    // Tiled kernel: the blocks of each inner class in launch order (the pair
    // order above), cut into groups of G; the groups of all classes run in the
    // order of their first block, so blocks joined by a straddling term run
    // side by side.
    {
        auto key = [&](uint32_t a) -> uint64_t {
            if (pair_bit < 0) return a;
            const uint32_t m = 1u << pair_bit;
            return ((uint64_t)(a & ~m) << 1) | ((a & m) ? 1u : 0u);
        };
        std::vector<std::pair<uint32_t, std::vector<WorkItem>>> classes;  // (inner_base, blocks)
        for (const auto& w : bitems) {
            size_t c = 0;
            while (c < classes.size() && classes[c].first != w.inner_base) ++c;
            if (c == classes.size()) classes.push_back({w.inner_base, {}});
            classes[c].second.push_back(w);
        }
        for (int gi = 0; gi < 3; ++gi) {
            const int G = gi == 0 ? 1 : gi == 1 ? 2 : 4;
            std::vector<std::pair<uint64_t, tilek::TileItem>> groups;
            for (const auto& cl : classes) {
                const auto& v = cl.second;
                for (size_t i = 0; i < v.size(); i += G) {
                    tilek::TileItem t{};
                    t.nblk = (uint32_t)std::min<size_t>(G, v.size() - i);
                    for (uint32_t k = 0; k < t.nblk; ++k) t.a[k] = v[i + k].a;
                    for (uint32_t k = t.nblk; k < (uint32_t)tilek::kMaxG; ++k) t.a[k] = v[i].a;
                    t.width = v[i].count;
                    t.inner_base = v[i].inner_base;
                    t.grp = v[i].pad;
                    groups.push_back({key(v[i].a), t});
                }
            }
            std::stable_sort(groups.begin(), groups.end(),
                             [](const auto& x, const auto& y) { return x.first < y.first; });
            std::vector<tilek::TileItem> tv;
            tv.reserve(groups.size());
            for (const auto& g : groups) tv.push_back(g.second);
            n_tile_[gi] = tv.size();
            upload_vec(tile_items_[gi], tv);
        }
        // Class-persistent kernel: the blocks sorted by inner class (classes of
        // more outer bits first), in launch order inside a class; per class its
        // width, inner_state base, inner-table groups and their entry range.
        std::vector<tilek::CClass> cinfo;
        std::vector<std::pair<uint64_t, tilek::CBlock>> cblk;
        class_maxw_ = class_ell_cap_ = class_gcap_ = 0;
        for (size_t c = 0; c < classes.size(); ++c) {
            const WorkItem& w0 = classes[c].second.front();
            tilek::CClass cc;
            cc.W = w0.count;
            cc.inner_base = w0.inner_base;
            cc.gbase = w0.pad;
            cc.ngroups = (w0.count + 31) / 32;
            cc.ell0 = gptr[cc.gbase];
            cc.ell1 = gptr[cc.gbase + cc.ngroups];
            cinfo.push_back(cc);
            class_maxw_ = std::max(class_maxw_, cc.W);
            class_ell_cap_ = std::max(class_ell_cap_, cc.ell1 - cc.ell0);
            class_gcap_ = std::max(class_gcap_, cc.ngroups);
            const int ic = B.inner_all ? 0 : B.inner_class_of(w0.a);
            for (const auto& w : classes[c].second)
                cblk.push_back({((uint64_t)(uint32_t)(64 - ic) << 40) | key(w.a), tilek::CBlock{w.a, (uint32_t)c}});
        }
        std::stable_sort(cblk.begin(), cblk.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
        std::vector<tilek::CBlock> cb;
        for (const auto& e : cblk) cb.push_back(e.second);
        class_nblocks_ = (uint32_t)cb.size();
        upload_vec(class_blocks_, cb);
        upload_vec(class_info_, cinfo);
        int sms = 0;
        QKG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_));
        class_grid_ = (unsigned)std::min<uint64_t>((uint64_t)std::max(sms, 1), class_nblocks_);
    }
    if (stage_bytes(8) <= kStageLimit) allow_stage_smem<float, float>(stage_bytes(8));
    if (stage_bytes(16) <= kStageLimit) allow_stage_smem<double, double>(stage_bytes(16));
    fast_ = true;
    {
        size_t t32 = 0, t64 = 0;
        for (int G : {1, 2, 4}) {
            if (can_tile(G, 8)) t32 = std::max(t32, tile_smem_bytes(G, 8));
            if (can_tile(G, 16)) t64 = std::max(t64, tile_smem_bytes(G, 16));
        }
        if (t32) tilek::tile_allow_smem<float, float>(t32);
        if (t64) tilek::tile_allow_smem<double, double>(t64);
    }
    autotune();
}

// Autotuner: for sectors large enough to matter, time each fast-kernel
// variant per precision and keep the fastest for mode 0.
void Hamiltonian::autotune() {
    const uint64_t n = dim();
    if (n < (1ull << 20)) return;  // small sectors: four rows per thread
    const int saved = mode_;
    for (int prec = 0; prec < 2; ++prec) {
        const size_t e = prec ? sizeof(double2) : sizeof(float2);
        DBuf x(n * e), y(n * e);
        QKG_CUDA(cudaMemsetAsync(x.p, 0, n * e, stream_));
        cudaEvent_t a, b;
        QKG_CUDA(cudaEventCreate(&a));
        QKG_CUDA(cudaEventCreate(&b));
        double best = 0.0;
        for (int v = 0; v < kFastVariants; ++v) {
            if ((v == FV_STAGED || v == FV_ROWS4_STAGED) && !(stage_bytes(e) <= kStageLimit)) continue;
            if (tile_g((FastVariant)v) && !can_tile(tile_g((FastVariant)v), e)) continue;
            if (v == FV_CLASS && !can_class(e)) continue;
            mode_ = 2 + v;  // modes 2..10 select variants 0..8
            auto run = [&] {
                if (prec) apply_f64(x.as<double2>(), y.as<double2>(), stream_);
                else apply_f32(x.as<float2>(), y.as<float2>(), stream_);
            };
            run();
            QKG_CUDA(cudaEventRecord(a, stream_));
            for (int r = 0; r < 3; ++r) run();
            QKG_CUDA(cudaEventRecord(b, stream_));
            QKG_CUDA(cudaEventSynchronize(b));
            float ms = 0.f;
            QKG_CUDA(cudaEventElapsedTime(&ms, a, b));
            tune_ms_[prec][v] = ms / 3.0;
            if (best == 0.0 || tune_ms_[prec][v] < best) {
                best = tune_ms_[prec][v];
                pref_[prec] = (FastVariant)v;
            }
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    mode_ = saved;
}

// Rank of each internal state in the reference's interleaved order
// (up bit i -> bit 2i, down bit i -> bit 2i+1; the same count as
// Basis::index_ref: for every set bit p, high to low, the valid states sharing
// the bits above p with 0 at p).  One thread per row of a work item.
__global__ void ref_perm_kernel(const WorkItem* __restrict__ items, const uint32_t* __restrict__ inner_state,
                                int n_in, int N, int nbits, int use_nup, int use_ndn, int nup, int ndn,
                                const unsigned long long* __restrict__ binom_tab, int idx32, void* out) {
    __shared__ unsigned long long C[33 * 33];
    for (int i = threadIdx.x; i < 33 * 33; i += blockDim.x) C[i] = binom_tab[i];
    __syncthreads();
    const WorkItem it = items[blockIdx.x];
    for (uint32_t r = threadIdx.x; r < it.count; r += blockDim.x) {
        const uint64_t b = inner_state ? (uint64_t)__ldg(inner_state + it.inner_base + r) : (uint64_t)(it.inner_base + r);
        const uint64_t up = b, dn = (uint64_t)it.a;  // internal state = dn << n_in | up, n_in = N
        unsigned long long rank = 0;
        int up_rem = nup, dn_rem = ndn;
        for (int p = nbits - 1; p >= 0; --p) {
            const int i = p >> 1;
            const bool set = (p & 1) ? ((dn >> i) & 1ull) : ((up >> i) & 1ull);
            if (!set) continue;
            const int us = (p + 1) >> 1, ds = p >> 1;
            const unsigned long long cu =
                use_nup ? ((up_rem >= 0 && up_rem <= us) ? C[us * 33 + up_rem] : 0ull) : (1ull << us);
            const unsigned long long cd =
                use_ndn ? ((dn_rem >= 0 && dn_rem <= ds) ? C[ds * 33 + dn_rem] : 0ull) : (1ull << ds);
            rank += cu * cd;
            if (p & 1) --dn_rem; else --up_rem;
        }
        const uint64_t row = it.row0 + r;
        if (idx32) static_cast<uint32_t*>(out)[row] = (uint32_t)rank;
        else static_cast<unsigned long long*>(out)[row] = rank;
    }
    (void)n_in;
    (void)N;
}

// Reference index of each internal row of a spin/fermion basis whose inner
// classes are reordered: the block offset (blocks are in ascending a in both
// orders) plus the colex rank of the row's inner configuration.
__global__ void ref_perm_colex_kernel(const WorkItem* __restrict__ items, const uint32_t* __restrict__ inner_state,
                                      const uint32_t* __restrict__ colex_rank, const void* outer_off, int idx32,
                                      void* out) {
    const WorkItem it = items[blockIdx.x];
    const uint64_t off = idx32 ? (uint64_t)static_cast<const uint32_t*>(outer_off)[it.a]
                               : (uint64_t)static_cast<const unsigned long long*>(outer_off)[it.a];
    for (uint32_t r = threadIdx.x; r < it.count; r += blockDim.x) {
        const uint64_t rank = off + __ldg(colex_rank + __ldg(inner_state + it.inner_base + r));
        const uint64_t row = it.row0 + r;
        if (idx32) static_cast<uint32_t*>(out)[row] = (uint32_t)rank;
        else static_cast<unsigned long long*>(out)[row] = rank;
    }
}

void ref_permutation_device(const DevBasis& d, const Sector& sec, const std::vector<WorkItem>& items,
                            const std::vector<uint32_t>* ref_inner_rank, void* out) {
    if (items.empty()) return;
    if (ref_inner_rank) {
        QKG_REQUIRE(!d.split && !d.inner_all && d.inner_state && ref_inner_rank->size() == (1ULL << d.n_in),
                    "device permutation: colex ranks of every inner configuration");
        DBuf cr, it;
        upload_vec(cr, *ref_inner_rank);
        upload_vec(it, items);
        ref_perm_colex_kernel<<<(unsigned)items.size(), 256>>>(it.as<WorkItem>(), d.inner_state, cr.as<uint32_t>(),
                                                               d.outer_off, d.idx32, out);
        QKG_LAUNCHED();
        QKG_CUDA(cudaDeviceSynchronize());
        return;
    }
    QKG_REQUIRE(d.split && d.N <= 32 && d.n_in == d.N, "device permutation: split basis with up bits inner");
    std::vector<unsigned long long> tab(33 * 33, 0);
    for (int n = 0; n <= 32; ++n)
        for (int k = 0; k <= n; ++k) tab[n * 33 + k] = binom(n, k);
    DBuf t, it;
    upload_vec(t, tab);
    upload_vec(it, items);
    ref_perm_kernel<<<(unsigned)items.size(), 256>>>(it.as<WorkItem>(), d.inner_all ? nullptr : d.inner_state, d.n_in,
                                                     d.N, d.nbits, sec.use_nup ? 1 : 0, sec.use_ndn ? 1 : 0, sec.nup,
                                                     sec.ndn, t.as<unsigned long long>(), d.idx32, out);
    QKG_LAUNCHED();
    QKG_CUDA(cudaDeviceSynchronize());
}

template <class A>
void Hamiltonian::fast_params(FastParams<A>& p) const {
    const DevBasis& b = *db_;
    const FastSet& fs = sizeof(A) == 8 ? f64s_ : f32s_;
    std::memset(&p, 0, sizeof(p));
    p.n_in = b.n_in;
    p.in_mask = (uint32_t)b.in_mask;
    p.ngroups = b.ngroups;
    p.no_double = b.no_double;
    p.N = b.N;
    p.gmask0 = (uint32_t)b.gmask[0];
    p.gmask1 = (uint32_t)b.gmask[1];
    p.gpop0 = b.gpop[0];
    p.gpop1 = b.gpop[1];
    p.outer_off = static_cast<const uint32_t*>(b.outer_off);
    p.inner_rank = b.inner_all ? nullptr : b.inner_rank;
    p.inner_state = b.inner_all ? nullptr : b.inner_state;
    p.items = items_.as<WorkItem>();
    p.iptr = iptr_.as<uint32_t>();
    p.ient = ient_.as<uint32_t>();
    p.rbits = rbits_;
    p.inner = fs.inner.as<KTerm<uint32_t, A>>();
    p.n_inner = fs.n_inner;
    p.u_ar = (A)u_ar_;
    p.u_ai = (A)u_ai_;
    p.outer = fs.outer.as<KTerm<uint32_t, A>>();
    p.n_outer = fs.n_outer;
    p.outer_has_j = fs.outer_has_j;
    p.mixed = fs.mixed.as<KTerm<uint32_t, A>>();
    p.vars = fs.vars.as<KVar<A>>();
    p.n_mixed = fs.n_mixed;
    p.optr = optr_.as<uint32_t>();
    p.oent = fs.oent.as<OutEnt<A>>();
    p.mptr = mptr_.as<uint32_t>();
    p.ment = ment_.as<uint2>();
    p.diag_mode = diag_mode_;
    const DBuf& dtab = sizeof(A) == 8 ? dtab64_ : dtab32_;
    p.n_dtab = (int)(dtab.bytes / (2 * sizeof(A)));
    p.dcode = dcode_.p;
    p.dtab = dtab.as<A>();
}
template void Hamiltonian::fast_params<float>(FastParams<float>&) const;
uint32_t spmv_wait_timeouts() {
    QKG_CUDA(cudaDeviceSynchronize());
    uint32_t c = 0;
    QKG_CUDA(cudaMemcpyFromSymbol(&c, g_spmv_wait_timeouts, sizeof(c)));
    return c + tilek::tile_wait_timeouts() + tc_wait_timeouts();
}

uint32_t Hamiltonian::tile_slot_elems(size_t elem_bytes) const { return tilek::tile_slot(max_block_, elem_bytes); }
size_t Hamiltonian::tile_smem_bytes(int G, size_t elem_bytes) const {
    const FastSet& fs = elem_bytes == 16 ? f64s_ : f32s_;
    return tilek::tile_smem(G, elem_bytes, tile_slot_elems(elem_bytes), fs.n_inner, unif_, elem_bytes / 2);
}
bool Hamiltonian::can_tile(int G, size_t elem_bytes) const {
    return fast_ && max_block_ > 0 && n_tile_[tile_index(G)] > 0 &&
           tile_smem_bytes(G, elem_bytes) <= tilek::kTileSmemLimit;
}

size_t Hamiltonian::class_smem_bytes(size_t elem_bytes) const {
    const FastSet& fs = elem_bytes == 16 ? f64s_ : f32s_;
    tilek::ClassPlan c{};
    c.slot = tilek::tile_slot(class_maxw_, elem_bytes);
    c.ell_cap = class_ell_cap_;
    c.gcap = class_gcap_;
    return tilek::class_smem(c, elem_bytes, fs.n_inner, unif_, elem_bytes / 2);
}
bool Hamiltonian::can_class(size_t elem_bytes) const {
    return fast_ && class_nblocks_ > 0 && class_maxw_ <= (uint32_t)(tilek::kClassThreads * tilek::kClassCols) &&
           class_smem_bytes(elem_bytes) <= tilek::kTileSmemLimit;
}

// Launch the class-persistent variant.
template <class T, class A>
static void launch_class_variant(const Hamiltonian& H, const FastParams<A>& p, bool real, bool unif,
                                 const typename V2<T>::t* x, typename V2<T>::t* y, cudaStream_t s) {
    const size_t e = sizeof(typename V2<T>::t);
    tilek::ClassPlan c;
    c.blocks = static_cast<const tilek::CBlock*>(H.class_blocks());
    c.classes = static_cast<const tilek::CClass*>(H.class_info());
    c.nblocks = H.class_nblocks();
    c.slot = tilek::tile_slot(H.class_maxw(), e);
    c.ell_cap = H.class_ell_cap();
    c.gcap = H.class_gcap();
    tilek::launch_class<T, A>(p, c, H.class_grid(), real, unif, x, y, H.class_smem_bytes(e), s);
}

// Launch a tiled variant on the Hamiltonian's group list for it.
template <class T, class A>
static void launch_tile_variant(const Hamiltonian& H, const FastParams<A>& p, FastVariant v, bool real, bool unif,
                                const typename V2<T>::t* x, typename V2<T>::t* y, cudaStream_t s) {
    const int G = tile_g(v);
    const size_t e = sizeof(typename V2<T>::t);
    tilek::launch_tile<T, A>(p, static_cast<const tilek::TileItem*>(H.tile_items(G)), H.n_tile_items(G), G, real,
                             unif, x, y, H.tile_slot_elems(e), H.tile_smem_bytes(G, e), s);
}

DBuf& Hamiltonian::krylov_workspace(size_t bytes) const {
    if (kws_.bytes < bytes) {
        kws_.reset();  // free first: the old and new spaces need not fit together
        kws_.alloc(bytes);
    }
    return kws_;
}

std::vector<WorkItem> Hamiltonian::items_host() const {
    std::vector<WorkItem> v(n_items_);
    if (n_items_) QKG_CUDA(cudaMemcpy(v.data(), items_.p, n_items_ * sizeof(WorkItem), cudaMemcpyDeviceToHost));
    return v;
}
template void Hamiltonian::fast_params<double>(FastParams<double>&) const;

// Launch the fast kernel in variant var; p.items must list the variant's work
// items (one per outer block for the staged variant).
template <class T, class A>
static void launch_fast(const FastParams<A>& p, size_t n_items, bool real, bool unif, const typename V2<T>::t* x,
                        typename V2<T>::t* y, cudaStream_t s, FastVariant var, size_t stage_smem) {
    if (!n_items) return;
    const int outer_has_j = p.outer_has_j;
    const unsigned g = (unsigned)n_items;
    const int key = (var == FV_STAGED ? 8 : 0) | (real ? 4 : 0) | (unif ? 2 : 0) | (outer_has_j ? 1 : 0);
    const size_t sm = stage_smem;
    if (var == FV_ROWS4_WIDE) {
        switch (key & 7) {
            case 0: spmv_rows_kernel<T, A, false, false, false, false, true><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 1: spmv_rows_kernel<T, A, false, false, true, false, true><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 2: spmv_rows_kernel<T, A, false, true, false, false, true><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 3: spmv_rows_kernel<T, A, false, true, true, false, true><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 4: spmv_rows_kernel<T, A, true, false, false, false, true><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 5: spmv_rows_kernel<T, A, true, false, true, false, true><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 6: spmv_rows_kernel<T, A, true, true, false, false, true><<<g, kBlock, 0, s>>>(p, x, y); break;
            default: spmv_rows_kernel<T, A, true, true, true, false, true><<<g, kBlock, 0, s>>>(p, x, y); break;
        }
        QKG_LAUNCHED();
        return;
    }
    if (var == FV_ROWS4 || var == FV_ROWS4_STAGED) {
        const bool st = var == FV_ROWS4_STAGED;
        switch ((st ? 8 : 0) | (key & 7)) {
            case 0: spmv_rows_kernel<T, A, false, false, false, false><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 1: spmv_rows_kernel<T, A, false, false, true, false><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 2: spmv_rows_kernel<T, A, false, true, false, false><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 3: spmv_rows_kernel<T, A, false, true, true, false><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 4: spmv_rows_kernel<T, A, true, false, false, false><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 5: spmv_rows_kernel<T, A, true, false, true, false><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 6: spmv_rows_kernel<T, A, true, true, false, false><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 7: spmv_rows_kernel<T, A, true, true, true, false><<<g, kBlock, 0, s>>>(p, x, y); break;
            case 8: spmv_rows_kernel<T, A, false, false, false, true><<<g, kBlock, sm, s>>>(p, x, y); break;
            case 9: spmv_rows_kernel<T, A, false, false, true, true><<<g, kBlock, sm, s>>>(p, x, y); break;
            case 10: spmv_rows_kernel<T, A, false, true, false, true><<<g, kBlock, sm, s>>>(p, x, y); break;
            case 11: spmv_rows_kernel<T, A, false, true, true, true><<<g, kBlock, sm, s>>>(p, x, y); break;
            case 12: spmv_rows_kernel<T, A, true, false, false, true><<<g, kBlock, sm, s>>>(p, x, y); break;
            case 13: spmv_rows_kernel<T, A, true, false, true, true><<<g, kBlock, sm, s>>>(p, x, y); break;
            case 14: spmv_rows_kernel<T, A, true, true, false, true><<<g, kBlock, sm, s>>>(p, x, y); break;
            default: spmv_rows_kernel<T, A, true, true, true, true><<<g, kBlock, sm, s>>>(p, x, y); break;
        }
        QKG_LAUNCHED();
        return;
    }
    switch (key) {
        case 0: spmv_fast_kernel<T, A, false, false, false, false><<<g, kBlock, 0, s>>>(p, x, y); break;
        case 1: spmv_fast_kernel<T, A, false, false, true, false><<<g, kBlock, 0, s>>>(p, x, y); break;
        case 2: spmv_fast_kernel<T, A, false, true, false, false><<<g, kBlock, 0, s>>>(p, x, y); break;
        case 3: spmv_fast_kernel<T, A, false, true, true, false><<<g, kBlock, 0, s>>>(p, x, y); break;
        case 4: spmv_fast_kernel<T, A, true, false, false, false><<<g, kBlock, 0, s>>>(p, x, y); break;
        case 5: spmv_fast_kernel<T, A, true, false, true, false><<<g, kBlock, 0, s>>>(p, x, y); break;
        case 6: spmv_fast_kernel<T, A, true, true, false, false><<<g, kBlock, 0, s>>>(p, x, y); break;
        case 7: spmv_fast_kernel<T, A, true, true, true, false><<<g, kBlock, 0, s>>>(p, x, y); break;
        case 8: spmv_fast_kernel<T, A, false, false, false, true><<<g, kBlock, sm, s>>>(p, x, y); break;
        case 9: spmv_fast_kernel<T, A, false, false, true, true><<<g, kBlock, sm, s>>>(p, x, y); break;
        case 10: spmv_fast_kernel<T, A, false, true, false, true><<<g, kBlock, sm, s>>>(p, x, y); break;
        case 11: spmv_fast_kernel<T, A, false, true, true, true><<<g, kBlock, sm, s>>>(p, x, y); break;
        case 12: spmv_fast_kernel<T, A, true, false, false, true><<<g, kBlock, sm, s>>>(p, x, y); break;
        case 13: spmv_fast_kernel<T, A, true, false, true, true><<<g, kBlock, sm, s>>>(p, x, y); break;
        case 14: spmv_fast_kernel<T, A, true, true, false, true><<<g, kBlock, sm, s>>>(p, x, y); break;
        default: spmv_fast_kernel<T, A, true, true, true, true><<<g, kBlock, sm, s>>>(p, x, y); break;
    }
    QKG_LAUNCHED();
}

// Staged variants may need more than 48 KB of dynamic shared memory.  The
// attribute belongs to the kernel on the current device, not to a Hamiltonian:
// it is raised once per device to the limit every staged launch stays under
// (kStageLimit), so a Hamiltonian built later with a smaller slice cannot
// shrink it below what an earlier one launches with.
template <class T, class A>
static void allow_stage_smem(size_t bytes) {
    static std::mutex mu;
    static uint64_t done = 0;  // devices already raised (bit per device id < 64)
    if (bytes == 0) return;
    int dev = 0;
    QKG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
    if (bit && (done & bit)) return;
    const int b = (int)Hamiltonian::kStageLimit;
    QKG_CUDA(cudaFuncSetAttribute(spmv_fast_kernel<T, A, false, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_fast_kernel<T, A, false, false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_fast_kernel<T, A, false, true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_fast_kernel<T, A, false, true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_fast_kernel<T, A, true, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_fast_kernel<T, A, true, false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_fast_kernel<T, A, true, true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_fast_kernel<T, A, true, true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_rows_kernel<T, A, false, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_rows_kernel<T, A, false, false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_rows_kernel<T, A, false, true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_rows_kernel<T, A, false, true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_rows_kernel<T, A, true, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_rows_kernel<T, A, true, false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_rows_kernel<T, A, true, true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QKG_CUDA(cudaFuncSetAttribute(spmv_rows_kernel<T, A, true, true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    done |= bit;
}

Hamiltonian::~Hamiltonian() {
    if (stream_) {
        cudaStreamSynchronize(stream_);
        cudaStreamDestroy(stream_);
    }
}

void Hamiltonian::build_diagonal() {
    const uint64_t n = dim();
    dfull64_.alloc(std::max<uint64_t>(1, n) * sizeof(double2));
    if (n) {
        const DevBasis b = *db_;
        if (wide_) {
            auto f = b.rank_kind == RANK_TABLE ? diag_kernel<uint64_t, RANK_TABLE> : diag_kernel<uint64_t, RANK_SEARCH>;
            f<<<(unsigned)n_items_, kBlock, 0, stream_>>>(b, items_.as<WorkItem>(), t64_.diag.as<KTerm<uint64_t, double>>(),
                                                         t64_.n_diag, t64_.vars.as<KVar<double>>(), dfull64_.as<double2>());
        } else {
            auto f = b.rank_kind == RANK_TABLE ? diag_kernel<uint32_t, RANK_TABLE> : diag_kernel<uint32_t, RANK_SEARCH>;
            f<<<(unsigned)n_items_, kBlock, 0, stream_>>>(b, items_.as<WorkItem>(), t64_.diag.as<KTerm<uint32_t, double>>(),
                                                         t64_.n_diag, t64_.vars.as<KVar<double>>(), dfull64_.as<double2>());
        }
        QKG_LAUNCHED();
    }
    // Distinct diagonal values -> small table + per-row code.
    std::set<std::pair<uint64_t, uint64_t>> table;
    const unsigned long long cap = 1 << 20;
    DBuf missing(cap * sizeof(ulonglong2)), nmiss(sizeof(unsigned long long)), tabbuf;
    DBuf codes(std::max<uint64_t>(1, n) * 2);
    std::vector<ulonglong2> hmiss;
    bool full = false;
    for (int round = 0; round < 64 && n; ++round) {
        std::vector<ulonglong2> tv;
        for (const auto& kv : table) tv.push_back(make_ulonglong2(kv.first, kv.second));
        upload_vec(tabbuf, tv);
        const int code_bytes = table.size() <= 256 ? 1 : 2;
        QKG_CUDA(cudaMemsetAsync(nmiss.p, 0, sizeof(unsigned long long), stream_));
        diag_code_kernel<<<grid_for(n), kBlock, 0, stream_>>>(dfull64_.as<double2>(), n, tabbuf.as<ulonglong2>(),
                                                              (int)tv.size(), codes.p, code_bytes,
                                                              missing.as<ulonglong2>(), nmiss.as<unsigned long long>(), cap);
        QKG_LAUNCHED();
        unsigned long long nm = 0;
        QKG_CUDA(cudaMemcpyAsync(&nm, nmiss.p, sizeof(nm), cudaMemcpyDeviceToHost, stream_));
        QKG_CUDA(cudaStreamSynchronize(stream_));
        if (nm == 0) {
            diag_mode_ = code_bytes == 1 ? DIAG_U8 : DIAG_U16;
            break;
        }
        const size_t take = (size_t)std::min<unsigned long long>(nm, cap);
        hmiss.resize(take);
        QKG_CUDA(cudaMemcpy(hmiss.data(), missing.p, take * sizeof(ulonglong2), cudaMemcpyDeviceToHost));
        for (const auto& m : hmiss) {
            table.insert({m.x, m.y});
            if (table.size() > 65536) break;  // too many values for codes: stop inserting
        }
        if (table.size() > 65536) { full = true; break; }
    }
    if (!n) { diag_mode_ = DIAG_U8; table.insert({0, 0}); }
    if (full) {
        diag_mode_ = DIAG_FULL;
        dfull32_.alloc(n * sizeof(float2));
        d2f_kernel<<<grid_for(n), kBlock, 0, stream_>>>(dfull64_.as<double2>(), dfull32_.as<float2>(), n);
        QKG_LAUNCHED();
    } else {
        std::vector<double> t64;
        std::vector<float> t32;
        for (const auto& kv : table) {
            double re, im;
            std::memcpy(&re, &kv.first, 8);
            std::memcpy(&im, &kv.second, 8);
            t64.push_back(re); t64.push_back(im);
            t32.push_back((float)re); t32.push_back((float)im);
        }
        n_dtab_ = (int)table.size();
        upload_vec(dtab64_, t64);
        upload_vec(dtab32_, t32);
        const size_t cb = diag_mode_ == DIAG_U8 ? 1 : 2;
        dcode_.alloc(std::max<uint64_t>(1, n) * cb);
        // The last round wrote every code with the final table's width.
        if (n) QKG_CUDA(cudaMemcpyAsync(dcode_.p, codes.p, n * cb, cudaMemcpyDeviceToDevice, stream_));
        QKG_CUDA(cudaStreamSynchronize(stream_));
        dfull64_.reset();
    }
    QKG_CUDA(cudaStreamSynchronize(stream_));
}

template <class S, class T, class A>
static void launch_spmv(const DevBasis& b, const TermSet& ts, const DBuf& items, size_t n_items, bool real, int diag_mode,
                        const DBuf& dcode, const DBuf& dtab, const DBuf& dfull, const typename V2<T>::t* x,
                        typename V2<T>::t* y, cudaStream_t s) {
    if (!n_items) return;
    SpmvParams<S, A> p;
    p.b = b;
    p.items = items.as<WorkItem>();
    p.outer = ts.outer.as<KTerm<S, A>>();
    p.inner = ts.inner.as<KTerm<S, A>>();
    p.mixed = ts.mixed.as<KTerm<S, A>>();
    p.vars = ts.vars.as<KVar<A>>();
    p.n_outer = ts.n_outer; p.n_inner = ts.n_inner; p.n_mixed = ts.n_mixed;
    p.n_vars = (int)(ts.vars.bytes / sizeof(KVar<A>));
    const size_t smem = (size_t)(p.n_outer + p.n_inner + p.n_mixed) * sizeof(KTerm<S, A>) + (size_t)p.n_vars * sizeof(KVar<A>);
    p.terms_in_smem = smem <= kSmemTermBudget;
    p.real = real;
    p.diag_mode = diag_mode;
    p.dcode = dcode.p;
    p.dtab = dtab.p;
    p.dfull = dfull.p;
    const size_t dyn = p.terms_in_smem ? smem : 0;
    if (b.rank_kind == RANK_TABLE)
        spmv_kernel<S, T, A, RANK_TABLE><<<(unsigned)n_items, kBlock, dyn, s>>>(p, x, y);
    else
        spmv_kernel<S, T, A, RANK_SEARCH><<<(unsigned)n_items, kBlock, dyn, s>>>(p, x, y);
    QKG_LAUNCHED();
}

void Hamiltonian::apply_f64(const double2* x, double2* y, cudaStream_t s) const {
    if (fast()) {
        const FastVariant v = variant(16);
        if (tile_g(v) || v == FV_CLASS) {
            FastParams<double> p;
            fast_params(p);
            if (v == FV_CLASS) launch_class_variant<double, double>(*this, p, all_real_, unif_, x, y, s);
            else launch_tile_variant<double, double>(*this, p, v, all_real_, unif_, x, y, s);
            return;
        }
        const bool st = v == FV_STAGED || v == FV_ROWS4_STAGED;
        FastParams<double> p;
        fast_params(p);
        size_t ni = 0;
        p.items = items_of(v, &ni);
        launch_fast<double, double>(p, ni, all_real_, unif_, x, y, s, v, st ? stage_bytes(16) : 0);
        return;
    }
    const DBuf& full = dfull64_;
    if (wide_)
        launch_spmv<uint64_t, double, double>(*db_, t64_, items_, n_items_, all_real_, diag_mode_, dcode_, dtab64_, full, x, y, s);
    else
        launch_spmv<uint32_t, double, double>(*db_, t64_, items_, n_items_, all_real_, diag_mode_, dcode_, dtab64_, full, x, y, s);
}

void Hamiltonian::apply_lanczos_f32(const LanczosHooks& lz, cudaStream_t s) const {
    QKG_REQUIRE(fast(), "the device-resident Lanczos step needs the fast SpMV kernel");
    const FastVariant v = variant(8);
    const bool st = v == FV_STAGED || v == FV_ROWS4_STAGED;
    FastParams<float> p;
    fast_params(p);
    p.lz = lz.op;
    p.apart = lz.apart;
    if (v == FV_CLASS) {
        launch_class_variant<float, float>(*this, p, all_real_, unif_, nullptr, nullptr, s);
        return;
    }
    if (tile_g(v)) {
        launch_tile_variant<float, float>(*this, p, v, all_real_, unif_, nullptr, nullptr, s);
        return;
    }
    size_t ni = 0;
    p.items = items_of(v, &ni);
    launch_fast<float, float>(p, ni, all_real_, unif_, nullptr, nullptr, s, v, st ? stage_bytes(8) : 0);
}

size_t Hamiltonian::lanczos_parts() const {
    if (!fast()) return n_items_;
    if (variant(8) == FV_CLASS) return class_grid_;
    if (tile_g(variant(8))) return n_tile_items(tile_g(variant(8)));
    size_t ni = 0;
    items_of(variant(8), &ni);
    return ni;
}

const WorkItem* Hamiltonian::items_of(FastVariant v, size_t* n) const {
    if (v == FV_STAGED || v == FV_ROWS4_STAGED) {
        *n = n_items_blk_;
        return items_blk_.as<WorkItem>();
    }
    *n = n_items_;
    return items_.as<WorkItem>();
}

void Hamiltonian::apply_f32(const float2* x, float2* y, cudaStream_t s) const {
    if (fast()) {
        const FastVariant v = variant(8);
        if (tile_g(v) || v == FV_CLASS) {
            FastParams<float> p;
            fast_params(p);
            if (v == FV_CLASS) launch_class_variant<float, float>(*this, p, all_real_, unif_, x, y, s);
            else launch_tile_variant<float, float>(*this, p, v, all_real_, unif_, x, y, s);
            return;
        }
        const bool st = v == FV_STAGED || v == FV_ROWS4_STAGED;
        FastParams<float> p;
        fast_params(p);
        size_t ni = 0;
        p.items = items_of(v, &ni);
        launch_fast<float, float>(p, ni, all_real_, unif_, x, y, s, v, st ? stage_bytes(8) : 0);
        return;
    }
    if (wide_)
        launch_spmv<uint64_t, float, float>(*db_, t32_, items_, n_items_, all_real_, diag_mode_, dcode_, dtab32_, dfull32_, x, y, s);
    else
        launch_spmv<uint32_t, float, float>(*db_, t32_, items_, n_items_, all_real_, diag_mode_, dcode_, dtab32_, dfull32_, x, y, s);
}

void Hamiltonian::diagonal_f64(double2* d, cudaStream_t s) const {
    const uint64_t n = dim();
    if (!n) return;
    if (diag_mode_ == DIAG_FULL) {
        QKG_CUDA(cudaMemcpyAsync(d, dfull64_.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        return;
    }
    diag_expand_kernel<double><<<grid_for(n), kBlock, 0, s>>>(dcode_.p, diag_mode_ == DIAG_U8 ? 1 : 2, dtab64_.as<double>(), n, d);
    QKG_LAUNCHED();
}

std::vector<std::complex<double>> Hamiltonian::diagonal_host_ref() const {
    const uint64_t n = dim();
    std::vector<std::complex<double>> out(n);
    if (!n) return out;
    DBuf a(n * sizeof(double2)), b2(n * sizeof(double2));
    diagonal_f64(a.as<double2>(), stream_);
    to_reference_f64(a.as<double2>(), b2.as<double2>(), stream_);
    QKG_CUDA(cudaMemcpyAsync(out.data(), b2.p, n * sizeof(double2), cudaMemcpyDeviceToHost, stream_));
    QKG_CUDA(cudaStreamSynchronize(stream_));
    return out;
}

template <class V>
static void permute(const DevBasis& b, bool permuted, const V* src, V* dst, uint64_t n, bool to_int, cudaStream_t s) {
    if (!n) return;
    if (!permuted) {
        if (src != dst) QKG_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(V), cudaMemcpyDeviceToDevice, s));
        return;
    }
    if (b.idx32) {
        const uint32_t* perm = static_cast<const uint32_t*>(b.ref_of_int);
        if (to_int) gather_kernel<V, uint32_t><<<grid_for(n), kBlock, 0, s>>>(src, dst, perm, n);
        else scatter_kernel<V, uint32_t><<<grid_for(n), kBlock, 0, s>>>(src, dst, perm, n);
    } else {
        const uint64_t* perm = static_cast<const uint64_t*>(b.ref_of_int);
        if (to_int) gather_kernel<V, uint64_t><<<grid_for(n), kBlock, 0, s>>>(src, dst, perm, n);
        else scatter_kernel<V, uint64_t><<<grid_for(n), kBlock, 0, s>>>(src, dst, perm, n);
    }
    QKG_LAUNCHED();
}

void Hamiltonian::to_internal_f64(const double2* r, double2* i, cudaStream_t s) const { permute(*db_, permuted(), r, i, dim(), true, s); }
void Hamiltonian::to_reference_f64(const double2* i, double2* r, cudaStream_t s) const { permute(*db_, permuted(), i, r, dim(), false, s); }
void Hamiltonian::to_internal_f32(const float2* r, float2* i, cudaStream_t s) const { permute(*db_, permuted(), r, i, dim(), true, s); }
void Hamiltonian::to_reference_f32(const float2* i, float2* r, cudaStream_t s) const { permute(*db_, permuted(), i, r, dim(), false, s); }

void Hamiltonian::emit_entries(std::vector<uint64_t>& row_offsets, std::vector<uint64_t>& cols,
                               std::vector<std::complex<double>>& vals) const {
    const uint64_t n = dim();
    row_offsets.assign(n + 1, 0);
    cols.clear();
    vals.clear();
    if (!n) return;
    DBuf counts(n * 8), offs((n + 1) * 8);
    const DevBasis b = *db_;
    auto run = [&](const unsigned long long* o, unsigned long long* c, unsigned long long* cl, double2* v) {
        if (wide_) {
            auto f = b.rank_kind == RANK_TABLE ? emit_kernel<uint64_t, RANK_TABLE> : emit_kernel<uint64_t, RANK_SEARCH>;
            f<<<(unsigned)n_items_, kBlock, 0, stream_>>>(b, items_.as<WorkItem>(), t64_.all.as<KTerm<uint64_t, double>>(),
                                                         t64_.n_all, t64_.vars.as<KVar<double>>(), o, c, cl, v);
        } else {
            auto f = b.rank_kind == RANK_TABLE ? emit_kernel<uint32_t, RANK_TABLE> : emit_kernel<uint32_t, RANK_SEARCH>;
            f<<<(unsigned)n_items_, kBlock, 0, stream_>>>(b, items_.as<WorkItem>(), t64_.all.as<KTerm<uint32_t, double>>(),
                                                         t64_.n_all, t64_.vars.as<KVar<double>>(), o, c, cl, v);
        }
        QKG_LAUNCHED();
    };
    run(nullptr, counts.as<unsigned long long>(), nullptr, nullptr);
    std::vector<uint64_t> cnt(n);
    QKG_CUDA(cudaMemcpyAsync(cnt.data(), counts.p, n * 8, cudaMemcpyDeviceToHost, stream_));
    QKG_CUDA(cudaStreamSynchronize(stream_));
    for (uint64_t i = 0; i < n; ++i) row_offsets[i + 1] = row_offsets[i] + cnt[i];
    const uint64_t nnz = row_offsets[n];
    QKG_CUDA(cudaMemcpy(offs.p, row_offsets.data(), (n + 1) * 8, cudaMemcpyHostToDevice));
    DBuf dc(std::max<uint64_t>(1, nnz) * 8), dv(std::max<uint64_t>(1, nnz) * sizeof(double2));
    run(offs.as<unsigned long long>(), nullptr, dc.as<unsigned long long>(), dv.as<double2>());
    cols.resize(nnz);
    vals.resize(nnz);
    QKG_CUDA(cudaMemcpyAsync(cols.data(), dc.p, nnz * 8, cudaMemcpyDeviceToHost, stream_));
    QKG_CUDA(cudaMemcpyAsync(vals.data(), dv.p, nnz * sizeof(double2), cudaMemcpyDeviceToHost, stream_));
    QKG_CUDA(cudaStreamSynchronize(stream_));
}

}  // namespace qkg
