// Device-resident mixed-precision Lanczos: one step = four kernels that read
// the step index, the vector pointers and the recurrence scalars from device
// memory, so the step is captured once as a CUDA graph and replayed.
//
// Stored vectors.  v_k = sig[k] * V_k with V_0 the normalised start vector and
// V_{k+1} = w_k (the un-normalised residual of step k), sig[k+1] = 1 / beta_k.
// The SpMV multiplies its output by sig[k], so y = H v_k and every stored
// vector has norm beta_{k-1}: no growth, no separate normalisation pass.
//   1. SpMV (fast kernel, Lanczos mode): V_{k+1} = sig_k H V_k - beta_{k-1}
//      sig_{k-1} V_{k-1} (the previous-vector term applied as each row is
//      written), plus per-block partials of Re<V_k, V_{k+1}>  =>  alpha_k =
//      sig_k * sum = <v_k, H v_k - beta_{k-1} v_{k-1}> (the modified
//      Gram-Schmidt order of Paige's Lanczos variant: equal to <v_k, H v_k> in
//      exact arithmetic, one pass over a vector fewer per step).
//   2. lz_alpha: alpha_k and the coefficient a = alpha_k sig_k.
//   3. lz_update: V_{k+1} -= a V_k; compensated |V_{k+1}|^2 partials.
//      (selective reorthogonalisation adds lz_proj, lz_proj_finish, lz_orth)
//   4. lz_beta: beta_k, sig_{k+1}, k += 1.
// alpha/beta are also written to mapped pinned host memory; the host reads
// them a few steps behind the GPU (convergence test, selective
// reorthogonalisation trigger) without stalling the stream.
#include "solvers.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <type_traits>

namespace qkg {

namespace {
constexpr int kT = 256;
constexpr int kUpdGrid = 152 * 8;
constexpr int kTimedSteps = 8;  // steps launched one by one with an SpMV timer before the graph takes over
constexpr int kInFlight = 6;    // steps the host lets the GPU run ahead of its checks
constexpr double kOrthTol = 3.4526698300124393e-4;  // sqrt(2^-23): FP32 semiorthogonality level

constexpr int kMaxPsi = kMaxRitzLocked;  // converged Ritz vectors held for selective reorthogonalisation

struct LzState {
    int k;
    int orth;               // this step's correction along the Ritz vectors is applied
    double a, b;            // update coefficients of the current step
    double pre[kMaxPsi], pim[kMaxPsi];  // projections on the Ritz vectors (selective reorthogonalisation)
};
struct PsiTab {
    const float2* p[kMaxPsi];
};

__device__ __forceinline__ void ff_acc(float& hi, float& lo, float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    const float t = hi + p;
    const float z = t - hi;
    lo += ((hi - (t - z)) + (p - z)) + e;
    hi = t;
}

__device__ __forceinline__ double2 bsum2(double x, double y) {
    __shared__ double2 sh[32];
    for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_down_sync(0xffffffffu, x, o);
        y += __shfl_down_sync(0xffffffffu, y, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = make_double2(x, y);
    __syncthreads();
    double2 v = (threadIdx.x < (blockDim.x >> 5)) ? sh[lane] : make_double2(0.0, 0.0);
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_down_sync(0xffffffffu, v.x, o);
            v.y += __shfl_down_sync(0xffffffffu, v.y, o);
        }
    return v;
}

// alpha from the SpMV's per-CTA partials: kAlphaBlocks blocks sum fixed
// slices, the last block to finish (arrival counter) adds their sums in block
// order and does the step's bookkeeping; the result does not depend on which
// block finishes last.
constexpr int kAlphaBlocks = 64;
__global__ void lz_alpha_kernel(const double2* __restrict__ apart, int nparts, LzState* st, double* alpha,
                                const double* beta, const double* sig, double* alpha_host, double* part2,
                                unsigned int* arrived) {
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nparts; i += gridDim.x * blockDim.x) s += apart[i].x;
    const double2 t = bsum2(s, 0.0);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part2[blockIdx.x] = t.x;
        __threadfence();
        last = atomicAdd(arrived, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const double v = threadIdx.x < gridDim.x ? *(volatile double*)(part2 + threadIdx.x) : 0.0;
    const double2 u = bsum2(v, 0.0);
    if (threadIdx.x == 0) {
        const int k = st->k;
        const double a = sig[k] * u.x;
        alpha[k] = a;
        alpha_host[k] = a;
        st->a = a * sig[k];
        st->b = 0.0;  // the SpMV already subtracted beta_{k-1} v_{k-1}
        *arrived = 0u;  // ready for the next step
    }
}

// One element of the update w -= a v + b v_prev with its ||w||^2 (and, with
// NP Ritz vectors psi_p, the <psi_p, w>) contributions.
template <int NP>
struct UpdAcc {
    float hi = 0.f, lo = 0.f;
    float rh[NP > 0 ? NP : 1] = {}, rl[NP > 0 ? NP : 1] = {}, ih[NP > 0 ? NP : 1] = {}, il[NP > 0 ? NP : 1] = {};
};
template <int NP>
__device__ __forceinline__ float2 upd_elem(float2 x, float2 c, float2 d, const float2 (&p)[NP > 0 ? NP : 1], float a,
                                           float b, bool has_prev, UpdAcc<NP>& s) {
    x.x = fmaf(-a, c.x, x.x);
    x.y = fmaf(-a, c.y, x.y);
    if (has_prev) {
        x.x = fmaf(-b, d.x, x.x);
        x.y = fmaf(-b, d.y, x.y);
    }
    ff_acc(s.hi, s.lo, x.x, x.x);
    ff_acc(s.hi, s.lo, x.y, x.y);
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        ff_acc(s.rh[q], s.rl[q], p[q].x, x.x);
        ff_acc(s.rh[q], s.rl[q], p[q].y, x.y);
        ff_acc(s.ih[q], s.il[q], p[q].x, x.y);
        ff_acc(s.ih[q], s.il[q], -p[q].y, x.x);
    }
    return x;
}

// w -= a v + b v_prev in place (b = 0: the SpMV applied the previous-vector
// term, and v_prev is not read), ||w||^2 partials (and the <psi_q, w> partials
// of the NP Ritz vectors, for selective reorthogonalisation): two elements per
// thread and iteration with 16-byte accesses (the Krylov vectors are 256-byte
// aligned).  ppart[q * gridDim.x + block] holds Ritz vector q's partial.
template <int NP>
__global__ void lz_update_t(void* const* __restrict__ vtab, const LzState* __restrict__ st, uint64_t n,
                            const PsiTab psi, double2* __restrict__ bpart, double2* __restrict__ ppart) {
    const int k = st->k;
    float2* __restrict__ w = static_cast<float2*>(vtab[k + 1]);
    const float2* __restrict__ v = static_cast<const float2*>(vtab[k]);
    const float a = (float)st->a, b = (float)st->b;
    const bool has_prev = k > 0 && b != 0.f;
    const float2* __restrict__ vp = has_prev ? static_cast<const float2*>(vtab[k - 1]) : v;
    UpdAcc<NP> s;
    constexpr int NQ = NP > 0 ? NP : 1;
    const uint64_t n2 = n / 2, step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n2; i += step) {
        const float4 x4 = reinterpret_cast<const float4*>(w)[i];
        const float4 c4 = reinterpret_cast<const float4*>(v)[i];
        float4 d4 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (has_prev) d4 = reinterpret_cast<const float4*>(vp)[i];
        float2 p0[NQ], p1[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            float4 p4 = make_float4(0.f, 0.f, 0.f, 0.f);
            if (q < NP) p4 = reinterpret_cast<const float4*>(psi.p[q])[i];
            p0[q] = make_float2(p4.x, p4.y);
            p1[q] = make_float2(p4.z, p4.w);
        }
        const float2 y0 = upd_elem<NP>(make_float2(x4.x, x4.y), make_float2(c4.x, c4.y), make_float2(d4.x, d4.y),
                                       p0, a, b, has_prev, s);
        const float2 y1 = upd_elem<NP>(make_float2(x4.z, x4.w), make_float2(c4.z, c4.w), make_float2(d4.z, d4.w),
                                       p1, a, b, has_prev, s);
        reinterpret_cast<float4*>(w)[i] = make_float4(y0.x, y0.y, y1.x, y1.y);
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        float2 pl[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) pl[q] = q < NP ? psi.p[q][n - 1] : make_float2(0.f, 0.f);
        w[n - 1] = upd_elem<NP>(w[n - 1], v[n - 1], vp[n - 1], pl, a, b, has_prev, s);
    }
    const double2 t = bsum2((double)s.hi + (double)s.lo, 0.0);
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        const double2 r = bsum2((double)s.rh[q] + (double)s.rl[q], (double)s.ih[q] + (double)s.il[q]);
        if (threadIdx.x == 0) ppart[(size_t)q * gridDim.x + blockIdx.x] = r;
    }
    if (threadIdx.x == 0) bpart[blockIdx.x] = t;
}

// c_q = <psi_q, W> for the NP Ritz vectors; the correction is applied only
// when some |c_q| exceeds orth_tol ||W|| (components below the square root of
// the working precision are harmless, Parlett & Scott 1979), so most steps skip
// the extra pass over W.
template <int NP>
__global__ void lz_proj_finish_kernel(const double2* __restrict__ ppart, const double2* __restrict__ bpart,
                                      int nparts, LzState* st, double orth_tol) {
    double w2 = 0.0;
    for (int j = threadIdx.x; j < nparts; j += blockDim.x) w2 += bpart[j].x;
    const double2 u = bsum2(w2, 0.0);
    int orth = 0;
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        double r = 0.0, i = 0.0;
        for (int j = threadIdx.x; j < nparts; j += blockDim.x) {
            r += ppart[(size_t)q * nparts + j].x;
            i += ppart[(size_t)q * nparts + j].y;
        }
        const double2 t = bsum2(r, i);
        if (threadIdx.x == 0) {
            st->pre[q] = t.x;
            st->pim[q] = t.y;
            orth |= (t.x * t.x + t.y * t.y) > orth_tol * orth_tol * u.x ? 1 : 0;
        }
    }
    if (threadIdx.x == 0) st->orth = orth;
}
// W -= sum_q c_q psi_q with c_q = <psi_q, W>; |W|^2 partials.
template <int NP>
__global__ void lz_orth_kernel(void* const* __restrict__ vtab, const LzState* __restrict__ st, const PsiTab psi,
                               uint64_t n, double2* __restrict__ bpart) {
    if (!st->orth) return;  // bpart keeps the partials of the unchanged W
    float2* __restrict__ w = static_cast<float2*>(vtab[st->k + 1]);
    float cr[NP], ci[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        cr[q] = (float)st->pre[q];
        ci[q] = (float)st->pim[q];
    }
    float hi = 0.f, lo = 0.f;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float2 x = w[i];
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            const float2 p = psi.p[q][i];
            x.x -= cr[q] * p.x - ci[q] * p.y;
            x.y -= cr[q] * p.y + ci[q] * p.x;
        }
        w[i] = x;
        ff_acc(hi, lo, x.x, x.x);
        ff_acc(hi, lo, x.y, x.y);
    }
    const double2 s = bsum2((double)hi + (double)lo, 0.0);
    if (threadIdx.x == 0) bpart[blockIdx.x] = s;
}

// beta_k, sig_{k+1}, k += 1, and the next step's SpMV operands:
// y = sig_{k+1} H V_{k+1} - beta_k sig_k V_k into V_{k+2}.
__global__ void lz_beta_kernel(const double2* __restrict__ bpart, int nparts, LzState* st, double* beta, double* sig,
                               double* beta_host, void* const* __restrict__ vtab, int nmax, LzOperands* op) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += bpart[i].x;
    const double2 t = bsum2(s, 0.0);
    if (threadIdx.x == 0) {
        const int k = st->k;
        const double b = sqrt(t.x);
        const double sn = b > 0.0 ? 1.0 / b : 0.0;
        beta[k] = b;
        beta_host[k] = b;
        sig[k + 1] = sn;
        st->k = k + 1;
        LzOperands o;
        o.x = vtab[min(k + 1, nmax)];
        o.y = vtab[min(k + 2, nmax)];  // no step runs past nmax - 1
        o.vprev = vtab[k];
        o.scale = sn;
        o.bprev = b * sig[k];
        o.scale32 = (float)o.scale;
        o.bprev32 = (float)o.bprev;
        *op = o;
    }
}

using clk = std::chrono::steady_clock;
inline double secs(clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); }

struct Mapped {
    double* h = nullptr;
    double* d = nullptr;
    explicit Mapped(size_t n) {
        QKG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&h), n * sizeof(double), cudaHostAllocMapped));
        QKG_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&d), h, 0));
        std::fill(h, h + n, 0.0);
    }
    ~Mapped() { if (h) cudaFreeHost(h); }
};
}  // namespace

bool lanczos_device_supported(const Hamiltonian& H) { return H.fast(); }

// Device memory of a device-resident run of maxiter steps: maxiter + 1 Krylov
// vectors, then kMaxPsi Ritz vectors psi (FP32), the Ritz vector (FP32), the
// refined Ritz vector and its residual (FP64), each vector on a 256-byte
// boundary.  The FP64 slots also stage a caller's start vector, the first two
// psi slots the reference-order copy of the eigenvector.
size_t lanczos_device_bytes(const Hamiltonian& H, int maxiter) {
    const uint64_t n = H.dim();
    const int nmax = (int)std::min<uint64_t>((uint64_t)std::max(maxiter, 0), n);
    const uint64_t stride = (n + 31) / 32 * 32;
    return (size_t)(nmax + 1 + kMaxPsi + 5) * stride * sizeof(float2);
}

LanczosOut lanczos_mixed_device(Hamiltonian& H, const LanczosOpts& o) {
    LanczosOut out;
    const uint64_t n = H.dim();
    if (n == 0) return out;
    const auto ws_lock = H.workspace_lock();
    cudaStream_t st = H.stream();
    const int nmax = (int)std::min<uint64_t>((uint64_t)std::max(o.maxiter, 0), n);
    if (nmax <= 0) return out;
    // all nmax + 1 Krylov vectors (FP32) up front: the graph addresses them through vtab
    // vectors start on 256-byte boundaries (a warp's 32 consecutive rows then
    // cover whole 128-byte lines)
    const uint64_t stride = (n + 31) / 32 * 32;
    const size_t need = lanczos_device_bytes(H, o.maxiter);
    if (H.workspace_bytes() < need) {
        H.release_workspace();
        size_t fr = 0, tot = 0;
        QKG_CUDA(cudaMemGetInfo(&fr, &tot));
        if (need + (512ull << 20) > fr)
            throw Error(CUDA_ERR, "out of device memory for " + std::to_string(nmax + 1) + " Krylov vectors");
    }
    // one allocation for all vectors (a cudaMalloc per vector costs more than a
    // step), kept on the Hamiltonian for the next run
    const DBuf& V = H.krylov_workspace(need);
    std::vector<void*> vptr;
    for (int i = 0; i <= nmax; ++i) vptr.push_back(V.as<float2>() + (size_t)i * stride);
    float2* const psi_p = V.as<float2>() + (size_t)(nmax + 1) * stride;
    float2* const r32_p = psi_p + (size_t)kMaxPsi * stride;
    double2* const r64_p = reinterpret_cast<double2*>(r32_p + stride);
    double2* const h64_p = r64_p + stride;
    DBuf vtab((nmax + 1) * sizeof(void*));
    QKG_CUDA(cudaMemcpy(vtab.p, vptr.data(), vptr.size() * sizeof(void*), cudaMemcpyHostToDevice));
    DBuf state(sizeof(LzState)), alpha((nmax + 2) * 8), beta((nmax + 2) * 8), sig((nmax + 2) * 8);
    DBuf apart(std::max<size_t>(1, H.lanczos_parts()) * sizeof(double2)), bpart(kUpdGrid * sizeof(double2)),
        ppart((size_t)kMaxPsi * kUpdGrid * sizeof(double2)), psitab(kMaxPsi * sizeof(float2*));
    Mapped ah(nmax + 2), bh(nmax + 2);
    DBuf part2(kAlphaBlocks * sizeof(double)), arrived(sizeof(unsigned int));
    QKG_CUDA(cudaMemsetAsync(arrived.p, 0, sizeof(unsigned int), st));
    Workspace ws(std::max<size_t>(1 << 16, (size_t)1216 * (size_t)(nmax + 2)));
    DBuf tmp;

    float2* v0 = static_cast<float2*>(vptr[0]);
    if (o.device_start) {
        philox_normal_f32(o.seed, 0, v0, n, st);
    } else {
        // the caller's vector is copied straight from its buffer (pinned memory takes the DMA path)
        std::vector<cd> h;
        const cd* src = o.v0_ref;
        if (!src) {
            h.resize(n);
            ref_uniform_complex(1234, n, h.data(), o.f32_stream);
            src = h.data();
        }
        QKG_CUDA(cudaMemcpyAsync(r64_p, src, n * sizeof(double2), cudaMemcpyHostToDevice, st));
        const double2* in = r64_p;
        if (H.permuted()) {
            H.to_internal_f64(r64_p, h64_p, st);
            in = h64_p;
        }
        f64_to_f32(in, v0, n, st);
        QKG_CUDA(cudaStreamSynchronize(st));
    }
    const double nr0 = std::sqrt(nrm2sq_f32(v0, n, ws, st));
    if (nr0 != 0.0) scal_f32(1.0 / nr0, v0, n, st);
    DBuf lzop(sizeof(LzOperands));
    {
        LzState s0{};
        const double one = 1.0;
        LzOperands op0;  // step 0: y = H v_0, no previous vector
        op0.x = vptr[0];
        op0.y = vptr[1];
        QKG_CUDA(cudaMemcpyAsync(state.p, &s0, sizeof(s0), cudaMemcpyHostToDevice, st));
        QKG_CUDA(cudaMemcpyAsync(sig.p, &one, sizeof(one), cudaMemcpyHostToDevice, st));
        QKG_CUDA(cudaMemcpyAsync(lzop.p, &op0, sizeof(op0), cudaMemcpyHostToDevice, st));
        QKG_CUDA(cudaStreamSynchronize(st));
    }

    LanczosHooks hooks;
    hooks.op = lzop.as<LzOperands>();
    hooks.apart = apart.as<double2>();
    const int nparts = (int)H.lanczos_parts();
    PsiTab psi{};   // converged Ritz vectors (selective reorthogonalisation)
    int npsi = 0;   // how many are held
    std::vector<double> locked;  // their Ritz values
    auto enqueue_step = [&](int np, LaunchTimer* timer) {
        if (timer) timer->start();
        H.apply_lanczos_f32(hooks, st);
        if (timer) timer->stop();
        lz_alpha_kernel<<<kAlphaBlocks, kT, 0, st>>>(apart.as<double2>(), nparts, state.as<LzState>(),
                                                     alpha.as<double>(), beta.as<double>(), sig.as<double>(), ah.d,
                                                     part2.as<double>(), arrived.as<unsigned int>());
        QKG_LAUNCHED();
        void* const* vt = static_cast<void* const*>(vtab.p);
        auto sel = [&](auto npc) {
            constexpr int NP = decltype(npc)::value;
            lz_update_t<NP><<<kUpdGrid, kT, 0, st>>>(vt, state.as<LzState>(), n, psi, bpart.as<double2>(),
                                                     ppart.as<double2>());
            QKG_LAUNCHED();
            if constexpr (NP > 0) {
                lz_proj_finish_kernel<NP><<<1, kT, 0, st>>>(ppart.as<double2>(), bpart.as<double2>(), kUpdGrid,
                                                            state.as<LzState>(), kOrthTol);
                QKG_LAUNCHED();
                lz_orth_kernel<NP><<<kUpdGrid, kT, 0, st>>>(vt, state.as<LzState>(), psi, n, bpart.as<double2>());
                QKG_LAUNCHED();
            }
        };
        switch (np) {
            case 0: sel(std::integral_constant<int, 0>{}); break;
            case 1: sel(std::integral_constant<int, 1>{}); break;
            case 2: sel(std::integral_constant<int, 2>{}); break;
            case 3: sel(std::integral_constant<int, 3>{}); break;
            default: sel(std::integral_constant<int, 4>{}); break;
        }
        lz_beta_kernel<<<1, kT, 0, st>>>(bpart.as<double2>(), kUpdGrid, state.as<LzState>(), beta.as<double>(),
                                         sig.as<double>(), bh.d, static_cast<void* const*>(vtab.p), nmax,
                                         lzop.as<LzOperands>());
        QKG_LAUNCHED();
    };
    int kernels[kMaxPsi + 1] = {};  // kernels per step graph (by Ritz vectors held), counted at capture
    auto capture = [&](int np) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        const uint64_t c0 = launch_count();
        QKG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        enqueue_step(np, nullptr);
        QKG_CUDA(cudaStreamEndCapture(st, &g));
        const int64_t captured = (int64_t)(launch_count() - c0);
        add_launches(-captured);
        kernels[np] = (int)captured;  // kernels per replay
        QKG_CUDA(cudaGraphInstantiate(&ge, g, 0));
        QKG_CUDA(cudaGraphDestroy(g));
        return ge;
    };
    cudaGraphExec_t graphs[kMaxPsi + 1] = {};
    auto destroy_graphs = [&] {
        for (auto& g : graphs)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    };
    std::vector<cudaEvent_t> ev(kInFlight + 2);
    for (auto& e : ev) QKG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));

    int stop_at = -1;       // last accepted step (inclusive)
    bool converged = false;
    double e_old = 1e100;
    const double so_tol = 3.5e-4;
    LaunchTimer timer(st);
    int launched = 0, checked = 0;
    const auto t0 = clk::now();
    try {
        auto check_step = [&](int j) {  // step j has completed
            const double b = bh.h[j];
            if (b < 1e-15) { converged = true; stop_at = j; return; }
            if (j + 1 == nmax) { stop_at = j; return; }
            if (j > 0) {
                std::vector<double> a(ah.h, ah.h + j + 1), bb(bh.h, bh.h + j);
                const double e = tridiag_lowest(a.data(), bb.data(), j + 1);
                if (!o.fixed_steps && std::abs(e - e_old) < o.tol) { converged = true; stop_at = j; return; }
                e_old = e;
                if (j + 1 >= 4) {
                    // Parlett-Scott: lock the Ritz vectors of newly converged low Ritz values
                    for (double theta : ritz_to_lock(a.data(), bb.data(), j + 1, b, so_tol, locked, o.ritz_guard)) {
                        if (npsi >= kMaxPsi) break;
                        std::vector<double> s;
                        if (!tridiag_vector(a.data(), bb.data(), j + 1, theta, s)) continue;
                        // Ritz vector of T_j from v_0..v_j = sig_i V_i (sig_0 = 1, sig_{i+1} = 1/beta_i)
                        std::vector<cd> c(j + 1);
                        double sg = 1.0;
                        for (int i = 0; i <= j; ++i) {
                            c[i] = s[i] * sg;
                            sg = 1.0 / bh.h[i];
                        }
                        float2* p = psi_p + (size_t)npsi * stride;
                        QKG_CUDA(cudaMemsetAsync(p, 0, n * sizeof(float2), st));
                        mcombine_f32(reinterpret_cast<const float2* const*>(vtab.p), j + 1, c.data(), p, n, ws, st);
                        double pn = std::sqrt(nrm2sq_f32(p, n, ws, st));
                        if (!(pn > 0.0)) continue;
                        scal_f32(1.0 / pn, p, n, st);
                        if (npsi > 0) {  // orthonormal to the Ritz vectors already held (two passes)
                            const auto* pt = static_cast<const float2* const*>(psitab.p);
                            for (int pass = 0; pass < 2; ++pass) {
                                std::vector<cd> h(npsi);
                                mdot_f32(pt, npsi, p, n, h.data(), ws, st);
                                for (auto& x : h) x = -x;
                                mcombine_f32(pt, npsi, h.data(), p, n, ws, st);
                            }
                            pn = std::sqrt(nrm2sq_f32(p, n, ws, st));
                            if (pn < 0.5) continue;  // in the span of those held: the same Ritz value again
                            scal_f32(1.0 / pn, p, n, st);
                        }
                        psi.p[npsi++] = p;
                        QKG_CUDA(cudaMemcpyAsync(psitab.p, psi.p, sizeof(psi.p), cudaMemcpyHostToDevice, st));
                        locked.push_back(theta);
                    }
                }
            }
        };
        while (launched < nmax && stop_at < 0) {
            if (launched < kTimedSteps) {
                enqueue_step(npsi, &timer);
                out.t_spmv += timer.collect();  // waits for this SpMV only
                ++out.n_spmv;
            } else {
                cudaGraphExec_t& g = graphs[npsi];
                if (!g) g = capture(npsi);
                QKG_CUDA(cudaGraphLaunch(g, st));
                for (int q = 0; q < kernels[npsi]; ++q) count_launch();
            }
            if (npsi) ++out.n_selective;
            QKG_CUDA(cudaEventRecord(ev[launched % ev.size()], st));
            ++launched;
            while (checked < launched && stop_at < 0) {
                cudaEvent_t e = ev[checked % ev.size()];
                if (launched - checked < kInFlight) {
                    const cudaError_t q = cudaEventQuery(e);
                    if (q == cudaErrorNotReady) break;
                    QKG_CUDA(q);
                } else {
                    QKG_CUDA(cudaEventSynchronize(e));
                }
                check_step(checked);
                ++checked;
            }
        }
        QKG_CUDA(cudaStreamSynchronize(st));
        while (stop_at < 0 && checked < launched) check_step(checked++);
    } catch (...) {
        cudaStreamSynchronize(st);
        for (auto& e : ev) cudaEventDestroy(e);
        destroy_graphs();
        throw;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    destroy_graphs();
    out.n_ritz_locked = npsi;
    out.t_loop = secs(t0, clk::now());
    if (stop_at < 0) stop_at = launched - 1;
    out.iters = stop_at + 1;
    out.converged = converged;
    out.alphas.assign(ah.h, ah.h + stop_at + 1);
    out.betas.assign(bh.h, bh.h + stop_at);  // the last step's beta is not part of T

    // Ritz vector from the FP32 basis, then FP64 Rayleigh quotient and residual.
    const auto t1 = clk::now();
    std::vector<double> s;
    out.energy_tridiag = tridiag_ground(out.alphas.data(), out.betas.data(), (int)out.alphas.size(), s);
    std::vector<cd> c(s.size());
    double sg = 1.0;
    for (size_t i = 0; i < s.size(); ++i) {
        c[i] = s[i] * sg;
        sg = 1.0 / bh.h[i];
    }
    QKG_CUDA(cudaMemsetAsync(r32_p, 0, n * sizeof(float2), st));
    mcombine_f32(reinterpret_cast<const float2* const*>(vtab.p), (int)c.size(), c.data(), r32_p, n, ws, st);
    f32_to_f64(r32_p, r64_p, n, st);
    const double nr = std::sqrt(nrm2sq_f64(r64_p, n, ws, st));
    scal_f64(1.0 / nr, r64_p, n, st);
    H.apply_f64(r64_p, h64_p, st);
    const double E = dot_f64(r64_p, h64_p, n, ws, st).real();
    axpy_f64(-E, r64_p, h64_p, n, st);
    out.residual = std::sqrt(nrm2sq_f64(h64_p, n, ws, st));
    out.energy = E;
    out.t_refine = secs(t1, clk::now());
    if (o.want_vec) {
        cd* dst = o.evec_out;
        if (!dst) {
            out.evec.resize(n);
            dst = out.evec.data();
        }
        const double2* src = r64_p;
        if (H.permuted()) {
            double2* t2 = reinterpret_cast<double2*>(psi_p);  // psi and the FP32 Ritz slot, no longer needed
            H.to_reference_f64(r64_p, t2, st);
            src = t2;
        }
        QKG_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
        QKG_CUDA(cudaStreamSynchronize(st));
    }
    return out;
}

}  // namespace qkg
