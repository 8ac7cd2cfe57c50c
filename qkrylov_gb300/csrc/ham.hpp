// Hamiltonian object, device vectors and the Krylov-algebra launchers.
#pragma once

#include "qkg.hpp"

#include <cuda_runtime.h>

#include <complex>
#include <memory>
#include <mutex>
#include <vector>

namespace qkg {

// Owning device buffer.
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    explicit DBuf(size_t n) { alloc(n); }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    DBuf& operator=(DBuf&& o) noexcept { reset(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; return *this; }
    ~DBuf() { reset(); }
    void alloc(size_t n);
    void reset();
    template <class T> T* as() const { return static_cast<T*>(p); }
};

enum DiagMode : int { DIAG_U8 = 0, DIAG_U16 = 1, DIAG_FULL = 2 };

// Fast SpMV kernel variants: one row per thread, the outer block's slice of x
// staged in shared memory, four rows per thread, four rows per thread with the
// block staged, four rows per thread with a larger register budget, the
// tiled kernel over 1, 2 or 4 outer blocks per CTA, and the class-persistent
// kernel (spmv_tile.cu).
enum FastVariant : int {
    FV_ROW = 0, FV_STAGED = 1, FV_ROWS4 = 2, FV_ROWS4_STAGED = 3, FV_ROWS4_WIDE = 4,
    FV_TILE1 = 5, FV_TILE2 = 6, FV_TILE4 = 7, FV_CLASS = 8
};
constexpr int kFastVariants = 9;
constexpr int kFastVariantsV1 = 5;  // variants reported by qkrylov_hamiltonian_tuning
inline int tile_g(FastVariant v) { return v == FV_TILE1 ? 1 : v == FV_TILE2 ? 2 : v == FV_TILE4 ? 4 : 0; }
inline int tile_index(int g) { return g == 1 ? 0 : g == 2 ? 1 : 2; }

// Bounded device waits of the SpMV kernels that gave up on the current GPU
// (waits for the GPU first).
uint32_t spmv_wait_timeouts();
// bounded waits of the tensor-core projection kernel that gave up (part of the above)
uint32_t tc_wait_timeouts();
namespace tilek {
// Test hook: one bounded wait (limit_ns of global time, clamped to 1 us .. 1 s)
// on an mbarrier that nothing completes, counted as a give-up.
void wait_probe(long long limit_ns);
}  // namespace tilek

// Device-resident Lanczos step.  The operands of one Lanczos-mode SpMV are kept
// in device memory and rewritten by the step's last kernel for the next step:
// y = scale H x - bprev vprev (vprev null: no previous-vector term); the SpMV
// writes one Re<x, y> partial per block to apart.
struct LzOperands {
    const void* x = nullptr;
    void* y = nullptr;
    const void* vprev = nullptr;
    double scale = 1.0, bprev = 0.0;
    float scale32 = 1.f, bprev32 = 0.f;  // the same, rounded once for FP32 kernels
};
struct LanczosHooks {
    const LzOperands* op = nullptr;  // device
    double2* apart = nullptr;        // per-block partials of Re<x, y>
};

namespace fastk {
template <class A> struct FastParams;
}

// Per-precision copy of the compiled term lists.
struct TermSet {
    DBuf outer, inner, mixed, diag, all, vars;
    int n_outer = 0, n_inner = 0, n_mixed = 0, n_diag = 0, n_all = 0;
};

class Hamiltonian {
public:
    Hamiltonian(std::shared_ptr<Basis> basis, SiteKind site, const std::vector<Term>& terms);
    ~Hamiltonian();

    uint64_t dim() const { return basis_->dim; }
    Basis& basis() { return *basis_; }
    cudaStream_t stream() const { return stream_; }
    int device() const { return dev_; }
    const DevBasis& dbasis() const { return *db_; }
    bool permuted() const { return basis_->permuted; }
    bool all_real() const { return all_real_; }

    // y = H x on device vectors in internal order (interleaved complex).
    void apply_f64(const double2* x, double2* y, cudaStream_t s) const;
    void apply_f32(const float2* x, float2* y, cudaStream_t s) const;
    // One FP32 SpMV of the device-resident Lanczos step (fast kernel only);
    // writes n_items() partials to lz.apart.
    void apply_lanczos_f32(const LanczosHooks& lz, cudaStream_t s) const;

    // Diagonal H_ii (complex, internal order) into a device buffer.
    void diagonal_f64(double2* d, cudaStream_t s) const;

    // Reference order <-> internal order for device vectors.
    void to_internal_f64(const double2* ref, double2* in, cudaStream_t s) const;
    void to_reference_f64(const double2* in, double2* ref, cudaStream_t s) const;
    void to_internal_f32(const float2* ref, float2* in, cudaStream_t s) const;
    void to_reference_f32(const float2* in, float2* ref, cudaStream_t s) const;

    // Debug: every generated matrix entry, rows in internal order, entries in
    // OpSum term order (row_offsets[dim+1], cols = internal indices, vals).
    void emit_entries(std::vector<uint64_t>& row_offsets, std::vector<uint64_t>& cols,
                      std::vector<std::complex<double>>& vals) const;

    // Host-side helpers
    std::vector<std::complex<double>> diagonal_host_ref() const;  // reference order

    // Compile statistics
    int n_outer() const { return t64_.n_outer; }
    int n_inner() const { return t64_.n_inner; }
    int n_mixed() const { return t64_.n_mixed; }
    int n_diag() const { return t64_.n_diag; }
    int diag_mode() const { return diag_mode_; }
    size_t n_items() const { return n_items_; }
    bool fast() const { return fast_ && !force_generic_; }
    // kernel mode: 0 automatic (autotuned), 1 generic kernel, 2 fast kernel
    // one row per thread, 3 fast kernel with shared-memory staging, 4 fast
    // kernel four rows per thread, 5 four rows per thread with staging, 6 four
    // rows per thread with the larger register budget, 7 / 8 / 9 the tiled
    // kernel over 1 / 2 / 4 outer blocks per CTA, 10 the class-persistent kernel
    static constexpr int kMaxMode = 10;
    void set_kernel_mode(int m) { mode_ = m; force_generic_ = (m == 1); }
    void force_generic(bool on) { set_kernel_mode(on ? 1 : 0); }
    // fast-kernel variant for vectors of elem_bytes per element
    // dynamic shared memory of a staged variant: the largest outer block's slice
    // of x plus one element on either side (the copy starts on a 16-byte boundary)
    size_t stage_bytes(size_t elem_bytes) const { return ((max_block_ + 2) * elem_bytes + 15) / 16 * 16; }
    // the tiled kernel over G blocks per CTA fits its shared memory
    bool can_tile(int G, size_t elem_bytes) const;
    size_t tile_smem_bytes(int G, size_t elem_bytes) const;
    uint32_t tile_slot_elems(size_t elem_bytes) const;
    const void* tile_items(int G) const { return tile_items_[tile_index(G)].p; }
    // class-persistent kernel: its shared memory fits; its plan (device
    // pointers), shared memory and grid (one CTA per SM, at most one per block)
    bool can_class(size_t elem_bytes) const;
    size_t class_smem_bytes(size_t elem_bytes) const;
    unsigned class_grid() const { return class_grid_; }
    const void* class_blocks() const { return class_blocks_.p; }  // tilek::CBlock
    const void* class_info() const { return class_info_.p; }      // tilek::CClass
    uint32_t class_nblocks() const { return class_nblocks_; }
    uint32_t class_ell_cap() const { return class_ell_cap_; }
    uint32_t class_gcap() const { return class_gcap_; }
    uint32_t class_maxw() const { return class_maxw_; }
    size_t n_tile_items(int G) const { return n_tile_[tile_index(G)]; }
    FastVariant variant(size_t elem_bytes) const {
        const bool can_stage = max_block_ > 0 && stage_bytes(elem_bytes) <= kStageLimit;
        if (mode_ >= 7 && mode_ <= 9) {
            const FastVariant t = (FastVariant)(FV_TILE1 + (mode_ - 7));
            return can_tile(tile_g(t), elem_bytes) ? t : FV_ROWS4;
        }
        if (mode_ == 10) return can_class(elem_bytes) ? FV_CLASS : FV_ROWS4;
        if (mode_ == 2) return FV_ROW;
        if (mode_ == 3) return can_stage ? FV_STAGED : FV_ROW;
        if (mode_ == 4) return FV_ROWS4;
        if (mode_ == 5) return can_stage ? FV_ROWS4_STAGED : FV_ROWS4;
        if (mode_ == 6) return FV_ROWS4_WIDE;
        const FastVariant v = pref_[elem_bytes == 16 ? 1 : 0];
        if (tile_g(v) && !can_tile(tile_g(v), elem_bytes)) return FV_ROWS4;
        if (v == FV_CLASS && !can_class(elem_bytes)) return FV_ROWS4;
        if (v == FV_STAGED && !can_stage) return FV_ROW;
        if (v == FV_ROWS4_STAGED && !can_stage) return FV_ROWS4;
        return v;
    }
    bool staged(size_t elem_bytes) const {
        return fast() && (variant(elem_bytes) == FV_STAGED || variant(elem_bytes) == FV_ROWS4_STAGED);
    }
    // autotuner record: mean ms of [precision][variant] (0 when not measured)
    double tuned_ms(int prec, int v) const { return tune_ms_[prec][v]; }
    size_t inner_table_entries() const { return n_ient_; }
    // Fast-kernel parameters (one work item per <= 1024 rows of an outer
    // block) for arithmetic type A (float or double).
    template <class A> void fast_params(fastk::FastParams<A>& p) const;
    bool uniform_inner() const { return unif_; }
    const WorkItem* items_device() const { return items_.as<WorkItem>(); }
    // host copy of the fast kernel's work items
    std::vector<WorkItem> items_host() const;
    size_t lanczos_parts() const;  // partial sums written by apply_lanczos_f32
    static constexpr size_t kStageLimit = 200 * 1024;

    // Device memory kept between solver calls on this Hamiltonian (the Krylov
    // space of the device-resident Lanczos, tens of GB): cudaFree of 64 GB
    // takes about 25 ms, a tenth of a 200-step run.  Grows on demand, contents
    // undefined; released with the Hamiltonian or by release_workspace().
    // A solver that uses the workspace holds workspace_lock() for the whole
    // call, so two calls on one Hamiltonian from different host threads take
    // turns instead of freeing each other's Krylov space.
    DBuf& krylov_workspace(size_t bytes) const;
    void release_workspace() const { kws_.reset(); }
    size_t workspace_bytes() const { return kws_.bytes; }
    std::unique_lock<std::mutex> workspace_lock() const { return std::unique_lock<std::mutex>(kws_mu_); }

private:
    void build_diagonal();
    void build_fast();
    template <class S> void upload_terms(const std::vector<HostTerm>& ht);

    // fast-path data (see spmv_fast_kernel)
    struct FastSet {
        DBuf outer, inner, mixed, vars;
        DBuf oent;  // per-block outer entries (OutEnt of this precision)
        int n_outer = 0, n_inner = 0, n_mixed = 0, outer_has_j = 0;
    };
    void autotune();
    // the work-item list and count a fast variant runs on
    const WorkItem* items_of(FastVariant v, size_t* n) const;
    bool fast_ = false, force_generic_ = false, unif_ = false;
    int mode_ = 0;
    FastVariant pref_[2] = {FV_ROWS4, FV_ROWS4};
    double tune_ms_[2][kFastVariants] = {};
    DBuf items_blk_;            // one work item per outer block (staged kernel)
    size_t n_items_blk_ = 0, max_block_ = 0;
    DBuf class_blocks_, class_info_;  // class-persistent kernel: sorted blocks, per-class table ranges
    uint32_t class_nblocks_ = 0, class_ell_cap_ = 0, class_gcap_ = 0, class_maxw_ = 0;
    unsigned class_grid_ = 0;
    DBuf tile_items_[3];        // tiled kernel: groups of 1, 2, 4 outer blocks
    size_t n_tile_[3] = {0, 0, 0};
    double u_ar_ = 0.0, u_ai_ = 0.0;
    int rbits_ = 0;
    size_t n_ient_ = 0;
    FastSet f64s_, f32s_;
    DBuf iptr_, ient_;
    DBuf optr_, mptr_, ment_;  // per-block outer-entry / straddling-term list offsets and straddling entries

    std::shared_ptr<Basis> basis_;
    const DevBasis* db_ = nullptr;
    SiteKind site_;
    int dev_ = 0;
    cudaStream_t stream_ = nullptr;
    bool wide_ = false;       // states need 64 bits
    bool all_real_ = true;
    std::vector<HostTerm> hterms_;
    TermSet t64_, t32_;
    DBuf items_;
    size_t n_items_ = 0;
    int diag_mode_ = DIAG_U8;
    DBuf dcode_, dtab64_, dtab32_, dfull64_, dfull32_;
    int n_dtab_ = 0;
    mutable DBuf kws_;
    mutable std::mutex kws_mu_;
};

// ------------------------------------------------------------ Krylov algebra
// Reductions return to the host (one sync); FP32 reductions are compensated
// (Ogita-Rump-Oishi Dot2: TwoProduct via fma, TwoSum accumulation) so their
// error is that of a computation in twice the working precision.
struct Workspace {
    DBuf partial;     // per-block partial sums
    DBuf result;      // device-side result slots
    double* host = nullptr;  // pinned host result slots
    size_t cap_partials = 0;
    explicit Workspace(size_t max_blocks_times_k = 1 << 16);
    ~Workspace();
};

std::complex<double> dot_f64(const double2* x, const double2* y, uint64_t n, Workspace& ws, cudaStream_t s);
std::complex<double> dot_f32(const float2* x, const float2* y, uint64_t n, Workspace& ws, cudaStream_t s);
double nrm2sq_f64(const double2* x, uint64_t n, Workspace& ws, cudaStream_t s);
double nrm2sq_f32(const float2* x, uint64_t n, Workspace& ws, cudaStream_t s);
void axpy_f64(std::complex<double> a, const double2* x, double2* y, uint64_t n, cudaStream_t s);
void axpy_f32(std::complex<double> a, const float2* x, float2* y, uint64_t n, cudaStream_t s);
void scal_f64(double a, double2* x, uint64_t n, cudaStream_t s);
void scal_f32(double a, float2* x, uint64_t n, cudaStream_t s);
void f64_to_f32(const double2* x, float2* y, uint64_t n, cudaStream_t s);
void f32_to_f64(const float2* x, double2* y, uint64_t n, cudaStream_t s);
// w -= alpha v + beta vprev (vprev may be null); returns ||w||^2 (fused pass).
double lanczos_update_f64(double2* w, const double2* v, const double2* vprev, double alpha, double beta, uint64_t n,
                          Workspace& ws, cudaStream_t s);
double lanczos_update_f32(float2* w, const float2* v, const float2* vprev, double alpha, double beta, uint64_t n,
                          Workspace& ws, cudaStream_t s);
// out[j] = <V_j, w> for j < k (one pass over w, V given as device pointer array).
void mdot_f64(const double2* const* V_dev, int k, const double2* w, uint64_t n, std::complex<double>* out,
              Workspace& ws, cudaStream_t s);
void mdot_f32(const float2* const* V_dev, int k, const float2* w, uint64_t n, std::complex<double>* out,
              Workspace& ws, cudaStream_t s);
// out[o * k + j] = <V_j, W_o> for j < k, o < nw <= 4: one pass over the V_j for
// all W_o (compensated FP32; W a host array of device pointers).
void mdot_multi_f32(const float2* const* V_dev, int k, float2* const* W, int nw, uint64_t n,
                    std::complex<double>* out, Workspace& ws, cudaStream_t s);
// The compensated CUDA-core kernel whatever the projection mode.
void mdot_multi_f32_cuda(const float2* const* V_dev, int k, float2* const* W, int nw, uint64_t n,
                         std::complex<double>* out, Workspace& ws, cudaStream_t s);
// the same with FP32 sums over runs of 32 elements (projection mode 2)
void mdot_multi_f32_fast(const float2* const* V_dev, int k, float2* const* W, int nw, uint64_t n,
                         std::complex<double>* out, Workspace& ws, cudaStream_t s);
// The same on the tensor cores (tcgen05, 3xTF32 products, FP32 accumulation
// read out into FP64 every thousand or so terms; mdot_tc.cu): k <= 128, nw <= 4.
bool mdot_tc_supported(int k, int nw);
size_t mdot_tc_smem(int k, int nw);
void mdot_multi_f32_tc(const float2* const* V_dev, int k, float2* const* W, int nw, uint64_t n,
                       std::complex<double>* out, Workspace& ws, cudaStream_t s);
// Which kernel mdot_multi_f32 uses: 0 the compensated CUDA-core kernel
// (FP64-accurate), 1 the tensor-core kernel where it applies.
void set_projection_mode(int mode);
int projection_mode();
// w += sum_j c[j] V_j  (c given on the host, k <= 1024)
void mcombine_f64(const double2* const* V_dev, int k, const std::complex<double>* c, double2* w, uint64_t n,
                  Workspace& ws, cudaStream_t s);
void mcombine_f32(const float2* const* V_dev, int k, const std::complex<double>* c, float2* w, uint64_t n,
                  Workspace& ws, cudaStream_t s);
// W_o = (accumulate ? W_o : 0) + sum_j c[o * k + j] V_j for o < nout <= 8 (one
// pass over the V_j; V and W given as device pointer arrays for V, host array
// of device pointers for W; c on the host, nout * k <= 1024).
void mcombine_multi_f64(const double2* const* V_dev, int k, const std::complex<double>* c, double2* const* W, int nout,
                        uint64_t n, bool accumulate, Workspace& ws, cudaStream_t s);
void mcombine_multi_f32(const float2* const* V_dev, int k, const std::complex<double>* c, float2* const* W, int nout,
                        uint64_t n, bool accumulate, Workspace& ws, cudaStream_t s);
// Davidson preconditioner t_i = r_i / (d_i - lambda) with the reference's clamp.
void davidson_precond_f64(const double2* r, const double2* d, double lambda, double2* t, uint64_t n, cudaStream_t s);
void davidson_precond_f32(const float2* r, const double2* d, double lambda, float2* t, uint64_t n, cudaStream_t s);

}  // namespace qkg
