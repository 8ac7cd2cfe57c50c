// The C ABI (include/qkrylov_c_api.h).  Handle layout and error translation
// follow the reference's src/c_api.cpp:32-78 (opaque structs, try/catch to
// status codes, NULL from failed creators); the engine behind it is the GPU
// library.
#include "../../include/qkrylov_c_api.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>

#include "block.hpp"
#include "solvers.hpp"

using qkg::cd;

struct qkrylov_sector_t { qkg::Sector sector; };
struct qkrylov_basis_t { std::shared_ptr<qkg::Basis> ptr; };
struct qkrylov_site_t { qkg::SiteKind kind; };
struct qkrylov_opsum_t { std::vector<qkg::Term> terms; };
struct qkrylov_hamiltonian_t {
    std::unique_ptr<qkg::Hamiltonian> ptr;
    // scratch for host-pointer applies, allocated on first use
    qkg::DBuf x64, y64, t64, x32, y32;
};

namespace {

int fail(const std::exception& e) {
    qkg::set_last_error(e.what());
    if (auto* q = dynamic_cast<const qkg::Error*>(&e)) return q->code;
    return QKRYLOV_ERROR_EXCEPTION;
}

template <class F>
int guarded(F&& f) {
    try {
        qkg::set_last_error("");
        f();
        return QKRYLOV_SUCCESS;
    } catch (const std::exception& e) {
        return fail(e);
    } catch (...) {
        qkg::set_last_error("unknown exception");
        return QKRYLOV_ERROR_EXCEPTION;
    }
}

// Solver calls run between two reads of the count of bounded device waits
// that gave up (qkrylov_device_wait_timeouts).  A give-up during the call
// makes its status QKRYLOV_ERROR_DEVICE_TIMEOUT; the kernel that gave up read
// its operand from global memory instead, so the outputs are complete, but the
// caller learns that a wait on an asynchronous copy ran out.
void set_device(qkrylov_hamiltonian_h h);
template <class F>
int guarded_solve(qkrylov_hamiltonian_h h, F&& f) {
    return guarded([&] {
        set_device(h);  // the count belongs to the Hamiltonian's device
        const uint32_t before = qkg::spmv_wait_timeouts();
        f();
        if (qkg::spmv_wait_timeouts() != before)
            throw qkg::Error(qkg::DEVICE_TIMEOUT, "a bounded device wait gave up during this call (outputs computed "
                                                  "from global memory)");
    });
}

qkrylov_basis_h make_basis(qkg::Model m, int n, qkrylov_sector_h sector) {
    try {
        auto h = std::make_unique<qkrylov_basis_t>();
        h->ptr = std::make_shared<qkg::Basis>(m, n, sector ? sector->sector : qkg::Sector());
        return h.release();
    } catch (const std::exception& e) {
        fail(e);
        return nullptr;
    }
}

qkrylov_site_h make_site(qkg::SiteKind k) {
    try {
        auto h = std::make_unique<qkrylov_site_t>();
        h->kind = k;
        return h.release();
    } catch (...) {
        return nullptr;
    }
}

void ensure(qkg::DBuf& b, size_t bytes) {
    if (b.bytes < bytes) b.alloc(bytes);
}

void set_device(qkrylov_hamiltonian_h h) { QKG_CUDA(cudaSetDevice(h->ptr->device())); }

// y = H x for host vectors in reference order, FP64 engine.
void apply_host_f64(qkrylov_hamiltonian_h h, const double* x, double* y) {
    auto& H = *h->ptr;
    const uint64_t n = H.dim();
    if (!n) return;
    set_device(h);
    cudaStream_t s = H.stream();
    ensure(h->x64, n * sizeof(double2));
    ensure(h->y64, n * sizeof(double2));
    ensure(h->t64, n * sizeof(double2));
    QKG_CUDA(cudaMemcpyAsync(h->t64.p, x, n * sizeof(double2), cudaMemcpyHostToDevice, s));
    H.to_internal_f64(h->t64.as<double2>(), h->x64.as<double2>(), s);
    H.apply_f64(h->x64.as<double2>(), h->y64.as<double2>(), s);
    H.to_reference_f64(h->y64.as<double2>(), h->t64.as<double2>(), s);
    QKG_CUDA(cudaMemcpyAsync(y, h->t64.p, n * sizeof(double2), cudaMemcpyDeviceToHost, s));
    QKG_CUDA(cudaStreamSynchronize(s));
}

// One reduction workspace per GPU for the device-vector BLAS calls.
qkg::Workspace& device_workspace() {
    static std::mutex mu;
    static std::vector<std::unique_ptr<qkg::Workspace>> ws;
    int dev = 0;
    QKG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if ((int)ws.size() <= dev) ws.resize(dev + 1);
    if (!ws[dev]) ws[dev] = std::make_unique<qkg::Workspace>();
    return *ws[dev];
}

void fill_result(qkrylov_lanczos_result_f64_t* r, const qkg::LanczosOut& o) {
    r->energy = o.energy;
    r->energy_tridiag = o.energy_tridiag;
    r->residual = o.residual;
    r->iterations = o.iters;
    r->converged = o.converged ? 1 : 0;
    r->selective_steps = o.n_selective;
    r->seconds_loop = o.t_loop;
    r->seconds_refine = o.t_refine;
    r->seconds_spmv = o.t_spmv;
    r->spmv_calls = o.n_spmv;
}

}  // namespace

extern "C" {

const char* qkrylov_last_error(void) { return qkg::last_error(); }

/* ------------------------------------------------------------------ sector */
qkrylov_sector_h qkrylov_sector_create(void) {
    try { return std::make_unique<qkrylov_sector_t>().release(); } catch (...) { return nullptr; }
}
void qkrylov_sector_destroy(qkrylov_sector_h s) { delete s; }
int qkrylov_sector_set_sz(qkrylov_sector_h s, int sz2) {
    if (!s) return QKRYLOV_ERROR_INVALID_ARG;
    s->sector.use_sz = true; s->sector.sz2 = sz2;
    return QKRYLOV_SUCCESS;
}
int qkrylov_sector_set_hubbard_particles(qkrylov_sector_h s, int nup, int ndn) {
    if (!s) return QKRYLOV_ERROR_INVALID_ARG;
    s->sector.use_nup = s->sector.use_ndn = true; s->sector.nup = nup; s->sector.ndn = ndn;
    return QKRYLOV_SUCCESS;
}
int qkrylov_sector_set_nup(qkrylov_sector_h s, int nup) {
    if (!s) return QKRYLOV_ERROR_INVALID_ARG;
    s->sector.use_nup = true; s->sector.nup = nup;
    return QKRYLOV_SUCCESS;
}
int qkrylov_sector_set_ndn(qkrylov_sector_h s, int ndn) {
    if (!s) return QKRYLOV_ERROR_INVALID_ARG;
    s->sector.use_ndn = true; s->sector.ndn = ndn;
    return QKRYLOV_SUCCESS;
}
int qkrylov_sector_set_n(qkrylov_sector_h s, int n) {
    if (!s) return QKRYLOV_ERROR_INVALID_ARG;
    s->sector.use_n = true; s->sector.n = n;
    return QKRYLOV_SUCCESS;
}
int qkrylov_sector_set_nb(qkrylov_sector_h s, int nb) {
    if (!s) return QKRYLOV_ERROR_INVALID_ARG;
    s->sector.use_nb = true; s->sector.nb = nb;
    return QKRYLOV_SUCCESS;
}
int qkrylov_sector_get_sz(qkrylov_sector_h s, int* sz2, int* active) {
    if (!s) return QKRYLOV_ERROR_INVALID_ARG;
    if (active) *active = s->sector.use_sz ? 1 : 0;
    if (sz2) *sz2 = s->sector.sz2;
    return QKRYLOV_SUCCESS;
}
int qkrylov_sector_get_hubbard_particles(qkrylov_sector_h s, int* nup, int* ndn, int* active) {
    if (!s) return QKRYLOV_ERROR_INVALID_ARG;
    if (active) *active = (s->sector.use_nup && s->sector.use_ndn) ? 1 : 0;
    if (nup) *nup = s->sector.nup;
    if (ndn) *ndn = s->sector.ndn;
    return QKRYLOV_SUCCESS;
}
int qkrylov_sector_get_n(qkrylov_sector_h s, int* n, int* active) {
    if (!s) return QKRYLOV_ERROR_INVALID_ARG;
    if (active) *active = s->sector.use_n ? 1 : 0;
    if (n) *n = s->sector.n;
    return QKRYLOV_SUCCESS;
}
int qkrylov_sector_get_nb(qkrylov_sector_h s, int* nb, int* active) {
    if (!s) return QKRYLOV_ERROR_INVALID_ARG;
    if (active) *active = s->sector.use_nb ? 1 : 0;
    if (nb) *nb = s->sector.nb;
    return QKRYLOV_SUCCESS;
}

/* ------------------------------------------------------------------ basis */
qkrylov_basis_h qkrylov_spinhalf_basis_create(int n, qkrylov_sector_h s) { return make_basis(qkg::SPIN, n, s); }
qkrylov_basis_h qkrylov_fermion_basis_create(int n, qkrylov_sector_h s) { return make_basis(qkg::FERMION, n, s); }
qkrylov_basis_h qkrylov_hubbard_basis_create(int n, qkrylov_sector_h s) { return make_basis(qkg::HUBBARD, n, s); }
qkrylov_basis_h qkrylov_tj_basis_create(int n, qkrylov_sector_h s) { return make_basis(qkg::TJ, n, s); }
void qkrylov_basis_destroy(qkrylov_basis_h b) { delete b; }
uint64_t qkrylov_basis_dimension(qkrylov_basis_h b) { return (b && b->ptr) ? b->ptr->dim : 0; }
int qkrylov_basis_nsites(qkrylov_basis_h b) { return (b && b->ptr) ? b->ptr->N : 0; }
uint64_t qkrylov_basis_state(qkrylov_basis_h b, uint64_t i) {
    if (!b || !b->ptr) return 0;
    try { return b->ptr->state_ref(i); } catch (const std::exception& e) { fail(e); return 0; }
}
int qkrylov_basis_states(qkrylov_basis_h b, uint64_t first, uint64_t count, uint64_t* out) {
    if (!b || !b->ptr || (count && !out)) return QKRYLOV_ERROR_INVALID_ARG;
    if (first > b->ptr->dim || count > b->ptr->dim - first) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        const qkg::Basis& B = *b->ptr;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)count; ++i) out[i] = B.state_ref(first + (uint64_t)i);
    });
}
int64_t qkrylov_basis_index(qkrylov_basis_h b, uint64_t s) {
    if (!b || !b->ptr) return -1;
    try { return b->ptr->index_ref(s); } catch (const std::exception& e) { fail(e); return -1; }
}
int qkrylov_basis_contains(qkrylov_basis_h b, uint64_t s) {
    if (!b || !b->ptr) return 0;
    try { return b->ptr->contains_ref(s) ? 1 : 0; } catch (...) { return 0; }
}

/* ------------------------------------------------------------------ site */
qkrylov_site_h qkrylov_spinhalf_site_create(void) { return make_site(qkg::SITE_SPIN); }
qkrylov_site_h qkrylov_fermion_site_create(void) { return make_site(qkg::SITE_FERMION); }
qkrylov_site_h qkrylov_hubbard_site_create(void) { return make_site(qkg::SITE_HUBBARD); }
qkrylov_site_h qkrylov_tj_site_create(void) { return make_site(qkg::SITE_TJ); }
void qkrylov_site_destroy(qkrylov_site_h s) { delete s; }

/* ------------------------------------------------------------------ opsum */
qkrylov_opsum_h qkrylov_opsum_create(void) {
    try { return std::make_unique<qkrylov_opsum_t>().release(); } catch (...) { return nullptr; }
}
void qkrylov_opsum_destroy(qkrylov_opsum_h o) { delete o; }
int qkrylov_opsum_clear(qkrylov_opsum_h o) {
    if (!o) return QKRYLOV_ERROR_INVALID_ARG;
    o->terms.clear();
    return QKRYLOV_SUCCESS;
}
int qkrylov_opsum_add_term_1body(qkrylov_opsum_h o, float cr, float ci, const char* op1, int s1) {
    if (!o || !op1) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] { o->terms.push_back({cd((double)cr, (double)ci), {{op1, s1}}}); });
}
int qkrylov_opsum_add_term_2body(qkrylov_opsum_h o, float cr, float ci, const char* op1, int s1, const char* op2, int s2) {
    if (!o || !op1 || !op2) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] { o->terms.push_back({cd((double)cr, (double)ci), {{op1, s1}, {op2, s2}}}); });
}
int qkrylov_opsum_add_term_nbody_f64(qkrylov_opsum_h o, double cr, double ci, int nf, const char** ops,
                                     const int* sites) {
    if (!o || !ops || !sites || nf <= 0) return QKRYLOV_ERROR_INVALID_ARG;
    for (int i = 0; i < nf; ++i) if (!ops[i]) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        qkg::Term t;
        t.coeff = cd(cr, ci);
        for (int i = 0; i < nf; ++i) t.factors.push_back({ops[i], sites[i]});
        o->terms.push_back(std::move(t));
    });
}
int qkrylov_opsum_add_term_nbody(qkrylov_opsum_h o, float cr, float ci, int nf, const char** ops, const int* sites) {
    return qkrylov_opsum_add_term_nbody_f64(o, (double)cr, (double)ci, nf, ops, sites);
}

/* ------------------------------------------------------------------ hamiltonian */
qkrylov_hamiltonian_h qkrylov_hamiltonian_create(qkrylov_basis_h b, qkrylov_site_h s, qkrylov_opsum_h o) {
    if (!b || !b->ptr || !s || !o) return nullptr;
    try {
        qkg::set_last_error("");
        auto h = std::make_unique<qkrylov_hamiltonian_t>();
        h->ptr = std::make_unique<qkg::Hamiltonian>(b->ptr, s->kind, o->terms);
        return h.release();
    } catch (const std::exception& e) {
        fail(e);
        return nullptr;
    }
}
void qkrylov_hamiltonian_destroy(qkrylov_hamiltonian_h h) {
    if (!h) return;
    if (h->ptr) cudaSetDevice(h->ptr->device());
    delete h;
}
uint64_t qkrylov_hamiltonian_dimension(qkrylov_hamiltonian_h h) { return (h && h->ptr) ? h->ptr->dim() : 0; }

int qkrylov_hamiltonian_apply(qkrylov_hamiltonian_h h, const float* xr, const float* xi, float* yr, float* yi) {
    if (!h || !h->ptr || !xr || !yr) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        const uint64_t n = h->ptr->dim();
        std::vector<cd> x(n), y(n);
        for (uint64_t i = 0; i < n; ++i) x[i] = cd(xr[i], xi ? xi[i] : 0.0f);
        apply_host_f64(h, reinterpret_cast<const double*>(x.data()), reinterpret_cast<double*>(y.data()));
        for (uint64_t i = 0; i < n; ++i) {
            yr[i] = (float)y[i].real();
            if (yi) yi[i] = (float)y[i].imag();
        }
    });
}
int qkrylov_hamiltonian_apply_complex(qkrylov_hamiltonian_h h, const float* x, float* y) {
    if (!h || !h->ptr || !x || !y) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        const uint64_t n = h->ptr->dim();
        std::vector<double> xd(2 * n), yd(2 * n);
        for (uint64_t i = 0; i < 2 * n; ++i) xd[i] = x[i];
        apply_host_f64(h, xd.data(), yd.data());
        for (uint64_t i = 0; i < 2 * n; ++i) y[i] = (float)yd[i];
    });
}
int qkrylov_hamiltonian_apply_complex_f64(qkrylov_hamiltonian_h h, const double* x, double* y) {
    if (!h || !h->ptr || !x || !y) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] { apply_host_f64(h, x, y); });
}
int qkrylov_hamiltonian_diagonal(qkrylov_hamiltonian_h h, float* d) {
    if (!h || !h->ptr || !d) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        set_device(h);
        const auto v = h->ptr->diagonal_host_ref();  // copied device -> host (the reference reads a device view on the host, c_api.cpp:462-466)
        for (size_t i = 0; i < v.size(); ++i) d[i] = (float)v[i].real();
    });
}
int qkrylov_hamiltonian_diagonal_f64(qkrylov_hamiltonian_h h, double* d) {
    if (!h || !h->ptr || !d) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        set_device(h);
        const auto v = h->ptr->diagonal_host_ref();
        for (size_t i = 0; i < v.size(); ++i) d[i] = v[i].real();
    });
}

// Device vectors are read and written as whole complex elements (8-byte float2,
// 16-byte double2): a pointer off that grid is refused before any launch.
static bool on_grid(const void* p, uintptr_t bytes) { return (reinterpret_cast<uintptr_t>(p) & (bytes - 1)) == 0; }

int qkrylov_hamiltonian_apply_device_f64(qkrylov_hamiltonian_h h, const void* dx, void* dy, void* stream) {
    if (!h || !h->ptr || !dx || !dy || !on_grid(dx, 16) || !on_grid(dy, 16)) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        auto& H = *h->ptr;
        set_device(h);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const auto* x = static_cast<const double2*>(dx);
        auto* y = static_cast<double2*>(dy);
        if (!H.permuted()) {
            H.apply_f64(x, y, s);
            return;
        }
        const uint64_t n = H.dim();
        ensure(h->x64, n * sizeof(double2));
        ensure(h->y64, n * sizeof(double2));
        H.to_internal_f64(x, h->x64.as<double2>(), s);
        H.apply_f64(h->x64.as<double2>(), h->y64.as<double2>(), s);
        H.to_reference_f64(h->y64.as<double2>(), y, s);
    });
}
int qkrylov_hamiltonian_apply_device_f32(qkrylov_hamiltonian_h h, const void* dx, void* dy, void* stream) {
    if (!h || !h->ptr || !dx || !dy || !on_grid(dx, 8) || !on_grid(dy, 8)) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        auto& H = *h->ptr;
        set_device(h);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const auto* x = static_cast<const float2*>(dx);
        auto* y = static_cast<float2*>(dy);
        if (!H.permuted()) {
            H.apply_f32(x, y, s);
            return;
        }
        const uint64_t n = H.dim();
        ensure(h->x32, n * sizeof(float2));
        ensure(h->y32, n * sizeof(float2));
        H.to_internal_f32(x, h->x32.as<float2>(), s);
        H.apply_f32(h->x32.as<float2>(), h->y32.as<float2>(), s);
        H.to_reference_f32(h->y32.as<float2>(), y, s);
    });
}

int qkrylov_vector_dot_device_f64(const void* dx, const void* dy, uint64_t n, double* result, void* stream) {
    if (!result || (n && (!dx || !dy || !on_grid(dx, 16) || !on_grid(dy, 16)))) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        result[0] = result[1] = 0.0;
        if (!n) return;
        const auto v = qkg::dot_f64(static_cast<const double2*>(dx), static_cast<const double2*>(dy), n,
                                    device_workspace(), static_cast<cudaStream_t>(stream));
        result[0] = v.real();
        result[1] = v.imag();
    });
}
int qkrylov_vector_dot_device_f32(const void* dx, const void* dy, uint64_t n, double* result, void* stream) {
    if (!result || (n && (!dx || !dy || !on_grid(dx, 8) || !on_grid(dy, 8)))) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        result[0] = result[1] = 0.0;
        if (!n) return;
        const auto v = qkg::dot_f32(static_cast<const float2*>(dx), static_cast<const float2*>(dy), n,
                                    device_workspace(), static_cast<cudaStream_t>(stream));
        result[0] = v.real();
        result[1] = v.imag();
    });
}

int qkrylov_hamiltonian_info(qkrylov_hamiltonian_h h, int* no, int* ni, int* nm, int* nd, int* dm) {
    if (!h || !h->ptr) return QKRYLOV_ERROR_INVALID_ARG;
    if (no) *no = h->ptr->n_outer();
    if (ni) *ni = h->ptr->n_inner();
    if (nm) *nm = h->ptr->n_mixed();
    if (nd) *nd = h->ptr->n_diag();
    if (dm) *dm = h->ptr->diag_mode();
    return QKRYLOV_SUCCESS;
}

int qkrylov_hamiltonian_select_kernel(qkrylov_hamiltonian_h h, int generic, int* fast_in_use) {
    if (!h || !h->ptr || generic < 0 || generic > qkg::Hamiltonian::kMaxMode) return QKRYLOV_ERROR_INVALID_ARG;
    h->ptr->set_kernel_mode(generic);
    if (fast_in_use) *fast_in_use = h->ptr->fast() ? 1 : 0;
    return QKRYLOV_SUCCESS;
}

int qkrylov_hamiltonian_tuning(qkrylov_hamiltonian_h h, int fp32, int* variant, double* ms) {
    if (!h || !h->ptr || !variant) return QKRYLOV_ERROR_INVALID_ARG;
    const auto& H = *h->ptr;
    *variant = H.fast() ? (int)H.variant(fp32 ? 8 : 16) : -1;
    if (*variant >= qkg::kFastVariantsV1) *variant = qkg::kFastVariantsV1;  // a variant this call does not list
    if (ms)
        for (int v = 0; v < qkg::kFastVariantsV1; ++v) ms[v] = H.tuned_ms(fp32 ? 0 : 1, v);
    return QKRYLOV_SUCCESS;
}

int qkrylov_hamiltonian_tuning_ex(qkrylov_hamiltonian_h h, int fp32, int* variant, double* ms, int n_ms) {
    if (!h || !h->ptr || !variant || n_ms < 0 || (n_ms > 0 && !ms)) return QKRYLOV_ERROR_INVALID_ARG;
    const auto& H = *h->ptr;
    *variant = H.fast() ? (int)H.variant(fp32 ? 8 : 16) : -1;
    for (int v = 0; v < n_ms; ++v) ms[v] = v < qkg::kFastVariants ? H.tuned_ms(fp32 ? 0 : 1, v) : 0.0;
    return QKRYLOV_SUCCESS;
}

int qkrylov_hamiltonian_workspace(qkrylov_hamiltonian_h h, int release, uint64_t* bytes) {
    if (!h || !h->ptr) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        set_device(h);
        const auto ws_lock = h->ptr->workspace_lock();
        if (release) h->ptr->release_workspace();
        if (bytes) *bytes = h->ptr->workspace_bytes();
    });
}

int qkrylov_hamiltonian_benchmark_apply(qkrylov_hamiltonian_h h, int fp32, int reps, double* ms) {
    if (!h || !h->ptr || !ms || reps <= 0) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        set_device(h);
        auto& H = *h->ptr;
        const uint64_t n = H.dim();
        *ms = 0.0;
        if (!n) return;
        cudaStream_t s = H.stream();
        const size_t e = fp32 ? sizeof(float2) : sizeof(double2);
        qkg::DBuf x(n * e), y(n * e);
        if (fp32) qkg::philox_normal_f32(7, 0, x.as<float2>(), n, s);
        else qkg::philox_normal_f64(7, 0, x.as<double2>(), n, s);
        auto run = [&] {
            if (fp32) H.apply_f32(x.as<float2>(), y.as<float2>(), s);
            else H.apply_f64(x.as<double2>(), y.as<double2>(), s);
        };
        run();  // warm-up
        qkg::LaunchTimer t(s);
        t.start();
        for (int r = 0; r < reps; ++r) run();
        t.stop();
        *ms = 1e3 * t.collect() / reps;
    });
}

int qkrylov_hamiltonian_entries(qkrylov_hamiltonian_h h, uint64_t* nnz_out, uint64_t* ro, uint64_t* cols, double* vals) {
    if (!h || !h->ptr || !nnz_out) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        set_device(h);
        auto& H = *h->ptr;
        std::vector<uint64_t> iro, icol;
        std::vector<cd> ival;
        H.emit_entries(iro, icol, ival);
        const uint64_t n = H.dim();
        *nnz_out = icol.size();
        if (!ro || !cols || !vals) return;
        // internal row i is reference row ref(i); re-order rows, map columns
        std::vector<uint64_t> ref(n), inv(n);
        for (uint64_t i = 0; i < n; ++i) { ref[i] = H.basis().ref_index_of_int(i); inv[ref[i]] = i; }
        ro[0] = 0;
        for (uint64_t r = 0; r < n; ++r) {
            const uint64_t i = inv[r];
            ro[r + 1] = ro[r] + (iro[i + 1] - iro[i]);
        }
        for (uint64_t r = 0; r < n; ++r) {
            const uint64_t i = inv[r];
            uint64_t o = ro[r];
            for (uint64_t k = iro[i]; k < iro[i + 1]; ++k, ++o) {
                cols[o] = ref[icol[k]];
                vals[2 * o] = ival[k].real();
                vals[2 * o + 1] = ival[k].imag();
            }
        }
    });
}

/* ------------------------------------------------------------------ solvers */
int qkrylov_lanczos_ground_state(qkrylov_hamiltonian_h h, int maxiter, float tol, qkrylov_lanczos_result_c_t* r) {
    return qkrylov_lanczos_ground_state_complex(h, maxiter, tol, r, nullptr);
}
int qkrylov_lanczos_ground_state_complex(qkrylov_hamiltonian_h h, int maxiter, float tol, qkrylov_lanczos_result_c_t* r,
                                         float* ev) {
    if (!h || !h->ptr || !r) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        qkg::LanczosOpts o;
        o.maxiter = maxiter;
        o.tol = (double)tol;
        o.want_vec = ev != nullptr;
        o.f32_stream = true;  // the reference's C API runs its FP32 engine
        const auto res = qkg::lanczos_f64(*h->ptr, o);
        r->energy = (float)res.energy;
        r->iterations = res.iters;
        r->converged = res.converged ? 1 : 0;
        if (ev) for (size_t i = 0; i < res.evec.size(); ++i) { ev[2 * i] = (float)res.evec[i].real(); ev[2 * i + 1] = (float)res.evec[i].imag(); }
    });
}
int qkrylov_lanczos_ground_state_f64(qkrylov_hamiltonian_h h, int maxiter, double tol, const double* v0,
                                     qkrylov_lanczos_result_f64_t* r, double* ev) {
    if (!h || !h->ptr || !r) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        qkg::LanczosOpts o;
        o.maxiter = maxiter;
        o.tol = tol;
        o.want_vec = ev != nullptr;
        o.v0_ref = reinterpret_cast<const cd*>(v0);
        o.evec_out = reinterpret_cast<cd*>(ev);
        const auto res = qkg::lanczos_f64(*h->ptr, o);
        fill_result(r, res);
    });
}
int qkrylov_lanczos_ground_state_mixed(qkrylov_hamiltonian_h h, int maxiter, double tol, const double* v0,
                                       qkrylov_lanczos_result_f64_t* r, double* ev) {
    if (!h || !h->ptr || !r) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        qkg::LanczosOpts o;
        o.maxiter = maxiter;
        o.tol = tol;
        o.want_vec = ev != nullptr;
        o.v0_ref = reinterpret_cast<const cd*>(v0);
        o.evec_out = reinterpret_cast<cd*>(ev);
        const auto res = qkg::lanczos_mixed(*h->ptr, o);
        fill_result(r, res);
    });
}
int qkrylov_lanczos_fixed_steps(qkrylov_hamiltonian_h h, int n_steps, uint64_t seed, int mixed, const double* v0,
                                qkrylov_lanczos_result_f64_t* r, double* ev) {
    if (!h || !h->ptr || !r || n_steps <= 0 || mixed < 0 || mixed > 2) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        qkg::LanczosOpts o;
        o.maxiter = n_steps;
        o.fixed_steps = true;
        o.selective = (mixed == 2);
        o.device_start = (v0 == nullptr);
        o.v0_ref = reinterpret_cast<const cd*>(v0);
        o.seed = seed;
        o.want_vec = ev != nullptr;
        o.evec_out = reinterpret_cast<cd*>(ev);
        const auto res = mixed == 1 ? qkg::lanczos_mixed(*h->ptr, o) : qkg::lanczos_f64(*h->ptr, o);
        fill_result(r, res);
    });
}

int qkrylov_lanczos_ritz_values(qkrylov_hamiltonian_h h, int n_steps, uint64_t seed, int mixed, int n_values,
                                double* values, int* n_out, int* n_locked) {
    if (!h || !h->ptr || !values || !n_out || n_steps <= 0 || n_values <= 0 || mixed < 0 || mixed > 2)
        return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        qkg::LanczosOpts o;
        o.maxiter = n_steps;
        o.fixed_steps = true;
        o.selective = (mixed == 2);
        o.device_start = true;
        o.seed = seed;
        o.ritz_guard = std::min(n_values, qkg::kMaxRitzLocked);  // the wanted end of the spectrum
        const auto res = mixed == 1 ? qkg::lanczos_mixed(*h->ptr, o) : qkg::lanczos_f64(*h->ptr, o);
        std::vector<double> d, z;
        qkg::tridiag_eig(res.alphas.data(), res.betas.data(), (int)res.alphas.size(), d, {}, z);
        std::sort(d.begin(), d.end());
        const int m = std::min<int>(n_values, (int)d.size());
        std::copy(d.begin(), d.begin() + m, values);
        *n_out = m;
        if (n_locked) *n_locked = res.n_ritz_locked;
    });
}

uint64_t qkrylov_kernel_launches(void) { return qkg::launch_count(); }

int qkrylov_device_wait_timeouts(uint32_t* count) {
    if (!count) return QKRYLOV_ERROR_INVALID_ARG;
    int rc = QKRYLOV_SUCCESS;
    const int g = guarded([&] { *count = qkg::spmv_wait_timeouts(); });
    if (g != QKRYLOV_SUCCESS) return g;
    if (*count) rc = QKRYLOV_ERROR_DEVICE_TIMEOUT;
    return rc;
}
constexpr int kMdotMaxVectors = 4088;  // the CUDA-core kernel's limit on k * nw (k alone at nw = 1)
namespace {
// One pointer table and workspace per device for the projection and
// combination entry points, kept between calls (no allocation per call);
// calls are serialised.
struct VectorScratch {
    qkg::DBuf tab;
    std::unique_ptr<qkg::Workspace> ws;
};
std::mutex g_vector_scratch_mu;
std::unique_lock<std::mutex> vector_scratch_lock() { return std::unique_lock<std::mutex>(g_vector_scratch_mu); }
VectorScratch& vector_scratch() {  // caller holds vector_scratch_lock()
    static std::map<int, VectorScratch> scratch;
    int dev = 0;
    QKG_CUDA(cudaGetDevice(&dev));
    VectorScratch& sc = scratch[dev];
    if (!sc.ws) {
        sc.tab.alloc((size_t)kMdotMaxVectors * sizeof(void*));
        sc.ws = std::make_unique<qkg::Workspace>(1 << 16);
    }
    return sc;
}
}  // namespace

int qkrylov_vector_mdot_device_f32(const void* const* v_dev, int k, const void* const* w_dev, int nw, uint64_t n,
                                   int method, double* out, void* stream) {
    if (!v_dev || !w_dev || !out || k < 1 || nw < 1 || nw > 4 || method < 0 || method > 2)
        return QKRYLOV_ERROR_INVALID_ARG;
    if (method == 1 && !qkg::mdot_tc_supported(k, nw)) return QKRYLOV_ERROR_INVALID_ARG;
    if (method != 1 && (size_t)k * nw > 4088) return QKRYLOV_ERROR_INVALID_ARG;
    // complex FP32 elements are loaded as 8-byte pairs (16-byte chunks by the
    // tensor-core kernel): a pointer off that grid is refused before any launch
    const uintptr_t grid = method == 1 ? 16u : 8u;
    for (int j = 0; j < k; ++j)
        if (!on_grid(v_dev[j], grid)) return QKRYLOV_ERROR_INVALID_ARG;
    for (int o = 0; o < nw; ++o)
        if (!on_grid(w_dev[o], grid)) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        auto lk = vector_scratch_lock();
        VectorScratch& sc = vector_scratch();
        QKG_CUDA(cudaMemcpyAsync(sc.tab.p, v_dev, (size_t)k * sizeof(void*), cudaMemcpyHostToDevice, s));
        std::vector<float2*> w(nw);
        for (int o = 0; o < nw; ++o) w[o] = const_cast<float2*>(static_cast<const float2*>(w_dev[o]));
        std::vector<cd> r((size_t)k * nw);
        const auto* V = static_cast<const float2* const*>(sc.tab.p);
        if (method == 1) qkg::mdot_multi_f32_tc(V, k, w.data(), nw, n, r.data(), *sc.ws, s);
        else if (method == 2) qkg::mdot_multi_f32_fast(V, k, w.data(), nw, n, r.data(), *sc.ws, s);
        else qkg::mdot_multi_f32_cuda(V, k, w.data(), nw, n, r.data(), *sc.ws, s);
        for (size_t i = 0; i < r.size(); ++i) {
            out[2 * i] = r[i].real();
            out[2 * i + 1] = r[i].imag();
        }
    });
}

int qkrylov_vector_mcombine_device_f32(const void* const* v_dev, int k, const double* coeffs, void* const* w_dev,
                                       int nw, uint64_t n, int accumulate, void* stream) {
    if (!v_dev || !w_dev || (!coeffs && k > 0) || k < 0 || nw < 1 || nw > 8 || (size_t)k * nw > 1024)
        return QKRYLOV_ERROR_INVALID_ARG;
    for (int j = 0; j < k; ++j)
        if (!on_grid(v_dev[j], 8)) return QKRYLOV_ERROR_INVALID_ARG;
    for (int o = 0; o < nw; ++o)
        if (!on_grid(w_dev[o], 8)) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        auto lk = vector_scratch_lock();
        VectorScratch& sc = vector_scratch();
        if (k > 0)
            QKG_CUDA(cudaMemcpyAsync(sc.tab.p, v_dev, (size_t)k * sizeof(void*), cudaMemcpyHostToDevice, s));
        std::vector<float2*> w(nw);
        for (int o = 0; o < nw; ++o) w[o] = static_cast<float2*>(w_dev[o]);
        std::vector<cd> c((size_t)k * nw);
        for (size_t i = 0; i < c.size(); ++i) c[i] = {coeffs[2 * i], coeffs[2 * i + 1]};
        qkg::mcombine_multi_f32(static_cast<const float2* const*>(sc.tab.p), k, c.data(), w.data(), nw, n,
                                accumulate != 0, *sc.ws, s);
    });
}

int qkrylov_set_projection_kernel(int method) {
    if (method < 0 || method > 2) return QKRYLOV_ERROR_INVALID_ARG;
    qkg::set_projection_mode(method);
    return QKRYLOV_SUCCESS;
}

int qkrylov_debug_inject_alloc_failure(int64_t after_n) {
    qkg::inject_alloc_failure(after_n);
    return QKRYLOV_SUCCESS;
}
int64_t qkrylov_debug_live_allocations(void) { return qkg::live_device_allocs(); }
int qkrylov_debug_device_wait_probe(int64_t limit_ns) {
    if (limit_ns <= 0) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded([&] { qkg::tilek::wait_probe((long long)limit_ns); });
}

int qkrylov_set_device(int id) {
    return guarded([&] { QKG_CUDA(cudaSetDevice(id)); });
}
int qkrylov_device_count(int* count) {
    if (!count) return QKRYLOV_ERROR_INVALID_ARG;
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();  // no driver or no device: zero GPUs, not an error
        c = 0;
    }
    *count = c;
    return QKRYLOV_SUCCESS;
}
int qkrylov_device_synchronize(void) {
    return guarded([&] { QKG_CUDA(cudaDeviceSynchronize()); });
}

int qkrylov_davidson_lowest_complex(qkrylov_hamiltonian_h h, int n_eig, int max_sub, float tol, float* evals, float* evecs,
                                    qkrylov_davidson_result_c_t* info) {
    if (!h || !h->ptr || !evals || n_eig <= 0) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        const auto res = qkg::davidson_f64(*h->ptr, n_eig, max_sub, (double)tol, evecs != nullptr, true);
        const size_t k = std::min<size_t>((size_t)n_eig, res.evals.size());
        for (size_t i = 0; i < k; ++i) evals[i] = (float)res.evals[i];
        if (info) { info->iterations = res.iters; info->converged = res.converged ? 1 : 0; }
        if (evecs) {
            const uint64_t n = h->ptr->dim();
            for (size_t j = 0; j < k && j < res.evecs.size(); ++j)
                for (uint64_t i = 0; i < n; ++i) {
                    evecs[j * 2 * n + 2 * i] = (float)res.evecs[j][i].real();
                    evecs[j * 2 * n + 2 * i + 1] = (float)res.evecs[j][i].imag();
                }
        }
    });
}
int qkrylov_davidson_lowest_complex_f64(qkrylov_hamiltonian_h h, int n_eig, int max_sub, double tol, double* evals,
                                        double* evecs, qkrylov_davidson_result_c_t* info) {
    if (!h || !h->ptr || !evals || n_eig <= 0) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        const auto res = qkg::davidson_f64(*h->ptr, n_eig, max_sub, tol, evecs != nullptr);
        const size_t k = std::min<size_t>((size_t)n_eig, res.evals.size());
        for (size_t i = 0; i < k; ++i) evals[i] = res.evals[i];
        if (info) { info->iterations = res.iters; info->converged = res.converged ? 1 : 0; }
        if (evecs) {
            const uint64_t n = h->ptr->dim();
            for (size_t j = 0; j < k && j < res.evecs.size(); ++j) std::memcpy(evecs + j * 2 * n, res.evecs[j].data(), n * sizeof(cd));
        }
    });
}

int qkrylov_davidson_lowest_ex(qkrylov_hamiltonian_h h, int n_eig, int max_sub, double tol, int mixed, int max_iter,
                               double* evals, double* evecs, double* residuals, qkrylov_davidson_result_c_t* info,
                               double* seconds) {
    if (!h || !h->ptr || !evals || n_eig <= 0 || max_iter < 1 || max_iter > 100) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        const auto res = mixed ? qkg::davidson_mixed(*h->ptr, n_eig, max_sub, tol, evecs != nullptr, max_iter)
                               : qkg::davidson_f64(*h->ptr, n_eig, max_sub, tol, evecs != nullptr, false, max_iter);
        const size_t k = std::min<size_t>((size_t)n_eig, res.evals.size());
        for (size_t i = 0; i < k; ++i) evals[i] = res.evals[i];
        if (residuals)
            for (size_t i = 0; i < k; ++i) residuals[i] = i < res.residuals.size() ? res.residuals[i] : -1.0;
        if (info) { info->iterations = res.iters; info->converged = res.converged ? 1 : 0; }
        if (seconds) *seconds = res.seconds;
        if (evecs) {
            const uint64_t n = h->ptr->dim();
            for (size_t j = 0; j < k && j < res.evecs.size(); ++j) std::memcpy(evecs + j * 2 * n, res.evecs[j].data(), n * sizeof(cd));
        }
    });
}

int qkrylov_continued_fraction_coeffs_complex(qkrylov_hamiltonian_h h, const float* phi0, int n_iter, float* alphas,
                                              float* betas, float* norm, int* num) {
    if (!h || !h->ptr || !phi0 || !alphas || !betas || !norm || n_iter <= 0) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        const uint64_t n = h->ptr->dim();
        std::vector<cd> p(n);
        for (uint64_t i = 0; i < n; ++i) p[i] = cd(phi0[2 * i], phi0[2 * i + 1]);
        const auto res = qkg::cf_f64(*h->ptr, p.data(), n_iter);
        *norm = (float)res.norm;
        for (size_t i = 0; i < res.alphas.size() && i < (size_t)n_iter; ++i) alphas[i] = (float)res.alphas[i];
        for (size_t i = 0; i < res.betas.size() && i < (size_t)n_iter; ++i) betas[i] = (float)res.betas[i];
        if (num) *num = (int)res.alphas.size();
    });
}
int qkrylov_continued_fraction_coeffs_complex_f64(qkrylov_hamiltonian_h h, const double* phi0, int n_iter, double* alphas,
                                                  double* betas, double* norm, int* num, int* num_betas) {
    if (!h || !h->ptr || !phi0 || !alphas || !betas || !norm || n_iter <= 0) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        const auto res = qkg::cf_f64(*h->ptr, reinterpret_cast<const cd*>(phi0), n_iter);
        *norm = res.norm;
        std::copy(res.alphas.begin(), res.alphas.end(), alphas);
        std::copy(res.betas.begin(), res.betas.end(), betas);
        if (num) *num = (int)res.alphas.size();
        if (num_betas) *num_betas = (int)res.betas.size();
    });
}
float qkrylov_evaluate_spectral_function(const float* alphas, const float* betas, size_t n, float norm, float omega,
                                         float E0, float eta) {
    if (!alphas || !betas || n == 0) return 0.0f;
    std::vector<double> a(alphas, alphas + n), b(n > 0 ? n - 1 : 0);
    for (size_t i = 0; i + 1 < n; ++i) b[i] = betas[i];
    b.push_back(0.0);
    return (float)qkg::spectral(a.data(), b.data(), n, norm, omega, E0, eta);
}
double qkrylov_evaluate_spectral_function_f64(const double* alphas, const double* betas, size_t n, double norm,
                                              double omega, double E0, double eta) {
    if (!alphas || !betas || n == 0) return 0.0;
    return qkg::spectral(alphas, betas, n, norm, omega, E0, eta);
}
int qkrylov_evaluate_spectral_grid_f64(const double* alphas, const double* betas, size_t n, double norm,
                                       const double* omegas, size_t n_omega, double E0, double eta, double* out) {
    if (!alphas || !betas || !omegas || !out) return QKRYLOV_ERROR_INVALID_ARG;
    // frequencies are independent: spread large grids over the host cores
    // (each value is computed exactly as in the serial loop)
#pragma omp parallel for schedule(static) if (n_omega * (n + 1) >= 65536)
    for (long long k = 0; k < (long long)n_omega; ++k)
        out[k] = n ? qkg::spectral(alphas, betas, n, norm, omegas[k], E0, eta) : 0.0;
    return QKRYLOV_SUCCESS;
}

int qkrylov_ftlm(qkrylov_hamiltonian_h h, float beta, int n_random, int n_steps, qkrylov_ftlm_result_c_t* r) {
    if (!h || !h->ptr || !r) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        r->beta = beta;
        r->partition_function = r->internal_energy = r->specific_heat = 0.0f;
        if (h->ptr->dim() == 0) return;
        // random vectors as the reference's FP32 engine draws them (normal_distribution<float>)
        const auto tri = qkg::ftlm_tridiags_f64(*h->ptr, n_random, n_steps, true);
        const double b = (double)beta;
        double Z, E, C;
        qkg::ftlm_observables(tri, &b, 1, &Z, &E, &C, false, nullptr);
        r->partition_function = (float)Z;
        r->internal_energy = (float)E;
        r->specific_heat = (float)C;
    });
}
int qkrylov_ftlm_f64(qkrylov_hamiltonian_h h, double beta, int n_random, int n_steps, qkrylov_ftlm_result_f64_t* r) {
    if (!h || !h->ptr || !r) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        r->beta = beta;
        r->partition_function = r->internal_energy = r->specific_heat = 0.0;
        if (h->ptr->dim() == 0) return;
        const auto tri = qkg::ftlm_tridiags_f64(*h->ptr, n_random, n_steps);
        double Z, E, C;
        qkg::ftlm_observables(tri, &beta, 1, &Z, &E, &C, false, nullptr);
        r->partition_function = Z;
        r->internal_energy = E;
        r->specific_heat = C;
    });
}
int qkrylov_ftlm_multi_beta_f64(qkrylov_hamiltonian_h h, const double* betas, int n_beta, int n_random, int n_steps,
                                double* Z, double* E, double* Cv, double* log_shift) {
    if (!h || !h->ptr || !betas || n_beta < 0 || !Z || !E || !Cv) return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(h, [&] {
        set_device(h);
        const auto tri = qkg::ftlm_tridiags_f64(*h->ptr, n_random, n_steps);
        qkg::ftlm_observables(tri, betas, n_beta, Z, E, Cv, log_shift != nullptr, log_shift);
    });
}

}  // extern "C"

// ---- batched Lanczos over block vectors ------------------------------------------
namespace {
bool collect_hams(const qkrylov_hamiltonian_h* hams, int n, std::vector<qkg::Hamiltonian*>& hs) {
    if (!hams || n <= 0) return false;
    for (int i = 0; i < n; ++i) {
        if (!hams[i] || !hams[i]->ptr) return false;
        hs.push_back(hams[i]->ptr.get());
    }
    return true;
}
void fill_stats(const qkg::BlockTridiag& t, qkrylov_block_stats_t* st) {
    if (!st) return;
    st->seconds = t.seconds;
    st->spmv_ms = t.spmv_ms;
    st->vectors_per_lane = t.vpl;
    st->padded_vectors = t.rp;
    st->rows = t.rows;
    for (int i = 0; i < 3; ++i) st->tune_ms[i] = i < (int)t.tune_ms.size() ? t.tune_ms[i] : 0.0;
}
qkg::BlockOpts block_opts(int n_vec, int n_steps, int mixed, int start_kind, uint64_t seed) {
    qkg::BlockOpts o;
    o.R = n_vec;
    o.steps = n_steps;
    o.mixed = mixed != 0;
    o.seed = seed;
    switch (start_kind) {
        case QKRYLOV_START_FTLM_STREAM: o.start = qkg::BlockStart::FtlmStream; break;
        case QKRYLOV_START_FTLM_STREAM_F32: o.start = qkg::BlockStart::FtlmStream; o.f32_stream = true; break;
        case QKRYLOV_START_PHILOX: o.start = qkg::BlockStart::Philox; break;
        case QKRYLOV_START_GIVEN: o.start = qkg::BlockStart::Given; break;
        default: throw qkg::Error(QKRYLOV_ERROR_INVALID_ARG, "unknown start kind");
    }
    return o;
}
}  // namespace

extern "C" {

int qkrylov_block_lanczos_tridiag(const qkrylov_hamiltonian_h* hams, int n_ham, int n_vec, int n_steps, int mixed,
                                  int vectors_per_lane, int start_kind, uint64_t seed, const double* start_vectors,
                                  double* alphas,
                                  double* betas, int* n_alpha, int* n_beta, double* norm2,
                                  qkrylov_block_stats_t* stats) {
    std::vector<qkg::Hamiltonian*> hs;
    if (!collect_hams(hams, n_ham, hs) || n_vec < 1 || n_vec > 32 || n_steps < 0 || !alphas || !betas || !n_alpha ||
        !n_beta || !norm2 || (start_kind == QKRYLOV_START_GIVEN && !start_vectors) ||
        (vectors_per_lane != 0 && vectors_per_lane != 1 && vectors_per_lane != 2 && vectors_per_lane != 4))
        return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(hams[0], [&] {
        set_device(hams[0]);
        qkg::BlockOpts o = block_opts(n_vec, n_steps, mixed, start_kind, seed);
        o.vpl = vectors_per_lane;
        if (o.start == qkg::BlockStart::Given) {
            const cd* p = reinterpret_cast<const cd*>(start_vectors);
            for (auto* H : hs)
                for (int v = 0; v < n_vec; ++v) {
                    o.given.push_back(p);
                    p += H->dim();
                }
        }
        const qkg::BlockTridiag t = qkg::block_lanczos(hs, o);
        const size_t nv = (size_t)n_ham * n_vec;
        for (size_t i = 0; i < nv; ++i) {
            n_alpha[i] = (int)t.alpha[i].size();
            n_beta[i] = (int)t.beta[i].size();
            norm2[i] = t.norm2[i];
            for (int k = 0; k < n_steps; ++k) {
                alphas[i * n_steps + k] = k < n_alpha[i] ? t.alpha[i][k] : 0.0;
                betas[i * n_steps + k] = k < n_beta[i] ? t.beta[i][k] : 0.0;
            }
        }
        fill_stats(t, stats);
    });
}

int qkrylov_ftlm_sectors_f64(const qkrylov_hamiltonian_h* hams, int n_ham, const double* betas, int n_beta,
                             int n_random, int n_steps, int mixed, int start_kind, uint64_t seed, double* Z, double* E,
                             double* Cv, double* log_shift, qkrylov_block_stats_t* stats) {
    std::vector<qkg::Hamiltonian*> hs;
    if (!collect_hams(hams, n_ham, hs) || !betas || n_beta < 0 || n_random < 1 || n_random > 32 || n_steps < 0 ||
        !Z || !E || !Cv || start_kind == QKRYLOV_START_GIVEN)
        return QKRYLOV_ERROR_INVALID_ARG;
    return guarded_solve(hams[0], [&] {
        set_device(hams[0]);
        const qkg::BlockTridiag t = qkg::block_lanczos(hs, block_opts(n_random, n_steps, mixed, start_kind, seed));
        qkg::ftlm_observables_block(t, betas, n_beta, Z, E, Cv, log_shift != nullptr, log_shift);
        fill_stats(t, stats);
    });
}

int qkrylov_cf_block_f64(qkrylov_hamiltonian_h h, const double* phi0, int n_rhs, int n_iter, int mixed,
                         double* alphas, double* betas, int* n_alpha, int* n_beta, double* norms,
                         qkrylov_block_stats_t* stats) {
    if (!h || !h->ptr || !phi0 || n_rhs < 1 || n_rhs > 32 || n_iter < 0 || !alphas || !betas || !n_alpha || !n_beta ||
        !norms)
        return QKRYLOV_ERROR_INVALID_ARG;
    std::vector<double> n2((size_t)n_rhs);
    const int rc = qkrylov_block_lanczos_tridiag(&h, 1, n_rhs, n_iter, mixed, 0, QKRYLOV_START_GIVEN, 0, phi0, alphas,
                                                 betas, n_alpha, n_beta, n2.data(), stats);
    if (rc == QKRYLOV_SUCCESS)
        for (int i = 0; i < n_rhs; ++i) {
            const double nr = std::sqrt(n2[i]);
            norms[i] = nr < 1e-15 ? 0.0 : nr;  // dynamics.cpp:27: a zero right-hand side has no coefficients
        }
    return rc;
}

}  // extern "C"
