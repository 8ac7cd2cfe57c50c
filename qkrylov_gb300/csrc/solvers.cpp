// Solver drivers.  All Krylov vectors stay on the device; the host holds
// only the small projected problems (tridiagonal / subspace matrices).
#include "solvers.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <limits>
#include <numeric>
#include <random>
#include <type_traits>

namespace qkg {

namespace {
using clk = std::chrono::steady_clock;
inline double secs(clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); }

// Device vectors of one size recycled within a solve: a Davidson iteration
// otherwise allocates and frees gigabytes (corrections, restarts), and both
// cudaFree and the first touch of fresh pages cost milliseconds per GB.
struct VecPool {
    size_t bytes;
    std::vector<DBuf> free;
    explicit VecPool(size_t b) : bytes(b) {}
    DBuf get(size_t held) {
        if (!free.empty()) {
            DBuf b = std::move(free.back());
            free.pop_back();
            return b;
        }
        size_t fr = 0, tot = 0;
        QKG_CUDA(cudaMemGetInfo(&fr, &tot));
        if (fr < bytes + (64ull << 20))
            throw Error(CUDA_ERR, "out of device memory for the Krylov basis (" + std::to_string(held) + " vectors held)");
        return DBuf(bytes);
    }
    void put(DBuf&& b) {
        if (b.p) free.push_back(std::move(b));
    }
};

// A growing list of device vectors plus the device array of their pointers
// (what the multi-vector kernels take); with a pool, vectors come from and go
// back to it.
template <class T2>
struct VecList {
    uint64_t n = 0;
    std::vector<DBuf> bufs;
    std::vector<T2*> host_ptrs;
    DBuf dev_ptrs;
    size_t cap = 0;
    VecPool* pool = nullptr;
    explicit VecList(uint64_t n_, VecPool* p = nullptr) : n(n_), pool(p) {}
    ~VecList() { clear(); }
    T2* push() {
        if (pool) {
            bufs.push_back(pool->get(bufs.size()));
        } else {
            size_t fr = 0, tot = 0;
            QKG_CUDA(cudaMemGetInfo(&fr, &tot));
            if (fr < n * sizeof(T2) + (64ull << 20))
                throw Error(CUDA_ERR, "out of device memory for the Krylov basis (" + std::to_string(bufs.size()) + " vectors held)");
            bufs.emplace_back(n * sizeof(T2));
        }
        host_ptrs.push_back(bufs.back().as<T2>());
        sync_ptrs();
        return host_ptrs.back();
    }
    // append a vector that is already on the device (n elements), taking ownership
    T2* adopt(DBuf&& b) {
        bufs.push_back(std::move(b));
        host_ptrs.push_back(bufs.back().as<T2>());
        sync_ptrs();
        return host_ptrs.back();
    }
    void sync_ptrs() {
        if (host_ptrs.size() > cap) {
            cap = std::max<size_t>(64, host_ptrs.size() * 2);
            dev_ptrs.alloc(cap * sizeof(T2*));
        }
        if (!host_ptrs.empty())
            QKG_CUDA(cudaMemcpy(dev_ptrs.p, host_ptrs.data(), host_ptrs.size() * sizeof(T2*), cudaMemcpyHostToDevice));
    }
    void clear() {
        if (pool)
            for (auto& b : bufs) pool->put(std::move(b));
        bufs.clear();
        host_ptrs.clear();
    }
    void pop() {  // drop the newest vector
        if (bufs.empty()) return;
        if (pool) pool->put(std::move(bufs.back()));
        bufs.pop_back();
        host_ptrs.pop_back();
    }
    void take(std::vector<DBuf>& nb) {
        clear();
        bufs = std::move(nb);
        host_ptrs.clear();
        for (auto& b : bufs) host_ptrs.push_back(b.as<T2>());
        sync_ptrs();
    }
    size_t size() const { return host_ptrs.size(); }
    T2* operator[](size_t i) const { return host_ptrs[i]; }
    const T2* const* dev() const { return static_cast<const T2* const*>(dev_ptrs.p); }
};

size_t ws_cap(int k) { return std::max<size_t>(1 << 16, (size_t)1216 * (size_t)std::max(k, 1)); }

// Appends the Ritz vector sum_i c_i V_i (normalised, Gram-Schmidt against the
// Ritz vectors already held) to psi; false, with nothing appended, when it lies
// in the span of those (the same Ritz value seen again).
template <class T2>
bool push_ritz(VecList<T2>& psi, const T2* const* V, int k, const std::vector<cd>& c, uint64_t n, Workspace& ws,
               cudaStream_t st) {
    constexpr bool F32 = sizeof(T2) == 8;
    T2* p = psi.push();
    QKG_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T2), st));
    auto nrm = [&](const T2* x) {
        if constexpr (F32) return std::sqrt(nrm2sq_f32(x, n, ws, st));
        else return std::sqrt(nrm2sq_f64(x, n, ws, st));
    };
    auto scal = [&](double a, T2* x) {
        if constexpr (F32) scal_f32(a, x, n, st);
        else scal_f64(a, x, n, st);
    };
    if constexpr (F32) mcombine_f32(V, k, c.data(), p, n, ws, st);
    else mcombine_f64(V, k, c.data(), p, n, ws, st);
    const double n0 = nrm(p);
    if (!(n0 > 0.0)) { psi.pop(); return false; }
    scal(1.0 / n0, p);
    const int m = (int)psi.size() - 1;
    if (m > 0) {
        for (int pass = 0; pass < 2; ++pass) {  // twice is enough (Kahan's "twice is enough")
            std::vector<cd> h(m);
            if constexpr (F32) mdot_f32(psi.dev(), m, p, n, h.data(), ws, st);
            else mdot_f64(psi.dev(), m, p, n, h.data(), ws, st);
            for (auto& x : h) x = -x;
            if constexpr (F32) mcombine_f32(psi.dev(), m, h.data(), p, n, ws, st);
            else mcombine_f64(psi.dev(), m, h.data(), p, n, ws, st);
        }
        const double n1 = nrm(p);
        if (n1 < 0.5) { psi.pop(); return false; }
        scal(1.0 / n1, p);
    }
    return true;
}

void upload_ref_f64(Hamiltonian& H, const cd* host_ref, double2* d_int, DBuf& tmp) {
    const uint64_t n = H.dim();
    if (!H.permuted()) {
        QKG_CUDA(cudaMemcpyAsync(d_int, host_ref, n * sizeof(double2), cudaMemcpyHostToDevice, H.stream()));
        return;
    }
    if (tmp.bytes < n * sizeof(double2)) tmp.alloc(n * sizeof(double2));
    QKG_CUDA(cudaMemcpyAsync(tmp.p, host_ref, n * sizeof(double2), cudaMemcpyHostToDevice, H.stream()));
    H.to_internal_f64(tmp.as<double2>(), d_int, H.stream());
}
void download_ref_f64(Hamiltonian& H, const double2* d_int, cd* host_ref, DBuf& tmp) {
    const uint64_t n = H.dim();
    const double2* src = d_int;
    if (H.permuted()) {
        if (tmp.bytes < n * sizeof(double2)) tmp.alloc(n * sizeof(double2));
        H.to_reference_f64(d_int, tmp.as<double2>(), H.stream());
        src = tmp.as<double2>();
    }
    QKG_CUDA(cudaMemcpyAsync(host_ref, src, n * sizeof(double2), cudaMemcpyDeviceToHost, H.stream()));
    QKG_CUDA(cudaStreamSynchronize(H.stream()));
}
}  // namespace

LaunchTimer::LaunchTimer(cudaStream_t s) : s_(s) {
    QKG_CUDA(cudaEventCreate(&a_));
    QKG_CUDA(cudaEventCreate(&b_));
}
LaunchTimer::~LaunchTimer() {
    if (a_) cudaEventDestroy(a_);
    if (b_) cudaEventDestroy(b_);
}
void LaunchTimer::start() { QKG_CUDA(cudaEventRecord(a_, s_)); }
void LaunchTimer::stop() { QKG_CUDA(cudaEventRecord(b_, s_)); }
double LaunchTimer::collect() {
    float ms = 0.0f;
    QKG_CUDA(cudaEventSynchronize(b_));
    QKG_CUDA(cudaEventElapsedTime(&ms, a_, b_));
    return ms * 1e-3;
}

// ============================================================ small eigenproblems
double tridiag_lowest(const double* a, const double* b, int n) {
    if (n <= 0) return 0.0;
    if (n == 1) return a[0];
    double lo = std::numeric_limits<double>::infinity(), hi = -lo;
    for (int i = 0; i < n; ++i) {
        const double r = (i > 0 ? std::abs(b[i - 1]) : 0.0) + (i < n - 1 ? std::abs(b[i]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
    }
    const double scale = std::max(std::abs(lo), std::abs(hi));
    const double tiny = std::numeric_limits<double>::min() / std::numeric_limits<double>::epsilon();
    auto count_below = [&](double x) {  // Sturm count: eigenvalues < x
        int cnt = 0;
        double q = a[0] - x;
        if (q < 0) ++cnt;
        for (int i = 1; i < n; ++i) {
            if (q == 0.0) q = tiny;
            q = a[i] - x - b[i - 1] * b[i - 1] / q;
            if (q < 0) ++cnt;
        }
        return cnt;
    };
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (hi - lo <= 2.0 * std::numeric_limits<double>::epsilon() * scale || mid == lo || mid == hi) break;
        if (count_below(mid) >= 1) hi = mid;
        else lo = mid;
    }
    return 0.5 * (lo + hi);
}

// Implicit QL with Wilkinson-type shifts (the symmetric tridiagonal QL of
// Bowdler, Martin, Reinsch & Wilkinson, Numer. Math. 11 (1968)), rotating only
// the requested rows of the eigenvector matrix.
void tridiag_eig(const double* a, const double* b, int n, std::vector<double>& d, const std::vector<int>& rows,
                 std::vector<double>& z) {
    d.assign(a, a + n);
    std::vector<double> e(n, 0.0);
    for (int i = 0; i + 1 < n; ++i) e[i] = b[i];
    const int nr = (int)rows.size();
    z.assign((size_t)nr * n, 0.0);
    for (int r = 0; r < nr; ++r) if (rows[r] >= 0 && rows[r] < n) z[(size_t)r * n + rows[r]] = 1.0;
    const double eps = std::numeric_limits<double>::epsilon();
    for (int l = 0; l < n; ++l) {
        for (int iter = 0; iter < 100; ++iter) {
            int m = l;
            for (; m < n - 1; ++m) {
                const double dd = std::abs(d[m]) + std::abs(d[m + 1]);
                if (std::abs(e[m]) <= eps * dd) break;
            }
            if (m == l) break;
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = std::hypot(g, 1.0);
            g = d[m] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
            double s = 1.0, c = 1.0, p = 0.0;
            int i = m - 1;
            bool underflow = false;
            for (; i >= l; --i) {
                const double f = s * e[i], bb = c * e[i];
                r = std::hypot(f, g);
                e[i + 1] = r;
                if (r == 0.0) {
                    d[i + 1] -= p;
                    e[m] = 0.0;
                    underflow = true;
                    break;
                }
                s = f / r;
                c = g / r;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * bb;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - bb;
                for (int q = 0; q < nr; ++q) {
                    double* zr = &z[(size_t)q * n];
                    const double t = zr[i + 1];
                    zr[i + 1] = s * zr[i] + c * t;
                    zr[i] = c * zr[i] - s * t;
                }
            }
            if (underflow) continue;
            d[l] -= p;
            e[l] = g;
            e[m] = 0.0;
        }
    }
}

// Lowest eigenpair of the symmetric tridiagonal (a, b) in O(n): the eigenvalue
// by Sturm bisection (tridiag_lowest), the eigenvector by inverse iteration on
// T - lambda I with a tridiagonal LU with row interchanges (Gaussian
// elimination with partial pivoting; zero pivots replaced by eps ||T||).  The
// QL algorithm with all eigenvector rows costs O(n^3): 13 ms at n = 200.
double tridiag_ground(const double* a, const double* b, int n, std::vector<double>& vec) {
    if (n <= 0) { vec.clear(); return 0.0; }
    if (n == 1) { vec.assign(1, 1.0); return a[0]; }
    const double lam = tridiag_lowest(a, b, n);
    if (!tridiag_vector(a, b, n, lam, vec)) return tridiag_ground_ql(a, b, n, vec);
    return lam;
}

bool tridiag_vector(const double* a, const double* b, int n, double lam, std::vector<double>& vec) {
    if (n <= 0) { vec.clear(); return true; }
    if (n == 1) { vec.assign(1, 1.0); return true; }
    double tn = 0.0;
    for (int i = 0; i < n; ++i)
        tn = std::max(tn, std::abs(a[i]) + (i > 0 ? std::abs(b[i - 1]) : 0.0) + (i + 1 < n ? std::abs(b[i]) : 0.0));
    const double pert = std::numeric_limits<double>::epsilon() * std::max(tn, std::numeric_limits<double>::min());
    // factor P (T - lam I) = L U: U has three diagonals u0, u1, u2; L unit lower with multipliers m
    std::vector<double> u0(n), u1(n, 0.0), u2(n, 0.0), m(n, 0.0);
    std::vector<char> swp(n, 0);
    double dcur = a[0] - lam, ucur = n > 1 ? b[0] : 0.0;  // row i of the remaining matrix: (dcur, ucur) at columns i, i+1
    for (int i = 0; i + 1 < n; ++i) {
        const double l = b[i], dn = a[i + 1] - lam, un = i + 2 < n ? b[i + 1] : 0.0;  // row i+1: (l, dn, un)
        if (std::abs(dcur) >= std::abs(l)) {
            if (dcur == 0.0) dcur = pert;
            u0[i] = dcur;
            u1[i] = ucur;
            m[i] = l / dcur;
            dcur = dn - m[i] * ucur;
            ucur = un;
        } else {  // rows i and i+1 interchanged
            swp[i] = 1;
            u0[i] = l;
            u1[i] = dn;
            u2[i] = un;
            m[i] = dcur / l;
            const double d2 = ucur - m[i] * dn;
            ucur = -m[i] * un;
            dcur = d2;
        }
    }
    u0[n - 1] = dcur == 0.0 ? pert : dcur;
    auto solve = [&](std::vector<double>& x) {
        for (int i = 0; i + 1 < n; ++i) {
            if (swp[i]) std::swap(x[i], x[i + 1]);
            x[i + 1] -= m[i] * x[i];
        }
        for (int i = n - 1; i >= 0; --i) {
            double t = x[i];
            if (i + 1 < n) t -= u1[i] * x[i + 1];
            if (i + 2 < n) t -= u2[i] * x[i + 2];
            x[i] = t / u0[i];
        }
    };
    std::vector<double> x(n, 1.0), prev;
    for (int it = 0; it < 6; ++it) {
        solve(x);
        double nr = 0.0;
        for (double v : x) nr += v * v;
        nr = std::sqrt(nr);
        if (!(nr > 0.0) || !std::isfinite(nr)) return false;
        for (double& v : x) v /= nr;
        if (it > 0) {
            double ov = 0.0;
            for (int i = 0; i < n; ++i) ov += x[i] * prev[i];
            if (std::abs(std::abs(ov) - 1.0) < 4.0 * std::numeric_limits<double>::epsilon()) break;
        }
        prev = x;
    }
    // a fixed sign: the largest component positive
    int im = 0;
    for (int i = 1; i < n; ++i) if (std::abs(x[i]) > std::abs(x[im])) im = i;
    if (x[im] < 0) for (double& v : x) v = -v;
    vec = std::move(x);
    return true;
}

std::vector<double> ritz_to_lock(const double* a, const double* b, int k, double beta, double tol,
                                 const std::vector<double>& locked, int max_locked) {
    std::vector<double> out;
    max_locked = std::max(1, std::min(max_locked, kMaxRitzLocked));
    if (k < 4 || (int)locked.size() >= max_locked) return out;
    std::vector<double> d, z;
    tridiag_eig(a, b, k, d, {k - 1}, z);
    std::vector<int> idx(k);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
    double tn = 0.0;
    for (double x : d) tn = std::max(tn, std::abs(x));
    for (int r = 0; r < std::min(k, max_locked) && (int)(locked.size() + out.size()) < max_locked; ++r) {
        const int i = idx[r];
        if (beta * std::abs(z[i]) > tol * tn) continue;  // not converged
        bool known = false;
        for (double t : locked) known = known || std::abs(t - d[i]) <= tol * tn;
        for (double t : out) known = known || std::abs(t - d[i]) <= tol * tn;
        if (!known) out.push_back(d[i]);
    }
    return out;
}

// The same by the QL algorithm with every eigenvector row (O(n^3)): the
// fallback of tridiag_ground when inverse iteration breaks down.
double tridiag_ground_ql(const double* a, const double* b, int n, std::vector<double>& vec) {
    if (n <= 0) { vec.clear(); return 0.0; }
    if (n == 1) { vec.assign(1, 1.0); return a[0]; }
    std::vector<int> rows(n);
    std::iota(rows.begin(), rows.end(), 0);
    std::vector<double> d, z;
    tridiag_eig(a, b, n, d, rows, z);
    int mi = 0;
    for (int j = 1; j < n; ++j) if (d[j] < d[mi]) mi = j;
    vec.resize(n);
    for (int i = 0; i < n; ++i) vec[i] = z[(size_t)i * n + mi];
    return d[mi];
}

void hermitian_eig(const std::vector<cd>& H, int m, std::vector<double>& evals, std::vector<std::vector<cd>>& vecs) {
    std::vector<cd> A = H, V((size_t)m * m, 0.0);
    for (int i = 0; i < m; ++i) V[(size_t)i * m + i] = 1.0;
    auto at = [&](std::vector<cd>& M, int i, int j) -> cd& { return M[(size_t)i * m + j]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < m; ++i) {
            diag += std::norm(at(A, i, i));
            for (int j = i + 1; j < m; ++j) off += std::norm(at(A, i, j));
        }
        if (off <= 1e-32 * std::max(diag, 1e-300)) break;
        for (int p = 0; p < m; ++p)
            for (int q = p + 1; q < m; ++q) {
                const cd apq = at(A, p, q);
                const double mag = std::abs(apq);
                if (mag < 1e-300) continue;
                const cd ph = apq / mag;  // e^{i phi}
                const double app = at(A, p, p).real(), aqq = at(A, q, q).real();
                const double tau = (aqq - app) / (2.0 * mag);
                const double t = (tau >= 0 ? 1.0 : -1.0) / (std::abs(tau) + std::sqrt(1.0 + tau * tau));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
                // U on (p,q): U_pp = c, U_pq = s, U_qp = -s e^{-i phi}, U_qq = c e^{-i phi}
                const cd upp = c, upq = s, uqp = -s * std::conj(ph), uqq = c * std::conj(ph);
                for (int k = 0; k < m; ++k) {  // A <- A U, V <- V U
                    const cd akp = at(A, k, p), akq = at(A, k, q);
                    at(A, k, p) = akp * upp + akq * uqp;
                    at(A, k, q) = akp * upq + akq * uqq;
                    const cd vkp = at(V, k, p), vkq = at(V, k, q);
                    at(V, k, p) = vkp * upp + vkq * uqp;
                    at(V, k, q) = vkp * upq + vkq * uqq;
                }
                for (int k = 0; k < m; ++k) {  // A <- U^H A
                    const cd apk = at(A, p, k), aqk = at(A, q, k);
                    at(A, p, k) = std::conj(upp) * apk + std::conj(uqp) * aqk;
                    at(A, q, k) = std::conj(upq) * apk + std::conj(uqq) * aqk;
                }
                at(A, p, q) = at(A, q, p) = 0.0;
                at(A, p, p) = at(A, p, p).real();
                at(A, q, q) = at(A, q, q).real();
            }
    }
    std::vector<int> idx(m);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int i, int j) { return at(A, i, i).real() < at(A, j, j).real(); });
    evals.clear();
    vecs.clear();
    for (int i : idx) {
        evals.push_back(at(A, i, i).real());
        std::vector<cd> v(m);
        for (int k = 0; k < m; ++k) v[k] = at(V, k, i);
        vecs.push_back(std::move(v));
    }
}

// ============================================================ random streams
void ref_uniform_complex(uint32_t seed, uint64_t n, cd* out, bool f32) {
    std::mt19937 rng(seed);
    if (f32) {
        std::uniform_real_distribution<float> dist(-1.0f, 1.0f);
        fill_stream(rng, dist, n, out);
    } else {
        std::uniform_real_distribution<double> dist(-1.0, 1.0);
        fill_stream(rng, dist, n, out);
    }
}

// ============================================================ Lanczos (FP64)
// A Krylov workspace an earlier mixed run left on H is freed when a run that
// allocates its own vectors (bytes of them) would not fit beside it.
void release_workspace_if_short(Hamiltonian& H, size_t bytes) {
    if (!H.workspace_bytes()) return;
    size_t fr = 0, tot = 0;
    QKG_CUDA(cudaMemGetInfo(&fr, &tot));
    if (bytes + (1ull << 30) < fr) return;
    const auto ws_lock = H.workspace_lock();
    H.release_workspace();
}

LanczosOut lanczos_f64(Hamiltonian& H, const LanczosOpts& o) {
    LanczosOut out;
    const uint64_t n = H.dim();
    if (n == 0) return out;
    cudaStream_t st = H.stream();
    const int nmax = (int)std::min<uint64_t>((uint64_t)std::max(o.maxiter, 0), n);
    release_workspace_if_short(H, (size_t)(nmax + 3) * n * sizeof(double2));
    Workspace ws(ws_cap(nmax + 2));
    VecList<double2> V(n);
    DBuf w(n * sizeof(double2)), tmp;
    double2* v = V.push();
    if (o.device_start) {
        philox_normal_f64(o.seed, 0, v, n, st);
    } else {
        std::vector<cd> h;
        const cd* src = o.v0_ref;
        if (!src) {
            h.resize(n);
            ref_uniform_complex(1234, n, h.data(), o.f32_stream);  // src/solvers/lanczos.cpp:115-120
            src = h.data();
        }
        upload_ref_f64(H, src, v, tmp);
        QKG_CUDA(cudaStreamSynchronize(st));
    }
    const double nr0 = std::sqrt(nrm2sq_f64(v, n, ws, st));
    if (nr0 != 0.0) scal_f64(1.0 / nr0, v, n, st);

    auto& alphas = out.alphas;
    auto& betas = out.betas;
    double e_old = 1e100;
    std::vector<cd> c;
    // o.selective: instead of the reference's full reorthogonalisation, the
    // mixed form's scheme in FP64 (Parlett-Scott: once one of the lowest Ritz
    // pairs has converged, |beta_k s_k| <= sqrt(eps_64) ||T||, later vectors are
    // kept orthogonal to its Ritz vector) -- the control that separates the
    // mixed form's precision from its reorthogonalisation
    VecList<double2> psi(n);
    std::vector<double> locked;  // Ritz values whose vectors are in psi
    const double so_tol = 1.5e-8;  // sqrt(eps_fp64)
    LaunchTimer timer(st);
    const auto t0 = clk::now();
    for (int iter = 0; iter < nmax; ++iter) {
        out.iters = iter + 1;
        v = V[V.size() - 1];
        const double2* vp = iter > 0 ? V[V.size() - 2] : nullptr;
        timer.start();
        H.apply_f64(v, w.as<double2>(), st);
        timer.stop();
        const double alpha = dot_f64(v, w.as<double2>(), n, ws, st).real();  // synchronises the stream
        out.t_spmv += timer.collect();
        ++out.n_spmv;
        alphas.push_back(alpha);
        double b2 = lanczos_update_f64(w.as<double2>(), v, vp, alpha, iter > 0 ? betas.back() : 0.0, n, ws, st);
        if (!o.selective) {
            // full reorthogonalisation against every stored vector (:148-151), one CGS pass
            const int k = (int)V.size();
            c.assign(k, 0.0);
            mdot_f64(V.dev(), k, w.as<double2>(), n, c.data(), ws, st);
            for (auto& x : c) x = -x;
            mcombine_f64(V.dev(), k, c.data(), w.as<double2>(), n, ws, st);
            b2 = nrm2sq_f64(w.as<double2>(), n, ws, st);
        } else if (psi.size()) {
            c.assign(psi.size(), 0.0);
            mdot_f64(psi.dev(), (int)psi.size(), w.as<double2>(), n, c.data(), ws, st);
            for (auto& x : c) x = -x;
            mcombine_f64(psi.dev(), (int)psi.size(), c.data(), w.as<double2>(), n, ws, st);
            b2 = nrm2sq_f64(w.as<double2>(), n, ws, st);
            ++out.n_selective;
        }
        const double beta = std::sqrt(b2);
        if (beta < 1e-15) { out.converged = true; break; }
        if (iter + 1 == nmax) break;
        betas.push_back(beta);
        double2* vn = V.push();
        QKG_CUDA(cudaMemcpyAsync(vn, w.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        scal_f64(1.0 / beta, vn, n, st);
        const int k = (int)alphas.size();
        if (iter > 0 && !o.fixed_steps) {
            const double e = tridiag_lowest(alphas.data(), betas.data(), k);
            if (std::abs(e - e_old) < o.tol) { out.converged = true; break; }
            e_old = e;
        }
        if (o.selective && k >= 4) {
            for (double theta : ritz_to_lock(alphas.data(), betas.data(), k, beta, so_tol, locked, o.ritz_guard)) {
                std::vector<double> sv;
                if (!tridiag_vector(alphas.data(), betas.data(), k, theta, sv)) continue;
                std::vector<cd> cc(sv.begin(), sv.end());
                if (push_ritz(psi, V.dev(), k, cc, n, ws, st)) locked.push_back(theta);
            }
        }
    }
    QKG_CUDA(cudaStreamSynchronize(st));
    out.t_loop = secs(t0, clk::now());
    out.n_ritz_locked = (int)psi.size();
    std::vector<double> s;
    out.energy = tridiag_ground(alphas.data(), betas.data(), (int)alphas.size(), s);
    out.energy_tridiag = out.energy;
    out.residual = -1.0;
    if (o.want_vec) {
        DBuf ritz(n * sizeof(double2));
        QKG_CUDA(cudaMemsetAsync(ritz.p, 0, n * sizeof(double2), st));
        std::vector<cd> cc(s.size());
        for (size_t i = 0; i < s.size(); ++i) cc[i] = s[i];
        mcombine_f64(V.dev(), (int)s.size(), cc.data(), ritz.as<double2>(), n, ws, st);
        const double nr = std::sqrt(nrm2sq_f64(ritz.as<double2>(), n, ws, st));
        if (nr != 0.0) scal_f64(1.0 / nr, ritz.as<double2>(), n, st);
        cd* dst = o.evec_out;
        if (!dst) {
            out.evec.resize(n);
            dst = out.evec.data();
        }
        download_ref_f64(H, ritz.as<double2>(), dst, tmp);
    }
    return out;
}

// ============================================================ Lanczos (mixed)
LanczosOut lanczos_mixed(Hamiltonian& H, const LanczosOpts& o) {
    LanczosOut out;
    const uint64_t n = H.dim();
    if (n == 0) return out;
    if (lanczos_device_supported(H)) {
        size_t fr = 0, tot = 0;
        QKG_CUDA(cudaMemGetInfo(&fr, &tot));
        // the Krylov workspace an earlier run left on the Hamiltonian is reused
        // (or freed first) by the device-resident run: it counts as available
        const size_t held = H.workspace_bytes();
        if (lanczos_device_bytes(H, o.maxiter) + (1ull << 30) < fr + held) return lanczos_mixed_device(H, o);
        // the host-driven run allocates its own vectors: give it that memory back
        const auto ws_lock = H.workspace_lock();
        H.release_workspace();
    }
    cudaStream_t st = H.stream();
    const int nmax = (int)std::min<uint64_t>((uint64_t)std::max(o.maxiter, 0), n);
    Workspace ws(ws_cap(nmax + 2));
    VecList<float2> V(n);
    VecList<float2> psi(n);  // converged Ritz vectors used for selective reorthogonalisation
    std::vector<double> locked;  // their Ritz values
    DBuf w(n * sizeof(float2)), tmp;
    float2* v = V.push();
    if (o.device_start) {
        philox_normal_f32(o.seed, 0, v, n, st);
    } else {
        std::vector<cd> h;
        const cd* src = o.v0_ref;
        if (!src) {
            h.resize(n);
            ref_uniform_complex(1234, n, h.data());
            src = h.data();
        }
        DBuf d64(n * sizeof(double2));
        upload_ref_f64(H, src, d64.as<double2>(), tmp);
        f64_to_f32(d64.as<double2>(), v, n, st);
        QKG_CUDA(cudaStreamSynchronize(st));
    }
    const double nr0 = std::sqrt(nrm2sq_f32(v, n, ws, st));
    if (nr0 != 0.0) scal_f32(1.0 / nr0, v, n, st);

    auto& alphas = out.alphas;
    auto& betas = out.betas;
    double e_old = 1e100;
    std::vector<cd> c;
    const double so_tol = 3.5e-4;  // sqrt(eps_fp32): Parlett-Scott selective-orthogonalisation threshold
    LaunchTimer timer(st);
    const auto t0 = clk::now();
    for (int iter = 0; iter < nmax; ++iter) {
        out.iters = iter + 1;
        v = V[V.size() - 1];
        const float2* vp = iter > 0 ? V[V.size() - 2] : nullptr;
        timer.start();
        H.apply_f32(v, w.as<float2>(), st);
        timer.stop();
        const double alpha = dot_f32(v, w.as<float2>(), n, ws, st).real();  // synchronises the stream
        out.t_spmv += timer.collect();
        ++out.n_spmv;
        alphas.push_back(alpha);
        double b2 = lanczos_update_f32(w.as<float2>(), v, vp, alpha, iter > 0 ? betas.back() : 0.0, n, ws, st);
        if (psi.size()) {
            c.assign(psi.size(), 0.0);
            mdot_f32(psi.dev(), (int)psi.size(), w.as<float2>(), n, c.data(), ws, st);
            for (auto& x : c) x = -x;
            mcombine_f32(psi.dev(), (int)psi.size(), c.data(), w.as<float2>(), n, ws, st);
            b2 = nrm2sq_f32(w.as<float2>(), n, ws, st);
            ++out.n_selective;
        }
        const double beta = std::sqrt(b2);
        if (beta < 1e-15) { out.converged = true; break; }
        if (iter + 1 == nmax) break;
        betas.push_back(beta);
        float2* vn = V.push();
        QKG_CUDA(cudaMemcpyAsync(vn, w.p, n * sizeof(float2), cudaMemcpyDeviceToDevice, st));
        scal_f32(1.0 / beta, vn, n, st);
        const int k = (int)alphas.size();
        if (iter > 0) {
            const double e = tridiag_lowest(alphas.data(), betas.data(), k);
            if (!o.fixed_steps && std::abs(e - e_old) < o.tol) { out.converged = true; break; }
            e_old = e;
            // Selective reorthogonalisation: once one of the lowest Ritz pairs
            // has converged to FP32 level (|beta_k s_k| <= sqrt(eps) ||T||),
            // keep later Lanczos vectors orthogonal to its Ritz vector.
            if (k >= 4) {
                for (double theta : ritz_to_lock(alphas.data(), betas.data(), k, beta, so_tol, locked, o.ritz_guard)) {
                    std::vector<double> sv;
                    if (!tridiag_vector(alphas.data(), betas.data(), k, theta, sv)) continue;
                    std::vector<cd> cc(sv.begin(), sv.end());
                    V.sync_ptrs();
                    if (!push_ritz(psi, V.dev(), k, cc, n, ws, st)) continue;
                    locked.push_back(theta);
                    // the newest Lanczos vector is also made orthogonal to it
                    const float2* p = psi[psi.size() - 1];
                    std::complex<double> cp = -dot_f32(p, vn, n, ws, st);
                    axpy_f32(cp, p, vn, n, st);
                    const double vnn = std::sqrt(nrm2sq_f32(vn, n, ws, st));
                    scal_f32(1.0 / vnn, vn, n, st);
                }
            }
        }
    }
    QKG_CUDA(cudaStreamSynchronize(st));
    out.t_loop = secs(t0, clk::now());
    out.n_ritz_locked = (int)psi.size();
    const auto t1 = clk::now();
    std::vector<double> s;
    out.energy_tridiag = tridiag_ground(alphas.data(), betas.data(), (int)alphas.size(), s);
    // Ritz vector from the FP32 basis, then FP64 Rayleigh quotient and residual.
    DBuf r32(n * sizeof(float2)), r64(n * sizeof(double2)), h64(n * sizeof(double2));
    QKG_CUDA(cudaMemsetAsync(r32.p, 0, n * sizeof(float2), st));
    std::vector<cd> cc(s.begin(), s.end());
    mcombine_f32(V.dev(), (int)s.size(), cc.data(), r32.as<float2>(), n, ws, st);
    f32_to_f64(r32.as<float2>(), r64.as<double2>(), n, st);
    const double nr = std::sqrt(nrm2sq_f64(r64.as<double2>(), n, ws, st));
    scal_f64(1.0 / nr, r64.as<double2>(), n, st);
    H.apply_f64(r64.as<double2>(), h64.as<double2>(), st);
    const double E = dot_f64(r64.as<double2>(), h64.as<double2>(), n, ws, st).real();
    axpy_f64(-E, r64.as<double2>(), h64.as<double2>(), n, st);
    out.residual = std::sqrt(nrm2sq_f64(h64.as<double2>(), n, ws, st));
    out.energy = E;
    out.t_refine = secs(t1, clk::now());
    if (o.want_vec) {
        cd* dst = o.evec_out;
        if (!dst) {
            out.evec.resize(n);
            dst = out.evec.data();
        }
        download_ref_f64(H, r64.as<double2>(), dst, tmp);
    }
    return out;
}

// ============================================================ continued fraction
CFOut cf_f64(Hamiltonian& H, const cd* phi0_ref, int n_iter) {
    CFOut out;
    const uint64_t n = H.dim();
    if (n == 0) return out;
    cudaStream_t st = H.stream();
    Workspace ws(ws_cap(2));
    DBuf a(n * sizeof(double2)), b(n * sizeof(double2)), w(n * sizeof(double2)), tmp;
    double2 *v = a.as<double2>(), *vp = b.as<double2>();
    upload_ref_f64(H, phi0_ref, v, tmp);
    const double np = std::sqrt(nrm2sq_f64(v, n, ws, st));
    if (np < 1e-15) return out;  // src/solvers/dynamics.cpp:26
    scal_f64(1.0 / np, v, n, st);
    out.norm = np;
    for (int it = 0; it < n_iter; ++it) {
        H.apply_f64(v, w.as<double2>(), st);
        const double alpha = dot_f64(v, w.as<double2>(), n, ws, st).real();
        out.alphas.push_back(alpha);
        const double b2 = lanczos_update_f64(w.as<double2>(), v, it > 0 ? vp : nullptr, alpha,
                                             it > 0 ? out.betas.back() : 0.0, n, ws, st);
        const double beta = std::sqrt(b2);
        if (beta < 1e-15) break;
        out.betas.push_back(beta);
        // rotate: vp <- v, v <- w / beta, w <- old vp buffer
        std::swap(vp, v);
        double2* wp = w.as<double2>();
        QKG_CUDA(cudaMemcpyAsync(v, wp, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        scal_f64(1.0 / beta, v, n, st);
    }
    QKG_CUDA(cudaStreamSynchronize(st));
    return out;
}

// Backward continued fraction at z = omega + E0 + i eta (dynamics.cpp:61-89).
double spectral(const double* alphas, const double* betas, size_t n, double norm, double omega, double E0, double eta) {
    if (n == 0) return 0.0;
    const cd z(omega + E0, eta);
    cd f = 0.0;
    for (int i = (int)n - 1; i >= 0; --i) {
        if (i == (int)n - 1) f = 1.0 / (z - alphas[i]);
        else f = 1.0 / (z - alphas[i] - betas[i] * betas[i] * f);
    }
    return -1.0 / M_PI * std::imag(norm * norm * f);
}

// ============================================================ FTLM
std::vector<FTLMTri> ftlm_tridiags_f64(Hamiltonian& H, int n_random, int n_steps, bool f32_stream) {
    std::vector<FTLMTri> out;
    const uint64_t n = H.dim();
    if (n == 0 || n_random <= 0) return out;
    cudaStream_t st = H.stream();
    Workspace ws(ws_cap(2));
    DBuf a(n * sizeof(double2)), b(n * sizeof(double2)), w(n * sizeof(double2)), tmp;
    NormalStream stream(f32_stream);  // mt19937(42), src/solvers/ftlm.cpp:133-134
    std::vector<cd> h(n);
    for (int r = 0; r < n_random; ++r) {
        stream.fill(n, h.data());
        double2 *v = a.as<double2>(), *vp = b.as<double2>();
        upload_ref_f64(H, h.data(), v, tmp);
        FTLMTri t;
        t.norm2 = nrm2sq_f64(v, n, ws, st);
        const double nr = std::sqrt(t.norm2);
        if (nr != 0.0) scal_f64(1.0 / nr, v, n, st);
        std::vector<double> al, be;
        for (int i = 0; i < n_steps; ++i) {
            H.apply_f64(v, w.as<double2>(), st);
            const double alpha = dot_f64(v, w.as<double2>(), n, ws, st).real();
            al.push_back(alpha);
            const double b2 = lanczos_update_f64(w.as<double2>(), v, i > 0 ? vp : nullptr, alpha, i > 0 ? be.back() : 0.0,
                                                 n, ws, st);
            const double beta = std::sqrt(b2);
            if (beta < 1e-15) break;
            be.push_back(beta);
            std::swap(vp, v);
            QKG_CUDA(cudaMemcpyAsync(v, w.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
            scal_f64(1.0 / beta, v, n, st);
        }
        std::vector<double> z;
        tridiag_eig(al.data(), be.data(), (int)al.size(), t.evals, {0}, z);
        t.w0.resize(t.evals.size());
        for (size_t j = 0; j < t.evals.size(); ++j) t.w0[j] = z[j] * z[j];
        out.push_back(std::move(t));
    }
    return out;
}

// Z, E, Cv at each beta (ftlm.cpp:151-167).  With `shifted`, weights use
// exp(-beta (e - e_min)) and log_zmax[b] = -beta e_min, so that Z = Zs e^{log_zmax}
// stays finite where exp(-beta e) overflows.
void ftlm_observables(const std::vector<FTLMTri>& tri, const double* betas, int nb, double* Zo, double* Eo, double* Co,
                      bool shifted, double* log_zmax) {
    double emin = std::numeric_limits<double>::infinity();
    for (const auto& t : tri) for (double e : t.evals) emin = std::min(emin, e);
    const int R = (int)tri.size();
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < nb; ++k) {
        const double beta = betas[k];
        const double sh = shifted ? emin : 0.0;
        double Z = 0, E = 0, E2 = 0;
        for (const auto& t : tri)
            for (size_t i = 0; i < t.evals.size(); ++i) {
                const double wgt = t.norm2 * t.w0[i] * std::exp(-beta * (t.evals[i] - sh));
                Z += wgt;
                E += t.evals[i] * wgt;
                E2 += t.evals[i] * t.evals[i] * wgt;
            }
        if (R > 0) { Z /= R; E /= R; E2 /= R; }
        Zo[k] = Z;
        Eo[k] = E / Z;
        Co[k] = beta * beta * (E2 / Z - (E / Z) * (E / Z));
        if (log_zmax) log_zmax[k] = shifted ? -beta * emin : 0.0;
    }
}

// ============================================================ Davidson
namespace {
// Vector operations of one storage precision.
template <class T2> struct DavOps;
template <> struct DavOps<double2> {
    static void apply(Hamiltonian& H, const double2* x, double2* y, cudaStream_t s) { H.apply_f64(x, y, s); }
    static void mdot(const double2* const* V, int k, const double2* w, uint64_t n, cd* o, Workspace& ws, cudaStream_t s) {
        mdot_f64(V, k, w, n, o, ws, s);
    }
    static void mcomb(const double2* const* V, int k, const cd* c, double2* w, uint64_t n, Workspace& ws, cudaStream_t s) {
        mcombine_f64(V, k, c, w, n, ws, s);
    }
    static void mmulti(const double2* const* V, int k, const cd* c, double2* const* W, int no, uint64_t n, bool acc,
                       Workspace& ws, cudaStream_t s) {
        mcombine_multi_f64(V, k, c, W, no, n, acc, ws, s);
    }
    static double nrm2sq(const double2* x, uint64_t n, Workspace& ws, cudaStream_t s) { return nrm2sq_f64(x, n, ws, s); }
    static void scal(double a, double2* x, uint64_t n, cudaStream_t s) { scal_f64(a, x, n, s); }
    static void precond(const double2* r, const double2* d, double l, double2* t, uint64_t n, cudaStream_t s) {
        davidson_precond_f64(r, d, l, t, n, s);
    }
    static void from64(const double2* x, double2* y, uint64_t n, cudaStream_t s) {
        QKG_CUDA(cudaMemcpyAsync(y, x, n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    }
    static void to64(const double2* x, double2* y, uint64_t n, cudaStream_t s) { from64(x, y, n, s); }
};
template <> struct DavOps<float2> {
    static void apply(Hamiltonian& H, const float2* x, float2* y, cudaStream_t s) { H.apply_f32(x, y, s); }
    static void mdot(const float2* const* V, int k, const float2* w, uint64_t n, cd* o, Workspace& ws, cudaStream_t s) {
        mdot_f32(V, k, w, n, o, ws, s);
    }
    static void mcomb(const float2* const* V, int k, const cd* c, float2* w, uint64_t n, Workspace& ws, cudaStream_t s) {
        mcombine_f32(V, k, c, w, n, ws, s);
    }
    static void mmulti(const float2* const* V, int k, const cd* c, float2* const* W, int no, uint64_t n, bool acc,
                       Workspace& ws, cudaStream_t s) {
        mcombine_multi_f32(V, k, c, W, no, n, acc, ws, s);
    }
    static double nrm2sq(const float2* x, uint64_t n, Workspace& ws, cudaStream_t s) { return nrm2sq_f32(x, n, ws, s); }
    static void scal(double a, float2* x, uint64_t n, cudaStream_t s) { scal_f32(a, x, n, s); }
    static void precond(const float2* r, const double2* d, double l, float2* t, uint64_t n, cudaStream_t s) {
        davidson_precond_f32(r, d, l, t, n, s);
    }
    static void mdot_multi(const float2* const* V, int k, float2* const* W, int nw, uint64_t n, cd* o, Workspace& ws,
                           cudaStream_t s) {
        mdot_multi_f32(V, k, W, nw, n, o, ws, s);
    }
    static void from64(const double2* x, float2* y, uint64_t n, cudaStream_t s) { f64_to_f32(x, y, n, s); }
    static void to64(const float2* x, double2* y, uint64_t n, cudaStream_t s) { f32_to_f64(x, y, n, s); }
};

inline void mdot_block(const float2* const* V, int k, float2* const* W, int nw, uint64_t n, cd* o, Workspace& ws,
                       cudaStream_t s) {
    mdot_multi_f32(V, k, W, nw, n, o, ws, s);
}
inline void mdot_block(const double2* const*, int, double2* const*, int, uint64_t, cd*, Workspace&, cudaStream_t) {
    QKG_REQUIRE(false, "block projection is used by the mixed form only");
}

// src/solvers/davidson.cpp:86-227 with the Krylov vectors stored in T2.
// Projections <V_i, HV_j> of vectors that did not change are kept from the
// previous iteration (the reference recomputes them; the values are the same
// dot products), the k residuals and the restart's Ritz vectors are formed in
// one pass over V and HV each.  MIXED (FP32 storage): SpMV in FP32, projections
// and norms by compensated reductions in FP64, corrections orthogonalised twice,
// and the final Ritz pairs refined in FP64 (Rayleigh quotient, residual).
template <class T2>
DavidsonOut davidson_impl(Hamiltonian& H, int n_eig, int max_sub, double tol, bool want_vecs, bool f32_stream,
                          int max_iter) {
    using Op = DavOps<T2>;
    constexpr bool MIXED = std::is_same<T2, float2>::value;
    DavidsonOut out;
    const uint64_t n = H.dim();
    if (n == 0) return out;
    cudaStream_t st = H.stream();
    const auto t_start = std::chrono::steady_clock::now();
    n_eig = (int)std::min<uint64_t>((uint64_t)n_eig, n);
    max_sub = std::max(max_sub, 2 * n_eig);
    QKG_REQUIRE(max_sub + n_eig <= 1024, "Davidson: subspace limited to 1024 vectors");
    // the Krylov space a mixed Lanczos left on the Hamiltonian is released
    // first: the Davidson vectors come from their own pool
    {
        const auto ws_lock = H.workspace_lock();
        H.release_workspace();
    }
    Workspace ws(ws_cap(4 * (max_sub + n_eig + 2)));  // block projections: 4 right-hand vectors
    DBuf diag(n * sizeof(double2)), tmp, d64(n * sizeof(double2));
    H.diagonal_f64(diag.as<double2>(), st);
    // Seeds: unit vectors at the n_eig smallest diagonal entries, in the order
    // std::sort leaves them (davidson.cpp:111-121); the diagonal is taken in the
    // reference's order so ties resolve as they do there.
    std::vector<cd> dref = H.diagonal_host_ref();
    if (f32_stream)  // the FP32 engine sorts its float diagonal
        for (auto& d : dref) d = cd((double)(float)d.real(), 0.0);
    std::vector<uint64_t> di(n);
    std::iota(di.begin(), di.end(), 0);
    if (n <= (1ull << 23)) {
        std::sort(di.begin(), di.end(), [&](uint64_t i, uint64_t j) { return dref[i].real() < dref[j].real(); });
    } else {
        std::partial_sort(di.begin(), di.begin() + n_eig, di.end(), [&](uint64_t i, uint64_t j) {
            return dref[i].real() < dref[j].real() || (dref[i].real() == dref[j].real() && i < j);
        });
    }
    std::vector<cd>().swap(dref);
    std::mt19937 rng(1234);
    std::uniform_real_distribution<double> dist(-1.0, 1.0);
    std::uniform_real_distribution<float> dist32(-1.0f, 1.0f);
    VecPool pool(n * sizeof(T2));  // declared before the lists, so it outlives them
    VecList<T2> V(n, &pool), HV(n, &pool);
    std::vector<cd> hv(n), c;
    const int passes = MIXED ? 2 : 1;
    // t -= V[from..] (V[from..]^H t), passes times, and ||t||
    auto orthonormalize = [&](T2* t, size_t from) -> double {
        const int kv = (int)(V.size() - std::min(from, V.size()));
        for (int p = 0; p < passes && kv; ++p) {
            c.assign(kv, 0.0);
            Op::mdot(V.dev() + from, kv, t, n, c.data(), ws, st);
            for (auto& x : c) x = -x;
            Op::mcomb(V.dev() + from, kv, c.data(), t, n, ws, st);
        }
        return std::sqrt(Op::nrm2sq(t, n, ws, st));
    };
    DBuf seed(n * sizeof(T2));
    for (int i = 0; i < n_eig; ++i) {
        std::fill(hv.begin(), hv.end(), cd(0.0));
        hv[di[i]] = 1.0;
        upload_ref_f64(H, hv.data(), d64.as<double2>(), tmp);
        Op::from64(d64.as<double2>(), seed.as<T2>(), n, st);
        double nrm = orthonormalize(seed.as<T2>(), 0);
        if (nrm < 1e-10) {
            if (f32_stream) fill_stream(rng, dist32, n, hv.data());
            else fill_stream(rng, dist, n, hv.data());
            upload_ref_f64(H, hv.data(), d64.as<double2>(), tmp);
            Op::from64(d64.as<double2>(), seed.as<T2>(), n, st);
            nrm = orthonormalize(seed.as<T2>(), 0);
        }
        T2* v = V.push();
        QKG_CUDA(cudaMemcpyAsync(v, seed.p, n * sizeof(T2), cudaMemcpyDeviceToDevice, st));
        Op::scal(1.0 / nrm, v, n, st);
        Op::apply(H, v, HV.push(), st);
    }
    std::vector<cd>().swap(hv);
    // cached projected matrix: rows[i][j] = <V_i, HV_j> for j <= i < m_cached
    std::vector<std::vector<cd>> rows;
    std::vector<DBuf> rbuf(n_eig);
    for (auto& r : rbuf) r.alloc(n * sizeof(T2));
    std::vector<T2*> rptr;
    for (auto& r : rbuf) rptr.push_back(r.as<T2>());
    for (int iter = 0; iter < max_iter; ++iter) {
        const int m = (int)V.size();
        if (MIXED && m - (int)rows.size() > 1) {
            // the new rows together: one pass over HV_0..HV_{m-1} for up to four new V_i
            for (int i0 = (int)rows.size(); i0 < m; i0 += 4) {
                const int nw = std::min(4, m - i0);
                std::vector<T2*> wp;
                for (int o = 0; o < nw; ++o) wp.push_back(V[i0 + o]);
                std::vector<cd> cc((size_t)nw * m);
                mdot_block(HV.dev(), m, wp.data(), nw, n, cc.data(), ws, st);  // <HV_j, V_{i0+o}>
                for (int o = 0; o < nw; ++o) {
                    std::vector<cd> col(i0 + o + 1);
                    for (int j = 0; j <= i0 + o; ++j) col[j] = std::conj(cc[(size_t)o * m + j]);
                    rows.push_back(std::move(col));
                }
            }
        }
        for (int i = (int)rows.size(); i < m; ++i) {
            std::vector<cd> col(i + 1);
            Op::mdot(HV.dev(), i + 1, V[i], n, col.data(), ws, st);  // <HV_j, V_i>
            for (auto& x : col) x = std::conj(x);
            rows.push_back(std::move(col));
        }
        std::vector<cd> Hs((size_t)m * m);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j <= i; ++j) {
                Hs[(size_t)i * m + j] = rows[i][j];
                if (i != j) Hs[(size_t)j * m + i] = std::conj(rows[i][j]);
            }
        std::vector<double> ev;
        std::vector<std::vector<cd>> evec;
        hermitian_eig(Hs, m, ev, evec);
        // residuals r_k = HV s_k - lambda_k V s_k for all k (one pass over HV, one over V)
        const int kc = std::max(1, std::min(8, 1024 / std::max(m, 1)));  // outputs per pass
        for (int k0 = 0; k0 < n_eig; k0 += kc) {
            const int nk = std::min(kc, n_eig - k0);
            std::vector<cd> cs((size_t)nk * m), cl((size_t)nk * m);
            for (int k = 0; k < nk; ++k)
                for (int i = 0; i < m; ++i) {
                    cs[(size_t)k * m + i] = evec[k0 + k][i];
                    cl[(size_t)k * m + i] = -ev[k0 + k] * evec[k0 + k][i];
                }
            Op::mmulti(HV.dev(), m, cs.data(), rptr.data() + k0, nk, n, false, ws, st);
            Op::mmulti(V.dev(), m, cl.data(), rptr.data() + k0, nk, n, true, ws, st);
        }
        bool all_conv = true;
        std::vector<DBuf> corr;
        out.residuals.assign(n_eig, 0.0);
        for (int k = 0; k < n_eig; ++k) {
            const double rn = std::sqrt(Op::nrm2sq(rptr[k], n, ws, st));
            out.residuals[k] = rn;
            if (rn > tol) {
                all_conv = false;
                DBuf t = pool.get(V.size() + HV.size());
                Op::precond(rptr[k], diag.as<double2>(), ev[k], t.as<T2>(), n, st);
                corr.push_back(std::move(t));
            }
        }
        if (all_conv || iter == max_iter - 1) {
            out.iters = iter + 1;
            out.converged = all_conv;
            out.evals.assign(ev.begin(), ev.begin() + n_eig);
            // Ritz vectors (into the residual buffers)
            std::vector<cd> cs((size_t)n_eig * m);
            for (int k = 0; k < n_eig; ++k)
                for (int i = 0; i < m; ++i) cs[(size_t)k * m + i] = evec[k][i];
            for (int k0 = 0; k0 < n_eig; k0 += kc)
                Op::mmulti(V.dev(), m, cs.data() + (size_t)k0 * m, rptr.data() + k0, std::min(kc, n_eig - k0), n, false,
                           ws, st);
            DBuf e64, h64;
            if (MIXED) {
                // FP64 refinement: Rayleigh quotient and residual of each normalised Ritz vector
                V.clear();
                HV.clear();
                pool.free.clear();  // give the basis memory back before the FP64 vectors
                e64.alloc(n * sizeof(double2));
                h64.alloc(n * sizeof(double2));
                bool conv64 = true;
                for (int k = 0; k < n_eig; ++k) {
                    Op::to64(rptr[k], e64.as<double2>(), n, st);
                    const double nr = std::sqrt(nrm2sq_f64(e64.as<double2>(), n, ws, st));
                    if (nr > 0.0) scal_f64(1.0 / nr, e64.as<double2>(), n, st);
                    H.apply_f64(e64.as<double2>(), h64.as<double2>(), st);
                    const double lam = dot_f64(e64.as<double2>(), h64.as<double2>(), n, ws, st).real();
                    axpy_f64(cd(-lam, 0.0), e64.as<double2>(), h64.as<double2>(), n, st);
                    out.residuals[k] = std::sqrt(nrm2sq_f64(h64.as<double2>(), n, ws, st));
                    out.evals[k] = lam;
                    if (out.residuals[k] > tol) conv64 = false;
                    if (want_vecs) {
                        std::vector<cd> h(n);
                        download_ref_f64(H, e64.as<double2>(), h.data(), tmp);
                        out.evecs.push_back(std::move(h));
                    }
                }
                out.converged = conv64;
            } else if (want_vecs) {
                for (int k = 0; k < n_eig; ++k) {
                    std::vector<cd> h(n);
                    download_ref_f64(H, reinterpret_cast<const double2*>(rptr[k]), h.data(), tmp);
                    out.evecs.push_back(std::move(h));
                }
            }
            QKG_CUDA(cudaStreamSynchronize(st));
            out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
            return out;
        }
        if (V.size() + corr.size() > (size_t)max_sub) {  // restart to the Ritz vectors (:196-211)
            std::vector<DBuf> nv, nh;
            std::vector<T2*> pv, ph;
            for (int k = 0; k < n_eig; ++k) {
                nv.push_back(pool.get(V.size() + HV.size()));
                nh.push_back(pool.get(V.size() + HV.size()));
                pv.push_back(nv.back().as<T2>());
                ph.push_back(nh.back().as<T2>());
            }
            std::vector<cd> cs((size_t)n_eig * m);
            for (int k = 0; k < n_eig; ++k)
                for (int i = 0; i < m; ++i) cs[(size_t)k * m + i] = evec[k][i];
            for (int k0 = 0; k0 < n_eig; k0 += kc) {
                const int nk = std::min(kc, n_eig - k0);
                Op::mmulti(V.dev(), m, cs.data() + (size_t)k0 * m, pv.data() + k0, nk, n, false, ws, st);
                Op::mmulti(HV.dev(), m, cs.data() + (size_t)k0 * m, ph.data() + k0, nk, n, false, ws, st);
            }
            V.take(nv);
            HV.take(nh);
            rows.clear();
        }
        // Orthogonalise each correction and extend (:213-223).  Mixed form: all
        // corrections are first projected off the current basis together (one
        // pass over V per Gram-Schmidt pass for all of them), then each off the
        // corrections accepted before it; in exact arithmetic the same as the
        // sequential projection off the growing basis.
        size_t from = 0;
        if (MIXED && corr.size() > 1 && V.size()) {
            const int kv = (int)V.size(), nc = (int)corr.size();
            std::vector<T2*> tp;
            for (auto& t : corr) tp.push_back(t.as<T2>());
            const int wmax = std::max(1, std::min(4, 1024 / kv));  // coefficient table limit of mmulti
            for (int c0 = 0; c0 < nc; c0 += wmax) {
                const int nw = std::min(wmax, nc - c0);
                std::vector<cd> cc((size_t)nw * kv);
                for (int p = 0; p < passes; ++p) {
                    mdot_block(V.dev(), kv, tp.data() + c0, nw, n, cc.data(), ws, st);
                    for (auto& x : cc) x = -x;
                    Op::mmulti(V.dev(), kv, cc.data(), tp.data() + c0, nw, n, true, ws, st);
                }
            }
            from = V.size();
        }
        for (auto& t : corr) {
            const double nrm = orthonormalize(t.as<T2>(), from);
            if (nrm > 1e-10) {
                Op::scal(1.0 / nrm, t.as<T2>(), n, st);
                T2* v = V.adopt(std::move(t));
                Op::apply(H, v, HV.push(), st);
            }
        }
        for (auto& t : corr) pool.put(std::move(t));  // the rejected ones
    }
    return out;
}
}  // namespace

DavidsonOut davidson_f64(Hamiltonian& H, int n_eig, int max_sub, double tol, bool want_vecs, bool f32_stream,
                         int max_iter) {
    return davidson_impl<double2>(H, n_eig, max_sub, tol, want_vecs, f32_stream, max_iter);
}
DavidsonOut davidson_mixed(Hamiltonian& H, int n_eig, int max_sub, double tol, bool want_vecs, int max_iter) {
    return davidson_impl<float2>(H, n_eig, max_sub, tol, want_vecs, false, max_iter);
}

}  // namespace qkg
