// Oracle restatement of qkrylov's hot path: CPU, FP64, test infrastructure
// only (see qko.h).  Every routine names the reference file:line it restates;
// paths are relative to the qkrylov source tree.
//
// Deliberate representation choices (behaviour is the reference's):
//  * the basis is a sorted std::vector<uint64_t> with binary-search lookup
//    instead of the reference's std::unordered_map; ascending order and the
//    state -> position mapping are identical (src/basis/*.cpp);
//  * Hubbard/t-J bases are generated from their constrained up/dn parts and
//    sorted, instead of scanning all 4^N integers; the resulting set and order
//    are those of src/basis/hubbard_basis.cpp:72-100 and tj_basis.cpp:161-201.
#include "qko.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using cd = std::complex<double>;
std::string g_err;

inline int popc(uint64_t x) { return __builtin_popcountll(x); }

struct LocalAction {  // include/qkrylov/operators/local_action.hpp:9-16
    bool valid = false;
    uint64_t new_state = 0;
    cd element = 0.0;
};

inline double jw(uint64_t state, int bit) {  // fermion_site.cpp:143-154, hubbard_site.cpp:31-49
    const uint64_t mask = (1ULL << bit) - 1;
    return (popc(state & mask) % 2 == 0) ? 1.0 : -1.0;
}

// Site actions, one per model.  The operator name is looked up once per
// factor (op_id); an unknown name gets id -1 and throws when first applied,
// which is when the reference's site.apply throws (its CSR build applies the
// factors of a term in order and stops at the first invalid one).
enum : int { OP_SZ, OP_SP, OP_SM, OP_SX, OP_SY, OP_N, OP_ID, OP_C, OP_CDAG, OP_NUP, OP_NDN, OP_NUPDN, OP_CUP,
             OP_CDAGUP, OP_CDN, OP_CDAGDN };
int op_id(int model, const std::string& op) {
    if (model == 0) {  // src/sites/spinhalf_site.cpp:18-121
        if (op == "Sz") return OP_SZ;
        if (op == "Sp") return OP_SP;
        if (op == "Sm") return OP_SM;
        if (op == "Sx") return OP_SX;
        if (op == "Sy") return OP_SY;
        return -1;
    }
    if (model == 1) {  // src/sites/fermion_site.cpp:19-84
        if (op == "N") return OP_N;
        if (op == "Id") return OP_ID;
        if (op == "C") return OP_C;
        if (op == "Cdag") return OP_CDAG;
        return -1;
    }
    if (op == "Nup") return OP_NUP;
    if (op == "Ndn") return OP_NDN;
    if (model != 3 && op == "Nupdn") return OP_NUPDN;
    if (op == "CUp") return OP_CUP;
    if (op == "CdagUp") return OP_CDAGUP;
    if (op == "CDn") return OP_CDN;
    if (op == "CdagDn") return OP_CDAGDN;
    return -1;
}
[[noreturn]] void unknown_op(int model, const std::string& op) {
    if (model == 0) throw std::runtime_error("Unknown spin operator: " + op);
    if (model == 1) throw std::runtime_error("Unknown fermion operator: " + op);
    throw std::runtime_error(std::string(model == 3 ? "Unknown TJ operator: " : "Unknown Hubbard operator: ") + op);
}
LocalAction site_apply_id(int model, int id, const std::string& op, int site, uint64_t state) {
    LocalAction a;
    if (id < 0) unknown_op(model, op);
    if (model == 0) {  // src/sites/spinhalf_site.cpp:18-121
        const bool up = (state >> site) & 1ULL;
        switch (id) {
            case OP_SZ: a.valid = true; a.new_state = state; a.element = up ? 0.5 : -0.5; return a;
            case OP_SP: if (up) return a; a.valid = true; a.new_state = state | (1ULL << site); a.element = 1.0; return a;
            case OP_SM: if (!up) return a; a.valid = true; a.new_state = state & ~(1ULL << site); a.element = 1.0; return a;
            case OP_SX: a.valid = true; a.new_state = state ^ (1ULL << site); a.element = 0.5; return a;
            default:  // OP_SY
                a.valid = true; a.new_state = state ^ (1ULL << site);
                a.element = up ? cd(0.0, -0.5) : cd(0.0, 0.5);
                return a;
        }
    }
    if (model == 1) {  // src/sites/fermion_site.cpp:19-84
        const bool occ = (state >> site) & 1ULL;
        switch (id) {
            case OP_N: a.valid = true; a.new_state = state; a.element = occ ? 1.0 : 0.0; return a;
            case OP_ID: a.valid = true; a.new_state = state; a.element = 1.0; return a;
            case OP_C: if (!occ) return a; a.valid = true; a.new_state = state & ~(1ULL << site); a.element = jw(state, site); return a;
            default:  // OP_CDAG
                if (occ) return a; a.valid = true; a.new_state = state | (1ULL << site); a.element = jw(state, site); return a;
        }
    }
    // Hubbard (src/sites/hubbard_site.cpp:51-125) and t-J (src/sites/tj_site.cpp:176-242):
    // up electron of site i at bit 2i, down electron at bit 2i+1.
    const int bu = 2 * site, bd = 2 * site + 1;
    const bool up = (state >> bu) & 1ULL, dn = (state >> bd) & 1ULL;
    const bool tj = (model == 3);
    switch (id) {
        case OP_NUP: a.valid = true; a.new_state = state; a.element = up ? 1.0 : 0.0; return a;
        case OP_NDN: a.valid = true; a.new_state = state; a.element = dn ? 1.0 : 0.0; return a;
        case OP_NUPDN: a.valid = true; a.new_state = state; a.element = (up && dn) ? 1.0 : 0.0; return a;
        case OP_CUP: if (!up) return a; a.valid = true; a.new_state = state & ~(1ULL << bu); a.element = jw(state, bu); return a;
        case OP_CDAGUP:
            if (up || (tj && dn)) return a;  // t-J forbids double occupancy (tj_site.cpp:214)
            a.valid = true; a.new_state = state | (1ULL << bu); a.element = jw(state, bu); return a;
        case OP_CDN: if (!dn) return a; a.valid = true; a.new_state = state & ~(1ULL << bd); a.element = jw(state, bd); return a;
        default:  // OP_CDAGDN
            if (dn || (tj && up)) return a;  // tj_site.cpp:232
            a.valid = true; a.new_state = state | (1ULL << bd); a.element = jw(state, bd); return a;
    }
}
LocalAction site_apply(int model, const std::string& op, int site, uint64_t state) {
    return site_apply_id(model, op_id(model, op), op, site, state);
}

struct Sector { bool use_sz = false; int sz2 = 0; bool use_nup = false, use_ndn = false; int nup = 0, ndn = 0; bool use_n = false; int n = 0; };

std::vector<uint64_t> fixed_pop(int nbits, int k) {  // all nbits-bit strings with popcount k, ascending
    std::vector<uint64_t> out;
    if (k < 0 || k > nbits) return out;
    if (k == 0) { out.push_back(0); return out; }
    uint64_t v = (k == 64) ? ~0ULL : ((1ULL << k) - 1);
    const uint64_t lim = (nbits == 64) ? 0 : (1ULL << nbits);
    while (true) {
        out.push_back(v);
        const uint64_t t = v | (v - 1);  // next permutation of bits (Gosper)
        const uint64_t w = (t + 1) | (((~t & -~t) - 1) >> (__builtin_ctzll(v) + 1));
        if (w >= lim || w <= v) break;
        v = w;
    }
    return out;
}

inline uint64_t interleave(uint64_t up, uint64_t dn, int N) {
    uint64_t s = 0;
    for (int i = 0; i < N; ++i) s |= (((up >> i) & 1ULL) << (2 * i)) | (((dn >> i) & 1ULL) << (2 * i + 1));
    return s;
}

struct Basis {
    int model = 0, N = 0;
    std::vector<uint64_t> states;
    int fixed_k = -1;  // spin/fermion sector of fixed popcount: states are all N-bit strings with k ones
    uint64_t size() const { return states.size(); }
    int64_t index(uint64_t s) const {
        auto it = std::lower_bound(states.begin(), states.end(), s);
        if (it == states.end() || *it != s) return -1;
        return it - states.begin();
    }
    // index() by the colex rank where the basis is a fixed-popcount class (the
    // ascending order of such a class is its colex order), else index().
    int64_t index_fast(uint64_t s) const;
};

uint64_t binom64(int n, int k) {
    static const std::vector<uint64_t> tab = [] {
        std::vector<uint64_t> t(65 * 65, 0);
        for (int a = 0; a <= 64; ++a) {
            t[a * 65] = 1;
            for (int b = 1; b <= a; ++b) t[a * 65 + b] = t[(a - 1) * 65 + b - 1] + (b <= a - 1 ? t[(a - 1) * 65 + b] : 0);
        }
        return t;
    }();
    return (k < 0 || k > n) ? 0 : tab[n * 65 + k];
}

int64_t Basis::index_fast(uint64_t s) const {
    if (fixed_k < 0) return index(s);
    if (popc(s) != fixed_k || (N < 64 && (s >> N) != 0)) return -1;
    uint64_t r = 0;
    int i = 0;
    for (uint64_t t = s; t; t &= t - 1) r += binom64(__builtin_ctzll(t), ++i);
    return (int64_t)r;
}

// src/basis/spinhalf_basis.cpp:12-30,59-104; fermion_basis.cpp:12-89;
// hubbard_basis.cpp:12-100; tj_basis.cpp:12-96.
Basis build_basis(int model, int N, const Sector& sec) {
    Basis b; b.model = model; b.N = N;
    if (model == 0 || model == 1) {
        if (N <= 0 || N > 63) throw std::runtime_error("basis: N must satisfy 1 <= N <= 63");
        const bool constrained = (model == 0) ? sec.use_sz : sec.use_n;
        if (!constrained) {
            const uint64_t dim = 1ULL << N;
            b.states.resize(dim);
            for (uint64_t s = 0; s < dim; ++s) b.states[s] = s;
        } else if (model == 0) {
            // 2*popcount - N == sz2  (spinhalf_basis.cpp:72-84)
            if ((sec.sz2 + N) % 2 == 0) { b.states = fixed_pop(N, (sec.sz2 + N) / 2); b.fixed_k = (sec.sz2 + N) / 2; }
        } else {
            b.states = fixed_pop(N, sec.n);
            b.fixed_k = sec.n;
        }
        if (b.states.empty()) b.fixed_k = -1;
        return b;
    }
    if (N <= 0 || N > 31) throw std::runtime_error("basis: N must satisfy 1 <= N <= 31");
    std::vector<uint64_t> ups, dns;
    const bool cu = sec.use_nup, cdn = sec.use_ndn;
    // The Hubbard basis filters only when a particle number is set
    // (hubbard_basis.cpp:26-29); t-J always filters double occupancy.
    auto all = [&](int n) { std::vector<uint64_t> v(1ULL << n); for (uint64_t i = 0; i < v.size(); ++i) v[i] = i; return v; };
    ups = cu ? fixed_pop(N, sec.nup) : all(N);
    dns = cdn ? fixed_pop(N, sec.ndn) : all(N);
    for (uint64_t u : ups)
        for (uint64_t d : dns) {
            if (model == 3 && (u & d)) continue;  // no double occupancy (tj_basis.cpp:169-180)
            b.states.push_back(interleave(u, d, N));
        }
    std::sort(b.states.begin(), b.states.end());
    return b;
}

struct Factor { std::string op; int site; int id = -1; };
struct Term { cd coeff; std::vector<Factor> factors; };

struct Ham {
    Basis basis;
    std::vector<Term> terms;
    std::vector<int32_t> rows;   // int32 like the reference (matrix_free_hamiltonian.cpp:36-37)
    std::vector<int32_t> cols;
    std::vector<cd> vals;
    std::vector<cd> diag;
    uint64_t row0 = 0, nrows = 0;
};

// matrix_free_hamiltonian.cpp:45-92: per row alpha, per term, apply the
// factors in order; keep (beta, conj(amp)) when valid and in the basis;
// accumulate the diagonal from entries with beta == alpha.
void build_csr(Ham& h, uint64_t row0, uint64_t nrows) {
    h.row0 = row0; h.nrows = nrows;
    h.rows.assign(nrows + 1, 0);
    h.diag.assign(nrows, cd(0.0, 0.0));
    for (uint64_t r = 0; r < nrows; ++r) {
        const uint64_t alpha = row0 + r;
        h.rows[r] = (int32_t)h.cols.size();
        const uint64_t s0 = h.basis.states[alpha];
        for (const auto& t : h.terms) {
            uint64_t s = s0; cd amp = t.coeff; bool valid = true;
            for (const auto& f : t.factors) {
                auto a = site_apply_id(h.basis.model, f.id, f.op, f.site, s);
                if (!a.valid) { valid = false; break; }
                s = a.new_state; amp *= a.element;
            }
            if (!valid) continue;
            const int64_t beta = h.basis.index(s);
            if (beta < 0) continue;
            const cd val(amp.real(), -amp.imag());
            h.cols.push_back((int32_t)beta);
            h.vals.push_back(val);
            if ((uint64_t)beta == alpha) h.diag[r] += val;
        }
    }
    h.rows[nrows] = (int32_t)h.cols.size();
}

// The same CSR as build_csr(h, 0, dim) (same rows, entries in the same order),
// built by all host threads in two passes (count, then fill) with the colex
// rank where the basis allows it.  Used where the reference's single-threaded
// assembly would take minutes (the CPU baseline at full size); the CSR build is
// not part of the timed work.
void build_csr_parallel(Ham& h) {
    const uint64_t n = h.basis.size();
    h.row0 = 0; h.nrows = n;
    h.rows.assign(n + 1, 0);
    h.diag.assign(n, cd(0.0, 0.0));
    std::vector<int32_t> cnt(n, 0);
    auto row_entries = [&](uint64_t alpha, auto&& emit) {
        const uint64_t s0 = h.basis.states[alpha];
        for (const auto& t : h.terms) {
            uint64_t s = s0; cd amp = t.coeff; bool valid = true;
            for (const auto& f : t.factors) {
                auto a = site_apply_id(h.basis.model, f.id, f.op, f.site, s);
                if (!a.valid) { valid = false; break; }
                s = a.new_state; amp *= a.element;
            }
            if (!valid) continue;
            const int64_t beta = h.basis.index_fast(s);
            if (beta < 0) continue;
            emit(beta, cd(amp.real(), -amp.imag()));
        }
    };
    std::string err;
#pragma omp parallel for schedule(dynamic, 4096)
    for (long long r = 0; r < (long long)n; ++r) {
        try {
            int32_t c = 0;
            row_entries((uint64_t)r, [&](int64_t, cd) { ++c; });
            cnt[r] = c;
        } catch (const std::exception& e) {
#pragma omp critical
            err = e.what();
        }
    }
    if (!err.empty()) throw std::runtime_error(err);
    uint64_t total = 0;
    for (uint64_t r = 0; r < n; ++r) {
        h.rows[r] = (int32_t)total;
        total += (uint64_t)cnt[r];
        if (total > 0x7fffffffULL) throw std::runtime_error("CSR: more than 2^31-1 entries (int32 offsets)");
    }
    h.rows[n] = (int32_t)total;
    std::vector<int32_t>().swap(cnt);
    h.cols.resize(total);
    h.vals.resize(total);
#pragma omp parallel for schedule(dynamic, 4096)
    for (long long r = 0; r < (long long)n; ++r) {
        int64_t k = h.rows[r];
        row_entries((uint64_t)r, [&](int64_t beta, cd val) {
            h.cols[k] = (int32_t)beta;
            h.vals[k] = val;
            ++k;
            if (beta == r) h.diag[r] += val;
        });
    }
}

// ---- vector algebra: include/qkrylov/linalg/vector_ops.hpp:14-137 --------------
// Reductions use static blocks per thread summed in thread order, the same
// scheme as the oracle's Kokkos stand-in (deterministic per thread count).
using Vec = std::vector<cd>;

cd dot(const Vec& x, const Vec& y) {
    const long long n = (long long)x.size();
#ifdef _OPENMP
    const int nt = omp_get_max_threads();
#else
    const int nt = 1;
#endif
    std::vector<cd> part(nt, cd(0.0, 0.0));
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        const int t = omp_get_thread_num();
#else
        const int t = 0;
#endif
        cd local(0.0, 0.0);
#pragma omp for schedule(static)
        for (long long i = 0; i < n; ++i) local += std::conj(x[i]) * y[i];
        part[t] = local;
    }
    cd acc(0.0, 0.0);
    for (int t = 0; t < nt; ++t) acc += part[t];
    return acc;
}
double norm(const Vec& x) { return std::sqrt(dot(x, x).real()); }
void scal(cd a, Vec& x) {
    const long long n = (long long)x.size();
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) x[i] *= a;
}
void axpy(cd a, const Vec& x, Vec& y) {
    const long long n = (long long)x.size();
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) y[i] += a * x[i];
}
void normalize(Vec& x) { const double n = norm(x); if (n == 0.0) return; scal(cd(1.0 / n, 0.0), x); }

// matrix_free_hamiltonian.cpp:141-168: y[alpha] = sum_j vals[j] * x[cols[j]].
void apply(const Ham& h, const cd* x, cd* y) {
    const long long n = (long long)h.nrows;
#pragma omp parallel for schedule(static)
    for (long long r = 0; r < n; ++r) {
        cd sum(0.0, 0.0);
        for (int32_t j = h.rows[r]; j < h.rows[r + 1]; ++j) sum += h.vals[j] * x[h.cols[j]];
        y[r] = sum;
    }
}
void apply(const Ham& h, const Vec& x, Vec& y) { apply(h, x.data(), y.data()); }

// ---- tridiagonal eigensolvers ---------------------------------------------------
// Implicit-shift QL as written in src/solvers/lanczos.cpp:25-98 (ground state +
// eigenvector) and src/solvers/ftlm.cpp:61-119 (all eigenvalues + first
// components); both accumulate the full rotation matrix z.
void tridiag_ql(std::vector<double>& d, std::vector<double>& e, std::vector<std::vector<double>>& z, int n) {
    for (int i = 0; i < n; ++i) { z[i].assign(n, 0.0); z[i][i] = 1.0; }
    for (int iter = 0; iter < 1000; ++iter) {
        for (int i = 0; i < n - 1; ++i)
            if (std::abs(e[i]) < 1e-14 * (std::abs(d[i]) + std::abs(d[i + 1]))) e[i] = 0.0;
        int m = n - 1;
        while (m > 0 && e[m - 1] == 0.0) m--;
        if (m == 0) break;
        int l = m - 1;
        while (l > 0 && e[l - 1] != 0.0) l--;
        const double b = (d[m - 1] - d[m]) / 2.0;
        const double c = e[m - 1] * e[m - 1];
        const double s = std::sqrt(b * b + c);
        const double shift = (b > 0) ? d[m] - c / (b + s) : d[m] - c / (b - s);
        double p = d[l] - shift;
        double g = e[l];
        for (int i = l; i < m; ++i) {
            const double r = std::hypot(p, g);
            const double ct = p / r, st = g / r;
            if (i > l) e[i - 1] = r;
            const double f = ct * d[i] + st * e[i];
            const double gn = ct * e[i] + st * d[i + 1];
            const double hh = st * d[i] - ct * e[i];
            const double k = st * e[i] - ct * d[i + 1];
            d[i] = ct * f + st * gn;
            e[i] = ct * hh + st * k;
            d[i + 1] = st * hh - ct * k;
            for (int j = 0; j < n; ++j) {
                const double z1 = z[j][i], z2 = z[j][i + 1];
                z[j][i] = ct * z1 + st * z2;
                z[j][i + 1] = st * z1 - ct * z2;
            }
            if (i < m - 1) { p = e[i]; g = st * e[i + 1]; e[i + 1] = -ct * e[i + 1]; }
        }
    }
}

double tridiag_ground(const std::vector<double>& a, const std::vector<double>& b, int n, std::vector<double>& vec) {
    if (n == 0) { vec.clear(); return 0.0; }
    if (n == 1) { vec.assign(1, 1.0); return a[0]; }
    std::vector<double> d(a.begin(), a.begin() + n), e(b.begin(), b.end());
    e.resize(std::max<size_t>(e.size(), (size_t)n), 0.0);
    std::vector<std::vector<double>> z(n);
    tridiag_ql(d, e, z, n);
    int mi = 0;
    for (int i = 1; i < n; ++i) if (d[i] < d[mi]) mi = i;
    vec.resize(n);
    for (int i = 0; i < n; ++i) vec[i] = z[i][mi];
    return d[mi];
}

void tridiag_components(const std::vector<double>& a, const std::vector<double>& b, std::vector<double>& ev, std::vector<double>& first) {
    const int n = (int)a.size();
    ev.clear(); first.clear();
    if (n == 0) return;
    if (n == 1) { ev.push_back(a[0]); first.push_back(1.0); return; }
    std::vector<double> d = a, e = b;
    e.resize(std::max<size_t>(e.size(), (size_t)n), 0.0);
    std::vector<std::vector<double>> z(n);
    tridiag_ql(d, e, z, n);
    for (int i = 0; i < n; ++i) { ev.push_back(d[i]); first.push_back(z[0][i]); }
}

// ---- reference random streams ---------------------------------------------------
// The reference fills KComplex(dist(rng), dist(rng)); g++ evaluates the two
// constructor arguments right to left, so the first draw is the imaginary
// part (src/solvers/lanczos.cpp:119, ftlm.cpp:143, davidson.cpp:128).
template <class Dist>
void fill_complex(std::mt19937& rng, Dist& dist, uint64_t n, cd* out) {
    for (uint64_t i = 0; i < n; ++i) { const double im = dist(rng); const double re = dist(rng); out[i] = cd(re, im); }
}

// ---- Lanczos: src/solvers/lanczos.cpp:101-202 -------------------------------------
struct LanczosOut { double energy = 0; int iters = 0; bool conv = false; Vec evec; std::vector<double> alphas, betas; };

LanczosOut lanczos(const Ham& H, Vec v_curr, int maxiter, double tol, std::vector<double>* step_s = nullptr) {
    LanczosOut out;
    const uint64_t dim = H.basis.size();
    if (dim == 0) return out;
    Vec v_prev(dim), w(dim);
    normalize(v_curr);
    std::vector<Vec> V;
    V.push_back(v_curr);
    std::vector<double>& alphas = out.alphas;
    std::vector<double>& betas = out.betas;
    bool conv = false; double e_old = 1e100; int iters = 0;
    const int nmax = std::min<int>(maxiter, (int)dim);
    auto t_step = std::chrono::steady_clock::now();
    auto lap = [&] {
        if (!step_s) return;
        const auto now = std::chrono::steady_clock::now();
        step_s->push_back(std::chrono::duration<double>(now - t_step).count());
        t_step = now;
    };
    for (int iter = 0; iter < nmax; ++iter) {
        iters = iter + 1;
        t_step = std::chrono::steady_clock::now();
        apply(H, v_curr, w);
        const double alpha = dot(v_curr, w).real();
        alphas.push_back(alpha);
        axpy(cd(-alpha, 0.0), v_curr, w);
        if (iter > 0) axpy(cd(-betas.back(), 0.0), v_prev, w);
        for (const auto& bv : V) axpy(-dot(bv, w), bv, w);  // full reorthogonalisation (:148-151)
        const double beta = norm(w);
        if (beta < 1e-15) { conv = true; lap(); break; }
        if (iter + 1 == nmax) { lap(); break; }
        betas.push_back(beta);
        v_prev = v_curr;
        v_curr = w;
        scal(cd(1.0 / beta, 0.0), v_curr);
        V.push_back(v_curr);
        if (iter > 0) {
            std::vector<double> tv;
            const double e = tridiag_ground(alphas, betas, (int)alphas.size(), tv);
            if (std::abs(e - e_old) < tol) { e_old = e; conv = true; lap(); break; }
            e_old = e;
        }
        lap();
    }
    std::vector<double> ev;
    out.energy = tridiag_ground(alphas, betas, (int)alphas.size(), ev);
    out.iters = iters; out.conv = conv;
    Vec ritz(dim);
    for (size_t i = 0; i < alphas.size(); ++i) axpy(cd(ev[i], 0.0), V[i], ritz);
    normalize(ritz);
    out.evec = std::move(ritz);
    return out;
}

// ---- Davidson: src/solvers/davidson.cpp:22-227 ------------------------------------
struct SmallEig { std::vector<double> vals; std::vector<std::vector<cd>> vecs; };

SmallEig small_hermitian(const std::vector<std::vector<cd>>& Hm) {  // :22-82 (complex Jacobi)
    const int n = (int)Hm.size();
    auto A = Hm;
    std::vector<std::vector<cd>> V(n, std::vector<cd>(n, 0.0));
    for (int i = 0; i < n; ++i) V[i][i] = 1.0;
    for (int iter = 0; iter < 1000; ++iter) {
        double max_off = 0.0; int p = 0, q = 0;
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j)
                if (std::abs(A[i][j]) > max_off) { max_off = std::abs(A[i][j]); p = i; q = j; }
        if (max_off < 1e-15) break;
        const cd app = A[p][p], aqq = A[q][q], apq = A[p][q];
        const double phi = 0.5 * std::atan2(2.0 * std::abs(apq), std::real(app - aqq));
        const cd c = std::cos(phi);
        const cd s = std::sin(phi) * apq / std::abs(apq);
        for (int i = 0; i < n; ++i) {
            const cd vip = V[i][p], viq = V[i][q];
            V[i][p] = c * vip + s * viq;
            V[i][q] = -std::conj(s) * vip + c * viq;
            if (i != p && i != q) {
                const cd aip = A[i][p], aiq = A[i][q];
                A[i][p] = A[p][i] = c * aip + s * aiq;
                A[i][q] = A[q][i] = -std::conj(s) * aip + c * aiq;
            }
        }
        A[p][p] = c * c * app + s * std::conj(s) * aqq + 2.0 * std::real(c * s * std::conj(apq));
        A[q][q] = s * std::conj(s) * app + c * c * aqq - 2.0 * std::real(c * s * std::conj(apq));
        A[p][q] = A[q][p] = 0.0;
    }
    SmallEig r;
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int i, int j) { return std::real(A[i][i]) < std::real(A[j][j]); });
    for (int i : idx) {
        r.vals.push_back(std::real(A[i][i]));
        std::vector<cd> v(n);
        for (int j = 0; j < n; ++j) v[j] = V[j][i];
        r.vecs.push_back(v);
    }
    return r;
}

struct DavidsonOut { std::vector<double> vals; std::vector<Vec> vecs; int iters = 0; bool conv = false; };

// max_iter: the reference's hard-coded 100 (:141,180); the CPU baseline times
// fewer iterations of the same loop.
DavidsonOut davidson(const Ham& H, int n_eig, int max_sub, double tol, int max_iter = 100) {  // :86-227
    DavidsonOut out;
    const uint64_t dim = H.basis.size();
    if (dim == 0) return out;
    n_eig = std::min<int>(n_eig, (int)dim);
    max_sub = std::max(max_sub, 2 * n_eig);
    std::vector<Vec> V, HV;
    std::mt19937 rng(1234);
    std::uniform_real_distribution<double> dist(-1.0, 1.0);
    std::vector<uint64_t> di(dim);
    for (uint64_t i = 0; i < dim; ++i) di[i] = i;
    std::sort(di.begin(), di.end(), [&](uint64_t i, uint64_t j) { return H.diag[i].real() < H.diag[j].real(); });
    for (int i = 0; i < n_eig; ++i) {
        Vec v(dim);
        v[di[i]] = 1.0;
        for (const auto& vp : V) axpy(-dot(vp, v), vp, v);
        double nrm = norm(v);
        if (nrm < 1e-10) {
            fill_complex(rng, dist, dim, v.data());
            for (const auto& vp : V) axpy(-dot(vp, v), vp, v);
            nrm = norm(v);
        }
        scal(cd(1.0 / nrm, 0.0), v);
        V.push_back(v);
        Vec hv(dim);
        apply(H, v, hv);
        HV.push_back(hv);
    }
    for (int iter = 0; iter < max_iter; ++iter) {
        const int m = (int)V.size();
        std::vector<std::vector<cd>> Hs(m, std::vector<cd>(m));
        for (int i = 0; i < m; ++i)
            for (int j = 0; j <= i; ++j) {
                Hs[i][j] = dot(V[i], HV[j]);
                if (i != j) Hs[j][i] = std::conj(Hs[i][j]);
            }
        auto eig = small_hermitian(Hs);
        bool all_conv = true;
        std::vector<Vec> corr;
        for (int k = 0; k < n_eig; ++k) {
            const double lambda = eig.vals[k];
            const auto& s = eig.vecs[k];
            Vec r(dim);
            for (int i = 0; i < m; ++i) {
                axpy(s[i], HV[i], r);
                axpy(cd(-lambda * s[i].real(), -lambda * s[i].imag()), V[i], r);
            }
            const double rn = norm(r);
            if (rn > tol) {
                all_conv = false;
                Vec t(dim);
                for (uint64_t i = 0; i < dim; ++i) {  // davidson_precond (:171-175)
                    cd diff = H.diag[i] - lambda;
                    if (std::abs(diff) < 1e-10) diff = (diff.real() >= 0) ? 1e-10 : -1e-10;
                    t[i] = r[i] / diff;
                }
                corr.push_back(std::move(t));
            }
        }
        if (all_conv || iter == max_iter - 1) {
            out.iters = iter + 1; out.conv = all_conv;
            for (int k = 0; k < n_eig; ++k) {
                out.vals.push_back(eig.vals[k]);
                Vec ev(dim);
                for (int i = 0; i < m; ++i) axpy(eig.vecs[k][i], V[i], ev);
                out.vecs.push_back(std::move(ev));
            }
            return out;
        }
        if (V.size() + corr.size() > (size_t)max_sub) {  // restart (:196-211)
            std::vector<Vec> nV, nHV;
            for (int k = 0; k < n_eig; ++k) {
                Vec rv(dim), rh(dim);
                for (int i = 0; i < m; ++i) { axpy(eig.vecs[k][i], V[i], rv); axpy(eig.vecs[k][i], HV[i], rh); }
                nV.push_back(std::move(rv)); nHV.push_back(std::move(rh));
            }
            V = std::move(nV); HV = std::move(nHV);
        }
        for (auto& t : corr) {  // single-pass CGS (:213-223)
            for (const auto& v : V) axpy(-dot(v, t), v, t);
            const double nrm = norm(t);
            if (nrm > 1e-10) {
                scal(cd(1.0 / nrm, 0.0), t);
                V.push_back(t);
                Vec ht(dim);
                apply(H, t, ht);
                HV.push_back(ht);
            }
        }
    }
    return out;
}

// ---- 3-term recurrence (no reorth): dynamics.cpp:13-59, ftlm.cpp:24-53 -------------
struct Tri { std::vector<double> a, b; };
Tri three_term(const Ham& H, Vec v_curr, int n_steps) {
    const uint64_t dim = H.basis.size();
    Vec v_prev(dim), w(dim);
    Tri t;
    for (int i = 0; i < n_steps; ++i) {
        apply(H, v_curr, w);
        const double alpha = dot(v_curr, w).real();
        t.a.push_back(alpha);
        axpy(cd(-alpha, 0.0), v_curr, w);
        if (i > 0) axpy(cd(-t.b.back(), 0.0), v_prev, w);
        const double beta = norm(w);
        if (beta < 1e-15) break;
        t.b.push_back(beta);
        v_prev = v_curr;
        v_curr = w;
        scal(cd(1.0 / beta, 0.0), v_curr);
    }
    return t;
}

Ham* make_ham(int model, int nsites, const int* sector, int n_terms, const double* cre, const double* cim,
              const int* nfac, const char* const* ops, const int* sites) {
    Sector sec;
    sec.use_sz = sector[0]; sec.sz2 = sector[1];
    sec.use_nup = sector[2]; sec.nup = sector[3];
    sec.use_ndn = sector[4]; sec.ndn = sector[5];
    sec.use_n = sector[6]; sec.n = sector[7];
    auto h = std::make_unique<Ham>();
    h->basis = build_basis(model, nsites, sec);
    int k = 0;
    for (int t = 0; t < n_terms; ++t) {
        Term term; term.coeff = cd(cre[t], cim[t]);
        for (int f = 0; f < nfac[t]; ++f, ++k)
            term.factors.push_back({std::string(ops[k]), sites[k], op_id(model, std::string(ops[k]))});
        h->terms.push_back(term);
    }
    return h.release();
}

}  // namespace

extern "C" {

const char* qko_last_error(void) { return g_err.c_str(); }

void* qko_create(int model, int nsites, const int* sector, int n_terms, const double* cre, const double* cim,
                 const int* nfac, const char* const* ops, const int* sites) {
    try {
        Ham* h = make_ham(model, nsites, sector, n_terms, cre, cim, nfac, ops, sites);
        build_csr(*h, 0, h->basis.size());
        return h;
    } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

void* qko_basis_create(int model, int nsites, const int* sector) {
    try {
        return make_ham(model, nsites, sector, 0, nullptr, nullptr, nullptr, nullptr, nullptr);
    } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

void qko_destroy(void* h) { delete static_cast<Ham*>(h); }
uint64_t qko_dim(void* h) { return static_cast<Ham*>(h)->basis.size(); }
void qko_states(void* h, uint64_t* out) {
    const auto& s = static_cast<Ham*>(h)->basis.states;
    std::memcpy(out, s.data(), s.size() * sizeof(uint64_t));
}
int64_t qko_index(void* h, uint64_t s) { return static_cast<Ham*>(h)->basis.index(s); }
uint64_t qko_nnz(void* h) { return static_cast<Ham*>(h)->cols.size(); }
void qko_csr(void* hp, int32_t* ro, int32_t* cols, double* vals) {
    auto* h = static_cast<Ham*>(hp);
    std::memcpy(ro, h->rows.data(), h->rows.size() * sizeof(int32_t));
    std::memcpy(cols, h->cols.data(), h->cols.size() * sizeof(int32_t));
    for (size_t j = 0; j < h->vals.size(); ++j) { vals[2 * j] = h->vals[j].real(); vals[2 * j + 1] = h->vals[j].imag(); }
}
void qko_apply(void* hp, const double* x, double* y) {
    apply(*static_cast<Ham*>(hp), reinterpret_cast<const cd*>(x), reinterpret_cast<cd*>(y));
}
void qko_diagonal(void* hp, double* d) {
    auto* h = static_cast<Ham*>(hp);
    for (size_t i = 0; i < h->diag.size(); ++i) { d[2 * i] = h->diag[i].real(); d[2 * i + 1] = h->diag[i].imag(); }
}

int qko_lanczos(void* hp, int maxiter, double tol, double* energy, int* iters, int* conv, double* evec) {
    try {
        auto* h = static_cast<Ham*>(hp);
        const uint64_t dim = h->basis.size();
        Vec v(dim);
        std::mt19937 rng(1234);  // lanczos.cpp:115-120
        std::uniform_real_distribution<double> dist(-1.0, 1.0);
        fill_complex(rng, dist, dim, v.data());
        auto r = lanczos(*h, v, maxiter, tol);
        *energy = r.energy; *iters = r.iters; *conv = r.conv ? 1 : 0;
        if (evec) std::memcpy(evec, r.evec.data(), r.evec.size() * sizeof(cd));
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

int qko_lanczos_from(void* hp, const double* v0, int maxiter, double tol, double* energy, int* iters, int* conv,
                     double* evec, double* alphas, double* betas) {
    try {
        auto* h = static_cast<Ham*>(hp);
        const uint64_t dim = h->basis.size();
        Vec v(reinterpret_cast<const cd*>(v0), reinterpret_cast<const cd*>(v0) + dim);
        auto r = lanczos(*h, v, maxiter, tol);
        *energy = r.energy; *iters = r.iters; *conv = r.conv ? 1 : 0;
        if (evec) std::memcpy(evec, r.evec.data(), r.evec.size() * sizeof(cd));
        if (alphas) for (size_t i = 0; i < r.alphas.size(); ++i) alphas[i] = r.alphas[i];
        if (betas) for (size_t i = 0; i < r.betas.size(); ++i) betas[i] = r.betas[i];
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

int qko_davidson(void* hp, int n_eig, int max_sub, double tol, double* evals, double* evecs, int* iters, int* conv,
                 int* n_out) {
    return qko_davidson_max(hp, n_eig, max_sub, tol, 100, evals, evecs, iters, conv, n_out);
}

int qko_davidson_max(void* hp, int n_eig, int max_sub, double tol, int max_iter, double* evals, double* evecs,
                     int* iters, int* conv, int* n_out) {
    try {
        auto* h = static_cast<Ham*>(hp);
        auto r = davidson(*h, n_eig, max_sub, tol, max_iter);
        const uint64_t dim = h->basis.size();
        *iters = r.iters; *conv = r.conv ? 1 : 0; *n_out = (int)r.vals.size();
        for (size_t k = 0; k < r.vals.size(); ++k) {
            evals[k] = r.vals[k];
            if (evecs) std::memcpy(evecs + k * 2 * dim, r.vecs[k].data(), dim * sizeof(cd));
        }
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

// dynamics.cpp:13-59
int qko_cf(void* hp, const double* phi0, int n_iter, double* alphas, double* betas, double* norm_out, int* n_alpha,
           int* n_beta) {
    try {
        auto* h = static_cast<Ham*>(hp);
        const uint64_t dim = h->basis.size();
        *n_alpha = 0; *n_beta = 0; *norm_out = 0.0;
        if (dim == 0) return 0;
        Vec p(reinterpret_cast<const cd*>(phi0), reinterpret_cast<const cd*>(phi0) + dim);
        const double np = norm(p);
        if (np < 1e-15) return 0;  // :26
        scal(cd(1.0 / np, 0.0), p);
        auto t = three_term(*h, p, n_iter);
        *norm_out = np; *n_alpha = (int)t.a.size(); *n_beta = (int)t.b.size();
        for (size_t i = 0; i < t.a.size(); ++i) alphas[i] = t.a[i];
        for (size_t i = 0; i < t.b.size(); ++i) betas[i] = t.b[i];
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

// dynamics.cpp:61-89: backward continued fraction at z = omega + E0 + i eta.
double qko_spectral(const double* alphas, const double* betas, size_t n, double norm_phi0, double omega, double E0,
                    double eta) {
    if (n == 0) return 0.0;
    const cd z(omega + E0, eta);
    cd f = 0.0;
    for (int i = (int)n - 1; i >= 0; --i) {
        if (i == (int)n - 1) f = 1.0 / (z - alphas[i]);
        else f = 1.0 / (z - alphas[i] - betas[i] * betas[i] * f);
    }
    return -1.0 / M_PI * std::imag(norm_phi0 * norm_phi0 * f);
}

// ftlm.cpp:123-170
int qko_ftlm(void* hp, double beta, int n_random, int n_steps, double* Zo, double* Eo, double* Co) {
    try {
        auto* h = static_cast<Ham*>(hp);
        const uint64_t dim = h->basis.size();
        if (dim == 0) { *Zo = 0; *Eo = 0; *Co = 0; return 0; }
        std::mt19937 rng(42);
        std::normal_distribution<double> dist(0.0, 1.0);
        double Z = 0, E = 0, E2 = 0;
        for (int r = 0; r < n_random; ++r) {
            Vec v(dim);
            fill_complex(rng, dist, dim, v.data());
            const double nrm = norm(v);
            normalize(v);
            auto t = three_term(*h, v, n_steps);
            std::vector<double> ev, first;
            tridiag_components(t.a, t.b, ev, first);
            for (size_t i = 0; i < ev.size(); ++i) {
                const double w = nrm * nrm * first[i] * first[i] * std::exp(-beta * ev[i]);
                Z += w; E += ev[i] * w; E2 += ev[i] * ev[i] * w;
            }
        }
        Z /= n_random; E /= n_random; E2 /= n_random;
        *Zo = Z; *Eo = E / Z; *Co = (beta * beta) * (E2 / Z - (E / Z) * (E / Z));
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

int qko_ftlm_tridiag(void* hp, int n_random, int n_steps, double* alphas, double* betas, int* n_alpha, int* n_beta,
                     double* norms) {
    try {
        auto* h = static_cast<Ham*>(hp);
        const uint64_t dim = h->basis.size();
        std::mt19937 rng(42);
        std::normal_distribution<double> dist(0.0, 1.0);
        for (int r = 0; r < n_random; ++r) {
            Vec v(dim);
            fill_complex(rng, dist, dim, v.data());
            norms[r] = norm(v);
            normalize(v);
            auto t = three_term(*h, v, n_steps);
            n_alpha[r] = (int)t.a.size(); n_beta[r] = (int)t.b.size();
            for (size_t i = 0; i < t.a.size(); ++i) alphas[(size_t)r * n_steps + i] = t.a[i];
            for (size_t i = 0; i < t.b.size(); ++i) betas[(size_t)r * n_steps + i] = t.b[i];
        }
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

void qko_tridiag_components(const double* a, const double* b, int n, double* evals, double* first) {
    std::vector<double> av(a, a + n), bv(b, b + (n > 0 ? n - 1 : 0)), ev, fc;
    tridiag_components(av, bv, ev, fc);
    for (size_t i = 0; i < ev.size(); ++i) { evals[i] = ev[i]; first[i] = fc[i]; }
}

double qko_tridiag_ground(const double* a, const double* b, int n, double* evec) {
    std::vector<double> av(a, a + n), bv(b, b + (n > 0 ? n - 1 : 0)), v;
    const double e = tridiag_ground(av, bv, n, v);
    if (evec) for (int i = 0; i < n; ++i) evec[i] = v[i];
    return e;
}

void qko_rng_uniform_complex(uint32_t seed, uint64_t n, double* out) {
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> dist(-1.0, 1.0);
    fill_complex(rng, dist, n, reinterpret_cast<cd*>(out));
}

void qko_rng_normal_complex(uint32_t seed, uint64_t n, double* out) {
    std::mt19937 rng(seed);
    std::normal_distribution<double> dist(0.0, 1.0);
    fill_complex(rng, dist, n, reinterpret_cast<cd*>(out));
}

void qko_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void* qko_create_parallel(int model, int nsites, const int* sector, int n_terms, const double* cre, const double* cim,
                          const int* nfac, const char* const* ops, const int* sites) {
    try {
        Ham* h = make_ham(model, nsites, sector, n_terms, cre, cim, nfac, ops, sites);
        build_csr_parallel(*h);
        return h;
    } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

int qko_lanczos_timed(void* hp, const double* v0, int n_steps, double* step_seconds, int* n_done, double* energy) {
    try {
        auto* h = static_cast<Ham*>(hp);
        const uint64_t dim = h->basis.size();
        Vec v(dim);
        if (v0) {
            std::memcpy(v.data(), v0, dim * sizeof(cd));
        } else {
            std::mt19937 rng(1234);  // lanczos.cpp:115-120
            std::uniform_real_distribution<double> dist(-1.0, 1.0);
            fill_complex(rng, dist, dim, v.data());
        }
        std::vector<double> st;
        auto r = lanczos(*h, v, n_steps, -1.0, &st);  // tol < 0: every step runs
        *n_done = (int)st.size();
        for (size_t i = 0; i < st.size(); ++i) step_seconds[i] = st[i];
        *energy = r.energy;
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

void* qko_sample_create(int model, int nsites, const int* sector, int n_terms, const double* cre, const double* cim,
                        const int* nfac, const char* const* ops, const int* sites, uint64_t row0, uint64_t nrows) {
    try {
        Ham* h = make_ham(model, nsites, sector, n_terms, cre, cim, nfac, ops, sites);
        const uint64_t dim = h->basis.size();
        if (row0 > dim) row0 = dim;
        if (row0 + nrows > dim) nrows = dim - row0;
        build_csr(*h, row0, nrows);
        return h;
    } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

int qko_sample_time(void* hp, int reps, int k_reorth, int n_threads, double* t_apply, double* t_vec) {
    try {
#ifdef _OPENMP
        if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
        auto* h = static_cast<Ham*>(hp);
        const uint64_t dim = h->basis.size(), n = h->nrows;
        Vec x(dim), y(n);
        for (uint64_t i = 0; i < dim; ++i) x[i] = cd(1.0 / (1.0 + (double)(i % 97)), 0.25);
        apply(*h, x.data(), y.data());  // warm-up
        auto t0 = std::chrono::steady_clock::now();
        for (int r = 0; r < reps; ++r) apply(*h, x.data(), y.data());
        auto t1 = std::chrono::steady_clock::now();
        *t_apply = std::chrono::duration<double>(t1 - t0).count() / reps;
        // One Lanczos step's vector algebra at reorthogonalisation depth k:
        // alpha dot, two axpys, k (dot + axpy) pairs, the norm, copies/scale.
        std::vector<Vec> V(std::max(1, k_reorth), Vec(n, cd(1e-3, 2e-3)));
        Vec w(n, cd(0.5, -0.25)), vp(n, cd(0.1, 0.2)), vc(n, cd(0.3, 0.1));
        auto t2 = std::chrono::steady_clock::now();
        for (int r = 0; r < reps; ++r) {
            const double a = dot(vc, w).real();
            axpy(cd(-a, 0.0), vc, w);
            axpy(cd(-0.5, 0.0), vp, w);
            for (int j = 0; j < k_reorth; ++j) axpy(-dot(V[j], w) * 1e-3, V[j], w);
            const double b = norm(w);
            vp = vc; vc = w; scal(cd(1.0 / (b + 1.0), 0.0), vc);
            V[r % V.size()] = vc;
        }
        auto t3 = std::chrono::steady_clock::now();
        *t_vec = std::chrono::duration<double>(t3 - t2).count() / reps;
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -2; }
}

}  // extern "C"
