// Basis layer: sector enumeration as combinatorial tables instead of the
// reference's enumerate-and-hash (src/basis/spinhalf_basis.cpp:59-104,
// fermion_basis.cpp:167-197, hubbard_basis.cpp:59-100, tj_basis.cpp:161-201).
//
// Internal encoding.  Spin-1/2 and spinless-fermion states are used as they
// are.  Hubbard and t-J states, which the reference stores interleaved (up
// electron of site i at bit 2i, down at 2i+1, src/sites/hubbard_site.cpp:11-29),
// are stored "split": up occupations at bits 0..N-1, down occupations at bits
// N..2N-1.
//
// Ranking (RANK_TABLE).  A state s splits into an outer part a = s >> n_in and
// an inner part b = s & (2^n_in - 1).  The states with a given a form one
// contiguous block, blocks in ascending a; rank(s) = outer_off[a] +
// inner_rank[b], where inner_rank is the position of b among the inner
// configurations of its popcount.  Those are ordered by the number of domain
// walls of b (adjacent inner bits that differ), then by value: rows whose
// inner nearest-neighbour flip lists have equal lengths sit together, so the
// threads of a warp walk lists of equal length in the SpMV.  The reference
// order is ascending states (colex within a class); a permutation
// (ref_of_int) converts at the C ABI wherever the two differ.
// RANK_SEARCH (t-J, and very wide spin chains) keeps the sorted internal states
// and ranks by binary search inside the block of a.
#include "qkg.hpp"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace qkg {

namespace {
thread_local std::string t_last_error;

struct BinomTable {
    uint64_t c[65][65];
    BinomTable() {
        std::memset(c, 0, sizeof(c));
        for (int n = 0; n <= 64; ++n) {
            c[n][0] = 1;
            for (int k = 1; k <= n; ++k) c[n][k] = c[n - 1][k - 1] + (k <= n - 1 ? c[n - 1][k] : 0);
        }
    }
};
const BinomTable& btab() { static BinomTable t; return t; }

inline int popc(uint64_t x) { return __builtin_popcountll(x); }

// All n-bit strings with popcount k in ascending order (Gosper's next-permutation).
std::vector<uint64_t> fixed_pop(int n, int k) {
    std::vector<uint64_t> out;
    if (k < 0 || k > n) return out;
    out.reserve(binom(n, k));
    if (k == 0) { out.push_back(0); return out; }
    uint64_t v = (k == 64) ? ~0ULL : ((1ULL << k) - 1);
    const uint64_t lim = (n >= 64) ? 0 : (1ULL << n);
    while (true) {
        out.push_back(v);
        const uint64_t t = v | (v - 1);
        const uint64_t w = (t + 1) | (((~t & (0 - ~t)) - 1) >> (__builtin_ctzll(v) + 1));
        if ((lim && w >= lim) || w <= v) break;
        v = w;
    }
    return out;
}

constexpr int kMaxTableBits = 22;
}  // namespace

std::atomic<uint64_t> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }
void add_launches(int64_t d) { g_launches.fetch_add((uint64_t)d, std::memory_order_relaxed); }

void set_last_error(const std::string& msg) { t_last_error = msg; }
const char* last_error() { return t_last_error.c_str(); }

uint64_t binom(int n, int k) {
    if (n < 0 || k < 0 || k > n || n > 64) return 0;
    return btab().c[n][k];
}

Basis::Basis(Model m, int N_, const Sector& s) : model(m), N(N_), sec(s) {
    const bool fermionic_pair = (m == HUBBARD || m == TJ);
    // N bounds of the reference (spinhalf_basis.cpp:19-24, hubbard_basis.cpp:19-24).
    if (!fermionic_pair) QKG_REQUIRE(N >= 1 && N <= 63, "basis: N must satisfy 1 <= N <= 63");
    else QKG_REQUIRE(N >= 1 && N <= 31, "basis: N must satisfy 1 <= N <= 31");
    nbits = fermionic_pair ? 2 * N : N;
    split = fermionic_pair;
    no_double = (m == TJ);

    if (!fermionic_pair) {
        const bool constrained = (m == SPIN) ? sec.use_sz : sec.use_n;
        int k = -1;
        if (constrained) {
            if (m == SPIN) k = ((sec.sz2 + N) % 2 == 0) ? (sec.sz2 + N) / 2 : -1;  // 2*pop - N == sz2
            else k = sec.n;
            if (k < 0 || k > N) k = -2;  // empty sector
        }
        if (k >= 0) { ngroups = 1; gmask[0] = (N == 64) ? ~0ULL : ((1ULL << N) - 1); gpop[0] = k; }
        total_pop = k;
        if (k == -2) { dim = 0; ngroups = 1; gmask[0] = (1ULL << N) - 1; gpop[0] = N + 1; }
        n_in = std::min((N + 1) / 2, kMaxTableBits);
        n_out = N - n_in;
        if (n_out > kMaxTableBits) {
            // Only tiny sectors of very wide chains are usable; rank them by search.
            rank_kind = RANK_SEARCH;
            QKG_REQUIRE(k >= 0 && binom(N, k) <= (1ULL << 28), "basis: sector too large for ranking by search (more than 2^28 states)");
            states_int = fixed_pop(N, k);
            dim = states_int.size();
            n_in = N; n_out = 0;
            outer_off = {0, dim};
            permuted = false;
            return;
        }
        inner_all = (k < 0 && k != -2);
    } else {
        if (sec.use_nup) { gmask[ngroups] = (1ULL << N) - 1; gpop[ngroups] = sec.nup; ++ngroups; }
        if (sec.use_ndn) { gmask[ngroups] = ((1ULL << N) - 1) << N; gpop[ngroups] = sec.ndn; ++ngroups; }
        n_in = N; n_out = N;
        QKG_REQUIRE(N <= kMaxTableBits, "basis: Hubbard/t-J rank tables need N <= 22");
        if (m == TJ) {
            rank_kind = RANK_SEARCH;
        } else {
            inner_all = !sec.use_nup;
            inner_fixed_class = sec.use_nup ? sec.nup : -1;
        }
    }

    const uint64_t nout_cfg = 1ULL << n_out;
    in_mask_ = (n_in >= 64) ? ~0ULL : ((1ULL << n_in) - 1);

    if (rank_kind == RANK_TABLE) {
        if (!inner_all) {
            class_base.assign(n_in + 2, 0);
            for (int c = 0; c <= n_in; ++c) class_base[c + 1] = class_base[c] + (uint32_t)binom(n_in, c);
            inner_state.resize(1ULL << n_in);
            inner_rank.resize(1ULL << n_in);
            std::vector<uint32_t> fill(n_in + 1, 0);
            for (uint64_t b = 0; b < (1ULL << n_in); ++b) {  // ascending b => colex within each class
                const int c = popc(b);
                inner_rank[b] = fill[c];
                inner_state[class_base[c] + fill[c]] = (uint32_t)b;
                ++fill[c];
            }
            bool reordered = false;
            if (n_in >= 3) {
                const uint32_t wmask = (uint32_t)((1ULL << (n_in - 1)) - 1);
                auto walls = [wmask](uint32_t b) { return popc((b ^ (b >> 1)) & wmask); };
                std::vector<uint32_t> colex_state = inner_state, colex_rank = inner_rank;
                for (int c = 0; c <= n_in; ++c)
                    std::stable_sort(inner_state.begin() + class_base[c], inner_state.begin() + class_base[c + 1],
                                     [&](uint32_t x, uint32_t y) { return walls(x) < walls(y); });
                for (int c = 0; c <= n_in; ++c)
                    for (uint32_t r = class_base[c]; r < class_base[c + 1]; ++r) inner_rank[inner_state[r]] = r - class_base[c];
                reordered = inner_state != colex_state;
                if (reordered && !split) {
                    ref_inner_rank = std::move(colex_rank);
                    ref_inner_state = std::move(colex_state);
                }
            }
            inner_reordered_ = reordered;
        }
        outer_off.assign(nout_cfg + 1, 0);
        for (uint64_t a = 0; a < nout_cfg; ++a) outer_off[a + 1] = outer_off[a] + block_size((uint32_t)a);
        dim = outer_off[nout_cfg];
        permuted = (split && N > 1) || (inner_reordered_ && dim > 1);
    } else {
        // t-J: blocks by down configuration a, inner up configurations avoid a.
        outer_off.assign(nout_cfg + 1, 0);
        for (uint64_t a = 0; a < nout_cfg; ++a) {
            if (sec.use_ndn && popc(a) != sec.ndn) { outer_off[a + 1] = outer_off[a]; continue; }
            const uint64_t start = states_int.size();
            for (uint64_t b = 0; b < (1ULL << N); ++b) {
                if (b & a) continue;
                if (sec.use_nup && popc(b) != sec.nup) continue;
                states_int.push_back(b | (a << N));
            }
            outer_off[a + 1] = start + (states_int.size() - start);
        }
        dim = states_int.size();
        states_ref.resize(dim);
        for (uint64_t i = 0; i < dim; ++i) states_ref[i] = to_reference(states_int[i]);
        std::sort(states_ref.begin(), states_ref.end());
        permuted = N > 1;
    }
}

uint64_t Basis::block_size(uint32_t a) const {
    if (rank_kind == RANK_SEARCH) return outer_off[a + 1] - outer_off[a];
    if (!split) {
        if (total_pop == -2) return 0;
        if (inner_all) return 1ULL << n_in;
        const int c = total_pop - popc(a);
        return (c >= 0 && c <= n_in) ? binom(n_in, c) : 0;
    }
    if (sec.use_ndn && popc(a) != sec.ndn) return 0;
    return inner_all ? (1ULL << n_in) : binom(n_in, sec.nup);
}

int Basis::inner_class_of(uint32_t a) const {
    if (inner_all) return -1;
    if (!split) return total_pop - popc(a);
    return inner_fixed_class;
}

uint64_t Basis::to_internal(uint64_t s) const {
    if (!split) return s;
    uint64_t u = 0, d = 0;
    for (int i = 0; i < N; ++i) { u |= ((s >> (2 * i)) & 1ULL) << i; d |= ((s >> (2 * i + 1)) & 1ULL) << i; }
    return u | (d << N);
}

uint64_t Basis::to_reference(uint64_t s) const {
    if (!split) return s;
    uint64_t r = 0;
    for (int i = 0; i < N; ++i) r |= (((s >> i) & 1ULL) << (2 * i)) | (((s >> (N + i)) & 1ULL) << (2 * i + 1));
    return r;
}

bool Basis::contains_int(uint64_t s) const {
    if (nbits < 64 && (s >> nbits)) return false;
    for (int g = 0; g < ngroups; ++g) if (popc(s & gmask[g]) != gpop[g]) return false;
    if (no_double && (s & (s >> N) & ((1ULL << N) - 1))) return false;
    if (rank_kind == RANK_SEARCH) return std::binary_search(states_int.begin(), states_int.end(), s);
    return dim > 0;
}

uint64_t Basis::rank_int(uint64_t s) const {
    const uint64_t a = (n_in >= 64) ? 0 : (s >> n_in);
    const uint64_t b = s & in_mask_;
    if (rank_kind == RANK_SEARCH) {
        auto lo = states_int.begin() + outer_off[a], hi = states_int.begin() + outer_off[a + 1];
        return std::lower_bound(lo, hi, s) - states_int.begin();
    }
    return outer_off[a] + (inner_all ? b : inner_rank[b]);
}

uint64_t Basis::unrank_int(uint64_t i) const {
    if (rank_kind == RANK_SEARCH) return states_int[i];
    const auto it = std::upper_bound(outer_off.begin(), outer_off.end(), i);
    const uint64_t a = (uint64_t)(it - outer_off.begin()) - 1;
    const uint64_t r = i - outer_off[a];
    const uint64_t b = inner_all ? r : inner_state[class_base[inner_class_of((uint32_t)a)] + r];
    return (a << n_in) | b;
}

bool Basis::contains_ref(uint64_t s_ref) const {
    if (nbits < 64 && (s_ref >> nbits)) return false;
    return contains_int(to_internal(s_ref));
}

// Rank of a Hubbard state in the reference's ascending interleaved order:
// for every set bit p (high to low) count the valid states that share the bits
// above p and have 0 at p; the bits below p hold (p+1)/2 up slots and p/2
// down slots.
namespace {
inline uint64_t hub_count(const Sector& sec, int up_slots, int dn_slots, int up_rem, int dn_rem) {
    const uint64_t cu = sec.use_nup ? binom(up_slots, up_rem) : (1ULL << up_slots);
    const uint64_t cd = sec.use_ndn ? binom(dn_slots, dn_rem) : (1ULL << dn_slots);
    return cu * cd;
}
}  // namespace

int64_t Basis::index_ref(uint64_t s_ref) const {
    if (!contains_ref(s_ref)) return -1;
    if (!split && !permuted) return (int64_t)rank_int(s_ref);
    if (!split) return (int64_t)(outer_off[s_ref >> n_in] + ref_inner_rank[s_ref & in_mask_]);
    if (model == TJ) {
        auto it = std::lower_bound(states_ref.begin(), states_ref.end(), s_ref);
        return it - states_ref.begin();
    }
    uint64_t rank = 0;
    int up_rem = sec.nup, dn_rem = sec.ndn;
    for (int p = nbits - 1; p >= 0; --p) {
        if (!((s_ref >> p) & 1ULL)) continue;
        rank += hub_count(sec, (p + 1) / 2, p / 2, up_rem, dn_rem);
        if (p % 2 == 0) --up_rem; else --dn_rem;
    }
    return (int64_t)rank;
}

uint64_t Basis::state_ref(uint64_t i) const {
    QKG_REQUIRE(i < dim, "basis: index out of range");
    if (!split && !permuted) return unrank_int(i);
    if (!split) {
        const auto it = std::upper_bound(outer_off.begin(), outer_off.end(), i);
        const uint64_t a = (uint64_t)(it - outer_off.begin()) - 1;
        return (a << n_in) | ref_inner_state[class_base[inner_class_of((uint32_t)a)] + (i - outer_off[a])];
    }
    if (model == TJ) return states_ref[i];
    uint64_t s = 0;
    int up_rem = sec.nup, dn_rem = sec.ndn;
    for (int p = nbits - 1; p >= 0; --p) {
        const uint64_t c0 = hub_count(sec, (p + 1) / 2, p / 2, up_rem, dn_rem);
        if (i >= c0) {
            i -= c0;
            s |= 1ULL << p;
            if (p % 2 == 0) --up_rem; else --dn_rem;
        }
    }
    return s;
}

uint64_t Basis::ref_index_of_int(uint64_t i_int) const {
    if (!permuted) return i_int;
    return (uint64_t)index_ref(to_reference(unrank_int(i_int)));
}

std::vector<WorkItem> Basis::work_items(uint32_t chunk) const {
    std::vector<WorkItem> items;
    if (rank_kind == RANK_SEARCH) {
        for (uint64_t r = 0; r < dim; r += chunk)
            items.push_back({r, (uint32_t)std::min<uint64_t>(chunk, dim - r), 0u, 0u, 0u});
        return items;
    }
    const uint64_t nout_cfg = 1ULL << n_out;
    for (uint64_t a = 0; a < nout_cfg; ++a) {
        const uint64_t size = outer_off[a + 1] - outer_off[a];
        if (!size) continue;
        const uint32_t base = inner_all ? 0u : class_base[inner_class_of((uint32_t)a)];
        for (uint64_t r = 0; r < size; r += chunk)
            items.push_back({outer_off[a] + r, (uint32_t)std::min<uint64_t>(chunk, size - r), (uint32_t)a,
                             (uint32_t)(base + r), 0u});
    }
    return items;
}

// ---------------------------------------------------------------- device copy
struct Basis::DevCopy {
    int dev = -1;
    DevBasis d;
    std::vector<void*> allocs;
    ~DevCopy() {
        int cur = 0;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != dev) cudaSetDevice(dev);
        for (void* p : allocs) device_free(p);
        if (cur != dev) cudaSetDevice(cur);
    }
    void* alloc(size_t bytes) {
        void* p = nullptr;
        device_alloc(&p, std::max<size_t>(bytes, 1));
        allocs.push_back(p);
        return p;
    }
    template <class T>
    const T* upload(const std::vector<T>& v) {
        if (v.empty()) return nullptr;
        void* p = nullptr;
        device_alloc(&p, v.size() * sizeof(T));
        allocs.push_back(p);
        QKG_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        return static_cast<const T*>(p);
    }
};

Basis::~Basis() = default;

const DevBasis& Basis::device(int dev) {
    std::lock_guard<std::mutex> lk(mu_);
    for (auto& c : dev_) if (c->dev == dev) return c->d;
    auto c = std::make_unique<DevCopy>();
    c->dev = dev;
    DevBasis& d = c->d;
    d.nbits = nbits; d.n_in = n_in; d.n_out = n_out; d.rank_kind = rank_kind;
    d.N = N; d.split = split; d.inner_all = inner_all;
    d.in_mask = in_mask_; d.dim = dim;
    d.ngroups = ngroups; d.no_double = no_double;
    d.gmask[0] = gmask[0]; d.gmask[1] = gmask[1]; d.gpop[0] = gpop[0]; d.gpop[1] = gpop[1];
    d.idx32 = dim < (1ULL << 32);
    if (d.idx32) {
        std::vector<uint32_t> o(outer_off.begin(), outer_off.end());
        d.outer_off = c->upload(o);
    } else {
        d.outer_off = c->upload(outer_off);
    }
    d.inner_rank = c->upload(inner_rank);
    d.inner_state = c->upload(inner_state);
    d.states_int = c->upload(states_int);
    if (permuted && dim && model != TJ && rank_kind == RANK_TABLE && nbits <= 64 && (split || !inner_all)) {
        // reference ranks computed on the device: interleaved count (Hubbard)
        // or block offset + colex rank of the inner configuration (spin/fermion)
        void* p = c->alloc(dim * (d.idx32 ? sizeof(uint32_t) : sizeof(uint64_t)));
        ref_permutation_device(d, sec, work_items(1024), split ? nullptr : &ref_inner_rank, p);
        d.ref_of_int = p;
    } else if (permuted && dim) {
        if (d.idx32) {
            std::vector<uint32_t> p(dim);
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < (long long)dim; ++i) p[i] = (uint32_t)ref_index_of_int((uint64_t)i);
            d.ref_of_int = c->upload(p);
        } else {
            std::vector<uint64_t> p(dim);
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < (long long)dim; ++i) p[i] = ref_index_of_int((uint64_t)i);
            d.ref_of_int = c->upload(p);
        }
    }
    dev_.push_back(std::move(c));
    return dev_.back()->d;
}

}  // namespace qkg
