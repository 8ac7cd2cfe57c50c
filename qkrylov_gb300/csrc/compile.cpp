// OpSum compiler: turns each OperatorTerm into bit masks on the row state.
//
// The reference applies a term to every basis state at Hamiltonian
// construction by walking its factors through Site::apply (a chain of string
// compares per factor, src/hamiltonian/matrix_free_hamiltonian.cpp:49-68,
// src/sites/*.cpp).  Every local action of the four site types is of the same
// shape on the current state t:
//     valid iff (t & cm) == cv;  amplitude = ((t & sm) == sm ? a1 : a0)
//     times (-1)^popcount(t & jm);  new state t ^ xm.
// Because t differs from the row state s only by the flips of the earlier
// factors (a constant P), the whole chain folds into conditions (C, V), one
// flip mask X, one Jordan-Wigner parity mask J and a constant amplitude, all
// on s.  Amplitude factors whose selector bits are not pinned by a condition
// stay as runtime "variable" factors.
#include "qkg.hpp"

#include <algorithm>

namespace qkg {

namespace {
using cd = std::complex<double>;

struct Action {
    uint64_t cm = 0, cv = 0, sm = 0, jm = 0, xm = 0;
    cd a0 = 0.0, a1 = 1.0;
};

inline uint64_t bit(int b) { return 1ULL << b; }
inline uint64_t below(int b) { return b == 0 ? 0 : ((1ULL << b) - 1); }
inline int parity(uint64_t x) { return __builtin_popcountll(x) & 1; }

// Local actions, restating the site files of the reference:
//   spin-1/2 src/sites/spinhalf_site.cpp:18-121 (bit = site, 1 = up)
//   fermion  src/sites/fermion_site.cpp:143-208 (JW sign from occupied modes below)
//   Hubbard  src/sites/hubbard_site.cpp:11-125  (up at 2i, down at 2i+1)
//   t-J      src/sites/tj_site.cpp:176-242      (creation needs an empty site)
Action local_action(SiteKind site, const std::string& op, int s) {
    Action a;
    if (site == SITE_SPIN || site == SITE_FERMION) {
        if (s < 0 || s >= 64) throw Error(INVALID_ARG, "site index out of range: " + std::to_string(s));
        const uint64_t m = bit(s);
        if (site == SITE_SPIN) {
            if (op == "Sz") { a.sm = m; a.a1 = 0.5; a.a0 = -0.5; return a; }
            if (op == "Sp") { a.cm = m; a.cv = 0; a.xm = m; return a; }
            if (op == "Sm") { a.cm = m; a.cv = m; a.xm = m; return a; }
            if (op == "Sx") { a.a1 = 0.5; a.xm = m; return a; }
            if (op == "Sy") { a.sm = m; a.a1 = cd(0.0, -0.5); a.a0 = cd(0.0, 0.5); a.xm = m; return a; }
            throw Error(INVALID_ARG, "Unknown spin operator: " + op);
        }
        if (op == "N") { a.sm = m; a.a1 = 1.0; a.a0 = 0.0; return a; }
        if (op == "Id") { return a; }
        if (op == "C") { a.cm = m; a.cv = m; a.jm = below(s); a.xm = m; return a; }
        if (op == "Cdag") { a.cm = m; a.cv = 0; a.jm = below(s); a.xm = m; return a; }
        throw Error(INVALID_ARG, "Unknown fermion operator: " + op);
    }
    if (s < 0 || s > 31) throw Error(INVALID_ARG, "site index out of range: " + std::to_string(s));
    const bool tj = (site == SITE_TJ);
    const int bu = 2 * s, bd = 2 * s + 1;
    if (op == "Nup") { a.sm = bit(bu); a.a1 = 1.0; a.a0 = 0.0; return a; }
    if (op == "Ndn") { a.sm = bit(bd); a.a1 = 1.0; a.a0 = 0.0; return a; }
    if (!tj && op == "Nupdn") { a.sm = bit(bu) | bit(bd); a.a1 = 1.0; a.a0 = 0.0; return a; }
    if (op == "CUp") { a.cm = bit(bu); a.cv = bit(bu); a.jm = below(bu); a.xm = bit(bu); return a; }
    if (op == "CdagUp") { a.cm = bit(bu) | (tj ? bit(bd) : 0); a.cv = 0; a.jm = below(bu); a.xm = bit(bu); return a; }
    if (op == "CDn") { a.cm = bit(bd); a.cv = bit(bd); a.jm = below(bd); a.xm = bit(bd); return a; }
    if (op == "CdagDn") { a.cm = bit(bd) | (tj ? bit(bu) : 0); a.cv = 0; a.jm = below(bd); a.xm = bit(bd); return a; }
    throw Error(INVALID_ARG, std::string(tj ? "Unknown TJ operator: " : "Unknown Hubbard operator: ") + op);
}

uint64_t permute_mask(const Basis& b, uint64_t m) {
    if (!b.split) return m;
    uint64_t r = 0;
    for (int i = 0; i < b.N; ++i) {
        r |= ((m >> (2 * i)) & 1ULL) << i;
        r |= ((m >> (2 * i + 1)) & 1ULL) << (b.N + i);
    }
    return r;
}
}  // namespace

std::vector<HostTerm> compile_terms(const Basis& b, SiteKind site, const std::vector<Term>& terms) {
    std::vector<HostTerm> out;
    const uint64_t phantom = (b.nbits >= 64) ? 0 : ~below(b.nbits);  // bits every basis state has at 0
    for (size_t ti = 0; ti < terms.size(); ++ti) {
        const Term& t = terms[ti];
        QKG_REQUIRE(!t.factors.empty(), "OpSum term without factors");
        uint64_t C = 0, V = 0, P = 0, J = 0;
        int csign = 0;
        cd amp = t.coeff;
        std::vector<DVar> vars;
        bool dead = false;
        for (const auto& f : t.factors) {
            const Action a = local_action(site, f.op, f.site);  // throws on unknown operators
            if (dead) continue;
            const uint64_t need = a.cv ^ (P & a.cm);  // condition on t = s ^ P, moved to s
            const uint64_t overlap = C & a.cm;
            if ((V & overlap) != (need & overlap)) { dead = true; continue; }
            C |= a.cm;
            V = (V & ~a.cm) | (need & a.cm);
            if (a.sm) vars.push_back({a.sm, P & a.sm, a.a0.real(), a.a0.imag(), a.a1.real(), a.a1.imag()});
            else amp *= a.a1;
            J ^= a.jm;
            csign ^= parity(P & a.jm);
            P ^= a.xm;
        }
        if (dead) continue;
        uint64_t X = P;
        // Bits above the basis width are 0 in every basis state.
        if ((C & phantom) & V) continue;
        C &= ~phantom; V &= ~phantom;
        if (X & phantom) continue;  // the target leaves the basis (never contained)
        J &= ~phantom;
        std::vector<DVar> keep;
        for (DVar v : vars) {
            const uint64_t ph = v.sm & phantom;
            if (ph && ((v.pf & ph) != ph)) { amp *= cd(v.a0r, v.a0i); continue; }  // selector always false
            v.sm &= ~phantom; v.pf &= ~phantom;
            if (!v.sm) { amp *= cd(v.a1r, v.a1i); continue; }
            if ((v.sm & ~C) == 0) {  // pinned by the conditions
                const bool sel = (((V ^ v.pf) & v.sm) == v.sm);
                amp *= sel ? cd(v.a1r, v.a1i) : cd(v.a0r, v.a0i);
                continue;
            }
            keep.push_back(v);
        }
        if (csign) amp = -amp;
        HostTerm h;
        h.C = permute_mask(b, C); h.V = permute_mask(b, V); h.X = permute_mask(b, X); h.J = permute_mask(b, J);
        h.amp = std::conj(amp);
        h.src = (int)ti;
        for (DVar v : keep) {
            v.sm = permute_mask(b, v.sm); v.pf = permute_mask(b, v.pf);
            v.a0i = -v.a0i; v.a1i = -v.a1i;  // conjugated with the rest of the amplitude
            h.vars.push_back(v);
        }
        // Does the target stay in the sector?  Flips whose direction the
        // conditions fix change each constrained popcount by a known amount.
        if (h.X) {
            for (int g = 0; g < b.ngroups && !dead; ++g) {
                const uint64_t xg = h.X & b.gmask[g];
                if (xg & ~h.C) { h.check = true; continue; }
                const int delta = __builtin_popcountll(xg & ~h.V) - __builtin_popcountll(xg & h.V);
                if (delta != 0) dead = true;
            }
            if (b.no_double) h.check = true;
        }
        if (dead || b.dim == 0) continue;
        out.push_back(std::move(h));
    }
    return out;
}

}  // namespace qkg
