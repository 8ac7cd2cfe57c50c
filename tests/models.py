"""Synthetic qkrylov model definitions shared by tests and the bench.

A model is (model_id, nsites, sector[8], terms); a term is
(coeff, [(op, site), ...]) with factors applied in list order, as in the
reference's OperatorTerm (include/qkrylov/operators/operator_term.hpp:22-32).
sector = [use_sz, sz2, use_nup, nup, use_ndn, ndn, use_n, n].
"""
SPIN, FERMION, HUBBARD, TJ = 0, 1, 2, 3


def sector(sz2=None, nup=None, ndn=None, n=None):
    return [int(sz2 is not None), sz2 or 0, int(nup is not None), nup or 0,
            int(ndn is not None), ndn or 0, int(n is not None), n or 0]


def heisenberg_terms(L, pbc, J=1.0, Jz=None):
    """J (Sz Sz) + J/2 (Sp Sm + Sm Sp) on bonds (i, i+1), and (L-1, 0) if pbc."""
    Jz = J if Jz is None else Jz
    terms = []
    for i in range(L if pbc else L - 1):
        j = (i + 1) % L
        terms += [(Jz, [("Sz", i), ("Sz", j)]), (0.5 * J, [("Sp", i), ("Sm", j)]),
                  (0.5 * J, [("Sm", i), ("Sp", j)])]
    return terms


def heisenberg(L, pbc, sz2=0, J=1.0):
    return (SPIN, L, sector(sz2=sz2) if sz2 is not None else sector(), heisenberg_terms(L, pbc, J))


def hubbard_terms(L, pbc, t=1.0, U=4.0):
    """-t (CdagS(i) CS(j) + CdagS(j) CS(i)) per bond and spin, plus U Nupdn(i)."""
    terms = []
    for i in range(L if pbc else L - 1):
        j = (i + 1) % L
        for s in ("Up", "Dn"):
            terms += [(-t, [("Cdag" + s, i), ("C" + s, j)]), (-t, [("Cdag" + s, j), ("C" + s, i)])]
    for i in range(L):
        terms.append((U, [("Nupdn", i)]))
    return terms


def hubbard(L, pbc, nup, ndn, t=1.0, U=4.0):
    return (HUBBARD, L, sector(nup=nup, ndn=ndn), hubbard_terms(L, pbc, t, U))


def tj_terms(L, pbc, t=1.0, J=0.5):
    """-t hopping per spin + J (Sz Sz + (S+ S- + S- S+)/2) written with number and 4-fermion factors."""
    terms = []
    for i in range(L if pbc else L - 1):
        j = (i + 1) % L
        for s in ("Up", "Dn"):
            terms += [(-t, [("Cdag" + s, i), ("C" + s, j)]), (-t, [("Cdag" + s, j), ("C" + s, i)])]
        terms += [(0.25 * J, [("Nup", i), ("Nup", j)]), (0.25 * J, [("Ndn", i), ("Ndn", j)]),
                  (-0.25 * J, [("Nup", i), ("Ndn", j)]), (-0.25 * J, [("Ndn", i), ("Nup", j)]),
                  (0.5 * J, [("CdagUp", i), ("CDn", i), ("CdagDn", j), ("CUp", j)]),
                  (0.5 * J, [("CdagDn", i), ("CUp", i), ("CdagUp", j), ("CDn", j)])]
    return terms


def fermion_chain_terms(L, pbc, t=1.0, V=0.7, mu=0.3):
    terms = []
    for i in range(L if pbc else L - 1):
        j = (i + 1) % L
        terms += [(-t, [("Cdag", i), ("C", j)]), (-t, [("Cdag", j), ("C", i)]), (V, [("N", i), ("N", j)])]
    for i in range(L):
        terms.append((-mu, [("N", i)]))
    return terms


def xyz_field_terms(L, pbc, hx=0.3, hy=0.2, cplx=0.1):
    """Hermitian spin model with terms that leave the Sz sector (Sx, Sy) and
    complex coefficients on conjugate pairs (a Dzyaloshinskii-Moriya-like bond)."""
    terms = heisenberg_terms(L, pbc)
    for i in range(L):
        terms.append((hx, [("Sx", i)]))
        terms.append((hy, [("Sy", i)]))
    for i in range(0, L - 1, 2):
        terms.append((complex(0.0, cplx), [("Sp", i), ("Sm", i + 1)]))
        terms.append((complex(0.0, -cplx), [("Sm", i), ("Sp", i + 1)]))
    terms.append((0.1, [("Sz", 0), ("Sz", 1), ("Sz", 2)]))
    terms.append((complex(0.2, -0.05), [("Sp", 0), ("Sz", 1), ("Sm", 2)]))
    terms.append((complex(0.2, 0.05), [("Sm", 0), ("Sz", 1), ("Sp", 2)]))
    return terms


def make_model(qk, model, nsites, sector, terms):
    """Basis, site and OpSum objects of the GPU library for a model tuple."""
    use_sz, sz2, use_nup, nup, use_ndn, ndn, use_n, n = [int(v) for v in sector]
    sec = qk.Sector(sz2=sz2 if use_sz else None, n=n if use_n else None,
                    nup=nup if use_nup else None, ndn=ndn if use_ndn else None)
    cls = {0: (qk.SpinHalfBasis, qk.SpinHalfSite), 1: (qk.FermionBasis, qk.FermionSite),
           2: (qk.HubbardBasis, qk.HubbardSite), 3: (qk.TJBasis, qk.TJSite)}[int(model)]
    basis = qk.Basis.__new__(cls[0])
    qk.Basis.__init__(basis, int(nsites), sec)
    site = cls[1]()
    ops = qk.OpSum()
    for c, facs in terms:
        args = []
        for o, s in facs:
            args += [o, s]
        ops.add_term(c, *args)
    return basis, site, ops
