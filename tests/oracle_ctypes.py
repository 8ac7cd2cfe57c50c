"""ctypes access to the two CPU checkers (test infrastructure only).

* ``Oracle("qko")``  -> oracle/_build/libqko.so, the oracle restatement (own code).
* ``Oracle("qkref64")`` -> oracle/_ref/libqkref.so, the reference sources compiled
  unchanged (exists only where the reference tree was present at build time).

Both expose the same call surface, so a test can run one model through both.
"""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_PATHS = {
    "qko": os.path.join(ROOT, "oracle", "_build", "libqko.so"),
    "qkref64": os.path.join(ROOT, "oracle", "_ref", "libqkref.so"),
}
_c = ctypes
_vp = _c.c_void_p
_dp = _c.POINTER(_c.c_double)
_ip = _c.POINTER(_c.c_int)


def available(kind):
    return os.path.exists(_PATHS[kind])


def _ptr(a, t=_c.c_double):
    return a.ctypes.data_as(_c.POINTER(t))


class Oracle:
    def __init__(self, kind="qko"):
        self.kind = kind
        self.lib = _c.CDLL(_PATHS[kind])
        p = kind + "_"
        L = self.lib
        self._f = lambda name: getattr(L, p + name)
        self._f("create").restype = _vp
        self._f("dim").restype = _c.c_uint64
        self._f("dim").argtypes = [_vp]
        self._f("index").restype = _c.c_int64
        self._f("index").argtypes = [_vp, _c.c_uint64]
        self._f("nnz").restype = _c.c_uint64
        self._f("nnz").argtypes = [_vp]
        self._f("destroy").argtypes = [_vp]
        self._f("spectral").restype = _c.c_double
        self._f("spectral").argtypes = [_dp, _dp, _c.c_size_t, _c.c_double, _c.c_double, _c.c_double, _c.c_double]
        self._f("last_error").restype = _c.c_char_p


class OHam:
    """One Hamiltonian inside an oracle library."""

    def __init__(self, oracle, model, nsites, sector, terms):
        self.o = oracle
        f = oracle._f
        n = len(terms)
        cre = np.array([complex(t[0]).real for t in terms], dtype=np.float64)
        cim = np.array([complex(t[0]).imag for t in terms], dtype=np.float64)
        nf = np.array([len(t[1]) for t in terms], dtype=np.int32)
        fl = [fac for t in terms for fac in t[1]]
        ops = (_c.c_char_p * max(1, len(fl)))(*[fac[0].encode() for fac in fl])
        sites = np.array([fac[1] for fac in fl] or [0], dtype=np.int32)
        sec = np.array(sector, dtype=np.int32)
        self._keep = (cre, cim, nf, ops, sites, sec)
        self.h = f("create")(int(model), int(nsites), _ptr(sec, _c.c_int), n, _ptr(cre), _ptr(cim),
                             _ptr(nf, _c.c_int), ops, _ptr(sites, _c.c_int))
        if not self.h:
            raise RuntimeError(oracle._f("last_error")().decode())
        self.dim = int(f("dim")(self.h))

    def __del__(self):
        if getattr(self, "h", None):
            self.o._f("destroy")(self.h)
            self.h = None

    def states(self):
        out = np.zeros(self.dim, dtype=np.uint64)
        self.o._f("states")(_vp(self.h), _ptr(out, _c.c_uint64))
        return out

    def index(self, s):
        return int(self.o._f("index")(self.h, int(s)))

    def csr(self):
        nnz = int(self.o._f("nnz")(self.h))
        ro = np.zeros(self.dim + 1, dtype=np.int32)
        cols = np.zeros(max(1, nnz), dtype=np.int32)
        vals = np.zeros(2 * max(1, nnz), dtype=np.float64)
        self.o._f("csr")(_vp(self.h), _ptr(ro, _c.c_int32), _ptr(cols, _c.c_int32), _ptr(vals))
        return ro, cols[:nnz], vals[: 2 * nnz].view(np.complex128)

    def apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros(self.dim, dtype=np.complex128)
        self.o._f("apply")(_vp(self.h), _ptr(x.view(np.float64)), _ptr(y.view(np.float64)))
        return y

    def diagonal(self):
        d = np.zeros(self.dim, dtype=np.complex128)
        self.o._f("diagonal")(_vp(self.h), _ptr(d.view(np.float64)))
        return d

    def lanczos(self, maxiter=200, tol=1e-12, want_vec=False):
        e = _c.c_double(); it = _c.c_int(); cv = _c.c_int()
        v = np.zeros(self.dim, dtype=np.complex128) if want_vec else None
        rc = self.o._f("lanczos")(_vp(self.h), int(maxiter), _c.c_double(tol), _c.byref(e), _c.byref(it),
                                  _c.byref(cv), _ptr(v.view(np.float64)) if want_vec else None)
        assert rc == 0
        return e.value, it.value, bool(cv.value), v

    def davidson(self, n_eig, max_sub=20, tol=1e-8, want_vecs=False):
        ev = np.zeros(n_eig); it = _c.c_int(); cv = _c.c_int(); no = _c.c_int()
        vecs = np.zeros((n_eig, self.dim), dtype=np.complex128) if want_vecs else None
        rc = self.o._f("davidson")(_vp(self.h), int(n_eig), int(max_sub), _c.c_double(tol), _ptr(ev),
                                   _ptr(vecs.view(np.float64)) if want_vecs else None, _c.byref(it),
                                   _c.byref(cv), _c.byref(no))
        assert rc == 0
        return ev[: no.value], it.value, bool(cv.value), (vecs[: no.value] if want_vecs else None)

    def cf(self, phi0, n_iter):
        phi0 = np.ascontiguousarray(phi0, dtype=np.complex128)
        a = np.zeros(n_iter); b = np.zeros(n_iter); nrm = _c.c_double(); na = _c.c_int(); nb = _c.c_int()
        rc = self.o._f("cf")(_vp(self.h), _ptr(phi0.view(np.float64)), int(n_iter), _ptr(a), _ptr(b),
                             _c.byref(nrm), _c.byref(na), _c.byref(nb))
        assert rc == 0
        return a[: na.value], b[: nb.value], nrm.value

    def ftlm(self, beta, n_random, n_steps):
        Z = _c.c_double(); E = _c.c_double(); C = _c.c_double()
        rc = self.o._f("ftlm")(_vp(self.h), _c.c_double(beta), int(n_random), int(n_steps), _c.byref(Z),
                               _c.byref(E), _c.byref(C))
        assert rc == 0
        return Z.value, E.value, C.value

    def ftlm_tridiag(self, n_random, n_steps):
        a = np.zeros((n_random, n_steps)); b = np.zeros((n_random, n_steps))
        na = np.zeros(n_random, dtype=np.int32); nb = np.zeros(n_random, dtype=np.int32); nr = np.zeros(n_random)
        rc = self.o._f("ftlm_tridiag")(_vp(self.h), int(n_random), int(n_steps), _ptr(a), _ptr(b),
                                       _ptr(na, _c.c_int), _ptr(nb, _c.c_int), _ptr(nr))
        assert rc == 0
        return a, b, na, nb, nr


def spectral(oracle, alphas, betas, norm, omega, E0, eta):
    a = np.ascontiguousarray(alphas, dtype=np.float64)
    b = np.ascontiguousarray(betas, dtype=np.float64)
    if b.size < 1:
        b = np.zeros(1)
    return oracle._f("spectral")(_ptr(a), _ptr(b), a.size, norm, omega, E0, eta)
