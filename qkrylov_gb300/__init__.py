"""qkrylov_gb300: GB300-native matrix-free Hamiltonian apply and Krylov solvers.

The compute library is ``qkrylov_gb300/_lib/libqkrylov_gb300.so`` (CUDA for
sm_103a behind the C ABI in ``include/qkrylov_c_api.h``).  This module is a thin
ctypes layer over that ABI that mirrors the reference's Python facade
(bindings/python/qkrylov/: ``SpinHalfBasis``, ``SpinHalfSite``, ``OpSum``,
``MatrixFreeHamiltonian(basis, site, ops).apply``, ``lanczos_ground_state``,
``davidson_lowest``, ``continued_fraction_coeffs``,
``evaluate_spectral_function``, ``ftlm``) with the same names, argument
meaning and result objects.  There is no CPU fallback: importing fails if the
library has not been built (``python -m qkrylov_gb300.build``).
"""
import ctypes as _c
import enum as _enum
import os as _os

import numpy as _np

_HERE = _os.path.dirname(_os.path.abspath(__file__))
LIB_PATH = _os.environ.get("QKRYLOV_GB300_LIB") or _os.path.join(_HERE, "_lib", "libqkrylov_gb300.so")

SUCCESS, ERROR_INVALID_ARG, ERROR_EXCEPTION, ERROR_CUDA, ERROR_DEVICE_TIMEOUT = 0, -1, -2, -3, -4

_vp, _i, _u64, _i64, _f, _d, _sz = _c.c_void_p, _c.c_int, _c.c_uint64, _c.c_int64, _c.c_float, _c.c_double, _c.c_size_t
_fp, _dp, _ip, _u64p = _c.POINTER(_c.c_float), _c.POINTER(_c.c_double), _c.POINTER(_c.c_int), _c.POINTER(_c.c_uint64)


class LanczosResultC(_c.Structure):
    _fields_ = [("energy", _f), ("iterations", _i), ("converged", _i)]


class DavidsonResultC(_c.Structure):
    _fields_ = [("iterations", _i), ("converged", _i)]


class FTLMResultC(_c.Structure):
    _fields_ = [("beta", _f), ("partition_function", _f), ("internal_energy", _f), ("specific_heat", _f)]


class LanczosResultF64(_c.Structure):
    _fields_ = [("energy", _d), ("energy_tridiag", _d), ("residual", _d), ("iterations", _i), ("converged", _i),
                ("selective_steps", _i), ("seconds_loop", _d), ("seconds_refine", _d), ("seconds_spmv", _d),
                ("spmv_calls", _i)]


class FTLMResultF64(_c.Structure):
    _fields_ = [("beta", _d), ("partition_function", _d), ("internal_energy", _d), ("specific_heat", _d)]


class BlockStatsC(_c.Structure):
    _fields_ = [("seconds", _d), ("spmv_ms", _d), ("vectors_per_lane", _i), ("padded_vectors", _i), ("rows", _u64),
                ("tune_ms", _d * 3)]


START_FTLM_STREAM, START_PHILOX, START_GIVEN, START_FTLM_STREAM_F32 = 0, 1, 2, 3

# name: (restype, argtypes)
_SIGS = {
    "qkrylov_last_error": (_c.c_char_p, []),
    "qkrylov_block_lanczos_tridiag": (_i, [_vp, _i, _i, _i, _i, _i, _i, _u64, _dp, _dp, _dp, _ip, _ip, _dp, _vp]),
    "qkrylov_ftlm_sectors_f64": (_i, [_vp, _i, _dp, _i, _i, _i, _i, _i, _u64, _dp, _dp, _dp, _dp, _vp]),
    "qkrylov_cf_block_f64": (_i, [_vp, _dp, _i, _i, _i, _dp, _dp, _ip, _ip, _dp, _vp]),
    "qkrylov_sector_create": (_vp, []),
    "qkrylov_sector_destroy": (None, [_vp]),
    "qkrylov_sector_set_sz": (_i, [_vp, _i]),
    "qkrylov_sector_set_hubbard_particles": (_i, [_vp, _i, _i]),
    "qkrylov_sector_set_n": (_i, [_vp, _i]),
    "qkrylov_sector_set_nup": (_i, [_vp, _i]),
    "qkrylov_sector_set_ndn": (_i, [_vp, _i]),
    "qkrylov_sector_set_nb": (_i, [_vp, _i]),
    "qkrylov_sector_get_sz": (_i, [_vp, _ip, _ip]),
    "qkrylov_sector_get_hubbard_particles": (_i, [_vp, _ip, _ip, _ip]),
    "qkrylov_sector_get_n": (_i, [_vp, _ip, _ip]),
    "qkrylov_sector_get_nb": (_i, [_vp, _ip, _ip]),
    "qkrylov_spinhalf_basis_create": (_vp, [_i, _vp]),
    "qkrylov_fermion_basis_create": (_vp, [_i, _vp]),
    "qkrylov_hubbard_basis_create": (_vp, [_i, _vp]),
    "qkrylov_tj_basis_create": (_vp, [_i, _vp]),
    "qkrylov_basis_destroy": (None, [_vp]),
    "qkrylov_basis_dimension": (_u64, [_vp]),
    "qkrylov_basis_nsites": (_i, [_vp]),
    "qkrylov_basis_state": (_u64, [_vp, _u64]),
    "qkrylov_basis_index": (_i64, [_vp, _u64]),
    "qkrylov_basis_contains": (_i, [_vp, _u64]),
    "qkrylov_spinhalf_site_create": (_vp, []),
    "qkrylov_fermion_site_create": (_vp, []),
    "qkrylov_hubbard_site_create": (_vp, []),
    "qkrylov_tj_site_create": (_vp, []),
    "qkrylov_site_destroy": (None, [_vp]),
    "qkrylov_opsum_create": (_vp, []),
    "qkrylov_opsum_destroy": (None, [_vp]),
    "qkrylov_opsum_clear": (_i, [_vp]),
    "qkrylov_opsum_add_term_1body": (_i, [_vp, _f, _f, _c.c_char_p, _i]),
    "qkrylov_opsum_add_term_2body": (_i, [_vp, _f, _f, _c.c_char_p, _i, _c.c_char_p, _i]),
    "qkrylov_opsum_add_term_nbody": (_i, [_vp, _f, _f, _i, _c.POINTER(_c.c_char_p), _ip]),
    "qkrylov_opsum_add_term_nbody_f64": (_i, [_vp, _d, _d, _i, _c.POINTER(_c.c_char_p), _ip]),
    "qkrylov_hamiltonian_create": (_vp, [_vp, _vp, _vp]),
    "qkrylov_hamiltonian_destroy": (None, [_vp]),
    "qkrylov_hamiltonian_dimension": (_u64, [_vp]),
    "qkrylov_hamiltonian_apply": (_i, [_vp, _fp, _fp, _fp, _fp]),
    "qkrylov_hamiltonian_apply_complex": (_i, [_vp, _fp, _fp]),
    "qkrylov_hamiltonian_diagonal": (_i, [_vp, _fp]),
    "qkrylov_lanczos_ground_state": (_i, [_vp, _i, _f, _c.POINTER(LanczosResultC)]),
    "qkrylov_lanczos_ground_state_complex": (_i, [_vp, _i, _f, _c.POINTER(LanczosResultC), _fp]),
    "qkrylov_davidson_lowest_complex": (_i, [_vp, _i, _i, _f, _fp, _fp, _c.POINTER(DavidsonResultC)]),
    "qkrylov_continued_fraction_coeffs_complex": (_i, [_vp, _fp, _i, _fp, _fp, _fp, _ip]),
    "qkrylov_evaluate_spectral_function": (_f, [_fp, _fp, _sz, _f, _f, _f, _f]),
    "qkrylov_ftlm": (_i, [_vp, _f, _i, _i, _c.POINTER(FTLMResultC)]),
    "qkrylov_hamiltonian_apply_complex_f64": (_i, [_vp, _dp, _dp]),
    "qkrylov_hamiltonian_diagonal_f64": (_i, [_vp, _dp]),
    "qkrylov_hamiltonian_apply_device_f64": (_i, [_vp, _vp, _vp, _vp]),
    "qkrylov_hamiltonian_apply_device_f32": (_i, [_vp, _vp, _vp, _vp]),
    "qkrylov_lanczos_ground_state_f64": (_i, [_vp, _i, _d, _dp, _c.POINTER(LanczosResultF64), _dp]),
    "qkrylov_lanczos_ground_state_mixed": (_i, [_vp, _i, _d, _dp, _c.POINTER(LanczosResultF64), _dp]),
    "qkrylov_lanczos_fixed_steps": (_i, [_vp, _i, _u64, _i, _dp, _c.POINTER(LanczosResultF64), _dp]),
    "qkrylov_kernel_launches": (_u64, []),
    "qkrylov_device_wait_timeouts": (_i, [_c.POINTER(_c.c_uint32)]),
    "qkrylov_debug_inject_alloc_failure": (_i, [_c.c_int64]),
    "qkrylov_vector_mdot_device_f32": (_i, [_c.POINTER(_c.c_void_p), _i, _c.POINTER(_c.c_void_p), _i, _c.c_uint64, _i,
                                            _dp, _vp]),
    "qkrylov_vector_mcombine_device_f32": (_i, [_c.POINTER(_c.c_void_p), _i, _dp, _c.POINTER(_c.c_void_p), _i,
                                                _c.c_uint64, _i, _vp]),
    "qkrylov_set_projection_kernel": (_i, [_i]),
    "qkrylov_lanczos_ritz_values": (_i, [_vp, _i, _c.c_uint64, _i, _i, _dp, _ip, _ip]),
    "qkrylov_debug_live_allocations": (_c.c_int64, []),
    "qkrylov_debug_device_wait_probe": (_i, [_c.c_int64]),
    "qkrylov_vector_dot_device_f64": (_i, [_vp, _vp, _u64, _dp, _vp]),
    "qkrylov_vector_dot_device_f32": (_i, [_vp, _vp, _u64, _dp, _vp]),
    "qkrylov_vector_dot_device_f64_noalloc": (_i, [_vp, _vp, _u64, _dp, _vp]),
    "qkrylov_set_device": (_i, [_i]),
    "qkrylov_device_count": (_i, [_ip]),
    "qkrylov_device_synchronize": (_i, []),
    "qkrylov_davidson_lowest_complex_f64": (_i, [_vp, _i, _i, _d, _dp, _dp, _c.POINTER(DavidsonResultC)]),
    "qkrylov_continued_fraction_coeffs_complex_f64": (_i, [_vp, _dp, _i, _dp, _dp, _dp, _ip, _ip]),
    "qkrylov_evaluate_spectral_function_f64": (_d, [_dp, _dp, _sz, _d, _d, _d, _d]),
    "qkrylov_evaluate_spectral_grid_f64": (_i, [_dp, _dp, _sz, _d, _dp, _sz, _d, _d, _dp]),
    "qkrylov_ftlm_f64": (_i, [_vp, _d, _i, _i, _c.POINTER(FTLMResultF64)]),
    "qkrylov_ftlm_multi_beta_f64": (_i, [_vp, _dp, _i, _i, _i, _dp, _dp, _dp, _dp]),
    "qkrylov_hamiltonian_info": (_i, [_vp, _ip, _ip, _ip, _ip, _ip]),
    "qkrylov_hamiltonian_entries": (_i, [_vp, _u64p, _u64p, _u64p, _dp]),
    "qkrylov_hamiltonian_select_kernel": (_i, [_vp, _i, _ip]),
    "qkrylov_hamiltonian_tuning": (_i, [_vp, _i, _ip, _dp]),
    "qkrylov_hamiltonian_tuning_ex": (_i, [_vp, _i, _ip, _dp, _i]),
    "qkrylov_basis_states": (_i, [_vp, _u64, _u64, _u64p]),
    "qkrylov_davidson_lowest_ex": (_i, [_vp, _i, _i, _d, _i, _i, _dp, _dp, _dp, _vp, _dp]),
    "qkrylov_hamiltonian_benchmark_apply": (_i, [_vp, _i, _i, _dp]),
    "qkrylov_hamiltonian_workspace": (_i, [_vp, _i, _u64p]),
}

_lib = None


def lib():
    """The loaded C-ABI library (ctypes.CDLL) with argument types declared."""
    global _lib
    if _lib is None:
        if not _os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m qkrylov_gb300.build`")
        L = _c.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class QKrylovError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"qkrylov error {code}: {msg}")
        self.code = code


def _check(rc):
    if rc != SUCCESS:
        raise QKrylovError(rc, (lib().qkrylov_last_error() or b"").decode())
    return rc


def _dptr(a):
    return a.ctypes.data_as(_dp)


def _fptr(a):
    return a.ctypes.data_as(_fp)


def _cvec(x, n, dtype=_np.complex128):
    x = _np.ascontiguousarray(x, dtype=dtype)
    if x.ndim != 1 or x.shape[0] != n:
        raise ValueError(f"vector of length {n} expected, got shape {x.shape}")
    return x


# ------------------------------------------------------------------ model objects
class _Handle:
    _destroy = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            getattr(_lib, self._destroy)(h)
            self._h = None


class Sector(_Handle):
    """Quantum-number sector (include/qkrylov/symmetry/sector.hpp:10-41)."""
    _destroy = "qkrylov_sector_destroy"

    def __init__(self, sz2=None, nup=None, ndn=None, n=None, nb=None):
        self._q = {k: v for k, v in (("sz2", sz2), ("nup", nup), ("ndn", ndn), ("n", n), ("nb", nb)) if v is not None}
        self._h = lib().qkrylov_sector_create()
        if sz2 is not None:
            _check(lib().qkrylov_sector_set_sz(self._h, int(sz2)))
        if nup is not None and ndn is not None:
            _check(lib().qkrylov_sector_set_hubbard_particles(self._h, int(nup), int(ndn)))
        elif nup is not None:
            _check(lib().qkrylov_sector_set_nup(self._h, int(nup)))
        elif ndn is not None:
            _check(lib().qkrylov_sector_set_ndn(self._h, int(ndn)))
        if n is not None:
            _check(lib().qkrylov_sector_set_n(self._h, int(n)))
        if nb is not None:
            _check(lib().qkrylov_sector_set_nb(self._h, int(nb)))

    def describe(self):
        """The quantum numbers set on this sector (e.g. {"sz2": 0})."""
        return dict(self._q)


class Basis(_Handle):
    _destroy = "qkrylov_basis_destroy"
    _create = None

    @property
    def sector(self):
        return self._sector

    def __init__(self, N, sector=None):
        self._sector = sector
        self._h = getattr(lib(), self._create)(int(N), sector._h if sector else None)
        if not self._h:
            raise ValueError((lib().qkrylov_last_error() or b"").decode())

    @property
    def size(self):
        return int(lib().qkrylov_basis_dimension(self._h))

    @property
    def nsites(self):
        return int(lib().qkrylov_basis_nsites(self._h))

    def state(self, i):
        return int(lib().qkrylov_basis_state(self._h, int(i)))

    def index(self, s):
        return int(lib().qkrylov_basis_index(self._h, int(s)))

    def contains(self, s):
        return bool(lib().qkrylov_basis_contains(self._h, int(s)))

    def states(self, first=0, count=None):
        """States (reference order and bit encoding) as a uint64 array."""
        n = self.size - first if count is None else int(count)
        out = _np.zeros(max(0, n), dtype=_np.uint64)
        _check(lib().qkrylov_basis_states(self._h, int(first), out.size, out.ctypes.data_as(_u64p)))
        return out


# The basis constructors take the reference facade's arguments
# (bindings/python/qkrylov/basis.py:64-190).  ``dtype`` is accepted and unused:
# bases are host tables here, and the arithmetic type is the Hamiltonian's.
class SpinHalfBasis(Basis):
    """Spin-1/2 chain; ``sz`` is the total Sz (the sector stores 2*Sz).  An
    explicit ``sz`` conserves Sz; ``conserve_sz`` alone selects Sz = 0."""
    _create = "qkrylov_spinhalf_basis_create"

    def __init__(self, N, conserve_sz=False, sz=None, dtype=None):
        if sz is not None or conserve_sz:
            super().__init__(N, Sector(sz2=int(round(2 * (sz or 0)))))
        else:
            super().__init__(N)


class FermionBasis(Basis):
    """Spinless fermions; a nonzero ``n`` (or ``conserve_n``) fixes the particle number."""
    _create = "qkrylov_fermion_basis_create"

    def __init__(self, N, conserve_n=False, n=0, dtype=None):
        if n or conserve_n:
            super().__init__(N, Sector(n=int(n)))
        else:
            super().__init__(N)


class HubbardBasis(Basis):
    """Spin-1/2 electrons; a nonzero ``nup`` / ``ndn`` (or the conserve flag)
    fixes that species' number, each independently."""
    _create = "qkrylov_hubbard_basis_create"

    def __init__(self, N, conserve_nup=False, nup=0, conserve_ndn=False, ndn=0, dtype=None):
        up = int(nup) if (nup or conserve_nup) else None
        dn = int(ndn) if (ndn or conserve_ndn) else None
        super().__init__(N, Sector(nup=up, ndn=dn) if (up is not None or dn is not None) else None)


class TJBasis(HubbardBasis):
    """t-J model: the Hubbard basis without doubly occupied sites."""
    _create = "qkrylov_tj_basis_create"


class Site(_Handle):
    _destroy = "qkrylov_site_destroy"
    _create = None

    def __init__(self, dtype=None):  # dtype: the reference facade's argument, unused here
        self._h = getattr(lib(), self._create)()


class SpinHalfSite(Site):
    _create = "qkrylov_spinhalf_site_create"


class FermionSite(Site):
    _create = "qkrylov_fermion_site_create"


class HubbardSite(Site):
    _create = "qkrylov_hubbard_site_create"


class TJSite(Site):
    _create = "qkrylov_tj_site_create"


class OpSum(_Handle):
    """Ordered list of ``coeff * op(site) * op(site) ...`` terms
    (include/qkrylov/operators/opsum.hpp:13-48)."""
    _destroy = "qkrylov_opsum_destroy"

    def __init__(self, dtype=None):  # dtype: the reference facade's argument, unused here
        self._h = lib().qkrylov_opsum_create()
        self.terms = []

    def add_term(self, coeff, *ops_sites):
        """add_term(coeff, "Sz", 0, "Sz", 1, ...); an operator may also be an ``Op`` member."""
        if len(ops_sites) < 2 or len(ops_sites) % 2:
            raise ValueError("expected coeff followed by (op, site) pairs")
        ops = [o.value if isinstance(o, Op) else str(o) for o in ops_sites[0::2]]
        sites = [int(s) for s in ops_sites[1::2]]
        c = complex(coeff)
        arr = (_c.c_char_p * len(ops))(*[o.encode() for o in ops])
        sarr = (_c.c_int * len(sites))(*sites)
        _check(lib().qkrylov_opsum_add_term_nbody_f64(self._h, c.real, c.imag, len(ops), arr, sarr))
        self.terms.append((c, list(zip(ops, sites))))
        return self

    def __iadd__(self, term):
        if isinstance(term, tuple):
            if len(term) < 3 or len(term) % 2 == 0:
                raise ValueError("Term must be a tuple of (coeff, op1, site1, ...)")
            return self.add_term(*term)
        raise ValueError("Unsupported type for += on OpSum")

    def __len__(self):
        return len(self.terms)

    @property
    def size(self):
        """Number of terms (the reference facade's OpSum.size)."""
        return len(self.terms)

    def clear(self):
        _check(lib().qkrylov_opsum_clear(self._h))
        self.terms = []


class MatrixFreeHamiltonian(_Handle):
    """y = H x on the GPU (include/qkrylov/hamiltonian/matrix_free_hamiltonian.hpp:24-77)."""
    _destroy = "qkrylov_hamiltonian_destroy"

    def __init__(self, basis, site, ops, device="cuda", dtype=_np.float64):
        """``device`` and ``dtype`` are the reference facade's arguments
        (bindings/python/qkrylov/hamiltonian.py:25-76).  Every Hamiltonian here
        lives on a CUDA device: "cuda:N" / "gpu:N" select GPU N (the reference's
        Device(id)), "cuda", "gpu" and "cpu" use the current one.  ``dtype``
        np.float64 makes ``apply`` return complex128, np.float32 complex64
        (computed in FP64 and rounded, as the float C ABI does)."""
        self.basis, self.site, self.ops = basis, site, ops
        self.device = str(device)
        self.dtype = _np.float32 if dtype in (_np.float32, "float32") else _np.float64
        d = self.device.lower()
        if ":" in d and (d.startswith("cuda") or d.startswith("gpu")):
            set_device(int(d.split(":", 1)[1]))
        elif d not in ("cuda", "gpu", "cpu"):
            raise ValueError(f"unknown device {device!r}: expected 'cuda[:N]', 'gpu[:N]' or 'cpu'")
        self._h = lib().qkrylov_hamiltonian_create(basis._h, site._h, ops._h)
        if not self._h:
            raise ValueError((lib().qkrylov_last_error() or b"").decode() or "hamiltonian creation failed")

    def to(self, device=None, dtype=None):
        """A new Hamiltonian of the same basis, site and terms on ``device`` with ``dtype``."""
        return MatrixFreeHamiltonian(self.basis, self.site, self.ops, device=self.device if device is None else device,
                                     dtype=self.dtype if dtype is None else dtype)

    @property
    def dimension(self):
        return int(lib().qkrylov_hamiltonian_dimension(self._h))

    def apply(self, x):
        """y = H x.  Host arrays (NumPy, complex128) go through host memory;
        a CUDA tensor (torch, complex128 or complex64, contiguous, on this
        device) is applied in place on the device without host copies, on the
        tensor's current stream, and a tensor of the same type is returned."""
        if hasattr(x, "__cuda_array_interface__"):
            return self._apply_cuda(x)
        x = _cvec(x, self.dimension)
        y = _np.empty_like(x)
        _check(lib().qkrylov_hamiltonian_apply_complex_f64(self._h, _dptr(x.view(_np.float64)), _dptr(y.view(_np.float64))))
        return y.astype(_np.complex64) if self.dtype == _np.float32 else y

    def _apply_cuda(self, x):
        import torch
        if not isinstance(x, torch.Tensor):
            raise TypeError("device arrays other than torch tensors: use apply_device with raw pointers")
        if x.dtype not in (torch.complex128, torch.complex64):
            raise TypeError("device vectors must be complex128 or complex64")
        if x.dim() != 1 or x.numel() != self.dimension or not x.is_contiguous():
            raise ValueError(f"expected a contiguous vector of length {self.dimension}")
        y = torch.empty_like(x)
        stream = torch.cuda.current_stream(x.device).cuda_stream
        self.apply_device(x.data_ptr(), y.data_ptr(), stream=stream, fp32=x.dtype == torch.complex64)
        return y

    __matmul__ = apply

    def apply_device(self, x_ptr, y_ptr, stream=None, fp32=False):
        """Device pointers (reference order); queued on `stream`, not synchronised."""
        fn = lib().qkrylov_hamiltonian_apply_device_f32 if fp32 else lib().qkrylov_hamiltonian_apply_device_f64
        _check(fn(self._h, _c.c_void_p(x_ptr), _c.c_void_p(y_ptr), _c.c_void_p(stream or 0)))

    def diagonal(self):
        d = _np.empty(self.dimension, dtype=_np.float64)
        _check(lib().qkrylov_hamiltonian_diagonal_f64(self._h, _dptr(d)))
        return d

    def info(self):
        v = [_c.c_int() for _ in range(5)]
        _check(lib().qkrylov_hamiltonian_info(self._h, *[_c.byref(x) for x in v]))
        return dict(zip(["n_outer", "n_inner", "n_mixed", "n_diag", "diag_mode"], [x.value for x in v]))

    def select_kernel(self, generic=False, mode=None):
        """Force the generic SpMV kernel (True) or allow the fast one (False).
        mode picks a kernel directly: 0 autotuned, 1 generic, 2 fast with one
        row per thread, 3 fast with shared-memory staging, 4 fast with four
        rows per thread, 5 four rows per thread staged, 6 four rows per thread
        with a larger register budget, 7 / 8 / 9 the tiled kernel over 1 / 2 /
        4 outer blocks per CTA, 10 the class-persistent kernel.
        Returns whether the fast kernel is in use."""
        m = int(mode) if mode is not None else int(bool(generic))
        f = _c.c_int()
        _check(lib().qkrylov_hamiltonian_select_kernel(self._h, m, _c.byref(f)))
        return bool(f.value)

    def workspace_bytes(self, release=False):
        """Device memory kept for the next solver call (the mixed Lanczos
        Krylov space); release=True frees it first."""
        b = _c.c_uint64()
        _check(lib().qkrylov_hamiltonian_workspace(self._h, int(bool(release)), _c.byref(b)))
        return b.value

    def tuning(self, fp32=True):
        """(variant, {variant: autotuned ms}) of the fast kernel used in mode 0;
        variant names: "row", "staged", "rows4", "rows4_staged", "rows4_wide",
        "tile1", "tile2", "tile4", "class" ("generic" when it does not apply)."""
        v = _c.c_int()
        names = ["row", "staged", "rows4", "rows4_staged", "rows4_wide", "tile1", "tile2", "tile4", "class"]
        ms = (_c.c_double * len(names))()
        _check(lib().qkrylov_hamiltonian_tuning_ex(self._h, int(bool(fp32)), _c.byref(v), ms, len(names)))
        return ("generic" if v.value < 0 else names[v.value]), {names[i]: ms[i] for i in range(len(names))}

    def benchmark_apply(self, fp32=True, reps=10):
        """Mean CUDA-event duration (ms) of one apply of the selected kernel."""
        ms = _c.c_double()
        _check(lib().qkrylov_hamiltonian_benchmark_apply(self._h, int(bool(fp32)), int(reps), _c.byref(ms)))
        return ms.value

    def entries(self):
        """(row_offsets, cols, vals) of every generated entry, reference order."""
        nnz = _c.c_uint64()
        _check(lib().qkrylov_hamiltonian_entries(self._h, _c.byref(nnz), None, None, None))
        n = self.dimension
        ro = _np.zeros(n + 1, dtype=_np.uint64)
        cols = _np.zeros(max(1, nnz.value), dtype=_np.uint64)
        vals = _np.zeros(2 * max(1, nnz.value), dtype=_np.float64)
        _check(lib().qkrylov_hamiltonian_entries(self._h, _c.byref(nnz), ro.ctypes.data_as(_u64p),
                                                 cols.ctypes.data_as(_u64p), _dptr(vals)))
        return ro, cols[: nnz.value], vals[: 2 * nnz.value].view(_np.complex128)

    def to_sparse(self):
        import scipy.sparse as sp
        ro, cols, vals = self.entries()
        n = self.dimension
        return sp.csr_matrix((vals, cols.astype(_np.int64), ro.astype(_np.int64)), shape=(n, n))

    def aslinearoperator(self):
        import scipy.sparse.linalg as sla
        n = self.dimension
        return sla.LinearOperator(shape=(n, n), matvec=self.apply, dtype=_np.complex128)

    def __repr__(self):
        return f"MatrixFreeHamiltonian(dim={self.dimension})"


# ------------------------------------------------------------------ solvers
class LanczosResult:
    def __init__(self, energy, eigenvector=None, iterations=0, converged=False, residual=None, energy_tridiag=None,
                 raw=None):
        self.energy, self.eigenvector = energy, eigenvector
        self.iterations, self.converged = iterations, converged
        self.residual, self.energy_tridiag, self.raw = residual, energy_tridiag, raw

    def __repr__(self):
        return f"LanczosResult(energy={self.energy:.10f})"


def lanczos_ground_state(H, maxiter=200, tol=1e-12, v0=None, mixed=False, return_state=True):
    """Ground state by Lanczos.  ``mixed=False`` is the reference algorithm in
    FP64 (src/solvers/lanczos.cpp:101-202); ``mixed=True`` is the FP32-vector
    form with FP64 refinement."""
    n = H.dimension
    r = LanczosResultF64()
    ev = _np.empty(n, dtype=_np.complex128) if return_state else None
    v0p = _dptr(_cvec(v0, n).view(_np.float64)) if v0 is not None else None
    fn = lib().qkrylov_lanczos_ground_state_mixed if mixed else lib().qkrylov_lanczos_ground_state_f64
    _check(fn(H._h, int(maxiter), float(tol), v0p, _c.byref(r), _dptr(ev.view(_np.float64)) if return_state else None))
    return LanczosResult(r.energy, ev, r.iterations, bool(r.converged), r.residual if r.residual >= 0 else None,
                         r.energy_tridiag, r)


def lanczos_fixed_steps(H, n_steps, seed=0, mixed=True, v0=None, eigenvector_out=None, selective=False):
    """Exactly n_steps Lanczos steps (performance form).  v0 / eigenvector_out
    are optional host arrays (complex128, reference order).  mixed=False,
    selective=True: FP64 with the mixed form's selective reorthogonalisation."""
    r = LanczosResultF64()
    n = H.dimension
    v0p = _dptr(_cvec(v0, n).view(_np.float64)) if v0 is not None else None
    evp = _dptr(eigenvector_out.view(_np.float64)) if eigenvector_out is not None else None
    m = 1 if mixed else (2 if selective else 0)
    _check(lib().qkrylov_lanczos_fixed_steps(H._h, int(n_steps), int(seed), m, v0p, _c.byref(r), evp))
    return r


def lanczos_ritz_values(H, n_steps, n_values, seed=0, mixed=True, selective=False):
    """Lowest n_values Ritz values of the tridiagonal after n_steps Lanczos
    steps from a seeded Philox start (the run of lanczos_fixed_steps), and the
    number of converged Ritz vectors selective reorthogonalisation held."""
    vals = _np.zeros(int(n_values))
    m, locked = _c.c_int(), _c.c_int()
    mode = 1 if mixed else (2 if selective else 0)
    _check(lib().qkrylov_lanczos_ritz_values(H._h, int(n_steps), int(seed), mode, int(n_values), _dptr(vals),
                                             _c.byref(m), _c.byref(locked)))
    return vals[:m.value], int(locked.value)


def kernel_launches():
    return int(lib().qkrylov_kernel_launches())


def device_wait_timeouts():
    """Bounded device-side waits that gave up on the current GPU (0 when every
    staged SpMV received its asynchronous copy)."""
    c = _c.c_uint32()
    rc = lib().qkrylov_device_wait_timeouts(_c.byref(c))
    if rc not in (0, -4):
        _check(rc)
    return int(c.value)


def set_projection_kernel(method):
    """Kernel of the solvers' FP32 projections: "fast" (CUDA cores, FP32 sums
    over runs of 32 elements folded into float-float sums; the default),
    "cuda" (compensated CUDA-core, FP64-accurate) or "tensor" (tcgen05 tensor
    cores, 3xTF32)."""
    _check(lib().qkrylov_set_projection_kernel({"cuda": 0, "tensor": 1, "fast": 2}[method]))


def set_device(device_id):
    _check(lib().qkrylov_set_device(int(device_id)))


def gpu_count():
    """Visible CUDA devices (the reference facade's gpu_count)."""
    c = _c.c_int()
    _check(lib().qkrylov_device_count(_c.byref(c)))
    return int(c.value)


def find_gpu():
    """"cuda" when a GPU is visible, else None (the reference facade's find_gpu)."""
    return "cuda" if gpu_count() > 0 else None


class Device:
    """The reference's Device (include/qkrylov/core/device.hpp:27-84):
    Device(id) or Device("cuda:1") names a GPU; select() makes it current for
    Hamiltonians created afterwards."""

    def __init__(self, spec=0):
        if isinstance(spec, str):
            s = spec.lower()
            self.id = int(s.split(":", 1)[1]) if ":" in s else 0
        else:
            self.id = int(spec)

    def select(self):
        set_device(self.id)
        return self

    @staticmethod
    def is_gpu_build():
        return True

    @staticmethod
    def backend_name():
        return "cuda"

    @staticmethod
    def gpu_count():
        return gpu_count()


__version__ = "0.1.0"


def synchronize():
    _check(lib().qkrylov_device_synchronize())


class DavidsonResult:
    def __init__(self, eigenvalues, eigenvectors, iterations=0, converged=False):
        self.eigenvalues, self.eigenvectors = eigenvalues, eigenvectors
        self.iterations, self.converged = iterations, converged

    def __repr__(self):
        return f"DavidsonResult(energies={self.eigenvalues})"


def davidson_lowest_ex(H, n_eig=1, max_subspace=20, tol=1e-8, mixed=False, return_vectors=False, max_iter=100):
    """Davidson (davidson.cpp:86-227) in the FP64 form or the mixed form (FP32
    vectors and SpMV, FP32 projections summed in runs and folded in float-float,
    FP64-refined Ritz pairs).
    Returns a DavidsonResult with ``residuals`` and ``seconds`` set."""
    n = H.dimension
    k = min(int(n_eig), n)
    ev = _np.zeros(max(1, int(n_eig)))
    res = _np.zeros(max(1, int(n_eig)))
    vecs = _np.zeros((max(1, k), n), dtype=_np.complex128) if return_vectors else None
    info = DavidsonResultC()
    sec = _c.c_double()
    _check(lib().qkrylov_davidson_lowest_ex(H._h, int(n_eig), int(max_subspace), float(tol), int(bool(mixed)),
                                            int(max_iter), _dptr(ev), _dptr(vecs.view(_np.float64)) if return_vectors else None,
                                            _dptr(res), _c.byref(info), _c.byref(sec)))
    r = DavidsonResult(ev[:k], list(vecs[:k]) if return_vectors else None, info.iterations, bool(info.converged))
    r.residuals, r.seconds = res[:k], sec.value
    return r


def davidson_lowest(H, n_eig=1, max_subspace=20, tol=1e-8, return_vectors=True):
    n = H.dimension
    k = min(int(n_eig), n)
    ev = _np.zeros(max(1, int(n_eig)))
    vecs = _np.zeros((max(1, k), n), dtype=_np.complex128) if return_vectors else None
    info = DavidsonResultC()
    _check(lib().qkrylov_davidson_lowest_complex_f64(H._h, int(n_eig), int(max_subspace), float(tol), _dptr(ev),
                                                     _dptr(vecs.view(_np.float64)) if return_vectors else None,
                                                     _c.byref(info)))
    return DavidsonResult(ev[:k], list(vecs[:k]) if return_vectors else None, info.iterations, bool(info.converged))


class DynamicsResult:
    def __init__(self, alphas, betas, norm_phi0):
        self.alphas, self.betas, self.norm_phi0 = alphas, betas, norm_phi0


def continued_fraction_coeffs(H, phi0, n_iter=100):
    n = H.dimension
    p = _cvec(phi0, n)
    a = _np.zeros(n_iter)
    b = _np.zeros(n_iter)
    nrm = _c.c_double()
    na = _c.c_int()
    nb = _c.c_int()
    _check(lib().qkrylov_continued_fraction_coeffs_complex_f64(H._h, _dptr(p.view(_np.float64)), int(n_iter), _dptr(a),
                                                               _dptr(b), _c.byref(nrm), _c.byref(na), _c.byref(nb)))
    return DynamicsResult(a[: na.value], b[: nb.value], nrm.value)


def evaluate_spectral_function(res, omega, E0, eta=0.1):
    a = _np.ascontiguousarray(res.alphas, dtype=_np.float64)
    b = _np.ascontiguousarray(res.betas, dtype=_np.float64)
    if b.size < max(1, a.size):
        b = _np.concatenate([b, _np.zeros(max(1, a.size) - b.size)])
    om = _np.atleast_1d(_np.asarray(omega, dtype=_np.float64))
    out = _np.zeros_like(om)
    _check(lib().qkrylov_evaluate_spectral_grid_f64(_dptr(a), _dptr(b), a.size, float(res.norm_phi0), _dptr(om), om.size,
                                                    float(E0), float(eta), _dptr(out)))
    return float(out[0]) if _np.ndim(omega) == 0 else out


class FTLMResult:
    def __init__(self, beta, partition_function, internal_energy, specific_heat, log_shift=None):
        self.beta, self.partition_function = beta, partition_function
        self.internal_energy, self.specific_heat, self.log_shift = internal_energy, specific_heat, log_shift


def ftlm(H, beta, n_random=50, n_steps=100, shifted=False):
    """FTLM with the reference's random vectors (src/solvers/ftlm.cpp:123-170).
    ``beta`` may be a scalar or an array (one run, many temperatures)."""
    b = _np.atleast_1d(_np.asarray(beta, dtype=_np.float64))
    Z, E, C = _np.zeros_like(b), _np.zeros_like(b), _np.zeros_like(b)
    ls = _np.zeros_like(b) if shifted else None
    _check(lib().qkrylov_ftlm_multi_beta_f64(H._h, _dptr(b), b.size, int(n_random), int(n_steps), _dptr(Z), _dptr(E),
                                             _dptr(C), _dptr(ls) if shifted else None))
    if _np.ndim(beta) == 0:
        return FTLMResult(float(b[0]), float(Z[0]), float(E[0]), float(C[0]), float(ls[0]) if shifted else None)
    return FTLMResult(b, Z, E, C, ls)


# ------------------------------------------------------------------ batched Lanczos
_STARTS = {"ftlm": START_FTLM_STREAM, "philox": START_PHILOX, "given": START_GIVEN, "ftlm32": START_FTLM_STREAM_F32}


def _stats(st):
    return {"seconds": st.seconds, "spmv_ms": st.spmv_ms, "vectors_per_lane": st.vectors_per_lane,
            "padded_vectors": st.padded_vectors, "rows": int(st.rows), "tune_ms": list(st.tune_ms)}


def _ham_array(hams):
    hams = list(hams)
    arr = (_c.c_void_p * len(hams))(*[h._h for h in hams])
    return hams, arr


class BlockTridiagResult:
    """Per vector i = h * n_vec + v: alphas[i], betas[i] (the recorded
    coefficients), norm2[i] (squared norm of its start vector); stats of the
    batched run (device seconds, block-SpMV time, tile shape)."""

    def __init__(self, alphas, betas, norm2, stats):
        self.alphas, self.betas, self.norm2, self.stats = alphas, betas, norm2, stats


def block_lanczos_tridiag(hams, n_vec, n_steps, mixed=True, start="ftlm", seed=0, start_vectors=None, vpl=0):
    """Three-term Lanczos (no reorthogonalisation, stop at beta < 1e-15) of
    n_vec vectors for each Hamiltonian in ``hams``, all advanced together by
    one block-SpMV launch per step.  ``start``: "ftlm" (the reference FTLM
    stream, mt19937(42) per Hamiltonian), "ftlm32" (its float variant),
    "philox" (device Gaussian vectors from ``seed``) or "given"
    (``start_vectors``: per Hamiltonian an (n_vec, dim) complex array).
    ``vpl``: block-SpMV vectors per lane (1, 2, 4; 0 = autotuned)."""
    hams, arr = _ham_array(hams)
    kind = _STARTS[start]
    buf = None
    if kind == START_GIVEN:
        parts = []
        for h, sv in zip(hams, start_vectors):
            a = _np.ascontiguousarray(sv, dtype=_np.complex128).reshape(n_vec, h.dimension)
            parts.append(a.ravel())
        buf = _np.ascontiguousarray(_np.concatenate(parts))
    nv = len(hams) * n_vec
    a = _np.zeros(nv * max(1, n_steps))
    b = _np.zeros(nv * max(1, n_steps))
    na = _np.zeros(nv, dtype=_np.int32)
    nb = _np.zeros(nv, dtype=_np.int32)
    n2 = _np.zeros(nv)
    st = BlockStatsC()
    _check(lib().qkrylov_block_lanczos_tridiag(arr, len(hams), int(n_vec), int(n_steps), int(bool(mixed)), int(vpl), kind,
                                               int(seed), _dptr(buf.view(_np.float64)) if buf is not None else None,
                                               _dptr(a), _dptr(b), na.ctypes.data_as(_ip), nb.ctypes.data_as(_ip),
                                               _dptr(n2), _c.byref(st)))
    a = a.reshape(nv, -1)
    b = b.reshape(nv, -1)
    return BlockTridiagResult([a[i, : na[i]].copy() for i in range(nv)], [b[i, : nb[i]].copy() for i in range(nv)],
                              n2, _stats(st))


def spectral_functions_block(H, phis, omegas, E0, eta=0.05, n_iter=100, mixed=True):
    """S_r(omega) (evaluate_spectral_function, dynamics.cpp:61-89) for several
    right-hand sides from one batched continued-fraction run; rows of zeros
    for zero right-hand sides.  Returns (S[r, omega], [DynamicsResult], stats)."""
    res, st = continued_fraction_block(H, phis, n_iter=n_iter, mixed=mixed)
    om = _np.atleast_1d(_np.asarray(omegas, dtype=_np.float64))
    S = _np.zeros((len(res), om.size))
    for i, r in enumerate(res):
        if len(r.alphas):
            S[i] = evaluate_spectral_function(r, om, E0, eta)
    return S, res, st


class FTLMSectorsResult:
    def __init__(self, beta, Z, E, Cv, log_shift, stats):
        self.beta, self.partition_function, self.internal_energy = beta, Z, E
        self.specific_heat, self.log_shift, self.stats = Cv, log_shift, stats


def ftlm_sectors(hams, beta, n_random=32, n_steps=100, mixed=True, start="ftlm", seed=0, shifted=False):
    """FTLM summed over several Hamiltonians (e.g. all Sz sectors), every
    sector's n_random vectors in one batched run: Z = sum of the per-sector
    reference estimates (ftlm.cpp:123-170), E and Cv of the combined ensemble."""
    hams, arr = _ham_array(hams)
    b = _np.atleast_1d(_np.asarray(beta, dtype=_np.float64))
    Z, E, C = _np.zeros_like(b), _np.zeros_like(b), _np.zeros_like(b)
    ls = _np.zeros_like(b) if shifted else None
    st = BlockStatsC()
    _check(lib().qkrylov_ftlm_sectors_f64(arr, len(hams), _dptr(b), b.size, int(n_random), int(n_steps),
                                          int(bool(mixed)), _STARTS[start], int(seed), _dptr(Z), _dptr(E), _dptr(C),
                                          _dptr(ls) if shifted else None, _c.byref(st)))
    return FTLMSectorsResult(b, Z, E, C, ls, _stats(st))


def continued_fraction_block(H, phi0s, n_iter=100, mixed=True):
    """continued_fraction_coeffs for several right-hand sides (<= 32) in one
    batched run; returns ([DynamicsResult per right-hand side], stats)."""
    n = H.dimension
    P = _np.ascontiguousarray(_np.asarray(phi0s, dtype=_np.complex128).reshape(-1, n))
    r = P.shape[0]
    a = _np.zeros(r * max(1, n_iter))
    b = _np.zeros(r * max(1, n_iter))
    na = _np.zeros(r, dtype=_np.int32)
    nb = _np.zeros(r, dtype=_np.int32)
    nr = _np.zeros(r)
    st = BlockStatsC()
    _check(lib().qkrylov_cf_block_f64(H._h, _dptr(P.view(_np.float64)), r, int(n_iter), int(bool(mixed)), _dptr(a),
                                      _dptr(b), na.ctypes.data_as(_ip), nb.ctypes.data_as(_ip), _dptr(nr),
                                      _c.byref(st)))
    a = a.reshape(r, -1)
    b = b.reshape(r, -1)
    return [DynamicsResult(a[i, : na[i]].copy(), b[i, : nb[i]].copy(), float(nr[i])) for i in range(r)], _stats(st)


# ------------------------------------------------------------------ expression sugar
# The reference facade's operator algebra (bindings/python/qkrylov/operators.py):
# Sz(0) * Sz(1) is a term, terms add into sums, numbers scale terms and sums,
# and ``OpSum += expression`` appends the terms in order.
class Op(str, _enum.Enum):
    """Operator names (the reference facade's ``Op``)."""
    Sz = "Sz"
    Sp = "Sp"
    Sm = "Sm"
    Sx = "Sx"
    Sy = "Sy"
    CdagUp = "CdagUp"
    CUp = "CUp"
    CdagDn = "CdagDn"
    CDn = "CDn"
    Nup = "Nup"
    Ndn = "Ndn"
    Nupdn = "Nupdn"
    Bdag = "Bdag"
    B = "B"
    N = "N"


class LocalOp:
    def __init__(self, name, site):
        self.name, self.site = name, site

    def __mul__(self, other):
        if isinstance(other, LocalOp):
            return Term(1.0, [self, other])
        if isinstance(other, Term):  # the operator stays on the left
            return Term(other.coeff, [self] + other.ops)
        if isinstance(other, (int, float, complex)):
            return Term(complex(other), [self])
        return NotImplemented

    def __rmul__(self, other):
        if isinstance(other, (int, float, complex)):
            return Term(complex(other), [self])
        return NotImplemented


class Term:
    def __init__(self, coeff, ops):
        self.coeff, self.ops = coeff, ops

    def __mul__(self, other):
        if isinstance(other, LocalOp):
            return Term(self.coeff, self.ops + [other])
        if isinstance(other, Term):
            return Term(self.coeff * other.coeff, self.ops + other.ops)
        if isinstance(other, (int, float, complex)):
            return Term(self.coeff * complex(other), self.ops)
        return NotImplemented

    def __rmul__(self, other):
        if isinstance(other, (int, float, complex)):
            return Term(self.coeff * complex(other), self.ops)
        return NotImplemented

    def __add__(self, other):
        return Expr([self]) + other

    def __sub__(self, other):
        return Expr([self]) - other


class Expr:
    def __init__(self, terms):
        self.terms = list(terms)

    def __add__(self, other):
        if isinstance(other, Term):
            return Expr(self.terms + [other])
        if isinstance(other, Expr):
            return Expr(self.terms + other.terms)
        return NotImplemented

    def __sub__(self, other):
        if isinstance(other, Term):
            return Expr(self.terms + [Term(-other.coeff, other.ops)])
        if isinstance(other, Expr):
            return Expr(self.terms + [Term(-t.coeff, t.ops) for t in other.terms])
        return NotImplemented

    def __mul__(self, other):
        if isinstance(other, (int, float, complex)):
            return Expr([t * other for t in self.terms])
        return NotImplemented

    __rmul__ = __mul__


def _opsum_iadd(self, x):
    if isinstance(x, Term):
        x = Expr([x])
    if isinstance(x, Expr):
        for t in x.terms:
            args = []
            for o in t.ops:
                args += [o.name, o.site]
            self.add_term(t.coeff, *args)
        return self
    return _tuple_iadd(self, x)


_tuple_iadd = OpSum.__iadd__
OpSum.__iadd__ = _opsum_iadd

for _name in ("Sz", "Sp", "Sm", "Sx", "Sy", "CdagUp", "CUp", "CdagDn", "CDn", "Nup", "Ndn", "Nupdn", "N", "C", "Cdag", "Id",
              "B", "Bdag"):
    globals()[_name] = (lambda nm: (lambda i: LocalOp(nm, i)))(_name)


from . import io  # noqa: E402  (eigenvector / tridiagonal files)
