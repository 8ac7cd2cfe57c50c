"""Eigenvector and Krylov-state files.

The reference stores eigenvectors from Python with h5py
(examples/hdf5_storage.py:5-27); h5py is not available here, so states are
written as NumPy ``.npz`` archives with the same content: the vector in the
reference's basis order, its energy, and enough of the basis to check that a
file is loaded against the basis it was computed in (model, site count,
sector, dimension and a digest of the state list).  Lanczos / continued-
fraction coefficients are stored the same way, so S(omega) or FTLM
observables can be re-evaluated without repeating the Krylov run.
"""
import hashlib
import json

import numpy as np

FORMAT = "qkrylov-gb300-state-v1"


def basis_signature(basis):
    """Model, site count, sector, dimension and a SHA-256 of the first and last
    4096 states (reference order and bit encoding)."""
    n = basis.size
    head = basis.states(0, min(n, 4096))
    tail = basis.states(max(0, n - 4096), min(n, 4096))
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(head, dtype="<u8").tobytes())
    h.update(np.ascontiguousarray(tail, dtype="<u8").tobytes())
    sec = getattr(basis, "sector", None)
    return {"model": type(basis).__name__, "nsites": int(basis.nsites), "dim": int(n),
            "sector": sec.describe() if sec is not None and hasattr(sec, "describe") else None,
            "states_sha256": h.hexdigest()}


def _check(meta, basis):
    if basis is None:
        return
    sig = basis_signature(basis)
    for k in ("dim", "nsites", "states_sha256"):
        if meta.get(k) != sig[k]:
            raise ValueError(f"state file was written for another basis ({k}: {meta.get(k)} != {sig[k]})")


def save_eigenvector(path, vector, energy, basis, extra=None):
    """Write one (or several, shape (k, dim)) eigenvectors and energies."""
    v = np.asarray(vector, dtype=np.complex128)
    meta = dict(basis_signature(basis), format=FORMAT, kind="eigenvector", extra=extra or {})
    if v.shape[-1] != meta["dim"]:
        raise ValueError("vector length differs from the basis dimension")
    np.savez(path, vectors=np.atleast_2d(v), energies=np.atleast_1d(np.asarray(energy, dtype=np.float64)),
             meta=json.dumps(meta))


def load_eigenvector(path, basis=None):
    """(vectors[k, dim], energies[k], meta); checks the basis when given."""
    with np.load(path, allow_pickle=False) as f:
        meta = json.loads(str(f["meta"]))
        if meta.get("format") != FORMAT or meta.get("kind") != "eigenvector":
            raise ValueError("not an eigenvector file of this format")
        _check(meta, basis)
        return f["vectors"].copy(), f["energies"].copy(), meta


def save_tridiagonals(path, results, basis=None, extra=None):
    """Continued-fraction / Lanczos coefficients: a list of objects with
    ``alphas``, ``betas`` and ``norm_phi0`` (DynamicsResult) or
    ``(alphas, betas, norm)`` tuples."""
    rows = []
    for r in results:
        a, b, n = (r.alphas, r.betas, r.norm_phi0) if hasattr(r, "alphas") else r
        rows.append((np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64), float(n)))
    meta = dict(basis_signature(basis) if basis is not None else {}, format=FORMAT, kind="tridiagonals",
                extra=extra or {})
    arrays = {"meta": json.dumps(meta), "norms": np.array([r[2] for r in rows]),
              "n_alpha": np.array([r[0].size for r in rows], dtype=np.int64),
              "n_beta": np.array([r[1].size for r in rows], dtype=np.int64)}
    arrays["alphas"] = np.concatenate([r[0] for r in rows]) if rows else np.zeros(0)
    arrays["betas"] = np.concatenate([r[1] for r in rows]) if rows else np.zeros(0)
    np.savez(path, **arrays)


def load_tridiagonals(path, basis=None):
    """[(alphas, betas, norm)], meta."""
    with np.load(path, allow_pickle=False) as f:
        meta = json.loads(str(f["meta"]))
        if meta.get("format") != FORMAT or meta.get("kind") != "tridiagonals":
            raise ValueError("not a tridiagonal file of this format")
        if basis is not None and "dim" in meta:
            _check(meta, basis)
        out, ia, ib = [], 0, 0
        for na, nb, nr in zip(f["n_alpha"], f["n_beta"], f["norms"]):
            out.append((f["alphas"][ia:ia + na].copy(), f["betas"][ib:ib + nb].copy(), float(nr)))
            ia += na
            ib += nb
        return out, meta
