"""Host logic of the sharded (one process per GPU) path: sector sharding and
the FTLM reduction across ranks, run as two gloo processes on the CPU with
the oracle's per-sector tridiagonals standing in for each rank's GPU run."""
import os
import socket
from math import comb

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import models as M
from oracle_ctypes import OHam, Oracle, available

from qkrylov_gb300.parallel import ftlm_combine, shard_units, tridiag_spectrum

L, R, MST = 8, 3, 12
BETAS = np.array([0.05, 0.5, 2.0, 20.0])


def sector_vectors(oracle, idx):
    sz2 = -L + 2 * idx
    h = OHam(oracle, M.SPIN, L, M.sector(sz2=sz2), M.heisenberg_terms(L, True))
    a, b, na, nb, nr = h.ftlm_tridiag(R, MST)
    return [(a[v, :na[v]], b[v, :nb[v]], nr[v] ** 2) for v in range(R)]


def _worker(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        oracle = Oracle("qko")
        sizes = [comb(L, k) for k in range(L + 1)]
        vecs = []
        for i in shard_units(sizes, world)[rank]:
            vecs += sector_vectors(oracle, i)
        Z, E, C, ls = ftlm_combine(vecs, BETAS, R)
        if rank == 0:
            np.save(out_path, np.stack([Z, E, C, ls]))
    finally:
        dist.destroy_process_group()


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_units_balance():
    sizes = [comb(24, k) for k in range(25)]
    for world in (1, 2, 3, 8):
        parts = shard_units(sizes, world)
        assert sorted(i for p in parts for i in p) == list(range(25))
        loads = [sum(sizes[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)
    assert shard_units(sizes, 2) == shard_units(sizes, 2)  # deterministic


def test_tridiag_spectrum_matches_oracle(oracle):
    rng = np.random.default_rng(1)
    a, b = rng.normal(size=9), np.abs(rng.normal(size=9))
    e, w = tridiag_spectrum(a, b)
    ev = np.zeros(9)
    fc = np.zeros(9)
    import ctypes as c
    oracle._f("tridiag_components")(a.ctypes.data_as(c.POINTER(c.c_double)), b.ctypes.data_as(c.POINTER(c.c_double)),
                                    9, ev.ctypes.data_as(c.POINTER(c.c_double)),
                                    fc.ctypes.data_as(c.POINTER(c.c_double)))
    order = np.argsort(ev)
    np.testing.assert_allclose(e, ev[order], atol=1e-12)
    np.testing.assert_allclose(w, fc[order] ** 2, atol=1e-12)


@pytest.mark.skipif(not available("qko"), reason="oracle not built")
def test_ftlm_two_ranks_gloo(oracle, tmp_path):
    out = str(tmp_path / "ftlm.npy")
    mp.start_processes(_worker, args=(2, free_port(), out), nprocs=2, start_method="spawn")
    Z2, E2, C2, ls2 = np.load(out)
    # one process, every sector
    vecs = []
    for i in range(L + 1):
        vecs += sector_vectors(oracle, i)
    Z1, E1, C1, ls1 = ftlm_combine(vecs, BETAS, R)
    np.testing.assert_allclose(Z2 * np.exp(ls2), Z1 * np.exp(ls1), rtol=1e-12)
    np.testing.assert_allclose(E2, E1, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(C2, C1, rtol=1e-10, atol=1e-10)
    # the sum of the oracle's own per-sector estimates (ftlm.cpp:151-167)
    parts = []
    for i in range(L + 1):
        h = OHam(oracle, M.SPIN, L, M.sector(sz2=-L + 2 * i), M.heisenberg_terms(L, True))
        parts.append(np.array([h.ftlm(b, R, MST) for b in BETAS]))
    Zs = sum(p[:, 0] for p in parts)
    Es = sum(p[:, 0] * p[:, 1] for p in parts) / Zs
    np.testing.assert_allclose(Z1 * np.exp(ls1), Zs, rtol=1e-10)
    np.testing.assert_allclose(E1, Es, rtol=1e-10, atol=1e-10)
