"""Independent units across ranks: FTLM sectors / random vectors and S(q)
right-hand sides need no exchange until the final host sums, so a
multi-process run shards the units (one GPU per rank) and reduces a handful
of scalars per temperature with torch.distributed (gloo or NCCL).

The per-vector quantities are the reference's (src/solvers/ftlm.cpp:123-170):
the tridiagonal (alpha, beta) of each start vector, its eigenvalues e_i and
squared first components w_i, and the squared norm |r|^2 of the start vector;
a sector contributes (1/R) sum_r |r|^2 sum_i w_i exp(-beta e_i) to Z.  With a
shift e_min common to all ranks the sums stay finite at low temperature.
"""
import numpy as np


def shard_units(weights, world_size):
    """Assign units (e.g. sectors, weight = rows) to ranks, heaviest first onto
    the least loaded rank.  Returns one sorted list of unit indices per rank."""
    loads = [0.0] * world_size
    out = [[] for _ in range(world_size)]
    for i in sorted(range(len(weights)), key=lambda j: (-float(weights[j]), j)):
        r = min(range(world_size), key=lambda q: (loads[q], q))
        out[r].append(i)
        loads[r] += float(weights[i])
    return [sorted(o) for o in out]


def tridiag_spectrum(alphas, betas):
    """Eigenvalues and squared first components of the symmetric tridiagonal
    with diagonal alphas and off-diagonal betas[:len(alphas) - 1]
    (ftlm.cpp:61-119 computes the same pairs by implicit QL)."""
    a = np.asarray(alphas, dtype=np.float64)
    n = a.size
    if n == 0:
        return np.zeros(0), np.zeros(0)
    T = np.diag(a)
    if n > 1:
        b = np.asarray(betas, dtype=np.float64)[: n - 1]
        T += np.diag(b, 1) + np.diag(b, -1)
    e, v = np.linalg.eigh(T)
    return e, v[0] ** 2


def ftlm_partial_sums(vectors, betas, shift):
    """sum over the given vectors of |r|^2 w_i e_i^p exp(-beta (e_i - shift)),
    p = 0, 1, 2, for every beta: array [3, n_beta]."""
    bs = np.asarray(betas, dtype=np.float64)
    out = np.zeros((3, bs.size))
    for alphas, bets, norm2 in vectors:
        e, w = tridiag_spectrum(alphas, bets)
        if e.size == 0:
            continue
        wt = norm2 * w[None, :] * np.exp(-bs[:, None] * (e[None, :] - shift))
        out[0] += wt.sum(axis=1)
        out[1] += (wt * e[None, :]).sum(axis=1)
        out[2] += (wt * e[None, :] ** 2).sum(axis=1)
    return out


def _min_eigenvalue(vectors):
    m = np.inf
    for alphas, bets, _ in vectors:
        e, _w = tridiag_spectrum(alphas, bets)
        if e.size:
            m = min(m, float(e.min()))
    return m


def ftlm_combine(local_vectors, betas, n_random, group=None):
    """Z, E, Cv and log_shift over every rank's vectors (Z is the sum of the
    per-sector estimates; the true partition function is Z * exp(log_shift)).
    local_vectors: [(alphas, betas, |r|^2)] of this rank; n_random: vectors per
    sector (the 1/R of each sector's estimate)."""
    emin = _min_eigenvalue(local_vectors)
    if group is not None or _dist_ready():
        import torch
        import torch.distributed as dist
        t = torch.tensor([emin], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MIN, group=group)
        emin = float(t.item())
    sums = ftlm_partial_sums(local_vectors, betas, emin)
    if group is not None or _dist_ready():
        import torch
        import torch.distributed as dist
        t = torch.from_numpy(sums.copy())
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        sums = t.numpy()
    bs = np.asarray(betas, dtype=np.float64)
    Z = sums[0] / n_random
    E = sums[1] / sums[0]
    Cv = bs ** 2 * (sums[2] / sums[0] - E ** 2)
    return Z, E, Cv, -bs * emin


def _dist_ready():
    try:
        import torch.distributed as dist
        return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1
    except Exception:
        return False


def ftlm_sectors_distributed(hams_for, weights, betas, n_random=32, n_steps=100, mixed=True, start="philox",
                             seed=0, group=None):
    """Batched FTLM over sectors sharded across the ranks of the default (or
    given) process group: this rank builds its sectors with
    ``hams_for(indices)`` and runs them as one block Lanczos on its GPU; the
    observables are reduced on the host.  ``start="philox"`` seeds each
    sector's vectors from ``seed`` and the sector index, so the result does not
    depend on the number of ranks."""
    import torch.distributed as dist
    import qkrylov_gb300 as qk
    world = dist.get_world_size(group) if (group is not None or _dist_ready()) else 1
    rank = dist.get_rank(group) if (group is not None or _dist_ready()) else 0
    mine = shard_units(weights, world)[rank]
    vectors = []
    for i in mine:  # one batch per sector keeps each sector's stream independent of the sharding
        (h,) = hams_for([i])
        r = qk.block_lanczos_tridiag([h], n_random, n_steps, mixed=mixed, start=start,
                                     seed=(int(seed) * 1000003 + i) & 0xFFFFFFFFFFFF)
        vectors += list(zip(r.alphas, r.betas, r.norm2))
    return ftlm_combine(vectors, betas, n_random, group)
