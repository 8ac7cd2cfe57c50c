"""Time the SpMV kernels on a chain model (also the commands the kernel
profiles are taken with).

    python -m qkrylov_gb300.timing --model heisenberg --L 28 --precision fp32 --mode 0 --reps 5
    python -m qkrylov_gb300.timing --L 22 --block 32 --steps 3 --vpl 4
    python -m qkrylov_gb300.timing --model hubbard --L 14 --davidson 4 --iters 14 [--projection tensor]

    python -m qkrylov_gb300.timing --peaks
    python -m qkrylov_gb300.timing --mdot 32 --nw 4 --n 50000000 --reps 20
    python -m qkrylov_gb300.timing --mcomb 32 --nw 4 --n 50000000 --reps 20
    python -m qkrylov_gb300.timing --L 28 --lanczos 8 [--mode 4]

The second form runs the batched Lanczos on every Sz sector of the chain (or
the Sz = 0 sector alone with ``--sz0-only``) with ``--block`` Philox start
vectors per sector and reports the block-SpMV time.  The third runs the
Davidson solver for the ``--davidson`` lowest states (subspace 32, mixed form
unless ``--precision fp64``) for ``--iters`` iterations, twice, and reports
the seconds per iteration of the second run.  ``--peaks`` compiles and runs
``peaks.cu`` (FP64/FP32 FMA rates, L2 and DRAM read bandwidth, scattered
8-byte reads from shared memory and L1) and prints its JSON line.  ``--mdot K``
times the projections <V_j, W_o> of K FP32 vectors against ``--nw`` others of
``--n`` complex elements (qkrylov_vector_mdot_device_f32) with the three
kernels (compensated CUDA-core, tcgen05, run-summed CUDA-core) and reports
microseconds per call and the algorithmic bandwidth (every vector read once).  ``--mcomb K``
times the combinations W_o = sum_j C_oj V_j of K FP32 vectors into ``--nw`` outputs
(qkrylov_vector_mcombine_device_f32, CUDA events, ``--reps`` calls).  ``--lanczos N``
runs N steps of the mixed Lanczos (qkrylov_lanczos_fixed_steps) on the
Heisenberg chain, twice, and reports the mean time of its SpMV launches, each
fused with the three-term recurrence (reads x and the previous Lanczos vector,
writes y): the Lanczos step's SpMV on a few vectors instead of the bench's 200.

Builds the Hamiltonian (Heisenberg chain ``Sz Sz + 0.5 (S+ S- + S- S+)`` per
bond, or Fermi-Hubbard chain ``-t c^dag c`` hopping per spin and direction plus
``U n_up n_dn``), periodic unless ``--obc``, in the Sz = 0 / half-filled
sector, then times ``reps`` back-to-back applies on internal device vectors
with CUDA events on the Hamiltonian's stream.  Prints one JSON line with the
mean launch time and the algorithmic bandwidth (read x once, write y once).
"""
import argparse
import json
import os
import subprocess
import time

import qkrylov_gb300 as qk


def heisenberg_chain(L, pbc=True, J=1.0, sz2=0):
    ops = qk.OpSum()
    for i in range(L if pbc else L - 1):
        j = (i + 1) % L
        ops.add_term(J, "Sz", i, "Sz", j)
        ops.add_term(0.5 * J, "Sp", i, "Sm", j)
        ops.add_term(0.5 * J, "Sm", i, "Sp", j)
    return qk.SpinHalfBasis(L, conserve_sz=True, sz=sz2 / 2), qk.SpinHalfSite(), ops


def hubbard_chain(L, pbc=True, t=1.0, U=4.0):
    ops = qk.OpSum()
    for i in range(L if pbc else L - 1):
        j = (i + 1) % L
        for s in ("Up", "Dn"):
            ops.add_term(-t, "Cdag" + s, i, "C" + s, j)
            ops.add_term(-t, "Cdag" + s, j, "C" + s, i)
    for i in range(L):
        ops.add_term(U, "Nupdn", i)
    return qk.HubbardBasis(L, nup=L // 2, ndn=L // 2), qk.HubbardSite(), ops


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--model", choices=["heisenberg", "hubbard"], default="heisenberg")
    p.add_argument("--L", type=int, default=28)
    p.add_argument("--obc", action="store_true")
    p.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    p.add_argument("--mode", type=int, default=0, help="0 autotuned, 1 generic, 2 fast, 3 fast staged, 4 fast rows4, 5 rows4 staged, 6 rows4 wide, 7/8/9 tiled over 1/2/4 blocks")
    p.add_argument("--reps", type=int, default=5)
    p.add_argument("--block", type=int, default=0, help="vectors per sector: batched Lanczos over all Sz sectors")
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--vpl", type=int, default=0, help="block SpMV vectors per lane (0: autotuned)")
    p.add_argument("--sz0-only", action="store_true", help="block mode on the Sz = 0 sector alone")
    p.add_argument("--davidson", type=int, default=0, help="states for a Davidson run (0: SpMV timing)")
    p.add_argument("--iters", type=int, default=14, help="Davidson iterations")
    p.add_argument("--peaks", action="store_true", help="FMA / L2 / DRAM / gather throughput probes")
    p.add_argument("--lanczos", type=int, default=0, help="mixed Lanczos steps (0: none)")
    p.add_argument("--mdot", type=int, default=0, help="vectors of a projection timing (0: none)")
    p.add_argument("--mcomb", type=int, default=0, help="vectors of a combination timing (0: none)")
    p.add_argument("--nw", type=int, default=4, help="right-hand vectors (outputs) of the projection (combination) timing")
    p.add_argument("--n", type=int, default=50_000_000, help="vector length of the projection timing")
    p.add_argument("--projection", choices=["cuda", "tensor", "fast"], default="fast",
                   help="kernel of the mixed Davidson's projections")
    a = p.parse_args()
    if a.peaks:
        return peaks()
    if a.block:
        return block(a)
    if a.davidson:
        return davidson(a)
    if a.mdot:
        return mdot(a)
    if a.mcomb:
        return mcomb(a)
    if a.lanczos:
        return lanczos(a)
    build = heisenberg_chain if a.model == "heisenberg" else hubbard_chain
    basis, site, ops = build(a.L, not a.obc)
    t0 = time.perf_counter()
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    tc = time.perf_counter() - t0
    fast = H.select_kernel(mode=a.mode)
    fp32 = a.precision == "fp32"
    ms = H.benchmark_apply(fp32=fp32, reps=a.reps)
    n = H.dimension
    e = 8 if fp32 else 16
    variant, tuned = H.tuning(fp32=fp32)
    print(json.dumps({"model": a.model, "L": a.L, "pbc": not a.obc, "dim": n, "precision": a.precision,
                      "mode": a.mode, "fast": fast, "ms": ms, "alg_GBs": 2 * n * e / ms / 1e6,
                      "construct_s": round(tc, 3), "autotuned": variant,
                      "tuned_ms": {k: round(v, 4) for k, v in tuned.items() if v}}), flush=True)


def peaks():
    from qkrylov_gb300 import build as b
    here = os.path.dirname(os.path.abspath(__file__))
    exe = os.path.join(b.BUILD, "peaks")
    os.makedirs(b.BUILD, exist_ok=True)
    subprocess.run([b._nvcc()] + b.ARCH + ["-O3", "-o", exe, os.path.join(here, "peaks.cu")], check=True)
    subprocess.run([exe], check=True)


def block(a):
    t0 = time.perf_counter()
    hams = []
    for sz2 in ([0] if a.sz0_only else range(-a.L, a.L + 1, 2)):
        hams.append(qk.MatrixFreeHamiltonian(*heisenberg_chain(a.L, not a.obc, sz2=sz2)))
    tc = time.perf_counter() - t0
    mixed = a.precision == "fp32"
    r = qk.block_lanczos_tridiag(hams, a.block, a.steps, mixed=mixed, start="philox", seed=1, vpl=a.vpl)
    st = r.stats
    e = 8 if mixed else 16
    print(json.dumps({"model": "heisenberg", "L": a.L, "sectors": len(hams), "rows": st["rows"],
                      "vectors_per_sector": a.block, "steps": a.steps, "precision": a.precision,
                      "vectors_per_lane": st["vectors_per_lane"], "spmv_ms": st["spmv_ms"],
                      "spmv_alg_GBs": 2 * st["rows"] * st["padded_vectors"] * e / st["spmv_ms"] / 1e6,
                      "loop_s": st["seconds"], "tune_ms": st["tune_ms"], "construct_s": round(tc, 3)}), flush=True)


def davidson(a):
    build = heisenberg_chain if a.model == "heisenberg" else hubbard_chain
    H = qk.MatrixFreeHamiltonian(*build(a.L, not a.obc))
    mixed = a.precision == "fp32"
    qk.set_projection_kernel(a.projection)
    for _ in range(2):  # the second run is timed (the first pays the one-time costs)
        r = qk.davidson_lowest_ex(H, n_eig=a.davidson, max_subspace=32, tol=1e-8, mixed=mixed, max_iter=a.iters)
    print(json.dumps({"model": a.model, "L": a.L, "dim": H.dimension, "states": a.davidson, "precision": a.precision,
                      "projection": a.projection, "iterations": r.iterations, "s_per_iteration": r.seconds / max(1, r.iterations),
                      "eigenvalues": [float(e) for e in r.eigenvalues],
                      "residuals": [float(e) for e in r.residuals]}), flush=True)


def lanczos(a):
    H = qk.MatrixFreeHamiltonian(*heisenberg_chain(a.L, not a.obc))
    if a.mode:  # a fixed variant (a profiler's slow-down can change the autotuner's choice)
        H.select_kernel(mode=a.mode)
    for _ in range(2):  # the second run is reported
        r = qk.lanczos_fixed_steps(H, a.lanczos, seed=1, mixed=True)
    n = H.dimension
    ms = 1e3 * r.seconds_spmv / max(1, r.spmv_calls)
    variant, _ = H.tuning(fp32=True)
    print(json.dumps({"model": "heisenberg", "L": a.L, "dim": n, "steps": a.lanczos, "spmv_calls": r.spmv_calls,
                      "spmv_ms": ms, "alg_bytes_per_launch": 3 * n * 8, "alg_GBs": 3 * n * 8 / ms / 1e6,
                      "variant": variant, "energy": r.energy}), flush=True)


def mdot(a):
    import ctypes
    import torch
    k, nw, n = a.mdot, a.nw, a.n
    g = torch.Generator(device="cuda").manual_seed(1)
    V = [torch.randn(n, dtype=torch.complex64, device="cuda", generator=g) for _ in range(k)]
    W = [torch.randn(n, dtype=torch.complex64, device="cuda", generator=g) for _ in range(nw)]
    va = (ctypes.c_void_p * k)(*[v.data_ptr() for v in V])
    wa = (ctypes.c_void_p * nw)(*[w.data_ptr() for w in W])
    out = (ctypes.c_double * (2 * k * nw))()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    res = {"k": k, "nw": nw, "n": n, "bytes_per_call": (k + nw) * n * 8}
    vals = {}
    for name, method in (("cuda", 0), ("tensor", 1), ("fast", 2)):
        call = lambda: qk.lib().qkrylov_vector_mdot_device_f32(va, k, wa, nw, n, method, out, stream)
        if call() != 0:  # a shape the kernel does not take (the tensor kernel: k <= 128)
            res[name + "_us"] = None
            continue
        for _ in range(2):
            assert call() == 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.reps):
            call()  # returns after the result is on the host
        t = (time.perf_counter() - t0) / a.reps
        vals[name] = list(out)
        res[name + "_us"] = round(t * 1e6, 1)
        res[name + "_GBs"] = round(res["bytes_per_call"] / t / 1e9, 1)
    big = max(map(abs, vals["cuda"]))
    for name in ("tensor", "fast"):
        if name in vals:
            res[name + "_max_rel_diff"] = max(abs(x - y) for x, y in zip(vals["cuda"], vals[name])) / big
    print(json.dumps(res), flush=True)


def mcomb(a):
    """W_o = sum_j C_oj V_j (qkrylov_vector_mcombine_device_f32), CUDA-event timed."""
    import ctypes
    import torch
    k, nw, n = a.mcomb, a.nw, a.n
    g = torch.Generator(device="cuda").manual_seed(1)
    V = [torch.randn(n, dtype=torch.complex64, device="cuda", generator=g) for _ in range(k)]
    W = [torch.empty(n, dtype=torch.complex64, device="cuda") for _ in range(nw)]
    va = (ctypes.c_void_p * k)(*[v.data_ptr() for v in V])
    wa = (ctypes.c_void_p * nw)(*[w.data_ptr() for w in W])
    c = (ctypes.c_double * (2 * k * nw))(*[((i * 7) % 13 - 6) / 13.0 for i in range(2 * k * nw)])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    call = lambda: qk.lib().qkrylov_vector_mcombine_device_f32(va, k, c, wa, nw, n, 0, stream)
    for _ in range(3):
        assert call() == 0
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        assert call() == 0
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / a.reps
    nbytes = (k + nw) * n * 8
    print(json.dumps({"k": k, "nw": nw, "n": n, "bytes_per_call": nbytes, "us": round(t * 1e6, 1),
                      "GBs": round(nbytes / t / 1e9, 1)}), flush=True)


if __name__ == "__main__":
    main()
