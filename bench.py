#!/usr/bin/env python
"""Lanczos steps/s on GB300: Heisenberg chain L=28, periodic, J=1, Sz=0
(dim 40,116,600), 200 Lanczos steps per run.

One bench step is one complete ground-state run of 200 Lanczos steps in the
mixed form (FP32 vectors and SpMV, compensated FP64-accurate reductions,
selective reorthogonalisation, FP64 Rayleigh-quotient/residual refinement),
from a seeded Gaussian start vector generated on the device.  `value` =
Lanczos steps/s over the K timed runs (all ranks); `e2e` = the same through the
C ABI with the start vector and the Ritz vector in pinned host memory.  The
plain FP64 path (reference semantics: full reorthogonalisation) is run once
on the same seed for |dE0|; the CPU baseline is the oracle port of the
reference algorithm (host CSR + CSR SpMV + full reorthogonalisation) timed on
a bounded row sample.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

L_SITES, PBC, SZ2, LANCZOS_STEPS = 28, True, 0, 200
METRIC = "lanczos_steps_per_s"
UNIT = "steps/s"
DIM = 40116600
BYTES_PER_ELEM_F32 = 8  # complex FP32


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--seed", type=int, default=2026)
    p.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison run")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-ftlm", action="store_true", help="skip the batched FTLM measurement")
    p.add_argument("--no-cf", action="store_true", help="skip the batched S(q, omega) measurement")
    p.add_argument("--no-davidson", action="store_true", help="skip the Hubbard Davidson measurement")
    return p.parse_args()


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as td
        td.init_process_group("gloo")
    return rank, local, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as td
        td.barrier()


def allreduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as td
    t = torch.tensor([x], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per SpMV launch of the Lanczos loop from the committed ncu
    summary of the fused launch: LANCZOS_STEPS - 1 launches that read x and
    the previous vector and write y, and the first one (no previous vector)."""
    p = os.path.join(ROOT, "profiles", "spmv_lanczos_fused_f32_heisenberg_L28.md")
    vals = {}
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_"):
                k, v = line.split(":")
                vals[k.strip()] = float(v)
    except OSError:
        return None
    if "traffic_bytes_per_fused_launch" not in vals or "traffic_bytes_per_first_launch" not in vals:
        return None
    return ((LANCZOS_STEPS - 1) * vals["traffic_bytes_per_fused_launch"] + vals["traffic_bytes_per_first_launch"]) / LANCZOS_STEPS


class Clocks:
    """nvidia-smi sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out, _ = self.p.communicate()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def heis_terms():
    import models as M
    return M.heisenberg_terms(L_SITES, PBC)


def _oracle():
    from oracle_ctypes import Oracle, available
    if not available("qko"):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)
    o = Oracle("qko")
    c = ctypes
    o.lib.qko_create_parallel.restype = c.c_void_p
    o.lib.qko_dim.restype = c.c_uint64
    o.lib.qko_nnz.restype = c.c_uint64
    return o


def _oracle_create(o, model, L, sector, terms, threads):
    """CSR of every row of the model, built by `threads` host threads (same CSR
    as the reference's single-threaded build); returns (handle, seconds)."""
    c = ctypes
    cre = np.array([complex(t[0]).real for t in terms], dtype=np.float64)
    cim = np.array([complex(t[0]).imag for t in terms], dtype=np.float64)
    nf = np.array([len(t[1]) for t in terms], dtype=np.int32)
    fl = [f for t in terms for f in t[1]]
    ops = (c.c_char_p * len(fl))(*[f[0].encode() for f in fl])
    sites = np.array([f[1] for f in fl], dtype=np.int32)
    sec = np.array(sector, dtype=np.int32)
    o.lib.qko_set_threads(threads)
    t0 = time.perf_counter()
    h = o.lib.qko_create_parallel(model, L, sec.ctypes.data_as(c.POINTER(c.c_int)), len(terms),
                                  cre.ctypes.data_as(c.POINTER(c.c_double)), cim.ctypes.data_as(c.POINTER(c.c_double)),
                                  nf.ctypes.data_as(c.POINTER(c.c_int)), ops, sites.ctypes.data_as(c.POINTER(c.c_int)))
    if not h:
        raise RuntimeError("oracle CSR build failed: " + o.lib.qko_last_error().decode())
    return h, time.perf_counter() - t0


def host_info():
    mem = None
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemTotal:"):
                mem = round(int(line.split()[1]) / 2 ** 20, 1)
    except OSError:
        pass
    return {"cores": os.cpu_count() or 1, "ram_gib": mem}


def cpu_lanczos_steps(n_steps, threads):
    """The reference's Lanczos on the host cores at full size (oracle port:
    host CSR of all 40,116,600 rows, CSR gather SpMV, full
    reorthogonalisation, tridiagonal ground state every step,
    src/solvers/lanczos.cpp:101-202), from the reference's mt19937(1234) start
    vector.  Returns (CSR build seconds, nnz, seconds of each step)."""
    import models as M
    c = ctypes
    o = _oracle()
    h, t_build = _oracle_create(o, 0, L_SITES, M.sector(sz2=SZ2), heis_terms(), threads)
    nnz = int(o.lib.qko_nnz(c.c_void_p(h)))
    st = np.zeros(n_steps)
    nd, e = c.c_int(), c.c_double()
    rc = o.lib.qko_lanczos_timed(c.c_void_p(h), None, n_steps, st.ctypes.data_as(c.POINTER(c.c_double)), c.byref(nd),
                                 c.byref(e))
    o.lib.qko_destroy(c.c_void_p(h))
    if rc != 0:
        raise RuntimeError("oracle Lanczos failed: " + o.lib.qko_last_error().decode())
    return t_build, nnz, st[:nd.value]


CPU_WARM, CPU_TIMED = 2, 6


def cpu_baseline(threads):
    """cpu_baseline of the Lanczos line: CPU_WARM + CPU_TIMED steps of the
    reference algorithm at full size; the timed steps' mean."""
    t_build, nnz, st = cpu_lanczos_steps(CPU_WARM + CPU_TIMED, threads)
    timed = st[CPU_WARM:]
    return {"value": len(timed) / float(timed.sum()), "unit": UNIT, "cores": threads, "kind": "port",
            "host": host_info(),
            "sample": (f"reference algorithm at full size (dim {DIM}, host CSR of {nnz} entries built by {threads} "
                       f"threads in {t_build:.1f} s, untimed): Lanczos steps {CPU_WARM + 1}..{CPU_WARM + CPU_TIMED} "
                       f"of a run from the reference start vector, each timed (SpMV, full reorthogonalisation at "
                       f"depth {CPU_WARM}..{CPU_WARM + CPU_TIMED - 1}, tridiagonal ground state): "
                       f"{1e3 * timed.mean():.0f} ms per step; a 200-step run reorthogonalises at mean depth 100, "
                       f"so its steps cost more than these")}


def run_reference(args, rank, ws):
    """The reference's CPU algorithm on the host cores (oracle port of
    src/solvers/lanczos.cpp at full size; the reference build does not
    travel), rank 0 only.  One bench step = one Lanczos step: warm-up + timed
    steps of one run, each timed."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    t_build, nnz, st = cpu_lanczos_steps(args.warmup + args.steps, threads)
    timed = st[args.warmup:args.warmup + args.steps]
    v = len(timed) / float(timed.sum())
    sample = (f"reference algorithm at full size (dim {DIM}; host CSR of {nnz} entries built by {threads} threads "
              f"in {t_build:.1f} s, untimed); one bench step = one Lanczos step (CSR SpMV, full "
              f"reorthogonalisation, tridiagonal ground state), steps {args.warmup + 1}..{args.warmup + args.steps} "
              f"of one run from the reference start vector (reorthogonalisation depth {args.warmup}.."
              f"{args.warmup + args.steps - 1}; a 200-step run's mean depth is 100, so its steps cost more)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * float(timed.mean()), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": workload_config(ws),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "host": host_info()},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_config(ws):
    return {"workload": f"heisenberg_chain_L{L_SITES}_pbc_sz0_{LANCZOS_STEPS}_lanczos_steps", "dim": DIM,
            "lanczos_steps_per_bench_step": LANCZOS_STEPS, "parallelism": f"replicas{ws}",
            "l2": "inputs larger than L2 (one FP32 Krylov vector = 321 MB)"}


def main():
    args = parse()
    rank, local, ws = dist()
    if args.impl == "reference":
        run_reference(args, rank, ws)
        return
    import qkrylov_gb300 as qk
    import models as M
    from models import make_model
    qk.set_device(local)
    basis, site, ops = make_model(qk, M.SPIN, L_SITES, M.sector(sz2=SZ2), heis_terms())
    t0 = time.perf_counter()
    H = qk.MatrixFreeHamiltonian(basis, site, ops)
    t_construct = time.perf_counter() - t0
    assert H.dimension == DIM

    for w in range(args.warmup):
        qk.lanczos_fixed_steps(H, LANCZOS_STEPS, seed=args.seed + 1000 + w, mixed=True)
    # ---- timed region: device-resident inputs ---------------------------------
    res = []
    qk.synchronize()
    barrier(ws)
    l0 = qk.kernel_launches()
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            res.append(qk.lanczos_fixed_steps(H, LANCZOS_STEPS, seed=args.seed + k, mixed=True))
        qk.synchronize()
        t_total = time.perf_counter() - t0
    barrier(ws)
    launches = qk.kernel_launches() - l0
    t_max = allreduce_max(t_total, ws)
    value = ws * args.steps * LANCZOS_STEPS / t_max
    spmv_s = sum(r.seconds_spmv for r in res) / max(1, sum(r.spmv_calls for r in res))

    # ---- e2e: through the C ABI with pinned host buffers -------------------------
    cudart = _cudart()
    nbytes = DIM * 16
    hv0 = _pinned(cudart, nbytes)
    hev = _pinned(cudart, nbytes)
    v0 = np.frombuffer((ctypes.c_char * nbytes).from_address(hv0), dtype=np.complex128)
    ev = np.frombuffer((ctypes.c_char * nbytes).from_address(hev), dtype=np.complex128)
    rng = np.random.default_rng(args.seed)
    v0.real[:] = rng.standard_normal(DIM)
    v0.imag[:] = rng.standard_normal(DIM)
    qk.lanczos_fixed_steps(H, LANCZOS_STEPS, mixed=True, v0=v0, eigenvector_out=ev)  # warm the host path
    qk.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    e2e_res, e2e_each = [], []
    for k in range(args.steps):
        tc = time.perf_counter()
        e2e_res.append(qk.lanczos_fixed_steps(H, LANCZOS_STEPS, mixed=True, v0=v0, eigenvector_out=ev))
        e2e_each.append(time.perf_counter() - tc)  # the call returns with the eigenvector on the host
    qk.synchronize()
    t_e2e = allreduce_max(time.perf_counter() - t0, ws)
    e2e_value = ws * args.steps * LANCZOS_STEPS / t_e2e

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "c64 (mixed: FP32 vectors/SpMV, FP64-accurate reductions, FP64 refinement)",
           "data": "synthetic (seeded Philox Gaussian start vectors)",
           "config": workload_config(ws), "construct_s": round(t_construct, 3),
           "gpu_launches": launches}
    if rank != 0:
        return
    hbm_peak, peak_kind = peaks()
    # each launch of the loop reads x and the previous Lanczos vector and writes y
    # (the recurrence is fused into the SpMV); the first has no previous vector
    alg_bytes = (3 * (LANCZOS_STEPS - 1) + 2) * DIM * BYTES_PER_ELEM_F32 / LANCZOS_STEPS
    achieved = alg_bytes / spmv_s / 1e9
    variant, _ = H.tuning(fp32=True)
    tr = profile_traffic() if variant == "rows4" else None  # the summary covers the four-rows kernel
    kname = {"rows4": "spmv_rows_kernel<float>", "rows4_staged": "spmv_rows_kernel<float, staged>",
             "rows4_wide": "spmv_rows_kernel<float, 4 CTAs/SM>",
             "row": "spmv_fast_kernel<float>",
             "staged": "spmv_fast_kernel<float, staged>"}.get(variant, "spmv_kernel<float>")
    out["roofline"] = {"kernel": kname + " (FP32 SpMV fused with the three-term recurrence)", "bound": "hbm",
                       "achieved": achieved,
                       "peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm_peak,
                       "traffic": tr, "algorithmic_bytes_per_launch": alg_bytes,
                       "launch_ms": spmv_s * 1e3}
    energies = [r.energy for r in res]
    out["mixed"] = {"energy": energies[-1], "energy_spread": max(energies) - min(energies),
                    "residual": res[-1].residual, "selective_steps": res[-1].selective_steps,
                    "loop_s": res[-1].seconds_loop, "refine_s": res[-1].seconds_refine}
    out["e2e"] = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes + 64,
                  # per call: device loop and refinement (the library's own timers), the rest is the
                  # start vector's upload and the Ritz vector's download with their permutations
                  "call_ms": 1e3 * t_e2e / args.steps, "call_ms_each": [round(1e3 * t, 2) for t in e2e_each],
                  "loop_ms": 1e3 * sum(r.seconds_loop for r in e2e_res) / len(e2e_res),
                  "refine_ms": 1e3 * sum(r.seconds_refine for r in e2e_res) / len(e2e_res),
                  "selective_steps": sum(r.selective_steps for r in e2e_res) / len(e2e_res)}
    out["clocks"] = clk.summary()
    if not args.no_fp64:
        t0 = time.perf_counter()
        r64 = qk.lanczos_fixed_steps(H, LANCZOS_STEPS, seed=args.seed, mixed=False)
        t64 = time.perf_counter() - t0
        de = abs(res[0].energy - r64.energy)
        out["fp64"] = {"steps_per_s": LANCZOS_STEPS / t64, "energy": r64.energy, "seconds": t64,
                       "spmv_ms": 1e3 * r64.seconds_spmv / max(1, r64.spmv_calls),
                       "form": "reference semantics: FP64 vectors and SpMV, full reorthogonalisation"}
        out["dE0_vs_fp64"] = {"abs": de, "rel": de / abs(r64.energy), "meets_1e-10": de <= 1e-10 * abs(r64.energy)}
        # FP64 with the mixed form's selective reorthogonalisation: separates the
        # gain of FP32 vectors from the gain of dropping full reorthogonalisation
        t0 = time.perf_counter()
        r64s = qk.lanczos_fixed_steps(H, LANCZOS_STEPS, seed=args.seed, mixed=False, selective=True)
        t64s = time.perf_counter() - t0
        out["fp64_selective"] = {"steps_per_s": LANCZOS_STEPS / t64s, "energy": r64s.energy, "seconds": t64s,
                                 "selective_steps": r64s.selective_steps,
                                 "spmv_ms": 1e3 * r64s.seconds_spmv / max(1, r64s.spmv_calls),
                                 "dE0_vs_fp64_full": abs(r64s.energy - r64.energy),
                                 "form": "FP64 vectors and SpMV, selective reorthogonalisation (host-driven steps)"}
    cpu = ws == 1 and not args.no_cpu_baseline
    if not args.no_ftlm:
        out["ftlm"] = ftlm_batch(qk, args.seed, hbm_peak, peak_kind, cpu=cpu)
    if not args.no_cf:
        out["cf"] = cf_batch(qk, hbm_peak, peak_kind, cpu=cpu)
    if not args.no_davidson:
        out["davidson"] = davidson_hubbard(qk, cpu=cpu)
    if ws == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(os.cpu_count() or 1)
    print(json.dumps(out), flush=True)


FTLM_L, FTLM_R, FTLM_M, FTLM_NT = 24, 32, 100, 200


def ftlm_batch(qk, seed, hbm_peak, peak_kind, cpu=True):
    """Batched FTLM: Heisenberg chain L=24 periodic, all 25 Sz sectors, 32
    Philox Gaussian vectors per sector, 100 Lanczos steps each, one block SpMV
    launch per step for all 800 vectors; Z, E, Cv at 200 log-spaced T in
    [0.01, 10] (shifted evaluation).  Mixed form (FP32 block vectors and SpMV,
    compensated reductions in FP64) and the FP64 form on the same vectors."""
    import models as M
    from models import make_model
    hams = []
    for sz2 in range(-FTLM_L, FTLM_L + 1, 2):
        b, s, o = make_model(qk, M.SPIN, FTLM_L, M.sector(sz2=sz2), M.heisenberg_terms(FTLM_L, True))
        hams.append(qk.MatrixFreeHamiltonian(b, s, o))
    betas = 1.0 / np.geomspace(0.01, 10.0, FTLM_NT)
    qk.ftlm_sectors(hams, betas, n_random=FTLM_R, n_steps=3, mixed=True, start="philox", seed=seed)  # warm-up
    res = {}
    for mixed in (True, False):
        t0 = time.perf_counter()
        r = qk.ftlm_sectors(hams, betas, n_random=FTLM_R, n_steps=FTLM_M, mixed=mixed, start="philox", seed=seed,
                            shifted=True)
        wall = time.perf_counter() - t0
        res[mixed] = (r, wall)
    r32, w32 = res[True]
    r64, w64 = res[False]
    st = r32.stats
    nvec = FTLM_R * len(hams)
    e = 8
    alg = 2 * st["rows"] * st["padded_vectors"] * e
    achieved = alg / (st["spmv_ms"] * 1e-3) / 1e9
    fin = np.isfinite(r64.internal_energy) & np.isfinite(r32.internal_energy)
    dE = np.abs(r32.internal_energy - r64.internal_energy)[fin]
    dC = np.abs(r32.specific_heat - r64.specific_heat)[fin]
    z64 = r64.partition_function
    z32 = r32.partition_function * np.exp(r32.log_shift - r64.log_shift)
    fz = np.isfinite(z64) & np.isfinite(z32) & (z64 > 0)
    rZ = np.abs(z32[fz] / z64[fz] - 1.0)
    rE = (dE / np.maximum(np.abs(r64.internal_energy[fin]), 1e-300))
    out = {"workload": f"heisenberg_chain_L{FTLM_L}_pbc_all_{len(hams)}_sz_sectors_R{FTLM_R}_M{FTLM_M}_T{FTLM_NT}",
            "rows": st["rows"], "vectors": nvec, "vectors_per_s": nvec / st["seconds"],
            "e2e_vectors_per_s": nvec / w32, "loop_s": st["seconds"],
            "fp64_vectors_per_s": nvec / r64.stats["seconds"], "fp64_loop_s": r64.stats["seconds"],
            "tile": {"vectors_per_lane": st["vectors_per_lane"], "tune_ms": st["tune_ms"]},
            "roofline": {"kernel": "spmv_block_kernel<float> (FP32 block SpMV, 32 vectors)", "bound": "hbm",
                         "achieved": achieved, "peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "algorithmic_bytes_per_launch": alg,
                         "launch_ms": st["spmv_ms"]},
            "mixed_vs_fp64": {"max_abs_dE": float(dE.max()) if dE.size else None,
                              "max_rel_dE": float(rE.max()) if rE.size else None,
                              "max_abs_dCv": float(dC.max()) if dC.size else None,
                              "max_rel_dZ": float(rZ.max()) if rZ.size else None},
            "start_vectors": "seeded Philox Gaussian (device)"}
    # the plain single-vector FP64 path (the reference's FTLM per sector and
    # vector, ftlm.cpp:123-170), one vector per sector
    t0 = time.perf_counter()
    for Hs in hams:
        qk.ftlm(Hs, 1.0, n_random=1, n_steps=FTLM_M)
    qk.synchronize()
    t_plain = time.perf_counter() - t0
    out["plain_fp64_ftlm_vectors_per_s"] = len(hams) / t_plain
    out["plain_fp64_ftlm_sample"] = f"qkrylov_ftlm_f64 per sector, 1 vector each, M={FTLM_M}: {len(hams)} vectors in {t_plain:.2f} s"
    if cpu:
        out["cpu_baseline"] = cpu_ftlm(os.cpu_count() or 1)
    return out


FTLM_CPU_R = 1


def cpu_ftlm(threads):
    """The reference's FTLM (src/solvers/ftlm.cpp:123-170: per random vector a
    100-step three-term Lanczos and its weights) on the host cores, every Sz
    sector of the L=24 chain with one random vector each (the vectors of a
    sector are independent, so vectors/s does not depend on R)."""
    import models as M
    c = ctypes
    o = _oracle()
    t_build, t_run, nvec = 0.0, 0.0, 0
    for sz2 in range(-FTLM_L, FTLM_L + 1, 2):
        h, tb = _oracle_create(o, 0, FTLM_L, M.sector(sz2=sz2), M.heisenberg_terms(FTLM_L, True), threads)
        t_build += tb
        Z, E, C = c.c_double(), c.c_double(), c.c_double()
        t0 = time.perf_counter()
        rc = o.lib.qko_ftlm(c.c_void_p(h), c.c_double(1.0), FTLM_CPU_R, FTLM_M, c.byref(Z), c.byref(E), c.byref(C))
        t_run += time.perf_counter() - t0
        o.lib.qko_destroy(c.c_void_p(h))
        if rc != 0:
            raise RuntimeError(o.lib.qko_last_error().decode())
        nvec += FTLM_CPU_R
    return {"value": nvec / t_run, "unit": "vectors/s", "cores": threads, "kind": "port", "host": host_info(),
            "sample": (f"reference FTLM on all {2 * FTLM_L // 2 + 1} Sz sectors of the L={FTLM_L} chain, "
                       f"R={FTLM_CPU_R} vector per sector, M={FTLM_M} steps each ({nvec} vectors in {t_run:.1f} s; "
                       f"host CSRs built by {threads} threads in {t_build:.1f} s, untimed)")}


CF_L, CF_STEPS, CF_NOMEGA, CF_ETA = 26, 300, 2000, 0.05


def cf_batch(qk, hbm_peak, peak_kind, cpu=True):
    """S(q, omega) of the Heisenberg chain L=26 periodic, Sz=0 (dim 10,400,600):
    FP64 Lanczos ground state psi0, right-hand sides Sz(q)|psi0> with
    Sz(q) = L^-1/2 sum_j e^{iqj} Sz_j for q = 2 pi k / 26, k = 0..13 (applied
    as OpSum operators; k = 0 is the zero vector), then all 14 continued
    fractions in one batched run of 300 steps (mixed form, and FP64 for the
    comparison), S on 2000 omega in [0, 4] with eta = 0.05."""
    import models as M
    from models import make_model
    b, s, o = make_model(qk, M.SPIN, CF_L, M.sector(sz2=0), M.heisenberg_terms(CF_L, True))
    H = qk.MatrixFreeHamiltonian(b, s, o)
    t0 = time.perf_counter()
    gs = qk.lanczos_ground_state(H, maxiter=300, tol=1e-12, mixed=False)
    t_gs = time.perf_counter() - t0
    psi, E0 = gs.eigenvector, gs.energy
    t0 = time.perf_counter()
    phis = []
    for k in range(CF_L // 2 + 1):
        ph = np.exp(2j * np.pi * k / CF_L * np.arange(CF_L)) / np.sqrt(CF_L)
        ops = qk.OpSum()
        for j in range(CF_L):
            ops.add_term(ph[j], "Sz", j)
        phis.append(qk.MatrixFreeHamiltonian(b, qk.SpinHalfSite(), ops).apply(psi))
    t_rhs = time.perf_counter() - t0
    # the right-hand sides in pinned host memory, as the e2e rule has it
    nbytes = len(phis) * H.dimension * 16
    P = np.frombuffer((ctypes.c_char * nbytes).from_address(_pinned(_cudart(), nbytes)), dtype=np.complex128)
    P = P.reshape(len(phis), H.dimension)
    for i, ph in enumerate(phis):
        P[i] = ph
    phis = P
    omegas = np.linspace(0.0, 4.0, CF_NOMEGA)
    for mixed in (True, False):  # warm-up: tile autotuning and the block workspace
        qk.spectral_functions_block(H, phis, omegas[:2], E0, eta=CF_ETA, n_iter=3, mixed=mixed)
    out = {}
    for mixed in (True, False):
        t0 = time.perf_counter()
        S, res, st = qk.spectral_functions_block(H, phis, omegas, E0, eta=CF_ETA, n_iter=CF_STEPS, mixed=mixed)
        out[mixed] = (S, st, time.perf_counter() - t0)
    S32, st32, w32 = out[True]
    S64, st64, _ = out[False]
    nrhs = len(phis)
    alg = 2 * st32["rows"] * st32["padded_vectors"] * 8
    achieved = alg / (st32["spmv_ms"] * 1e-3) / 1e9
    out = {"workload": f"heisenberg_chain_L{CF_L}_pbc_sz0_Szq_{nrhs}_rhs_{CF_STEPS}_steps_{CF_NOMEGA}_omega",
            "dim": H.dimension, "rhs": nrhs, "E0": E0, "ground_state_s": t_gs, "rhs_build_s": t_rhs,
            "rhs_steps_per_s": nrhs * CF_STEPS / st32["seconds"], "loop_s": st32["seconds"],
            "e2e_s": w32, "fp64_rhs_steps_per_s": nrhs * CF_STEPS / st64["seconds"], "fp64_loop_s": st64["seconds"],
            "tile": {"vectors_per_lane": st32["vectors_per_lane"], "padded_vectors": st32["padded_vectors"]},
            "roofline": {"kernel": "spmv_block_kernel<float> (FP32 block SpMV, 16 vectors)", "bound": "hbm",
                         "achieved": achieved, "peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "algorithmic_bytes_per_launch": alg,
                         "launch_ms": st32["spmv_ms"]},
            "mixed_vs_fp64_max_rel_dS": float(np.abs(S32 - S64).max() / np.abs(S64).max())}
    # the plain single-right-hand-side FP64 path (dynamics.cpp:13-59), one q
    t0 = time.perf_counter()
    cf1 = qk.continued_fraction_coeffs(H, phis[1], n_iter=CF_STEPS)
    t_plain = time.perf_counter() - t0
    out["plain_fp64_rhs_steps_per_s"] = len(cf1.alphas) / t_plain
    if cpu:
        out["cpu_baseline"] = cpu_cf(os.cpu_count() or 1, phis[1])
    return out


CF_CPU_STEPS = 100


def cpu_cf(threads, phi):
    """The reference's continued fraction (src/solvers/dynamics.cpp:13-59: a
    three-term Lanczos without reorthogonalisation) on the host cores for one
    right-hand side of the L=26 run (q = 2 pi / 26), CF_CPU_STEPS steps; every
    step costs the same, so right-hand-side steps/s carries over to 300."""
    import models as M
    c = ctypes
    o = _oracle()
    h, t_build = _oracle_create(o, 0, CF_L, M.sector(sz2=0), M.heisenberg_terms(CF_L, True), threads)
    ph = np.ascontiguousarray(phi, dtype=np.complex128)
    a, b = np.zeros(CF_CPU_STEPS), np.zeros(CF_CPU_STEPS)
    nrm, na, nb = c.c_double(), c.c_int(), c.c_int()
    t0 = time.perf_counter()
    rc = o.lib.qko_cf(c.c_void_p(h), ph.ctypes.data_as(c.POINTER(c.c_double)), CF_CPU_STEPS,
                      a.ctypes.data_as(c.POINTER(c.c_double)), b.ctypes.data_as(c.POINTER(c.c_double)), c.byref(nrm),
                      c.byref(na), c.byref(nb))
    t = time.perf_counter() - t0
    o.lib.qko_destroy(c.c_void_p(h))
    if rc != 0:
        raise RuntimeError(o.lib.qko_last_error().decode())
    return {"value": na.value / t, "unit": "rhs-steps/s", "cores": threads, "kind": "port", "host": host_info(),
            "sample": (f"reference continued fraction, one right-hand side (Sz(q) psi0, q = 2 pi/{CF_L}) of dim "
                       f"{len(ph)}, {na.value} steps in {t:.1f} s (host CSR built by {threads} threads in "
                       f"{t_build:.1f} s, untimed)")}


DAV_L, DAV_K, DAV_SUB, DAV_TOL, DAV_ITERS = 16, 4, 32, 1e-8, 100
DAV_MID_L = 12
DAV_CPU_ITERS = 14  # two restart cycles (4 + 7 x 4 = 32 vectors per cycle)
E0_CF_STEPS = 300


def tridiag_lowest(a, b):
    from scipy.linalg import eigh_tridiagonal
    n = len(a)
    return float(eigh_tridiagonal(np.asarray(a), np.asarray(b[:n - 1]), eigvals_only=True,
                                  select="i", select_range=(0, 0))[0])


def davidson_hubbard(qk, cpu=True):
    """Davidson on the Fermi-Hubbard chain L=16 periodic, t=1, U=4,
    N_up = N_dn = 8 (dim 165,636,900): lowest 4 eigenpairs, subspace <= 32,
    4 corrections per iteration, tol 1e-8, the reference's algorithm and
    its cap of 100 iterations (src/solvers/davidson.cpp:141,180), both forms
    to the cap or to convergence.  The lowest eigenvalue is checked against E0
    from an FP64 Lanczos recurrence on the same sector (three-term, 300 steps,
    lowest Ritz value): |lambda_0 - E0| <= ||r_0|| for a Hermitian operator.
    The same solve at L=12 (dim 853,776) is timed on the GPU and, through the
    oracle port of the reference, on the host cores."""
    import models as M
    from models import make_model
    b, s, o = make_model(qk, M.HUBBARD, DAV_L, M.sector(nup=DAV_L // 2, ndn=DAV_L // 2), M.hubbard_terms(DAV_L, True))
    t0 = time.perf_counter()
    H = qk.MatrixFreeHamiltonian(b, s, o)
    t_build = time.perf_counter() - t0
    res = {}
    for mixed in (True, False):
        t0 = time.perf_counter()
        r = qk.davidson_lowest_ex(H, n_eig=DAV_K, max_subspace=DAV_SUB, tol=DAV_TOL, mixed=mixed, max_iter=DAV_ITERS)
        res[mixed] = (r, time.perf_counter() - t0)
    (r32, w32), (r64, w64) = res[True], res[False]
    # E0 of the sector: FP64 three-term Lanczos from a seeded start vector
    rng = np.random.default_rng(11)
    n = H.dimension
    phi = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    t0 = time.perf_counter()
    cf = qk.continued_fraction_coeffs(H, phi, n_iter=E0_CF_STEPS)
    e0 = tridiag_lowest(cf.alphas, cf.betas)
    t_e0 = time.perf_counter() - t0
    del phi
    out = {"workload": f"hubbard_chain_L{DAV_L}_pbc_U4_half_filling_k{DAV_K}_sub{DAV_SUB}_tol1e-8_cap{DAV_ITERS}",
           "dim": n, "construct_s": t_build,
           "mixed": {"iterations": r32.iterations, "converged": r32.converged, "seconds": w32,
                     "s_per_iter": r32.seconds / max(1, r32.iterations),
                     "evals": [float(x) for x in r32.eigenvalues],
                     "residuals_fp64": [float(x) for x in r32.residuals]},
           "fp64": {"iterations": r64.iterations, "converged": r64.converged, "seconds": w64,
                    "s_per_iter": r64.seconds / max(1, r64.iterations),
                    "evals": [float(x) for x in r64.eigenvalues],
                    "residuals": [float(x) for x in r64.residuals]},
           "E0_lanczos_fp64": {"value": e0, "steps": E0_CF_STEPS, "seconds": t_e0},
           "form": "mixed: FP32 vectors and SpMV, run-summed FP32 projections (float-float across runs of 32), FP64-refined Ritz pairs"}
    for key, r in (("mixed", r32), ("fp64", r64)):
        d = abs(float(r.eigenvalues[0]) - e0)
        out[key]["lambda0_minus_E0"] = d
        out[key]["within_residual_bound"] = bool(d <= float(r.residuals[0]) + 1e-12 * abs(e0))
    del H
    # the same solve at L=12, GPU and host cores
    b, s, o = make_model(qk, M.HUBBARD, DAV_MID_L, M.sector(nup=DAV_MID_L // 2, ndn=DAV_MID_L // 2),
                         M.hubbard_terms(DAV_MID_L, True))
    Hm = qk.MatrixFreeHamiltonian(b, s, o)
    mid = {}
    for mixed in (True, False):
        r = qk.davidson_lowest_ex(Hm, n_eig=DAV_K, max_subspace=DAV_SUB, tol=DAV_TOL, mixed=mixed, max_iter=DAV_ITERS)
        mid["mixed" if mixed else "fp64"] = {"iterations": r.iterations, "s_per_iter": r.seconds / max(1, r.iterations),
                                             "evals": [float(x) for x in r.eigenvalues],
                                             "residuals": [float(x) for x in r.residuals]}
    out[f"L{DAV_MID_L}"] = mid
    if cpu:
        out["cpu_baseline"] = cpu_davidson(os.cpu_count() or 1)
    return out


def cpu_davidson(threads):
    """The reference's Davidson (src/solvers/davidson.cpp:86-227) on the host
    cores at Hubbard L=12 (the reference cannot build L=16: its int32 CSR
    offsets overflow at 5.5e9 entries), timed over its first DAV_CPU_ITERS
    iterations."""
    import models as M
    c = ctypes
    o = _oracle()
    h, t_build = _oracle_create(o, M.HUBBARD, DAV_MID_L, M.sector(nup=DAV_MID_L // 2, ndn=DAV_MID_L // 2),
                                M.hubbard_terms(DAV_MID_L, True), threads)
    dim = int(o.lib.qko_dim(c.c_void_p(h)))
    ev = np.zeros(DAV_K)
    it, conv, nout = c.c_int(), c.c_int(), c.c_int()
    t0 = time.perf_counter()
    rc = o.lib.qko_davidson_max(c.c_void_p(h), DAV_K, DAV_SUB, c.c_double(DAV_TOL), DAV_CPU_ITERS,
                                ev.ctypes.data_as(c.POINTER(c.c_double)), None, c.byref(it), c.byref(conv),
                                c.byref(nout))
    t = time.perf_counter() - t0
    o.lib.qko_destroy(c.c_void_p(h))
    if rc != 0:
        raise RuntimeError(o.lib.qko_last_error().decode())
    return {"value": t / max(1, it.value), "unit": "s/iteration", "cores": threads, "kind": "port",
            "host": host_info(), "evals": [float(x) for x in ev[:nout.value]], "iterations": it.value,
            "sample": (f"reference Davidson, Hubbard L={DAV_MID_L} (dim {dim}), k={DAV_K}, subspace {DAV_SUB}, the "
                       f"first {it.value} iterations (two restart cycles) in {t:.1f} s (host CSR built by {threads} "
                       f"threads in {t_build:.1f} s, untimed); compare the GPU's L{DAV_MID_L} s_per_iter")}


def _cudart():
    import glob
    import ctypes.util
    names = ["libcudart.so", "libcudart.so.13", ctypes.util.find_library("cudart")]
    names += glob.glob("/usr/local/cuda/lib64/libcudart.so*") + glob.glob("/usr/local/cuda/targets/*/lib/libcudart.so*")
    for n in names:
        if not n:
            continue
        try:
            lib = ctypes.CDLL(n)
            lib.cudaMallocHost.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
            return lib
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


def _pinned(cudart, nbytes):
    p = ctypes.c_void_p()
    if cudart.cudaMallocHost(ctypes.byref(p), nbytes) != 0:
        raise RuntimeError("cudaMallocHost failed")
    return p.value


if __name__ == "__main__":
    main()
