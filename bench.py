"""Benchmark: time to a converged CCD E/A on one lattice per GPU.

Workload (default): pure neutron matter, A=66 at rho=0.16 fm^-3 on the nmax=4
lattice (9^3 momenta x 2 spins = 1458 states), synthetic Minnesota interaction,
single twist, MP2 start.  A step is one full solve: MP2 amplitudes, then CCD
iterations (Jacobi + DIIS(8)) until the FP64 residual ||R - D T|| < 1e-10, with the
interaction resident in HBM.  value = seconds per solve of the mixed-precision form
(--precision bf16x3, default; tf32x3; or fp64 for the plain form), device time from
CUDA events on the engine's stream.  The plain FP64 solve of the same lattice is timed
beside it (plain_fp64, speedup_vs_plain_fp64), and the E/A difference between the two
is reported in keV.  e2e = the same solve driven through the C ABI from pinned host
buffers holding the reference-layout V blocks and Fock matrix, with the host->device
copies and the T2 readback inside the timed region.

--impl reference times the CPU path (the oracle restatement of the reference's
complex<double> solver, all host cores) on a bounded sample: single CCD iterations
of the same lattice, scaled by the reference algorithm's iteration count.

Multi-GPU: the lattice is one twist; N GPUs solve N independent twists (replicas,
no collective); value is the slowest rank's time, scaling "weak".
"""
from __future__ import annotations

import argparse
import ctypes as C
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "coupled-cluster-nuclearmatter_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")

METRIC = "time-to-converged E/A (<1 keV vs FP64) mixed+batched+learned vs plain GPU"
WORKLOADS = {
    "pnm66": dict(nmax=4, A=66, rho=0.16, snm=False, potential=0,
                  desc="PNM A=66, rho=0.16 fm^-3, nmax=4 (1458 states), Minnesota, theta=0"),
    "pnm14": dict(nmax=2, A=14, rho=0.08, snm=False, potential=0,
                  desc="PNM A=14, rho=0.08 fm^-3, nmax=2 (250 states), Minnesota, theta=0"),
}
# Iterations the reference algorithm (0.75/0.25 mixing + DIIS every 6, |dE| < 1e-6 MeV,
# ccm_iter.f90:67-96) takes on each lattice, as run by the engine's reference mode.
REFERENCE_ITERATIONS = {"pnm66": 13, "pnm14": 13}


def load_pkg():
    if "ccnm_gb300" in sys.modules:
        return sys.modules["ccnm_gb300"]
    spec = importlib.util.spec_from_file_location("ccnm_gb300", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    m = importlib.util.module_from_spec(spec)
    sys.modules["ccnm_gb300"] = m
    spec.loader.exec_module(m)
    return m


def packed_sizes(L, ccx):
    """Packed (a<b, i<j) sizes per hhpp channel and ring-channel sizes."""
    c = L.counts()
    P, H = [], []
    for ch in range(c["hhpp"]):
        hh, pp = L.pairs(ccx.CH_HHPP, ch)
        H.append(int((hh[:, 0] < hh[:, 1]).sum()))
        P.append(int((pp[:, 0] < pp[:, 1]).sum()))
    ring = []
    for q in range(c["ph_phhp"]):
        _, nph, nhp = L.channel(ccx.CH_PH_PHHP, q)
        ring.append((nph, nhp))
    return P, H, ring


def flop_model(P, H, ring, real=True):
    """Algorithmic FLOPs per CCD iteration on unique pairs (a<b, i<j); 2 per real MAC."""
    m = 2.0 if real else 8.0
    pp = sum(m * p * p * h for p, h in zip(P, H))
    hh = sum(m * p * h * h for p, h in zip(P, H))
    x = sum(m * h * h * p for p, h in zip(P, H))
    i4 = sum(m * nhp * nhp * nph for nph, nhp in ring)
    rg = sum(m * nph * nhp * nhp for nph, nhp in ring)
    return {"pp_ladder": pp, "hh_ladder": hh, "i9": x, "i4": i4, "ring": rg, "ladders": pp + hh,
            "total": pp + hh + x + i4 + rg}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile(prefix="clocks", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def oracle_sample(wl: dict, iters: int, warm: int):
    """Seconds per CCD iteration of the CPU oracle on the full lattice (reference mode)."""
    sys.path.insert(0, ORACLE_DIR)
    import oracle as O
    O.build()
    o = O.Oracle(O.Config(nmax=wl["nmax"], A=wl["A"], rho=wl["rho"], snm=wl["snm"], potential=wl["potential"]))
    o.mp2()
    o.diis_setup()
    cnt = 0
    times = []
    for k in range(warm + iters):
        t = time.perf_counter()
        o.t2_intermediate()
        cnt = o.diis_t1t2(cnt + 1)
        o.energy()
        dt = time.perf_counter() - t
        if k >= warm:
            times.append(dt)
    return statistics.mean(times), O.num_threads(), o


def run_reference(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    n_ref = REFERENCE_ITERATIONS[args.workload]
    per_it, cores, _ = oracle_sample(wl, args.steps, args.warmup)
    value = per_it * n_ref
    sample = (f"{args.steps} timed CCD iterations (after {args.warmup} warm-up) of the oracle restatement "
              f"(complex<double> ordered blocks, as the reference), x {n_ref} reference-mode iterations")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_it * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": wl["desc"], "algorithm": "reference (0.75/0.25 mixing, DIIS every 6, |dE|<1e-6)",
                       "sample_unit": "one CCD iteration"},
            "cpu_baseline": {"value": value, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


PRECISIONS = {"fp64": 0, "bf16x3": 1, "tf32x3": 2}
FALLBACK_HBM_GBS = 6800.0


def hbm_peak():
    """Measured copy bandwidth (GB/s) of this GPU model, else the fallback figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (of measured)"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback 6.8 TB/s (of fallback)"


def kernel_work(P, H, ring, precision):
    """Algorithmic work of one timed bracket per kernel slot: ('flop', F) or ('byte', B).

    FP64 GEMMs count 2 flops per multiply-add on unique pairs.  Tensor-core launches are
    HBM-bound (arithmetic intensity far below the BF16 ridge): their bytes are the split
    operands read once (hi + lo, es bytes each), C read and written in FP64."""
    es = 2 if precision == 1 else 4
    pp = sum(2.0 * p * p * h for p, h in zip(P, H))
    hh = sum(2.0 * p * h * h for p, h in zip(P, H))
    x = sum(2.0 * h * h * p for p, h in zip(P, H))
    i4 = sum(2.0 * nhp * nhp * nph for nph, nhp in ring)
    rg = sum(2.0 * nph * nhp * nhp for nph, nhp in ring)
    # pp-ladder launch: V_pppp' dT' plus the two hh-ladder corrections (dT' I9', T_b' dI9')
    # into one accumulator; R' read and written, PP_b + HH_b read
    b_pp = sum(2 * es * (p * p + p * h) + 2 * 2 * es * (p * h + h * h) + 24.0 * p * h for p, h in zip(P, H))
    # dI4 launch: 1/2 V_ph dT_ph, and dX = V_hhpp'^T dT' (H x H, K = P) for I9' - I9_b'
    b_i4 = (sum(2 * es * (2.0 * nhp * nph) + 16.0 * nhp * nhp for nph, nhp in ring)
            + sum(2 * es * (2.0 * h * p) + 16.0 * h * h for p, h in zip(P, H)))
    # ring launch: dR_ph = T_ph,b dI4 + dT_ph I4 (two accumulators), written without reading
    b_ring = sum(2 * 2 * es * (nph * nhp + nhp * nhp) + 8.0 * nph * nhp for nph, nhp in ring)
    # digit-product GEMM: 9 BF16 digit planes of V_pppp' and of T_b read once, C written
    b_oz = sum(9 * 2.0 * (p * p + p * h) + 16.0 * p * h for p, h in zip(P, H))
    b_i4_oz = sum(9 * 2.0 * (2.0 * nhp * nph) + 16.0 * nhp * nhp for nph, nhp in ring)
    b_ring_oz = sum(9 * 2.0 * (nph * nhp + nhp * nhp) + 16.0 * nph * nhp for nph, nhp in ring)
    return {"x_fp64": ("flop", x), "i4_fp64": ("flop", i4), "ring_fp64": ("flop", rg),
            "ladder_fp64": ("flop", pp + hh), "pp_rebase_fp64": ("flop", pp), "hh_fp64": ("flop", hh),
            "pp_tc": ("byte", b_pp), "i4_tc": ("byte", b_i4), "ring_tc": ("byte", b_ring),
            "pp_rebase_digits": ("byte", b_oz), "i4_rebase_digits": ("byte", b_i4_oz),
            "ring_rebase_digits": ("byte", b_ring_oz)}


KERNEL_NAMES = {"x_fp64": "k_xdot X = V_hhpp'^T T' (FP64 column dots)", "i4_fp64": "k_gemm<double> I4",
                "ring_fp64": "k_gemm<double> ring", "ladder_fp64": "k_gemm<double> fused pp+hh ladder",
                "pp_rebase_fp64": "k_gemm<double> pp-ladder at a re-base", "hh_fp64": "k_gemm<double> hh-ladder",
                "pp_tc": "k_tc_gemm pp + hh ladder corrections (3 products, one accumulator)", "i4_tc": "k_tc_gemm dI4 and dX corrections",
                "ring_tc": "k_tc_gemm ring corrections (2 products, one accumulator)", "split": "k_tc_split",
                "pp_rebase_digits": "k_oz_gemm pp-ladder at a re-base (exact digit products)",
                "i4_rebase_digits": "k_oz_gemm I4 at a re-base (exact digit products)",
                "ring_rebase_digits": "k_oz_gemm ring at a re-base (exact digit products)",
                "i7_fp64": "k_i7dots I7 of a mixed residual (FP64 column dots)"}


def replica_theta(rank: int):
    """Twist of a replica: rank 0 solves the untwisted lattice, the others their own
    twist (replicas, no data exchange between ranks)."""
    return (0.0, 0.0, 0.0) if rank == 0 else (0.1 * rank, -0.07 * rank, 0.05 * rank)


def max_over_ranks(value: float, dist, device) -> float:
    """The slowest rank's time: all_reduce MAX (the only collective of the bench)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args, wl):
    import torch
    ccx = load_pkg()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    theta = replica_theta(rank)
    L = ccx.Layout.from_basis(wl["nmax"], wl["A"], wl["rho"], snm=wl["snm"], theta=theta)
    real = wl["potential"] == ccx.POT_MINNESOTA
    prec = PRECISIONS[args.precision] if real else 0
    e = ccx.Engine(L, device=local, real=real)
    e.generate(potential=wl["potential"])
    e.setup_t_amplitudes()
    tuned_shapes, _ = e.autotune()  # FP64 GEMM tile shape per column-count bucket
    stream = torch.cuda.ExternalStream(e.stream(), device=local)
    P, H, ring = packed_sizes(L, ccx)
    flops = flop_model(P, H, ring, real=real)

    def solve(eng, precision):
        eng.setup_t_amplitudes()
        return eng.ccd_iter(mode=ccx.MODE_STANDARD, precision=precision, tol=args.tol, max_iter=200, diis_dim=8,
                            defect_period=args.defect_period,
                            rebase=ccx.REBASE_DIGITS if (precision and args.rebase == "digits") else ccx.REBASE_FP64)

    def timed(precision, steps, sample_clocks):
        """The timed solves, without the per-term event records (profiling off)."""
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e.set_profiling(False)
        clocks = ClockSampler(local) if sample_clocks else None
        launches0 = e.launches()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        results = []
        for _ in range(steps):
            results.append(solve(e, precision))
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
        clk = clocks.stop() if clocks else None
        ms = ev0.elapsed_time(ev1) / steps
        ms = max_over_ranks(ms, dist, "cuda")
        return ms, results, e.launches() - launches0, clk

    def breakdown(precision, steps):
        """Per-term and per-kernel device times from the same number of solves with
        profiling on, after the timed region."""
        timers, ktimers = {}, {}
        e.set_profiling(True)
        for _ in range(steps):
            solve(e, precision)
            for k, v in e.timers().items():
                timers[k] = timers.get(k, 0.0) + v
            for k, (ms_k, n_k) in e.kernel_timers().items():
                a, b = ktimers.get(k, (0.0, 0))
                ktimers[k] = (a + ms_k, b + n_k)
        e.set_profiling(False)
        return timers, ktimers

    # warm-up: both forms (tensor-core tiles are prepared by the first mixed solve)
    for _ in range(args.warmup):
        solve(e, prec)
        if prec:
            solve(e, 0)
    ms, results, launches, clk = timed(prec, args.steps, True)
    r = results[-1]
    iters = sum(x["iterations"] for x in results) / len(results)
    ea = (e.e0() + r["e_ccd"]).real / wl["A"]
    if prec:
        ms64, res64, _, _ = timed(0, args.steps, False)
        ea64 = (e.e0() + res64[-1]["e_ccd"]).real / wl["A"]
        plain = {"s": ms64 * 1e-3, "iterations": res64[-1]["iterations"], "E_per_A_MeV": ea64,
                 "res_norm": res64[-1]["res_norm"]}
    else:
        ms64, ea64, plain = ms, ea, None

    # ---- roofline of the dominant kernel (largest device time in the profiled solves) ----
    timers, ktimers = breakdown(prec, args.steps)
    work = kernel_work(P, H, ring, prec)
    dom = max((k for k in ktimers if k in work and ktimers[k][1] > 0), key=lambda k: ktimers[k][0])
    kms, kn = ktimers[dom]
    per_launch_ms = kms / kn
    kind, amount = work[dom]
    if kind == "flop":
        peak = ccx.device_fp64_peak(local)
        achieved = amount / (per_launch_ms * 1e-3) / 1e12
        roofline = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                    "peak_source": "measured FP64 FMA probe on this GPU (ccx_device_fp64_peak); "
                                   "MEASURED_PEAKS.json holds no FP64 figure",
                    "flop_per_launch": amount}
    else:
        peak, src = hbm_peak()
        achieved = amount / (per_launch_ms * 1e-3) / 1e9
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "peak_source": src, "bytes_per_launch": amount}
    roofline.update({"kernel": KERNEL_NAMES[dom], "ms_per_launch": per_launch_ms, "launches_timed": kn,
                     "traffic": PROFILED_TRAFFIC.get((args.workload, args.precision, dom))})
    kernel_ms = {k: {"ms": v[0] / args.steps, "brackets": v[1] // args.steps} for k, v in ktimers.items() if v[1]}

    # ---- end to end through the C ABI from pinned host buffers ----
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, ccx, torch, L, e, local, real, lambda eng: solve(eng, prec))

    form = {0: "plain FP64", 1: "mixed BF16x3 + FP64 defect correction",
            2: "mixed TF32x3 + FP64 defect correction"}[prec]
    if prec and args.rebase == "digits":
        form += " (re-base products as exact digit products on the tensor cores)"
    line = {"metric": METRIC, "value": ms * 1e-3, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if real else "c128", "data": "synthetic",
            "form": form + " (packed unique pairs, real arithmetic)" if real else form,
            "config": {"workload": wl["desc"], "solver": f"Jacobi + DIIS(8) to ||R-DT||<{args.tol:g} (FP64 residual)",
                       "precision": args.precision if prec else "fp64",
                       "defect_period": args.defect_period or "adaptive",
                       "rebase": args.rebase if prec else None,
                       "gemm_tile_shapes_by_N_bucket": tuned_shapes,
                       "l2": "inputs larger than L2 (V_pppp packed, %.2f GB, read every iteration)"
                             % (sum(p * p for p in P) * 8 / 1e9),
                       "replicas": world},
            "iterations": iters, "fp64_sweeps": r["fp64_sweeps"], "mixed_iterations": r["mixed_iterations"],
            "ccd_iterations_per_s": iters / (ms * 1e-3), "E_per_A_MeV": ea, "res_norm": r["res_norm"],
            "plain_fp64": plain, "speedup_vs_plain_fp64": (ms64 / ms) if prec else None,
            "dE_per_A_keV_vs_fp64": abs(ea - ea64) * 1e3 if prec else 0.0,
            "gflop_per_iteration": flops["total"] / 1e9,
            "breakdown": "term_ms_per_solve and kernel_ms_per_solve (and the roofline's launch time) from "
                         "as many further solves with per-term CUDA events on, after the timed region",
            "term_ms_per_solve": {k: v / args.steps for k, v in timers.items()},
            "kernel_ms_per_solve": kernel_ms,
            "roofline": roofline, "clocks": clk, "gpu_launches": launches, "e2e": e2e}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        n_ref = REFERENCE_ITERATIONS[args.workload] or reference_iterations(e, ccx)
        per_it, cores, _ = oracle_sample(wl, 1, 0)
        line["cpu_baseline"] = {"value": per_it * n_ref, "unit": "s", "cores": cores, "kind": "port",
                                "sample": f"1 CCD iteration of the oracle (complex<double>, as the reference) on the "
                                          f"full lattice, x {n_ref} reference-mode iterations"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from ncu
# captures of `bench.py --steps 1 --warmup 1 --no-e2e --no-cpu-baseline` on this workload:
# (workload, precision, kernel slot) -> bytes
PROFILED_TRAFFIC = {
    ("pnm66", "bf16x3", "x_fp64"): 32.0e6,
    ("pnm66", "bf16x3", "pp_tc"): 643.7e6,
    ("pnm66", "bf16x3", "pp_rebase_digits"): 2426.5e6,
    ("pnm66", "bf16x3", "i4_rebase_digits"): 506.5e6,
    ("pnm66", "bf16x3", "ring_rebase_digits"): 505.4e6,
}


def reference_iterations(e, ccx):
    e.setup_t_amplitudes()
    return e.ccd_iter(mode=ccx.MODE_REFERENCE)["iterations"]


def run_e2e(args, ccx, torch, L, e, local, real, solve):
    lib = ccx.lib()
    c = L.counts()
    dims = L.hhpp_dims()
    n = len(L.orbits()["nx"])
    # reference-layout host blocks (pinned), exported once from the resident interaction
    blocks = []

    def pinned(nd):
        return torch.empty(nd, dtype=torch.float64, pin_memory=True)

    def export(kind, ch, rows, cols):
        buf = pinned(2 * rows * cols)
        ccx._check(lib.ccx_get_vblock(e._h, kind, ch, C.c_void_p(buf.data_ptr())))
        blocks.append((kind, ch, buf))

    for ch in range(c["hhpp"]):
        nh, npp = dims[ch]
        export(ccx.CH_HHPP, ch, nh, npp)
        export(ccx.V_PPPP, ch, npp, npp)
    for ch in range(c["hhhh"]):
        _, nh, _ = L.channel(ccx.CH_HHHH, ch)
        export(ccx.CH_HHHH, ch, nh, nh)
    for ch in range(c["hphp"]):
        _, nhp, _ = L.channel(ccx.CH_HPHP, ch)
        export(ccx.CH_HPHP, ch, nhp, nhp)
    fock = pinned(2 * n * n)
    ccx._check(lib.ccx_get_fock(e._h, C.c_void_p(fock.data_ptr())))
    e0 = e.e0()
    e0buf = (C.c_double * 2)(e0.real, e0.imag)
    t_out = pinned(2 * c["amps"])
    h2d = sum(b.numel() * 8 for _, _, b in blocks) + fock.numel() * 8
    d2h = t_out.numel() * 8 + 16
    eb = ccx.Engine(L, device=local, real=real)
    stream = torch.cuda.ExternalStream(eb.stream(), device=local)

    # one ccx_set_vblocks call per block family
    families = {}
    for kind, ch, buf in blocks:
        families.setdefault(kind, []).append((ch, buf))
    calls = []
    for kind, lst in families.items():
        chs = (C.c_int32 * len(lst))(*[ch for ch, _ in lst])
        ptrs = (C.c_void_p * len(lst))(*[buf.data_ptr() for _, buf in lst])
        calls.append((kind, len(lst), chs, ptrs))

    def step():
        ccx._check(lib.ccx_set_fock(eb._h, C.c_void_p(fock.data_ptr()), e0buf))
        for kind, n, chs, ptrs in calls:
            ccx._check(lib.ccx_set_vblocks(eb._h, kind, n, chs, ptrs))
        r = solve(eb)
        ccx._check(lib.ccx_get_t2_all(eb._h, C.c_void_p(t_out.data_ptr())))
        return r

    for _ in range(max(1, args.warmup // 2)):
        step()
    eb.autotune()  # once per engine, as a host would after handing over the interaction
    step()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        r = step()
    ev1.record(stream)
    ev1.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    ms = ev0.elapsed_time(ev1) / args.steps
    eb.close()
    return {"value": ms * 1e-3, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "host_wall_s": wall, "iterations": r["iterations"],
            "path": "ccx_set_fock + ccx_set_vblocks (all HHPP/PPPP/HHHH/HPHP blocks, one call per family) + "
                    "ccx_setup_t_amplitudes + ccx_ccd_iter + ccx_get_t2_all",
            "host_buffers": "pinned: the packing kernels read the reference-layout blocks in place over "
                            "NVLink-C2C (only the cache lines of unique pairs) and the amplitudes are "
                            "unpacked straight into the host buffer; h2d_bytes_per_step is the size of "
                            "the host inputs"}


TWIST_LATTICES = {
    "pnm66": dict(nmax=4, A=66, rho=0.16, snm=False, desc="PNM A=66, rho=0.16 fm^-3, nmax=4 (1458 states), Minnesota"),
    "snm132n3": dict(nmax=3, A=132, rho=0.16, snm=True, desc="SNM A=132, rho=0.16 fm^-3, nmax=3 (1372 states), Minnesota"),
    "snm132n3chiral": dict(nmax=3, A=132, rho=0.16, snm=True, potential=1,
                           desc="SNM A=132, rho=0.16 fm^-3, nmax=3 (1372 states), chiral-like (complex)"),
}


def gauss_legendre_twists():
    """4 x 4 x 4 Gauss-Legendre product grid on [-pi, pi]^3 with its weights (sum 1)."""
    import itertools
    import math
    x = (-0.8611363115940526, -0.3399810435848563, 0.3399810435848563, 0.8611363115940526)
    w = (0.3478548451374538, 0.6521451548625461, 0.6521451548625461, 0.3478548451374538)
    out = []
    for (xa, wa), (xb, wb), (xc, wc) in itertools.product(zip(x, w), repeat=3):
        out.append(((math.pi * xa, math.pi * xb, math.pi * xc), wa * wb * wc / 8.0))
    return out


def run_twists(args):
    """Twist batch: the same lattice at N twists, solved as one lockstep batch
    (ccx_ccd_iter_batch) against a per-twist sequential loop (ccx_ccd_iter), both in the
    mixed form with digit-product re-bases, MP2 start, ||R - D T|| < tol."""
    import torch
    ccx = load_pkg()
    lat = TWIST_LATTICES[args.lattice]
    grid = gauss_legendre_twists()
    # a spread subset when fewer than 64 twists are asked for
    step = max(1, len(grid) // args.twists)
    grid = grid[::step][:args.twists]
    prec = PRECISIONS[args.precision]
    rb = ccx.REBASE_DIGITS if (prec and args.rebase == "digits") else ccx.REBASE_FP64
    opts = dict(precision=prec, rebase=rb, tol=args.tol, max_iter=200, diis_dim=8)
    engines = []
    for th, _ in grid:
        L = ccx.Layout.from_basis(lat["nmax"], lat["A"], lat["rho"], snm=lat["snm"], theta=th)
        pot = lat.get("potential", 0)
        e = ccx.Engine(L, real=pot == 0)
        e.generate(potential=pot)
        e.setup_t_amplitudes()
        e.ccd_iter(mode=ccx.MODE_STANDARD, **opts)  # warm-up: operand tiles and digit planes
        engines.append(e)
    seq, bat = [], []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rs = []
        for e in engines:
            e.setup_t_amplitudes()
            rs.append(e.ccd_iter(mode=ccx.MODE_STANDARD, **opts))
        torch.cuda.synchronize()
        seq.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        for e in engines:
            e.setup_t_amplitudes()
        rb_, _ = ccx.ccd_iter_batch(engines, **opts)
        torch.cuda.synchronize()
        bat.append(time.perf_counter() - t0)
    wsum = sum(w for _, w in grid)
    ea = sum(w * (e.e0() + r["e_ccd"]).real / lat["A"] for (_, w), e, r in zip(grid, engines, rb_)) / wsum
    ea_seq = sum(w * (e.e0() + r["e_ccd"]).real / lat["A"] for (_, w), e, r in zip(grid, engines, rs)) / wsum
    line = {"metric": "time to converged twist-averaged E/A", "impl": "ours", "workload": "twist batch",
            "lattice": lat["desc"], "twists": len(grid), "form": args.precision + " + " + args.rebase + " re-base",
            "batched_s": statistics.median(bat), "sequential_s": statistics.median(seq),
            "speedup_batched_vs_sequential": statistics.median(seq) / statistics.median(bat),
            "iterations": [r["iterations"] for r in rb_], "E_per_A_twist_averaged_MeV": ea,
            "dE_per_A_keV_batched_vs_sequential": abs(ea - ea_seq) * 1e3, "steps": args.steps,
            "device_GB_per_engine": engines[0].memory() / 1e9}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="pnm66", choices=sorted(WORKLOADS))
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--precision", default="bf16x3", choices=sorted(PRECISIONS))
    ap.add_argument("--defect-period", type=int, default=0, help="FP64 re-base every k iterations (0: adaptive)")
    ap.add_argument("--twists", type=int, default=0,
                    help="run the twist-batch comparison with this many twists instead of the headline")
    ap.add_argument("--lattice", default="pnm66", choices=sorted(TWIST_LATTICES))
    ap.add_argument("--rebase", default="digits", choices=["fp64", "digits"],
                    help="pp-ladder product of a re-base: FP64 FMA GEMM or exact digit products on the tensor cores")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.twists > 0 and args.impl == "ours":
        return run_twists(args)
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_ours(args, wl)


if __name__ == "__main__":
    sys.exit(main())
