"""Benchmark: time to a converged CCD E/A on one lattice per GPU.

Workload (default, --workload snm132n4): symmetric nuclear matter, A=132 at rho=0.16
fm^-3 on the nmax=4 lattice (9^3 momenta x 4 spin-isospin states = 2916 states), the
synthetic chiral-like interaction (regulated one-pion exchange plus contact terms; its
V is complex), single twist, MP2 start.  A step is one full solve: MP2 amplitudes, then
CCD iterations (Jacobi + DIIS(8)) until the FP64 residual ||R - D T|| < 1e-10, with the
interaction resident in HBM.  value = seconds per solve of the mixed-precision form
(--precision bf16x3, default; tf32x3; or fp64 for the plain form), device time from
CUDA events on the engine's stream.  The plain FP64 solve of the same lattice is timed
beside it (plain_fp64, speedup_vs_plain_fp64), and the E/A difference between the two
is reported in keV.  e2e = the same solve driven through the C ABI from pinned host
buffers holding the reference-layout V blocks and Fock matrix, with the host->device
copies and the T2 readback inside the timed region.  --workload pnm66 runs pure
neutron matter A=66 at nmax=4 with the Minnesota interaction instead.

--impl reference times the CPU path (the oracle restatement of the reference's
complex<double> solver, all host cores) on a bounded sample: single CCD iterations
of the same lattice, scaled by the reference algorithm's iteration count.

--twists N runs the twist-averaged form instead: N twists of the 4x4x4 Gauss-Legendre
grid on [-pi, pi]^3 of one lattice, each converged to ||R - D T|| < 1e-10, solved in
lockstep batches of as many twists as the device holds, against the plain FP64 GPU
solve of the same twists.

Multi-GPU: the lattice is one twist; N GPUs solve N independent twists (replicas,
no collective); value is the slowest rank's time, scaling "weak".
"""
from __future__ import annotations

import argparse
import ctypes as C
import importlib.util
import json
import math
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
    "snm132n4": dict(nmax=4, A=132, rho=0.16, snm=True, potential=1,
                     desc="SNM A=132, rho=0.16 fm^-3, nmax=4 (2916 states), chiral-like (complex V), theta=0"),
    "snm132n3": dict(nmax=3, A=132, rho=0.16, snm=True, potential=1,
                     desc="SNM A=132, rho=0.16 fm^-3, nmax=3 (1372 states), chiral-like (complex V), theta=0"),
    "snm76n2": dict(nmax=2, A=76, rho=0.16, snm=True, potential=1,
                    desc="SNM A=76, rho=0.16 fm^-3, nmax=2 (500 states), chiral-like (complex V), theta=0"),
    "pnm66": dict(nmax=4, A=66, rho=0.16, snm=False, potential=0,
                  desc="PNM A=66, rho=0.16 fm^-3, nmax=4 (1458 states), Minnesota, theta=0"),
    "pnm14": dict(nmax=2, A=14, rho=0.08, snm=False, potential=0,
                  desc="PNM A=14, rho=0.08 fm^-3, nmax=2 (250 states), Minnesota, theta=0"),
}
# Iterations the reference algorithm (0.75/0.25 mixing + DIIS every 6, |dE| < 1e-6 MeV,
# ccm_iter.f90:67-96) takes on each lattice, as run by the engine's reference mode
# (None: measured by the engine when needed).
REFERENCE_ITERATIONS = {"pnm66": 13, "pnm14": 13, "snm132n4": 19, "snm132n3": None, "snm76n2": None}


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


def oracle_iterations(o, n: int, cnt: int = 0):
    """Seconds of each of n reference-mode iterations of the oracle (t2_intermediate, the
    DIIS step and the energy), and the DIIS counter after them."""
    times = []
    for _ in range(n):
        t = time.perf_counter()
        o.t2_intermediate()
        cnt = o.diis_t1t2(cnt + 1)
        o.energy()
        times.append(time.perf_counter() - t)
    return times, cnt


def oracle_build(wl: dict):
    sys.path.insert(0, ORACLE_DIR)
    import oracle as O
    O.build()
    o = O.Oracle(O.Config(nmax=wl["nmax"], A=wl["A"], rho=wl["rho"], snm=wl["snm"], potential=wl["potential"]))
    o.mp2()
    o.diis_setup()
    return O, o


def oracle_sample(wl: dict, iters: int, warm: int):
    """Seconds per CCD iteration of the CPU oracle on the full lattice (reference mode)."""
    O, o = oracle_build(wl)
    _, cnt = oracle_iterations(o, warm)
    times, _ = oracle_iterations(o, iters, cnt)
    return statistics.mean(times), O.num_threads(), o


# Oracle iterations per timed step and warm-up of the reference arm are capped so that
# the whole run stays within a few minutes on the larger lattices (one SNM 132 nmax=4
# iteration takes about 8 s on 16 Grace cores, after about 40 s of V set-up).
REFERENCE_ARM_CAP = {"snm132n4": (3, 1), "snm132n3": (5, 1)}
# The reference arm times one whole reference-mode solve from MP2 when its warm-up
# iterations predict the solve within this many seconds (on 16 Grace cores about 7 s at
# PNM 66 and 155 s at SNM 132 nmax=4); otherwise it extrapolates timed iterations.
REFERENCE_FULL_SOLVE_S = 240.0


def run_reference(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    n_ref = REFERENCE_ITERATIONS[args.workload]
    if n_ref is None:
        raise SystemExit("no reference-mode iteration count recorded for " + args.workload)
    cap_s, cap_w = REFERENCE_ARM_CAP.get(args.workload, (args.steps, args.warmup))
    steps, warm = max(1, min(args.steps, cap_s)), max(1, min(args.warmup, cap_w))
    O, o = oracle_build(wl)
    cores = O.num_threads()
    t_warm, cnt = oracle_iterations(o, warm)
    what = "of the oracle restatement (complex<double> ordered blocks, as the reference) on the full lattice"
    if statistics.mean(t_warm) * n_ref <= REFERENCE_FULL_SOLVE_S:
        o.mp2()
        t = time.perf_counter()
        r = o.ccd_iter(mode=O.MODE_REFERENCE, max_iter=n_ref + 10)  # bounded if it stalls
        value = time.perf_counter() - t
        iters = r["iterations"]
        ms_per_step = value * 1e3
        unit = "one whole reference-mode solve"
        sample = (f"one whole reference-mode solve from MP2, measured ({iters} iterations to |dE| < 1e-6, "
                  f"converged {r['converged']}), after {warm} warm-up iteration(s), {what}")
    else:
        times, _ = oracle_iterations(o, steps, cnt)
        per_it = statistics.mean(times)
        value = per_it * n_ref
        iters = n_ref
        ms_per_step = per_it * 1e3
        unit = "one CCD iteration"
        sample = (f"{steps} timed CCD iterations (after {warm} warm-up) {what}, x {n_ref} "
                  f"reference-mode iterations (extrapolated)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": wl["desc"], "algorithm": "reference (0.75/0.25 mixing, DIIS every 6, |dE|<1e-6)",
                       "sample_unit": unit, "iterations": iters},
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


def kernel_work(P, H, ring, precision, real=True):
    """Algorithmic work of one timed bracket per kernel slot: ('flop', F) or ('byte', B),
    and the bytes of the operand representation the kernel actually streams.

    Unique pairs (a<b, i<j) throughout.  FP64 GEMMs count 2 flops per real multiply-add
    (8 per complex one).  Tensor-core launches are HBM-bound (arithmetic intensity far
    below the BF16 ridge): their algorithmic bytes are the FP64 (or complex FP64)
    elements of every matrix the product reads, once, and of C written once, e = 8 (16)
    bytes per element.  The representation the kernel streams instead -- BF16 (TF32)
    hi/lo halves or the 9 BF16 digit planes of the exact digit products -- is returned
    beside it, so that the report can show both."""
    e = 8.0 if real else 16.0
    nc = 1 if real else 2                     # real components per element
    mac = 2.0 if real else 8.0
    es = 2 if precision == 1 else 4           # bytes of one hi or lo half
    pp = sum(mac * p * p * h for p, h in zip(P, H))
    hh = sum(mac * p * h * h for p, h in zip(P, H))
    x = sum(mac * h * h * p for p, h in zip(P, H))
    i4 = sum(mac * nhp * nhp * nph for nph, nhp in ring)
    rg = sum(mac * nph * nhp * nhp for nph, nhp in ring)
    PH = sum(p * h for p, h in zip(P, H))
    P2 = sum(p * p for p in P)
    H2 = sum(h * h for h in H)
    PHr = sum(nph * nhp for nph, nhp in ring)
    HP2 = sum(nhp * nhp for nph, nhp in ring)
    # pp-ladder launch: V_pppp' dT' + dT' I9' + T_b' dI9' into R' (read and written) with
    # PP_b + HH_b read: V_pppp', dT', T_b', I9', dI9', R' (2x), PP_b, HH_b
    a_pp = e * (P2 + 6 * PH + 2 * H2)
    r_pp = nc * (2 * es * (P2 + PH) + 2 * 2 * es * (PH + H2)) + e * 4 * PH
    # dI4 launch: dI4 = 1/2 V_ph dT_ph (n_hp x n_hp) and dX = V_hhpp'^T dT' (H x H)
    a_i4 = e * (2 * PHr + HP2) + e * (2 * PH + H2)
    r_i4 = nc * (2 * es * (2 * PHr) + 2 * es * 2 * PH) + e * (HP2 + H2)
    # ring launch: dR_ph = T_ph,b dI4 + dT_ph I4 (written without reading)
    a_rg = e * (2 * PHr + 2 * HP2 + PHr)
    r_rg = nc * 2 * 2 * es * (PHr + HP2) + e * PHr
    # digit products at a re-base: A, B read once, C written once
    a_oz = e * (P2 + 2 * PH)
    r_oz = nc * 9 * 2.0 * (P2 + PH) + e * PH
    a_i4_oz = e * (2 * PHr + HP2)
    r_i4_oz = nc * 9 * 2.0 * (2 * PHr) + e * HP2
    a_rg_oz = e * (2 * PHr + HP2)
    r_rg_oz = nc * 9 * 2.0 * (PHr + HP2) + e * PHr
    # X = V_hhpp'^T T' (H x H, K = P) and HH_b = T' I9' (P x H, K = H) at a re-base
    a_x_oz = e * (2 * PH + H2)
    r_x_oz = nc * 9 * 2.0 * (2 * PH) + e * H2
    a_hh_oz = e * (2 * PH + H2)
    r_hh_oz = nc * 9 * 2.0 * (PH + H2) + e * 2 * PH
    return {"x_fp64": ("flop", x, None), "i4_fp64": ("flop", i4, None), "ring_fp64": ("flop", rg, None),
            "ladder_fp64": ("flop", pp + hh, None), "pp_rebase_fp64": ("flop", pp, None), "hh_fp64": ("flop", hh, None),
            "pp_tc": ("byte", a_pp, r_pp), "i4_tc": ("byte", a_i4, r_i4), "ring_tc": ("byte", a_rg, r_rg),
            "pp_rebase_digits": ("byte", a_oz, r_oz), "i4_rebase_digits": ("byte", a_i4_oz, r_i4_oz),
            "ring_rebase_digits": ("byte", a_rg_oz, r_rg_oz), "x_rebase_digits": ("byte", a_x_oz, r_x_oz),
            "hh_rebase_digits": ("byte", a_hh_oz, r_hh_oz)}


KERNEL_NAMES = {"x_fp64": "k_xdot X = V_hhpp'^T T' (FP64 column dots)", "i4_fp64": "k_gemm<double> I4",
                "ring_fp64": "k_gemm<double> ring", "ladder_fp64": "k_gemm<double> fused pp+hh ladder",
                "pp_rebase_fp64": "k_gemm<double> pp-ladder at a re-base", "hh_fp64": "k_gemm<double> hh-ladder",
                "pp_tc": "k_tc_gemm pp + hh ladder corrections (3 products, one accumulator)", "i4_tc": "k_tc_gemm dI4 and dX corrections",
                "ring_tc": "k_tc_gemm ring corrections (2 products, one accumulator)", "split": "k_tc_split",
                "pp_rebase_digits": "k_oz_gemm pp-ladder at a re-base (exact digit products)",
                "i4_rebase_digits": "k_oz_gemm I4 at a re-base (exact digit products)",
                "ring_rebase_digits": "k_oz_gemm ring at a re-base (exact digit products)",
                "i7_fp64": "k_i7dots I7 of a mixed residual (FP64 column dots)",
                "x_rebase_digits": "k_oz_gemm X = V_hhpp'^T T' at a re-base (exact digit products)",
                "hh_rebase_digits": "k_oz_gemm hh-ladder T' I9' at a re-base (exact digit products)"}


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
    real = wl["potential"] == ccx.POT_MINNESOTA and not any(theta)
    prec = PRECISIONS[args.precision]
    e = ccx.Engine(L, device=local, real=real)
    e.generate(potential=wl["potential"])
    e.setup_t_amplitudes()
    tuned_shapes, _ = e.autotune()  # FP64 GEMM tile shape per column-count bucket
    tc_form = None
    if prec:  # launch form of each tensor-core correction product
        tc_merged, tc_ms = e.autotune_tc(prec)
        tc_form = {name: {"form": "one launch" if mg else "one launch per column bucket",
                          "ms_per_bucket_launches": t[0], "ms_one_launch": t[1]}
                   for name, mg, t in zip(("pp_hh_ladders", "dI4_dX", "ring"), tc_merged, tc_ms)}
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

    # warm-up: the headline form W times (tensor-core tiles and digit planes are prepared
    # by the first mixed solve), the plain FP64 form once
    for _ in range(args.warmup):
        solve(e, prec)
    if prec:
        solve(e, 0)
    ms, results, launches, clk = timed(prec, args.steps, True)
    r = results[-1]
    iters = sum(x["iterations"] for x in results) / len(results)
    ea = (e.e0() + r["e_ccd"]).real / wl["A"]
    if prec:
        # the plain FP64 solve is 10-20x slower: a bounded number of timed solves
        n64 = max(1, min(args.steps, args.plain_steps))
        ms64, res64, _, _ = timed(0, n64, False)
        ea64 = (e.e0() + res64[-1]["e_ccd"]).real / wl["A"]
        plain = {"s": ms64 * 1e-3, "solves_timed": n64, "iterations": res64[-1]["iterations"],
                 "E_per_A_MeV": ea64, "res_norm": res64[-1]["res_norm"]}
    else:
        ms64, ea64, plain = ms, ea, None

    # ---- roofline of the dominant kernel (largest device time in the profiled solves) ----
    timers, ktimers = breakdown(prec, args.steps)
    work = kernel_work(P, H, ring, prec, real=real)
    dom = max((k for k in ktimers if k in work and ktimers[k][1] > 0), key=lambda k: ktimers[k][0])
    kms, kn = ktimers[dom]
    per_launch_ms = kms / kn
    kind, amount, rep = work[dom]
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
                    "peak_source": src, "bytes_per_launch": amount,
                    "bytes_basis": "algorithmic: unique-pair %s elements of every operand read once and of C "
                                   "written once" % ("FP64" if real else "complex FP64"),
                    "representation_bytes_per_launch": rep,
                    "representation_frac": rep / (per_launch_ms * 1e-3) / 1e9 / peak}
    traffic = PROFILED_TRAFFIC.get((args.workload, args.precision, dom))
    roofline.update({"kernel": KERNEL_NAMES[dom], "ms_per_launch": per_launch_ms, "launches_timed": kn,
                     "traffic": traffic,
                     "traffic_over_algorithmic": (traffic / amount) if (traffic and kind == "byte") else None})
    kernel_ms = {k: {"ms": v[0] / args.steps, "brackets": v[1] // args.steps} for k, v in ktimers.items() if v[1]}

    # ---- end to end through the C ABI from pinned host buffers ----
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, ccx, torch, L, e, local, real, lambda eng: solve(eng, prec))

    form = {0: "plain FP64", 1: "mixed BF16x3 + FP64 defect correction",
            2: "mixed TF32x3 + FP64 defect correction"}[prec]
    if prec and args.rebase == "digits":
        form += " (re-base products as exact digit products on the tensor cores)"
    form += " (packed unique pairs, real arithmetic)" if real else " (packed unique pairs, complex arithmetic)"
    e_bytes = 8 if real else 16
    line = {"metric": METRIC, "value": ms * 1e-3, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if real else "c128", "data": "synthetic",
            "form": form,
            "config": {"workload": wl["desc"], "solver": f"Jacobi + DIIS(8) to ||R-DT||<{args.tol:g} (FP64 residual)",
                       "precision": args.precision if prec else "fp64",
                       "defect_period": args.defect_period or "adaptive",
                       "rebase": args.rebase if prec else None,
                       "gemm_tile_shapes_by_N_bucket": tuned_shapes, "tensor_core_launch_form": tc_form,
                       "l2": "inputs larger than L2 (V_pppp packed, %.2f GB, read every iteration)"
                             % (sum(p * p for p in P) * e_bytes / 1e9),
                       "replicas": world},
            "iterations": iters, "fp64_sweeps": r["fp64_sweeps"], "mixed_iterations": r["mixed_iterations"],
            "ccd_iterations_per_s": iters / (ms * 1e-3), "E_per_A_MeV": ea, "res_norm": r["res_norm"],
            "plain_fp64": plain, "speedup_vs_plain_fp64": (ms64 / ms) if prec else None,
            "dE_per_A_keV_vs_fp64": abs(ea - ea64) * 1e3 if prec else 0.0,
            "gflop_per_iteration": flops["total"] / 1e9,
            "device_GB": e.memory() / 1e9,
            "breakdown": "term_ms_per_solve and kernel_ms_per_solve (and the roofline's launch time) from "
                         "as many further solves with per-term CUDA events on, after the timed region",
            "term_ms_per_solve": {k: v / args.steps for k, v in timers.items()},
            "kernel_ms_per_solve": kernel_ms,
            "roofline": roofline, "clocks": clk, "gpu_launches": launches, "e2e": e2e}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        n_ref = REFERENCE_ITERATIONS.get(args.workload) or reference_iterations(e, ccx)
        per_it, cores, o = oracle_sample(wl, 1, 0)
        o.close()
        line["cpu_baseline"] = {"value": per_it * n_ref, "unit": "s", "cores": cores, "kind": "port",
                                "sample": f"1 CCD iteration of the oracle (complex<double>, as the reference) on the "
                                          f"full lattice, x {n_ref} reference-mode iterations (extrapolated)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


# DRAM bytes per timed bracket (dram__bytes_read.sum + dram__bytes_write.sum) from ncu
# captures of `bench.py --steps 1 --warmup 1 --no-e2e --no-cpu-baseline` on the workload:
# (workload, precision, kernel slot) -> bytes
PROFILED_TRAFFIC = {
    # profiles/k_oz_gemm_snm132n3.md: both phase launches of the pp re-base product
    ("snm132n3", "bf16x3", "pp_rebase_digits"): 4.09e9,
    # the same scaled to SNM 132 nmax=4 by the algorithmic bytes (12.0 GB / 1.51 GB)
    ("snm132n4", "bf16x3", "pp_rebase_digits"): 32.6e9,
    ("pnm66", "bf16x3", "x_fp64"): 32.0e6,
    ("pnm66", "bf16x3", "pp_tc"): 643.7e6,
    ("pnm66", "bf16x3", "pp_rebase_digits"): 2426.5e6,
    ("pnm66", "bf16x3", "i4_rebase_digits"): 506.5e6,
    ("pnm66", "bf16x3", "ring_rebase_digits"): 505.4e6,
}


def reference_iterations(e, ccx):
    e.setup_t_amplitudes()
    return e.ccd_iter(mode=ccx.MODE_REFERENCE)["iterations"]


class PinnedHost:
    """One page-locked, device-addressable host buffer (ccx_host_alloc) holding many blocks
    back to back."""

    def __init__(self, torch, ndoubles: int):
        self.b = load_pkg().HostBuffer(ndoubles)
        self.used = 0

    def take(self, n: int) -> int:
        """Pointer to the next n doubles."""
        p = self.b.ptr + 8 * self.used
        self.used += n
        return p

    def close(self):
        self.b.close()


def run_e2e(args, ccx, torch, L, e, local, real, solve):
    lib = ccx.lib()
    c = L.counts()
    dims = L.hhpp_dims()
    n = len(L.orbits()["nx"])
    # reference-layout host blocks in one registered buffer per family, exported once from
    # the resident interaction
    fams = {ccx.CH_HHPP: [(ch, nh, npp) for ch, (nh, npp) in enumerate(dims)],
            ccx.V_PPPP: [(ch, npp, npp) for ch, (nh, npp) in enumerate(dims)],
            ccx.CH_HHHH: [(ch, L.channel(ccx.CH_HHHH, ch)[1], L.channel(ccx.CH_HHHH, ch)[1])
                          for ch in range(c["hhhh"])],
            ccx.CH_HPHP: [(ch, L.channel(ccx.CH_HPHP, ch)[1], L.channel(ccx.CH_HPHP, ch)[1])
                          for ch in range(c["hphp"])]}
    bufs, calls = [], []
    h2d = 0
    for kind, lst in fams.items():
        tot = sum(2 * r * q for _, r, q in lst)
        buf = PinnedHost(torch, tot)
        bufs.append(buf)
        ptrs = []
        for ch, r, q in lst:
            ptr = buf.take(2 * r * q)
            ccx._check(lib.ccx_get_vblock(e._h, kind, ch, C.c_void_p(ptr)))
            ptrs.append(ptr)
        h2d += 8 * tot
        chs = (C.c_int32 * len(lst))(*[ch for ch, _, _ in lst])
        calls.append((kind, len(lst), chs, (C.c_void_p * len(lst))(*ptrs)))
    fb = PinnedHost(torch, 2 * n * n)
    fock = fb.take(2 * n * n)
    ccx._check(lib.ccx_get_fock(e._h, C.c_void_p(fock)))
    h2d += 16 * n * n
    e0 = e.e0()
    e0buf = (C.c_double * 2)(e0.real, e0.imag)
    tb = PinnedHost(torch, 2 * c["amps"])
    t_out = tb.take(2 * c["amps"])
    d2h = 16 * c["amps"] + 16
    bufs += [fb, tb]
    eb = ccx.Engine(L, device=local, real=real)
    stream = torch.cuda.ExternalStream(eb.stream(), device=local)

    fam_name = {ccx.CH_HHPP: "set_vblocks_hhpp", ccx.V_PPPP: "set_vblocks_pppp", ccx.CH_HHHH: "set_vblocks_hhhh",
                ccx.CH_HPHP: "set_vblocks_hphp"}
    phase = {"set_fock": 0.0, **{v: 0.0 for v in fam_name.values()}, "solve": 0.0, "get_t2_all": 0.0}

    def step():
        t0 = time.perf_counter()
        ccx._check(lib.ccx_set_fock(eb._h, C.c_void_p(fock), e0buf))
        t1 = time.perf_counter()
        phase["set_fock"] += t1 - t0
        for kind, nb, chs, ptrs in calls:  # each call returns once its blocks are packed
            ccx._check(lib.ccx_set_vblocks(eb._h, kind, nb, chs, ptrs))
            t2 = time.perf_counter()
            phase[fam_name[kind]] += t2 - t1
            t1 = t2
        r = solve(eb)
        t2 = time.perf_counter()
        ccx._check(lib.ccx_get_t2_all(eb._h, C.c_void_p(t_out)))
        t3 = time.perf_counter()
        phase["solve"] += t2 - t1
        phase["get_t2_all"] += t3 - t2
        return r

    try:
        for _ in range(max(1, args.warmup // 2)):
            step()
        eb.autotune()  # once per engine, as a host would after handing over the interaction
        if PRECISIONS[args.precision]:
            eb.autotune_tc(PRECISIONS[args.precision])
        step()
        torch.cuda.synchronize()
        for k in phase:
            phase[k] = 0.0
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
    finally:
        eb.close()
        for b in bufs:
            b.close()
    return {"value": ms * 1e-3, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "host_wall_s": wall, "iterations": r["iterations"],
            "host_phase_s_per_step": {k: v / args.steps for k, v in phase.items()},
            "path": "ccx_set_fock + ccx_set_vblocks (all HHPP/PPPP/HHHH/HPHP blocks, one call per family) + "
                    "ccx_setup_t_amplitudes + ccx_ccd_iter + ccx_get_t2_all",
            "host_buffers": "page-locked (ccx_host_alloc): blocks are read in place over NVLink-C2C by the "
                            "packing kernels (only the cache lines of unique pairs; V_pppp a reference column "
                            "per CTA); the amplitudes are unpacked straight into the host buffer; "
                            "h2d_bytes_per_step is the size of the host inputs"}


TWIST_LATTICES = {
    "pnm66": dict(nmax=4, A=66, rho=0.16, snm=False, desc="PNM A=66, rho=0.16 fm^-3, nmax=4 (1458 states), Minnesota"),
    "pnm14": dict(nmax=2, A=14, rho=0.08, snm=False, desc="PNM A=14, nmax=2 (250 states), Minnesota"),
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
    """Twist-averaged E/A of one lattice at N twists (ccm_main.f90:163-279 solves them one
    after the other).  The headline form (mixed precision, digit-product re-bases) runs the
    twists in lockstep batches (ccx_ccd_iter_batch) of half as many twists as the device
    holds, the next batch built while one solves; the per-twist sequential loop of the same
    form and the plain FP64 GPU solve are timed beside it.  Every step covers the whole job: engines (layout on the host, interaction
    generated on the device, operand tiles and digit planes) are built per batch, so
    total_s includes that set-up; solve_s counts only the solves.  The plain FP64 form is
    timed on a seeded sample of the twists (plain_twists) and scaled to N."""
    import random
    from concurrent.futures import ThreadPoolExecutor
    import torch
    ccx = load_pkg()
    lat = TWIST_LATTICES[args.lattice]
    grid = gauss_legendre_twists()
    step = max(1, len(grid) // args.twists)
    grid = grid[::step][:args.twists]
    pot = lat.get("potential", 0)
    prec = PRECISIONS[args.precision]
    rb = ccx.REBASE_DIGITS if (prec and args.rebase == "digits") else ccx.REBASE_FP64
    opts = dict(precision=prec, rebase=rb, tol=args.tol, max_iter=200, diis_dim=8)

    def layout(th):
        return ccx.Layout.from_basis(lat["nmax"], lat["A"], lat["rho"], snm=lat["snm"], theta=th)

    def engine(L, th, precision, rebase):
        e = ccx.Engine(L, real=(pot == 0))  # the Minnesota V and Fock stay real at any twist
        e.generate(potential=pot)
        e.setup_t_amplitudes()
        e.prepare(precision=precision, rebase=rebase)
        return e

    def build(th, precision, rebase):
        return engine(layout(th), th, precision, rebase)

    # host threads: the C library releases the interpreter lock in every call, so the
    # layouts of the next batch are built while the current batch solves, and a batch's
    # engines are set up side by side (each on its own stream)
    workers = ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)))
    ahead = ThreadPoolExecutor(max_workers=1)

    # engines per batch: the device memory of one prepared engine of the largest twist
    probe = build(grid[0][0], prec, rb)
    per = probe.memory()
    probe.close()
    del probe
    torch.cuda.synchronize()
    free = torch.cuda.mem_get_info()[0]
    wave = max(1, min(len(grid), int(0.9 * free / (per * 1.15))))

    # two batches in flight: the next batch's engines are built (layouts on host threads,
    # interaction generated and operands prepared on their own streams) while the current
    # batch solves, so each batch takes half of what the device holds
    batch = max(1, wave // 2)
    if args.twist_batch:
        batch = min(batch, args.twist_batch)

    def build_batch(w0):
        ths = [th for th, _ in grid[w0:w0 + batch]]
        return list(workers.map(lambda th: build(th, prec, rb), ths))

    def batched_pass():
        """All twists, batch after batch; returns (total_s, solve_s, results)."""
        res = [None] * len(grid)
        solve_s = 0.0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nxt = ahead.submit(build_batch, 0)
        for w0 in range(0, len(grid), batch):
            engines = nxt.result()
            if w0 + batch < len(grid):
                nxt = ahead.submit(build_batch, w0 + batch)
            t1 = time.perf_counter()
            rs, _ = ccx.ccd_iter_batch(engines, **opts)
            solve_s += time.perf_counter() - t1
            for k, (e, r) in enumerate(zip(engines, rs)):
                res[w0 + k] = (e.e0(), r)
                e.close()
            del engines
        torch.cuda.synchronize()
        return time.perf_counter() - t0, solve_s, res

    def sequential_pass(idx, precision, rebase, sample_clocks=False):
        """The twists idx one after the other, one engine at a time."""
        res = {}
        solve_s = 0.0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in idx:
            e = build(grid[k][0], precision, rebase)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            r = e.ccd_iter(mode=ccx.MODE_STANDARD, precision=precision, rebase=rebase, tol=args.tol, max_iter=200,
                           diis_dim=8)
            solve_s += time.perf_counter() - t1
            res[k] = (e.e0(), r)
            e.close()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, solve_s, res

    def twist_average(res_by_index):
        wsum = sum(grid[k][1] for k in res_by_index)
        return sum(grid[k][1] * (e0 + r["e_ccd"]).real / lat["A"] for k, (e0, r) in res_by_index.items()) / wsum

    for _ in range(args.warmup if args.warmup < 2 else 1):
        batched_pass()
    clocks = ClockSampler(0)
    tot, sol = [], []
    for _ in range(args.steps):
        t, so, res = batched_pass()
        tot.append(t)
        sol.append(so)
    clk = clocks.stop()
    res_b = {k: v for k, v in enumerate(res)}
    ea = twist_average(res_b)
    # the same form, per twist in sequence (one pass)
    seq_t, seq_s, res_s = sequential_pass(range(len(grid)), prec, rb)
    ea_seq = twist_average(res_s)
    # plain FP64 on a seeded sample of the twists, scaled to all of them
    rng = random.Random(20261203)
    sample = sorted(rng.sample(range(len(grid)), min(args.plain_twists, len(grid))))
    p_t, p_s, res_p = sequential_pass(sample, 0, ccx.REBASE_FP64)
    scale = len(grid) / len(sample)
    d_kev = max(abs((res_p[k][0] + res_p[k][1]["e_ccd"]).real - (res_b[k][0] + res_b[k][1]["e_ccd"]).real)
                / lat["A"] for k in sample) * 1e3
    value = statistics.median(tot)
    line = {"metric": METRIC, "impl": "ours", "value": value, "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128" if pot else "f64", "data": "synthetic",
            "config": {"workload": f"twist-averaged {lat['desc']}, {len(grid)} twists of the 4x4x4 "
                                   f"Gauss-Legendre grid on [-pi, pi]^3",
                       "form": f"{args.precision} + {args.rebase} re-bases, lockstep batches of {batch} twists, "
                               f"the next batch built while one solves",
                       "start": "MP2 (the learned start is not used: it costs an iteration here)",
                       "solver": f"Jacobi + DIIS(8) to ||R-DT||<{args.tol:g} (FP64 residual) per twist"},
            "twists": len(grid), "twists_per_batch": batch, "device_GB_per_twist": per / 1e9,
            "total_s": value, "solve_s": statistics.median(sol),
            "sequential_same_form": {"total_s": seq_t, "solve_s": seq_s},
            "speedup_batched_vs_sequential_solve": seq_s / statistics.median(sol),
            "plain_fp64_gpu": {"twists_timed": len(sample), "total_s_sample": p_t, "solve_s_sample": p_s,
                               "total_s_scaled": p_t * scale, "solve_s_scaled": p_s * scale,
                               "iterations": [res_p[k][1]["iterations"] for k in sample]},
            "speedup_vs_plain_fp64_gpu": p_t * scale / value,
            "iterations": [res_b[k][1]["iterations"] for k in range(len(grid))],
            "E_per_A_twist_averaged_MeV": ea,
            "dE_per_A_keV_batched_vs_sequential": abs(ea - ea_seq) * 1e3,
            "max_dE_per_A_keV_vs_fp64_on_sample": d_kev,
            "clocks": clk}
    workers.shutdown()
    ahead.shutdown()
    print(json.dumps(line), flush=True)
    return 0


def run_learned(args):
    """The learned warm start over a density sweep (17 densities 0.04 .. 0.20 fm^-3 of one
    lattice at seeded twists).  The network is trained on the even-indexed densities of
    the training twists, each sample with its prior: the converged-minus-MP2 correction
    interpolated from the even densities on either side.  On held-out twists, the even
    densities are converged from MP2, and every odd density is solved twice to ||R - D T||
    < tol: from MP2 and from the network with the prior of its two even neighbours.  Both
    reach the same E/A; the report gives the iterations and device seconds of both."""
    import random
    import torch
    ccx = load_pkg()
    lat = TWIST_LATTICES[args.lattice]
    rhos = [round(0.04 + 0.01 * k, 2) for k in range(17)]
    rng = random.Random(20261203)
    twists = [tuple(rng.uniform(-math.pi, math.pi) for _ in range(3)) for _ in range(32)]
    train_tw, eval_tw = twists[:args.learn_twists], twists[args.learn_twists:args.learn_twists + args.eval_twists]
    prec = PRECISIONS[args.precision]
    rb = ccx.REBASE_DIGITS if (prec and args.rebase == "digits") else ccx.REBASE_FP64
    opts = dict(mode=ccx.MODE_STANDARD, precision=prec, rebase=rb, tol=args.tol, max_iter=200, diis_dim=8)
    ref_opts = dict(mode=ccx.MODE_REFERENCE, tol=1e-6, max_iter=100)

    def converged(rho, th):
        L = ccx.Layout.from_basis(lat["nmax"], lat["A"], rho, snm=lat["snm"], theta=th)
        e = ccx.Engine(L, real=True)
        e.generate(potential=lat.get("potential", 0))
        e.setup_t_amplitudes()
        r = e.ccd_iter(**opts)
        return e, r

    lrn = ccx.Learner(seed=20261203)
    stride = max(1, args.learn_stride)
    t0 = time.perf_counter()
    for th in train_tw:
        even = {k: converged(rhos[k], th)[0] for k in range(0, 17, 2)}
        for k, e in even.items():
            nb = [j for j in (k - 2, k + 2) if j in even]
            lrn.set_prior(e, [even[j] for j in nb], [1.0 / len(nb)] * len(nb))
            lrn.add_solution(e, stride=stride)
        for e in even.values():
            e.close()
    loss = lrn.train(steps=args.learn_steps, batch=8192, lr=2e-3, seed=1)
    train_s = time.perf_counter() - t0
    rows = []
    for th in eval_tw:
        even = {k: converged(rhos[k], th)[0] for k in range(0, 17, 2)}
        for k in range(1, 17, 2):
            e, _ = converged(rhos[k], th)  # the first solve also prepares the engine
            e.setup_t_amplitudes()
            r_mp2 = e.ccd_iter(**opts)
            lrn.set_prior(e, [even[k - 1], even[k + 1]], [0.5, 0.5])
            # the residual norm at each start: one FP64 residual evaluation
            e.setup_t_amplitudes()
            s_mp2 = e.ccd_iter(mode=ccx.MODE_STANDARD, tol=args.tol, max_iter=1)["res_norm"]
            lrn.warm_start(e)
            s_ml = e.ccd_iter(mode=ccx.MODE_STANDARD, tol=args.tol, max_iter=1)["res_norm"]
            lrn.warm_start(e)
            r_ml = e.ccd_iter(**opts)
            ea_mp2 = (e.e0() + r_mp2["e_ccd"]).real / lat["A"]
            ea_ml = (e.e0() + r_ml["e_ccd"]).real / lat["A"]
            # the reference's own loop (FP64, mixing + DIIS every 6th step, |dE| < 1e-6 MeV)
            e.setup_t_amplitudes()
            q_mp2 = e.ccd_iter(**ref_opts)
            lrn.warm_start(e)
            q_ml = e.ccd_iter(**ref_opts)
            dq = max(abs((e.e0() + q["e_ccd"]).real / lat["A"] - ea_mp2) * 1e3 for q in (q_mp2, q_ml))
            rows.append((r_mp2["iterations"], r_ml["iterations"], r_mp2["seconds"], r_ml["seconds"],
                         abs(ea_ml - ea_mp2) * 1e3, r_mp2["converged"] and r_ml["converged"],
                         r_mp2["fp64_sweeps"], r_ml["fp64_sweeps"], s_mp2, s_ml,
                         q_mp2["iterations"], q_ml["iterations"], q_mp2["seconds"], q_ml["seconds"], dq,
                         q_mp2["converged"] and q_ml["converged"]))
            e.close()
        for x in even.values():
            x.close()
    it0 = sum(x[0] for x in rows) / len(rows)
    it1 = sum(x[1] for x in rows) / len(rows)
    s0 = sum(x[2] for x in rows)
    s1 = sum(x[3] for x in rows)
    line = {"metric": "CCD iterations and device seconds to ||R - D T|| < %g (and in the reference's own loop), "
                      "learned vs MP2 start" % args.tol,
            "impl": "ours", "lattice": lat["desc"], "densities": rhos, "train_twists": len(train_tw),
            "eval_twists": len(eval_tw), "held_out_solves": len(rows),
            "form": args.precision + (" + " + args.rebase + " re-bases" if prec else ""),
            "training": {"samples": lrn.samples(), "stride": stride, "steps": args.learn_steps, "loss": loss,
                         "seconds_incl_solves": train_s},
            "iterations_mp2_mean": it0, "iterations_learned_mean": it1,
            "solve_s_mp2_total": s0, "solve_s_learned_total": s1, "speedup_learned": s0 / s1 if s1 else None,
            "fewer_iterations_on": sum(1 for x in rows if x[1] < x[0]), "more_iterations_on": sum(1 for x in rows if x[1] > x[0]),
            "max_dE_per_A_keV": max(x[4] for x in rows), "all_converged": all(x[5] for x in rows),
            "fp64_rebases_mp2_mean": sum(x[6] for x in rows) / len(rows),
            "fp64_rebases_learned_mean": sum(x[7] for x in rows) / len(rows),
            "start_residual_ratio_learned_over_mp2_median": statistics.median(x[9] / x[8] for x in rows),
            "reference_loop": {
                "stop": "|dE| < 1e-6 MeV, 0.75/0.25 mixing, DIIS every 6th iteration, FP64 (ccm_iter.f90:67-96)",
                "iterations_mp2_mean": sum(x[10] for x in rows) / len(rows),
                "iterations_learned_mean": sum(x[11] for x in rows) / len(rows),
                "solve_s_mp2_total": sum(x[12] for x in rows), "solve_s_learned_total": sum(x[13] for x in rows),
                "fewer_iterations_on": sum(1 for x in rows if x[11] < x[10]),
                "more_iterations_on": sum(1 for x in rows if x[11] > x[10]),
                "max_dE_per_A_keV_vs_tight": max(x[14] for x in rows), "all_converged": all(x[15] for x in rows)}}
    print(json.dumps(line), flush=True)
    return 0


def run_precision_sweep(args, wl):
    """Mixed-precision variants of one lattice against its plain FP64 solve: BF16x3 and
    TF32x3 corrections with the adaptive re-base policy (drop factors 1e-4, 1e-5, 1e-6)
    and with a fixed defect period k in {1, 2, 4, 8, 16}, digit-product re-bases.  For each:
    iterations, FP64 re-bases, device seconds (best of --steps solves) and the E/A
    difference to the FP64 solve in keV."""
    import torch
    ccx = load_pkg()
    L = ccx.Layout.from_basis(wl["nmax"], wl["A"], wl["rho"], snm=wl["snm"])
    real = wl["potential"] == ccx.POT_MINNESOTA
    e = ccx.Engine(L, real=real)
    e.generate(potential=wl["potential"])

    def solve(precision, **kw):
        best = None
        for _ in range(max(1, args.steps)):
            e.setup_t_amplitudes()
            r = e.ccd_iter(mode=ccx.MODE_STANDARD, precision=precision, tol=args.tol, max_iter=200, diis_dim=8,
                           rebase=ccx.REBASE_DIGITS if precision else ccx.REBASE_FP64, **kw)
            if best is None or r["seconds"] < best["seconds"]:
                best = r
        return best

    r64 = solve(0)
    ea64 = (e.e0() + r64["e_ccd"]).real / wl["A"]
    variants = [("bf16x3", 1, dict()), ("bf16x3", 1, dict(rebase_drop=1e-5)), ("bf16x3", 1, dict(rebase_drop=1e-6)),
                ("tf32x3", 2, dict()), ("tf32x3", 2, dict(rebase_drop=1e-6))]
    variants += [("bf16x3", 1, dict(defect_period=k)) for k in (1, 2, 4, 8, 16)]
    rows = []
    for name, pr, kw in variants:
        solve(pr, **kw)  # warm-up: operand tiles of this kind
        r = solve(pr, **kw)
        ea = (e.e0() + r["e_ccd"]).real / wl["A"]
        rows.append({"precision": name, "policy": kw or {"rebase_drop": 1e-4}, "converged": r["converged"],
                     "iterations": r["iterations"], "fp64_rebases": r["fp64_sweeps"], "seconds": r["seconds"],
                     "speedup_vs_fp64": r64["seconds"] / r["seconds"], "dE_per_A_keV": abs(ea - ea64) * 1e3})
    line = {"metric": "mixed-precision variants vs plain FP64 GPU", "impl": "ours", "workload": wl["desc"],
            "tol": args.tol, "fp64": {"iterations": r64["iterations"], "seconds": r64["seconds"], "E_per_A_MeV": ea64},
            "variants": rows}
    print(json.dumps(line), flush=True)
    return 0


def run_triples(args, wl):
    """CCD + (T) of one lattice: the mixed-precision CCD solve (digit-product re-bases) and
    the plain FP64 one, then (T) on the converged amplitudes with FP32 contractions (the
    default) and with FP64 contractions.  Reports the seconds of each, the CCD E/A of both
    solves and the relative differences of E(T) between the forms."""
    import torch
    ccx = load_pkg()
    L = ccx.Layout.from_basis(wl["nmax"], wl["A"], wl["rho"], snm=wl["snm"])
    real = wl["potential"] == ccx.POT_MINNESOTA
    e = ccx.Engine(L, real=real)
    e.generate(potential=wl["potential"])
    out = {}
    for name, prec in (("fp64", 0), ("mixed", 1)):
        e.setup_t_amplitudes()
        r = e.ccd_iter(mode=ccx.MODE_STANDARD, precision=prec, tol=args.tol, max_iter=200, diis_dim=8,
                       rebase=ccx.REBASE_DIGITS if prec else ccx.REBASE_FP64)
        ts = {}
        for tname, fp32 in (("fp32", True), ("fp64", False)):
            e.set_triples_precision(fp32)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            et = e.pert_triples()
            ts[tname] = {"seconds": time.perf_counter() - t0, "E_T_MeV": et.real}
        out[name] = {"ccd_seconds": r["seconds"], "iterations": r["iterations"],
                     "E_per_A_MeV": (e.e0() + r["e_ccd"]).real / wl["A"], "triples": ts}
    ref = out["fp64"]["triples"]["fp64"]["E_T_MeV"]
    line = {"metric": "CCD + (T) seconds and FP64-stated errors", "impl": "ours", "workload": wl["desc"],
            "tol": args.tol, "forms": out,
            "dE_per_A_keV_mixed_vs_fp64": abs(out["mixed"]["E_per_A_MeV"] - out["fp64"]["E_per_A_MeV"]) * 1e3,
            "rel_dE_T_fp32_contractions": abs(out["fp64"]["triples"]["fp32"]["E_T_MeV"] - ref) / abs(ref),
            "rel_dE_T_mixed_ccd_fp32_contractions": abs(out["mixed"]["triples"]["fp32"]["E_T_MeV"] - ref) / abs(ref),
            "triples_pairs_note": "E(T) is summed over every (abc, ijk) pair of the triple channels"}
    if args.triples_cpu_s > 0:
        line["cpu_baseline"] = triples_cpu_sample(wl, args.triples_cpu_s)
    print(json.dumps(line), flush=True)
    return 0


def triples_cpu_sample(wl: dict, budget_s: float) -> dict:
    """Seconds of the oracle's pert_triples2 (the reference algorithm, complex<double>) on
    the whole lattice on all host cores, extrapolated by (abc, ijk) pairs from every k-th
    (abc) triple of every triple channel, k refined from short samples until the sample
    takes about budget_s.  The amplitudes are MP2's: the work of a pair does not depend
    on the values."""
    O, o = oracle_build(wl)
    n_ch, total = o.triples_channels(), o.triples_count()
    # a short first sample; the per-channel overhead makes it look slower per pair, so the
    # stride is refined until the sample takes at least half the budget
    nxt = 4096
    for _ in range(4):
        stride = nxt
        t = time.perf_counter()
        _, pairs = o.triples_sample(stride // 2, stride)
        secs = time.perf_counter() - t
        if secs >= 0.5 * budget_s or stride == 1:
            break
        nxt = max(1, int(stride * secs / budget_s))
    value = secs * total / max(pairs, 1)
    return {"value": value, "unit": "s", "cores": O.num_threads(), "kind": "port",
            "sample": (f"(T) of the oracle over every {stride}-th (abc) triple of all {n_ch} triple channels "
                       f"({pairs} of {total} (abc, ijk) pairs, {secs:.1f} s), extrapolated by pairs; "
                       f"MP2 amplitudes")}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="snm132n4", choices=sorted(WORKLOADS))
    ap.add_argument("--plain-steps", type=int, default=2, help="timed plain FP64 solves beside the headline form")
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--triples-cpu-s", type=float, default=20.0,
                    help="--triples: seconds of oracle (T) sampled for the CPU baseline (0: none)")
    ap.add_argument("--precision", default="bf16x3", choices=sorted(PRECISIONS))
    ap.add_argument("--defect-period", type=int, default=0, help="FP64 re-base every k iterations (0: adaptive)")
    ap.add_argument("--twists", type=int, default=0,
                    help="run the twist-batch comparison with this many twists instead of the headline")
    ap.add_argument("--lattice", default="snm132n3chiral", choices=sorted(TWIST_LATTICES))
    ap.add_argument("--twist-batch", type=int, default=0, help="cap on the twists per lockstep batch (0: memory)")
    ap.add_argument("--plain-twists", type=int, default=4, help="twists of the plain FP64 GPU sample")
    ap.add_argument("--rebase", default="digits", choices=["fp64", "digits"],
                    help="pp-ladder product of a re-base: FP64 FMA GEMM or exact digit products on the tensor cores")
    ap.add_argument("--learned", action="store_true",
                    help="run the learned-warm-start density sweep on --lattice instead of the headline")
    ap.add_argument("--learn-twists", type=int, default=4)
    ap.add_argument("--eval-twists", type=int, default=4)
    ap.add_argument("--learn-steps", type=int, default=3000)
    ap.add_argument("--learn-stride", type=int, default=4, help="every k-th amplitude as a training sample")
    ap.add_argument("--triples", action="store_true", help="run CCD + (T) on --workload instead")
    ap.add_argument("--precision-sweep", action="store_true",
                    help="run the mixed-precision variants of --workload against its FP64 solve instead")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.learned and args.impl == "ours":
        return run_learned(args)
    if args.precision_sweep and args.impl == "ours":
        return run_precision_sweep(args, wl)
    if args.triples and args.impl == "ours":
        return run_triples(args, wl)
    if args.twists > 0 and args.impl == "ours":
        return run_twists(args)
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_ours(args, wl)


if __name__ == "__main__":
    sys.exit(main())
