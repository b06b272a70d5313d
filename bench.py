#!/usr/bin/env python3
"""Throughput of the GB300 RPMD step in bead-molecule-steps/s.

Workload (one "step" = one outer evolve_pi step, evolve_pi.f90:1-322):
q-SPC/Fw water, 4096 H2O on a 16^3 CUB lattice (L = 49.71 A, rho = 0.997
g/cm^3), nb = 32 beads, T = 298 K, MTS = 5 (dt = 1.25 fs outer, 0.25 fs inner),
ring-polymer contraction: Ewald on the centroid (nbdf1 = 1), Lennard-Jones on
5 normal modes (nbdf2 = 5; the reference requires an odd count), intramolecular
forces on all 32 beads.  Inputs are synthetic: the reference's deterministic
CUB lattice and momenta drawn from the reference's ran2/gaussian stream
(sample_rpmd) after an initial full_forces.

--precision mixed (default): FP32 pair / reciprocal / transform arithmetic with
        compensated sums, FP64 state, propagator, energies and virials; the
        plain-FP64 arm is timed in the same run ("fp64_arm", "mixed_over_fp64")
        and the force error against it is reported ("error_vs_fp64").
--precision fp64: the plain-FP64 path alone.
value:  nb * nm * K / (sum of the K steps' CUDA-event times), state resident in
        HBM, L2 flushed (256 MiB write) between steps outside the timed events.
e2e:    the same metric through the drop-in C-ABI call gbrpmd_evolve_pi with
        pinned host arrays: p, r, dvdr, dvdr2 copied in and out every step.
--impl reference: the reference's algorithm on the host CPU (the C++
        restatement in oracle/, since the Fortran reference has no compiler
        here), one independent trajectory per host thread.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PARAM = os.path.join(ROOT, "tests", "golden", "params", "param_qspcfw")
WORKLOADS = {
    "qspcfw_4096_nb32_mts5_contracted": dict(ncell=(16, 16, 16), nb=32, mts=5, dtfs=1.25, nbdf1=1, nbdf2=5),
    "qspcfw_216_nb32": dict(ncell=(6, 6, 6), nb=32, mts=1, dtfs=0.5),
}
DEFAULT = "qspcfw_4096_nb32_mts5_contracted"
# multi-trajectory workloads (rpmd_mainz_gb300/workloads.py)
BATCH_WORKLOADS = ("replicas_256", "served_stream", "qspcfw_216_nb32_nve")
REGIONS = ["mts_block", "pair_lists", "ewald_real", "recip_sk", "recip_weights", "recip_force", "lj",
           "tem", "expand_kick", "msite", "rattle"]
# algorithmic flops per work unit of a region (declared weights):
# real-space in-cut pair 60; reciprocal (k vector, site) 12 with kz and -kz
# taken together: 4 in the structure-factor pass (two complex-times-real FMAs
# per pair of vectors), 8 in the force pass (eight FMAs per pair of vectors);
# LJ pair 45
PROF_STEPS = 10
FLOPS_PER_UNIT = {"ewald_real": 60.0, "recip_sk": 4.0, "recip_force": 8.0, "lj": 45.0}
# the multiple-time-step block streams the FP64 state: r, p, dvdr, dvdr2 read
# and written once per outer step, 8 arrays x 3 coordinates x 8 bytes per
# bead-atom = 576 bytes per bead-molecule (its ALU work is a few flops per byte)
BYTES_PER_BEAD_MOLECULE = {"mts_block": 576.0}
# regions whose kernel can be watched inside the timed (graph-replayed) steps
WATCHABLE = ("mts_block", "ewald_real", "recip_force", "lj")
FALLBACK_HBM_GBS = 6800.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, torch):
    """The slowest rank's value on every rank (all-reduce MAX on the process
    group's device: CUDA for NCCL, host for gloo); x itself when world is 1."""
    if world <= 1:
        return float(x)
    dev = "cuda" if torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank_step, steps, world, total_ms):
    """Whole-job throughput: every rank's units over the slowest rank's time
    (replicas only: each rank advances its own trajectory, weak scaling)."""
    return world * steps * units_per_rank_step / (total_ms * 1e-3)


def make_system(name):
    from rpmd_mainz_gb300 import lib, system

    cfg = WORKLOADS[name]
    s = system.water_box(PARAM, **cfg)
    lib.init(s["params"])
    irun = C.c_int(-4711)
    s["p"] = system.sample_momenta(s["na"], s["nb"], s["mass"], s["beta"], irun)
    return s


def make_system_oracle(name):
    """The same workload set up by the oracle's own restatement of the
    reference's set-up (setup_box_size, the CUB lattice, setup_ewald,
    sample_rpmd from seed -4711): the reference arm loads no product code."""
    from tests import oracle_lib as orc
    from tests import systems

    s = systems.build(param="param_qspcfw", **WORKLOADS[name])
    s["p"] = orc.sample_rpmd(s["na"], s["nb"], s["mass"], s["beta"], orc.Rng(4711))
    return s


def workload_config(name, s):
    """The `config` of both arms: the workload and its sizes only."""
    return {"workload": name, "nm": s["nm"], "nb": s["nb"], "mts": s["params"].mts, "nbdf1": s["params"].nbdf1,
            "nbdf2": s["params"].nbdf2,
            "l2": "GPU arm: 256 MiB written between timed steps (L2 flush), outside the timed events",
            "parallelism": "replicas only: one trajectory per GPU, one per host thread on the CPU"}


def measured_hbm_peak():
    """HBM copy bandwidth from MEASURED_PEAKS.json, else the fallback figure."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            v = float(json.load(f)["hbm_gbs"])
        return v, "measured (MEASURED_PEAKS.json hbm_gbs: STREAM-style copy on this pool's GB300)"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback (no MEASURED_PEAKS.json): 6.8 TB/s, one earlier GB300 measurement"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) >= 9:
                for k, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(k)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops(torch):
    """Measured FP64 peak: cuBLAS DGEMM 8192^3 (2 N^3 flops), best of 3."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def fp32_peak_tflops(torch):
    """Measured FP32 CUDA-core peak: cuBLAS SGEMM 8192^3 with TF32 off, best of 3."""
    n = 8192
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(n, n, dtype=torch.float32, device="cuda")
    b = torch.randn(n, n, dtype=torch.float32, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    torch.backends.cuda.matmul.allow_tf32 = old
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def read_profile_traffic(region, precision):
    """DRAM bytes per launch of `region` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#") and parts[0] == region and parts[1] == precision:
            try:
                return float(parts[2])
            except ValueError:
                return None
    return None


def cpu_baseline(s, seconds_target=15.0):
    """The oracle port on the host cores: one trajectory per thread, bounded sample."""
    from tests import oracle_lib as orc

    orc.set_params(s["params"])
    ff = orc.full_forces(s["r"], s["box"], s["z"])
    st = orc.State(s["r"], s["p"], ff["dvdr"], ff["dvdr2"], s["box"])
    threads = os.cpu_count() or 1
    t1 = orc.bench_replicas(1, st, s["dt"], s["mass"], s["z"], s["beta"], 1)
    steps = max(1, min(20, int(seconds_target / max(t1, 1e-3))))
    wall = orc.bench_replicas(threads, st, s["dt"], s["mass"], s["z"], s["beta"], steps)
    value = threads * steps * s["nb"] * s["nm"] / wall
    return {"value": value, "unit": "bead-molecule-steps/s", "cores": threads, "kind": "port",
            "sample": f"{threads} independent trajectories x {steps} evolve_pi steps of the same workload "
                      f"(one per host thread, {wall:.1f} s wall); single-thread step {t1:.2f} s"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    s = make_system_oracle(args.workload)
    from tests import oracle_lib as orc

    orc.set_params(s["params"])
    ff = orc.full_forces(s["r"], s["box"], s["z"])
    st = orc.State(s["r"], s["p"], ff["dvdr"], ff["dvdr2"], s["box"])
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        orc.bench_replicas(threads, st, s["dt"], s["mass"], s["z"], s["beta"], 1)
    times = []
    for _ in range(args.steps):
        times.append(orc.bench_replicas(threads, st, s["dt"], s["mass"], s["z"], s["beta"], 1))
    total = sum(times)
    value = threads * args.steps * s["nb"] * s["nm"] / total
    out = {
        "impl": "reference", "metric": "bead-molecule-steps/s", "value": value, "unit": "bead-molecule-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.workload, s),
        "cpu_baseline": {"value": value, "unit": "bead-molecule-steps/s", "cores": threads, "kind": "port",
                         "sample": f"each step: {threads} host threads advance one independent trajectory by one "
                                   f"evolve_pi step (C++ restatement of the Fortran reference)"},
        "e2e": {"value": value, "unit": "bead-molecule-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "p50_ms": 1e3 * statistics.median(times), "p99_ms": 1e3 * float(np.percentile(times, 99)),
    }
    print(json.dumps(out), flush=True)
    return 0


def set_precision(s, prec):
    from rpmd_mainz_gb300 import lib

    s["params"].precision = prec
    lib.init(s["params"])


def measure(args, s, prec, torch, world, local):
    """One arm on the resident context: profiled pass, timed steps, e2e drop-in."""
    from rpmd_mainz_gb300 import lib

    set_precision(s, prec)
    na, nb, nm = s["na"], s["nb"], s["nm"]
    ff = lib.full_forces(s["r"], s["box"], s["z"])
    ctx = lib.Context(na, nb, s["mass"], s["z"])
    ctx.upload(r=s["r"], p=s["p"], dvdr=ff["dvdr"], dvdr2=ff["dvdr2"], box=s["box"])
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # launch shapes for this system (gbrpmd_ctx_autotune), outside the timed region
    t_tune = time.perf_counter()
    tune = ctx.autotune(s["dt"], s["beta"], steps=5) if not args.no_autotune else None
    t_tune = time.perf_counter() - t_tune
    for _ in range(args.warmup):
        ctx.evolve(1, s["dt"], s["beta"])
    ctx.sync()

    # profiled pass (not timed): per-region CUDA-event times for the roofline,
    # averaged over PROF_STEPS steps so that skin-list rebuilds enter at their rate
    lib.load().gbrpmd_ctx_set_profiling(ctx.h, 1)
    ctx.evolve(PROF_STEPS, s["dt"], s["beta"])
    ctx.sync()
    R = len(REGIONS)
    ms, units, cnt = np.zeros(R), np.zeros(R), np.zeros(R, dtype=np.int32)
    lib.load().gbrpmd_ctx_region_times(ctx.h, lib._ptr(ms), lib._ptr(units), cnt.ctypes.data_as(C.POINTER(C.c_int)),
                                       C.c_int(R))
    lib.load().gbrpmd_ctx_set_profiling(ctx.h, 0)
    ctx.evolve(2, s["dt"], s["beta"])  # re-capture the step graph outside the timed region
    ctx.sync()
    regions = {REGIONS[i]: {"ms": float(ms[i]) / PROF_STEPS, "launches": int(cnt[i]) / PROF_STEPS,
                            "units": float(units[i]) / PROF_STEPS}
               for i in range(R) if cnt[i]}
    # the dominant kernel region of the profiled pass is watched in the timed
    # steps: timing events around its launch, captured into the step graph
    dom = max((k for k in regions if k in WATCHABLE), key=lambda k: regions[k]["ms"])
    if args.watch != "auto" and args.watch in regions:
        dom = args.watch
    ctx.watch(dom)
    ctx.evolve(2, s["dt"], s["beta"])  # capture the graph with the watch events
    ctx.sync()

    # timed region
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches
    rebuilds0 = ctx.list_rebuilds()
    step_ms, kern_ms = [], []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            ctx.evolve(1, s["dt"], s["beta"])
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            kern_ms.append(ctx.watch_ms())
    ctx.sync()
    torch.cuda.synchronize()
    ctx.watch(None)
    launches = ctx.launches - launches0
    rebuilds = [b - a for a, b in zip(rebuilds0, ctx.list_rebuilds())]
    total_ms = float(sum(step_ms))
    total_ms = max_over_ranks(total_ms, world, torch)
    if world > 1:
        torch.distributed.barrier()
    value = job_value(nb * nm, args.steps, world, total_ms)
    energies = ctx.energies()

    # e2e through the drop-in C ABI with pinned host buffers
    shape = (nb, na, 3)
    r_h, p_h, f_h, f2_h = (torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy() for _ in range(4))
    r0, p0, f0, f20 = ctx.download()
    r_h[:], p_h[:], f_h[:], f2_h[:] = r0, p0, f0, f20
    st = lib.State.__new__(lib.State)
    st.r, st.p, st.dvdr, st.dvdr2 = r_h, p_h, f_h, f2_h
    st.box = s["box"].copy()
    st.vir, st.vir_lf = np.zeros(9), np.zeros(9)
    lib.evolve_pi(st, s["dt"], s["mass"], s["z"], s["beta"])  # warm the drop-in context
    e2e_times = []
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        lib.evolve_pi(st, s["dt"], s["mass"], s["z"], s["beta"])
        e2e_times.append(time.perf_counter() - t0)
    e2e_value = world * nb * nm * len(e2e_times) / sum(e2e_times)
    nbytes = 4 * r_h.nbytes
    evolved = ctx.download()  # an evolved (non-lattice) state for the parity and error checks
    ctx.close()
    del flush
    return dict(value=value, total_ms=total_ms, step_ms=step_ms, launches=launches, rebuilds=rebuilds,
                energies=energies, regions=regions, clocks=clk.summary(), e2e_value=e2e_value, e2e_bytes=nbytes,
                tune=tune, tune_s=t_tune, dom=dom, kern_ms=kern_ms, evolved=evolved)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def force_error(s, r, box, on):
    """Relative RMS force error (total, low-frequency, worst bead) and energy and
    virial errors of the mixed path against the FP64 path on positions r."""
    from rpmd_mainz_gb300 import lib

    out = []
    for prec in (0, 1):
        set_precision(s, prec)
        out.append(lib.full_forces(r, box, s["z"]))
    f64, fmx = out
    t64, tmx = f64["dvdr"] + f64["dvdr2"], fmx["dvdr"] + fmx["dvdr2"]
    return {"force_rel_rms": rel(tmx, t64), "lowfreq_force_rel_rms": rel(fmx["dvdr"], f64["dvdr"]),
            "force_rel_rms_worst_bead": max(rel(tmx[k], t64[k]) for k in range(t64.shape[0])),
            "energy_rel": abs(fmx["v"] - f64["v"]) / abs(f64["v"]),
            "virial_rel": rel(fmx["vir"], f64["vir"]), "bound": 1e-5, "on": on}


def parity_vs_oracle(s, state):
    """One evolve_pi step of the plain-FP64 device path (the drop-in C ABI) and
    of the oracle from the same evolved state: relative L2 errors of r, p, dvdr,
    dvdr2 and of the energies and virial (bound 1e-10)."""
    from rpmd_mainz_gb300 import lib
    from tests import oracle_lib as orc

    r, p, f, f2 = state
    set_precision(s, 0)
    orc.set_params(s["params"])
    t0 = time.perf_counter()
    so = orc.State(r, p, f, f2, s["box"])
    eo = orc.evolve_pi(so, s["dt"], s["mass"], s["z"], s["beta"], orc.Rng(1))
    t_orc = time.perf_counter() - t0
    sd = lib.State(r, p, f, f2, s["box"])
    ed = lib.evolve_pi(sd, s["dt"], s["mass"], s["z"], s["beta"])
    errs = {k: rel(getattr(sd, k), getattr(so, k)) for k in ("r", "p", "dvdr", "dvdr2")}
    for k in ("v", "vew", "vlj", "vint"):
        errs[k] = abs(ed[k] - eo[k]) / max(abs(eo[k]), 1e-300)
    errs["vir"] = rel(sd.vir, so.vir)
    errs["vir_lf"] = rel(sd.vir_lf, so.vir_lf)
    worst = max(errs.values())
    return {"max_rel": worst, "bound": 1e-10, "ok": bool(worst <= 1e-10), "errors": errs,
            "on": "one evolve_pi step from the FP64 arm's final (evolved) state, plain-FP64 drop-in call vs oracle",
            "oracle_seconds": t_orc}


def run_replicas(args, torch):
    """256 independent NVT replicas (molecules in {64, 128, 216, 343, 512}, nb in
    {8, 16, 32, 64}, T in [250, 350] K, Andersen thresh 0.01, dt 0.5 fs): the
    mixed-precision batch (one CUDA-graph launch per step for all replicas)
    against the plain-FP64 contexts stepped in a loop (each on its own stream,
    all synchronised once per step)."""
    from rpmd_mainz_gb300 import lib, workloads

    reps = workloads.replica_set(n=args.replicas, precision=1)
    lib.init(reps[0]["params"])
    work = sum(s["nb"] * s["nm"] for s in reps)

    def contexts(prec):
        out = []
        for s in reps:
            prm = s["params"].copy()
            prm.precision = prec
            ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
            ctx.set_params(prm)
            ctx.upload(r=s["r"], p=s["p"], box=s["box"])
            ctx.full_forces()
            out.append(ctx)
        return out

    # mixed-precision batch
    ctxs = contexts(1)
    batch = lib.Batch()
    for i, (s, ctx) in enumerate(zip(reps, ctxs)):
        batch.add(ctx, s["dt"], s["beta"], 0.01, -(5000 + i))
    stream = torch.cuda.ExternalStream(batch.stream)
    # launch shapes per distinct replica shape (gbrpmd_batch_autotune), before the timed steps
    t_tune = time.perf_counter()
    lib.autotune_reset()
    batch.autotune(steps=5)
    t_tune = time.perf_counter() - t_tune
    shapes = {}
    for s, ctx in zip(reps, ctxs):
        ch = ctx.autotune(s["dt"], s["beta"], steps=5)  # cached: returns the choice
        key = f"nm{s['nm']}_nb{s['nb']}"
        shapes[key] = (f"ew_np={ch['ew_np']} lj_np={ch['lj_np']} rf_g={ch['rf_g']} rf_ns={ch['rf_ns']} "
                       f"mts_mpb={ch['mts_mpb']} skin={ch['skin']}")
    batch.step(args.warmup)
    batch.sync()
    step_ms = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            batch.step(1)
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
    batch.sync()
    value = args.steps * work / (sum(step_ms) * 1e-3)
    evolved = [c.download()[0] for c in ctxs[:8]]  # configurations for the force-error check
    batch.close()
    for c in ctxs:
        c.close()
    # the same replicas in plain FP64, batched the same way (like for like)
    ctxs = contexts(0)
    for c, s in zip(ctxs, reps):
        c.autotune(s["dt"], s["beta"], steps=3)
    batch = lib.Batch()
    for i, (s, ctx) in enumerate(zip(reps, ctxs)):
        batch.add(ctx, s["dt"], s["beta"], 0.01, -(5000 + i))
    stream64 = torch.cuda.ExternalStream(batch.stream)
    batch.step(args.warmup)
    batch.sync()
    b64_ms = []
    for _ in range(max(2, args.steps // 4)):
        with torch.cuda.stream(stream64):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream64)
        batch.step(1)
        with torch.cuda.stream(stream64):
            e1.record(stream64)
        e1.synchronize()
        b64_ms.append(e0.elapsed_time(e1))
    batch.sync()
    batch.close()
    fp64_batch_value = len(b64_ms) * work / (sum(b64_ms) * 1e-3)
    # and as a plain host loop over the contexts (each on its own stream, all
    # synchronised once per step)
    for c, s in zip(ctxs, reps):
        c.evolve(args.warmup, s["dt"], s["beta"])
    for c in ctxs:
        c.sync()
    loop_ms = []
    for _ in range(max(2, args.steps // 4)):
        t0 = time.perf_counter()
        for c, s in zip(ctxs, reps):
            c.evolve(1, s["dt"], s["beta"])
        for c in ctxs:
            c.sync()
        loop_ms.append(1e3 * (time.perf_counter() - t0))
    fp64_value = len(loop_ms) * work / (sum(loop_ms) * 1e-3)
    for c in ctxs:
        c.close()
    # force error of the mixed path on the first eight replicas' evolved
    # configurations (the starting lattices are symmetric: forces nearly cancel)
    errs = []
    for s, r in zip(reps[:8], evolved):
        out = []
        for prec in (0, 1):
            prm = s["params"].copy()
            prm.precision = prec
            lib.init(prm)
            out.append(lib.full_forces(r, s["box"], s["z"]))
        f64, fmx = out
        tot64 = f64["dvdr"] + f64["dvdr2"]
        errs.append(float(np.linalg.norm(fmx["dvdr"] + fmx["dvdr2"] - tot64) / np.linalg.norm(tot64)))
    return {
        "metric": "bead-molecule-steps/s", "value": value, "unit": "bead-molecule-steps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(step_ms)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 mixed",
        "data": "synthetic (CUB lattices, momenta from the reference's ran2 stream, seeded per replica)",
        "config": {"workload": "replicas_256", "replicas": len(reps), "bead_molecules_per_step": work,
                   "sizes": "nm in {64,128 (8x4x4 non-cubic box),216,343,512}, nb in {8,16,32,64}, T in [250,350] K",
                   "l2": "inputs larger than L2 in aggregate", "parallelism": "one batch, one graph per step"},
        "p50_ms": float(np.median(step_ms)), "p99_ms": float(np.percentile(step_ms, 99)),
        "autotune": {"seconds": t_tune, "distinct_shapes": len(shapes), "choices": shapes},
        "fp64_batch": {"value": fp64_batch_value, "ms_per_step": float(np.mean(b64_ms))},
        "fp64_loop": {"value": fp64_value, "ms_per_step": float(np.mean(loop_ms))},
        "batched_mixed_over_fp64_batch": value / fp64_batch_value,
        "batched_mixed_over_fp64_loop": value / fp64_value,
        "error_vs_fp64": {"force_rel_rms_max_of_8": max(errs), "bound": 1e-5,
                          "on": "the first 8 replicas after the timed steps"},
        "clocks": clk.summary(),
    }


def run_nve(args, torch):
    """Mixed precision on the 216-molecule, nb = 32 system (dt 0.5 fs, every
    bead, no contraction): the force / energy / virial error against the FP64
    path on 20 seeded snapshots (an FP64 Andersen NVT run from the lattice,
    one snapshot every 50 steps, thresh = 1/sqrt(1000) as md_eq sets it for
    ttaufs = 0), then `--nve-ps` of NVE (no thermostat) from the last snapshot
    with both paths, sampling the conserved RPMD energy nb*v + tk + vrp
    (md_eq.f90:274) every 100 steps; drift = least-squares slope."""
    from rpmd_mainz_gb300 import lib, system

    s = system.water_box(PARAM, ncell=(6, 6, 6), nb=32, mts=1, dtfs=args.nve_dtfs)
    irun = C.c_int(-4711)
    s["p"] = system.sample_momenta(s["na"], s["nb"], s["mass"], s["beta"], irun)
    na, nm, nb, dt, beta = s["na"], s["nm"], s["nb"], s["dt"], s["beta"]

    def params(prec, therm):
        prm = s["params"].copy()
        prm.precision = prec
        prm.therm = therm
        return prm

    lib.init(params(0, 1))
    ctx = lib.Context(na, nb, s["mass"], s["z"])
    ctx.set_params(params(0, 1))
    ctx.upload(r=s["r"], p=s["p"], box=s["box"])
    ctx.full_forces()
    seed = C.c_int(-2026)
    snaps = []
    for _ in range(20):
        ctx.run_md_eq(50, dt, beta, 1.0 / np.sqrt(1000.0), seed)
        snaps.append(ctx.download())
    ctx.close()
    per_bead, energy, virial, total = [], [], [], []
    for r, _, _, _ in snaps:
        out = []
        for prec in (0, 1):
            lib.init(params(prec, 0))
            out.append(lib.full_forces(r, s["box"], s["z"]))
        f64, fmx = out
        F64, Fmx = f64["dvdr"] + f64["dvdr2"], fmx["dvdr"] + fmx["dvdr2"]
        per_bead.append(float(max(np.linalg.norm(Fmx[k] - F64[k]) / np.linalg.norm(F64[k]) for k in range(nb))))
        total.append(float(np.linalg.norm(Fmx - F64) / np.linalg.norm(F64)))
        energy.append(abs(fmx["v"] - f64["v"]) / abs(f64["v"]))
        virial.append(float(np.linalg.norm(fmx["vir"] - f64["vir"]) / np.linalg.norm(f64["vir"])))

    r0, p0 = snaps[-1][0], snaps[-1][1]
    nsteps = int(round(args.nve_ps * 1000.0 / args.nve_dtfs))
    block = 100
    arms = {}
    for name, prec in (("mixed", 1), ("fp64", 0)):
        lib.init(params(prec, 0))
        c = lib.Context(na, nb, s["mass"], s["z"])
        c.set_params(params(prec, 0))
        c.upload(r=r0, p=p0, box=s["box"])
        c.full_forces()
        stream = torch.cuda.ExternalStream(c.stream)
        e_t, e_h, ms = [0.0], [c.estimators(beta)["econs"]], 0.0
        launches0 = c.launches
        with ClockSampler(0) as clk:
            for b in range(nsteps // block):
                with torch.cuda.stream(stream):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                c.evolve(block, dt, beta)
                with torch.cuda.stream(stream):
                    e1.record(stream)
                e1.synchronize()
                ms += e0.elapsed_time(e1)
                e_t.append((b + 1) * block * args.nve_dtfs * 1e-3)  # ps
                e_h.append(c.estimators(beta)["econs"])
        c.sync()
        t = np.array(e_t) * 1e-3  # ns
        e = np.array(e_h) * 2625.49963 / nm  # kJ/mol per molecule
        slope, icpt = np.polyfit(t, e, 1)
        e_ref = abs(float(e[0]))
        arms[name] = {"value": nsteps * nb * nm / (ms * 1e-3), "ms_per_step": ms / nsteps,
                      "drift_kjmol_per_ns_per_molecule": float(slope),
                      "drift_relative_per_ns": float(slope) / e_ref,
                      "fluctuation_rms_kjmol_per_molecule": float(np.std(e - (slope * t + icpt))),
                      "econs_first_last_kjmol_per_molecule": [float(e[0]), float(e[-1])],
                      "gpu_launches": int(c.launches - launches0 - (nsteps // block)), "clocks": clk.summary()}
        c.close()
    mx = arms["mixed"]
    return {
        "metric": "bead-molecule-steps/s", "value": mx["value"], "unit": "bead-molecule-steps/s", "n_gpus": 1,
        "steps": nsteps, "warmup": 0, "ms_per_step": mx["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 mixed",
        "data": "synthetic (CUB lattice, momenta from the reference's ran2 stream, FP64 Andersen NVT snapshots)",
        "config": {"workload": "qspcfw_216_nb32_nve", "nm": nm, "nb": nb, "dt_fs": args.nve_dtfs, "nve_ps": args.nve_ps,
                   "snapshots": len(snaps), "l2": "state smaller than L2 (resident NVE run, no flush)",
                   "parallelism": "single GPU"},
        "gpu_launches": mx["gpu_launches"],
        "error_vs_fp64": {"snapshots": len(snaps), "force_rel_rms_per_bead_max": max(per_bead),
                          "force_rel_rms_per_bead_median": float(np.median(per_bead)),
                          "force_rel_rms_total_max": max(total), "energy_rel_max": max(energy),
                          "virial_rel_max": max(virial), "bound": 1e-5},
        "nve": {"mixed": mx, "fp64": arms["fp64"]},
        "mixed_over_fp64": mx["value"] / arms["fp64"]["value"],
        "clocks": mx["clocks"],
    }


def serve_once(args, rate, n, seed):
    """One Poisson stream of `n` trajectory requests (mean `rate` per second)
    through the continuous-batching server; returns its measurements."""
    from rpmd_mainz_gb300 import lib, workloads

    stream = workloads.request_stream(n=n, rate=rate, seed=seed, nsteps=args.request_steps)
    lib.init(stream[0][1]["params"])
    work = sum(s["nb"] * s["nm"] * k for _, s, k in stream)
    srv = lib.Server(budget_bytes=args.budget_gb << 30, max_slots=args.slots)
    t0 = time.perf_counter()
    nxt = 0
    done = []
    shape, sidx = {}, {}
    with ClockSampler(0) as clk:
        while len(done) < len(stream):
            now = time.perf_counter() - t0
            while nxt < len(stream) and stream[nxt][0] <= now:
                _, s, k = stream[nxt]
                rid = srv.submit(s, s["r"], s["p"], k)
                shape[rid] = (s["nm"], s["nb"])
                sidx[rid] = nxt
                nxt += 1
            c = srv.counts()
            if c["active"] == 0 and c["queued"] == 0:
                time.sleep(max(0.0, min(0.01, stream[nxt][0] - now)) if nxt < len(stream) else 0.0)
                continue
            srv.tick(args.tick_steps)
            for res in srv.poll():
                if res["status"] != 0:
                    raise RuntimeError(f"request {res['id']} (nm, nb = {shape[res['id']]}) ended with status "
                                       f"{res['status']}: {lib.last_error()}")
                done.append(res)
    wall = time.perf_counter() - t0
    srv.close()
    lat = np.array([d["t_done"] for d in done])
    wait = np.array([d["t_admit"] for d in done])
    # force error of the mixed path on served final states: up to three rigid
    # and three flexible requests
    by_id = {d["id"]: d for d in done}
    ids = sorted(by_id)
    rigid_ids = [i for i in ids if stream[sidx[i]][1]["rigid"]][:3]
    flex_ids = [i for i in ids if not stream[sidx[i]][1]["rigid"]][:3]
    errs = {}
    for i in rigid_ids + flex_ids:
        s = stream[sidx[i]][1]
        out = []
        for prec in (0, 1):
            prm = s["params"].copy()
            prm.precision = prec
            lib.init(prm)
            out.append(lib.full_forces(by_id[i]["r"], s["box"], s["z"]))
        f64, fmx = out
        t64 = f64["dvdr"] + f64["dvdr2"]
        errs[i] = float(np.linalg.norm(fmx["dvdr"] + fmx["dvdr2"] - t64) / np.linalg.norm(t64))
    return {"value": work / wall, "requests": len(stream), "arrival_rate_per_s": rate,
            "rigid_requests": int(sum(1 for _, s, _ in stream if s["rigid"])),
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "queue_wait_p50": float(np.percentile(wait, 50)),
                          "queue_wait_p99": float(np.percentile(wait, 99))},
            "error_vs_fp64": {"force_rel_rms_max": max(errs.values()) if errs else None, "bound": 1e-5,
                              "on": f"final states of {len(rigid_ids)} rigid and {len(flex_ids)} flexible requests"},
            "wall_s": wall, "clocks": clk.summary()}


def run_served(args, torch):
    """Poisson arrivals of trajectory requests of mixed sizes (64-2048
    molecules, nb 4-64), half of them rigid 4-site water (evolve_rig_pi with
    RATTLE; TIP4P/Ice charges and LJ, M-site 0.1546 A), each `--request-steps`
    steps, served by the continuous-batching loop under a device-memory
    budget: once at 50 requests per second (beyond what the device sustains:
    throughput and the latency of a growing queue) and once at
    `--sustain-rate` (latency of a stream the device keeps up with)."""
    hot = serve_once(args, 50.0, args.requests, seed=7)
    kept = serve_once(args, args.sustain_rate, args.sustain_requests, seed=8)
    ps = 1e-3 * args.request_steps * 0.5  # dt = 0.5 fs
    return {
        "metric": "bead-molecule-steps/s", "value": hot["value"], "unit": "bead-molecule-steps/s", "n_gpus": 1,
        "steps": args.request_steps, "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 mixed", "data": "synthetic request streams (seeded Poisson arrivals, CUB lattices)",
        "config": {"workload": "served_stream", "requests": hot["requests"], "arrival_rate_per_s": 50.0,
                   "steps_per_request": args.request_steps,
                   "request_length": f"{ps:g} ps at dt 0.5 fs: the 20 ps requests scaled down {20.0 / ps:g}x so "
                                     f"that the stream ends in about a minute",
                   "tick_steps": args.tick_steps, "slots": args.slots, "budget_gib": args.budget_gb,
                   "sizes": "nm in 64..2048 (CUB lattices; 2048 on 16x16x8, a non-cubic box), nb in {4,8,16,32,64}",
                   "rigid_requests": hot["rigid_requests"],
                   "models": "flexible q-SPC/Fw (evolve_pi) and rigid 4-site water (evolve_rig_pi, RATTLE: qH "
                             "+0.5897 e, sigma 3.1668 A, epsilon 0.21084 kcal/mol, M-site 0.1546 A)"},
        "error_vs_fp64": hot["error_vs_fp64"],
        "latency_s": hot["latency_s"],
        "sustained": {k: kept[k] for k in ("value", "requests", "arrival_rate_per_s", "rigid_requests", "latency_s",
                                          "error_vs_fp64", "wall_s")},
        "wall_s": hot["wall_s"], "clocks": hot["clocks"],
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT, choices=sorted(WORKLOADS) + list(BATCH_WORKLOADS))
    ap.add_argument("--replicas", type=int, default=256)
    ap.add_argument("--requests", type=int, default=60)
    ap.add_argument("--request-steps", type=int, default=400)
    ap.add_argument("--sustain-rate", type=float, default=1.0, help="arrivals per second of the sustained stream")
    ap.add_argument("--sustain-requests", type=int, default=16)
    ap.add_argument("--tick-steps", type=int, default=10)
    ap.add_argument("--slots", type=int, default=32)
    ap.add_argument("--budget-gb", type=int, default=64)
    ap.add_argument("--nve-ps", type=float, default=10.0, help="NVE length of the qspcfw_216_nb32_nve workload")
    ap.add_argument("--nve-dtfs", type=float, default=0.5, help="time step (fs) of the qspcfw_216_nb32_nve workload")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-arm", action="store_true", help="skip the plain-FP64 comparison arm")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes instead of tuned ones")
    ap.add_argument("--no-parity", action="store_true", help="skip the one-step oracle parity check")
    ap.add_argument("--watch", default="auto", choices=("auto",) + WATCHABLE,
                    help="kernel region timed inside the timed steps (auto: the largest of the profiled pass)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import __graft_entry__ as g

    g.build()

    if args.workload in BATCH_WORKLOADS:
        if rank == 0:
            runner = {"replicas_256": run_replicas, "served_stream": run_served, "qspcfw_216_nb32_nve": run_nve}
            out = runner[args.workload](args, torch)
            print(json.dumps(out), flush=True)
        return 0

    s = make_system(args.workload)
    prec = 1 if args.precision == "mixed" else 0
    m = measure(args, s, prec, torch, world, local)
    fp64 = None
    f = None
    if prec == 0 or not args.no_fp64_arm:
        f = m if prec == 0 else measure(args, s, 0, torch, world, local)
    if prec == 1 and f is not None:
        fp64 = {"value": f["value"], "ms_per_step": f["total_ms"] / args.steps, "autotune": f["tune"],
                "p50_ms": float(np.median(f["step_ms"])), "p99_ms": float(np.percentile(f["step_ms"], 99)),
                "regions_ms_one_step": {k: v["ms"] for k, v in f["regions"].items()}}
    evolved = (f or m)["evolved"]
    err = force_error(s, evolved[0], s["box"], "the FP64 arm's final state (evolved from the lattice by the "
                      "autotune, warm-up, profiled and timed steps)") if prec == 1 else None
    parity = parity_vs_oracle(s, evolved) if (rank == 0 and not args.no_parity) else None
    regions = m["regions"]
    out = {
        "metric": "bead-molecule-steps/s", "value": m["value"], "unit": "bead-molecule-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": m["total_ms"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 mixed" if prec == 1 else "f64",
        "data": "synthetic (CUB lattice, Maxwell-Boltzmann momenta from the reference's ran2 stream)",
        "config": workload_config(args.workload, s),
        "precision": args.precision,
        "p50_ms": float(np.median(m["step_ms"])), "p99_ms": float(np.percentile(m["step_ms"], 99)),
        "gpu_launches": int(m["launches"]),
        "list_rebuilds": {"ewald": m["rebuilds"][0], "lj": m["rebuilds"][1], "tem": m["rebuilds"][2],
                          "skin": "0.1 of each cut-off; exact pair sets filtered from the skin list every step"},
        "e2e": {"value": m["e2e_value"], "unit": "bead-molecule-steps/s", "h2d_bytes_per_step": int(m["e2e_bytes"]),
                "d2h_bytes_per_step": int(m["e2e_bytes"] + 8 * 22),
                "path": "gbrpmd_evolve_pi drop-in, pinned host p/r/dvdr/dvdr2"},
        "energies_last_step": {k: m["energies"][k] for k in ("v", "vew", "vlj", "vint")},
        "autotune": {"choice": m["tune"], "seconds": m["tune_s"],
                     "note": "gbrpmd_ctx_autotune before the warm-up; the drop-in e2e context takes the cached shape"},
        "regions_ms_one_step": regions,
    }
    if fp64 is not None:
        out["fp64_arm"] = fp64
        out["mixed_over_fp64"] = m["value"] / fp64["value"]
    if err is not None:
        out["error_vs_fp64"] = err
    if parity is not None:
        out["parity_vs_oracle"] = parity
    if rank == 0:
        # roofline of the dominant kernel region (largest in the profiled pass),
        # its duration from the watch events around its launch in the timed steps
        dom = m["dom"]
        rr = regions[dom]
        kern_ms = float(np.mean(m["kern_ms"]))
        pname = "mixed" if prec == 1 else "fp64"
        common = {"kernel_region": dom, "kernel_ms_per_launch": kern_ms,
                  "kernel_ms_source": "CUDA events around the kernel's launch on its own stream, recorded inside "
                                      "each timed (graph-replayed) step; mean over the timed steps",
                  "traffic": read_profile_traffic(dom, pname)}
        if dom in BYTES_PER_BEAD_MOLECULE:
            peak, src = measured_hbm_peak()
            nbytes = BYTES_PER_BEAD_MOLECULE[dom] * s["nm"] * s["nb"]
            achieved = nbytes / (kern_ms * 1e-3) / 1e9
            out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                               "frac": achieved / peak, "peak_source": src, "bytes_per_launch": nbytes,
                               "bytes_per_unit": BYTES_PER_BEAD_MOLECULE[dom], "unit_of_work": "bead-molecule",
                               **common}
        else:
            units = rr["units"] / rr["launches"]
            achieved = FLOPS_PER_UNIT[dom] * units / (kern_ms * 1e-3) / 1e12
            if prec == 0:
                peak = fp64_peak_tflops(torch)
                src = "measured in this run: cuBLAS DGEMM 8192^3 (FP64 rate; MEASURED_PEAKS.json holds only HBM and BF16)"
            else:
                peak = fp32_peak_tflops(torch)
                src = ("measured in this run: cuBLAS SGEMM 8192^3 without TF32 (FP32 CUDA-core rate; "
                       "MEASURED_PEAKS.json holds only HBM and BF16)")
            out["roofline"] = {"bound": "fp64" if prec == 0 else "fp32", "achieved": achieved, "peak": peak,
                               "unit": "TFLOP/s", "frac": achieved / peak, "peak_source": src,
                               "flops_per_unit": FLOPS_PER_UNIT[dom], "units_per_launch": units, **common}
        out["clocks"] = m["clocks"]
        # the normal-mode transform of the workload's 3 na coordinate rows (nb = 32)
        # as the propagator runs it and on the tensor cores
        if s["nb"] == 32:
            from rpmd_mainz_gb300 import lib

            nm = lib.bench_nm_transform(3 * s["na"], reps=6)
            nm["rows"] = 3 * s["na"]
            nm["transforms_per_outer_step"] = 2 * s["params"].mts + 2
            out["nm_transform"] = nm
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(s)
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
