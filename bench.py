#!/usr/bin/env python
"""Benchmark of the GB300 gravity hot path.

Workload (one "step"): one all-pairs FP64 acceleration evaluation of the
16,385-body planetesimal disk (a 1 MSun star plus 16,384 bodies of 1e-9 MSun,
a uniform in 5..40 au, e Rayleigh 0.01, i Rayleigh 0.005; seeded synthetic
input), 268,451,840 interactions.

* ``value``: Ginteractions/s with inputs resident in GPU memory, timed with
  CUDA events on the launching stream, L2 flushed (256 MiB write) between
  timed steps outside the timed interval.
* ``e2e``: the same metric through the reference-facing C entry point
  ``ode_n_body_second_order`` on pinned host arrays: host-to-device copy of
  positions and masses, the kernels, device-to-host copy of the
  accelerations, every step.
* ``roofline``: the force kernel is bound by the FP64 pipe; the peak is the
  FMA throughput measured on this device by the library's probe kernel;
  ``achieved`` counts 20 flop per interaction.
* ``cpu_baseline``: the oracle (a C restatement of the reference's
  ode_n_body_second_order, bit-identical to it) on all host cores.
* ``ensemble``: Radau15 over a batch of independent planetary systems
  (system-steps/s), when --ensemble-systems > 0.

``--impl reference`` times the reference algorithm on the host cores instead
(the oracle port, since the reference library itself cannot be built on the
benchmark host) and prints the same line with "impl": "reference".

Multi-GPU (torchrun): every rank runs the same workload on its own GPU
(replicas, weak scaling); timing is the max over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from abie_gb300 import dist as D  # noqa: E402
from abie_gb300 import ics  # noqa: E402

G = ics.G_SOLAR
FLOP_PER_INTERACTION = 20  # the convention of the reference's tiled kernel comments
FP64_INSTR_PER_INTERACTION = 6  # the fast form's pair term (abie_gb300/csrc/common.cuh pair_fast)
# From one ncu capture of this workload's force kernel (fp64 form, 16,385
# bodies, force_sym_kernel; ncu --metrics smsp__inst_executed_pipe_fp64.sum,
# sm__thread_inst_executed_pipe_fp64_pred_on.sum, dram__bytes_read.sum,
# dram__bytes_write.sum): DRAM bytes per launch (1,075,968 read, 89,481,728
# of partial sums written) and FP64 thread instructions per launch
# (37,917,882 warp instructions x 32 lanes), which equals the instruction
# model below to the instruction.  Not measured by the bench itself, which
# runs without a profiler.
DRAM_BYTES_PER_LAUNCH = {("fp64", 16385): 1075968 + 89481728}
NCU_FP64_THREAD_INSTR_PER_LAUNCH = {("fp64", 16385): 1213372224}


SYM_MAX_BODIES = 131072  # the symmetric form's limit (abie_gb300/csrc/force.cu)


def force_path(m):
    """Which fast FP64 force form a call takes (abie_gb300/csrc/force.cu):
    "sym" (8,192 .. 131,072 bodies, all massive), "chunked" (from 8,192
    sinks with more than 1,024 sources) or "queue"."""
    n, n_src = int(m.size), int((m > 0).sum())
    if n_src > 1024 and n >= 8192:
        return "sym" if (n_src == n and n <= SYM_MAX_BODIES) else "chunked"
    return "queue"


def launches_per_force_call(m):
    """Kernels of one fast FP64 force call: the source compaction (one
    block, or a count and a scatter pass above 4,096 bodies), then the
    force kernel, plus: for "chunked" the chunk sum; for "sym" its reduction
    pass and the chunked pair, launched too and leaving at once (the device
    picks the form)."""
    path = force_path(m)
    comp = 2 if m.size > 4096 else 1
    return comp + {"queue": 1, "chunked": 2, "sym": 4}[path]


def fp64_instructions_per_call(m, inter):
    """FP64 instructions one force call executes (lanes x warp instructions):
    6 per interaction (3 separations, 3 sums) in the one-sided forms; in the
    symmetric form 9 per unordered pair of an off-diagonal 32 x 32 tile (3
    separations, 3 + 3 sums) and 6 per step of the 31-step diagonal tiles."""
    if force_path(m) != "sym":
        return FP64_INSTR_PER_INTERACTION * inter
    nt = (int(m.size) + 31) // 32
    return 32 * (nt * 31 * 6 + nt * (nt - 1) // 2 * 32 * 9)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="fp64", choices=["fp64", "exact", "mixed", "naive"])
    ap.add_argument("--n", type=int, default=16384, help="planetesimals (plus one star)")
    ap.add_argument("--ensemble-systems", type=int, default=4096)
    ap.add_argument("--ensemble-years", type=float, default=1.0)
    ap.add_argument("--wh-steps", type=int, default=64)
    ap.add_argument("--gr-years", type=float, default=1.0)
    ap.add_argument("--disk-years", type=float, default=1.0)
    ap.add_argument("--no-extras", action="store_true", help="only the headline force line")
    ap.add_argument("--extras", default="ensemble,wh,radau,disk,next",
                    help="comma list of sub-measurements: ensemble, wh, radau, disk, next "
                         "(Runge-Kutta 4, post-Newtonian Radau15, snapshots)")
    ap.add_argument("--ensemble-forms",
                    default="reference_ops,plain_fp64,fp64,mixed,learned,mixed_learned",
                    help="comma list of ensemble forms to time")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--horizon", default="",
                    help="comma list of long-horizon runs instead of the headline bench: "
                         "ens64 (64 ensemble systems over 1e4 yr, fp64 and mixed forms, against "
                         "the reference method's |dE/E| distribution), ens4096 (all 4,096 systems "
                         "over 1e4 yr), disk (the 16,385-body disk over 10 yr, exact and fp64 "
                         "forms), wh (1e6 Wisdom-Holman steps at 1,048,582 bodies)")
    ap.add_argument("--horizon-forms", default="fp64,mixed")
    return ap.parse_args()


def dist_env():
    return D.rank_info()


def interactions(m):
    """(sink, source) pairs: sinks are bodies with m >= 0, sources bodies with
    m > 0, a body never acting on itself."""
    nm = int((m > 0).sum())
    sinks = int((m >= 0).sum())
    return sinks * nm - nm


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling every 50 ms from just before the timed region to
    its end.  start(busy) keeps the GPU under the same load (untimed steps)
    while the sampler comes up, so the samples see the clocks of that load
    and not of an idle GPU; the timed region follows without a gap."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self, busy=None):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        t_end = time.perf_counter() + 0.3
        while time.perf_counter() < t_end:
            if busy is None:
                time.sleep(0.3)
            else:
                busy()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" == r[5 + k]})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(num(r[3]) or 0 for r in rows),
                "window": "every 50 ms from 0.3 s of untimed steps of the same work "
                          "through the end of the timed region"}


# ---------------------------------------------------------------------------
def cpu_force_rate(p, m, threads, sinks=None, reps=1):
    """Oracle (reference algorithm) force on host cores; returns Gint/s and details."""
    from oracle import Oracle
    O = Oracle()
    n = m.size
    j1 = n if sinks is None else min(n, sinks)
    acc = np.zeros(p.size)
    O.force(p, m, G, j0=0, j1=min(j1, 64), threads=threads, acc=acc)  # warm
    t0 = time.perf_counter()
    for _ in range(reps):
        O.force(p, m, G, j0=0, j1=j1, threads=threads, acc=acc)
    dt = (time.perf_counter() - t0) / reps
    nm = int((m > 0).sum())
    inter = j1 * nm - int((m[:j1] > 0).sum())
    return inter / dt / 1e9, dt, inter


def _ensemble_cpu_chunk(job):
    """Oracle Radau15 (the reference's algorithm and predictor) over systems
    lo..hi-1 of the ensemble; returns accepted steps.  A spawn-pool worker."""
    lo, hi, seed0, years = job
    from oracle import Oracle
    O = Oracle()
    P, V, M, offs = ics.ensemble(n_systems=hi - lo, seed0=seed0 + lo)
    steps = 0
    for s in range(offs.size - 1):
        a, b = offs[s], offs[s + 1]
        res = O.radau15(P[3 * a:3 * b], V[3 * a:3 * b], M[a:b], np.zeros(b - a), G, 0.0, years)
        steps += res["stats"]["accepts"]
    return steps


def cpu_baselines_extras(args, extra):
    """The reference's algorithms (the oracle) on the host cores beside each
    sub-measurement: bounded samples of the same workloads."""
    import multiprocessing as mp
    from oracle import Oracle
    O = Oracle()
    cores = os.cpu_count() or 1
    if "ensemble" in extra:
        ns, years = args.ensemble_systems, args.ensemble_years
        seed0 = D.ensemble_seed0(10000, 0, ns)
        per = max(1, (ns + 4 * cores - 1) // (4 * cores))
        jobs = [(lo, min(ns, lo + per), seed0, years) for lo in range(0, ns, per)]
        from concurrent.futures import ProcessPoolExecutor
        try:
            # spawned workers (this process has used the GPU); a worker that
            # dies raises here instead of hanging the pool
            with ProcessPoolExecutor(cores, mp_context=mp.get_context("spawn")) as pool:
                list(pool.map(_ensemble_cpu_chunk, [(0, 1, seed0, 0.01)] * cores))  # start them
                t0 = time.perf_counter()
                steps = sum(pool.map(_ensemble_cpu_chunk, jobs))
                dt = time.perf_counter() - t0
            extra["ensemble"]["cpu_baseline"] = {
                "value": steps / dt, "unit": "system-steps/s", "cores": cores, "kind": "port",
                "sample": "all %d systems over %.2f yr, one process per core (oracle orc_radau15, "
                          "the reference's operations and predictor)" % (ns, years),
                "system_steps": int(steps), "seconds": dt}
        except Exception as exc:  # reported, not fatal: the GPU figures stand alone
            extra["ensemble"]["cpu_baseline"] = {"unavailable": "%s: %s" % (type(exc).__name__, exc)}
    if "wh" in extra:
        out = {}
        for n_tp in (1024, 4096):
            p, v, m, r = ics.test_particle_swarm(n_tp=n_tp)
            p, v = ics.to_heliocentric(p, v)
            steps = 10
            t0 = time.perf_counter()
            O.wh(p, v, m, G, 0.0, steps * 0.01 - 1e-9, 0.01, sparse=False)
            out["ms_per_step_%d_particles" % n_tp] = 1e3 * (time.perf_counter() - t0) / steps
        extra["wh"]["cpu_baseline"] = dict(out, cores=1, kind="port",
                                           sample="10 steps of swarms of 1,024 and 4,096 "
                                                  "particles from the same generator (the star and "
                                                  "5 planets; oracle orc_wh with the reference's "
                                                  "O(N^2) accelerations)")
    if "next" in extra and "rk4_1009" in extra["next"]:
        p, v, m, r = ics.planetary_system()
        steps = 5
        t0 = time.perf_counter()
        O.rk(p, v, m, G, 0.0, steps * 1e-3, 1e-3)
        dt = time.perf_counter() - t0
        extra["next"]["rk4_1009"]["cpu_baseline"] = {
            "steps_per_s": steps / dt, "cores": 1, "kind": "port",
            "sample": "5 steps of the same system (oracle orc_rk, the reference's stages and "
                      "O(N^2) accelerations)"}
    if "radau_1009" in extra:
        p, v, m, r = ics.planetary_system()
        t0 = time.perf_counter()
        res = O.radau15(p, v, m, r, G, 0.0, 0.2)
        dt = time.perf_counter() - t0
        att = res["stats"]["attempts"]
        extra["radau_1009"]["cpu_baseline"] = {
            "ms_per_attempt": 1e3 * dt / max(att, 1), "attempts": int(att), "seconds": dt,
            "cores": 1, "kind": "port",
            "sample": "0.2 yr of the same system (oracle orc_radau15, the reference's operations)"}


def headline_config(args, m, inter, world):
    """The ``config`` of the headline line, the same for both arms."""
    return {"workload": "all-pairs %s force, planetesimal disk of %d bodies (1 star + %d x 1e-9 MSun)"
                        % (args.mode, m.size, m.size - 1),
            "bodies": int(m.size), "interactions_per_step": int(inter),
            "force_mode": args.mode, "l2": "flushed (256 MiB write) between timed GPU steps",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    p, v, m, r = ics.planetesimal_disk(n=args.n)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_force_rate(p, m, threads, sinks=256)
    rates, times = [], []
    for _ in range(args.steps):
        g, dt, inter = cpu_force_rate(p, m, threads)
        rates.append(g)
        times.append(dt)
    value = float(np.mean(rates))
    line = {
        "impl": "reference", "metric": "Gint/s", "value": value, "unit": "Ginteractions/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * float(np.mean(times)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(args, m, interactions(m), world),
        "cpu_baseline": {"value": value, "unit": "Ginteractions/s", "cores": threads, "kind": "port",
                         "sample": "full force evaluation per step (all %d sinks), sinks split "
                                   "over %d threads; oracle/abie_oracle.c orc_force, bit-identical "
                                   "to src/common.c:39-77" % (m.size, threads)},
        "e2e": {"value": value, "unit": "Ginteractions/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
def run_ours(args):
    import ctypes

    import torch

    from abie_gb300 import FORCE_MODES, build
    from abie_gb300.clibabie import CLibABIE

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    build.build()
    lib = CLibABIE()
    L = lib.lib
    mode = FORCE_MODES[args.mode]

    p, v, m, r = ics.planetesimal_disk(n=args.n)
    inter = interactions(m)
    dev = torch.device("cuda", local)
    pos_d = torch.from_numpy(p).to(dev)
    m_d = torch.from_numpy(m).to(dev)
    acc_d = torch.zeros_like(pos_d)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > L2
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    def step():
        rc = L.abie_force_device(ctypes.c_void_p(pos_d.data_ptr()), ctypes.c_void_p(m_d.data_ptr()),
                                 ctypes.c_size_t(m.size), ctypes.c_double(G),
                                 ctypes.c_void_p(acc_d.data_ptr()), ctypes.c_int(mode), sp)
        if rc != 0:
            raise RuntimeError("abie_force_device failed: %d" % rc)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    stream.synchronize()
    peaks = lib.measure_peaks()
    clocks = Clocks(local)

    def busy():  # untimed steps under the sampler, then the timed region
        with torch.cuda.stream(stream):
            for _ in range(8):
                flush.zero_()
                step()
        stream.synchronize()

    clocks.start(busy)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    evs = []
    with torch.cuda.stream(stream):
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            evs.append((e0, e1))
    stream.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    times_ms = [a.elapsed_time(b) for a, b in evs]
    tot_s, units = D.reduce_timing(1e-3 * float(sum(times_ms)), inter * args.steps, device=dev)
    ms_step = 1e3 * tot_s / args.steps
    value = units / tot_s / 1e9

    # e2e through the reference-facing host entry point
    hp = torch.from_numpy(p).pin_memory()
    hm = torch.from_numpy(m).pin_memory()
    ha = torch.zeros(p.size, dtype=torch.float64).pin_memory()
    hr = torch.zeros(m.size, dtype=torch.float64).pin_memory()
    L.abie_set_force_mode(ctypes.c_int(mode))

    def e2e_step():
        rc = L.ode_n_body_second_order(ctypes.c_void_p(hp.data_ptr()), ctypes.c_size_t(m.size),
                                       ctypes.c_double(G), ctypes.c_void_p(hm.data_ptr()),
                                       ctypes.c_void_p(hr.data_ptr()), ctypes.c_void_p(ha.data_ptr()))
        if rc != 0:
            raise RuntimeError("ode_n_body_second_order failed")

    for _ in range(args.warmup):
        e2e_step()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s, e2e_units = D.reduce_timing(time.perf_counter() - t0, inter * args.steps, device=dev)
    e2e_value = e2e_units / e2e_s / 1e9

    # Roofline of the force kernel.  The fast FP64 form is bound by the FP64
    # pipe: frac = executed FP64 instructions per second / the pipe's
    # instruction rate (the measured FMA peak / 2 flop), each executed FP64
    # lane instruction counted as one FMA (2 flop) in `achieved`.  The fast
    # form executes 6 FP64 instructions per interaction (3 separations, 3
    # sums), 4.52 in the symmetric form (each pair once for both bodies),
    # with r^2 and G m r^-3 in integer arithmetic; the count is the model of
    # fp64_instructions_per_call, which the ncu capture of the kernel
    # (smsp__inst_executed_pipe_fp64.sum x 32 lanes) confirms.  The
    # reference's 20-flop-per-interaction convention is kept beside it as
    # `convention_frac`: it reads above 1 because those flops are not all
    # executed on the FP64 pipe.
    peak = peaks["fp64_tflops"] if args.mode != "mixed" else peaks["fp32_tflops"]
    conv = FLOP_PER_INTERACTION * inter / (ms_step * 1e-3) / 1e12
    roof = {"bound": "fp64" if args.mode != "mixed" else "fp32", "unit": "TFLOP/s",
            "peak": peak,
            "peak_source": "FMA throughput measured by abie_measure_fp64_peak (fp32: "
                           "abie_measure_fp32_peak) on this GPU in this run; the driver's "
                           "measured peaks hold only HBM and bf16 figures",
            "flop_per_interaction": FLOP_PER_INTERACTION,
            "convention_achieved": conv, "convention_frac": conv / peak if peak else None}
    if args.mode == "fp64":
        f64 = fp64_instructions_per_call(m, inter)
        ach = 2.0 * f64 / (ms_step * 1e-3) / 1e12
        ncu_f64 = NCU_FP64_THREAD_INSTR_PER_LAUNCH.get((args.mode, int(m.size)))
        roof.update({"achieved": ach, "frac": ach / peak if peak else None,
                     "force_form": force_path(m),
                     "fp64_instructions_per_interaction": f64 / inter,
                     "fp64_instructions_source": "model (fp64_instructions_per_call)",
                     "fp64_instructions_ncu_per_launch": ncu_f64,
                     "fp64_instructions_model_per_launch": int(f64)})
    else:
        roof.update({"achieved": conv, "frac": conv / peak if peak else None})
    roof["traffic"] = DRAM_BYTES_PER_LAUNCH.get((args.mode, int(m.size)))
    roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum, one capture of "
                              "force_sym_kernel on this workload (fp64, 16,385 bodies)"
                              if roof["traffic"] else None)

    extra = {}
    if not args.no_extras:
        which = set(args.extras.split(","))
        if args.ensemble_systems > 0 and "ensemble" in which:
            extra["ensemble"] = run_ensemble(lib, args, rank, dev)
        if args.wh_steps > 0 and "wh" in which:
            extra["wh"] = run_wh(lib, args)
        if args.gr_years > 0 and "radau" in which:
            extra["radau_1009"] = run_radau_single(lib, args)
        if args.disk_years > 0 and "disk" in which:
            extra["radau_disk"] = run_radau_disk(lib, args)
        if "next" in which:
            extra["next"] = run_next(lib, args)

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            g, dt, ci = cpu_force_rate(p, m, threads, reps=3)
            cpu = {"value": g, "unit": "Ginteractions/s", "cores": threads, "kind": "port",
                   "sample": "3 full force evaluations of the same %d-body disk, sinks split over "
                             "%d threads (oracle/abie_oracle.c orc_force, bit-identical to "
                             "src/common.c:39-77)" % (m.size, threads)}
        line = {
            "metric": "Gint/s", "value": value, "unit": "Ginteractions/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.mode != "mixed" else "f32+f64",
            "data": "synthetic",
            "config": headline_config(args, m, inter, world),
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "Ginteractions/s",
                    "h2d_bytes_per_step": int(8 * (p.size + m.size)),
                    "d2h_bytes_per_step": int(8 * p.size),
                    "entry_point": "ode_n_body_second_order (host arrays, pinned)"},
            "clocks": clk,
            "gpu_launches": launches_per_force_call(m) * args.steps,
            "peaks_measured": peaks,
        }
        if not args.no_cpu_baseline and extra:
            cpu_baselines_extras(args, extra)
        line.update(extra)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


def _energy_errors(lib, P0, V0, P1, V1, M, offs):
    """|dE/E| of every system, energies from the library's FP64 energy kernel."""
    errs = np.zeros(offs.size - 1)
    for s in range(offs.size - 1):
        a, b = offs[s], offs[s + 1]
        e0 = lib.energy(P0[3 * a:3 * b], V0[3 * a:3 * b], M[a:b], G)
        e1 = lib.energy(P1[3 * a:3 * b], V1[3 * a:3 * b], M[a:b], G)
        errs[s] = abs((e1 - e0) / e0)
    return errs


def run_ensemble(lib, args, rank, dev):
    """Radau15 over independent systems (4,096 systems per GPU of 4..13
    bodies: a 0.5..1.5 MSun star and 3..12 planets) for a bounded slice of
    time.  Every rank draws its own systems (weak scaling).

    Forms: reference_ops = the reference's FP64 operations and predictor in
    the batched kernel without FMA (bit-level parity form); plain_fp64 = the
    plain FP64 GPU port, the comparator: the same operations compiled with
    FMA contraction and gpuforce_v2's rsqrt pair term; fp64 = the fast form
    (integer r^-3, each pair once for both bodies, the corrector on the
    Newton-form coefficients, each step starting from g consistent with the
    reference's plain guess); mixed = the fast form with light partners'
    terms summed in FP32 two-float arithmetic; learned = the fast form with
    the BF16 network's guess, trained online on samples the ensemble records
    on a separate set of systems; mixed_learned = the mixed form with that
    guess (the three patterns together)."""
    import time as _t

    from abie_gb300.learned import collect_samples, train_predictor
    P, V, M, offs = ics.ensemble(n_systems=args.ensemble_systems,
                                 seed0=D.ensemble_seed0(10000, rank, args.ensemble_systems))
    out = {"systems": int(offs.size - 1), "bodies": int(M.size), "years": args.ensemble_years}
    # online training on other systems
    wanted = set(args.ensemble_forms.split(","))
    if wanted & {"learned", "mixed_learned"}:
        t0 = _t.perf_counter()
        TP, TV, TM, toffs = ics.ensemble(n_systems=2048, seed0=900000 + 4096 * rank)
        samples, _ = collect_samples(lib, TP, TV, TM, toffs, G, 1.0)
        info = train_predictor(lib, samples, steps=1500, batch=2048, lr=1e-3)
        out["training"] = {"systems": 2048, "years": 1.0, "samples": info["samples"],
                           "seconds": _t.perf_counter() - t0, "holdout_loss": info["holdout_loss"],
                           "holdout_loss_plain_guess": info["holdout_loss_plain"]}
    forms = (("reference_ops", "exact", {}), ("plain_fp64", "naive", {}), ("fp64", "fp64", {}),
             ("mixed", "mixed", {}), ("learned", "fp64", {"learned": True}),
             ("mixed_learned", "mixed", {"learned": True}))
    for label, mode, kw in forms:
        if label not in wanted:
            continue
        old = lib.set_force_mode(mode)
        lib.reset_counters()
        res = lib.gr_ensemble(P, V, M, offs, G, 0.0, args.ensemble_years, **kw)
        c = lib.counters()
        lib.set_force_mode(old)
        secs, steps = D.reduce_timing(res["seconds"], int(res["steps"].sum()), device=dev)
        rate = steps / secs if secs else None
        de = _energy_errors(lib, P, V, res["pos"], res["vel"], M, offs)
        out[label] = {"system_steps": int(steps), "seconds": secs, "system_steps_per_s": rate,
                      "attempts": int(c["attempts"]), "force_calls": int(c["force_calls"]),
                      "corrector_iterations_per_attempt": c["iterations"] / max(c["attempts"], 1),
                      "max_abs_dE_over_E": float(de.max()),
                      "abs_dE_over_E_percentiles_50_90_99": [float(np.percentile(de, q))
                                                             for q in (50, 90, 99)],
                      "failed_systems": int((res["status"] != 0).sum()),
                      "max_steps_one_system": int(res["steps"].max()),
                      "launch_shape": lib.ensemble_tuning()}
        if label in ("learned", "mixed_learned"):
            out[label]["attempts_redone_from_plain_guess"] = int(c["learned_fallbacks"])
    lib.mlp_enable(False)
    base = out.get("plain_fp64", {}).get("system_steps_per_s")
    for label in ("reference_ops", "fp64", "mixed", "learned", "mixed_learned"):
        if base and label in out and out[label]["system_steps_per_s"]:
            out[label]["speedup_vs_plain_fp64"] = out[label]["system_steps_per_s"] / base
    return out


def run_wh(lib, args):
    """Wisdom-Holman, 1 MSun star + 5 planets + 1,048,576 test particles, dt = 0.01 yr."""
    import time as _t
    p, v, m, r = ics.test_particle_swarm()
    p, v = ics.to_heliocentric(p, v)
    n = m.size
    lib.initialize_code(G, 0.0, max(n, 1 << 21), MAX_CE_EVENTS=3, MAX_COLLISION_EVENTS=2, deviceID=0)
    n_m = int(np.count_nonzero(m > 0))
    kick = (n - n_m) * n_m + n_m * (n_m - 1)  # particle-massive and massive pairs per step

    def one(form):
        old = lib.set_force_mode(form)
        try:
            lib.set_state(p, v, m, r, n, G, 0.0)
            lib.integrator_wh(0.0, 0.02, 0.01)  # warm-up (graph capture, first launches)
            lib.set_state(p, v, m, r, n, G, 0.0)
            lib.reset_counters()
            t0 = _t.perf_counter()
            lib.integrator_wh(0.0, args.wh_steps * 0.01 - 1e-9, 0.01)
            dt = _t.perf_counter() - t0
        finally:
            lib.set_force_mode(old)
        c = lib.counters()
        steps = c["wh_steps"]
        return {"steps": int(steps), "seconds": dt, "steps_per_s": steps / dt,
                "kepler_solves_per_s": steps * (n - 1) / dt,
                "kick_gint_per_s": steps * kick / dt / 1e9, "kepler_failures": c["kepler_failures"]}

    out = {"bodies": int(n), "kick_interactions_per_step": int(kick),
           "timing": "wall clock around integrator_wh (device-resident state)"}
    out.update(one("fp64"))
    # the mixed kick: the planets' pull on each particle in FP32 two-float
    out["mixed"] = one("mixed")
    return out


def run_radau_single(lib, args):
    """Radau15 on the 1,009-body system (1 star, 8 planets, 1,000 test particles)."""
    import time as _t
    p, v, m, r = ics.planetary_system()
    lib.initialize_code(G, 0.0, 1 << 21, MAX_CE_EVENTS=3, MAX_COLLISION_EVENTS=2, deviceID=0)
    out = {"bodies": int(m.size), "years": args.gr_years}
    for mode in ("fp64", "exact"):
        old = lib.set_force_mode(mode)
        # warm-up: loads the engine kernels and sizes the buffers
        lib.set_state(p, v, m, r, m.size, G, 0.0)
        lib.integrator_gr(0.0, 0.01, 1.0)
        lib.set_state(p, v, m, r, m.size, G, 0.0)
        e0 = lib.get_total_energy()
        lib.reset_counters()
        t0 = _t.perf_counter()
        lib.integrator_gr(0.0, args.gr_years, 1.0)
        dt = _t.perf_counter() - t0
        c = lib.counters()
        e1 = lib.get_total_energy()
        lib.set_force_mode(old)
        out[mode] = {"seconds": dt, "accepts": c["accepts"], "rejects": c["rejects"],
                     "attempts": c["attempts"], "ms_per_attempt": 1e3 * dt / max(c["attempts"], 1),
                     "force_calls": c["force_calls"], "abs_dE_over_E": abs((e1 - e0) / e0)}
    return out


def run_next(lib, args):
    """The rows around the path, each on a bounded workload (fast FP64 form,
    wall clock around the ABI call, device-resident state):
    Runge-Kutta 4 (integrator_rk) on the 1,009-body system and the 16,385-body
    disk; Radau15 with the post-Newtonian terms on a 1,025-body all-massive
    disk over 0.2 yr against the same run without them; Radau15 on the 1,009-body system
    with a snapshot (state, a/e/i about the centre of mass, energy) every
    0.01 yr against the same run without snapshots.  The close-encounter and
    collision scan runs after every accepted Radau15 step in every run."""
    import time as _t
    out = {}
    lib.initialize_code(G, 0.0, 1 << 21, MAX_CE_EVENTS=3, MAX_COLLISION_EVENTS=2, deviceID=0)
    old = lib.set_force_mode("fp64")
    try:
        for name, (p, v, m, r), h, years in (
                ("rk4_1009", ics.planetary_system(), 1e-3, 0.2),
                ("rk4_disk16385", ics.planetesimal_disk(), 1e-3, 0.01)):
            lib.set_state(p, v, m, r, m.size, G, 0.0)
            lib.integrator_rk(0.0, 2 * h, h)  # warm-up: kernels, graph, buffers
            lib.set_state(p, v, m, r, m.size, G, 0.0)
            e0 = lib.get_total_energy()
            lib.reset_counters()
            t0 = _t.perf_counter()
            lib.integrator_rk(0.0, years, h)
            dt = _t.perf_counter() - t0
            steps = lib.counters()["force_calls"] // 4  # the reference's while t < t_end count
            e1 = lib.get_total_energy()
            out[name] = {"bodies": int(m.size), "step": h, "steps": steps, "seconds": dt,
                         "steps_per_s": steps / dt,
                         "gint_per_s": 4 * steps * interactions(m) / dt / 1e9,
                         "abs_dE_over_E": abs((e1 - e0) / e0)}
        p, v, m, r = ics.planetesimal_disk(n=1024)
        c_light = 63239.7263  # au / yr
        res = {"bodies": int(m.size), "years": 0.2, "C": c_light}
        for key, C in (("newtonian", 0.0), ("post_newtonian", c_light)):
            lib.set_state(p, v, m, r, m.size, G, C)
            lib.integrator_gr(0.0, 1e-3, 1.0)
            lib.set_state(p, v, m, r, m.size, G, C)
            lib.reset_counters()
            t0 = _t.perf_counter()
            lib.integrator_gr(0.0, 0.2, 1.0)
            dt = _t.perf_counter() - t0
            c = lib.counters()
            res[key] = {"seconds": dt, "attempts": c["attempts"], "force_calls": c["force_calls"],
                        "ms_per_attempt": 1e3 * dt / max(c["attempts"], 1),
                        "ms_per_force_call": 1e3 * dt / max(c["force_calls"], 1)}
        out["pn_radau_1025"] = res
        p, v, m, r = ics.planetary_system()
        res = {"bodies": int(m.size), "years": 1.0, "store_dt": 0.01}
        lib.set_state(p, v, m, r, m.size, G, 0.0)
        lib.integrate_snapshots(0.0, 0.02, 0.01)  # warm-up
        # integrate() restarts the step control in every chunk, as the
        # reference does, so the snapshot run makes more step attempts
        lib.set_state(p, v, m, r, m.size, G, 0.0)
        lib.reset_counters()
        t0 = _t.perf_counter()
        snaps = lib.integrate_snapshots(0.0, 1.0, 0.01)
        res["with_snapshots_s"] = _t.perf_counter() - t0
        res["with_snapshots_attempts"] = lib.counters()["attempts"]
        res["snapshots"] = int(snaps["t"].size)
        lib.set_state(p, v, m, r, m.size, G, 0.0)
        lib.reset_counters()
        t0 = _t.perf_counter()
        lib.integrator_gr(0.0, 1.0, 1.0)
        res["plain_s"] = _t.perf_counter() - t0
        res["plain_attempts"] = lib.counters()["attempts"]
        per_att = res["plain_s"] / max(res["plain_attempts"], 1)
        res["ms_per_snapshot"] = 1e3 * (res["with_snapshots_s"] - res["plain_s"]) / max(res["snapshots"], 1)
        res["ms_per_snapshot_beyond_attempts"] = 1e3 * (
            res["with_snapshots_s"] - per_att * res["with_snapshots_attempts"]) / max(res["snapshots"], 1)
        out["snapshots_1009"] = res
    finally:
        lib.set_force_mode(old)
    return out


def run_radau_disk(lib, args):
    """Radau15 (fast form) on the 16,385-body planetesimal disk, a bounded
    slice of the reference's 10-yr run: every body massive, so each force
    call is 268 M interactions inside the general engine."""
    import time as _t
    p, v, m, r = ics.planetesimal_disk()
    n = m.size
    lib.initialize_code(G, 0.0, 1 << 21, MAX_CE_EVENTS=3, MAX_COLLISION_EVENTS=2, deviceID=0)
    old = lib.set_force_mode("fp64")
    lib.set_state(p, v, m, r, n, G, 0.0)
    lib.integrator_gr(0.0, 1e-3, 1.0)  # warm-up: kernels, buffers
    lib.set_state(p, v, m, r, n, G, 0.0)
    e0 = lib.get_total_energy()
    lib.reset_counters()
    t0 = _t.perf_counter()
    lib.integrator_gr(0.0, args.disk_years, 1.0)
    dt = _t.perf_counter() - t0
    c = lib.counters()
    e1 = lib.get_total_energy()
    lib.set_force_mode(old)
    inter = interactions(m)
    out = {"bodies": int(n), "years": args.disk_years, "t_reached": lib.get_model_time(),
           "seconds": dt, "accepts": c["accepts"], "rejects": c["rejects"],
           "attempts": c["attempts"], "force_calls": c["force_calls"],
           "ms_per_attempt": 1e3 * dt / max(c["attempts"], 1),
           "gint_per_s_in_engine": c["force_calls"] * inter / dt / 1e9,
           "abs_dE_over_E": abs((e1 - e0) / e0),
           "timing": "wall clock around integrator_gr (device-resident state)"}
    # the mixed form: the same sweep with the mixed all-pairs force
    old = lib.set_force_mode("mixed")
    try:
        lib.set_state(p, v, m, r, n, G, 0.0)
        lib.integrator_gr(0.0, 1e-3, 1.0)
        lib.set_state(p, v, m, r, n, G, 0.0)
        lib.reset_counters()
        t0 = _t.perf_counter()
        lib.integrator_gr(0.0, args.disk_years, 1.0)
        dtm = _t.perf_counter() - t0
        cm = lib.counters()
        e1m = lib.get_total_energy()
    finally:
        lib.set_force_mode(old)
    out["mixed"] = {"seconds": dtm, "t_reached": lib.get_model_time(), "accepts": cm["accepts"],
                    "attempts": cm["attempts"], "force_calls": cm["force_calls"],
                    "gint_per_s_in_engine": cm["force_calls"] * inter / dtm / 1e9,
                    "abs_dE_over_E": abs((e1m - e0) / e0)}
    return out


def _de_stats(de, ref=None):
    q = [float(np.percentile(de, x)) for x in (50, 90, 99, 100)]
    out = {"abs_dE_over_E_p50_p90_p99_max": q,
           "systems_at_or_below_1e-12": int((de <= 1e-12).sum()), "systems": int(de.size)}
    if ref is not None:
        out["reference_method_p50_p90_p99_max"] = [float(np.percentile(ref, x))
                                                   for x in (50, 90, 99, 100)]
        out["reference_method_at_or_below_1e-12"] = int((ref <= 1e-12).sum())
        out["systems_within_10x_of_reference"] = int((de <= 10 * np.maximum(ref, 1e-15)).sum())
    return out


def run_horizons(args):
    """Long-horizon runs of the stated configurations, each against the
    reference's own runs where those exist (tests/golden/horizon_*.npz,
    made by tests/golden/make_horizons.py).  One JSON line."""
    import time as _t

    import torch

    from abie_gb300.clibabie import CLibABIE
    torch.cuda.set_device(0)
    lib = CLibABIE()
    lib.initialize_code(G, 0.0, 1 << 21, MAX_CE_EVENTS=3, MAX_COLLISION_EVENTS=2, deviceID=0)
    gold = os.path.join(ROOT, "tests", "golden")
    which = set(args.horizon.split(","))
    forms = args.horizon_forms.split(",")
    out = {"horizon": sorted(which)}

    def ens(ns, years, form, ref=None):
        P, V, M, offs = ics.ensemble(n_systems=ns, seed0=10000)
        old = lib.set_force_mode(form)
        lib.reset_counters()
        try:
            res = lib.gr_ensemble(P, V, M, offs, G, 0.0, years)
        finally:
            lib.set_force_mode(old)
        c = lib.counters()
        de = _energy_errors(lib, P, V, res["pos"], res["vel"], M, offs)
        steps = int(res["steps"].sum())
        r = {"systems": ns, "years": years, "seconds": res["seconds"], "system_steps": steps,
             "system_steps_per_s": steps / res["seconds"], "launch_shape": lib.ensemble_tuning(),
             "corrector_iterations_per_attempt": c["iterations"] / max(c["attempts"], 1),
             "max_steps_one_system": int(res["steps"].max()),
             "failed_systems": int((res["status"] != 0).sum())}
        r.update(_de_stats(de, ref))
        r["per_system_abs_dE_over_E_first_64"] = [float(x) for x in de[:64]]
        worst = np.argsort(-de)[:8]
        r["worst_systems"] = [{"system": int(s), "abs_dE_over_E": float(de[s]),
                               "steps": int(res["steps"][s]),
                               "bodies": int(offs[s + 1] - offs[s])} for s in worst]
        r["per_system_steps_first_64"] = [int(x) for x in res["steps"][:64]]
        return r

    g = np.load(os.path.join(gold, "horizon_ensemble.npz"))
    h = list(g["horizons"]).index(10000.0)
    ref64 = g["de"][:, h]
    # the reference method's runs of the same systems with one coordinate
    # moved by one unit in the last place: over 10^4 yr some systems are
    # chaotic, and these give the spread of its own |dE/E|
    sp = np.load(os.path.join(gold, "horizon_ensemble_spread.npz"))["de"]
    ref_all = np.concatenate([ref64, sp.ravel()])
    # the fast form's arithmetic emulated on the host (same 64 systems)
    ff = np.load(os.path.join(gold, "horizon_ensemble_fastform.npz"))["de"]

    def with_spread(r):
        r["reference_method_with_perturbed_runs_p50_p90_p99_max"] = [
            float(np.percentile(ref_all, x)) for x in (50, 90, 99, 100)]
        r["reference_method_with_perturbed_runs_samples"] = int(ref_all.size)
        r["reference_method_per_system_max_over_runs_first_64"] = [
            float(x) for x in np.maximum(ref64, sp.max(axis=1))]
        r["fast_form_arithmetic_on_the_host_p50_p90_p99_max"] = [
            float(np.percentile(ff, x)) for x in (50, 90, 99, 100)]
        r["fast_form_arithmetic_on_the_host_at_or_below_1e-12"] = int((ff <= 1e-12).sum())
        return r

    if "ens64" in which:
        out["ens64_1e4yr"] = {f: with_spread(ens(64, 10000.0, f, ref64)) for f in forms}
        out["ens64_1e4yr"]["reference_method_cpu_seconds_one_core"] = float(g["wall"][:, h].sum())
    if "ens4096" in which:
        out["ens4096_1e4yr"] = {f: with_spread(ens(4096, 10000.0, f)) for f in forms}
    if "disk" in which:
        p, v, m, r = ics.planetesimal_disk()
        e0 = lib.energy(p, v, m, G)
        runs = {}
        for form in ("fp64", "exact"):
            old = lib.set_force_mode(form)
            lib.reset_counters()
            try:
                lib.set_state(p, v, m, r, m.size, G, 0.0)
                t0 = _t.perf_counter()
                lib.integrator_gr(0.0, 10.0, 1.0)
                secs = _t.perf_counter() - t0
                P, Vv = np.zeros(p.size), np.zeros(v.size)
                lib.get_state(P, Vv, np.zeros(m.size), np.zeros(m.size))
                t = lib.get_model_time()
            finally:
                lib.set_force_mode(old)
            c = lib.counters()
            runs[form] = (P, Vv, t)
            out.setdefault("disk_10yr", {})[form] = {
                "seconds": secs, "t": t, "force_calls": int(c["force_calls"]),
                "accepts": int(c["accepts"]), "rejects": int(c["rejects"]),
                "abs_dE_over_E": abs((lib.energy(P, Vv, m, G) - e0) / e0),
                "gint_per_s": c["force_calls"] * interactions(m) / secs / 1e9}
        # the two forms at the exact form's final time: shift the fast form's
        # state by RK4 substeps on the library's exact force
        P, Vv, t = runs["fp64"]
        Pe, Ve, te = runs["exact"]
        hsub = (te - t) / max(8, int(np.ceil(abs(te - t) / 2e-4)))
        nsub = int(round((te - t) / hsub)) if hsub else 0
        for _ in range(nsub):
            a1 = lib.force(P, m, G, "exact")
            a2 = lib.force(P + 0.5 * hsub * Vv, m, G, "exact")
            a3 = lib.force(P + 0.5 * hsub * Vv + 0.25 * hsub * hsub * a1, m, G, "exact")
            a4 = lib.force(P + hsub * Vv + 0.5 * hsub * hsub * a2, m, G, "exact")
            P, Vv = (P + hsub * Vv + hsub * hsub / 6.0 * (a1 + a2 + a3),
                     Vv + hsub / 6.0 * (a1 + 2 * a2 + 2 * a3 + a4))
        d = (np.linalg.norm((P - Pe).reshape(-1, 3), axis=1) /
             np.linalg.norm(Pe.reshape(-1, 3), axis=1))
        out["disk_10yr"]["fp64_vs_exact_at_common_time"] = {
            "max_rel_pos": float(d.max()), "median_rel_pos": float(np.median(d))}
    if "wh" in which:
        g = np.load(os.path.join(gold, "horizon_cfg3.npz"))
        p, v, m, r = ics.test_particle_swarm(seed=int(g["seed"][0]))
        p, v = ics.to_heliocentric(p, v)
        idx = g["idx"]
        t_end, dt = float(g["span"][1]), float(g["span"][2])
        # relative to each body's distance from the star (the star itself,
        # pinned at the origin, is left out)
        ref_r = np.linalg.norm(g["pos"].reshape(-1, 3), axis=1)
        live = ref_r > 0
        spread = (np.linalg.norm((g["pert_pos"] - g["pos"]).reshape(-1, 3), axis=1)[live] /
                  ref_r[live])
        for form in forms:
            old = lib.set_force_mode(form)
            lib.reset_counters()
            try:
                lib.set_state(p, v, m, r, m.size, G, 0.0)
                e0 = lib.get_total_energy()
                t0 = _t.perf_counter()
                lib.integrator_wh(0.0, t_end, dt)
                secs = _t.perf_counter() - t0
                P, Vv = np.zeros(p.size), np.zeros(v.size)
                lib.get_state(P, Vv, np.zeros(m.size), np.zeros(m.size))
                e1 = lib.get_total_energy()
            finally:
                lib.set_force_mode(old)
            c = lib.counters()
            d = (np.linalg.norm((P.reshape(-1, 3)[idx] - g["pos"].reshape(-1, 3)), axis=1)[live] /
                 ref_r[live])
            out.setdefault("wh_1e6", {})[form] = {
                "steps": int(c["wh_steps"]), "seconds": secs, "steps_per_s": c["wh_steps"] / secs,
                "t": lib.get_model_time(), "t_reference": float(g["t"][0]),
                "abs_dE_over_E_massive": abs((e1 - e0) / e0),
                "abs_dE_over_E_massive_reference": abs((g["energy"][1] - g["energy"][0]) /
                                                       g["energy"][0]),
                "kepler_failures": int(c["kepler_failures"]),
                "sample_nonfinite": int((~np.isfinite(d)).sum()),
                "sample_vs_oracle_rel_pos_median_p99_max": [
                    float(np.median(d[np.isfinite(d)])), float(np.percentile(d[np.isfinite(d)], 99)),
                    float(d[np.isfinite(d)].max())],
                "bodies_nonfinite": int((~np.isfinite(P.reshape(-1, 3)).all(1)).sum()),
                "rounding_spread_median_p99_max": [float(np.median(spread)),
                                                   float(np.percentile(spread, 99)),
                                                   float(spread.max())]}
    print(json.dumps(out), flush=True)
    return 0


def main():
    args = parse()
    if args.horizon:
        return run_horizons(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
