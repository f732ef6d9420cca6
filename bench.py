"""Benchmark: Fr NTT throughput at 2^24 on GB300 (plus the other operators).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one forward NTT of 2^24 seeded random canonical Fr elements
(512 MiB, larger than the 129 MB L2, so no flush is needed between steps).
`value` is device throughput with the input resident in HBM (Melem/s =
2^24 * K * n_gpus / max-over-ranks time); `e2e` is the same metric through the
C ABI with pinned host buffers in and out.  Three forms are timed: pp_ntt_host
(the first pass reads the host input over NVLink-C2C and the last pass writes
the host output), copies + transform one step at a time, and copies of
neighbouring steps overlapped with the transform on three streams.  The
headline is the faster of the first and last.  `roofline` is the integer-multiply
pipe bound of the transform kernel; `roofline_hbm` its HBM view.  Extra
operators (INTT, LDE, grand products, evaluation, division) are timed after
the headline and reported under `ops`.

--impl reference times the reference's CPU path for the same workload on the
host cores (the oracle's restatement: the reference has no CPU NTT of its own)
and prints the same metric with "impl": "reference".
Under torchrun with N > 1 each rank transforms its own polynomial on its own
GPU (replicas; there is no exchange step).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LG_N = 24
N = 1 << LG_N
MM_PER_NTT = (N // 2) * LG_N          # algorithmic Montgomery multiplies (radix-2 count)
INSTR_PER_MM = 256                     # 8x8 limbs: 4 n^2 integer multiply instructions
BYTES_PER_NTT = 2 * 32 * N             # read + write once
IMAD_PER_CLK_PER_SM = 64               # 32-bit multiply-add lanes per SM per clock (nominal)
EXEC_MM_PER_NTT = int(11.375 * N)      # multiplies the shipped 9,6,9 split executes (unit twiddles skipped)
WIDE_PER_MM = 112                      # mad.wide products per Montgomery multiply (r's two low limbs are free)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-ops", action="store_true", help="skip the secondary operator timings")
    ap.add_argument("--lean", action="store_true",
                    help="device timing only (no e2e, CPU baseline, ops): the profiling case")
    ap.add_argument("--lg", type=int, default=LG_N, help="transform size (profiling of smaller cases)")
    ap.add_argument("--op", default="ntt",
                    choices=["ntt", "msm", "msmfixed", "gate", "perm", "gpperm", "scans", "div"],
                    help="with --lean: time one operator alone at 2^lg points (profiling case)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ helpers
def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


def profile_traffic(name: str):
    """dram bytes per launch recorded from an ncu capture (profiles/<name>)."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def measure_int_rates(ppfr):
    """Measured integer-pipe rates of this GPU (pp_measure_int_rates_ex), the
    denominators of the integer roofline: lane operations per second of
    mad.lo.u32 / mad.hi.u32 / mad.wide.u32 loops at full occupancy, the
    standalone Montgomery multiply rate, and the wide product without its
    64-bit addend (alone, and with the addend as a separate add.u64)."""
    import ctypes

    L = ppfr.lib()
    f = L.pp_measure_int_rates_ex
    f.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    f.restype = ctypes.c_int
    out = (ctypes.c_double * 6)()
    ppfr.check(f(out, 6))
    return {"mad_lo_per_s": out[0], "mad_hi_per_s": out[1], "mad_wide_per_s": out[2],
            "mont_mul_per_s": out[3], "mul_wide_no_addend_per_s": out[4],
            "mul_wide_then_add_u64_per_s": out[5]}


def reduce_max_over_ranks(values, dist, device):
    """Element-wise maximum of this rank's timings (ms) over all ranks: the
    slowest rank sets every whole-job rate.  dist is torch.distributed (or
    None for one process); device is where the backend reduces ("cuda" for
    NCCL, "cpu" for gloo)."""
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def whole_job_rate(elems_per_step, steps, world, ms):
    """Melem/s of the whole job: every rank transforms its own elems_per_step
    elements per step (independent replicas), and the slowest rank's ms for
    `steps` steps is the job's time."""
    return elems_per_step * steps * world / (ms / 1e3) / 1e6


def time_device(fn, steps, warmup, torch):
    """CUDA-event time of `steps` calls of fn() on the current stream (ms total)."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        fn()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def cpu_ntt_rate(lg: int, reps: int, threads: int):
    from oracle import oracle as O

    x = O.random_fr(1 << lg, 0x5EED0018)
    O.ntt(x[:1024].copy(), nthreads=threads)  # load / warm the library
    t0 = time.perf_counter()
    for _ in range(reps):
        O.ntt(x, nthreads=threads)
    dt = time.perf_counter() - t0
    return (1 << lg) * reps / dt / 1e6, dt


# ------------------------------------------------------------------ arms
def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # one step = one full 2^24 NTT of the CPU implementation (about 1.5 s on
    # 16 Arm cores); warm-up steps at 2^20 load and warm the library
    reps = max(1, min(args.steps, 200))
    for _ in range(args.warmup):
        cpu_ntt_rate(20, 1, threads)
    rate, dt = cpu_ntt_rate(LG_N, reps, threads)
    line = {
        "impl": "reference", "metric": "fr_ntt_2^24_throughput", "value": round(rate, 3),
        "unit": "Melem/s", "n_gpus": args.gpus, "steps": reps, "warmup": args.warmup,
        "ms_per_step": round(dt / reps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32x8 (Fr, Montgomery)", "data": "synthetic (seeded SplitMix64 Fr)",
        "config": {"workload": "ntt forward 2^24, natural order in/out", "lg_n": LG_N,
                   "l2_flush": "not needed: 512 MiB input > 129 MB L2",
                   "parallelism": "replicas" if args.gpus > 1 else "1 GPU"},
        "cpu_baseline": {"value": round(rate, 3), "unit": "Melem/s", "cores": threads, "kind": "port",
                         "sample": "%d full 2^24 NTTs (oracle restatement; the reference has no CPU NTT)" % reps},
        "e2e": {"value": round(rate, 3), "unit": "Melem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local):
    import torch

    torch.cuda.set_device(local)
    import __graft_entry__ as ge

    pp = ge.load_package()
    ppfr = pp.ppfr
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl", device_id=torch.device("cuda", local))
        dist = dist_mod

    def barrier():
        if dist:
            dist.barrier()

    if args.lean and args.op != "ntt":
        if rank == 0:
            profile_op(args, pp, torch)
        if dist:
            dist.destroy_process_group()
        return

    # ---- device-resident headline
    n = 1 << args.lg
    x = pp.random_fr(n, 0x5EED0018 + rank)
    out = ppfr.empty(n)
    ppfr.prepare(args.lg, False)
    fn = lambda: pp.ntt(x, out=out)  # noqa: E731
    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize()
    barrier()
    clocks = ClockSampler(local)
    if not args.lean:
        clocks.start()
        time.sleep(0.3)
    launches0 = pp.launch_count()
    torch.cuda.synchronize()
    barrier()
    ms = time_device(fn, args.steps, 0, torch)
    launches = pp.launch_count() - launches0
    torch.cuda.synchronize()
    barrier()
    if args.lean or args.lg != LG_N:
        # profiling case: device time only
        if rank == 0:
            print(json.dumps({"metric": "fr_ntt_2^%d_throughput" % args.lg, "lean": True,
                              "value": round(n * args.steps / (ms / 1e3) / 1e6, 3), "unit": "Melem/s",
                              "ms_per_step": round(ms / args.steps, 4), "gpu_launches": int(launches)}),
                  flush=True)
        if dist:
            dist.destroy_process_group()
        return
    # ---- end to end through the C ABI with host buffers
    hin = torch.empty((N, 4), dtype=torch.int64, pin_memory=True)
    hin.copy_(x.cpu())
    hout = torch.empty_like(hin, pin_memory=True)
    dbuf = ppfr.empty(N)

    def e2e_step():
        dbuf.copy_(hin, non_blocking=True)
        pp.ntt(dbuf, out=dbuf)
        hout.copy_(dbuf, non_blocking=True)

    e2e_steps = max(3, args.steps // 2)
    e2e_serial_ms = time_device(e2e_step, e2e_steps, 1, torch)
    # streaming form: one pp_ntt_host_many call over the steps' page-locked
    # polynomials; inside it H2D, transform and D2H of neighbouring steps
    # overlap on three streams with three rotating device buffers
    houts = [hout] + [torch.empty_like(hin, pin_memory=True) for _ in range(2)]

    def e2e_stream(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        ppfr.ntt_host_many([hin] * steps, outs=[houts[j % 3] for j in range(steps)])
        e1.record()  # the call's last copy is ordered before this
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    e2e_stream(3)
    e2e_ms = e2e_stream(e2e_steps)
    # host-resident form (pp_ntt_host): the first pass reads the pinned input
    # over NVLink-C2C and the last pass writes the pinned output; no copies
    hout_d = torch.empty_like(hin, pin_memory=True)
    e2e_direct_ms = time_device(lambda: ppfr.ntt_host(hin, out=hout_d), e2e_steps, 1, torch)
    clk = clocks.stop()
    # max over ranks
    ms, e2e_ms_norm, e2e_serial_norm, e2e_direct_norm = reduce_max_over_ranks(
        [ms, e2e_ms / e2e_steps * args.steps, e2e_serial_ms / e2e_steps * args.steps,
         e2e_direct_ms / e2e_steps * args.steps], dist, "cuda")
    value = whole_job_rate(N, args.steps, world, ms)
    e2e_stream_value = whole_job_rate(N, args.steps, world, e2e_ms_norm)
    e2e_serial_value = whole_job_rate(N, args.steps, world, e2e_serial_norm)
    e2e_direct_value = whole_job_rate(N, args.steps, world, e2e_direct_norm)
    same = torch.equal(hout_d, hout)  # both forms transformed the same input
    if e2e_direct_value >= e2e_stream_value:
        e2e_value, e2e_form = e2e_direct_value, (
            "host-resident: pp_ntt_host on pinned host buffers, pass 1 reads the input over "
            "NVLink-C2C and the last pass writes the output; one call per step, no overlap between steps")
    else:
        e2e_value, e2e_form = e2e_stream_value, (
            "streamed (pp_ntt_host_many): H2D / NTT / D2H of neighbouring steps overlap on 3 streams")

    rates = measure_int_rates(ppfr)
    ops = {}
    if not args.no_ops and rank == 0:
        ops = secondary_ops(pp, torch, rates["mad_lo_per_s"])

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks, peak_kind = load_peaks()
    sm_mhz = clk.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    nominal_int_peak = n_sm * IMAD_PER_CLK_PER_SM * sm_mhz * 1e6 / 1e12  # T instr / s
    int_peak = rates["mad_lo_per_s"] / 1e12  # measured in this run
    sec_per_ntt = ms / args.steps / 1e3
    achieved_int = MM_PER_NTT * INSTR_PER_MM / sec_per_ntt / 1e12
    achieved_hbm = BYTES_PER_NTT / sec_per_ntt / 1e9
    # one NTT is len(split) kernel launches; per-launch figures are the same ratio
    traffic = profile_traffic("ntt_pass_2p24_launches.md")
    cpu_rate, cpu_dt = cpu_ntt_rate(LG_N, 2, os.cpu_count() or 1)
    line = {
        "metric": "fr_ntt_2^24_throughput", "value": round(value, 3), "unit": "Melem/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32x8 (Fr, Montgomery)", "data": "synthetic (seeded SplitMix64 Fr)",
        "config": {"workload": "ntt forward 2^24, natural order in/out", "lg_n": LG_N,
                   "l2_flush": "not needed: 512 MiB input > 129 MB L2", "parallelism": "replicas" if world > 1 else "1 GPU"},
        "e2e": {"value": round(e2e_value, 3), "unit": "Melem/s", "h2d_bytes_per_step": 32 * N,
                "d2h_bytes_per_step": 32 * N, "steps": e2e_steps, "form": e2e_form,
                "host_resident_value": round(e2e_direct_value, 3),
                "streamed_value": round(e2e_stream_value, 3),
                "serial_value": round(e2e_serial_value, 3), "forms_agree": bool(same)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "int", "kernel": "k_ntt_pass", "achieved": round(achieved_int, 3),
                     "peak": round(int_peak, 3), "unit": "Tinstr/s", "frac": round(achieved_int / int_peak, 4),
                     "peak_kind": "measured in this run: mad.lo.u32 lane operations/s of a full-occupancy "
                                  "loop (pp_measure_int_rates)",
                     "nominal_peak": round(nominal_int_peak, 3),
                     "frac_of_nominal": round(achieved_int / nominal_int_peak, 4),
                     "measured_rates_T_per_s": {k: round(v / 1e12, 4) for k, v in rates.items()},
                     "traffic": traffic,
                     "frac_of_wide_multiply_rate": round(
                         EXEC_MM_PER_NTT * WIDE_PER_MM / sec_per_ntt / rates["mad_wide_per_s"], 4),
                     "wide_product_ceiling": round(2 * rates["mad_wide_per_s"] / 1e12, 3),
                     "frac_of_wide_product_ceiling": round(achieved_int / (2 * rates["mad_wide_per_s"] / 1e12), 4),
                     "note": "algorithmic (N/2)lgN Montgomery multiplies x 256 32-bit multiply instructions; "
                             "peak = the measured low-half (mad.lo) rate; half of the 256 are high halves, "
                             "which run at 0.38 of that rate; the fastest measured instruction for a low and "
                             "high half is one mad.wide, so wide_product_ceiling = 2 x the measured mad.wide "
                             "rate bounds the 256 instructions. frac_of_wide_multiply_rate: the 11.375 N multiplies the "
                             "transform executes x 112 mad.wide products each, over the measured mad.wide "
                             "rate"},
        "roofline_hbm": {"bound": "hbm", "achieved": round(achieved_hbm, 2), "peak": peaks.get("hbm_gbs"),
                         "unit": "GB/s", "frac": round(achieved_hbm / peaks.get("hbm_gbs", 6800.0), 4),
                         "peak_kind": peak_kind},
        "cpu_baseline": {"value": round(cpu_rate, 3), "unit": "Melem/s", "cores": os.cpu_count(),
                         "kind": "port", "sample": "2 full 2^24 NTTs of the oracle restatement, all host threads"},
        "clocks": clk,
        "ops": ops,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def secondary_ops(pp, torch, int_peak=None):
    """Quick device timings of the other operators (inputs resident).
    int_peak: the measured mad.lo lane-operation rate (instr / s)."""
    import numpy as np

    ppfr = pp.ppfr
    res = {}

    def rate(name, fn, elems, reps=5):
        ms = time_device(fn, reps, 2, torch)
        res[name] = {"ms": round(ms / reps, 4), "Melem_per_s": round(elems * reps / (ms / 1e3) / 1e6, 2)}

    sm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    peak = int_peak or sm * IMAD_PER_CLK_PER_SM * 2070e6  # instr / s

    hbm = load_peaks()[0].get("hbm_gbs", 6800.0) * 1e9

    def int_frac(name, mm, nbytes=None):
        # algorithmic Montgomery multiplies x 256 multiply instructions; with
        # the algorithmic bytes, the roofline time is the larger of the two
        # bounds and frac_of_roofline = that time / the measured time
        sec = res[name]["ms"] / 1e3
        res[name]["MM"] = mm
        res[name]["int_frac_of_peak"] = round(mm * INSTR_PER_MM / sec / peak, 4)
        if nbytes is not None:
            t_int, t_hbm = mm * INSTR_PER_MM / peak, nbytes / hbm
            res[name].update({"bytes": nbytes, "hbm_frac": round(nbytes / sec / hbm, 4),
                              "roofline_bound": "int" if t_int >= t_hbm else "hbm",
                              "frac_of_roofline": round(max(t_int, t_hbm) / sec, 4)})

    for lg in (22, 26):
        x = pp.random_fr(1 << lg, lg)
        o = ppfr.empty(1 << lg)
        rate("ntt_2^%d" % lg, lambda: pp.ntt(x, out=o), 1 << lg, 3)
        int_frac("ntt_2^%d" % lg, (1 << lg) // 2 * lg, 64 << lg)
        del x, o
    x = pp.random_fr(N, 1)
    o = ppfr.empty(N)
    rate("intt_2^24", lambda: pp.ntt(x, True, out=o), N)
    int_frac("intt_2^24", N // 2 * LG_N + N, 64 * N)
    del o
    for lam in (2, 3):
        o = ppfr.empty(N << lam)
        # coefficients: 2^lam coset transforms of N points plus the N-point
        # diagonal; evaluations add the N-point INTT
        coset_mm = (N << lam) // 2 * LG_N + N
        lde_bytes = 32 * N * (1 + (1 << lam))
        for form, mode, mm in (("coeffs", pp.LDE_COEFFS, coset_mm),
                               ("evals", pp.LDE_EVALS, coset_mm + N // 2 * LG_N + N)):
            name = "lde_%s_2^24_l%d" % (form, lam)
            rate(name, lambda: pp.lde(x, lam, mode, out=o), N, 3)
            int_frac(name, mm, lde_bytes)
            res[name]["out_Melem_per_s"] = round(res[name]["Melem_per_s"] * (1 << lam), 2)
        del o
    del x
    # the scans at the reference's miss_ops sizes: 2^20 (the BASELINE
    # config) and 2^22 (its shipped main)
    z = pp.random_fr(1, 3)
    y = ppfr.empty(1)
    for lg in (22, 20):
        n = 1 << lg
        p = pp.random_fr(n, 2)
        rate("gp_prefix_2^%d" % lg, lambda: pp.gp_prefix_(p), n, 10)
        int_frac("gp_prefix_2^%d" % lg, n, 64 * n)
        rate("eval_2^%d" % lg, lambda: pp.evaluate(p, z, out=y), n, 10)
        int_frac("eval_2^%d" % lg, n, 32 * n)
        rate("div_2^%d" % lg, lambda: pp.div_xplusc_(p, z), n, 10)
        int_frac("div_2^%d" % lg, n, 64 * n)
    w = [pp.random_fr(n, 10 + j) for j in range(3)]
    s = [pp.random_fr(n, 20 + j) for j in range(3)]
    params = pp.random_fr(5, 30)
    zz = ppfr.empty(n)
    rate("gp_perm_2^20", lambda: pp.gp_perm(w, s, params, out=zz), n, 10)
    int_frac("gp_perm_2^20", 16 * n, 224 * n)
    del w, s, p
    host_resident_bench(pp, torch, rate, res)
    elementwise_bench(pp, torch, rate, res)
    constraint_bench(pp, torch, rate, res, peak)
    msm_bench(pp, torch, rate, res, peak)
    res["batched"] = batched_bench(pp, torch, peak=peak)
    # the launch-bound regime: many small polynomials
    res["batched_small"] = batched_bench(pp, torch, 1024, 8, 14, peak=peak)
    res["serving"] = serving_bench(pp, torch)
    return res


def host_resident_bench(pp, torch, rate, res):
    """The reference's own host-resident configurations, page-locked host
    input and output: our_ntt at 2^22, 2^24, 2^26 (ntt.cu:1193-1206) against
    pp_ntt_host, and our_lde at 2^20, 2^22, 2^24 with lambda = 2, 3
    (lde.cu:1550-1580; coefficients in) against pp_lde_host.  Events bracket
    the whole call, as the reference's own timers do."""
    ppfr = pp.ppfr
    hin = ppfr.empty_pinned(1 << 26)
    hin.copy_(ppfr.random_fr(1 << 26, 0x4057).cpu())
    hout = ppfr.empty_pinned(1 << 27)
    for lg in (22, 24, 26):
        x, o = hin[:1 << lg], hout[:1 << lg]
        rate("ntt_host_2^%d" % lg, lambda: ppfr.ntt_host(x, out=o), 1 << lg, 3)
    for lg in (20, 22, 24):
        for lam in (2, 3):
            x, o = hin[:1 << lg], hout[:1 << (lg + lam)]
            name = "lde_host_2^%d_l%d" % (lg, lam)
            rate(name, lambda: ppfr.lde_host(x, lam, pp.LDE_COEFFS, out=o), 1 << lg, 3)
    # out of core: every pass reads and writes host memory over the C2C link;
    # the device holds only the twiddle tables
    for lg in (24, 26):
        n = 1 << lg
        x, o, sc = hin[:n], hout[:n], hout[1 << 26:(1 << 26) + n]
        name = "ntt_out_of_core_2^%d" % lg
        rate(name, lambda: ppfr.ntt_out_of_core(x, out=o, scratch=sc), n, 3)
        passes = -(-lg // 9)  # the plan splits lg into passes of at most 9 bits
        gbs = 64 * passes * n / (res[name]["ms"] / 1e3) / 1e9
        res[name].update({"passes": passes, "host_GB_per_s": round(gbs, 1)})
    # out-of-core LDE from coefficients, 2^24 -> 2^26 (lambda = 2)
    lg, lam = 24, 2
    m = 1 << (lg + lam)
    x, o, sc = hin[:1 << lg], hout[:m], hout[m:2 * m]
    name = "lde_out_of_core_2^24_l2"
    rate(name, lambda: ppfr.lde_out_of_core(x, lam, pp.LDE_COEFFS, out=o, scratch=sc), 1 << lg, 3)
    res[name]["out_Melem_per_s"] = round(m / (res[name]["ms"] / 1e3) / 1e6, 2)
    del hin, hout


def elementwise_bench(pp, torch, rate, res):
    """Element-wise operators over 2^24 elements (512 MiB per vector, larger
    than L2), with their HBM fraction: mul_mod reads two vectors and writes
    one (96 B per element), div_mod the same plus 3 multiplies and 1/32 of an
    inversion per element, gen_sequence writes one (32 B per element)."""
    ppfr = pp.ppfr
    n = N
    a, b = pp.random_fr(n, 40), pp.random_fr(n, 41)
    c = ppfr.empty(n)
    x = pp.random_fr(1, 42)
    peaks, _ = load_peaks()
    for name, fn, nbytes in (("mul_mod_2^24", lambda: ppfr.fr_binary(ppfr.FR_MUL, a, b, out=c), 96),
                             ("add_mod_2^24", lambda: ppfr.fr_binary(ppfr.FR_ADD, a, b, out=c), 96),
                             ("div_mod_2^24", lambda: ppfr.fr_binary(ppfr.FR_DIV, a, b, out=c), 96),
                             ("gen_sequence_2^24", lambda: ppfr.fr_powers(x, n, out=c), 32)):
        rate(name, fn, n, 5)
        gbs = nbytes * n / (res[name]["ms"] / 1e3) / 1e9
        res[name].update({"GB_per_s": round(gbs, 1), "hbm_frac": round(gbs / peaks["hbm_gbs"], 3)})
    del a, b, c


def constraint_bench(pp, torch, rate, res, peak):
    """Quotient-constraint operators over 2^22 extended-domain points (the 8x
    LDE of a 2^19-row circuit), with the integer-pipe fraction of each:
    18 Montgomery multiplies per point for the fused permutation terms and 104
    for the gate terms at sbox_alpha = 5, 256 multiply instructions each."""
    ppfr = pp.ppfr
    n = 1 << 22

    def vec(i):
        return ppfr.random_fr(n, 0xC0 + i)

    def scal(i):
        return ppfr.random_fr(1, 0xD0 + i)

    w = [vec(j) for j in range(4)]
    sig = [vec(4 + j) for j in range(4)]
    x, z, zn, mod, l1 = vec(8), vec(9), vec(10), vec(11), vec(12)
    ks = [scal(j) for j in range(3)]
    al, be, ga, one = scal(3), scal(4), scal(5), scal(6)
    out = ppfr.empty(n)
    name = "quotient_permutation_2^22"
    rate(name, lambda: ppfr.quotient_permutation(x, w, z, zn, sig, mod, l1, al, be, ga, ks, one,
                                                 out=out), n, 5)
    res[name].update({"MM_per_point": 18, "bytes_per_point": 448})
    del w, sig, x, z, zn, mod, l1
    V = {k: vec(20 + i) for i, k in enumerate(ppfr.GATE_VECTORS)}
    S = {k: scal(20 + i) for i, k in enumerate(ppfr.GATE_SCALARS)}
    # the prover's constants (one .. eightythree as integers): 81 multiplies
    # per point; any other scalars: 104
    name = "gate_constraint_2^22_general_scalars"
    rate(name, lambda: ppfr.gate_constraint(V, S, 5, out=out), n, 3)
    res[name].update({"MM_per_point": 104, "bytes_per_point": 736})
    S.update(gate_small_constants(ppfr))
    name = "gate_constraint_2^22"
    rate(name, lambda: ppfr.gate_constraint(V, S, 5, out=out), n, 3)
    res[name].update({"MM_per_point": 81, "bytes_per_point": 736})
    for k in ("quotient_permutation_2^22", "gate_constraint_2^22",
              "gate_constraint_2^22_general_scalars"):
        pts = res[k]["Melem_per_s"] * 1e6
        mm = res[k]["MM_per_point"]
        res[k]["int_frac_of_peak"] = round(pts * mm * 256 / peak, 4)


def gate_small_constants(ppfr):
    """four, one, two, three, nine, eighteen, eightyone, eightythree as the
    prover passes them: Montgomery forms of those integers, made on the
    device as powers of one plus additions."""
    one = ppfr.fr_powers(ppfr.random_fr(1, 0xE0), 1)  # x^0 = one
    out = {"one": one}
    for k, v in (("two", 2), ("three", 3), ("four", 4), ("nine", 9), ("eighteen", 18),
                 ("eightyone", 81), ("eightythree", 83)):
        acc = one
        for _ in range(v - 1):
            acc = ppfr.fr_binary(ppfr.FR_ADD, acc, one)
        out[k] = acc
    return out


def profile_op(args, pp, torch):
    """--lean --op msm|gate|perm|gpperm|scans|div: one operator at 2^lg
    points, device time only (the profiling case for ncu launch lists of
    those kernels).  gpperm is the copy-constraint grand product; scans is one
    grand product, one evaluation and one division by (X + c); div is the
    element-wise division a / b (div_mod)."""
    import numpy as np

    ppfr = pp.ppfr
    n = 1 << args.lg
    if args.op in ("msm", "msmfixed"):
        pts = msm_points(ppfr, n)
        sc = ppfr.random_fr(n, 5)
        out = torch.empty((3, 6), dtype=torch.int64, device="cuda")
        if args.op == "msm":
            fn = lambda: ppfr.msm_g1(pts, sc, out=out)  # noqa: E731
        else:
            bases = ppfr.MsmBases(pts)
            fn = lambda: bases.msm(sc, out=out)  # noqa: E731
    elif args.op == "gate":
        V = {k: ppfr.random_fr(n, 0x20 + i) for i, k in enumerate(ppfr.GATE_VECTORS)}
        S = {k: ppfr.random_fr(1, 0x80 + i) for i, k in enumerate(ppfr.GATE_SCALARS)}
        S.update(gate_small_constants(ppfr))
        out = ppfr.empty(n)
        fn = lambda: ppfr.gate_constraint(V, S, 5, out=out)  # noqa: E731
    elif args.op == "gpperm":
        w = [ppfr.random_fr(n, 0xA0 + j) for j in range(3)]
        sig = [ppfr.random_fr(n, 0xA8 + j) for j in range(3)]
        params = ppfr.random_fr(5, 0xAF)
        out = ppfr.empty(n)
        fn = lambda: ppfr.gp_perm(w, sig, params, out=out)  # noqa: E731
    elif args.op == "scans":
        x = ppfr.random_fr(n, 0xB0)
        pt = ppfr.random_fr(1, 0xB1)
        y = ppfr.empty(1)
        work = ppfr.empty(n)

        def fn():
            work.copy_(x)
            ppfr.gp_prefix_(work)
            ppfr.evaluate(x, pt, out=y)
            work.copy_(x)
            ppfr.div_xplusc_(work, pt)
    elif args.op == "div":
        a, b = ppfr.random_fr(n, 0xE1), ppfr.random_fr(n, 0xE2)
        out = ppfr.empty(n)
        fn = lambda: ppfr.fr_binary(ppfr.FR_DIV, a, b, out=out)  # noqa: E731
    else:
        vec = [ppfr.random_fr(n, 0xC0 + i) for i in range(13)]
        sca = [ppfr.random_fr(1, 0xD0 + i) for i in range(7)]
        out = ppfr.empty(n)
        fn = lambda: ppfr.quotient_permutation(  # noqa: E731
            vec[8], vec[0:4], vec[9], vec[10], vec[4:8], vec[11], vec[12], sca[3], sca[4], sca[5],
            sca[0:3], sca[6], out=out)
    l0 = pp.launch_count()
    ms = time_device(fn, args.steps, args.warmup, torch)
    print(json.dumps({"metric": "%s_2^%d" % (args.op, args.lg), "lean": True,
                      "ms_per_step": round(ms / args.steps, 4),
                      "gpu_launches": int(pp.launch_count() - l0)}), flush=True)


def msm_points(ppfr, n):
    """n G1 points: 1024 distinct multiples s_i G of the generator (seeded
    random s_i, made on the device by pp_g1_mul_gen, a set-up step outside
    any timed region) repeated to n.  The bucket method's work does not
    depend on repeated points."""
    base = ppfr.g1_mul_gen(ppfr.random_fr(1024, 77))
    reps = (n + 1023) // 1024
    return base.repeat(reps, 1)[:n].contiguous()


def msm_bench(pp, torch, rate, res, peak):
    """G1 multi-scalar multiplication of 2^20 points (msm_points); the
    scalars are seeded random canonical Fr values.  Integer fraction: W n
    mixed additions of ~10 Fq Montgomery multiplies (W = 256 / c + 1
    windows), each 4 * 12^2 = 576 32-bit multiply instructions, against the
    measured integer peak.  The fixed-base form times pp_msm_g1_fixed on
    window tables built once, outside the timed region."""
    ppfr = pp.ppfr
    n = 1 << 20
    pts = msm_points(ppfr, n)
    sc = ppfr.random_fr(n, 5)
    out = torch.empty((3, 6), dtype=torch.int64, device="cuda")
    name = "msm_g1_2^20"
    rate(name, lambda: ppfr.msm_g1(pts, sc, out=out), n, 3)
    c = ppfr.msm_window_bits(n)
    windows = 256 // c + 1
    instr = windows * n * 10 * 576
    res[name].update({"window_bits": c, "windows": windows,
                      "int_frac_of_peak": round(instr / (res[name]["ms"] / 1e3) / peak, 4),
                      "points": "1024 distinct generator multiples, tiled"})
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bases = ppfr.MsmBases(pts)
    torch.cuda.synchronize()
    build_ms = (time.perf_counter() - t0) * 1e3
    name = "msm_g1_fixed_2^20"
    rate(name, lambda: bases.msm(sc, out=out), n, 3)
    same = torch.equal(bases.msm(sc), ppfr.msm_g1(pts, sc))
    res[name].update({"window_bits": bases.window_bits, "windows": 256 // bases.window_bits + 1,
                      "table_gb": round(bases.table_bytes / 1e9, 3),
                      "table_build_ms": round(build_ms, 1), "same_as_plain": bool(same)})
    bases.close()


def batched_bench(pp, torch, count=96, lg_lo=12, lg_hi=22, peak=None):
    """count polynomials, sizes log-uniform in 2^lg_lo..2^lg_hi (seeded), in
    the proportions 2/3 NTT and INTT, 1/4 lambda=2 LDEs, 1/12 grand products
    (96 polynomials of 2^12..2^22: 64 / 24 / 8).  Loop of single calls vs one
    batch plan (a few persistent launches) vs its CUDA-graph replay."""
    import numpy as np

    P = pp.ppfr
    rng = np.random.default_rng(0xBA7C4)
    lgs = [int(v) for v in np.floor(rng.uniform(lg_lo, lg_hi + 1, count))]
    n_gp, n_lde = count // 12, count // 4
    n_ntt = count - n_gp - n_lde
    kinds = ([P.JOB_NTT] * (n_ntt - n_ntt // 2) + [P.JOB_INTT] * (n_ntt // 2) +
             [P.JOB_LDE_COEFFS] * n_lde + [P.JOB_GP] * n_gp)
    rng.shuffle(kinds)
    jobs, loop = [], []
    for i, (k, lg) in enumerate(zip(kinds, lgs)):
        lam = 2 if k == P.JOB_LDE_COEFFS else 0
        x = P.random_fr(1 << lg, 0xB000 + i)
        out = P.empty(1 << (lg + lam))
        jobs.append((k, x, out, lam))
        if k == P.JOB_NTT:
            loop.append(lambda x=x, out=out: P.ntt(x, out=out))
        elif k == P.JOB_INTT:
            loop.append(lambda x=x, out=out: P.ntt(x, True, out=out))
        elif k == P.JOB_LDE_COEFFS:
            loop.append(lambda x=x, out=out: P.lde(x, 2, P.LDE_COEFFS, out=out))
        else:
            loop.append(lambda x=x, out=out: (out.copy_(x), P.gp_prefix_(out)))
    elems = sum(1 << lg for lg in lgs)
    # algorithmic multiplies of the mix: NTT (N/2) lg N, INTT + N, lambda = 2
    # LDE from coefficients N + (4N/2)(lg N + 2), grand product N
    mm = 0
    for k, lg in zip(kinds, lgs):
        n = 1 << lg
        if k == P.JOB_NTT:
            mm += n // 2 * lg
        elif k == P.JOB_INTT:
            mm += n // 2 * lg + n
        elif k == P.JOB_LDE_COEFFS:
            mm += n + 2 * n * (lg + 2)
        else:
            mm += n
    l0 = P.launch_count()
    ms_loop = time_device(lambda: [f() for f in loop], 3, 1, torch) / 3
    loop_launches = (P.launch_count() - l0) // 4
    # the same loop captured in a CUDA graph: no host cost per call, so the
    # batch plan's gain over it is the device-side one (fewer, fuller launches)
    ms_loop_graph = None
    try:
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            [f() for f in loop]  # per-stream workspaces exist before capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            [f() for f in loop]
        ms_loop_graph = time_device(g.replay, 5, 2, torch) / 5
        del g
    except RuntimeError:
        torch.cuda.synchronize()
    b = P.Batch(jobs)
    info = b.info()
    ms_batch = time_device(b.run, 5, 2, torch) / 5
    b.capture()
    ms_graph = time_device(b.run, 10, 2, torch) / 10
    b.close()
    # the same comparison for each kind of job alone (plan against loop)
    by_kind = {}
    for label, ks in (("ntt_intt", (P.JOB_NTT, P.JOB_INTT)), ("lde_l2", (P.JOB_LDE_COEFFS,)),
                      ("gp", (P.JOB_GP,))):
        sel = [i for i, j in enumerate(jobs) if j[0] in ks]
        if not sel:
            continue
        sub = [loop[i] for i in sel]
        ms_l = time_device(lambda: [f() for f in sub], 3, 1, torch) / 3
        bk = P.Batch([jobs[i] for i in sel])
        ms_b = time_device(bk.run, 5, 2, torch) / 5
        bk.close()
        by_kind[label] = {"jobs": len(sel), "loop_ms": round(ms_l, 3), "batch_ms": round(ms_b, 3)}
    return {"polys": count, "lg_range": [lg_lo, lg_hi], "input_elems": elems,
            "loop_ms": round(ms_loop, 3),
            "loop_graph_ms": round(ms_loop_graph, 3) if ms_loop_graph else None,
            "batch_ms": round(ms_batch, 3),
            "graph_ms": round(ms_graph, 3), "loop_launches": int(loop_launches),
            "batch_launches": info["launches"], "speedup_batch": round(ms_loop / ms_batch, 3),
            "by_kind": by_kind,
            "algorithmic_MM": mm,
            # the mix's time at the measured mad.lo rate (256 instructions per
            # multiply), and the largest speed-up over the graph-captured loop
            # that this integer ceiling allows
            "int_ceiling_ms": round(mm * INSTR_PER_MM / peak * 1e3, 3) if peak else None,
            "max_speedup_vs_loop_graph": (round(ms_loop_graph / (mm * INSTR_PER_MM / peak * 1e3), 2)
                                          if peak and ms_loop_graph else None),
            "speedup_graph": round(ms_loop / ms_graph, 3),
            "Melem_per_s_graph": round(elems / (ms_graph / 1e3) / 1e6, 1)}


def serving_bench(pp, torch):
    """Poisson-arriving prover-round bundles (3 lambda=2 LDEs, 1 grand product,
    1 division, 6 evaluations), sizes log-uniform in 2^16..2^24, 200 per load
    point, at offered loads of 0.5, 0.8, 1.0 and 1.2 times the serial form's
    capacity: the continuous-batching server (150 GB budget, 8 slots, the work
    of running bundles capped near one 2^22 bundle) against the same bundles
    processed one at a time with the plain operators under the same arrivals.
    At 1.0 and 1.2 the server also runs without the work cap (every slot
    admits as soon as it is free)."""
    import numpy as np

    P = pp.ppfr
    rng = np.random.default_rng(0x5E7E)
    M = 200
    lgs = [int(v) for v in np.floor(rng.uniform(16, 25, M))]

    def serial_one(lg, seed):
        n = 1 << lg
        buf = P.empty(7 * n)
        P.check(P.lib().pp_random_fr(P._ptr(buf), 7 * n, seed, 0, P._stream()))
        prm = P.empty(12)
        P.check(P.lib().pp_random_fr(P._ptr(prm), 12, seed ^ 0x9A7A9A7A, 0, P._stream()))
        w = [buf[j * n:(j + 1) * n] for j in range(3)]
        s = [buf[(3 + j) * n:(4 + j) * n] for j in range(3)]
        for j in range(3):
            P.lde(w[j], 2, P.LDE_COEFFS)
        P.gp_perm(w, s, prm[:5].contiguous())
        P.div_xplusc_(buf[6 * n:7 * n], prm[5:6].contiguous())
        y = P.empty(6)
        for k in range(6):
            P.evaluate((w + s)[k], prm[6 + k:7 + k].contiguous(), out=y[k:k + 1])
        torch.cuda.synchronize()

    # warm service time of each size; their mean over the mix is the serial
    # form's capacity
    svc = {}
    for lg in sorted(set(lgs)):
        serial_one(lg, 1)
        t0 = time.perf_counter()
        for r in range(3):
            serial_one(lg, 2 + r)
        svc[lg] = (time.perf_counter() - t0) / 3
    mean_svc = sum(svc[lg] for lg in lgs) / M

    def pct(v, q):
        v = sorted(v)
        return v[min(len(v) - 1, int(round(q * (len(v) - 1))))]

    def run_serial(arrivals):
        lat = []
        start = time.perf_counter()
        for i, lg in enumerate(lgs):
            now = time.perf_counter() - start
            if now < arrivals[i]:
                time.sleep(arrivals[i] - now)
            serial_one(lg, 100 + i)
            lat.append((time.perf_counter() - start - arrivals[i]) * 1e3)
        span = time.perf_counter() - start
        return {"bundles_per_s": round(M / span, 2), "p50_ms": round(pct(lat, 0.5), 2),
                "p99_ms": round(pct(lat, 0.99), 2)}

    cap = P.bundle_work(22, 2)

    def run_server(arrivals, work_cap):
        import queue
        import threading

        srv = P.Server(budget_bytes=150 * 10**9, slots=8, min_lg=16, max_lg=24, lam=2,
                       max_inflight_mm=work_cap)
        for lg in sorted(set(lgs)):  # warm the slot streams
            srv.release(srv.wait(srv.submit(lg, 1)).ticket)
        srv.reset_stats()
        # the client consumes each result as it completes and releases its
        # memory (waits run in C, outside the interpreter lock)
        pending = queue.Queue()

        def consume():
            while True:
                t = pending.get()
                if t is None:
                    return
                srv.wait(t, 300000)
                srv.release(t)

        consumer = threading.Thread(target=consume)
        consumer.start()
        start = time.perf_counter()
        for i, lg in enumerate(lgs):
            now = time.perf_counter() - start
            if now < arrivals[i]:
                time.sleep(arrivals[i] - now)
            pending.put(srv.submit(lg, 100 + i))
        pending.put(None)
        consumer.join()
        st = srv.stats()
        srv.close()
        return {"bundles_per_s": round(st["bundles_per_s"], 2), "p50_ms": round(st["p50_ms"], 2),
                "p99_ms": round(st["p99_ms"], 2), "max_concurrent": int(st["max_concurrent"]),
                "admitted_while_busy": int(st["admitted_while_busy"]),
                "budget_peak_gb": round(st["budget_peak"] / 1e9, 2)}

    points = []
    for k, rho in enumerate((0.5, 0.8, 1.0, 1.2)):
        gaps = np.random.default_rng(0xA221 + k).exponential(mean_svc / rho, M)
        arrivals = np.cumsum(gaps) - gaps[0]
        pt = {"offered_load": rho, "offered_bundles_per_s": round(rho / mean_svc, 2),
              "serial": run_serial(arrivals), "server": run_server(arrivals, cap)}
        if rho >= 1.0:
            pt["server_no_work_cap"] = run_server(arrivals, 0)
        points.append(pt)
    return {"bundles_per_point": M, "lg_range": [16, 24], "serial_capacity_bundles_per_s": round(1 / mean_svc, 2),
            "work_cap_mm": cap, "points": points}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
