"""Time the reference's own GPU operators and blst CPU baselines on this machine.

TEST/MEASUREMENT INFRASTRUCTURE.  Needs a GPU and the staged reference copy
(``make -C oracle stage REF_CHECKOUT=<checkout>``); builds the reference with
``make -C oracle refgpu`` and runs, on seeded synthetic inputs:

* ``Ntt::forward`` / ``Intt::forward`` (in HBM; CUDA events around the call,
  with and without the output allocation the call makes) at 2^22, 2^24, 2^26,
  and at 2^22, 2^24 from the as-shipped build (sm_75 code and compute_75 PTX,
  which the GB300 compiles at load: ``make -C oracle refgpu_jit``);
* the reference's own benchmark commands, unmodified, from its main functions:
  ``NTT --bench-split`` and ``--bench-baseline`` (ntt.cu:1471), ``LDE --bench``
  and ``--bench-naive`` (lde.cu:1808), and miss_ops' main (miss_ops.cu:88, its
  fixed 2^22 size).  Their ``../../input*.bin`` files are seeded random
  vectors of the right size;
* ``multi_scalar_mult`` (PLONK/utils/function.cu:396-412; wall clock, since
  its last step runs on the host) at 2^16 and 2^20 points: 1024 distinct
  multiples of the generator, tiled, and seeded scalars, as ``bench.py`` times
  ``pp_msm_g1``;
* the grand product, evaluation and division GPU calls and ``naive_gp`` /
  ``naive_div`` (one host thread) at 2^20, as the reference builds them
  (``-O0`` host code) and from an ``-O2`` build of the same source
  (``make -C oracle ref``).

    python oracle/ref_gpu_timings.py <out.json> [--quick]

Prints and writes one JSON object.
"""
from __future__ import annotations

import json
import os
import platform
import re
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

GPU_DIR = os.path.join(HERE, "_ref", "gpu")
SEED = 0x5EED7000


def run(args, cwd=None, timeout=1200):
    t0 = time.time()
    r = subprocess.run(args, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=timeout)
    dt = time.time() - t0
    print(f"  [{dt:6.1f} s] {' '.join(os.path.basename(a) if i == 0 else a for i, a in enumerate(args))}"
          f" -> rc {r.returncode}", flush=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-3000:])
    return r.stdout


def refjson(text: str) -> dict:
    for line in text.splitlines():
        if line.startswith("REFJSON "):
            return json.loads(line[len("REFJSON "):])
    raise RuntimeError("no REFJSON line")


def floats(pattern: str, text: str) -> list[float]:
    return [float(x) for x in re.findall(pattern, text)]


def summary(v: list[float]) -> dict:
    return {"min_ms": min(v), "mean_ms": sum(v) / len(v), "reps": len(v)} if v else {}


def main() -> int:
    out_path = sys.argv[1] if len(sys.argv) > 1 else "ref_gpu_timings.json"
    quick = "--quick" in sys.argv
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    subprocess.run(["make", "-s", "-C", HERE, "-j16", "refgpu"], check=True)
    jit_ok = subprocess.run(["make", "-s", "-C", HERE, "-j16", "refgpu_jit"]).returncode == 0
    ntt, lde, ops = (os.path.join(GPU_DIR, b) for b in ("ref_ntt", "ref_lde", "ref_ops"))
    ntt_jit = os.path.join(HERE, "_ref", "gpu_jit", "ref_ntt")
    res: dict = {"host": {"machine": platform.machine(), "nproc": os.cpu_count()},
                 "build": "reference sources, reference flags (-O0 -g host), device code sm_103a"}
    try:
        res["host"]["cpu"] = subprocess.run(["lscpu"], stdout=subprocess.PIPE, text=True).stdout
        m = re.search(r"Model name:\s*(.*)", res["host"]["cpu"])
        res["host"]["cpu"] = m.group(1).strip() if m else ""
    except OSError:
        res["host"]["cpu"] = ""
    sizes = (22, 24) if quick else (22, 24, 26)
    with tempfile.TemporaryDirectory() as tmp:
        wd = os.path.join(tmp, "a", "b")
        os.makedirs(wd)
        for lg, name in ((22, "input.bin"), (24, "input-24.bin"), (26, "input-26.bin")):
            if lg in sizes:
                O.random_fr(1 << lg, SEED + lg).tofile(os.path.join(tmp, name))
        # in-HBM Ntt::forward / Intt::forward
        res["ntt_in_hbm"] = {}
        for lg in sizes:
            res["ntt_in_hbm"][lg] = refjson(run([ntt, "time", str(lg), "10",
                                                 os.path.join(tmp, "input.bin" if lg == 22 else f"input-{lg}.bin")]))
        # the same from the as-shipped build (PTX compiled by the driver at load)
        res["ntt_in_hbm_as_shipped"] = {}
        for lg in (22, 24):
            if not jit_ok:
                res["ntt_in_hbm_as_shipped"] = {"unavailable": "make -C oracle refgpu_jit failed"}
                break
            res["ntt_in_hbm_as_shipped"][lg] = refjson(run([ntt_jit, "time", str(lg), "10",
                                                           os.path.join(tmp, "input.bin" if lg == 22
                                                                        else f"input-{lg}.bin")]))
        # the reference's own NTT benchmarks
        res["our_ntt"], res["standard4_ntt"] = {}, {}
        for lg in sizes:
            t = run([ntt, "refmain", "--bench-split", str(lg)], cwd=wd)
            res["our_ntt"][lg] = summary(floats(r"our-ntt execution time: ([0-9.]+) ms", t))
        for lg in sizes[:2]:
            t = run([ntt, "refmain", "--bench-baseline", str(lg)], cwd=wd, timeout=2400)
            per_k = {}
            for block in re.split(r"=== lg_N", t)[1:]:
                m = re.search(r"chunk_size = ([0-9.]+ [KM]B)", block)
                v = floats(r"standard4[_-]ntt execution time: ([0-9.]+) ms", block)
                if m and v:
                    per_k[m.group(1)] = summary(v)
            res["standard4_ntt"][lg] = {"per_chunk": per_k,
                                        "best_min_ms": min((x["min_ms"] for x in per_k.values()), default=None),
                                        "raw_tail": t[-600:] if not per_k else ""}
        # the reference's own LDE benchmarks
        res["our_lde"], res["naive_lde"] = {}, {}
        for lg in (20, 22, 24):
            if lg == 24 and quick:
                continue
            t = run([lde, "refmain", "--bench", str(lg)], cwd=wd, timeout=2400)
            for lam, block in zip((2, 3), re.split(r"\[lde\] lg_N=", t)[1:]):
                res["our_lde"][f"{lg}_{lam}"] = summary(floats(r"our-lde execution time: ([0-9.]+) ms", block))
        for lg in (20, 22):
            t = run([lde, "refmain", "--bench-naive", str(lg)], cwd=wd, timeout=2400)
            for lam, block in zip((2, 3), re.split(r"\[naive-lde\] lg_N=", t)[1:]):
                avgs = floats(r"\[naive_lde\] avg .*?: ([0-9.]+) ms", block)
                res["naive_lde"][f"{lg}_{lam}"] = {"best_avg_ms": min(avgs) if avgs else None,
                                                   "avg_per_k_ms": avgs}
        # grand product / evaluation / division at 2^20, and blst naive_gp / naive_div
        fin, fx, fc = (os.path.join(tmp, f) for f in ("ops_in.bin", "x.bin", "c.bin"))
        O.random_fr(1 << 20, SEED + 120).tofile(fin)
        O.random_fr(1, SEED + 121).tofile(fx)
        O.random_fr(1, SEED + 122).tofile(fc)
        res["miss_ops_2p20"] = refjson(run([ops, "time", "20", "10", fin, fx, fc]))
        # G1 multi-scalar multiplication
        import numpy as np
        base = O.g1_mul_gen(O.random_fr(1024, SEED + 130))
        fp, fs, fo = (os.path.join(tmp, f) for f in ("msm_p.bin", "msm_s.bin", "msm_o.bin"))
        res["msm"] = {}
        for lg in (16, 20):
            n = 1 << lg
            np.ascontiguousarray(np.tile(base, (n // 1024, 1)), dtype=np.uint64).tofile(fp)
            O.random_fr(n, SEED + 131).tofile(fs)
            res["msm"][lg] = refjson(run([ops, "msm", str(lg), "3", fp, fs, fo]))
        t = run([ops, "refmain"], cwd=wd, timeout=2400)
        res["miss_ops_main_2p22"] = {
            "naive_gp": summary(floats(r"\[naive_gp\] execution time: ([0-9.]+) ms", t)),
            "ours_gp": summary(floats(r"\[ours_gp\] execution time: ([0-9.]+) ms", t)),
            "ours_eval": summary(floats(r"\[ours_eval\] execution time: ([0-9.]+) ms", t)),
            "naive_div": summary(floats(r"\[naive_div\] execution time: ([0-9.]+) ms", t)),
            "ours_div": summary(floats(r"\[ours_div\] execution time: ([0-9.]+) ms", t)),
        }
    # the same naive_gp / naive_div from the -O2 build (oracle/Makefile ref)
    L = O.ref_lib()
    if L is not None:
        import numpy as np
        n = 1 << 20
        a = O.random_fr(n, SEED + 120)
        c = O.random_fr(1, SEED + 122)
        out = np.empty_like(a)
        t_gp, t_div = [], []
        for _ in range(3):
            t0 = time.perf_counter()
            L.ref_naive_gp(20, a.ctypes.data, out.ctypes.data)
            t_gp.append((time.perf_counter() - t0) * 1e3)
            t0 = time.perf_counter()
            L.ref_naive_div(20, a.ctypes.data, c.ctypes.data, out.ctypes.data)
            t_div.append((time.perf_counter() - t0) * 1e3)
        res["naive_O2_2p20"] = {"naive_gp": summary(t_gp), "naive_div": summary(t_div),
                                "note": "ctypes call into the -O2 build; includes the harness's two 32 MiB copies"}
    else:
        res["naive_O2_2p20"] = {"unavailable": "oracle/_ref/libppref.so could not be built"}
    text = json.dumps(res, indent=1, sort_keys=True)
    with open(out_path, "w") as f:
        f.write(text + "\n")
    print(text)
    return 0


if __name__ == "__main__":
    sys.exit(main())
