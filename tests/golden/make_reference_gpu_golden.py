"""Record golden outputs of the reference's own GPU operators.

Runs on a machine with a GPU and a staged copy of the reference sources
(``make -C oracle stage REF_CHECKOUT=<checkout>`` where a checkout exists; the
staged copy travels with the repository).  It builds the reference's GPU
operators for sm_103a (``make -C oracle refgpu``), runs them on seeded inputs
and writes ``reference_gpu.npz``:

    python tests/golden/make_reference_gpu_golden.py <out.npz> [--quick]

Inputs are ``oracle.random_fr(n, seed)`` (SplitMix64 limbs, rejection-sampled
below r, stored as the Montgomery representation), so a test regenerates them
from the seeds stored in the file.  Operators and what is kept:

* ``Ntt::forward`` / ``Intt::forward`` (PLONK/utils/function.cu:280,330):
  SHA-256 of the output plus 64 sampled elements at 2^18, 2^20, ..., 2^26.
  Nothing smaller: the reference's CTkernel advances its stage counter by the
  kernel radix, at least 6, instead of the kernel's iteration count
  (zksnark_ntt/ntt_kernel/ct_mixed_radix_wide.cuh:205,314), so below 2^18,
  where CT_NTT gives a kernel fewer than 6 iterations (algorithm.cuh:20-56),
  the later kernels index past the buffer.  At 2^13 that was an illegal
  address; those sizes are not run.
* ``our_ntt`` (ntt.cu:979) at the sizes the reference configures (2^22, 2^24,
  2^26; ntt.cu:1193-1206) and ``standard4_ntt`` (ntt.cu:1039) at 2^22 and
  2^24, on the same inputs as ``Ntt::forward``: SHA-256 of the output.
* ``our_lde`` (lde.cu:1267) at 2^20, 2^22, 2^24 with lambda = 2 and 3
  (lde.cu:1550-1580), input = N coefficients: SHA-256 plus 64 samples of the
  N * 2^lambda outputs.
* ``accumulate_mul_poly``, ``evaluate``, ``poly_div_poly``
  (PLONK/utils/function.cu:170-260): full outputs at 2^10; SHA-256 plus
  samples at 2^16, 2^20 and 2^22; the evaluation at every size.

Keys: ``<op>_<lg>[_<lambda>]_{full,sha,idx,val}`` and ``seed_<op>_<lg>[_<lambda>]``.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile
import time
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

GPU_DIR = os.path.join(ROOT, "oracle", "_ref", "gpu")
SEED_BASE = 0x5EED6000
NSAMPLE = 64

NTT_HASH = (18, 20, 22, 24, 26)
NTT_SPLIT = (22, 24, 26)
NTT_STD4 = (22, 24)
LDE_CASES = ((20, 2), (20, 3), (22, 2), (22, 3), (24, 2), (24, 3))
OPS_FULL = (10,)
OPS_HASH = (16, 20, 22)


def seed_for(op: str, lg: int, lam: int = 0) -> int:
    """Deterministic seed of an input vector; the tests use the same function."""
    code = {"ntt": 1, "lde": 2, "ops": 3, "opsx": 4, "opsc": 5}[op]
    return SEED_BASE + (code << 12) + (lg << 4) + lam


def sample_indices(n: int, key: int) -> np.ndarray:
    rng = np.random.default_rng(key)
    idx = rng.integers(0, n, size=NSAMPLE - 2, dtype=np.int64)
    return np.concatenate([[0, n - 1], idx]).astype(np.int64)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.uint64).tobytes()).hexdigest()


def run(args, timeout=900):
    t0 = time.time()
    r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(args)} exited {r.returncode}:\n{r.stdout[-2000:]}")
    print(f"  {os.path.basename(args[0])} {' '.join(args[1:2])} {args[2] if len(args) > 2 else ''}"
          f" ... {time.time() - t0:.1f} s", flush=True)
    return r.stdout


def write(path: str, a: np.ndarray) -> None:
    np.ascontiguousarray(a, dtype=np.uint64).tofile(path)


def read(path: str, n: int) -> np.ndarray:
    a = np.fromfile(path, dtype=np.uint64)
    assert a.size == 4 * n, (path, a.size, n)
    return a.reshape(n, 4)


def keep(out: dict, key: str, a: np.ndarray, full: bool, lg: int) -> None:
    if full:
        out[key + "_full"] = a
    else:
        idx = sample_indices(a.shape[0], zlib.crc32(key.encode()))
        out[key + "_sha"] = np.array(sha(a))
        out[key + "_idx"] = idx
        out[key + "_val"] = a[idx]


def main() -> int:
    if len(sys.argv) < 2:
        print(__doc__)
        return 2
    out_path = sys.argv[1]
    quick = "--quick" in sys.argv
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j16", "refgpu"], check=True)
    ntt_bin = os.path.join(GPU_DIR, "ref_ntt")
    lde_bin = os.path.join(GPU_DIR, "ref_lde")
    ops_bin = os.path.join(GPU_DIR, "ref_ops")
    out: dict = {"nsample": np.array(NSAMPLE)}
    ntt_hash = NTT_HASH[:2] if quick else NTT_HASH
    with tempfile.TemporaryDirectory() as tmp:
        fin, fout = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
        # --- Ntt::forward / Intt::forward, our_ntt, standard4_ntt
        for lg in ntt_hash:
            n = 1 << lg
            s = seed_for("ntt", lg)
            out[f"seed_ntt_{lg}"] = np.array(s)
            write(fin, O.random_fr(n, s))
            for op, cmd in (("ntt_fwd", "fwd"), ("ntt_inv", "inv")):
                run([ntt_bin, cmd, str(lg), fin, fout])
                keep(out, f"{op}_{lg}", read(fout, n), False, lg)
            for op, cmd, sizes in (("ntt_split", "split", NTT_SPLIT), ("ntt_std4", "std4", NTT_STD4)):
                if lg in sizes:
                    run([ntt_bin, cmd, str(lg), fin, fout])
                    out[f"{op}_{lg}_sha"] = np.array(sha(read(fout, n)))
        # --- our_lde
        for lg, lam in (LDE_CASES[:2] if quick else LDE_CASES):
            n = 1 << lg
            s = seed_for("lde", lg, lam)
            out[f"seed_lde_{lg}_{lam}"] = np.array(s)
            write(fin, O.random_fr(n, s))
            run([lde_bin, "lde", str(lg), str(lam), fin, fout], timeout=1800)
            keep(out, f"lde_{lg}_{lam}", read(fout, n << lam), False, lg)
        # --- grand product, evaluation, division
        fx, fc = os.path.join(tmp, "x.bin"), os.path.join(tmp, "c.bin")
        for lg in OPS_FULL + OPS_HASH:
            n = 1 << lg
            s, sx, sc = seed_for("ops", lg), seed_for("opsx", lg), seed_for("opsc", lg)
            out[f"seed_ops_{lg}"] = np.array([s, sx, sc])
            a = O.random_fr(n, s)
            write(fx, O.random_fr(1, sx))
            write(fc, O.random_fr(1, sc))
            write(fin, a)
            run([ops_bin, "gp", str(lg), fin, fout])
            keep(out, f"gp_{lg}", read(fout, n), lg in OPS_FULL, lg)
            run([ops_bin, "eval", str(lg), fin, fx, fout])
            out[f"eval_{lg}_full"] = read(fout, 1)
            run([ops_bin, "div", str(lg), fin, fc, fout])
            keep(out, f"div_{lg}", read(fout, n), lg in OPS_FULL, lg)
    np.savez_compressed(out_path, **out)
    print(f"wrote {out_path}: {len(out)} arrays")
    return 0


if __name__ == "__main__":
    sys.exit(main())
