"""Record golden outputs of the reference's own GPU multi-scalar
multiplication, ``multi_scalar_mult`` (PLONK/utils/function.cu:396-412:
cuda::msm_zkp_cuda, zkp/cuda/zksnark_msm.cu:48-88, then the host step
cpu::msm_collect_cpu, zkp/cpu/msmcollect.cpp:5-41).

Runs on a machine with a GPU and the staged reference copy (as
make_reference_gpu_golden.py); builds it with ``make -C oracle refgpu``:

    python tests/golden/make_reference_msm_golden.py <out.npz>

Inputs, regenerated by the test from the stored seeds: points s_i G with
s_i = oracle.random_fr(n, seed_points) read as plain integers (affine,
Montgomery coordinates, by the oracle's g1_mul_gen), scalars =
oracle.random_fr(n, seed_scalars) read as plain integers (below r).  Kept per
size 2^lg: ``msm_<lg>_seeds`` and ``msm_<lg>_jacobian`` -- the reference's
result as it returns it, Jacobian X, Y, Z in Montgomery form (18 words).
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

GPU_DIR = os.path.join(ROOT, "oracle", "_ref", "gpu")
SIZES = (10, 12, 14)
SEED_BASE = 0x5EED9000


def seeds_for(lg: int):
    """(points seed, scalars seed) of size 2^lg; the test uses the same function."""
    return SEED_BASE + 2 * lg, SEED_BASE + 2 * lg + 1


def inputs(lg: int):
    sp, ss = seeds_for(lg)
    n = 1 << lg
    points = O.g1_mul_gen(O.random_fr(n, sp))
    scalars = O.random_fr(n, ss)
    return points, scalars


def main() -> int:
    if len(sys.argv) < 2:
        print(__doc__)
        return 2
    out_path = sys.argv[1]
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j16", "refgpu"], check=True)
    ops_bin = os.path.join(GPU_DIR, "ref_ops")
    out: dict = {}
    with tempfile.TemporaryDirectory() as tmp:
        fp, fs, fo = (os.path.join(tmp, f) for f in ("p.bin", "s.bin", "o.bin"))
        for lg in SIZES:
            points, scalars = inputs(lg)
            np.ascontiguousarray(points, dtype=np.uint64).tofile(fp)
            np.ascontiguousarray(scalars, dtype=np.uint64).tofile(fs)
            r = subprocess.run([ops_bin, "msm", str(lg), "0", fp, fs, fo], stdout=subprocess.PIPE,
                               stderr=subprocess.STDOUT, text=True, timeout=600)
            if r.returncode != 0:
                raise RuntimeError(r.stdout[-2000:])
            out[f"msm_{lg}_seeds"] = np.array(seeds_for(lg), dtype=np.uint64)
            out[f"msm_{lg}_jacobian"] = np.fromfile(fo, dtype=np.uint64)
            print(f"  msm 2^{lg} done", flush=True)
    np.savez_compressed(out_path, **out)
    print(f"wrote {out_path}: {len(out)} arrays")
    return 0


if __name__ == "__main__":
    sys.exit(main())
