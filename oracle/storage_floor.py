"""TEST / MEASUREMENT INFRASTRUCTURE, not product code.

Builds oracle/storage_floor.c (gcc -O2 -fopenmp) into oracle/_ref/ and runs
the D3Q19 sphere channel 128x64x64 (r = 6, tau = 0.5343, inlet u = 0.05, the
sphere case of bench.py at 1/4 of its size) in every candidate storage,
printing each one's velocity relative L2 error against the FP64 run after
the same steps:

    python oracle/storage_floor.py [steps]        (default 5000)

The storages and arithmetic are described in storage_floor.c.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CASE = ["128", "64", "64", "6", "32", "32", "32", "0.5343147850940348"]
VARIANTS = [
    (1, 2, "FP32 storage of the shifted state, FP32 arithmetic"),
    (4, 2, "FP16 of the shifted state, FP32 arithmetic (the engine's f16dev)"),
    (2, 0, "FP16 of the unshifted deviation, FP64 arithmetic"),
    (4, 0, "FP16 of the shifted state, FP64 arithmetic"),
    (14, 2, "FP16 of the shifted state with stochastic rounding, FP32 arithmetic"),
    (6, 2, "1-4-11 16-bit float of the shifted state, FP32 arithmetic"),
    (7, 2, "1-3-12 16-bit float of the shifted state, FP32 arithmetic"),
    (8, 2, "16-bit fixed point of the shifted state, FP32 arithmetic"),
    (9, 2, "16-bit block floating point of the shifted state (one exponent per cell), FP32 arithmetic"),
    (10, 2, "the same with the slot owner's exponent as AA in-place streaming would hold it, FP32 arithmetic"),
]


def build() -> str:
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "storage_floor")
    src = os.path.join(HERE, "storage_floor.c")
    if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-fopenmp", "-o", exe, src, "-lm"], check=True)
    return exe


def velocity(exe, steps, store, arith, tmp):
    out = os.path.join(tmp, f"u_{store}_{arith}.bin")
    subprocess.run([exe] + CASE + [str(steps), str(store), str(arith), out], check=True)
    return np.fromfile(out).reshape(-1, 4)[:, 1:]


def main(argv):
    steps = int(argv[1]) if len(argv) > 1 else 5000
    exe = build()
    with tempfile.TemporaryDirectory() as tmp:
        ref = velocity(exe, steps, 0, 0, tmp)
        print(f"D3Q19 sphere 128x64x64, {steps} steps from the free stream; velocity relative L2 against FP64")
        for store, arith, what in VARIANTS:
            u = velocity(exe, steps, store, arith, tmp)
            print(f"{np.linalg.norm(u - ref) / np.linalg.norm(ref):.3e}  {what}", flush=True)


if __name__ == "__main__":
    main(sys.argv)
