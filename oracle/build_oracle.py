"""Compile the C restatement (lbm_ref.c) into oracle/_build/liblbm_oracle.so.

Test infrastructure: the checker and the CPU baseline, never the product.
gcc with OpenMP and -ffp-contract=off (no fused multiply-add), no -ffast-math.
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "liblbm_oracle.so")
SRCS = [os.path.join(HERE, "lbm_ref.c"), os.path.join(HERE, "lbm_ref_body.h")]


def build(force=False):
    if not force and os.path.exists(OUT) and all(os.path.getmtime(s) <= os.path.getmtime(OUT) for s in SRCS + [__file__]):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           SRCS[0], "-o", OUT + ".tmp", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
