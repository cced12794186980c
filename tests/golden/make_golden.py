"""Generate tests/golden/gpblocks_bcc.npz from the reference's own CPU stepper.

Runs oracle/_ref/ref_gpblocks (built by oracle/build_ref.sh from the unmodified
reference sources GrossPitaevskii/GPBlocks.cpp + VortexState + Mesh + Output +
Types) in a temporary directory and stores its set-up arrays and the
normsq/error values it printed after each iteration
(GrossPitaevskii/GPBlocks.cpp:531-538).  Run where the reference tree exists:

    sh oracle/build_ref.sh && python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(ROOT, "oracle", "_ref", "ref_gpblocks")

# kappa, g, block_scale, half box, iterations, vortex relaxation iterations
CASES = {"gpblocks_bcc": ("1", "40", "0.25", "3.0", "3", "400")}


def read_dump(path):
    b = open(path, "rb").read()
    X, Y, Z, V, deg, steps, iters = np.frombuffer(b[:28], dtype=np.int32)
    lapfac, lapfac0, g, volume, dt = np.frombuffer(b[28:68])
    off = 68
    lapind = np.frombuffer(b[off:off + 8 * V * deg], dtype=np.int64)
    off += 8 * V * deg
    bsize, bxsize = V, (X + 1) * V
    bxysize = (Y + 1) * bxsize
    ii0 = bxysize + bxsize + bsize
    vsize = ii0 + (Z + 1) * bxysize

    def take(n):
        nonlocal off
        a = np.frombuffer(b[off:off + 8 * n]).copy()
        off += 8 * n
        return a

    psi0, pot, even, odd = take(2 * vsize), take(vsize), take(2 * vsize), take(2 * vsize)
    ne = take(2 * (iters + 1)).reshape(-1, 2)
    return dict(dims=np.array([X, Y, Z, V, deg, steps, iters], dtype=np.int64), scal=np.array([lapfac, lapfac0, g, volume, dt]),
                lapind=lapind, psi0=psi0, pot=pot, even=even, odd=odd, normsq_error=ne)


def main():
    if not os.path.exists(EXE):
        sys.exit("build oracle/_ref first: sh oracle/build_ref.sh")
    for name, args in CASES.items():
        with tempfile.TemporaryDirectory() as d:
            out = os.path.join(d, "dump.bin")
            subprocess.run([EXE, out] + list(args), check=True, cwd=d, capture_output=True)
            data = read_dump(out)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), args=np.array(args), **data)
        print(name, data["dims"], data["normsq_error"].tolist())


if __name__ == "__main__":
    main()
