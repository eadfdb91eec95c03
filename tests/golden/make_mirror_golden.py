"""Regenerates mirror_hex_fatigue.npz: the class-interface example
lpm-mac_gb300/cpp/examples/hex_plate_tension.cpp compiled against the LPM
reference's own headers (unmodified, with the Eigen/Boost stand-in in
oracle/shim/) and run on the CPU.  The GPU test compiles the same source
against lpm-mac_gb300/cpp/ and compares the final positions.

Needs the reference sources (REF, default /root/reference); run by hand:

    python tests/golden/make_mirror_golden.py
"""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXAMPLE = os.path.join(ROOT, "lpm-mac_gb300", "cpp", "examples", "hex_plate_tension.cpp")
CG_TOL = "1e-12"
STEPS = "2"


def main():
    ref = os.environ.get("REF", "/root/reference")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "hex_ref")
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-I" + os.path.join(ref, "include"),
                        "-I" + os.path.join(ROOT, "oracle", "shim"), EXAMPLE, "-o", exe], check=True)
        out = os.path.join(tmp, "out.txt")
        env = dict(os.environ, LPM_ORACLE_CG_TOL=CG_TOL)
        log = subprocess.run([exe, out, "fatigue", STEPS], check=True, env=env, cwd=tmp, capture_output=True,
                             text=True).stdout
        data = np.loadtxt(out)
    newton = [line for line in log.splitlines() if "Iteration-" in line]
    np.savez_compressed(os.path.join(HERE, "mirror_hex_fatigue.npz"), id=data[:, 0].astype(np.int64),
                        xyz=data[:, 1:4], xyz0=data[:, 4:7], newton_iters=np.int64(len(newton)),
                        meta=np.array(["hex_plate_tension fatigue " + STEPS, "cg_tol=" + CG_TOL]))
    print("mirror_hex_fatigue.npz:", data.shape[0], "particles,", len(newton), "Newton iterations")


if __name__ == "__main__":
    main()
