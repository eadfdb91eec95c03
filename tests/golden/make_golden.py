"""Regenerates the golden fixtures in this directory.

The fixtures come from the LPM reference itself: its headers, unmodified,
compiled against the Eigen/Boost stand-in in oracle/shim/ into
oracle/_ref/ref_driver (``make -C oracle ref``).  This script needs the
reference sources (REF, default /root/reference) and is run by hand; the
tests only read the .npz files it writes.

    python tests/golden/make_golden.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")

# name: (driver case, options, CG tolerance for the shim's knob)
CASES = {
    # force state + tangent + one CG solve at a perturbed, partly damaged state
    "kernels_hex": ("kernels-hex", ["ncol=9", "nrow=9", "a=0.5", "mapping=row", "damage_every=7"], "1e-10"),
    "kernels_sc": ("kernels-sc", ["n=5", "a=0.2", "mapping=row", "damage_every=7"], "1e-10"),
    "kernels_hex_refmap": ("kernels-hex", ["ncol=9", "nrow=9", "a=0.5", "mapping=ref", "damage_every=5"], "1e-10"),
    "kernels_sc_undamaged": ("kernels-sc", ["n=4", "a=0.2", "mapping=row", "amp=0.01"], "1e-10"),
    # load steps through SolverFatigue::solveProblemStatic (BC elimination)
    "steps_hex_fatigue": ("steps-hex", ["ncol=15", "nrow=15", "a=0.5", "mapping=row", "steps=3", "du=0.001",
                                        "solver=fatigue", "all_xyz=1"], "1e-10"),
    "steps_sc_fatigue": ("steps-sc", ["n=5", "a=0.2", "mapping=row", "steps=2", "du=0.002", "solver=fatigue",
                                      "all_xyz=1"], "1e-10"),
    # one update of each material law (state variables, nonlocal damage rate,
    # damage, plastic bond stretch) at a stretched, perturbed state
    "law_damage_hex": ("laws-hex", ["ncol=11", "nrow=11", "a=0.5", "law=damage", "nonlocal_L=0.6", "stretch=0.015"],
                       "1e-10"),
    "law_j2_sc": ("laws-sc", ["n=5", "a=0.2", "law=j2", "nonlocal_L=0.25", "stretch=0.02", "amp=0.002"], "1e-10"),
    "law_j2_hex": ("laws-hex", ["ncol=9", "nrow=9", "a=0.5", "law=j2", "nonlocal_L=0.6", "stretch=0.02",
                                "amp=0.002"], "1e-10"),
    "law_hcf_hex": ("laws-hex", ["ncol=11", "nrow=11", "a=0.5", "law=hcf", "nonlocal_L=0.6", "stretch=0.004",
                                 "dNdt=1000"], "1e-10"),
    # configuration 1: 41 x 41 hexagonal plate, 1,661 particles, 10 steps
    "config1_hex": ("steps-hex", ["ncol=41", "nrow=41", "a=0.5", "mapping=row", "steps=10", "du=0.001",
                                  "solver=fatigue"], "1e-10"),
}


def read_bin(path):
    out = {}
    with open(path, "rb") as f:
        while True:
            line = f.readline()
            if not line:
                break
            name, dt, n = line.decode().split()
            n = int(n)
            out[name] = np.frombuffer(f.read(8 * n), dtype="<f8" if dt == "f8" else "<i8").copy()
    return out


def main():
    ref = os.environ.get("REF", "/root/reference")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + ref], check=True)
    only = sys.argv[1:]
    for name, (case, opts, tol) in CASES.items():
        if only and name not in only:
            continue
        tmp = os.path.join(HERE, name + ".bin")
        env = dict(os.environ, LPM_ORACLE_CG_TOL=tol)
        subprocess.run([DRIVER, case, tmp] + opts, check=True, env=env, stdout=subprocess.DEVNULL)
        data = read_bin(tmp)
        os.remove(tmp)
        meta = np.array([case] + opts + ["cg_tol=" + tol])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), _meta=meta, **data)
        print(name, sum(v.nbytes for v in data.values()), "bytes")


if __name__ == "__main__":
    main()
