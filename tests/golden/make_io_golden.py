"""Regenerates tests/golden/io/: lpm-mac_gb300/cpp/examples/io_roundtrip.cpp
compiled against the LPM reference's own headers (unmodified, with the
Eigen/Boost stand-in in oracle/shim/), run in write mode (the reference's
writeConfigurationDump and writeBond of a hexagonal plate) and then in read
mode (readDump and readBond, then writeBond, writeConfigurationDump and three
writeDump calls).  tests/test_class_mirror.py runs read mode against
lpm-mac_gb300/cpp/ on the same inputs and compares the files byte for byte.

Needs the reference sources (REF, default /root/reference); run by hand:

    python tests/golden/make_io_golden.py
"""
import os
import shutil
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(ROOT, "lpm-mac_gb300", "cpp", "examples", "io_roundtrip.cpp")
OUT = os.path.join(HERE, "io")
FILES = ["config.dump", "plate.bond", "rt.bond", "rt_config.dump", "rt.dump"]


def main():
    ref = os.environ.get("REF", "/root/reference")
    os.makedirs(OUT, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "io_ref")
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-w",
                        "-I" + os.path.join(ref, "include"), "-I" + os.path.join(ROOT, "oracle", "shim"), SRC, "-o",
                        exe], check=True)
        subprocess.run([exe, "write", tmp], check=True, cwd=tmp)
        subprocess.run([exe, "read", tmp], check=True, cwd=tmp, capture_output=True)
        for f in FILES:
            shutil.copy(os.path.join(tmp, f), os.path.join(OUT, f))
    print("tests/golden/io:", ", ".join("%s (%d B)" % (f, os.path.getsize(os.path.join(OUT, f))) for f in FILES))


if __name__ == "__main__":
    main()
