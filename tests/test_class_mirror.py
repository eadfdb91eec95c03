"""The LPM class interface on the GPU path (lpm-mac_gb300/cpp/).

A program written against the reference's classes (Assembly, Particle*,
LoadStep, SolverStatic, SolverFatigue, utilities.h) compiles against these
headers unchanged and runs its solve on the device.  The GPU test runs the
example in lpm-mac_gb300/cpp/examples/ and compares it with the same source
compiled against the reference's own headers (tests/golden/mirror_hex_fatigue.npz,
made by tests/golden/make_mirror_golden.py).
"""
import glob
import os
import subprocess

import numpy as np
import pytest

from lpm_cases import pkg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "lpm-mac_gb300", "cpp")
EXAMPLE = os.path.join(CPP, "examples", "hex_plate_tension.cpp")
GOLDEN = os.path.join(ROOT, "tests", "golden", "mirror_hex_fatigue.npz")
# examples of the reference that do not compile against its own headers
# either (members and enum values its headers no longer have)
BROKEN_UPSTREAM = {"ex1_isoelasticity_3d_sc", "ex3_singlecrystal_3d_fcc"}


def compile_example(src, out, link=True):
    # no FMA contraction, so that the lattice generator rounds as on x86
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-I" + CPP, "-I" + os.path.join(ROOT, "include"),
           src]
    if link:
        lib = pkg.build.build()
        d = os.path.dirname(lib)
        cmd += ["-o", out, "-L" + d, "-llpmgpu", "-Wl,-rpath," + d]
    else:
        cmd += ["-fsyntax-only"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_example_compiles_and_links(tmp_path):
    compile_example(EXAMPLE, str(tmp_path / "hex"), link=True)
    assert os.path.exists(tmp_path / "hex")


def test_reference_examples_compile_against_mirror(tmp_path):
    ref = os.environ.get("REF", "/root/reference")
    examples = sorted(glob.glob(os.path.join(ref, "examples", "ex*.cpp")))
    if not examples:
        pytest.skip("reference examples not present")
    failed = []
    for ex in examples:
        name = os.path.splitext(os.path.basename(ex))[0]
        main = tmp_path / (name + "_main.cpp")
        main.write_text('#include "%s"\nint main() { run(); return 0; }\n' % ex)
        cmd = ["g++", "-std=c++17", "-fsyntax-only", "-fopenmp", "-I" + CPP, "-I" + os.path.join(ROOT, "include"),
               str(main)]
        if subprocess.run(cmd, capture_output=True).returncode != 0:
            failed.append(name)
    assert set(failed) == BROKEN_UPSTREAM, failed
    assert len(examples) - len(failed) >= 16


@pytest.mark.gpu
def test_example_matches_reference_headers(tmp_path):
    g = np.load(GOLDEN)
    exe = str(tmp_path / "hex")
    compile_example(EXAMPLE, exe, link=True)
    out = str(tmp_path / "out.txt")
    env = dict(os.environ, LPM_CG_TOL="1e-12")
    r = subprocess.run([exe, out, "fatigue", "2"], capture_output=True, text=True, env=env, cwd=str(tmp_path),
                       timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    newton = [line for line in r.stdout.splitlines() if "Iteration-" in line]
    assert len(newton) == int(g["newton_iters"])
    d = np.loadtxt(out)
    assert np.array_equal(d[:, 0].astype(np.int64), g["id"])
    # the same generator arithmetic; allow last-bit differences of libm
    assert np.abs(d[:, 4:7] - g["xyz0"]).max() <= 1e-13 * np.abs(g["xyz0"]).max()
    u_ref = g["xyz"] - g["xyz0"]
    u_gpu = d[:, 1:4] - d[:, 4:7]
    assert np.abs(u_gpu - u_ref).max() <= 1e-8 * np.abs(u_ref).max()


FD_PROGRAM = r'''
#include "lpm.h"
#include "particle.h"
#include "assembly.h"
#include "utilities.h"
#include "stiffness.h"
#include "load_step.h"
#include "solver_static.h"
int main() {
  UnitCell cell(LatticeType::Hexagon2D, 0.25);
  double angles[] = {0.0, 0.0, 0.0};
  Eigen::MatrixXd R = createRMatrix(0, angles);
  std::array<double, 2 * NDIM> box{0.0, 3.0, 0.0, 3.0, 0.0, 1.0};
  std::vector<std::array<double, NDIM>> xyz = createPlateHEX2D(box, cell, R);
  Assembly<2> ass{xyz, box, cell, ParticleType::Elastic};
  for (Particle<2>* p : ass.pt_sys)
    dynamic_cast<ParticleElastic<2>*>(p)->setParticleProperty(0.0, true, 69e3, 0.3, 1.0);
  SolverStatic<2> solv{-1, ass, StiffnessMode::FiniteDifference, SolverMode::CG, "fd.dump", 30, 1e-5};
  printf("constructed\n");
  return 0;
}
'''


@pytest.mark.gpu
def test_finite_difference_tangent_is_refused(tmp_path):
    """StiffnessMode::FiniteDifference (stiffness.h:103-154) has no device
    version: a program asking for it stops with an error when the solver is
    constructed, instead of running with the analytical tangent.  (The
    Assembly constructor already searches bonds on the GPU.)"""
    src = tmp_path / "fd.cpp"
    src.write_text(FD_PROGRAM)
    exe = str(tmp_path / "fd")
    compile_example(str(src), exe, link=True)
    r = subprocess.run([exe], capture_output=True, text=True, cwd=str(tmp_path), timeout=120)
    assert r.returncode == 1
    assert "FiniteDifference is not supported" in r.stderr
    assert "constructed" not in r.stdout


IO_SRC = os.path.join(CPP, "examples", "io_roundtrip.cpp")
IO_GOLDEN = os.path.join(ROOT, "tests", "golden", "io")


@pytest.mark.parametrize("sync", ["0", "1"])
def test_dump_and_bond_files_match_reference_writers(tmp_path, sync):
    """readDump and readBond on files the reference's writers made, then
    writeBond, writeConfigurationDump and three writeDump calls: the files
    equal the reference build's byte for byte (tests/golden/io, made by
    tests/golden/make_io_golden.py).  The dumps go through the asynchronous
    writer (LPM_DUMP_SYNC=0) or the calling thread (LPM_DUMP_SYNC=1).  No
    device call is made, so this runs without a GPU."""
    import shutil
    exe = str(tmp_path / "io")
    compile_example(IO_SRC, exe, link=True)
    for f in ("config.dump", "plate.bond"):
        shutil.copy(os.path.join(IO_GOLDEN, f), tmp_path / f)
    r = subprocess.run([exe, "read", str(tmp_path)], capture_output=True, text=True, timeout=120,
                       env=dict(os.environ, LPM_DUMP_SYNC=sync))
    assert r.returncode == 0, r.stderr[-2000:]
    for f in ("rt.bond", "rt_config.dump", "rt.dump"):
        with open(tmp_path / f, "rb") as a, open(os.path.join(IO_GOLDEN, f), "rb") as b:
            assert a.read() == b.read(), f


@pytest.mark.gpu
def test_plate_files_written_like_reference(tmp_path):
    """Write mode: the plate's configuration dump equals the reference's;
    its bond file lists the same directed bonds (layer, p1, p2) in the same
    order (the reference numbers bonds from a counter that its O(N^2) search
    also advances, so the id column differs)."""
    exe = str(tmp_path / "io")
    compile_example(IO_SRC, exe, link=True)
    r = subprocess.run([exe, "write", str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    with open(tmp_path / "config.dump", "rb") as a, open(os.path.join(IO_GOLDEN, "config.dump"), "rb") as b:
        assert a.read() == b.read()
    mine = np.loadtxt(tmp_path / "plate.bond", dtype=np.int64)
    ref = np.loadtxt(os.path.join(IO_GOLDEN, "plate.bond"), dtype=np.int64)
    assert np.array_equal(mine[:, 1:], ref[:, 1:])
