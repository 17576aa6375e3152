"""The C++ drop-in header (include/dfm2g.hpp) compiles and links against
libdfm2g.so (CPU), and a DelFEM2-style caller written against it reproduces
the reference's solve (GPU)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cxx", "dropin_main.cpp")
EXE = os.path.join(ROOT, "delfem2_gb300", "_build", "dropin_main")


@pytest.fixture(scope="module")
def exe(built_lib):
    libdir = os.path.join(ROOT, "delfem2_gb300", "_build")
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), SRC, "-o", EXE, "-L" + libdir,
           "-ldfm2g", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return EXE


def test_dropin_header_compiles_and_links(exe):
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_dropin_caller_matches_oracle(exe, gpu, port, tmp_path):
    dump = str(tmp_path / "compat.bin")
    out = subprocess.run([exe, "8", dump], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    f = out.stdout.split()
    its, res, xsum = int(f[1]), float(f[3]), float(f[5])
    its2, xsum2 = int(f[7]), float(f[9])
    # the compatibility path (device vectors through the ADL primitives) takes
    # the same iterations as the whole-loop device solve
    assert abs(its2 - its) <= 1
    assert abs(xsum2 - xsum) <= 1e-8 * abs(xsum)
    # the same problem through the oracle
    xyz, tet = port.voxel_tet_mesh(8, 8, 8, 1 / 8)
    np_ = xyz.size // 3
    ind, psup = port.psup(tet, 4, np_)
    vc, vd, b = np.zeros(psup.size * 9), np.zeros(np_ * 9), np.zeros(np_ * 3)
    port.assemble_tet_linear(ind, psup, vc, vd, b, xyz, tet, np.ones(tet.size // 4), 0.3, 1.0, [0, 0, -1e-3])
    bc = np.zeros(np_ * 3, np.int32)
    bc[np.repeat(xyz[2::3] == 0.0, 3)] = 1
    port.set_fixed_bc(ind, psup, vc, vd, bc)
    port.rhs_zero(b, bc)
    col, dia = port.ilu_pattern0(ind, psup)
    ivc, ivd = port.ilu_copy_value(ind, col, psup, vc, vd)
    port.ilu_decompose(ind, col, dia, ivc, ivd)
    x, _, h = port.solve_pcg(ind, psup, vc, vd, col, dia, ivc, ivd, b, 1e-10, 1000)
    assert abs(its - (len(h) - 1)) <= 1
    # the compatibility path (a PCG written step for step as the reference's
    # Solve_PCG over device vectors): its history and solution against the oracle's
    raw = np.fromfile(dump, np.uint8)
    nh = int(np.frombuffer(raw[:8], np.uint64)[0])
    hist2 = np.frombuffer(raw[8:8 + 8 * nh], np.float64)
    x2 = np.frombuffer(raw[8 + 8 * nh:], np.float64)
    assert abs(len(hist2) - len(h)) <= 1
    assert abs(hist2[0] - h[0]) <= 1e-12 * h[0]  # |r0|: the same right-hand side
    assert np.abs(x2 - x).max() <= 1e-8 * np.abs(x).max()
    assert res < 1e-9
    assert abs(xsum - x.sum()) <= 1e-8 * np.abs(x).sum()


COMPAT = os.path.join(ROOT, "tests", "cxx", "compat_reference_pcg.cpp")
# The DelFEM2 source tree, when the environment names it (no default).
REF_ROOT = os.environ.get("DFM2_REFERENCE_ROOT", "")
REF_INCLUDE = os.path.join(REF_ROOT, "include") if REF_ROOT else ""


@pytest.mark.skipif(not (REF_INCLUDE and os.path.isdir(os.path.join(REF_INCLUDE, "delfem2"))),
                    reason="DFM2_REFERENCE_ROOT does not name a DelFEM2 source tree")
def test_reference_solve_pcg_template_accepts_device_views():
    """The reference's own generic Solve_PCG (lsitrsol.h:80-148) instantiates
    with delfem2::gb300::DeviceVectorView, CMatrixSparse<double> and
    CPreconditionerILU<double>: the compatibility path is a type-level drop-in
    (compile check, no GPU)."""
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-I" + REF_INCLUDE, "-I" + os.path.join(ROOT, "include"), COMPAT]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
