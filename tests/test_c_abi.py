"""The C-ABI from C: tests/c/qgpu_drop_in.c, built with gcc against
include/qgpu.h and linked to libqgpu.so, makes qdyn's call sequence
(qgpu_create, qgpu_build_lists, qgpu_forces, qgpu_shake, qgpu_destroy) on the
reference's sphere test system at step 0 and checks the 12 printed columns of
tests/basic_tests/SPH_leap-frog_berendsen_benchmark.en row 1 itself.  Its
SHAKE result (every atom displaced, then qgpu_shake) is compared here with
the oracle's SHAKE of the same coordinates.  No Python binding is involved in
the calls: the test only writes the descriptor file and runs the program."""
import ctypes as C
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_system

SRC = os.path.join(ROOT, "tests", "c", "qgpu_drop_in.c")
COLUMNS = ["QEL", "QVdW", "EL", "VdW", "QBND", "QANG", "QTOR", "QIMP", "BND", "ANG", "TOR", "IMP"]


def _cuda_lib_dir():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.isdir(os.path.join(d, "lib64")):
            return os.path.join(d, "lib64")
    return None


def build_program(out_dir: str) -> str:
    """gcc the C host against include/qgpu.h and the in-tree libqgpu.so."""
    from qsource_gb300 import build
    lib = build.build()
    gcc = shutil.which("gcc") or shutil.which("cc")
    if not gcc:
        pytest.skip("no C compiler")
    exe = os.path.join(out_dir, "qgpu_drop_in")
    libdir = os.path.dirname(lib)
    cmd = [gcc, "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-o", exe, "-L" + libdir, "-lqgpu", "-Wl,-rpath," + libdir, "-lm"]
    cuda = _cuda_lib_dir()
    if cuda:
        cmd.append("-Wl,-rpath-link," + cuda)
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    return exe


def write_descriptor(system, path: str) -> None:
    """The qgpu_system_desc of `system` as the program reads it: the struct
    bytes, the byte offsets of its pointer fields, and the arrays they point
    to, each pointer replaced by its array's offset in the array block (-1 for
    NULL)."""
    from qsource_gb300.abi import SystemDesc
    d = system.desc()
    arrays = {a.ctypes.data: a for a in system._keep}
    raw = bytearray(bytes(d))
    rel, blocks, off = [], [], 0
    for name, typ in SystemDesc._fields_:
        if typ is not C.c_void_p:
            continue
        fo = getattr(SystemDesc, name).offset
        p = getattr(d, name)
        if p:
            a = arrays[p]
            struct.pack_into("<q", raw, fo, off)
            b = a.tobytes()
            b += b"\0" * ((-len(b)) % 8)
            blocks.append(b)
            off += len(b)
        else:
            struct.pack_into("<q", raw, fo, -1)
        rel.append(fo)
    with open(path, "wb") as f:
        f.write(b"QGPUDESC")
        f.write(struct.pack("<3Q", len(raw), len(rel), off))
        f.write(bytes(raw))
        f.write(struct.pack(f"<{len(rel)}Q", *rel))
        for b in blocks:
            f.write(b)


def test_c_host_builds_against_the_header(tmp_path):
    """The header compiles as C99 with every warning an error, and the program
    links against the library (no GPU needed)."""
    exe = build_program(str(tmp_path))
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
def test_c_host_reproduces_the_golden_columns(tmp_path, golden):
    from oracle.oracle import Oracle
    g = golden_system("basic_sph")
    o = Oracle(g)
    o.maxwell(g.Tmaxw, int(g.seed))
    assert o.initial_shaking() == 0
    o.stop_cm_translation()
    g.x, g.v = o.coords()
    g.rand_state = o.rand_state()
    desc = os.path.join(str(tmp_path), "basic_sph.desc")
    write_descriptor(g, desc)
    exe = build_program(str(tmp_path))
    want = [f"{golden['basic_sph'][c]:.2f}" for c in COLUMNS]
    xout = os.path.join(str(tmp_path), "x_shaken.bin")
    res = subprocess.run([exe, desc, xout, *want], capture_output=True, text=True, timeout=300)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "all checks passed" in res.stdout
    # the same displacement as the program's, then the oracle's SHAKE
    xx = np.asarray(g.x, dtype=np.float64).copy()
    k = np.arange(xx.size)
    x = xx + 0.004 * np.sin(0.37 * k + 1.0)
    assert o.shake(xx.copy(), x) >= 1
    xg = np.fromfile(xout, dtype=np.float64)
    assert np.abs(xg - x).max() < 1e-9
