"""The C-ABI boundary: the library builds for sm_103a, loads, exports every
entry point declared in include/qgpu.h, and its structs match the ctypes mirror."""
import ctypes as C
import os
import re

from conftest import ROOT


def declared_entry_points():
    with open(os.path.join(ROOT, "include", "qgpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^(?:int|int64_t|void\s*\*)\s*(qgpu_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_entry_point(engine_lib):
    names = declared_entry_points()
    assert len(names) >= 14
    for n in names:
        assert hasattr(engine_lib, n), n


def test_python_mirror_covers_every_entry_point():
    from qsource_gb300.abi import EXPORTS
    assert set(declared_entry_points()) == set(EXPORTS)


def test_struct_layout_matches_c():
    from oracle.oracle import lib
    from qsource_gb300.abi import Energies, QEnergy, SystemDesc
    L = lib()
    L.oracle_sizeof_energies.restype = C.c_int
    L.oracle_sizeof_qenergy.restype = C.c_int
    assert L.oracle_sizeof_desc() == C.sizeof(SystemDesc)
    assert L.oracle_sizeof_energies() == C.sizeof(Energies)
    assert L.oracle_sizeof_qenergy() == C.sizeof(QEnergy)


def test_error_reporting_without_device(engine_lib):
    """qgpu_create refuses a null descriptor with a message, no device needed."""
    from qsource_gb300.abi import last_error
    h = C.c_void_p()
    rc = engine_lib.qgpu_create(None, 1, C.byref(h))
    assert rc != 0
    assert "bad arguments" in last_error(engine_lib)
