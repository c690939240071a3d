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


def test_calc_entries_refuse_bad_arguments_without_device(engine_lib):
    """The qcalc entry points check their arguments on the host before any
    device call: a decreasing list offset, a pair atom out of range, a
    non-positive frame interval and an empty mask are refused with a message."""
    import numpy as np
    from qsource_gb300 import abi
    from qsource_gb300.abi import last_error
    fr = np.zeros((1, 3 * 4))
    lam = np.ones(1)
    A = np.ones(2)
    out = np.zeros(8)
    pairs = np.array([0, 1, 2, 3], dtype=np.int32)
    p = abi.ptr
    rc = engine_lib.qgpu_calc_nb(p(fr), 1, 4, 2, p(np.array([0, 2, 1], dtype=np.int64)), p(pairs), 1, p(lam),
                                 p(A), p(A), p(A), 0, p(out))
    assert rc != 0 and "decreases" in last_error(engine_lib)
    bad = np.array([0, 1, 2, 9], dtype=np.int32)
    rc = engine_lib.qgpu_calc_nb(p(fr), 1, 4, 1, p(np.array([0, 2], dtype=np.int64)), p(bad), 1, p(lam),
                                 p(A), p(A), p(A), 0, p(out))
    assert rc != 0 and "out of range" in last_error(engine_lib)
    mask = np.array([0, 1], dtype=np.int32)
    mass = np.ones(4)
    rc = engine_lib.qgpu_calc_com_ke(p(fr), 1, 4, p(mask), 2, p(mass), C.c_double(0.0), p(out))
    assert rc != 0 and "bad arguments" in last_error(engine_lib)
    rc = engine_lib.qgpu_calc_rmsf(p(fr), 1, 4, p(mask), 0, p(out))
    assert rc != 0 and "bad arguments" in last_error(engine_lib)


def test_create_refuses_malformed_descriptors_without_device(engine_lib):
    """qgpu_create checks every index the device would follow before any
    device call: a negative solute bond count, a bond or SHAKE atom outside
    the system, a parameter code outside its library, a charge group outside
    the atoms and a Q atom outside the solute are refused with a message (a
    well-formed descriptor gets as far as the device check)."""
    import numpy as np
    from qsource_gb300 import abi, synth
    from qsource_gb300.abi import last_error

    def create(g):
        arr = (abi.SystemDesc * 1)(g.desc())
        h = C.c_void_p()
        return engine_lib.qgpu_create(arr, 1, C.byref(h)), last_error(engine_lib)

    def fresh():
        qa = synth.neutral_charges(np.random.default_rng(1), 4, 0.4)
        return synth.synthetic(8.0, 12, 4, np.stack([qa, -qa], 1), (0.5, 0.5), 3)

    g = fresh()
    rc, msg = create(g)
    assert "out of range" not in msg and "bonded" not in msg
    cases = []
    g = fresh(); g.nbonds_solute = -1; cases.append((g, "solute bonded counts"))
    g = fresh(); g.bnd = np.array(g.bnd).copy(); g.bnd[0, 1] = g.natom + 7; cases.append((g, "bonded terms"))
    g = fresh(); g.bnd = np.array(g.bnd).copy(); g.bnd[0, 2] = len(g.bondlib) + 1; cases.append((g, "bonded terms"))
    g = fresh(); g.shake_j = np.array(g.shake_j).copy(); g.shake_j[0] = -2; cases.append((g, "SHAKE constraint"))
    g = fresh(); g.cgp_last = np.array(g.cgp_last).copy(); g.cgp_last[-1] = g.natom; cases.append((g, "charge group"))
    g = fresh(); g.iqseq = np.array(g.iqseq).copy(); g.iqseq[0] = g.nat_solute; cases.append((g, "Q atom"))
    for g, want in cases:
        rc, msg = create(g)
        assert rc == 1 and want in msg, (want, rc, msg)        # QGPU_E_INVALID
    # a water count that disagrees with the solvent atoms
    d = fresh().desc()
    d.nwat += 1
    h = C.c_void_p()
    rc = engine_lib.qgpu_create((abi.SystemDesc * 1)(d), 1, C.byref(h))
    assert rc == 1 and "nwat" in last_error(engine_lib)
