"""ctypes mirror of include/qgpu.h and the loader of the engine library.

The engine's product path is ``libqgpu.so`` (CUDA, sm_103a).  It is loaded
from the package's ``_build`` directory; importing a compute entry point
without it raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

MAX_STATES = 10

QGPU_TERMS_NONBOND = 0x1
QGPU_TERMS_QQ = 0x2
QGPU_TERMS_QBONDED = 0x4
QGPU_TERMS_BONDED = 0x8
QGPU_TERMS_RESTRAINT = 0x10
QGPU_TERMS_ALL = 0x1F
QGPU_TERMS_STEP_PRECISION = 0x100
QGPU_PRECISION_MIXED = 0
QGPU_PRECISION_FP64 = 1
QGPU_PRECISION_FP64_UNFUSED = 2
# step precision by name (bench and tests)
PRECISION = {"mixed": QGPU_PRECISION_MIXED, "fp64": QGPU_PRECISION_FP64, "fp64_unfused": QGPU_PRECISION_FP64_UNFUSED}

STATUS = {0: "ok", 1: "invalid", 2: "cuda", 3: "list overflow", 4: "shake failure", 5: "nan",
          6: "unsupported", 7: "fixed-point range"}

_P = C.c_void_p
_i32 = C.c_int32
_f64 = C.c_double


class SystemDesc(C.Structure):
    """qgpu_system_desc (include/qgpu.h)."""

    _fields_ = [
        ("natom", _i32), ("nat_solute", _i32), ("solv_atom", _i32), ("nwat", _i32), ("natyps", _i32),
        ("ncgp", _i32), ("ncgp_solute", _i32), ("nqat", _i32), ("nstates", _i32),
        ("x", _P), ("v", _P), ("xtop", _P),
        ("crg", _P), ("iac", _P), ("excl", _P), ("shell", _P), ("iqatom", _P),
        ("mass", _P), ("avdw", _P), ("bvdw", _P), ("ljcod", _P),
        ("el14_scale", _f64), ("ivdw_rule", _i32), ("ff_type", _i32),
        ("chg_solv", _f64 * 3), ("aLJ_solv", _f64 * 6), ("bLJ_solv", _f64 * 6),
        ("cgp_first", _P), ("cgp_last", _P), ("cgp_switch", _P), ("cgpatom", _P),
        ("nexcl", _i32), ("excl_pairs", _P), ("n14", _i32), ("pairs14", _P),
        ("iqseq", _P), ("qcrg", _P), ("qvdw_flag", _i32), ("qiac", _P), ("nqlib", _i32),
        ("qavdw", _P), ("qbvdw", _P), ("sc_lookup", _P), ("lambda_", _f64 * MAX_STATES),
        ("qp_skip", _P), ("nqp14", _i32), ("qp14_pairs", _P),
        ("nbqq_count", _i32 * MAX_STATES), ("nbqq_iq", _P), ("nbqq_j", _P), ("nbqq_jq", _P),
        ("nbqq_ljcod", _P), ("nbqq_elscale", _P),
        ("nqbond", _i32), ("qbnd", _P), ("nqbcod", _i32), ("qbondlib", _P),
        ("nqangle", _i32), ("qang", _P), ("nqacod", _i32), ("qanglib", _P),
        ("nqtor", _i32), ("qtor", _P), ("nqtcod", _i32), ("qtorlib", _P),
        ("nqimp", _i32), ("qimp", _P), ("nqicod", _i32), ("qimplib", _P),
        ("nbonds", _i32), ("nbonds_solute", _i32), ("bnd", _P), ("nbndcod", _i32), ("bondlib", _P),
        ("nangles", _i32), ("nangles_solute", _i32), ("ang", _P), ("nangcod", _i32), ("anglib", _P),
        ("ntors", _i32), ("ntors_solute", _i32), ("tor", _P), ("ntorcod", _i32), ("torlib", _P),
        ("nimps", _i32), ("nimps_solute", _i32), ("imp", _P), ("nimpcod", _i32), ("implib", _P),
        ("shake_molecules", _i32), ("shake_first", _P), ("shake_i", _P), ("shake_j", _P), ("shake_dist2", _P),
        ("noffd", _i32), ("offd_ij", _P), ("offd_kl", _P), ("offd_Amu", _P),
        ("xpcent", _f64 * 3), ("xwcent", _f64 * 3), ("rexcl_o", _f64), ("rwat", _f64),
        ("fk_wsphere", _f64), ("Dwmz", _f64), ("awmz", _f64), ("fk_pshell", _f64), ("fk_fix", _f64),
        ("wpol_restr", _i32),
        ("Rcpp", _f64), ("Rcww", _f64), ("Rcpw", _f64), ("Rcq", _f64), ("RcLRF", _f64), ("use_LRF", _i32),
        ("dt", _f64), ("Temp0", _f64), ("tau_T", _f64), ("separate_scaling", _i32), ("NBcycle", _i32),
        ("Ndegf", _i32), ("Ndegfree", _i32), ("Ndegf_solvent", _i32), ("Ndegfree_solvent", _i32),
        ("Ndegf_solute", _i32), ("Ndegfree_solute", _i32), ("detail_temps", _i32),
        ("any_atom_lists", _i32),
        ("nrstr_seq", _i32), ("rstseq_ij", _P), ("rstseq_fk", _P), ("rstseq_flags", _P), ("heavy", _P),
        ("excluded_freeze", _i32),
        ("fkwpol", _f64), ("nwpolr_shell", _i32), ("wshell_rout", _P), ("wshell_dr", _P), ("wshell_cstb", _P),
        ("wshell_theta_corr", _P), ("itdis_update", _i32),
        ("thermostat", _i32), ("integrator", _i32), ("friction", _f64), ("langevin_gauss", _i32),
        ("rand_state", _i32), ("nhchains", _i32), ("nhq", _f64),
        ("use_pbc", _i32), ("boxlength", _f64 * 3), ("boxcentre", _f64 * 3), ("qswitch", _i32),
        ("put_solute_back", _i32), ("put_solvent_back", _i32), ("rigid_box_centre", _i32),
        ("nmol", _i32), ("istart_mol", _P), ("nsolute_mol", _i32),
        ("nrstr_pos", _i32), ("rstpos_i", _P), ("rstpos_x", _P),
        ("nrstr_dist", _i32), ("rstdis_i", _P), ("rstdis_p", _P),
        ("nrstr_angl", _i32), ("rstang_i", _P), ("rstang_p", _P),
        ("nrstr_wall", _i32), ("rstwal_i", _P), ("rstwal_p", _P),
    ]


ENERGY_FIELDS = ["potential", "kinetic", "lrf", "p_bond", "p_angle", "p_torsion", "p_improper",
                 "w_bond", "w_angle", "w_torsion", "w_improper", "q_bond", "q_angle", "q_torsion", "q_improper",
                 "pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw", "qx_el", "qx_vdw",
                 "rst_total", "rst_fix", "rst_shell", "rst_protein", "rst_solvent_radial", "rst_water_pol"]
QENERGY_FIELDS = ["lambda_", "q_bond", "q_angle", "q_torsion", "q_improper", "qq_el", "qq_vdw", "qp_el",
                  "qp_vdw", "qw_el", "qw_vdw", "qx_el", "qx_vdw", "restraint", "total"]


class Energies(C.Structure):
    _fields_ = [(n, _f64) for n in ENERGY_FIELDS]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n in ENERGY_FIELDS}


class QEnergy(C.Structure):
    _fields_ = [(n, _f64) for n in QENERGY_FIELDS]

    def as_dict(self) -> dict:
        d = {n: getattr(self, n) for n in QENERGY_FIELDS}
        d["lambda"] = d.pop("lambda_")
        return d


MAX_STATES = 10
QFEP_MAXCOUP = 45
QFEP_P2 = 5 + MAX_STATES
QFEP_P3 = 7


class QfepParams(C.Structure):
    """qgpu_qfep_params: qfep's input in the order it reads it."""
    _fields_ = [("nstates", _i32), ("noffd", _i32), ("kT", _f64), ("nskip", _i32), ("gas", _i32), ("nbins", _i32),
                ("nmin", _i32), ("alpha", _f64 * MAX_STATES), ("scale_hij", _f64), ("ncoup", _i32),
                ("coup_ij", _i32 * (2 * QFEP_MAXCOUP)), ("coup_A", _f64 * QFEP_MAXCOUP),
                ("coup_mu", _f64 * QFEP_MAXCOUP), ("coup_eta", _f64 * QFEP_MAXCOUP),
                ("coup_rxy0", _f64 * QFEP_MAXCOUP), ("coeff", _f64 * MAX_STATES)]


ENE_SINK = C.CFUNCTYPE(None, C.c_void_p, _i32, _i32, C.POINTER(QEnergy), _i32, C.POINTER(Energies))

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libqgpu.so")

# Every exported entry point of include/qgpu.h, with its ctypes signature.
EXPORTS = {
    "qgpu_create": (_i32, [C.POINTER(SystemDesc), _i32, C.POINTER(C.c_void_p)]),
    "qgpu_destroy": (_i32, [C.c_void_p]),
    "qgpu_last_error": (_i32, [C.c_char_p, _i32]),
    "qgpu_ntraj": (_i32, [C.c_void_p]),
    "qgpu_get_q_lists": (_i32, [C.c_void_p, _i32, _P, C.c_int64, _P, _P, C.c_int64, _P]),
    "qgpu_set_coords": (_i32, [C.c_void_p, _i32, _P, _P]),
    "qgpu_get_coords": (_i32, [C.c_void_p, _i32, _P, _P]),
    "qgpu_set_coords_all": (_i32, [C.c_void_p, _P, _P]),
    "qgpu_get_coords_all": (_i32, [C.c_void_p, _P, _P]),
    "qgpu_build_lists": (_i32, [C.c_void_p]),
    "qgpu_forces": (_i32, [C.c_void_p, _i32, _i32, _P, C.POINTER(Energies), C.POINTER(QEnergy)]),
    "qgpu_shake": (_i32, [C.c_void_p, _i32, _P, _P, C.POINTER(_i32)]),
    "qgpu_run": (_i32, [C.c_void_p, _i32, _i32, ENE_SINK, C.c_void_p]),
    "qgpu_enqueue": (_i32, [C.c_void_p, _i32, _i32]),
    "qgpu_set_precision": (_i32, [C.c_void_p, _i32]),
    "qgpu_set_step": (_i32, [C.c_void_p, C.c_int64]),
    "qgpu_autotune": (_i32, [C.c_void_p, _P]),
    "qgpu_mlp_nparams": (_i32, []),
    "qgpu_mlp_predict": (_i32, [_P, _P, _i32, _P]),
    "qgpu_mlp_train": (_i32, [_P, _P, _P, _P, _P, _i32, _i32, C.c_float, _i32, _P, _P]),
    "qgpu_set_tuning": (_i32, [C.c_void_p, _P]),
    "qgpu_run_rows": (_i32, [C.c_void_p, _i32, _i32, _P, _P, _P, _P, _i32, _P]),
    "qgpu_calc_rms": (_i32, [_P, _i32, _i32, _P, _i32, _P, _P]),
    "qgpu_calc_com": (_i32, [_P, _i32, _i32, _P, _i32, _P, _P]),
    "qgpu_calc_com_ke": (_i32, [_P, _i32, _i32, _P, _i32, _P, _f64, _P]),
    "qgpu_calc_rmsf": (_i32, [_P, _i32, _i32, _P, _i32, _P]),
    "qgpu_calc_fit": (_i32, [_P, _i32, _i32, _i32, _P, _i32, _P, _P, _P, _P]),
    "qgpu_calc_geom": (_i32, [_P, _i32, _i32, _i32, _P, _P, _P]),
    "qgpu_calc_rdf": (_i32, [_P, _i32, _i32, _P, _i32, _P, _i32, _f64, _i32, _P, _P]),
    "qgpu_calc_nb": (_i32, [_P, _i32, _i32, _i32, _P, _P, _i32, _P, _P, _P, _P, _i32, _P]),
    "qgpu_ene_open": (_i32, [C.c_void_p, _i32, C.c_char_p]),
    "qgpu_ene_close": (_i32, [C.c_void_p, _i32]),
    "qgpu_enefile_write": (_i32, [C.c_char_p, _i32, _i32, C.POINTER(QEnergy), _i32, _P, _P]),
    "qgpu_qfep_evb": (_i32, [_i32, C.POINTER(C.c_char_p), C.POINTER(QfepParams), _P, _P, _P, _P, _P]),
    "qgpu_fep_start": (_i32, [C.c_void_p, _i32, _P, _f64, _i32]),
    "qgpu_fep_result": (_i32, [C.c_void_p, _P, _P, _P, _P]),
    "qgpu_sync": (_i32, [C.c_void_p]),
    "qgpu_get_group_pairs": (_i32, [C.c_void_p, _i32, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "qgpu_get_lrf": (_i32, [C.c_void_p, _i32, _P]),
    "qgpu_get_temperature": (_i32, [C.c_void_p, _i32, _P]),
    "qgpu_kernel_launches": (C.c_int64, [C.c_void_p]),
    "qgpu_stream": (C.c_void_p, [C.c_void_p]),
    "qgpu_profile": (_i32, [C.c_void_p, _i32, C.c_char_p, _P, _P, _i32, C.POINTER(_i32)]),
    "qgpu_fp32_peak": (_i32, [C.POINTER(_f64)]),
    "qgpu_fp64_peak": (_i32, [C.POINTER(_f64)]),
    "qgpu_set_branches": (_i32, [C.c_void_p, _i32]),
    "qgpu_get_branches": (_i32, [C.c_void_p]),
    "qgpu_shake_counts": (_i32, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "qgpu_lrf_scan_static": (_i32, [_i32, _P, _P, _P, _P, _P, _P, C.POINTER(_f64), _f64, _f64, _f64, _f64,
                                    _P, _P, _P]),
}

_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load libqgpu.so (built by qsource_gb300.build); raises when missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"qgpu engine library not built: {p} (run qsource_gb300.build.build())")
    lib = C.CDLL(p)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def last_error(lib) -> str:
    buf = C.create_string_buffer(1024)
    lib.qgpu_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)
