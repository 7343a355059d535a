"""ctypes view of the C ABI in ``include/oxdna_gb300.h``.

The parameter structs mirror the reference plugin's ``param_type`` PODs field by
field; the ``*_from_dict`` converters mirror their pybind dict constructors (same
keys, tuple widths and defaults):

* ``src/EvaluatorPairOxDNAExcVol.h:54-63``        -> :func:`excvol_from_dict`
* ``src/EvaluatorPairOxDNAHBond.h:244-262``       -> :func:`hbond_from_dict`
* ``src/EvaluatorPairOxDNACrossStacking.h:367-385`` -> :func:`cross_from_dict`
* ``src/EvaluatorPairOxDNAHBondCross.h:69-101``   -> :func:`hbondcross_from_dict`
* ``src/EvaluatorPairOxDNACoaxStacking.h:68-97``  -> :func:`coax_from_dict`
* ``src/EvaluatorPairOxDNADebye.h:204-213``       -> :func:`debye_from_dict`
* ``src/OxDNABondedParams.h:97-127,183-220``      -> :func:`bonded_from_dict`

The native library is loaded from the package directory only. If it is missing the
import fails loudly: there is no CPU fallback for the force path.
"""

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "liboxdna_gb300.so")

OK = 0
ERR_INVALID_ARG = 1
ERR_CUDA = 2
ERR_NLIST_OVERFLOW = 3
ERR_BAD_INDEX = 4
ERR_TIMEOUT = 5
ERR_NO_PARAMS = 6
ERR_CAPACITY = 7
ERR_NONFINITE = 8

EXCVOL, HBOND, CROSS, HBONDCROSS, COAX, DEBYE = range(6)
N_PAIR_TERMS = 6
TERM_NAMES = ("oxdna_excvol", "oxdna_hbond", "oxdna_crossstacking", "oxdna_hbondcross",
              "oxdna_coaxstacking", "oxdna_debye")


def bit(t):
    return 1 << t


D3 = C.c_double * 3
D4 = C.c_double * 4
D5 = C.c_double * 5
D8 = C.c_double * 8
D9 = C.c_double * 9


class ExcVolParams(C.Structure):
    _fields_ = [("eps", C.c_double), ("base_site", D3), ("back_site", D3),
                ("sigma", D4), ("rstar", D4), ("b", D4), ("rc", D4)]


class HBondParams(C.Structure):
    _fields_ = [("eps", C.c_double), ("shift_factor", C.c_double), ("base_site", D3),
                ("f1", D8), ("t1", D5), ("t23", D5), ("t4", D5), ("t78", D5)]


class CrossParams(C.Structure):
    _fields_ = [("base_site", D3), ("f2", D9), ("t1", D5), ("t23", D5), ("t4", D5),
                ("t78", D5), ("t4_enabled", C.c_int32), ("pad_", C.c_int32)]


class HBondCrossParams(C.Structure):
    _fields_ = [("base_site", D3), ("eps", C.c_double), ("shift_factor", C.c_double),
                ("f1", D8), ("hb_t1", D5), ("hb_t23", D5), ("hb_t4", D5), ("hb_t78", D5),
                ("f2", D9), ("cs_t1", D5), ("cs_t23", D5), ("cs_t4", D5), ("cs_t78", D5)]


class CoaxParams(C.Structure):
    _fields_ = [("stack_site", D3), ("stack_back_ref", D3), ("gamma", C.c_double),
                ("f2", D9), ("t1", D5), ("t4", D5), ("t56", D5), ("phi3", D4), ("phi4", D4),
                ("t1_mode", C.c_int32), ("pad0_", C.c_int32), ("t1_sa", C.c_double),
                ("t1_sb", C.c_double), ("phi3_enabled", C.c_int32), ("rna_coax", C.c_int32)]


class DebyeParams(C.Structure):
    _fields_ = [("back_site", D3), ("minus_kappa", C.c_double), ("prefactor", C.c_double),
                ("b_smooth", C.c_double), ("rc", C.c_double), ("rhigh", C.c_double)]


class BondedParams(C.Structure):
    _fields_ = [("eps_backbone", C.c_double), ("r0_backbone", C.c_double),
                ("delta_backbone", C.c_double), ("delta2", C.c_double),
                ("back_site", D3), ("base_site", D3), ("excl_eps", C.c_double),
                ("bx_sigma", D3), ("bx_rstar", D3), ("bx_b", D3), ("bx_rc", D3),
                ("stacking_enabled", C.c_int32), ("rna_stacking", C.c_int32),
                ("stack_site", D3), ("stack_back_ref", D3), ("st_gamma", C.c_double),
                ("st_f1", D9), ("st_eps", (C.c_double * 4) * 4), ("t4", D5), ("t5", D5),
                ("p1", D4), ("stack_3_site", D3), ("stack_5_site", D3),
                ("bbvector_3", D3), ("bbvector_5", D3), ("tB1", D5), ("tB2", D5)]


PARAM_STRUCTS = {EXCVOL: ExcVolParams, HBOND: HBondParams, CROSS: CrossParams,
                 HBONDCROSS: HBondCrossParams, COAX: CoaxParams, DEBYE: DebyeParams}


def _set(arr, values, n, key):
    values = tuple(float(v) for v in values)
    if len(values) != n:
        raise ValueError(f"parameter {key!r} needs {n} values, got {len(values)}")
    for k, v in enumerate(values):
        arr[k] = v


def excvol_from_dict(d):
    p = ExcVolParams()
    p.eps = float(d["eps"])
    _set(p.base_site, d["base_site"], 3, "base_site")
    _set(p.back_site, d["back_site"], 3, "back_site")
    for k, key in enumerate(("back_back", "base_base", "base_back", "back_base")):
        t = tuple(d[key])
        if len(t) != 4:
            raise ValueError(f"parameter {key!r} needs 4 values")
        p.sigma[k], p.rstar[k], p.b[k], p.rc[k] = (float(x) for x in t)
    return p


def hbond_from_dict(d):
    p = HBondParams()
    p.eps = float(d["eps"])
    p.shift_factor = float(d["shift_factor"])
    _set(p.base_site, d["base_site"], 3, "base_site")
    _set(p.f1, d["f1"], 8, "f1")
    for f in ("t1", "t23", "t4", "t78"):
        _set(getattr(p, f), d["f4_" + f], 5, "f4_" + f)
    return p


def cross_from_dict(d):
    p = CrossParams()
    _set(p.base_site, d["base_site"], 3, "base_site")
    _set(p.f2, d["f2"], 9, "f2")
    for f in ("t1", "t23", "t4", "t78"):
        _set(getattr(p, f), d["f4_" + f], 5, "f4_" + f)
    p.t4_enabled = 1 if d.get("t4_enabled", True) else 0
    return p


def hbondcross_from_dict(d):
    p = HBondCrossParams()
    _set(p.base_site, d["base_site"], 3, "base_site")
    p.eps = float(d["eps"])
    p.shift_factor = float(d["shift_factor"])
    _set(p.f1, d["f1"], 8, "f1")
    for f in ("t1", "t23", "t4", "t78"):
        _set(getattr(p, "hb_" + f), d["hb_f4_" + f], 5, "hb_f4_" + f)
        _set(getattr(p, "cs_" + f), d["cs_f4_" + f], 5, "cs_f4_" + f)
    _set(p.f2, d["f2"], 9, "f2")
    return p


def coax_from_dict(d):
    p = CoaxParams()
    _set(p.stack_site, d["stack_site"], 3, "stack_site")
    _set(p.stack_back_ref, d["stack_back_ref"], 3, "stack_back_ref")
    p.gamma = float(d["gamma"])
    _set(p.f2, d["f2"], 9, "f2")
    _set(p.t1, d["f4_t1"], 5, "f4_t1")
    _set(p.t4, d["f4_t4"], 5, "f4_t4")
    _set(p.t56, d["f4_t56"], 5, "f4_t56")
    _set(p.phi3, d["f5_phi3"], 4, "f5_phi3")
    # reference: phi4 defaults to phi3 when absent (EvaluatorPairOxDNACoaxStacking.h:92-96)
    _set(p.phi4, d["f5_phi4"] if "f5_phi4" in d else d["f5_phi3"], 4, "f5_phi4")
    p.t1_mode = int(d["t1_mode"])
    p.t1_sa = float(d["t1_sa"])
    p.t1_sb = float(d["t1_sb"])
    p.phi3_enabled = 1 if d["phi3_enabled"] else 0
    p.rna_coax = 1 if d.get("rna_coax", False) else 0
    return p


def debye_from_dict(d):
    p = DebyeParams()
    _set(p.back_site, d["back_site"], 3, "back_site")
    t = tuple(float(x) for x in d["debye"])
    if len(t) != 5:
        raise ValueError("parameter 'debye' needs 5 values")
    p.minus_kappa, p.prefactor, p.b_smooth, p.rc, p.rhigh = t
    return p


def bonded_from_dict(d):
    """src/OxDNABondedParams.h:97-127 (stacking read only when stack_enabled)."""
    p = BondedParams()
    p.eps_backbone = float(d["epsilon"])
    p.r0_backbone = float(d["r0"])
    p.delta_backbone = float(d["delta"])
    p.delta2 = p.delta_backbone * p.delta_backbone
    _set(p.back_site, d["pos_back"], 3, "pos_back")
    _set(p.base_site, d["pos_base"], 3, "pos_base")
    p.excl_eps = float(d["excl_eps"])
    for k, key in enumerate(("bexc_base_base", "bexc_base_back", "bexc_back_base")):
        t = tuple(float(x) for x in d[key])
        if len(t) != 4:
            raise ValueError(f"parameter {key!r} needs 4 values")
        p.bx_sigma[k], p.bx_rstar[k], p.bx_b[k], p.bx_rc[k] = t
    p.stacking_enabled = 1 if d.get("stack_enabled", False) else 0
    if p.stacking_enabled:
        _set(p.stack_site, d["stack_site"], 3, "stack_site")
        _set(p.stack_back_ref, d["stack_back_ref"], 3, "stack_back_ref")
        p.st_gamma = float(d["stack_gamma"])
        _set(p.st_f1, d["stack_f1"], 9, "stack_f1")
        eps = tuple(float(x) for x in d["stack_eps"])
        if len(eps) != 16:
            raise ValueError("parameter 'stack_eps' needs 16 values")
        for i in range(4):
            for j in range(4):
                p.st_eps[i][j] = eps[4 * i + j]
        _set(p.t4, d["stack_f4_t4"], 5, "stack_f4_t4")
        _set(p.t5, d["stack_f4_t5"], 5, "stack_f4_t5")
        _set(p.p1, d["stack_f5_p1"], 4, "stack_f5_p1")
        p.rna_stacking = 1 if d.get("stack_rna", False) else 0
        if p.rna_stacking:
            _set(p.stack_3_site, d["stack_3_site"], 3, "stack_3_site")
            _set(p.stack_5_site, d["stack_5_site"], 3, "stack_5_site")
            _set(p.bbvector_3, d["stack_bbvector_3"], 3, "stack_bbvector_3")
            _set(p.bbvector_5, d["stack_bbvector_5"], 3, "stack_bbvector_5")
            _set(p.tB1, d["stack_f4_tB1"], 5, "stack_f4_tB1")
            _set(p.tB2, d["stack_f4_tB2"], 5, "stack_f4_tB2")
    return p


FROM_DICT = {EXCVOL: excvol_from_dict, HBOND: hbond_from_dict, CROSS: cross_from_dict,
             HBONDCROSS: hbondcross_from_dict, COAX: coax_from_dict, DEBYE: debye_from_dict}

# ------------------------------------------------------------------ library loading
EXPORTS = [
    "oxg_create", "oxg_destroy", "oxg_set_excvol_params", "oxg_set_hbond_params",
    "oxg_set_cross_params", "oxg_set_hbondcross_params", "oxg_set_coax_params",
    "oxg_set_debye_params", "oxg_set_bonded_params", "oxg_pair_forces", "oxg_bonded_forces",
    "oxg_context_status", "oxg_system_create", "oxg_system_destroy", "oxg_system_set_stream",
    "oxg_system_set_state", "oxg_system_get_state", "oxg_system_device_state",
    "oxg_system_set_nlist_buffer", "oxg_system_compute", "oxg_system_set_integrator",
    "oxg_system_run", "oxg_system_energies", "oxg_system_stats", "oxg_last_error",
    "oxg_version", "oxg_status_string", "oxg_pair_forces_noalloc",
    "oxg_batch_create", "oxg_batch_destroy", "oxg_batch_set_stream", "oxg_batch_set_state",
    "oxg_batch_get_state", "oxg_batch_set_integrator", "oxg_batch_set_tiling", "oxg_batch_tune",
    "oxg_batch_run", "oxg_batch_compute",
    "oxg_mlp_create", "oxg_mlp_destroy", "oxg_mlp_set_params", "oxg_mlp_get_params",
    "oxg_mlp_set_normalization", "oxg_mlp_gradient", "oxg_mlp_train_step", "oxg_mlp_predict",
    "oxg_system_set_surrogate", "oxg_system_surrogate_stats", "oxg_system_hbx_samples",
    "oxg_system_run_timing", "oxg_device_peaks", "oxg_system_run_host", "oxg_selftest_barrier",
    "oxg_system_set_timestep", "oxg_system_set_host_session",
]

MLP_PARAMS = 9480  # OXG_MLP_PARAMS
SURROGATE_RUN = 1
SURROGATE_COMPUTE = 2

_lib = None

vp = C.c_void_p
i32 = C.c_int32
u32 = C.c_uint32
f64 = C.c_double
fp = C.POINTER(C.c_float)
dp = C.POINTER(C.c_double)


class OxgError(RuntimeError):
    def __init__(self, code, where, text):
        super().__init__(f"{where} failed with status {code}: {text}")
        self.code = code


def lib():
    """The loaded native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"native library {LIB_PATH} is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    sig = {
        "oxg_create": ([C.POINTER(vp), i32, i32], i32),
        "oxg_destroy": ([vp], i32),
        "oxg_set_excvol_params": ([vp, i32, i32, C.POINTER(ExcVolParams), f64], i32),
        "oxg_set_hbond_params": ([vp, i32, i32, C.POINTER(HBondParams), f64], i32),
        "oxg_set_cross_params": ([vp, i32, i32, C.POINTER(CrossParams), f64], i32),
        "oxg_set_hbondcross_params": ([vp, i32, i32, C.POINTER(HBondCrossParams), f64], i32),
        "oxg_set_coax_params": ([vp, i32, i32, C.POINTER(CoaxParams), f64], i32),
        "oxg_set_debye_params": ([vp, i32, i32, C.POINTER(DebyeParams), f64], i32),
        "oxg_set_bonded_params": ([vp, i32, C.POINTER(BondedParams)], i32),
        "oxg_pair_forces": ([vp, u32, i32, vp, vp, vp, fp, vp, vp, vp, vp, vp, vp, vp, vp], i32),
        "oxg_bonded_forces": ([vp, i32, vp, vp, fp, i32, vp, vp, vp, vp, vp, vp], i32),
        "oxg_context_status": ([vp, i32], i32),
        "oxg_system_create": ([C.POINTER(vp), vp, i32, fp, i32, C.POINTER(C.c_int32)], i32),
        "oxg_system_destroy": ([vp], i32),
        "oxg_system_set_stream": ([vp, vp], i32),
        "oxg_system_set_state": ([vp, vp, vp, vp, vp, vp, vp], i32),
        "oxg_system_get_state": ([vp, vp, vp, vp, vp, vp], i32),
        "oxg_system_device_state": ([vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp),
                                     C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)], i32),
        "oxg_system_set_nlist_buffer": ([vp, f64], i32),
        "oxg_system_set_timestep": ([vp, C.c_uint64], i32),
        "oxg_system_compute": ([vp, u32, i32, vp, vp, vp, vp], i32),
        "oxg_system_set_integrator": ([vp, f64, f64, f64, f64, C.c_uint64, u32, i32], i32),
        "oxg_system_run": ([vp, C.c_long], i32),
        "oxg_system_energies": ([vp, vp, vp], i32),
        "oxg_system_stats": ([vp, C.POINTER(C.c_int64), i32], i32),
        "oxg_pair_forces_noalloc": ([vp, u32, i32, vp, vp, vp, fp, i32, vp, vp, vp, vp, vp], i32),
        "oxg_batch_create": ([C.POINTER(vp), i32, C.POINTER(vp), C.POINTER(C.c_int32), fp,
                              C.POINTER(C.c_int32), C.POINTER(C.c_int32)], i32),
        "oxg_batch_destroy": ([vp], i32),
        "oxg_batch_set_stream": ([vp, vp], i32),
        "oxg_batch_set_state": ([vp, vp, vp, vp, vp, vp, vp], i32),
        "oxg_batch_get_state": ([vp, vp, vp, vp, vp, vp], i32),
        "oxg_batch_set_integrator": ([vp, f64, dp, f64, f64, C.c_uint64, u32, i32], i32),
        "oxg_batch_set_tiling": ([vp, i32, i32], i32),
        "oxg_batch_tune": ([vp, i32, C.POINTER(C.c_int), C.POINTER(C.c_int), dp], i32),
        "oxg_batch_run": ([vp, C.c_long], i32),
        "oxg_batch_compute": ([vp, u32, i32, vp, vp, vp], i32),
        "oxg_mlp_create": ([C.POINTER(vp)], i32),
        "oxg_mlp_destroy": ([vp], i32),
        "oxg_mlp_set_params": ([vp, vp], i32),
        "oxg_mlp_get_params": ([vp, vp], i32),
        "oxg_mlp_set_normalization": ([vp, i32, vp, vp, C.c_float, C.c_float], i32),
        "oxg_mlp_gradient": ([vp, i32, vp, vp, vp, i32, vp, vp, vp], i32),
        "oxg_mlp_train_step": ([vp, i32, vp, vp, vp, i32, C.c_float, vp, vp], i32),
        "oxg_mlp_predict": ([vp, i32, vp, i32, vp, vp, vp], i32),
        "oxg_system_set_surrogate": ([vp, vp, i32, i32, i32, f64], i32),
        "oxg_system_surrogate_stats": ([vp, dp, i32], i32),
        "oxg_system_hbx_samples": ([vp, i32, vp, vp, C.POINTER(C.c_int)], i32),
        "oxg_system_run_timing": ([vp, dp, i32, i32], i32),
        "oxg_device_peaks": ([dp, i32, vp], i32),
        "oxg_selftest_barrier": ([i32, i32, C.POINTER(C.c_int), vp], i32),
        "oxg_system_run_host": ([vp, C.c_long, vp, vp, vp, vp, vp], i32),
        "oxg_system_set_host_session": ([vp, C.c_int], i32),
        "oxg_last_error": ([], C.c_char_p),
        "oxg_version": ([], C.c_char_p),
        "oxg_status_string": ([i32], C.c_char_p),
    }
    for name, (argt, rest) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = argt
        fn.restype = rest
    _lib = L
    return L


def check(code, where):
    if code != OK:
        L = lib()
        text = (L.oxg_status_string(code) or b"").decode()
        detail = (L.oxg_last_error() or b"").decode()
        raise OxgError(code, where, f"{text}: {detail}")
