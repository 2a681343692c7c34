"""ctypes binding of libmsl.so (include/msl.h).

The library is built in-tree by multislice_gb300/build.py.  Loading fails loudly
when it is missing: there is no CPU fallback anywhere in this package.
"""
import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_int64, c_size_t, c_void_p

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libmsl.so")

MSL_OK = 0
MSL_E_ARG = -1
MSL_E_CUDA = -2
MSL_E_NOMEM = -3
MSL_E_UNSUPPORTED = -4
MAX_DETECTORS = 8

# every symbol include/msl.h declares
EXPORTS = (
    "msl_ctx_create", "msl_ctx_destroy", "msl_last_error", "msl_version", "msl_kernel_launches",
    "msl_fparams_parse", "msl_wavelength", "msl_sigma", "msl_potential_build",
    "msl_transmission_build", "msl_fft2d", "msl_multislice", "msl_stem_scan",
    "msl_set_probe_batch", "msl_profile_enable", "msl_profile_read", "msl_multislice_noalloc",
    "msl_ctem_image", "msl_phonon_displacements", "msl_frozen_phonon", "msl_coo_parse",
    "msl_run_jobs", "msl_ctem_partial_coherence", "msl_check_wait_timeout", "msl_set_memory_limit",
    "msl_memory_in_use", "msl_stem_scan_phonon", "msl_tc_gemm_bf16", "msl_closure_create",
    "msl_closure_destroy", "msl_closure_param_count", "msl_closure_get_params", "msl_closure_set_params",
    "msl_closure_apply", "msl_closure_gradients", "msl_closure_train_step", "msl_stem_exit_waves",
    "msl_stem_scan_closure", "msl_autotune", "msl_set_schedule", "msl_get_schedule", "msl_set_autotune",
    "msl_stem_scan_resident", "msl_amorphous",
)
PLANE_WAVE, PROBE = 0, 1
# Muslib-shaped exports (reference names, no msl_ prefix)
_RS_FORMS = [(kind, src, coord, wrap) for kind in ("PG", "Potential") for src in ("curve", "DT")
             for coord in ("DW", "TV") for wrap in ("cutpot", "periodic")]
MUSLIB_RS = tuple(f"{k}_rs_{s}_{c}_{w}" for k, s, c, w in _RS_FORMS)
MUSLIB_EXPORTS = ("CreatePropagator", "ApplyPropagator", *MUSLIB_RS, "PG_rs_curve_DW_cutpot_oneatom",
                  "Potential_rec_DT_DW", "Potential_rec_curve_DW", "scat_ampl_rs_DT_DW",
                  "scat_ampl_rs2_DT_DW", "scat_ampl_rs2_DT_DW0", "CreatePots_rec_DT_DW",
                  "CreatePots_rs_DT_DW")
PROF_ROW, PROF_COL, PROF_POTENTIAL, PROF_OTHER = 0, 1, 2, 3


class Grid(ctypes.Structure):
    _fields_ = [("nx", c_int), ("ny", c_int), ("ax", c_double), ("by", c_double)]


class Atoms(ctypes.Structure):
    _fields_ = [("natom", c_int), ("x", c_void_p), ("y", c_void_p), ("z", c_void_p),
                ("Z", c_void_p), ("cz", c_double)]


class Optics(ctypes.Structure):
    _fields_ = [("kev", c_double), ("bandlimit", c_double), ("tilt_x", c_double),
                ("tilt_y", c_double), ("f32_prop_args", c_int)]


class Probe(ctypes.Structure):
    _fields_ = [("k_in", c_double), ("k_out", c_double), ("df", c_double), ("cs", c_double)]


class Detectors(ctypes.Structure):
    _fields_ = [("ndet", c_int), ("k_in", c_void_p), ("k_out", c_void_p)]


class Cell(ctypes.Structure):
    _fields_ = [("a", c_double), ("b", c_double), ("c", c_double), ("alpha", c_double),
                ("beta", c_double), ("gamma", c_double), ("natom", c_int)]


class Lens(ctypes.Structure):
    _fields_ = [("cs", c_double), ("df", c_double), ("k_obj", c_double), ("df_spread", c_double),
                ("df_step", c_double), ("dfa2", c_double), ("dfa2phi", c_double),
                ("dfa3", c_double), ("dfa3phi", c_double)]


class Job(ctypes.Structure):
    _fields_ = [("grid", Grid), ("kev", c_double), ("trans", c_void_p), ("ntrans", c_int),
                ("dz", c_void_p), ("layer_seq", c_void_p), ("nslice", c_int),
                ("illumination", c_int), ("probe", Probe), ("probe_x", c_double),
                ("probe_y", c_double), ("exit_wave", c_void_p)]


class MslError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"msl error {code}: {msg}")
        self.code = code


_lib = None


def load(path=LIB_PATH):
    """Load libmsl.so and declare every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libmsl.so not built ({path}); run multislice_gb300/build.py")
    lib = ctypes.CDLL(path)
    P = c_void_p
    sig = {
        "msl_ctx_create": (c_int, [c_int, POINTER(c_void_p)]),
        "msl_ctx_destroy": (c_int, [P]),
        "msl_last_error": (c_char_p, [P]),
        "msl_version": (c_char_p, []),
        "msl_kernel_launches": (c_int64, [P]),
        "msl_fparams_parse": (c_int, [c_char_p, c_size_t, P]),
        "msl_wavelength": (c_double, [c_double]),
        "msl_sigma": (c_double, [c_double]),
        "msl_potential_build": (c_int, [P, POINTER(Atoms), P, POINTER(Grid), c_int, c_double, P]),
        "msl_transmission_build": (c_int, [P, POINTER(Grid), POINTER(Optics), P, c_int, P]),
        "msl_fft2d": (c_int, [P, POINTER(Grid), P, c_int, c_int]),
        "msl_multislice": (c_int, [P, POINTER(Grid), POINTER(Optics), P, c_int, P, P, c_int, P,
                                   c_int, c_int]),
        "msl_stem_scan": (c_int, [P, POINTER(Grid), POINTER(Optics), P, c_int, P, P, c_int,
                                  POINTER(Probe), P, c_int, POINTER(Detectors), P, c_int, P]),
        "msl_set_probe_batch": (c_int, [P, c_int]),
        "msl_set_memory_limit": (c_int, [P, c_size_t]),
        "msl_memory_in_use": (c_int, [P, POINTER(c_size_t)]),
        "msl_profile_enable": (c_int, [P, c_int]),
        "msl_profile_read": (c_int, [P, c_int, POINTER(c_int64), POINTER(c_double)]),
        "msl_multislice_noalloc": (c_int, [POINTER(Grid), POINTER(Optics), P, c_int, P, P, c_int,
                                           P, c_int, c_int, P]),
        "msl_ctem_image": (c_int, [P, POINTER(Grid), POINTER(Optics), P, c_int, P, P, c_int,
                                   POINTER(Lens), P, c_int, c_int, c_double, P, P]),
        "msl_phonon_displacements": (c_int, [ctypes.c_uint64, c_int, c_int, c_double, P]),
        "msl_coo_parse": (c_int, [c_char_p, c_size_t, POINTER(Cell), P, c_int]),
        "msl_run_jobs": (c_int, [P, P, c_int, c_double]),
        "msl_check_wait_timeout": (c_int, [P, ctypes.c_uint32]),
        "msl_ctem_partial_coherence": (c_int, [P, POINTER(Grid), POINTER(Optics), P, c_int, P, P, c_int,
                                               POINTER(Lens), c_double, c_double, P, P]),
        "CreatePropagator": (c_int, [c_double] * 7 + [ctypes.c_uint32, ctypes.c_uint32, P, P]),
        "ApplyPropagator": (c_int, [c_double] * 7 + [ctypes.c_uint32, ctypes.c_uint32, P, P]),
        "msl_frozen_phonon": (c_int, [P, POINTER(Atoms), P, POINTER(Grid), c_int, c_double,
                                      POINTER(Optics), POINTER(Lens), c_int, c_double,
                                      ctypes.c_uint64, P, P]),
        "msl_tc_gemm_bf16": (c_int, [P, P, P, P, c_int, c_int, c_int]),
        "msl_closure_create": (c_int, [P, ctypes.c_uint64, P]),
        "msl_autotune": (c_int, [P, c_int, c_int, c_int, P, P, P]),
        "msl_amorphous": (c_int, [ctypes.c_uint64, c_double, c_double, c_double, c_double, c_double, c_int, P, P,
                                  c_int, P, P, P]),
        "msl_stem_scan_resident": (c_int, [P, POINTER(Grid), POINTER(Optics), P, c_int, P, P, c_int,
                                           POINTER(Probe), P, c_int, POINTER(Detectors), P, c_int, P]),
        "msl_set_schedule": (c_int, [P, c_int, c_int, c_int]),
        "msl_get_schedule": (c_int, [P, c_int, P, P]),
        "msl_set_autotune": (c_int, [P, c_int]),
        "msl_stem_exit_waves": (c_int, [P, POINTER(Grid), POINTER(Optics), P, c_int, P, P, c_int,
                                        POINTER(Probe), P, c_int, P]),
        "msl_stem_scan_closure": (c_int, [P, P, POINTER(Grid), POINTER(Optics), P, c_int, P, P, c_int,
                                          POINTER(Probe), P, c_int, POINTER(Detectors), P]),
        "msl_closure_destroy": (c_int, [P]),
        "msl_closure_param_count": (c_int, []),
        "msl_closure_get_params": (c_int, [P, P, P]),
        "msl_closure_set_params": (c_int, [P, P, P]),
        "msl_closure_apply": (c_int, [P, P, P, c_int, c_int, c_int]),
        "msl_closure_gradients": (c_int, [P, P, P, P, c_int, c_int, c_int, P, P]),
        "msl_closure_train_step": (c_int, [P, P, P, P, c_int, c_int, c_int, ctypes.c_float, P]),
        "msl_stem_scan_phonon": (c_int, [P, POINTER(Atoms), P, POINTER(Grid), c_int, c_double,
                                         POINTER(Optics), POINTER(Probe), P, c_int,
                                         POINTER(Detectors), P, c_int, c_int, c_double,
                                         ctypes.c_uint64, P]),
    }
    U = ctypes.c_uint32
    for kind, src, coord, wrap in _RS_FORMS:
        head = [c_double] * (5 if kind == "PG" else 4) + [U] * 3 + [P, P]
        if src == "curve":
            tail = [P, P, P, P, U, c_double, P, P]        # ads occ type curves Npoints dds gli cpro
        elif coord == "DW":
            tail = [P, P, P, P, P, P]                     # dw ads occ type gli cpro
        else:
            tail = [P, P, P, P, P]                        # ads occ type gli cpro
        sig[f"{kind}_rs_{src}_{coord}_{wrap}"] = (c_int, head + tail)
    sig["PG_rs_curve_DW_cutpot_oneatom"] = (c_int, [c_double] * 5 + [U, U] + [c_double] * 4 +
                                            [P, U, c_double, P])
    rec_head = [c_double] * 3 + [U] * 7 + [P, P]
    sig["Potential_rec_DT_DW"] = (c_int, rec_head + [P, P, P, P, P, P])
    sig["Potential_rec_curve_DW"] = (c_int, rec_head + [P, P, P, P, U, c_double, P, P])
    sig["scat_ampl_rs_DT_DW"] = (c_double, [c_int, c_double, c_double])
    sig["scat_ampl_rs2_DT_DW"] = (c_double, [c_int, c_double, c_double])
    sig["scat_ampl_rs2_DT_DW0"] = (c_double, [c_int, c_double])
    sig["CreatePots_rec_DT_DW"] = (None, [U, U, c_double, P, P, c_double, P])
    sig["CreatePots_rs_DT_DW"] = (None, [U, U, c_double, P, P, P])
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
