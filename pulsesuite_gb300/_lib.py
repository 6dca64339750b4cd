"""ctypes binding of libsbe_gb300.so (the C ABI declared in include/sbe_gb300.h).

The library is built in-tree by ``pulsesuite_gb300.build``.  There is no CPU
fallback: if the shared object is missing or no CUDA device is present, every
entry point raises.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsbe_gb300.so")

# flag bits (mb.params order)
F_OPTICS, F_EXCITONS, F_EHS, F_SCREENED, F_PHONON, F_DCTRANS, F_LF, F_FREEPOT, F_DIAGDPH, \
    F_OFFDIAGDPH, F_RECOMB, F_LORENTZ = (1 << i for i in range(12))
FLAG_BITS = dict(Optics=F_OPTICS, Excitons=F_EXCITONS, EHs=F_EHS, Screened=F_SCREENED,
                 Phonon=F_PHONON, DCTrans=F_DCTRANS, LF=F_LF, FreePot=F_FREEPOT,
                 DiagDph=F_DIAGDPH, OffDiagDph=F_OFFDIAGDPH, Recomb=F_RECOMB,
                 LorentzDelta=F_LORENTZ)

PREC_FP64 = 0
PREC_MIXED = 1

# C-ABI exported symbols (must match include/sbe_gb300.h)
EXPORTS = (
    "sbe_last_error", "sbe_version", "sbe_constants", "sbe_ctx_create", "sbe_ctx_destroy",
    "sbe_ctx_layout", "sbe_ctx_table", "sbe_dpdt", "sbe_dCdt", "sbe_dDdt", "sbe_calch",
    "sbe_screened_arrays", "sbe_gamma", "sbe_offdiag", "sbe_phonon_rates", "sbe_carrier_rates",
    "sbe_spont_emission", "sbe_sources",
    "sbe_prop2qw", "sbe_qw2prop", "sbe_leapfrog_step", "sbe_rk4_step", "sbe_rhs",
    "sbe_tc_selftest", "sbe_rk4_graph_create", "sbe_graph_launch", "sbe_graph_destroy",
    "sbe_ctx_profile", "sbe_ctx_profile_read", "sbe_prop2qw_noalloc", "sbe_ctx_check",
    "sbe_ctx_charge", "sbe_wait_selftest",
    "sbe_convert_selftest", "sbe_deph_selftest",
    "sbe_pstd_create", "sbe_pstd_destroy", "sbe_pstd_grid", "sbe_pstd_deriv", "sbe_pstd_update_h",
    "sbe_pstd_update_e", "sbe_pstd_step", "sbe_pstd_elong", "sbe_couple_create",
    "sbe_couple_destroy", "sbe_couple_buffers", "sbe_couple_set_step", "sbe_couple_reset",
    "sbe_couple_sample",
    "sbe_couple_deposit", "sbe_couple_step", "sbe_couple_graph_create",
    "sbe_backup_format", "sbe_backup_parse", "sbe_wire_info", "sbe_wire_pdote",
    "sbe_deph_extrema", "sbe_calc_jfx",
    "sbe_qw_placement", "sbe_e_at_xyz", "sbe_autotune", "sbe_ctx_tiles",
    "sbe_local_field", "sbe_pstd3_create", "sbe_pstd3_destroy", "sbe_pstd3_grid",
    "sbe_pstd3_curl", "sbe_pstd3_update_h", "sbe_pstd3_update_e", "sbe_pstd3_step",
    "sbe_pstd3_elong", "sbe_couple3_create", "sbe_couple3_destroy", "sbe_couple3_buffers",
    "sbe_couple3_reset", "sbe_couple3_sample", "sbe_couple3_deposit", "sbe_couple3_step",
    "sbe_couple3_graph_create",
)


class SbeWireDesc(ctypes.Structure):
    _fields_ = [("nk", ctypes.c_int), ("wire_index", ctypes.c_int), ("flags", ctypes.c_int),
                ("pad0", ctypes.c_int), ("L", ctypes.c_double), ("Delta0", ctypes.c_double),
                ("gap", ctypes.c_double), ("me", ctypes.c_double), ("mh", ctypes.c_double),
                ("HO", ctypes.c_double), ("gam_e", ctypes.c_double), ("gam_h", ctypes.c_double),
                ("gam_eh", ctypes.c_double), ("epsr", ctypes.c_double), ("Oph", ctypes.c_double),
                ("Gph", ctypes.c_double), ("temp", ctypes.c_double), ("Edc", ctypes.c_double)]


class SbePstdDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("n_abc", ctypes.c_int), ("pad0", ctypes.c_int),
                ("pad1", ctypes.c_int), ("dx", ctypes.c_double), ("epsr", ctypes.c_double),
                ("abc_strength", ctypes.c_double)]


class SbePstd3Desc(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int * 3), ("n_abc", ctypes.c_int * 3), ("fp32_work", ctypes.c_int),
                ("pad0", ctypes.c_int), ("d", ctypes.c_double * 3), ("epsr", ctypes.c_double),
                ("abc_strength", ctypes.c_double)]


class SbeCouple3Desc(ctypes.Structure):
    _fields_ = [("src_index", ctypes.c_int), ("pol", ctypes.c_int), ("pad0", ctypes.c_int),
                ("pad1", ctypes.c_int), ("E0", ctypes.c_double), ("tau", ctypes.c_double),
                ("w0", ctypes.c_double), ("tpeak", ctypes.c_double), ("t0", ctypes.c_double),
                ("waist", ctypes.c_double), ("gate", ctypes.c_double)]


class SbeCoupleDesc(ctypes.Structure):
    _fields_ = [("src_index", ctypes.c_int), ("longitudinal", ctypes.c_int),
                ("pad0", ctypes.c_int), ("pad1", ctypes.c_int), ("E0", ctypes.c_double),
                ("tau", ctypes.c_double), ("w0", ctypes.c_double), ("tpeak", ctypes.c_double),
                ("t0", ctypes.c_double)]


class SbeError(RuntimeError):
    pass


_lib = None


def load(path=LIB_PATH):
    """Load the shared library (no rebuild); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise SbeError(f"{path} is missing: run `python -m pulsesuite_gb300.build` (needs nvcc)")
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    I = ctypes.c_int
    Dbl = ctypes.c_double
    lib.sbe_last_error.restype = ctypes.c_char_p
    lib.sbe_version.restype = I
    sig = {
        "sbe_constants": [P],
        "sbe_backup_format": [P, ctypes.c_longlong, P, ctypes.c_longlong, P, I],
        "sbe_backup_parse": [P, ctypes.c_longlong, P, ctypes.c_longlong, I],
        "sbe_ctx_create": [P, I, P, P],
        "sbe_ctx_destroy": [P],
        "sbe_ctx_layout": [P, P, P, P],
        "sbe_ctx_table": [P, I, I, P, ctypes.c_longlong, P],
        "sbe_dpdt": [I, P, P, P, P, P, P, P, P, P, P, P],
        "sbe_dCdt": [I, P, P, P, P, P, P, P, P],
        "sbe_dDdt": [I, P, P, P, P, P, P, P, P],
        "sbe_calch": [I, P, P, P, P, P, P, P, P, P, Dbl, I, I, I, P, P, P, P],
        "sbe_screened_arrays": [P, I, P, P, P, P, P],
        "sbe_gamma": [P, I, P, P, P, P, P, P],
        "sbe_offdiag": [P, I, P, P, P, P, P, P, P, P, P],
        "sbe_phonon_rates": [P, I, P, P, P, P, P, P, P, P, P],
        "sbe_carrier_rates": [P, I, P, P, P, P, P, P, P, I, P],
        "sbe_spont_emission": [P, I, P, P, P, P, P],
        "sbe_wire_info": [P, I, P, P, P, P, P, P, P],
        "sbe_wire_pdote": [P, I, P, P, P, P, P],
        "sbe_deph_extrema": [P, I, P, P],
        "sbe_calc_jfx": [ctypes.c_longlong, P, P, Dbl, Dbl, P, P],
        "sbe_qw_placement": [I, I, I, P, P, P, P, P, P],
        "sbe_e_at_xyz": [P, P, I, P, I, P, I, P, I, P, P],
        "sbe_sources": [P, I, P, P, P, P, P, P, P, P, P, P, P],
        "sbe_prop2qw": [P, I, P, I, P, P, P],
        "sbe_prop2qw_noalloc": [P, I, P, I, P, P, P],
        "sbe_qw2prop": [P, I, P, I, P, P, I, P],
        "sbe_leapfrog_step": [P, P, P, Dbl, P, P],
        "sbe_rk4_step": [P, P, P, P, P, P, Dbl, I, P, P],
        "sbe_rhs": [P, P, P, P, P, I, P, P, P, P],
        "sbe_tc_selftest": [I, I, P, P, I, I, I, P, P],
        "sbe_rk4_graph_create": [P, P, P, P, P, P, Dbl, I, P, P, P],
        "sbe_graph_launch": [P, P],
        "sbe_graph_destroy": [P],
        "sbe_ctx_profile": [P, I],
        "sbe_ctx_profile_read": [P, I, P, P],
        "sbe_ctx_check": [P, P],
        "sbe_wait_selftest": [P, P, P],
        "sbe_ctx_charge": [P, P, P],
        "sbe_convert_selftest": [P, P, ctypes.c_longlong, P, P, P],
        "sbe_deph_selftest": [P, P, P, I, P, P, P],
        "sbe_pstd_create": [P, P, P],
        "sbe_pstd_destroy": [P],
        "sbe_pstd_grid": [P, P, P, P],
        "sbe_pstd_deriv": [P, P, I, P, P],
        "sbe_pstd_update_h": [P, P, P, Dbl, P],
        "sbe_pstd_update_e": [P, P, P, P, Dbl, P],
        "sbe_pstd_step": [P, P, P, P, Dbl, P],
        "sbe_pstd_elong": [P, P, P, P, P],
        "sbe_couple_create": [P, P, P, P, P, P],
        "sbe_couple_destroy": [P],
        "sbe_couple_buffers": [P, P, P, P, P, P],
        "sbe_couple_set_step": [P, ctypes.c_longlong, P],
        "sbe_couple_reset": [P, P],
        "sbe_couple_sample": [P, P, P, P],
        "sbe_couple_deposit": [P, P],
        "sbe_couple_step": [P, P, P, P, P, P, P, Dbl, I, P],
        "sbe_couple_graph_create": [P, P, P, P, P, P, P, Dbl, I, P, P],
        "sbe_autotune": [P, ctypes.c_char_p],
        "sbe_local_field": [P, P, P, I, P, P, P],
        "sbe_pstd3_create": [P, P, P],
        "sbe_pstd3_destroy": [P],
        "sbe_pstd3_grid": [P, I, P, P, P],
        "sbe_pstd3_curl": [P, P, P, P],
        "sbe_pstd3_update_h": [P, P, P, Dbl, P],
        "sbe_pstd3_update_e": [P, P, P, P, Dbl, P],
        "sbe_pstd3_step": [P, P, P, P, Dbl, P],
        "sbe_pstd3_elong": [P, P, P, P, P, P, P, P, P],
        "sbe_couple3_create": [P, P, P, P, P, P],
        "sbe_couple3_destroy": [P],
        "sbe_couple3_buffers": [P, P, P, P, P],
        "sbe_couple3_reset": [P, P],
        "sbe_couple3_sample": [P, P, I, P],
        "sbe_couple3_deposit": [P, Dbl, P],
        "sbe_couple3_step": [P, P, P, P, P, P, Dbl, I, P],
        "sbe_couple3_graph_create": [P, P, P, P, P, P, Dbl, I, P, P],
        "sbe_ctx_tiles": [P, P, I, P],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = I
    _lib = lib
    return lib


def check(rc, what=""):
    if rc != 0:
        msg = load().sbe_last_error().decode(errors="replace")
        raise SbeError(f"{what} failed (code {rc}): {msg}")


def ptr(t):
    """Device pointer of a contiguous torch CUDA tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise SbeError("tensor argument must live on the GPU")
    if not t.is_contiguous():
        raise SbeError("tensor argument must be contiguous")
    return ctypes.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def backup_format(values, threads=0):
    """Backup-file text of complex values (host), one "re im" line each, numbers as
    Python's repr (SBEs.py:5524-5546 write_sbes_data); returns a memoryview of bytes."""
    import numpy as np
    v = np.ascontiguousarray(values, dtype=np.complex128).reshape(-1)
    out = np.empty(max(50 * v.size, 1), dtype=np.uint8)
    n = ctypes.c_longlong(0)
    check(load().sbe_backup_format(v.ctypes.data, v.size, out.ctypes.data, out.size,
                                   ctypes.byref(n), int(threads)), "sbe_backup_format")
    return memoryview(out)[:n.value]


def backup_parse(text, count, threads=0):
    """Inverse of backup_format: the first count lines of text (bytes) as complex128
    (SBEs.py:5548-5569 read_sbes_data)."""
    import numpy as np
    b = np.frombuffer(bytes(text), dtype=np.uint8)
    out = np.empty(count, dtype=np.complex128)
    check(load().sbe_backup_parse(b.ctypes.data if b.size else None, b.size, out.ctypes.data,
                                  int(count), int(threads)), "sbe_backup_parse")
    return out
