"""ctypes binding of libcatana_gpu.so (the C ABI in include/catana_gpu.h).

The library is built in-tree by ``catana_gb300.build`` into ``catana_gb300/_lib/``.
Loading it needs no GPU; calling its compute entry points does.  There is no CPU
fallback: if the library is missing, importing this module raises ImportError.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libcatana_gpu.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        "libcatana_gpu.so not found at %s; build it with `python catana_gb300/build.py` "
        "(nvcc for sm_103a). catana_gb300 has no CPU fallback." % LIB_PATH)

lib = ctypes.CDLL(LIB_PATH)

_D = ctypes.c_double
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_U16 = ctypes.c_uint16
_U32 = ctypes.c_uint32
_I32 = ctypes.c_int32

# status codes (catana_status_t)
OK, ERR_ARG, ERR_DOMAIN, ERR_CUDA, ERR_NOMEM, ERR_UNSUPPORTED = range(6)
# flags
JL_AUTO, JL_INTERP, JL_EXACT, JL_POLY = 0, 1, 2, 3
FORM_PLAIN, FORM_SPLIT = 0, 4
SPLIT_ACCURATE = 32
HEALPIX_CONJ_FIX = 8
BATCH_NO_GRAPH = 16
BATCH_MBLK64 = 64


class Catalog(ctypes.Structure):
    """catana_catalog_t: one catalog of a batched decomposition."""
    _fields_ = [("points", ctypes.c_void_p), ("weights", ctypes.c_void_p), ("npoints", ctypes.c_int64),
                ("rmax", ctypes.c_double), ("kmax", ctypes.c_double), ("k_ln", ctypes.c_void_p),
                ("c_ln", ctypes.c_void_p), ("f_lmn", ctypes.c_void_p), ("lmax", ctypes.c_uint16),
                ("nmax", ctypes.c_uint16), ("reserved", ctypes.c_uint32)]

REC_FLOAT64, REC_FLOAT32 = 0, 1
REC_SPHERICAL, REC_CARTESIAN = 0, 2


class IngestSpec(ctypes.Structure):
    """catana_ingest_t: record layout and point filters for the device ingest."""
    _fields_ = [("layout", ctypes.c_uint32), ("reserved", ctypes.c_uint32), ("tophat_r0", ctypes.c_double),
                ("gauss_r0", ctypes.c_double), ("window", ctypes.c_void_p), ("window_n", ctypes.c_int64),
                ("window_min", ctypes.c_double), ("window_max", ctypes.c_double), ("mask", ctypes.c_void_p),
                ("mask_nside", ctypes.c_int64), ("seed", ctypes.c_uint64), ("index0", ctypes.c_uint64)]


SIGNATURES = {
    "catana_gpu_flmn_size": (ctypes.c_size_t, [_U16, _U16]),
    "catana_gpu_sfb_raw": (ctypes.c_int, [_P, _P, _I64, _U16, _U16, _D, _U32, _P, _P, _P, _P]),
    "catana_gpu_sfb_raw_dev": (ctypes.c_int, [_P, _P, _I64, _U16, _U16, _D, _U32, _P, _P, _P, _P, _P]),
    "catana_gpu_sfb_raw_noalloc": (ctypes.c_int, [_P, _P, _I64, _U16, _U16, _D, _U32, _P, _P, _P, _P]),
    "catana_gpu_sfb_raw_batched": (ctypes.c_int, [_P, _I32, _U32, _D, _P]),
    "catana_gpu_sfb_raw_batched_dev": (ctypes.c_int, [_P, _I32, _U32, _D, _P, _P]),
    "catana_gpu_batch_waves": (ctypes.c_double, []),
    "catana_gpu_batch_mblk": (ctypes.c_int32, []),
    "catana_gpu_accum_create": (ctypes.c_int, [_U16, _U16, _D, _U32, _P]),
    "catana_gpu_accum_add_f32": (ctypes.c_int, [_P, _P, _P, _I64]),
    "catana_gpu_accum_add": (ctypes.c_int, [_P, _P, _P, _I64]),
    "catana_gpu_accum_finish": (ctypes.c_int, [_P, _P, _P, _P]),
    "catana_gpu_accum_add_records": (ctypes.c_int, [_P, _P, _I64, _P]),
    "catana_gpu_accum_add_file": (ctypes.c_int, [_P, ctypes.c_char_p, _I64, _I64, _I64, _P, _P]),
    "catana_gpu_ingest": (ctypes.c_int, [_P, _I64, _P, _P, _P, _P]),
    "catana_gpu_accum_destroy": (ctypes.c_int, [_P]),
    "catana_gpu_sfb_healpix": (ctypes.c_int, [_I64, _P, _P, _U16, _U16, _D, _U32, _P, _P, _P, _P]),
    "catana_gpu_sfb_reverse": (ctypes.c_int, [_I64, _P, _P, _U16, _U16, _D, _U32, _P, _P, _P, _P]),
    "catana_gpu_bin_points": (ctypes.c_int, [_I64, _P, _I64, _P, _P, _P]),
    "catana_gpu_ang2pix_ring": (ctypes.c_int, [_I64, _P, _P, _I64, _P, _P]),
    "catana_gpu_pix2ang_ring": (ctypes.c_int, [_I64, _P, _I64, _P, _P, _P]),
    "catana_gpu_sbessel_zeros": (ctypes.c_int, [_U32, _I32, _P]),
    "catana_gpu_compute_kln": (ctypes.c_int, [_U16, _U16, _D, _P]),
    "catana_gpu_sbessel_integrals": (ctypes.c_int, [_P, _I64, _D, _D, _U32, _D, _P, _P, _I64, _P, _P]),
    "catana_gpu_last_error": (ctypes.c_char_p, []),
    "catana_gpu_fp64_peak": (ctypes.c_int, [ctypes.c_int32, _P]),
    "catana_gpu_test_split_stall": (ctypes.c_int, [_U32]),
    "catana_gpu_profile_enable": (None, [ctypes.c_int]),
    "catana_gpu_profile_report": (ctypes.c_int, [_P, _P, _P]),
    "catana_gpu_launch_count": (ctypes.c_uint64, []),
}

for _name, (_res, _args) in SIGNATURES.items():
    if hasattr(lib, _name):
        _f = getattr(lib, _name)
        _f.restype = _res
        _f.argtypes = _args


def last_error():
    return lib.catana_gpu_last_error().decode(errors="replace")


class CatanaError(RuntimeError):
    pass


def check(status, what=""):
    """Map a catana_status_t to the exception the reference's bindings raise."""
    if status == OK:
        return
    msg = last_error() or what
    if status in (ERR_ARG, ERR_DOMAIN):
        raise ValueError(msg)
    if status == ERR_NOMEM:
        raise MemoryError(msg)
    raise CatanaError("catana_gpu error %d: %s" % (status, msg))


def ptr(a):
    """Data pointer of a numpy array (None for None)."""
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)
