"""ctypes binding of ``include/phgpu.h`` (the C ABI of the GPU hot path).

Loading fails loudly when ``libphgpu.so`` has not been built: there is no CPU
fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libphgpu.so"

PHGPU_OK = 0
STATUS = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NONFINITE", 4: "SINGULAR", 5: "UNSUPPORTED", 6: "NOMEM", 7: "TOO_LARGE",
          8: "IO", 9: "NOTFOUND"}
PHGPU_FP64, PHGPU_MIXED = 0, 1
PHGPU_AP_FD, PHGPU_AP_LINEAR, PHGPU_AP_SPARSE, PHGPU_AP_EBE = 0, 1, 2, 3
PHGPU_RES_FP64, PHGPU_RES_GALERKIN64, PHGPU_RES_SPLITDF = 0, 1, 2
PHGPU_ERR_INVALID, PHGPU_ERR_UNSUPPORTED, PHGPU_ERR_TOO_LARGE = 1, 5, 7
PHGPU_ERR_IO, PHGPU_ERR_NOTFOUND = 8, 9
PHGPU_RSTAT_NOALLOC_MAX_N = 33554432
PHGPU_PRECOND_BDIAG, PHGPU_PRECOND_LEARNED = 0, 1
PHGPU_NET_USED, PHGPU_NET_FELL_BACK, PHGPU_NET_PLAIN = 0, 1, 2
PHGPU_NET_NPARAM, PHGPU_NET_NTRAIN = 53583, 53573
LU_FACT, LU_FORWARD, LU_BACKWARD, LU_PRODUCT = 0, 1, 2, 3

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


class Config(C.Structure):
    _fields_ = [
        ("Rgas", C.c_double), ("gamma", C.c_double), ("gamma1", C.c_double), ("pr", C.c_double),
        ("rmu", C.c_double),
        ("Dtgl", C.c_double), ("almi", C.c_double), ("alfi", C.c_double), ("gami", C.c_double),
        ("dtsfct", C.c_double), ("taucfct", C.c_double), ("temper", C.c_double),
        ("itau", C.c_int), ("ivart", C.c_int), ("iremoveStabTimeTerm", C.c_int), ("Navier", C.c_int),
        ("ipord", C.c_int), ("EntropyPressure", C.c_int),
        ("Kspace", C.c_int), ("nGMRES", C.c_int), ("minIters", C.c_int),
        ("etol", C.c_double), ("epsM", C.c_double), ("eGMRES", C.c_double),
        ("iter", C.c_int), ("istep", C.c_int),
        ("precision", C.c_int), ("ap_mode", C.c_int), ("outer_residual", C.c_int), ("idiff", C.c_int),
        ("no_graph", C.c_int), ("iDC", C.c_int), ("no_pipe", C.c_int), ("precond", C.c_int),
    ]


class BndBlock(C.Structure):
    _fields_ = [("lcsyst", C.c_int), ("nelem", C.c_int), ("ien", _ip), ("iBCB", _ip), ("BCB", _dp)]


class Mesh(C.Structure):
    _fields_ = [
        ("nshg", C.c_int), ("nelem", C.c_int), ("ien", _ip), ("x", _dp),
        ("nbelem", C.c_int), ("ienb", _ip), ("iBCB", _ip), ("BCB", _dp),
        ("iBC", _ip), ("BC", _dp), ("iper", _ip),
        ("nhex", C.c_int), ("ienh", _ip), ("nwedge", C.c_int), ("ienw", _ip),
        ("nbblk", C.c_int), ("bblk", C.POINTER(BndBlock)),
    ]


class GeombcInfo(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("numnp", "nshg", "numel", "numelb", "nen", "nelblk", "nelblb", "numpbc",
                                       "ntopsh", "nsd", "nbccols")]


class TopBlock(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("neltp", "nenl", "ipordl", "nshl", "nshlb", "nenbl", "lcsyst", "numnbc")]


class Stats(C.Structure):
    _fields_ = [
        ("iKs", C.c_int), ("lGMRES", C.c_int), ("ntotGM", C.c_int), ("status", C.c_int),
        ("unorm0", C.c_double), ("echeck", C.c_double), ("eGMRES", C.c_double), ("totres", C.c_double),
        ("rnorm", C.c_double), ("t_assembly_ms", C.c_double), ("t_gmres_ms", C.c_double),
        ("net_its", C.c_int), ("net_fallback", C.c_int),
    ]


class NetTrainConfig(C.Structure):
    _fields_ = [("epochs", C.c_int), ("npairs", C.c_int), ("lr", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("eps", C.c_float), ("clip", C.c_float), ("seed", C.c_uint),
                ("renormalize", C.c_int)]


class NetTrainStats(C.Structure):
    _fields_ = [("loss_first", C.c_double), ("loss_last", C.c_double), ("ms", C.c_double),
                ("steps", C.c_longlong)]


_lib = None


def lib():
    """Load libphgpu.so (raises if it is missing: build it with phasta_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing; run phasta_gb300.build.build() (needs nvcc)")
    L = C.CDLL(str(LIB_PATH))
    vp = C.c_void_p
    sig = {
        "phgpu_create": ([C.POINTER(Mesh), C.POINTER(Config), C.POINTER(vp)], C.c_int),
        "phgpu_destroy": ([vp], C.c_int),
        "phgpu_set_config": ([vp, C.POINTER(Config)], C.c_int),
        "phgpu_get_config": ([vp, C.POINTER(Config)], C.c_int),
        "phgpu_last_error": ([vp], C.c_char_p),
        "phgpu_stream": ([vp], vp),
        "phgpu_num_colors": ([vp], C.c_int),
        "phgpu_kernel_launches": ([vp], C.c_longlong),
        "phgpu_graph_cycles": ([vp], C.c_longlong),
        "phgpu_step_graphs": ([vp], C.c_longlong),
        "phgpu_rcm_order": ([C.POINTER(Mesh), C.POINTER(C.c_int), C.POINTER(C.c_longlong),
                             C.POINTER(C.c_longlong)], C.c_int),
        "phgpu_set_tuning": ([vp, C.c_int, C.c_int], C.c_int),
        "phgpu_tuning": ([vp, C.POINTER(C.c_int), C.POINTER(C.c_int), _dp], C.c_int),
        "phgpu_elmmfg": ([vp, _dp, _dp, _dp, _dp, _dp, C.c_int], C.c_int),
        "phgpu_elmres": ([vp, _dp, _dp, _dp], C.c_int),
        "phgpu_itrres": ([vp, _dp, _dp, _dp, _dp], C.c_int),
        "phgpu_i3lu": ([vp, _dp, _dp, C.c_int], C.c_int),
        "phgpu_solmfg": ([vp, _dp, _dp, _dp, _dp, _dp, C.POINTER(Stats)], C.c_int),
        "phgpu_itrcorrect": ([vp, _dp, _dp, _dp, _dp, _dp], C.c_int),
        "phgpu_newton": ([vp, _dp, _dp, _dp, _dp, C.POINTER(Stats)], C.c_int),
        "phgpu_time_step": ([vp, _dp, _dp, _dp, _dp, C.c_int, C.POINTER(Stats)], C.c_int),
        "phgpu_upload_state": ([vp, _dp, _dp, _dp, _dp], C.c_int),
        "phgpu_download_state": ([vp, _dp, _dp, _dp, _dp], C.c_int),
        "phgpu_newton_dev": ([vp, C.POINTER(Stats)], C.c_int),
        "phgpu_time_step_dev": ([vp, C.c_int, C.POINTER(Stats)], C.c_int),
        "phgpu_residual_norm_dev": ([vp, _dp], C.c_int),
        "phgpu_sweep_dev": ([vp, C.c_int], C.c_int),
        "phgpu_rstat_noalloc": ([vp, C.c_int, vp, vp], C.c_int),
        "phgpu_selftest_wait_limit": ([C.c_int, _ip], C.c_int),
        "phgpu_genadj": ([C.POINTER(Mesh), C.c_int, _ip, _ip, C.POINTER(C.c_int)], C.c_int),
        "phgpu_nnz_tot": ([vp, C.POINTER(C.c_int)], C.c_int),
        "phgpu_elmgmrs": ([vp, _dp, _dp, _dp, _dp, _dp], C.c_int),
        "phgpu_spsi3pre": ([vp, _dp, _dp], C.c_int),
        "phgpu_sparseap": ([vp, _dp, _dp], C.c_int),
        "phgpu_solgmrs": ([vp, _dp, _dp, C.c_int, _dp, _dp, _dp, _dp, C.POINTER(Stats)], C.c_int),
        "phgpu_elmgmre": ([vp, _dp, _dp, _dp, _dp, _dp], C.c_int),
        "phgpu_i3pre": ([vp, _dp, _dp], C.c_int),
        "phgpu_au1gmr": ([vp, _dp, _dp], C.c_int),
        "phgpu_solgmre": ([vp, _dp, _dp, _dp, _dp, _dp, _dp, C.POINTER(Stats)], C.c_int),
        "phgpu_set_bc": ([vp, _dp], C.c_int),
        "phgpu_net_set_weights": ([vp, _fp, C.c_int], C.c_int),
        "phgpu_net_get_weights": ([vp, _fp, C.c_int], C.c_int),
        "phgpu_net_graph": ([vp, _ip, C.POINTER(C.c_uint), C.c_longlong, C.POINTER(C.c_longlong), _fp], C.c_int),
        "phgpu_net_features": ([vp, _fp], C.c_int),
        "phgpu_net_usage": ([vp, C.POINTER(C.c_longlong)], C.c_int),
        "phgpu_net_apply": ([vp, _dp, _dp, _fp, _fp], C.c_int),
        "phgpu_net_loss_grad": ([vp, _dp, _dp, _dp, _fp], C.c_int),
        "phgpu_net_pairs": ([vp, C.c_int], C.c_int),
        "phgpu_net_collect": ([vp, C.c_int, C.c_int], C.c_int),
        "phgpu_net_train": ([vp, C.POINTER(NetTrainConfig), C.POINTER(NetTrainStats)], C.c_int),
        # include/phgpu_io.h
        "phgpu_io_openfile": ([C.c_char_p, C.c_char_p, _ip], C.c_int),
        "phgpu_io_closefile": ([C.c_int, C.c_char_p], C.c_int),
        "phgpu_io_readheader": ([C.c_int, C.c_char_p, _ip, C.c_int, C.c_char_p, C.c_char_p], C.c_int),
        "phgpu_io_readdatablock": ([C.c_int, C.c_char_p, vp, C.c_int, C.c_char_p, C.c_char_p], C.c_int),
        "phgpu_io_writeheader": ([C.c_int, C.c_char_p, _ip, C.c_int, C.c_int, C.c_char_p, C.c_char_p], C.c_int),
        "phgpu_io_writedatablock": ([C.c_int, C.c_char_p, vp, C.c_int, C.c_char_p, C.c_char_p], C.c_int),
        "phgpu_io_writestring": ([C.c_int, C.c_char_p], C.c_int),
        "phgpu_io_togglestrictmode": ([], C.c_int),
        "phgpu_io_last_error": ([], C.c_char_p),
        "phgpu_io_write_restart": ([C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp], C.c_int),
        "phgpu_io_read_restart": ([C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _ip], C.c_int),
        "phgpu_io_geombc_open": ([C.c_char_p, C.c_int, C.c_int, C.POINTER(vp)], C.c_int),
        "phgpu_io_geombc_free": ([vp], C.c_int),
        "phgpu_io_geombc_info": ([vp, C.POINTER(GeombcInfo)], C.c_int),
        "phgpu_io_geombc_arrays": ([vp, _dp, _ip, _ip, _dp, _ip], C.c_int),
        "phgpu_io_geombc_interior": ([vp, C.c_int, C.POINTER(TopBlock), _ip], C.c_int),
        "phgpu_io_geombc_boundary": ([vp, C.c_int, C.POINTER(TopBlock), _ip, _ip, _dp], C.c_int),
        "phgpu_io_genibc": ([C.c_int, C.c_int, _ip, _ip, _ip], C.c_int),
        "phgpu_io_genbc": ([C.c_int, C.c_int, C.c_int, _ip, _dp, C.c_int, _ip, _dp], C.c_int),
        "phgpu_io_checkphasta": ([C.c_char_p, C.c_char_p, C.c_int, _dp, _ip], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def exported_symbols() -> list[str]:
    """Names declared in include/phgpu.h and include/phgpu_io.h (used to check the library's exports)."""
    import re
    inc = Path(__file__).resolve().parent.parent / "include"
    names = set()
    for h in ("phgpu.h", "phgpu_io.h"):
        names |= set(re.findall(r"\b(phgpu_[a-z0-9_]+)\s*\(", (inc / h).read_text()))
    return sorted(names)


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous, "expected a contiguous float64 array"
    return a.ctypes.data_as(_dp)


def fptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous, "expected a contiguous float32 array"
    return a.ctypes.data_as(_fp)


def iptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous, "expected a contiguous int32 array"
    return a.ctypes.data_as(_ip)
