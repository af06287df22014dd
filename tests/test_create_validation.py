"""phgpu_create's argument checks, which run on the host before any device call.

Each case corrupts one field of a valid mesh or configuration and expects the status that
include/phgpu.h documents: PHGPU_ERR_INVALID for malformed input (connectivity or periodic
masters out of range, inconsistent periodic bits, counts and pointers that do not agree,
out-of-range solver settings), PHGPU_ERR_UNSUPPORTED for PHASTA input outside the implemented
path (chained periodic masters, scaled-plane extraction, itau other than 0 and 1, p > 1,
entropy-variable pressure, idiff = 2).  A rejected call never reaches the device, so these
run without a GPU; the unmodified mesh passes the checks (status 0 with a GPU, PHGPU_ERR_CUDA
without one)."""
from __future__ import annotations

import copy
import ctypes as C

import numpy as np
import pytest

from phasta_gb300 import _lib as L
from phasta_gb300 import mesh
from phasta_gb300.solver import _config, _MeshArrays, make_params

PHGPU_ERR_CUDA = 2


def _create(lib, case, params, mutate=None, cfg_mutate=None):
    # the mesh arrays may alias the case's own (contiguous int32 arrays are not copied)
    ma = _MeshArrays(copy.deepcopy(case))
    if mutate:
        mutate(ma)
    cfg = _config(params)
    if cfg_mutate:
        cfg_mutate(cfg)
    h = C.c_void_p()
    rc = lib.phgpu_create(C.byref(ma.m), C.byref(cfg), C.byref(h))
    if rc == 0:
        lib.phgpu_destroy(h)
    return rc


@pytest.fixture(scope="module")
def tet(gpu_lib):
    case, ph = mesh.channel_case(2)
    return case, make_params(ph["mu"], ph["dt"])


def _set(arr, i, v):
    arr[i] = v


def _master_and_slave(case):
    iper = np.asarray(case.iper)
    s = int(np.flatnonzero(iper != np.arange(case.nshg))[0])
    return int(iper[s]), s


def _free_node(case):
    iper = np.asarray(case.iper)
    return int(np.flatnonzero(iper == np.arange(case.nshg))[0])


def test_the_valid_mesh_passes(gpu_lib, tet):
    case, p = tet
    assert _create(gpu_lib, case, p) in (0, PHGPU_ERR_CUDA)


@pytest.mark.parametrize("name,mutate", [
    ("ien at nshg", lambda ma: _set(ma.ien, 0, ma.m.nshg)),
    ("ien negative", lambda ma: _set(ma.ien, 5, -1)),
    ("boundary ien at nshg", lambda ma: _set(ma.ienb, 3, ma.m.nshg)),
    ("iper at nshg", lambda ma: _set(ma.iper, 0, ma.m.nshg)),
    ("iper negative", lambda ma: _set(ma.iper, 1, -2)),
    ("no elements", lambda ma: setattr(ma.m, "nelem", 0)),
    ("negative element count", lambda ma: setattr(ma.m, "nelem", -1)),
    ("negative boundary count", lambda ma: setattr(ma.m, "nbelem", -1)),
    ("boundary count without connectivity", lambda ma: setattr(ma.m, "ienb", None)),
    ("no coordinates", lambda ma: setattr(ma.m, "x", None)),
    ("no iBC", lambda ma: setattr(ma.m, "iBC", None)),
    ("no iper", lambda ma: setattr(ma.m, "iper", None)),
    ("no nodes", lambda ma: setattr(ma.m, "nshg", 0)),
    ("hex count without connectivity", lambda ma: setattr(ma.m, "nhex", 3)),
])
def test_malformed_mesh_is_invalid(gpu_lib, tet, name, mutate):
    case, p = tet
    assert _create(gpu_lib, case, p, mutate) == L.PHGPU_ERR_INVALID, name


def test_periodic_bits_must_match_the_masters(gpu_lib, tet):
    case, p = tet
    n = _free_node(case)
    _m, s = _master_and_slave(case)

    def set_bit(ma):
        ma.iBC[n] |= 1 << 10  # a node without a master marked periodic

    def clear_bit(ma):
        ma.iBC[s] &= ~(1 << 10)  # a slave not marked periodic

    assert _create(gpu_lib, case, p, set_bit) == L.PHGPU_ERR_INVALID
    assert _create(gpu_lib, case, p, clear_bit) == L.PHGPU_ERR_INVALID


def test_chained_masters_and_scaled_planes_are_unsupported(gpu_lib, tet):
    case, p = tet
    m, s = _master_and_slave(case)
    n = _free_node(case)

    def chain(ma):
        ma.iper[m] = s  # the master points back at its slave: a two-node cycle
        ma.iBC[m] |= 1 << 10

    def irscale(ma):
        ma.iBC[n] |= 1 << 11

    assert _create(gpu_lib, case, p, chain) == L.PHGPU_ERR_UNSUPPORTED
    assert _create(gpu_lib, case, p, irscale) == L.PHGPU_ERR_UNSUPPORTED


@pytest.mark.parametrize("field,value,code", [
    ("Kspace", 0, L.PHGPU_ERR_INVALID),
    ("Kspace", 64, L.PHGPU_ERR_INVALID),
    ("nGMRES", 0, L.PHGPU_ERR_INVALID),
    ("iDC", 4, L.PHGPU_ERR_INVALID),
    ("iDC", -1, L.PHGPU_ERR_INVALID),
    ("precond", 2, L.PHGPU_ERR_INVALID),
    ("itau", 2, L.PHGPU_ERR_UNSUPPORTED),
    ("itau", 10, L.PHGPU_ERR_UNSUPPORTED),
    ("ipord", 2, L.PHGPU_ERR_UNSUPPORTED),
    ("EntropyPressure", 1, L.PHGPU_ERR_UNSUPPORTED),
    ("idiff", 2, L.PHGPU_ERR_UNSUPPORTED),
])
def test_configuration_outside_the_path(gpu_lib, tet, field, value, code):
    case, p = tet
    assert _create(gpu_lib, case, p, cfg_mutate=lambda c: setattr(c, field, value)) == code


def test_franca_tau_is_fp64_only(gpu_lib, tet):
    case, p = tet
    assert _create(gpu_lib, case, dict(p, itau=1, precision=L.PHGPU_MIXED)) == L.PHGPU_ERR_UNSUPPORTED
    assert _create(gpu_lib, case, dict(p, itau=1)) in (0, PHGPU_ERR_CUDA)


@pytest.mark.parametrize("make,field", [
    (lambda: mesh.channel_hex_case(2), "ienh"),
    (lambda: mesh.channel_wedge_case((2, 2, 2)), "ienw"),
])
def test_hex_and_wedge_connectivity_in_range(gpu_lib, make, field):
    case, ph = make()
    p = make_params(ph["mu"], ph["dt"])
    assert _create(gpu_lib, case, p) in (0, PHGPU_ERR_CUDA)
    assert _create(gpu_lib, case, p, lambda ma: _set(getattr(ma, field), 2, case.nshg)) == L.PHGPU_ERR_INVALID
    assert _create(gpu_lib, case, p, lambda ma: _set(getattr(ma, field), 7, -1)) == L.PHGPU_ERR_INVALID
