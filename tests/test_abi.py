"""CPU checks of the C ABI: the library builds, loads and exports what include/phgpu.h declares."""
from __future__ import annotations

import ctypes as C
import subprocess

from phasta_gb300 import _lib as L


def test_library_exports_every_declared_symbol(gpu_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(L.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    declared = L.exported_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if s not in exported]
    assert not missing, missing


def test_create_rejects_invalid_arguments_before_touching_the_device(gpu_lib):
    h = C.c_void_p()
    assert gpu_lib.phgpu_create(None, None, C.byref(h)) == 1  # PHGPU_ERR_INVALID
    m = L.Mesh()
    cfg = L.Config()
    m.nshg = 0
    assert gpu_lib.phgpu_create(C.byref(m), C.byref(cfg), C.byref(h)) == 1
    assert gpu_lib.phgpu_destroy(None) == 0
    assert gpu_lib.phgpu_last_error(None) == b"null context"


def test_struct_sizes_match_header():
    # phgpu_config: 12 doubles, 9 ints, 3 doubles, 2 ints, 2 ints + 6 reserved (packed by the C ABI rules)
    assert C.sizeof(L.Config) % 8 == 0
    assert C.sizeof(L.Stats) == 4 * 4 + 7 * 8
