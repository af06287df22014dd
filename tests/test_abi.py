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


def test_wait_self_test_rejects_bad_arguments_before_touching_the_device(gpu_lib):
    st = C.c_int(-1)
    assert gpu_lib.phgpu_selftest_wait_limit(0, C.byref(st)) == L.PHGPU_ERR_INVALID
    assert gpu_lib.phgpu_selftest_wait_limit((1 << 19) + 1, C.byref(st)) == L.PHGPU_ERR_INVALID
    assert gpu_lib.phgpu_selftest_wait_limit(16, None) == L.PHGPU_ERR_INVALID
    assert st.value == -1


def test_struct_layouts_match_the_header_as_gcc_lays_them_out(tmp_path):
    """Every struct of include/phgpu.h: sizeof and the offset of every field as gcc computes them
    (tests/abi/layout.c), against the ctypes declarations."""
    import json
    from pathlib import Path
    src = Path(__file__).resolve().parent / "abi" / "layout.c"
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-o", str(exe), str(src)], check=True)
    got = json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    for cname, ct in (("phgpu_config", L.Config), ("phgpu_mesh", L.Mesh), ("phgpu_bnd_block", L.BndBlock),
                      ("phgpu_stats", L.Stats),
                      ("phgpu_net_train_config", L.NetTrainConfig), ("phgpu_net_train_stats", L.NetTrainStats)):
        c = got[cname]
        assert c["__size"] == C.sizeof(ct), cname
        fields = [f[0] for f in ct._fields_]
        assert sorted(fields) == sorted(k for k in c if k != "__size"), cname
        for f in fields:
            assert getattr(ct, f).offset == c[f], (cname, f)
    k = got["constants"]
    assert k["PHGPU_NET_NPARAM"] == L.PHGPU_NET_NPARAM and k["PHGPU_NET_NTRAIN"] == L.PHGPU_NET_NTRAIN
    assert k["PHGPU_RSTAT_NOALLOC_MAX_N"] == L.PHGPU_RSTAT_NOALLOC_MAX_N
    assert k["PHGPU_PRECOND_LEARNED"] == L.PHGPU_PRECOND_LEARNED and k["PHGPU_NET_PLAIN"] == L.PHGPU_NET_PLAIN


def test_network_parameter_layout_matches_the_oracle():
    from oracle import net_oracle as no
    assert no.NPARAM == L.PHGPU_NET_NPARAM and no.NTRAIN == L.PHGPU_NET_NTRAIN
