"""The C ABI from a C compiler's side: tests/abi/c_caller.c, built with gcc against
include/phgpu.h and linked to libphgpu.so, runs ElmMFG and SolMFG on the GPU; its outputs must
equal the same calls through the ctypes binding bit for bit."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from helpers import channel
from phasta_gb300 import _lib as L
from phasta_gb300.solver import GpuSolver

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent


def _write(path, case, p, y, ac):
    N = case.nshg
    with open(path, "wb") as f:
        np.array([N, case.nelem, case.nbelem], "<i4").tofile(f)
        np.ascontiguousarray(case.ien, "<i4").tofile(f)
        case.x_ref().astype("<f8").tofile(f)
        np.ascontiguousarray(case.iBC, "<i4").tofile(f)
        np.ascontiguousarray(case.BC, "<f8").tofile(f)
        np.ascontiguousarray(case.iper, "<i4").tofile(f)
        np.ascontiguousarray(case.ienb, "<i4").tofile(f)
        np.ascontiguousarray(case.iBCB, "<i4").tofile(f)
        np.ascontiguousarray(case.BCB, "<f8").tofile(f)
        np.asarray(y, "<f8").tofile(f)
        np.asarray(ac, "<f8").tofile(f)
        d = [p[k] for k in ("Rgas", "gamma", "gamma1", "pr", "rmu", "Dtgl", "almi", "alfi", "gami", "dtsfct",
                            "taucfct", "temper")]
        np.array(d, "<f8").tofile(f)
        np.array([p[k] for k in ("itau", "ivart", "iremoveStabTimeTerm", "Navier", "ipord", "EntropyPressure",
                                 "Kspace", "nGMRES", "minIters")], "<i4").tofile(f)
        np.array([p["etol"], p["epsM"], p["eGMRES"]], "<f8").tofile(f)
        np.array([p["iter"], p["istep"], p["precision"], p["ap_mode"], p["outer_residual"], p["idiff"], 0,
                  p["iDC"], 0, p["precond"]], "<i4").tofile(f)


def test_c_caller_matches_the_ctypes_binding(gpu_lib, tmp_path):
    exe = tmp_path / "c_caller"
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-o", str(exe), str(HERE / "abi" / "c_caller.c"),
                    str(L.LIB_PATH), f"-Wl,-rpath,{L.LIB_PATH.parent}"], check=True)
    case, p, y, ac = channel(6, ac_scale=0.05)
    _write(tmp_path / "in.bin", case, p, y, ac)
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    N = case.nshg
    out = np.fromfile(tmp_path / "out.bin", dtype="<f8", count=5 * N * 4 + 25 * N * 2)
    iks = int(np.fromfile(tmp_path / "out.bin", dtype="<i4")[-1])
    parts, o = [], 0
    for n in (5 * N, 5 * N, 25 * N, 5 * N, 25 * N, 5 * N):
        parts.append(out[o:o + n])
        o += n
    g = GpuSolver(case, p)
    res, rmes, bd = g.ElmMFG(y, ac)
    res2, bd2, Dy, st = g.SolMFG(y, ac)
    for a, b in zip(parts, (res, rmes, bd, res2, bd2, Dy)):
        assert np.array_equal(a, b)
    assert iks == st.iKs
