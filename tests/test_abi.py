"""The C-ABI boundary (CPU: load and inspect only, no compute calls that need a GPU)."""
import re
import subprocess
from pathlib import Path

import pytest

from gpucode_gb300 import _abi

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "heydem_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?(?:void|int|dem_status|char)\s*\*?\s*(\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def exported_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_abi.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_library_loads_and_layout_matches():
    lib = _abi.load()  # raises on a struct-layout mismatch
    assert b"sm_103a" in lib.dem_version()


def test_every_declared_function_is_exported():
    names = declared_functions()
    # the reference's entry points (heydem.h:366-613) and the native ones
    for must in ("BldNeborList", "PpInterCalc", "CirPWCalc", "UpdateSystem", "HstryCopy", "HstryCopyPW",
                 "BldCirWall", "PPCntHstryCopy", "WallCntHstryCopy", "VarInit", "setMaterial", "setLiquid",
                 "setParameters", "setCalpara", "IndexOffset", "ReadData", "UnitReduce", "DiaInput", "FindRec",
                 "LoadPara", "WrtTec", "ParticleFeed", "NeborToCPU", "ParticleInfoAlloc", "PPCntHstry_Alloc",
                 "WallCntHstry_Alloc", "NeborListAlloc", "ParamAlloc", "SearchCellAlloc", "FeedZoneAlloc",
                 "dem_create", "dem_step", "dem_set_state", "dem_get_state"):
        assert must in names, must
    syms = exported_symbols()
    missing = [n for n in names if n not in syms]
    assert not missing, f"declared but not exported: {missing}"


def test_reference_globals_are_exported():
    syms = exported_symbols()
    for g in ("dPos", "dVel", "dAngVel", "dForce", "dMom", "dRMom", "dRad", "hPos", "hVel", "hAngVel", "hForce",
              "hRad", "d_GridParticleHash", "d_GridParticleIndex", "d_CellStart", "d_CellEnd"):
        assert g in syms, g


def test_header_compiles_as_c_and_cxx(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "heydem_gb300.h"\nint main(void){ dem_setup s; (void)s; return 0; }\n')
    for comp in (["gcc", "-std=c11"], ["g++", "-std=c++17", "-x", "c++"]):
        r = subprocess.run(comp + ["-fsyntax-only", "-I", str(ROOT / "include"), "-I", "/usr/local/cuda/include",
                                   str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError, match="not built"):
        _abi.load(tmp_path / "libdem_gb300.so")


def test_compat_precision_switch():
    """DEM_COMPAT_PRECISION=mixed selects the mixed mode of the reference's entry
    points for an unchanged driver; dem_compat_set_precision overrides it and
    rejects other values (no GPU call: fresh processes, so the environment is
    read anew)"""
    import os
    import sys

    code = ("from gpucode_gb300 import _abi; lib = _abi.load(); print(lib.dem_compat_precision()); "
            "print(lib.dem_compat_set_precision(7)); print(lib.dem_compat_set_precision(1), "
            "lib.dem_compat_precision())")
    env = {k: v for k, v in os.environ.items() if k != "DEM_COMPAT_PRECISION"}
    for value, first in ((None, "0"), ("mixed", "1"), ("fp64", "0")):
        e = dict(env)
        if value:
            e["DEM_COMPAT_PRECISION"] = value
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, env=e)
        assert r.returncode == 0, r.stderr
        lines = r.stdout.split()
        assert lines[0] == first, (value, r.stdout)
        assert int(lines[1]) == _abi.DEM_ERR_ARG
        assert lines[2:] == ["0", "1"]
