"""The drop-in boundary against the reference's own driver and header (CPU only,
needs the reference sources: $DEM_REF_DIR, else ../reference beside this
repository; skipped where they are absent).

1. The reference's main.cpp, unmodified, compiles against its own heydem.h and
   links against libdem_gb300.so alone: every symbol the driver uses
   (heydem.h:366-613 functions, the Allocation.cpp process globals) resolves in
   the library.  Link only; nothing runs.
2. Every host function heydem.h:366-613 declares has, in
   include/heydem_gb300.h, the same return type and parameter list, where the
   reference's C++ reference parameters (T&) are pointers (T*): identical at the
   ABI level.  Checked by the compiler on both headers in one translation unit,
   so a slip in parameter order, count or type in a 19-argument signature is a
   build error, which a link of C symbols cannot catch.

main.cpp includes thrust/scan.h from a host translation unit and never uses it
(main.cpp:6); CCCL 3 rejects that include in host code, so an empty
thrust/scan.h on an include path given first stands in for it."""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

import _harness

ROOT = Path(__file__).resolve().parents[1]
LIB = ROOT / "gpucode_gb300" / "libdem_gb300.so"


def _ref_dir() -> Path:
    d = _harness.REF_SRC
    if not (d / "main.cpp").exists() or not (d / "heydem.h").exists():
        pytest.skip(f"reference sources not found at {d} (set DEM_REF_DIR)")
    return d


def _nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        pytest.skip("nvcc not found")
    return exe


def _host_functions(header: str) -> list[str]:
    """names of the host functions the reference header declares extern "C" (its kernels excluded)"""
    names = re.findall(r'extern\s+"C"\s+(?!__global__)[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(', header)
    return sorted(set(names))


def test_reference_main_links_against_the_library(tmp_path):
    ref = _ref_dir()
    nvcc = _nvcc()
    assert LIB.exists(), "libdem_gb300.so is built by the session fixture"
    (tmp_path / "thrust").mkdir()
    (tmp_path / "thrust" / "scan.h").write_text("")
    obj, exe = tmp_path / "main.o", tmp_path / "gapp"
    r = subprocess.run([nvcc, "-std=c++17", "-w", "-I", str(tmp_path), "-I", str(ref), "-c", str(ref / "main.cpp"),
                        "-o", str(obj)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([nvcc, "-o", str(exe), str(obj), "-L", str(LIB.parent), "-ldem_gb300",
                        "-Xlinker", f"-rpath={LIB.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert exe.exists()
    # what the driver needs from the library: every extern "C" host function it calls and the globals
    und = subprocess.run(["nm", "-u", str(obj)], capture_output=True, text=True).stdout.split()
    exported = set(subprocess.run(["nm", "-D", "--defined-only", str(LIB)], capture_output=True,
                                  text=True).stdout.split())
    wanted = [s for s in und if s in _host_functions((ref / "heydem.h").read_text()) or s.startswith(("d", "h"))
              and s in ("dPos", "dVel", "dAngVel", "dForce", "dMom", "dRMom", "dRad", "hPos", "hVel", "hAngVel",
                        "hForce", "hRad", "d_GridParticleHash", "d_GridParticleIndex", "d_CellStart",
                        "d_CellEnd")]
    assert len(wanted) >= 35, wanted
    missing = [s for s in wanted if s not in exported]
    assert not missing, missing


def test_exported_signatures_match_the_reference_header(tmp_path):
    ref = _ref_dir()
    nvcc = _nvcc()
    names = _host_functions((ref / "heydem.h").read_text())
    assert len(names) >= 29, names
    src = ['#include "heydem.h"  /* the reference: its structs, then its declarations */']
    src += [f"#define {n} ours_{n}" for n in names]
    src += ['#include "heydem_gb300.h"  /* this library, declarations renamed; the structs are the reference\'s */',
            "#include <type_traits>",
            "template <class T> struct abi { using type = T; };",
            "template <class T> struct abi<T&> { using type = T*; };  /* a C++ reference is a pointer in the ABI */",
            "template <class F> struct abi_fn;",
            "template <class R, class... A> struct abi_fn<R(A...)> { using type = R(typename abi<A>::type...); };"]
    for n in names:
        src.append(f"#undef {n}")
        src.append(f"static_assert(std::is_same<abi_fn<decltype({n})>::type, decltype(ours_{n})>::value, "
                   f'"{n}: signature differs from the reference\'s");')
    tu = tmp_path / "abi_check.cpp"
    tu.write_text("\n".join(src) + "\n")
    r = subprocess.run([nvcc, "-std=c++17", "-x", "c++", "-w", "-I", str(ref), "-I", str(ROOT / "include"), "-c",
                        str(tu), "-o", str(tmp_path / "abi_check.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_a_signature_slip_is_a_build_error(tmp_path):
    """the check above fails when one parameter of one declaration changes type"""
    ref = _ref_dir()
    nvcc = _nvcc()
    hdr = (ROOT / "include" / "heydem_gb300.h").read_text()
    slipped = hdr.replace("void IndexOffset(int* d_Num, int* d_nei, int Nn);",
                          "void IndexOffset(int* d_Num, int* d_nei, long Nn);")
    assert slipped != hdr
    (tmp_path / "inc").mkdir()
    (tmp_path / "inc" / "heydem_gb300.h").write_text(slipped)
    src = "\n".join(['#include "heydem.h"', "#define IndexOffset ours_IndexOffset", '#include "heydem_gb300.h"',
                     "#include <type_traits>", "#undef IndexOffset",
                     "static_assert(std::is_same<decltype(IndexOffset), decltype(ours_IndexOffset)>::value, "
                     '"IndexOffset");']) + "\n"
    tu = tmp_path / "slip.cpp"
    tu.write_text(src)
    r = subprocess.run([nvcc, "-std=c++17", "-x", "c++", "-w", "-I", str(ref), "-I", str(tmp_path / "inc"), "-c",
                        str(tu), "-o", str(tmp_path / "slip.o")], capture_output=True, text=True)
    assert r.returncode != 0 and "IndexOffset" in r.stderr
