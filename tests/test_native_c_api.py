"""The native API from C, as a C driver uses it (CPU only): a C11 program that
reads the reference's keyword files, derives the set-up and, given a GPU,
creates an engine, steps it and reads the state back, compiles with gcc against
include/heydem_gb300.h and links against libdem_gb300.so.  Its host part runs
here (no GPU): dem_read_input + dem_build_setup from C give the set-up the
Python binding derives from the same files."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from gpucode_gb300 import configs
from gpucode_gb300.engine import Setup

ROOT = Path(__file__).resolve().parents[1]
CUDA = Path("/usr/local/cuda")

DRIVER = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "heydem_gb300.h"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const char* genfile = argv[1];
  const int run = strcmp(argv[2], "run") == 0;
  dem_input in;
  if (dem_read_input(genfile, &in, NULL) != DEM_OK) { fprintf(stderr, "%s\n", dem_last_error()); return 1; }
  double* dia = (double*)malloc(sizeof(double) * in.np);
  double* rad = (double*)malloc(sizeof(double) * in.np);
  int* lvl = (int*)malloc(sizeof(int) * in.np);
  int* rank = (int*)malloc(sizeof(int) * in.np);
  dem_setup s;
  if (dem_read_input(genfile, &in, dia) != DEM_OK ||
      dem_build_setup(&in, dia, &s, rad, lvl, rank) != DEM_OK) {
    fprintf(stderr, "%s\n", dem_last_error());
    return 1;
  }
  printf("setup %d %d %d %lld %.17g %.17g\n", s.np, s.n_levels, s.sys_ncells, s.n_pp_slots, s.prm.dt,
         s.unit.rlunit);
  if (!run) return 0;
  /* with a GPU: positions (reduced units, np x 3 doubles) from argv[3], the
   * engine in mixed precision, ten steps, the state back */
  double3* pos = (double3*)calloc(s.np, sizeof(double3));
  double3* vel = (double3*)calloc(s.np, sizeof(double3));
  double3* spin = (double3*)calloc(s.np, sizeof(double3));
  double3* force = (double3*)calloc(s.np, sizeof(double3));
  FILE* f = argc > 3 ? fopen(argv[3], "rb") : NULL;
  if (!f || fread(pos, sizeof(double3), (size_t)s.np, f) != (size_t)s.np) return 3;
  fclose(f);
  dem_options o;
  dem_default_options(&o);
  dem_ctx* c = NULL;
  if (dem_create(&s, rad, lvl, rank, &o, &c) != DEM_OK || dem_set_state(c, pos, vel, spin) != DEM_OK ||
      dem_step(c, 10) != DEM_OK || dem_sync(c) != DEM_OK ||
      dem_get_state(c, pos, vel, spin, force, NULL) != DEM_OK) {
    fprintf(stderr, "%s\n", dem_last_error());
    dem_destroy(c);
    return 1;
  }
  FILE* g = fopen(argv[4], "wb");
  if (!g || fwrite(pos, sizeof(double3), (size_t)s.np, g) != (size_t)s.np) return 4;
  fclose(g);
  printf("stepped\n");
  dem_destroy(c);
  return 0;
}
"""


def _driver(tmp_path):
    """the C driver built against the library, and a small wet workload's keyword files"""
    lib = ROOT / "gpucode_gb300" / "libdem_gb300.so"
    if not lib.exists():
        pytest.fail("libdem_gb300.so is missing: run the build first")
    src = tmp_path / "driver.c"
    src.write_text(DRIVER)
    exe = tmp_path / "driver"
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-I", str(CUDA / "include"),
                        str(src), "-o", str(exe), "-L", str(lib.parent), "-ldem_gb300",
                        f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath-link,{CUDA / 'lib64'}", "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    w = configs.small_wet(n=300)
    prefix = tmp_path / "heyi"
    configs.write_heyi(str(prefix), w.inp, w.dia)
    return exe, prefix, w


def test_c_driver_compiles_links_and_derives_the_set_up(tmp_path):
    exe, prefix, w = _driver(tmp_path)
    r = subprocess.run([str(exe), str(prefix), "setup"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    tag, np_, levels, cells, slots, dt, lunit = r.stdout.split()
    ref = Setup.from_files(str(prefix)).s
    assert tag == "setup"
    assert (int(np_), int(levels), int(cells), int(slots)) == (ref.np, ref.n_levels, ref.sys_ncells, ref.n_pp_slots)
    assert float(dt) == ref.prm.dt and float(lunit) == ref.unit.rlunit
    assert int(np_) == 300 and np.isfinite(float(dt))


@pytest.mark.gpu
def test_c_driver_steps_like_the_python_binding(tmp_path, cuda):
    """the C driver's ten mixed steps from a bed's positions: the same bits as
    the same steps through the Python binding"""
    from gpucode_gb300.engine import Engine

    exe, prefix, w = _driver(tmp_path)
    setup = Setup.from_files(str(prefix))
    pos = np.ascontiguousarray(setup.to_reduced(w.pos0), np.float64)
    pos.tofile(tmp_path / "pos.bin")
    r = subprocess.run([str(exe), str(prefix), "run", str(tmp_path / "pos.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, cwd=tmp_path, timeout=120)
    assert r.returncode == 0 and "stepped" in r.stdout, r.stderr
    got = np.fromfile(tmp_path / "out.bin", np.float64).reshape(-1, 3)
    with Engine(setup, precision="mixed") as e:
        e.set_state(pos)
        e.step(10)
        e.sync()
        want = e.get_state()["pos"]
    assert got.shape == want.shape and np.array_equal(got, want)
    assert not np.array_equal(got, pos)
