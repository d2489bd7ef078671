"""The packed 200,000-sphere bed file (tests/golden/packed_wet200k.npz) that the
benchmark's two arms and the large parity tests start from (CPU only)."""
import subprocess
import sys
from pathlib import Path

import numpy as np

from gpucode_gb300 import configs
from gpucode_gb300.engine import packing_metrics

ROOT = Path(__file__).resolve().parents[1]
BED = ROOT / "tests" / "golden" / "packed_wet200k.npz"


def test_bed_loads_without_the_gpu_library():
    """the reference arm reads the bed and runs the oracle on it without
    mapping libdem_gb300.so"""
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from gpucode_gb300 import configs, _abi\n"
            "w = configs.load_bed(%r)\n"
            "assert w.setup.n == 200000 and _abi._lib is None\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libdem_gb300' not in maps\n"
            "print('ok')\n") % (str(ROOT), str(BED))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr


def test_bed_is_the_wet_workload_packed():
    """the stored set-up is the wet workload's (levels, slots and cells equal a
    fresh set-up from the seeded diameters; radii to the last ulp of numpy's
    exp on the machine that made the file) and the bed is packed"""
    bed = configs.load_bed(BED)
    s = bed.setup.s
    w = configs.wet(n=bed.setup.n)
    f = w.setup.s
    assert s.n_levels == f.n_levels == 4
    assert s.n_pp_slots == f.n_pp_slots and s.sys_ncells == f.sys_ncells
    assert list(s.level_nnebors)[:4] == list(f.level_nnebors)[:4]
    assert list(s.level_npars)[:4] == list(f.level_npars)[:4]
    np.testing.assert_allclose(bed.setup.rad, w.setup.rad, rtol=4e-16, atol=0)
    assert np.array_equal(bed.setup.plevel, w.setup.plevel) and np.array_equal(bed.setup.nidx, w.setup.nidx)
    assert s.prm.dt == f.prm.dt and s.force_cap == 1 and s.lqd.stension == f.lqd.stension
    pos = bed.pos0_reduced
    r = bed.setup.rad
    cyl = s.cyl
    # inside the cylinder, up to the contact overlaps under the bed's weight (~µm: 1e-2 reduced units is 20 µm)
    assert (np.hypot(pos[:, 0] - cyl.cir_x, pos[:, 1] - cyl.cir_y) + r <= cyl.R + 1e-2).all()
    assert (pos[:, 2] - r >= cyl.Bw - 1e-2).all() and (pos[:, 2] + r <= cyl.Tw).all()
    m = packing_metrics(bed.setup, pos)
    assert m["phi"] > 0.6 and m["z"] > 6.0, m
