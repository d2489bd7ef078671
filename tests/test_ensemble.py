"""Batched ensembles and the cell-size knob on the CPU: the layout keeps the
systems apart and inside their own cylinders; larger cells rederive the grids."""
import copy

import numpy as np

import _workloads
from gpucode_gb300 import configs


def test_ensemble_layout_separates_the_systems():
    from scipy.spatial import cKDTree

    e = configs.ensemble(n_systems=8, n_range=(300, 1500), seed=5, threads=4)
    comb = e.combined
    assert comb.setup.n == sum(m.inp.np for m in e.members) == len(e.system)
    assert set(np.unique(e.system)) == set(range(8))
    assert e.wet.tolist() == [0, 1] * 4
    # no pair of particles from two systems within twice the largest diameter
    t = cKDTree(comb.pos0)
    pairs = t.query_pairs(2 * comb.dia.max(), output_type="ndarray")
    assert (e.system[pairs[:, 0]] == e.system[pairs[:, 1]]).all()
    p = comb.pos0_reduced
    for k, c in enumerate(e.cylinders):
        idx = e.system == k
        r = np.hypot(p[idx, 0] - c.cir_x, p[idx, 1] - c.cir_y) + comb.setup.rad[idx]
        assert (r <= c.R * (1 + 1e-9)).all()
        assert (p[idx, 2] + comb.setup.rad[idx] <= c.Tw).all()
        # the member alone: the same spheres, centred on its own axis
        m = e.members[k]
        np.testing.assert_allclose(m.pos0[:, :2] + e.offsets[k], comb.pos0[idx, :2], rtol=0, atol=1e-15)
        np.testing.assert_array_equal(m.dia, comb.dia[idx])
    # every system's container lies inside the combined computing zone
    s = comb.setup.s
    for c in e.cylinders:
        assert s.prm.Origin.x <= c.cir_x - c.R and c.cir_x + c.R <= s.prm.EndPoint.x
        assert s.prm.Origin.y <= c.cir_y - c.R and c.cir_y + c.R <= s.prm.EndPoint.y


def test_scale_cells_rederives_the_grids():
    w = _workloads.small_wet()
    st = copy.deepcopy(w.setup)
    st.scale_cells(1.5)
    a, b = w.setup.s, st.s
    total = 0
    for i in range(a.n_levels):
        assert abs(b.cell_size[i] - 1.5 * a.cell_size[i]) < 1e-15
        for ax in ("x", "y", "z"):
            ext = getattr(a.prm.EndPoint, ax) - getattr(a.prm.Origin, ax)
            assert getattr(b.grid_size[i], ax) == int(np.ceil(ext / b.cell_size[i]))
            assert getattr(b.grid_size[i], ax) <= getattr(a.grid_size[i], ax)
        total += b.num_cells[i]
        assert b.ncell_idx[i] == total
    assert b.sys_ncells == total < a.sys_ncells
    same = copy.deepcopy(w.setup)
    same.scale_cells(1.0)
    assert same.s.sys_ncells == a.sys_ncells
