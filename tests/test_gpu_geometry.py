"""Gradient-driven geometry optimisation (HFBuilder.buildOtimizer mirror) on
the GPU: BFGS with the analytic gradient must reach a stationary point
(max|g| < 1e-4 Eh/bohr) whose energy is below the start and matches the
known RHF/STO-3G water minimum (-74.9659 Eh) within 1e-4 Eh."""
import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry

pytestmark = pytest.mark.gpu
E_STO3G_WATER_MIN = -74.9659


def _distorted_water():
    return [(z, x * 1.08 + 0.02 * i, y * 0.95, w + 0.01 * i) for i, (z, x, y, w) in enumerate(geometry.water())]


def test_bfgs_reaches_stationary_point(built_library, cuda):
    atoms = _distorted_water()
    e0, g0 = gg.energy_and_gradient_at(atoms, gg.basis_path("sto-3g"), {"convergence_threshold": 1e-10})
    e, final, hist = gg.optimize_geometry(atoms, gg.basis_path("sto-3g"), {"convergence_threshold": 1e-10})
    assert np.abs(g0).max() > 1e-2
    assert e < e0
    assert hist[-1][1] < 1e-4
    assert abs(e - E_STO3G_WATER_MIN) < 1e-4
    # the first atom stays where it was
    assert np.allclose(final[0][1:], atoms[0][1:])


def test_build_optimizer_recipe(built_library, cuda, tmp_path):
    xyz = tmp_path / "w.xyz"
    geometry.write_xyz(xyz, _distorted_water())
    pm = gg.ParameterManager()
    pm["xyzfilename"] = str(xyz)
    pm["gbsfilename"] = str(gg.basis_path("sto-3g"))
    e = gg.HFBuilder.buildOtimizer(pm)
    assert abs(e - E_STO3G_WATER_MIN) < 1e-4
