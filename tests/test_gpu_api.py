"""Simulation.run() through the opengate-shaped API on the GPU, checked against the oracle."""

import numpy as np
import pytest

import opengate_gb300 as gate

from .test_cpu_api import water_sim

pytestmark = pytest.mark.gpu


def test_simulation_run_matches_oracle_and_writes_outputs(tmp_path, built_lib):
    from oracle import oracle as O

    n = 20000
    sim = water_sim(tmp_path, n=n)
    sim.run()
    dose = sim.actors["dose"]
    stats = sim.actors["stats"]
    scene, *_ = sim.build_scene()
    e, e2, cnt = O.run_dose(scene, n, sim.last_seed)
    assert np.array_equal(dose.edep.get_data().array, e)
    assert np.array_equal(dose.edep_squared.get_data().array, e2)
    assert dose.number_of_samples == n
    assert stats.counts.events == n and stats.counts.steps == cnt["woodcock_steps"] + cnt["world_steps"]
    for out in (dose.edep, dose.edep_uncertainty, dose.dose, dose.dose_uncertainty):
        p = out.get_output_path()
        assert p.exists(), p
        back = gate.read_mhd(p)
        np.testing.assert_array_equal(back.array, out.get_data().array)
    unc = dose.edep_uncertainty.get_data().array
    assert np.all((unc >= 0) & (unc <= 1.0 + 1e-12))
    # dose uncertainty equals edep uncertainty when the dose grid is the image grid
    np.testing.assert_allclose(dose.dose_uncertainty.get_data().array, unc, rtol=1e-12, atol=1e-15)
