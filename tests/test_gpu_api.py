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


def test_uncertainty_goal_stops_early(tmp_path, built_lib):
    """DoseActor.uncertainty_goal: the run stops once the mean uncertainty of the high-dose voxels
    reaches the goal; the images equal the oracle's for the events simulated."""
    from oracle import oracle as O

    sim = water_sim(tmp_path, n=2_000_000)
    dose = sim.actors["dose"]
    dose.uncertainty_goal = 0.05
    dose.uncertainty_first_check_after_n_events = 20_000
    sim.run()
    n = dose.number_of_samples
    assert 20_000 <= n < 2_000_000
    edep = dose.edep.get_data().array
    e2 = dose.edep_squared.get_data().array
    from opengate_gb300 import dose as D

    assert D.compute_mean_uncertainty(edep, e2, n) <= 0.05
    # the run went in chunks between the checks: the oracle replays the same chunks
    scene, *_ = sim.build_scene()
    e = np.zeros_like(edep)
    e2o = np.zeros_like(e2)
    done = 0
    for upto, _ in dose.uncertainty_checks:
        a, b, _ = O.run_dose(scene, upto - done, sim.last_seed, first=done, threads=8)
        e += a
        e2o += b
        done = upto
    assert done == n and len(dose.uncertainty_checks) >= 2
    assert np.array_equal(edep, e) and np.array_equal(e2, e2o)


def test_spect_simulation_matches_oracle(tmp_path, built_lib):
    """SPECT through the API (contrib helpers, VoxelSource, projection actors) equals the oracle."""
    from oracle import oracle as O

    from .test_cpu_api_spect import spect_sim

    sim, heads = spect_sim(tmp_path, n_per_run=300_000, angles=3)
    sim.random_seed = 4321
    sim.run()
    scene, sp, sources, projs, head_of = sim.build_spect()
    ref, _ = O.run_spect(scene, sp, 300_000, 4321, threads=8)
    for head, digi in heads:
        proj = digi.projection.counts.get_data().array
        np.testing.assert_array_equal(proj, ref[head_of[digi.projection.attached_to]])
        assert digi.projection.counts.get_output_path().exists()
    assert ref.sum() > 0


def test_free_flight_recipe_through_the_api(tmp_path, built_lib):
    """The reference's free-flight recipe through the API: a primary simulation
    (GammaFreeFlightActor) and a scatter simulation (ScatterSplittingFreeFlightActor) write
    projection_<h>_counts / _squared_counts per component; spect_freeflight_helpers merges
    them; each component equals its oracle run bit for bit."""
    from oracle import oracle as O

    from opengate_gb300 import image_io
    from opengate_gb300.contrib.spect import spect_freeflight_helpers as ffh

    from .test_cpu_api_spect import spect_sim

    n = 200_000
    for sub, kind in (("primary", "GammaFreeFlightActor"), ("scatter", "ScatterSplittingFreeFlightActor")):
        sim, heads = spect_sim(tmp_path / sub, n_per_run=n, angles=2)
        sim.random_seed = 99
        for h, (head, digi) in enumerate(heads):
            digi.projection.output_filename = f"projection_{h}.mhd"
            digi.projection.squared_counts.active = True
        ff = sim.add_actor(kind, "ff")
        ff.exclude_volumes = [head.name for head, _ in heads]
        if kind == "ScatterSplittingFreeFlightActor":
            ff.kill_interacting_in_volumes = [head.name for head, _ in heads]
            ff.compton_splitting_factor = 20
            ff.rayleigh_splitting_factor = 5
        sim.run()
        scene, sp, _, _, head_of = sim.build_spect()
        w, w2, _ = O.run_spect_ff(scene, sp, n, 99, threads=8)
        for h, (head, digi) in enumerate(heads):
            got = image_io.read_mhd(tmp_path / sub / f"projection_{h}_counts.mhd").array
            got2 = image_io.read_mhd(tmp_path / sub / f"projection_{h}_squared_counts.mhd").array
            k = head_of[digi.projection.attached_to]
            np.testing.assert_array_equal(got, w[k].astype(got.dtype))
            np.testing.assert_array_equal(got2, w2[k].astype(got2.dtype))
    merged = ffh.merge_freeflight_uncertainty_for_all_heads(tmp_path, 2 * n, ["primary", "scatter"], [2 * n, 2 * n], 2)
    for counts, unc in merged:
        assert counts.array.sum() > 0 and np.all(unc.array >= 0)
