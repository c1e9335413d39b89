"""opengate-shaped API on the CPU: activity-driven primaries, uncertainty goal, SPECT set-up."""

import math

import numpy as np
import pytest

import opengate_gb300 as gate
from opengate_gb300 import api as A
from opengate_gb300 import dose as D
from opengate_gb300 import units as U
from opengate_gb300.contrib.spect import ge_discovery_nm670 as nm670
from opengate_gb300.contrib.spect import spect_helpers

u = U.g4_units


def test_expected_number_of_events():
    # GateVSource::GetExpectedNumberOfEvents: round(A dt), or with decay A/l (e^-l t0 - e^-l t1)
    assert A.expected_number_of_events(1000.0, None, 0.0, 2.5) == 2500
    hl = 6.0
    lam = math.log(2) / hl
    assert A.expected_number_of_events(1000.0, hl, 1.0, 3.0) == round(1000.0 / lam * (math.exp(-lam) - math.exp(-3 * lam)))


def _source(sim, **kw):
    s = sim.add_source("GenericSource", "src")
    s.particle = "gamma"
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def test_events_per_run_from_activity_and_n():
    sim = gate.Simulation()
    sim.run_timing_intervals = [[0, 1 * u.s], [1 * u.s, 3 * u.s]]
    s = _source(sim, activity=2000 * u.Bq)
    s.energy.type = "spectrum_discrete"
    s.energy.spectrum_energies = [0.113, 0.208]
    s.energy.spectrum_weights = [0.062, 0.104]  # yield 0.166: activity x 0.166
    rng = np.random.default_rng(1)
    draws = np.array([A.events_per_run(s, sim.run_timing_intervals, rng) for _ in range(400)])
    expect = np.array([2000 * 0.166 * 1, 2000 * 0.166 * 2])
    np.testing.assert_allclose(draws.mean(axis=0), expect, rtol=0.03)
    np.testing.assert_allclose(draws.var(axis=0), expect, rtol=0.2)  # Poisson
    s2 = _source(gate.Simulation(), n=[5, 7])
    assert A.events_per_run(s2, [[0, 1], [1, 2]], rng) == [5, 7]
    s3 = _source(gate.Simulation(), n=9)
    assert A.events_per_run(s3, [[0, 1], [1, 2], [2, 3]], rng) == [9, 9, 9]


def test_mean_uncertainty_criterion():
    rng = np.random.default_rng(2)
    n = 1000
    e = rng.gamma(2.0, 1.0, size=(8, 9, 10))
    e2 = e * e / n * 1.5 + 1e-3
    top = np.sort(e.ravel())[-10:].mean()
    sel = e > 0.7 * top
    val = e[sel] / n
    unc = np.sqrt(np.clip((e2[sel] / n - val ** 2) / (n - 1), 0, None)) / val
    expect = float(np.minimum(unc, 1.0).mean())
    assert D.compute_mean_uncertainty(e, e2, n) == pytest.approx(expect, rel=1e-12)
    assert D.compute_mean_uncertainty(np.zeros((2, 2, 2)), np.zeros((2, 2, 2)), n) == 1.0
    assert D.next_uncertainty_check(0.2, 0.1, 1000, 1.05) == int(4 * 1000 * 1.05)


def test_precision_error_statement():
    rng = np.random.default_rng(3)
    n = 1000
    # per-history values: sum and sum of squares of n draws per voxel
    h = rng.exponential(1.0, size=(n, 200))
    e, e2 = h.sum(0), (h * h).sum(0)
    same = D.precision_error(e, e2, e.copy(), e2.copy(), n)
    assert same["integral_rel"] == 0 and same["equal"] == 1.0 and same["within_2sigma"] == 1.0
    assert same["max_z"] == 0.0
    # one voxel shifted by 3 combined sigma, one by a rounding-sized amount
    sig = np.sqrt(2 * (e2 - e * e / n) * n / (n - 1))
    f = e.copy()
    f[0] += 3 * sig[0]
    f[1] *= 1 + 1e-12
    err = D.precision_error(f, e2, e, e2, n, threshold=0.0)
    assert err["voxels"] == 200
    va = np.clip(e2[0] - f[0] ** 2 / n, 0, None) * n / (n - 1)
    vb = (e2[0] - e[0] ** 2 / n) * n / (n - 1)
    assert err["max_z"] == pytest.approx(3 * sig[0] / np.sqrt(va + vb), rel=1e-9)
    assert err["within_2sigma"] == pytest.approx(199 / 200)
    assert err["equal"] == pytest.approx(198 / 200)
    assert err["integral_rel"] == pytest.approx((f.sum() - e.sum()) / e.sum(), rel=1e-9)


def spect_sim(tmp_path, n_per_run=1000, angles=3):
    sim = gate.Simulation()
    sim.output_dir = tmp_path
    sim.world.size = [2 * u.m] * 3
    sim.world.material = "G4_AIR"
    sim.physics_manager.physics_list_name = "G4EmStandardPhysics"
    sim.physics_manager.set_min_ekine("world", 1 * u.MeV)
    sim.physics_manager.set_user_limits_particles(["e-", "e+"])
    img = sim.add_volume("Image", "ct")
    hu = np.full((20, 32, 32), -1000, np.int16)
    hu[4:16, 8:24, 8:24] = 0
    img.image = gate.Image(hu, spacing=(6.0, 6.0, 6.0))
    img.material = "G4_AIR"
    img.voxel_materials = [[-1100, -500, "G4_AIR"], [-500, 1000, "G4_WATER"]]
    heads = []
    for i, start in enumerate((0, 180)):
        head, _, crystal = nm670.add_spect_head(sim, f"spect{i}", "lehr")
        nm670.rotate_gantry(head, 25 * u.cm, start, 120, angles)
        d = nm670.add_digitizer(sim, crystal.name, channels=spect_helpers.get_default_energy_windows("tc99m"),
                                size=[64, 64], spacing=[8.84 * u.mm] * 2)
        heads.append((head, d))
    act = np.zeros((20, 32, 32))
    act[6:14, 12:20, 12:20] = 1.0
    src = sim.add_source("VoxelSource", "act")
    src.particle = "gamma"
    src.image = gate.Image(act, spacing=(6.0, 6.0, 6.0))
    src.energy.type = "mono"
    src.energy.mono = 140.5 * u.keV
    src.n = n_per_run
    sim.run_timing_intervals = [[k * u.s, (k + 1) * u.s] for k in range(angles)]
    return sim, heads


def test_spect_setup_from_the_helpers(tmp_path):
    sim, heads = spect_sim(tmp_path)
    scene, sp, sources, projs, head_of = sim.build_spect()
    assert sp.n_heads == 2 and sp.n_runs == 3 and sp.n_windows == 2
    assert sp.windows[1] == pytest.approx((0.12959, 0.15061))
    assert [round(math.degrees(sp.angle(r, h))) for r in range(3) for h in range(2)] == [0, 180, 120, 300, 240, 420]
    assert sp.collimator_thickness == 35.0 and sp.crystal_thickness == pytest.approx(9.525)
    fr = sp.frames(1)
    np.testing.assert_allclose(np.linalg.norm(fr[0, :3]), 250.0)
    spec = sources[0][1]
    assert spec.pos_type == 4 and spec.vox_dims == [32, 32, 20]
    np.testing.assert_allclose(spec.vox_corner, [-96.0, -96.0, -60.0])
    assert head_of == {"spect0_crystal": 0, "spect1_crystal": 1}
    assert len(scene.pt.mat_rho) >= 4 and sp.collimator_material != sp.crystal_material


def test_digitizer_chain_sets_blur_and_adder(tmp_path):
    from opengate_gb300 import _capi as C
    from opengate_gb300.contrib.spect import siemens_intevo as intevo

    sim, _ = spect_sim(tmp_path)
    _, sp, _, _, _ = sim.build_spect()
    # the NM670 chain: energy winner, 6.3 % FWHM at 140.57 keV, 3 mm FWHM kept in the crystal
    assert sp.adder_policy == "EnergyWinnerPosition"
    assert sp.blur.energy_method == C.GG_BLUR_INVERSE_SQUARE
    assert sp.blur.energy_resolution == pytest.approx(0.063) and sp.blur.energy_reference == pytest.approx(0.14057)
    assert sp.blur.spatial == 1 and sp.blur.keep_in_solid_limits == 1 and sp.blur.truncated == 0
    assert sp.blur.spatial_sigma[0] == pytest.approx(3.0 / 2.3548200450309493)
    # the Intevo chain: centroid adder, 9.9 % at 140.5 keV, 3.6 mm
    sim2 = gate.Simulation()
    sim2.output_dir = tmp_path
    head, _, crystal = intevo.add_spect_head(sim2, "intevo", "melp")
    intevo.add_digitizer(sim2, crystal.name)
    actors = {a.type_name for a in sim2.actors.values()}
    assert {"DigitizerAdderActor", "DigitizerBlurringActor", "DigitizerSpatialBlurringActor",
            "DigitizerProjectionActor"} <= actors
    adder = [a for a in sim2.actors.values() if a.type_name == "DigitizerAdderActor"][0]
    assert adder.adder_policy() == "EnergyWeightedCentroidPosition"
    eb = [a for a in sim2.actors.values() if a.type_name == "DigitizerBlurringActor"][0]
    assert eb.energy_blur() == dict(method="InverseSquare", resolution=0.099, reference=pytest.approx(0.1405),
                                    slope=0.0)
    sb = [a for a in sim2.actors.values() if a.type_name == "DigitizerSpatialBlurringActor"][0]
    assert sb.spatial_blur()["sigma"][0] == pytest.approx(3.6 / 2.3548200450309493)


def test_blur_actor_validation():
    b = gate.Simulation().add_actor("DigitizerBlurringActor", "eb")
    b.blur_attribute = "TotalEnergyDeposit"
    with pytest.raises(ValueError):
        b.energy_blur()  # Gaussian without sigma or fwhm
    b.blur_fwhm = 0.01
    assert b.energy_blur()["sigma"] == pytest.approx(0.01 / 2.3548200450309493)
    b.blur_sigma = 0.002
    with pytest.raises(ValueError):
        b.energy_blur()  # both
    b.blur_attribute = "GlobalTime"
    with pytest.raises(NotImplementedError):
        b.energy_blur()


def test_free_flight_actors_set_the_modes(tmp_path):
    """GammaFreeFlightActor -> primary free flight; ScatterSplittingFreeFlightActor ->
    scatter splitting with its factors (-1 = splitting_factor), level and angle check."""
    from opengate_gb300 import _capi as C

    sim, heads = spect_sim(tmp_path)
    ff = sim.add_actor("GammaFreeFlightActor", "ff")
    ff.exclude_volumes = [h.name for h, _ in heads]
    _, sp, _, _, _ = sim.build_spect()
    assert sp.free_flight.enabled == C.FF_PRIMARY
    sim.actors.pop("ff")
    ss = sim.add_actor("ScatterSplittingFreeFlightActor", "ss")
    ss.exclude_volumes = [h.name for h, _ in heads]
    with pytest.raises(NotImplementedError):
        sim.build_spect()  # the heads must be kill volumes
    ss.kill_interacting_in_volumes = [f"{h.name}_crystal" for h, _ in heads]
    ss.splitting_factor = 7
    ss.rayleigh_splitting_factor = 3
    ss.max_compton_level = 4
    ss.weight_cutoff = 1e-9
    ss.angular_acceptance.policy = "Rejection"
    ss.angular_acceptance.enable_intersection_check = True
    ss.angular_acceptance.enable_angle_check = True
    ss.angular_acceptance.angle_tolerance_max = 10 * u.deg
    _, sp, _, _, _ = sim.build_spect()
    f = sp.free_flight
    assert (f.enabled, f.compton_splitting, f.rayleigh_splitting, f.max_compton_level) == (C.FF_SCATTER, 7, 3, 4)
    assert f.weight_cutoff == 1e-9 and f.angle_tolerance_max == pytest.approx(math.radians(10))
    ss.angular_acceptance.angle_tolerance_min = 1 * u.deg
    with pytest.raises(NotImplementedError):
        sim.build_spect()
    ss.angular_acceptance.angle_tolerance_min = 0.0
    sim.add_actor("GammaFreeFlightActor", "ff2").exclude_volumes = [h.name for h, _ in heads]
    with pytest.raises(NotImplementedError):
        sim.build_spect()  # one free-flight actor


def test_scatter_splitting_arguments():
    from opengate_gb300 import spect as S

    sp = S.SpectSpec()
    with pytest.raises(ValueError):
        sp.set_scatter_splitting(-1, 2)
    with pytest.raises(ValueError):
        sp.set_scatter_splitting(5000, 2)
    with pytest.raises(ValueError):
        sp.set_scatter_splitting(5, 2, max_compton_level=-1)
    sp.set_scatter_splitting(5, 2)
    assert sp.free_flight.max_compton_level == 10


def test_projection_output_names_follow_the_reference(tmp_path):
    """output_filename 'projection_1_ffa.mhd' -> projection_1_ffa_counts.mhd and, with
    squared_counts.active, projection_1_ffa_squared_counts.mhd."""
    sim, heads = spect_sim(tmp_path)
    proj = heads[0][1].projection
    proj.output_filename = "projection_1_ffa.mhd"
    proj.squared_counts.active = True
    assert proj.counts.get_output_path() == tmp_path / "projection_1_ffa_counts.mhd"
    assert proj.squared_counts.get_output_path() == tmp_path / "projection_1_ffa_squared_counts.mhd"
    assert proj.counts_squared is proj.squared_counts


def test_merge_freeflight_uncertainty(tmp_path):
    """Primary + scatter components merged as the reference's helper does: means add, the
    variances of the means add; files written with the reference's names."""
    from opengate_gb300 import image_io
    from opengate_gb300.contrib.spect import spect_freeflight_helpers as ffh

    rng = np.random.default_rng(3)
    shape = (2, 4, 5)
    comps = {"primary": 1000, "scatter": 400, "skipped": 1}
    cs, c2s = {}, {}
    for name, n in comps.items():
        c = rng.uniform(0.0, 5.0, shape)
        c2 = c * rng.uniform(0.05, 0.5, shape)
        cs[name], c2s[name] = c, c2
        for h in range(2):
            image_io.write_mhd(tmp_path / name / f"projection_{h}_counts.mhd", image_io.Image(c * (h + 1), [2, 2, 1]))
            image_io.write_mhd(tmp_path / name / f"projection_{h}_squared_counts.mhd",
                               image_io.Image(c2 * (h + 1), [2, 2, 1]))
    out = ffh.merge_freeflight_uncertainty_for_all_heads(tmp_path, 5000, list(comps), list(comps.values()), 2)
    e = sum(cs[k] / n for k, n in comps.items() if n > 1)
    v = sum(np.clip((c2s[k] / n - (cs[k] / n) ** 2) / (n - 1), 0, None) for k, n in comps.items() if n > 1)
    np.testing.assert_allclose(out[0][0].array, e * 5000, rtol=1e-12)
    np.testing.assert_allclose(out[0][1].array, np.sqrt(v) / e, rtol=1e-12)
    h1 = image_io.read_mhd(tmp_path / "projection_1_counts.mhd").array
    np.testing.assert_allclose(h1, 2 * e * 5000, rtol=1e-6)
    assert (tmp_path / "relative_uncertainty_1_counts.mhd").exists()
    with pytest.raises(ValueError):
        ffh.merge_freeflight_uncertainty(tmp_path, 1, ["primary"], [1000, 2])
