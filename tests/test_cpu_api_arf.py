"""ARF workflow on the opengate-shaped API, host side (no GPU).

Covers the dataset and network files (round trip, garf .pth names refused),
the ARFActor / ARFTrainingDatasetActor configuration checks of the reference
(arfactors.py:19-30 channel overlap, 147-226 user info), and how an ARF
acquisition is set up from a network file: its windows, adder and blurring
come from the network, its image size and spacing from the actor.
"""

import numpy as np
import pytest

import opengate_gb300 as gate
from opengate_gb300 import _capi as C
from opengate_gb300 import arf as ARF
from opengate_gb300 import spect as S
from opengate_gb300 import units as U
from opengate_gb300.contrib.spect import ge_discovery_nm670 as nm670

u = U.g4_units
LU177 = [{"name": "peak208", "min": 187.2 * u.keV, "max": 228.8 * u.keV},
         {"name": "scatter", "min": 166.0 * u.keV, "max": 187.0 * u.keV},
         {"name": "peak113", "min": 101.7 * u.keV, "max": 124.3 * u.keV}]


def _meta(coll="melp", blur=True):
    sp = S.SpectSpec(collimator=S.COLLIMATORS[coll], n_heads=1, n_runs=1,
                     windows=[(c["min"] / u.MeV, c["max"] / u.MeV) for c in LU177])
    if blur:
        sp.set_energy_blur("InverseSquare", resolution=0.1, reference=0.208)
        sp.set_spatial_blur(1.5, keep_in_solid_limits=True)
    sp.housing = "nm670"  # a network of the NM670 head (the contrib helpers build its housing)
    return ARF.head_meta(sp, coll, "3/8")


def _model_file(path, coll="melp"):
    m = C.ArfModel()
    m.n_classes = 4
    m.x_mean[:] = [40.0, 0.0, 0.15]
    m.x_std[:] = [20.0, 100.0, 0.03]
    m.russian_roulette, m.e_min, m.e_max, m.theta_max_deg, m.distance_to_crystal = 40.0, 0.1, 0.21, 80.0, 45.4
    params = np.random.default_rng(1).normal(size=C.GG_ARF_N_PARAMS).astype(np.float32)
    ARF.save_model(path, m, params, _meta(coll))
    return m, params


def test_dataset_and_model_files_round_trip(tmp_path):
    rows = np.random.default_rng(0).random((1000, 4)).astype(np.float32)
    rows[:, 3] = np.floor(rows[:, 3] * 4)
    meta = _meta()
    p = ARF.save_dataset(tmp_path / "d.npz", rows, meta, 0.1, 0.21, 80.0, 40.0)
    r2, m2, dom = ARF.load_dataset(p)
    np.testing.assert_array_equal(rows, r2)
    assert dom == {"e_min": 0.1, "e_max": 0.21, "theta_max_deg": 80.0, "russian_roulette": 40.0}
    assert m2["collimator_type"] == "melp" and np.allclose(m2["windows"], meta["windows"])
    with np.load(p) as z:  # the reference's attribute names
        assert set(("E", "Theta", "Phi", "window")) <= set(z.files)
    m, params = _model_file(tmp_path / "m.npz")
    m3, p3, meta3 = ARF.load_model(tmp_path / "m.npz")
    np.testing.assert_array_equal(params, p3)
    assert m3.n_classes == 4 and list(m3.x_std) == pytest.approx(list(m.x_std))
    assert m3.distance_to_crystal == pytest.approx(45.4)
    sp = S.SpectSpec(n_heads=1, n_runs=1)
    ARF.apply_head_meta(sp, meta3)
    assert sp.n_windows == 3 and sp.blur.energy_method == C.GG_BLUR_INVERSE_SQUARE
    assert sp.blur.spatial == 1 and sp.blur.spatial_sigma[0] == pytest.approx(1.5)
    for bad in ("net.pth", "rows.root"):
        with pytest.raises(NotImplementedError):
            ARF.load_model(tmp_path / bad)


def _arf_sim(tmp_path, model_path, n=1000, angles=2):
    sim = gate.Simulation()
    sim.output_dir = tmp_path
    sim.world.size = [2 * u.m] * 3
    sim.physics_manager.physics_list_name = "G4EmStandardPhysics"
    sim.physics_manager.set_min_ekine("world", 1 * u.MeV)
    sim.physics_manager.set_user_limits_particles(["e-", "e+"])
    img = sim.add_volume("Image", "ct")
    hu = np.full((10, 16, 16), -1000, np.int16)
    hu[2:8, 4:12, 4:12] = 0
    img.image = gate.Image(hu, spacing=(8.0, 8.0, 8.0))
    img.material = "G4_AIR"
    img.voxel_materials = [[-1100, -500, "G4_AIR"], [-500, 1000, "G4_WATER"]]
    dets = []
    for i, start in enumerate((0, 180)):
        plane, arf = nm670.add_arf_detector(sim, f"arf{i}", "melp", [64, 64], [8.84 * u.mm] * 2, model_path)
        nm670.rotate_gantry(plane, 25 * u.cm, start, 90, angles)
        dets.append((plane, arf))
    src = sim.add_source("GenericSource", "s")
    src.particle = "gamma"
    src.position.type = "sphere"
    src.position.radius = 20 * u.mm
    src.direction.type = "iso"
    src.energy.type = "mono"
    src.energy.mono = 208 * u.keV
    src.n = n
    sim.run_timing_intervals = [[k * u.s, (k + 1) * u.s] for k in range(angles)]
    return sim, dets


def test_arf_acquisition_takes_windows_and_digitizer_from_the_network(tmp_path):
    m, _ = _model_file(tmp_path / "net.npz")
    sim, dets = _arf_sim(tmp_path, tmp_path / "net.npz")
    scene, sp, sources, arfs, head_of = sim.build_spect()
    assert sp.n_heads == 2 and sp.n_runs == 2 and sp.n_windows == 3
    assert sp.windows[0] == pytest.approx((0.1872, 0.2288))
    assert sp.size == [64, 64] and sp.spacing == pytest.approx([8.84, 8.84])
    assert sp.blur.energy_method == C.GG_BLUR_INVERSE_SQUARE and sp.blur.spatial == 1
    assert sp.collimator_thickness == pytest.approx(40.6)
    model, params, meta = sp.arf
    # add_arf_detector's depth: collimator + the housing's aluminium cover + half the crystal
    assert model.distance_to_crystal == pytest.approx(40.6 + 1.3 + 9.525 / 2)
    assert sp.housing == "nm670" and sp.desc().n_back == 4 and sp.desc().shielded_sides == 1
    assert head_of == {"arf0": 0, "arf1": 1} and [a.name for a in arfs] == ["arf0_arf", "arf1_arf"]


@pytest.mark.parametrize("option,value", [("flip_plane", True), ("enable_hit_slice", True),
                                          ("plane_axis", [1, 0, 2]), ("gpu_mode", "cpu")])
def test_arf_actor_unsupported_options_raise(tmp_path, option, value):
    _model_file(tmp_path / "net.npz")
    sim, dets = _arf_sim(tmp_path, tmp_path / "net.npz")
    setattr(dets[0][1], option, value)
    with pytest.raises(NotImplementedError):
        sim.build_spect()


def test_arf_network_must_match_the_heads(tmp_path):
    _model_file(tmp_path / "lehr.npz", coll="lehr")
    sim, _ = _arf_sim(tmp_path, tmp_path / "lehr.npz")
    with pytest.raises(ValueError, match="trained for a lehr"):
        sim.build_spect()
    sim, dets = _arf_sim(tmp_path, tmp_path / "garf.pth")
    with pytest.raises(NotImplementedError, match="pth"):
        sim.build_spect()


def _dataset_sim(tmp_path, channels=LU177, rr=20):
    sim = gate.Simulation()
    sim.output_dir = tmp_path
    sim.world.size = [2 * u.m] * 3
    sim.physics_manager.physics_list_name = "G4EmStandardPhysics"
    sim.physics_manager.set_min_ekine("world", 1 * u.MeV)
    sim.physics_manager.set_user_limits_particles(["e-", "e+"])
    head, _, crystal = nm670.add_spect_head(sim, "spect", "melp")
    cc = nm670.add_digitizer_energy_windows(sim, crystal.name, channels)
    plane, actor = nm670.add_actor_for_arf_training_dataset(sim, "melp", cc, rr)
    src = nm670.add_source_for_arf_training_dataset(sim, "train", 1e5 * u.Bq, plane, 100 * u.keV, 230 * u.keV)
    return sim, plane, actor, src


def test_training_dataset_checks_and_domain(tmp_path):
    sim, plane, actor, src = _dataset_sim(tmp_path)
    assert actor.energy_windows_actor == "EnergyWindows_spect_crystal"
    assert actor.output_filename == "arf_training_dataset.npz" and actor.russian_roulette == 20
    # the disc (5 cm) sits 5 cm in front of the plane (25 cm from the axis): wide angles
    th = sim._arf_theta_max(actor, plane, src)
    assert 80.0 < th <= 89.0
    actor.theta_max_deg = 60.0
    assert sim._arf_theta_max(actor, plane, src) == 60.0
    # overlapping windows are refused (arfactors.py:111-124)
    over = [dict(c) for c in LU177]
    over[1]["max"] = 200 * u.keV
    sim2, _, _, _ = _dataset_sim(tmp_path, channels=over)
    with pytest.raises(ValueError, match="overlap"):
        sim2.run()
    sim3, _, actor3, _ = _dataset_sim(tmp_path)
    actor3.energy_windows_actor = "nope"
    with pytest.raises(ValueError, match="energy_windows_actor"):
        sim3.run()


def test_digitizer_has_an_energy_windows_module(tmp_path):
    sim = gate.Simulation()
    head, _, crystal = nm670.add_spect_head(sim, "spect", "lehr")
    d = nm670.add_digitizer(sim, crystal.name)
    ew = d.find_module("energy_window")
    assert ew.type_name == "DigitizerEnergyWindowsActor" and ew.channels == d.projection.channels


def _ff_arf_sim(tmp_path, model_path, deg=10.0, n=1000):
    """The reference's primary free-flight recipe (spect_config.py:937-970) with ARF detectors:
    GammaFreeFlightActor on the world with the detection planes excluded, the source's angular
    acceptance with the intersection and angle checks against the planes."""
    sim, dets = _arf_sim(tmp_path, model_path, n=n)
    ff = sim.add_actor("GammaFreeFlightActor", "ff")
    ff.attached_to = "world"
    ff.exclude_volumes = [p.name for p, _ in dets]
    aa = sim.sources["s"].direction.angular_acceptance
    aa.policy = "Rejection"
    aa.skip_policy = "SkipEvents"
    aa.target_volumes = [p.name for p, _ in dets]
    aa.enable_intersection_check = True
    aa.enable_angle_check = True
    aa.angle_tolerance_max = deg * u.deg
    return sim, dets


def test_free_flight_with_arf_detectors_maps_to_the_engine(tmp_path):
    _model_file(tmp_path / "net.npz")
    sim, dets = _ff_arf_sim(tmp_path, tmp_path / "net.npz", deg=12.0)
    scene, sp, sources, arfs, head_of = sim.build_spect()
    assert sp.arf is not None and sp.free_flight.enabled == C.FF_PRIMARY
    assert sp.free_flight.angle_tolerance_max == pytest.approx(np.radians(12.0))
    assert sources[0][1].accept_boxes == []  # the acceptance is the free flight's own
    # scatter splitting with ARF detectors
    sim2, dets2 = _arf_sim(tmp_path / "b", tmp_path / "net.npz")
    ss = sim2.add_actor("ScatterSplittingFreeFlightActor", "ss")
    ss.exclude_volumes = ss.kill_interacting_in_volumes = [p.name for p, _ in dets2]
    ss.compton_splitting_factor, ss.rayleigh_splitting_factor = 8, 2
    ss.angular_acceptance.policy = "Rejection"
    ss.angular_acceptance.enable_angle_check = True
    ss.angular_acceptance.angle_tolerance_max = 20 * u.deg
    _, sp2, *_ = sim2.build_spect()
    assert sp2.arf is not None and sp2.free_flight.enabled == C.FF_SCATTER
    assert (sp2.free_flight.compton_splitting, sp2.free_flight.rayleigh_splitting) == (8, 2)
    # an angle check without free flight is still refused
    sim3, _ = _arf_sim(tmp_path / "c", tmp_path / "net.npz")
    aa = sim3.sources["s"].direction.angular_acceptance
    aa.policy, aa.enable_intersection_check, aa.enable_angle_check = "Rejection", True, True
    with pytest.raises(NotImplementedError):
        sim3.build_spect()


def test_force_direction_policy_maps_to_forced_sources(tmp_path):
    """angular_acceptance.policy = "ForceDirection" with a GammaFreeFlightActor (the reference's
    setup_force_direction): the source aims each history at a head within the cone."""
    _model_file(tmp_path / "net.npz")
    sim, dets = _ff_arf_sim(tmp_path, tmp_path / "net.npz")
    aa = sim.sources["s"].direction.angular_acceptance
    aa.policy = "ForceDirection"
    aa.angle_tolerance_max = 8 * u.deg
    scene, sp, sources, arfs, head_of = sim.build_spect()
    spec = sources[0][1]
    assert spec.dir_type == C.GG_DIR_FORCED
    assert spec.fd_angle_min == 0.0 and spec.fd_angle_max == pytest.approx(np.radians(8.0))
    assert sp.free_flight.enabled == C.FF_PRIMARY and sp.free_flight.angle_tolerance_max == 0.0
    d = spec_desc = scene.source_desc
    assert d.dir_type == C.GG_DIR_FORCED and d.fd_cos_max == pytest.approx(np.cos(np.radians(8.0)))
    assert spec_desc.fd_cos_min == pytest.approx(1.0)
    aa.angle_tolerance_min, aa.angle_tolerance_max = 9 * u.deg, 8 * u.deg
    with pytest.raises(ValueError):
        sim.build_spect()
