"""opengate-shaped API: configuration, validation and image I/O (no GPU)."""

import numpy as np
import pytest

import opengate_gb300 as gate
from opengate_gb300 import _capi as C
from opengate_gb300 import workloads as W

u = gate.g4_units


def water_sim(tmp_path, n=1000):
    """The 64^3 water cube / 1 MeV pencil beam written the way an opengate script does it."""
    sim = gate.Simulation()
    sim.output_dir = tmp_path
    sim.random_seed = 12345678
    sim.world.size = [2 * u.m, 2 * u.m, 2 * u.m]
    sim.world.material = "G4_AIR"
    img = sim.add_volume("Image", "phantom")
    img.image = gate.Image(np.zeros((64, 64, 64), np.int16), spacing=(2.0, 2.0, 2.0))
    img.material = "G4_AIR"
    img.voxel_materials = [[-1000, 1000, "G4_WATER"]]
    sim.physics_manager.physics_list_name = "G4EmStandardPhysics"
    sim.physics_manager.set_min_ekine("world", 10 * u.MeV)
    sim.physics_manager.set_user_limits_particles(["e-", "e+"])
    src = sim.add_source("GenericSource", "beam")
    src.particle = "gamma"
    src.n = n
    src.position.type = "point"
    src.position.translation = [0, 0, -64 * u.mm]
    src.direction.type = "momentum"
    src.direction.momentum = [0, 0, 1]
    src.energy.type = "mono"
    src.energy.mono = 1 * u.MeV
    dose = sim.add_actor("DoseActor", "dose")
    dose.attached_to = "phantom"
    dose.size = [64, 64, 64]
    dose.spacing = [2 * u.mm] * 3
    dose.edep_uncertainty.active = True
    dose.dose.active = True
    dose.dose_uncertainty.active = True
    sim.add_actor("SimulationStatisticsActor", "stats")
    return sim


def test_api_scene_equals_workload_scene(tmp_path):
    sim = water_sim(tmp_path)
    scene, vol, hu, names, sources = sim.build_scene()
    ref = W.water_pencil()
    assert names == ["G4_AIR", "G4_WATER"]
    # label 0 = image material (air), 1 = water: all voxels are water here
    assert np.all(scene.labels == 1)
    assert scene.corner == ref.corner and scene.spacing == ref.spacing
    s, r = scene.source_desc, ref.source_desc
    assert list(s.translation) == list(r.translation) and s.mono == r.mono and s.dir_type == r.dir_type
    water = names.index("G4_WATER")
    np.testing.assert_array_equal(scene.pt.sig[scene.pt.mat_comp[water]], ref.pt.sig[ref.pt.mat_comp[0]])


def test_unsupported_options_raise(tmp_path):
    sim = water_sim(tmp_path)
    sim.physics_manager.physics_list_name = "QGSP_BERT_EMV"
    with pytest.raises(NotImplementedError):
        sim.build_scene()
    sim = water_sim(tmp_path)
    sim.physics_manager.user_limits_particles = set()
    with pytest.raises(NotImplementedError):
        sim.build_scene()
    sim = water_sim(tmp_path)
    sim.sources["beam"].energy.type = "F18_analytic"
    with pytest.raises(NotImplementedError):
        sim.build_scene()
    with pytest.raises(AttributeError):
        sim.sources["beam"].not_a_parameter = 3
    with pytest.raises(NotImplementedError):
        sim.add_actor("LETActor", "let")
    sim = water_sim(tmp_path)
    sim.actors["dose"].score_in = "G4_WATER"
    scene, vol, hu, names, sources = sim.build_scene()
    with pytest.raises(NotImplementedError):
        sim.actors["dose"].check(vol, hu)
    sim.actors["dose"].score_in = "material"
    sim.actors["dose"].output_coordinate_system = "elsewhere"
    with pytest.raises(ValueError):
        sim.actors["dose"].check(vol, hu)


def test_dose_grid_placement_and_output_coordinates(tmp_path):
    """A dose grid of its own: centred on the image volume + translation, axis-aligned
    (AttachImageToVolume); output origin / direction per output_coordinate_system as in
    VoxelDepositActor._update_output_coordinate_system (doseactors.py:170-232)."""
    from scipy.spatial.transform import Rotation

    sim = water_sim(tmp_path)
    vol = sim.volumes["phantom"]
    vol.translation = [5 * u.mm, -3 * u.mm, 2 * u.mm]
    d = sim.actors["dose"]
    d.size = [10, 12, 14]
    d.spacing = [4 * u.mm, 5 * u.mm, 6 * u.mm]
    d.translation = [1 * u.mm, 2 * u.mm, 3 * u.mm]
    rot = Rotation.from_euler("z", 30, degrees=True).as_matrix()
    d.rotation = rot
    scene, v, hu, names, sources = sim.build_scene()
    d.check(v, hu)
    assert not d.on_image_grid(hu)
    dims, sp, corner = d.scoring_grid(v)
    assert dims == [10, 12, 14] and sp == pytest.approx([4, 5, 6])
    np.testing.assert_allclose(corner, np.array([6, -1, 5]) - np.array([40, 60, 84]) / 2.0)
    size, spa = np.array([10, 12, 14.0]), np.array([4.0, 5.0, 6.0])
    origin = -size * spa / 2 + spa / 2
    local = Rotation.from_matrix(rot).apply(origin) + np.array([1.0, 2.0, 3.0])
    for cs, o, r in ((None, origin, np.eye(3)), ("local", local, rot),
                     ("global", local + np.array([5.0, -3.0, 2.0]), rot)):
        d.output_coordinate_system = cs
        s2, o2, r2 = d.output_geometry(v, hu)
        np.testing.assert_allclose(o2, o, atol=1e-12)
        np.testing.assert_allclose(r2, r, atol=1e-12)
    d.output_coordinate_system = "attached_to_image"
    _, o3, r3 = d.output_geometry(v, hu)
    n_tr = np.asarray(hu.origin) + (np.array(hu.size) - 1.0) * hu.spacing / 2.0
    np.testing.assert_allclose(o3, local + n_tr, atol=1e-12)
    # the image grid itself is recognised
    d.size, d.spacing, d.translation = list(hu.size), list(hu.spacing), [0, 0, 0]
    assert d.on_image_grid(hu)


def test_spectrum_and_acceptance_conversion(tmp_path):
    sim = water_sim(tmp_path)
    src = sim.sources["beam"]
    src.energy.type = "spectrum_histogram"
    src.energy.spectrum_energy_bin_edges = [0.1, 0.2, 0.4]
    src.energy.spectrum_weights = [2.0, 1.0]
    src.direction.type = "iso"
    field = sim.add_volume("Box", "field")
    field.size = [10 * u.cm, 1 * u.mm, 10 * u.cm]
    field.translation = [0, -20 * u.cm, 0]
    src.direction.angular_acceptance.policy = "Rejection"
    src.direction.angular_acceptance.enable_intersection_check = True
    src.direction.angular_acceptance.target_volumes = ["field"]
    spec = src.to_spec(sim.volumes)
    assert spec.ene_type == C.GG_ENE_HISTOGRAM
    np.testing.assert_allclose(spec.spec_cdf, [0.2 / 0.4, 1.0])  # cumulative of w * dE
    assert spec.accept_boxes == [((-50.0, -200.5, -50.0), (50.0, -199.5, 50.0))]
    src.energy.type = "spectrum_discrete"
    src.energy.spectrum_energies = [0.1405, 0.364]
    src.energy.spectrum_weights = [0.89, 0.11]
    spec = src.to_spec(sim.volumes)
    np.testing.assert_allclose(spec.spec_cdf, [0.89, 1.0])


def test_hounsfield_api_wrapper_uses_g4_density_units(tmp_path):
    sim = gate.Simulation()
    vm, created = gate.HounsfieldUnit_to_material(sim, 0.05 * u.g_cm3, W.CT10_MATERIALS, W.CT10_DENSITIES)
    ref_vm, _ = W.ct_materials(0.05)[:2]
    assert vm == ref_vm
    assert sim.volume_manager.material_database.get(created[0]).density == pytest.approx(0.0012)


def test_mhd_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    for dt in (np.int16, np.float32, np.float64, np.uint16):
        arr = (rng.normal(size=(5, 6, 7)) * 100).astype(dt)
        img = gate.Image(arr, spacing=(1.5, 2.0, 2.5), origin=(-3.0, 4.0, 5.5))
        p = gate.write_mhd(tmp_path / f"img_{np.dtype(dt).name}.mhd", img)
        back = gate.read_mhd(p)
        assert back.array.dtype == arr.dtype
        np.testing.assert_array_equal(back.array, arr)
        np.testing.assert_array_equal(back.spacing, img.spacing)
        np.testing.assert_array_equal(back.origin, img.origin)
        assert back.size == (7, 6, 5)


def test_units_follow_clhep():
    assert u.mm == 1 and u.MeV == 1 and u.cm == 10
    assert u.g_cm3 == pytest.approx(6.241509074460763e18, rel=1e-12)
    assert u.Gy == pytest.approx(1e-12, rel=1e-12)
    assert u.deg == pytest.approx(np.pi / 180)


def test_dose_density_output_on_image_grid(tmp_path):
    """density output = the HU-interval density map in g/cm3, 0 outside every interval
    (create_density_img, materials.py:294-324); no resampling when the output grid is the image's."""
    sim = water_sim(tmp_path)
    vol = sim.volumes["phantom"]
    arr = np.full((64, 64, 64), -2000, np.int16)
    arr[10:20] = 0
    arr[20:30] = 1500
    vol.image = gate.Image(arr, spacing=(2.0, 2.0, 2.0))
    vol.voxel_materials = [[-1000, 1000, "G4_WATER"], [1000, 3000, "G4_BONE_CORTICAL_ICRP"]]
    d = sim.actors["dose"]
    d.output_coordinate_system = "attached_to_image"
    d.density.active = True
    scene, v, hu, names, sources = sim.build_scene()
    d.check(v, hu)
    db = sim.volume_manager.material_database
    spacing, origin, direction = d.output_geometry(v, hu)
    rho = d.density_image(v, hu, db, spacing, origin, direction)
    assert rho.dtype == np.float32 and rho.shape == arr.shape
    assert np.all(rho[:10] == 0) and np.all(rho[30:] == 0)
    assert np.all(rho[10:20] == np.float32(db.get("G4_WATER").density))
    assert np.all(rho[20:30] == np.float32(db.get("G4_BONE_CORTICAL_ICRP").density))
    d.counts.active = True
    with pytest.raises(NotImplementedError):
        d.check(v, hu)


def test_dose_density_output_resampled_like_itk(tmp_path):
    """A dose grid of its own: the density map is resampled linearly by physical position with 0
    outside (resample_itk_image_like, image.py:532-557), checked against scipy's trilinear
    map_coordinates on the continuous indices, and for a rotated output grid point by point."""
    from scipy.ndimage import map_coordinates
    from scipy.spatial.transform import Rotation

    from opengate_gb300 import dose as D

    rng = np.random.default_rng(7)
    sim = water_sim(tmp_path)
    vol = sim.volumes["phantom"]
    arr = rng.integers(-1500, 2500, size=(20, 24, 28)).astype(np.int16)
    vol.image = gate.Image(arr, spacing=(2.0, 2.5, 3.0), origin=(-20.0, 7.0, 3.0))
    vol.voxel_materials = [[-1000, 0, "G4_ADIPOSE_TISSUE_ICRP"], [0, 1000, "G4_WATER"],
                           [1000, 3000, "G4_BONE_CORTICAL_ICRP"]]
    d = sim.actors["dose"]
    d.size, d.spacing, d.translation = [11, 9, 13], [5.0, 6.0, 4.5], [3.0, -2.0, 1.0]
    scene, v, hu, names, sources = sim.build_scene()
    db = sim.volume_manager.material_database
    rho_ct = D.density_image(hu.array, v.voxel_materials, db).astype(np.float64)
    for cs in ("attached_to_image", None):
        d.output_coordinate_system = cs
        spacing, origin, direction = d.output_geometry(v, hu)
        rho = d.density_image(v, hu, db, spacing, origin, direction)
        assert rho.shape == (13, 9, 11) and rho.dtype == np.float32
        grid = np.stack(np.meshgrid(*[np.arange(n) for n in (11, 9, 13)], indexing="ij"), -1)
        p = np.asarray(origin) + (grid * np.asarray(spacing)) @ np.asarray(direction).T
        c = (p - hu.origin) / hu.spacing  # [x][y][z][3], x-fastest axis first
        n = np.array(hu.size)
        inside = np.all((c >= -0.5) & (c < n - 0.5), axis=-1)
        # trilinear with clamped neighbours = map_coordinates order 1, mode "nearest"
        ref = map_coordinates(rho_ct, [c[..., 2], c[..., 1], c[..., 0]], order=1, mode="nearest")
        ref[~inside] = 0.0
        np.testing.assert_allclose(rho, ref.transpose(2, 1, 0).astype(np.float32), rtol=1e-6, atol=1e-7)
        assert inside.any() and (~inside).any()
    # rotated output grid
    rot = Rotation.from_euler("zy", [25, -10], degrees=True).as_matrix()
    out = D.resample_linear(rho_ct, hu.spacing, hu.origin, [7, 8, 9], [3.0, 3.0, 3.0], [-5.0, 10.0, 20.0], rot)
    for (i, j, k) in [(0, 0, 0), (3, 4, 5), (6, 7, 8), (2, 0, 7)]:
        p = np.array([-5.0, 10.0, 20.0]) + rot @ (np.array([i, j, k]) * 3.0)
        c = (p - hu.origin) / hu.spacing
        if np.all((c >= -0.5) & (c < np.array(hu.size) - 0.5)):
            want = map_coordinates(rho_ct, [[c[2]], [c[1]], [c[0]]], order=1, mode="nearest")[0]
        else:
            want = 0.0
        assert out[k, j, i] == pytest.approx(want, rel=1e-12, abs=1e-12)
