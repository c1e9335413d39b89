"""GE Discovery NM670 heads on the opengate-shaped API
(opengate/contrib/spect/ge_discovery_nm670.py counterparts, same function names).

A head is one SpectHead volume (collimator with hexagonal holes, gap, NaI
crystal); its crystal is addressed as f"{name}_crystal" by add_digitizer.
Collimators: lehr (1.5 mm holes, 35 mm, 0.2 mm septa), megp (3 mm, 58 mm,
1.05 mm), hegp (4 mm, 66 mm, 1.8 mm); crystal 3/8" or 5/8".  The digitizer is
adder (energy winner) -> energy blurring -> spatial blurring -> energy windows
-> projection, with the reference's add_digitizer parameters (inverse-square
energy blur of 6.3 % FWHM at 140.57 keV, 3 mm FWHM spatial blur kept inside
the crystal; ge_discovery_nm670.py:1166-1230).
"""

from ...units import g4_units as _u
from ...api import Box
from .spect_helpers import get_default_energy_windows


def add_spect_head(sim, name="spect", collimator_type="lehr", rotation_deg=0, debug=False, crystal_size="3/8"):
    if rotation_deg:
        raise NotImplementedError("collimator rotation about the head axis")
    if collimator_type in (False, None, "none", "False"):
        raise NotImplementedError("heads without collimator")
    head = sim.add_volume("SpectHead", name)
    head.collimator_type = str(collimator_type).lower()
    head.crystal_size = crystal_size
    head.housing = "nm670"  # the shielding box of add_spect_box (ge_discovery_nm670.py:215-262)
    crystal = Box({"name": head.crystal_name, "head": name})
    return head, Box({"name": f"{name}_collimator", "head": name}), crystal


def add_spect_two_heads(sim, name="spect", collimator_type="lehr", debug=False, radius=None):
    radius = 36 * _u.cm if radius is None else radius
    h1, _, c1 = add_spect_head(sim, f"{name}_1", collimator_type, debug=debug)
    h2, _, c2 = add_spect_head(sim, f"{name}_2", collimator_type, debug=debug)
    rotate_gantry(h1, radius, start_angle_deg=0, step_angle_deg=1, nb_angle=1)
    rotate_gantry(h2, radius, start_angle_deg=180, step_angle_deg=1, nb_angle=1)
    return [h1, h2], [c1, c2]


def rotate_gantry(head, radius, start_angle_deg, step_angle_deg=1, nb_angle=1):
    """Head positions of the runs: collimator face at `radius`, angle start + r * step."""
    head.radius = radius
    head.start_angle_deg = float(start_angle_deg)
    head.step_angle_deg = float(step_angle_deg)
    head.nb_angle = int(nb_angle)


def get_default_size_and_spacing():
    mm = _u.mm
    return [128, 128], [2.21 * mm * 2, 2.21 * mm * 2]


class Digitizer:
    """The chain of one head: blurring modules and the projection actor (find_module)."""

    def __init__(self, name, projection, modules=()):
        self.name = name
        self.projection = projection
        self.modules = list(modules)

    def find_module(self, kind):
        k = kind.lower()
        if "projection" in k:
            return self.projection
        for m in self.modules:
            if k in m.name.lower() or k == m.type_name.lower():
                return m
        raise KeyError(f"digitizer '{self.name}' has no module '{kind}'")


def add_digitizer(sim, crystal_name, name=None, size=None, spacing=None, channels=None, filename=None,
                  policy="EnergyWinnerPosition", resolution=0.063, reference_energy=140.57 * _u.keV,
                  spatial_fwhm=3 * _u.mm):
    """The NM670 chain: adder, inverse-square energy blur (FWHM/E = resolution at
    reference_energy), spatial blur (spatial_fwhm, kept in the crystal), windows, projection."""
    name = crystal_name if name is None else name
    d_size, d_spacing = get_default_size_and_spacing()
    # singles
    sc = sim.add_actor("DigitizerAdderActor", f"{name}_singles")
    sc.attached_to = crystal_name
    sc.group_volume = None
    sc.policy = policy
    # energy blurring
    eb = sim.add_actor("DigitizerBlurringActor", f"{name}_eblur")
    eb.attached_to = crystal_name
    eb.blur_attribute = "TotalEnergyDeposit"
    eb.blur_method = "InverseSquare"
    eb.blur_resolution = resolution
    eb.blur_reference_value = reference_energy
    # spatial blurring
    sb = sim.add_actor("DigitizerSpatialBlurringActor", f"{name}_sblur")
    sb.attached_to = crystal_name
    sb.blur_attribute = "PostPosition"
    sb.blur_fwhm = spatial_fwhm
    sb.keep_in_solid_limits = True
    sb.use_truncated_Gaussian = False
    # energy windows and projection
    cc = sim.add_actor("DigitizerEnergyWindowsActor", f"{name}_energy_window")
    cc.attached_to = crystal_name
    cc.channels = channels if channels is not None else get_default_energy_windows("tc99m")
    proj = sim.add_actor("DigitizerProjectionActor", f"{name}_projection")
    proj.attached_to = crystal_name
    proj.channels = cc.channels
    proj.input_digi_collections = [c["name"] for c in proj.channels]
    proj.size = size if size is not None else d_size
    proj.spacing = spacing if spacing is not None else d_spacing
    if filename is not None:
        proj.output_filename = filename
    return Digitizer(name, proj, [sc, eb, sb, cc])


def add_digitizer_energy_windows(sim, crystal_volume_name, channels, policy="EnergyWinnerPosition"):
    """Singles (adder) and energy windows of a head crystal, no blurring and no projection
    (the chain of add_digitizer_energy_windows_OLD, ge_discovery_nm670.py:601-630); returns the
    DigitizerEnergyWindowsActor, e.g. for an ARFTrainingDatasetActor."""
    sc = sim.add_actor("DigitizerAdderActor", f"Singles_{crystal_volume_name}")
    sc.attached_to = crystal_volume_name
    sc.group_volume = None
    sc.policy = policy
    cc = sim.add_actor("DigitizerEnergyWindowsActor", f"EnergyWindows_{crystal_volume_name}")
    cc.attached_to = crystal_volume_name
    cc.input_digi_collection = sc.name
    cc.channels = channels
    return cc


# ---------------------------------------------------------------------------------- ARF
def add_detection_plane_for_arf(sim, det_name, colli_type, plane_size=None):
    """The ARF detection plane (ge_discovery_nm670.py:957-991): on the GPU path, the collimator
    face of a `colli_type` head placed by rotate_gantry like a SpectHead (the reference puts a
    1 nm G4_Galactic box in front of the head).  plane_size: [576 mm, 446 mm] by default."""
    mm = _u.mm
    plane = sim.add_volume("ArfDetectorPlane", det_name)
    plane.collimator_type = str(colli_type).lower()
    plane.housing = "nm670"  # the NM670 head behind the plane
    if plane_size is None:
        plane_size = [576 * mm, 446 * mm]
    plane.size = [plane_size[0], plane_size[1], 1 * _u.nm]
    rotate_gantry(plane, plane.radius, start_angle_deg=0)
    return plane


def add_source_for_arf_training_dataset(sim, source_name, activity, detector_plane, min_energy, max_energy):
    """The training source of ge_discovery_nm670.py:994-1011: a 5 cm disc 20 cm in front of the
    plane, isotropic directions accepted towards the plane, energies uniform in [min, max]."""
    cm = _u.cm
    source = sim.add_source("GenericSource", source_name)
    source.particle = "gamma"
    source.activity = activity
    source.position.type = "disc"
    source.position.radius = 5 * cm
    source.position.translation = [0, -20 * cm, 0]
    source.direction.type = "iso"
    source.energy.type = "range"
    source.energy.min_energy = min_energy
    source.energy.max_energy = max_energy
    source.direction.angular_acceptance.target_volumes = [detector_plane.name]
    source.direction.angular_acceptance.enable_intersection_check = True
    return source


def add_actor_for_arf_training_dataset(sim, colli_type, ene_win_actor, rr):
    """Detection plane + ARFTrainingDatasetActor (ge_discovery_nm670.py:1014-1026); the rows go
    to arf_training_dataset.npz (this library's dataset format) in the output directory."""
    detector_plane = add_detection_plane_for_arf(sim, "arf_plane", colli_type)
    arf = sim.add_actor("ARFTrainingDatasetActor", "ARF (training)")
    arf.energy_windows_actor = ene_win_actor.name
    arf.attached_to = detector_plane.name
    arf.output_filename = "arf_training_dataset.npz"
    arf.russian_roulette = rr
    arf.plane_axis = [0, 1, 2]
    return detector_plane, arf


def distance_to_crystal(colli_type, crystal_size="3/8", gap=0.0, housing="nm670"):
    """Distance (mm units) from the collimator face to the middle of the crystal (behind the
    housing's entrance cover): the depth of the ARF projection plane."""
    from ... import spect as S

    coll = S.COLLIMATORS[str(colli_type).lower()]
    cover, _ = S.housing_layers(housing, S.CRYSTALS[crystal_size])
    c = cover[0] if cover else 0.0
    return (coll["collimator_thickness"] + gap + c + 0.5 * S.CRYSTALS[crystal_size]) * _u.mm


def add_arf_detector(sim, name, colli_type, image_size, image_spacing, pth_filename):
    """Detection plane + ARFActor (ge_discovery_nm670.py:1029-1053); `pth_filename` is a network
    file of this library (train_arf), the projection depth the middle of the crystal."""
    det_plane = add_detection_plane_for_arf(sim, det_name=name, colli_type=colli_type)
    arf = sim.add_actor("ARFActor", f"{name}_arf")
    arf.attached_to = det_plane.name
    arf.output_filename = f"projection_{arf.name}.mhd"
    arf.batch_size = 1e5
    arf.image_size = image_size
    arf.image_spacing = image_spacing
    arf.verbose_batch = False
    arf.distance_to_crystal = distance_to_crystal(colli_type, det_plane.crystal_size, det_plane.gap,
                                                  det_plane.housing)
    arf.pth_filename = pth_filename
    arf.flip_plane = False
    arf.plane_axis = [0, 1, 2]
    arf.enable_hit_slice = False
    arf.gpu_mode = "auto"
    return det_plane, arf
