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
    proj = sim.add_actor("DigitizerProjectionActor", f"{name}_projection")
    proj.attached_to = crystal_name
    proj.channels = channels if channels is not None else get_default_energy_windows("tc99m")
    proj.input_digi_collections = [c["name"] for c in proj.channels]
    proj.size = size if size is not None else d_size
    proj.spacing = spacing if spacing is not None else d_spacing
    if filename is not None:
        proj.output_filename = filename
    return Digitizer(name, proj, [sc, eb, sb])
