"""opengate-shaped Python API of the GPU path.

Mirrors the subset of the reference's user API that the voxel photon path
uses, with the same names, units and semantics:

* ``Simulation`` (opengate/managers.py:1805): ``add_volume``, ``add_source``,
  ``add_actor``, ``world``, ``physics_manager``, ``random_seed``,
  ``output_dir``, ``run()``;
* volumes: the world box, ``Box`` (only as a virtual volume in the world
  material, e.g. an angular-acceptance target) and ``Image``
  (``ImageVolume``, opengate/geometry/volumes.py:882) with ``image``,
  ``material``, ``voxel_materials``, ``translation``;
* ``HounsfieldUnit_to_material(sim, density_tolerance, file_mat,
  file_density)`` (opengate/geometry/materials.py:149);
* ``physics_manager.physics_list_name``, ``set_min_ekine``,
  ``set_user_limits_particles`` (opengate/managers.py:701, 1071, 1102);
* ``GenericSource`` (opengate/sources/generic.py:333) with ``n``,
  ``position``, ``direction`` (incl. ``angular_acceptance``), ``energy``;
* ``DoseActor`` (opengate/actors/doseactors.py:317): edep / edep_squared /
  edep_uncertainty / dose / dose_squared / dose_uncertainty / density
  outputs (``counts`` raises), ``number_of_samples``; ``SimulationStatisticsActor`` (miscactors.py:30).

Options the GPU path does not implement raise errors at ``run()`` instead of
being ignored; electron transport is not modelled, so the simulation must
stop e-/e+ at creation with the user limits, exactly as the reference is
configured for this path.
"""

import copy
import math
import os
import pathlib
import time

import numpy as np

from . import _capi as C
from . import dose as D
from . import image_io
from . import materials as M
from . import tables as T
from .scene import Scene, SourceSpec
from .units import g4_units

u = g4_units


class Box(dict):
    """dict with attribute access; nested dicts become Boxes (python-box subset)."""

    def __init__(self, *a, **k):
        super().__init__(*a, **k)
        for key, v in list(self.items()):
            if isinstance(v, dict) and not isinstance(v, Box):
                self[key] = Box(v)

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e

    def __setattr__(self, k, v):
        self[k] = Box(v) if isinstance(v, dict) and not isinstance(v, Box) else v


class GateObject:
    """Named object holding user parameters with defaults (GateObject pattern, base.py:362)."""

    type_name = "GateObject"
    user_info_defaults = {}

    def __init__(self, name, simulation=None, **kw):
        object.__setattr__(self, "name", name)
        object.__setattr__(self, "simulation", simulation)
        for k, v in self.user_info_defaults.items():
            object.__setattr__(self, k, copy.deepcopy(v))
        for k, v in kw.items():
            setattr(self, k, v)

    def __setattr__(self, k, v):
        if k not in self.user_info_defaults and not k.startswith("_") and k not in ("name", "simulation"):
            raise AttributeError(f"{self.type_name} '{self.name}' has no parameter '{k}'")
        if isinstance(v, dict) and not isinstance(v, Box):
            v = Box(v)
        object.__setattr__(self, k, v)


# --------------------------------------------------------------------------- volumes
class BoxVolume(GateObject):
    type_name = "Box"
    user_info_defaults = {"mother": "world", "size": [10 * u.cm] * 3, "translation": [0.0, 0.0, 0.0],
                          "rotation": np.eye(3), "material": "G4_AIR", "color": [1, 1, 1, 1]}


class ImageVolume(GateObject):
    type_name = "Image"
    user_info_defaults = {"mother": "world", "image": "", "material": "G4_AIR",
                          "voxel_materials": [[-np.inf, np.inf, "G4_AIR"]], "translation": [0.0, 0.0, 0.0],
                          "rotation": np.eye(3), "dump_label_image": None, "color": [1, 1, 1, 1]}

    def load_image(self):
        """HU image as an image_io.Image (array [z][y][x], spacing in mm)."""
        img = self.image
        if isinstance(img, image_io.Image):
            return img
        if isinstance(img, (str, pathlib.Path)) and str(img):
            return image_io.read_mhd(img)
        raise ValueError(f"ImageVolume '{self.name}': set .image to an .mhd path or an image_io.Image")


class SpectHead(GateObject):
    """A SPECT head as one volume: parallel-hole collimator (hexagonal holes), gap and NaI crystal
    (the heads built by contrib/spect/ge_discovery_nm670.py:125-164 add_spect_head and
    siemens_intevo.py:84-130), placed by rotate_gantry (ge_discovery_nm670.py:1056-1080): at run r
    the collimator face is at `radius` from the z axis, angle start_angle_deg + r step_angle_deg."""

    type_name = "SpectHead"
    user_info_defaults = {"mother": "world", "collimator_type": "lehr", "crystal_size": "3/8",
                          "radius": 25 * u.cm, "start_angle_deg": 0.0, "step_angle_deg": 1.0, "nb_angle": 1,
                          "gap": 0.0, "half_width": None, "collimator_material": "G4_Pb",
                          "crystal_material": "G4_SODIUM_IODIDE", "housing": "none"}

    @property
    def crystal_name(self):
        return f"{self.name}_crystal"


class ArfDetectorPlane(SpectHead):
    """Detection plane of an ARF detector or of an ARF training dataset
    (contrib/spect/ge_discovery_nm670.py:957-991 add_detection_plane_for_arf).
    On the GPU path the plane is the collimator face of a head of
    `collimator_type`, placed like a SpectHead by rotate_gantry: photons that
    reach it inside the network's domain are scored by the ARFActor's
    network, the others are tracked through the collimator and crystal
    behind it.  `size` (the plane's extent, default 576 x 446 mm) bounds the
    face; the thickness (1 nm in the reference) is not used."""

    type_name = "ArfDetectorPlane"
    user_info_defaults = dict(SpectHead.user_info_defaults, size=[576 * u.mm, 446 * u.mm, 1 * u.nm],
                              material="G4_Galactic", color=[1, 0, 0, 1])


class VolumeManager:
    def __init__(self, simulation):
        self.simulation = simulation
        self.material_database = M.MaterialDatabase()
        self.world = BoxVolume("world", simulation, size=[3 * u.m] * 3, material="G4_AIR", mother=None)
        self.volumes = {"world": self.world}

    def add_volume(self, volume_type, name):
        if name in self.volumes:
            raise ValueError(f"a volume named '{name}' already exists")
        cls = {"Box": BoxVolume, "BoxVolume": BoxVolume, "Image": ImageVolume, "ImageVolume": ImageVolume,
               "SpectHead": SpectHead, "ArfDetectorPlane": ArfDetectorPlane}.get(volume_type)
        if cls is None:
            raise NotImplementedError(f"volume type '{volume_type}' is not supported by the GPU path")
        v = cls(name, self.simulation)
        self.volumes[name] = v
        return v


def HounsfieldUnit_to_material(simulation, density_tolerance, file_mat, file_density):
    """Same signature as the reference's; the tolerance carries G4 density units."""
    return M.hounsfield_unit_to_material(simulation.volume_manager.material_database,
                                         density_tolerance / u.g_cm3, file_mat, file_density)


# --------------------------------------------------------------------------- physics
class PhysicsManager:
    def __init__(self, simulation):
        self.simulation = simulation
        self.physics_list_name = "QGSP_BERT_EMV"
        self.min_ekine = {}
        self.user_limits_particles = set()
        self.production_cuts = {}

    def set_min_ekine(self, volume_name, value):
        self.min_ekine[volume_name] = float(value)

    def set_user_limits_particles(self, particles):
        for p in ([particles] if isinstance(particles, str) else particles):
            self.user_limits_particles.add(p)

    def set_production_cut(self, volume_name, particle_name, value):
        self.production_cuts[(volume_name, particle_name)] = value

    def check_supported(self, max_energy):
        if self.physics_list_name != "G4EmStandardPhysics":
            raise NotImplementedError(
                f"physics list '{self.physics_list_name}': the GPU path implements G4EmStandardPhysics photons")
        if not {"e-", "e+"} <= self.user_limits_particles:
            raise NotImplementedError("electron transport is not modelled: call "
                                      "set_user_limits_particles(['e-', 'e+']) and set_min_ekine above the "
                                      "source energy so electrons and positrons stop at creation")
        if not self.min_ekine or min(self.min_ekine.values()) < max_energy:
            raise NotImplementedError("set_min_ekine(<world or image volume>, value) must exceed the highest "
                                      "source energy so e-/e+ stop at creation")


# --------------------------------------------------------------------------- sources
def _default_angular_acceptance():
    # same keys and defaults as generic_source_default_aa (actors/biasingactors.py:16-66)
    return Box({"policy": None, "skip_policy": "SkipEvents", "max_rejection": 10000, "target_volumes": [],
                "enable_intersection_check": False, "enable_angle_check": False,
                "angle_check_reference_vector": [0, 0, 1], "angle_check_proximity_distance": 0.0,
                "angle_tolerance_proximal": 90 * u.deg, "angle_tolerance_min": 0.0,
                "angle_tolerance_max": 6 * u.deg})


class GenericSource(GateObject):
    """Parameters as in opengate/sources/generic.py:24-77, 353-422 (photons)."""

    type_name = "GenericSource"
    user_info_defaults = {
        "attached_to": "world", "particle": "gamma", "n": 0, "activity": 0.0, "half_life": -1,
        "weight": -1, "weight_sigma": -1,
        "position": Box({"type": "point", "radius": 0.0, "sigma_x": 0.0, "sigma_y": 0.0, "size": [0, 0, 0],
                         "translation": [0, 0, 0], "rotation": np.eye(3), "confine": None, "dz": None}),
        "direction": Box({"type": "iso", "theta": [0.0, 180 * u.deg], "phi": [0.0, 360 * u.deg],
                          "momentum": [0, 0, 1], "focus_point": [0, 0, 0], "sigma": [0, 0],
                          "angular_acceptance": _default_angular_acceptance()}),
        "energy": Box({"type": "mono", "mono": 0.0, "sigma_gauss": 0.0, "is_cdf": False, "min_energy": None,
                       "max_energy": None, "spectrum_weights": [], "spectrum_energies": [],
                       "spectrum_energy_bin_edges": [], "spectrum_histogram_interpolation": None}),
    }

    def to_spec(self, volumes, free_flight=False):
        """SourceSpec (mm, rad, MeV) of this source; raises on unsupported options.  With
        ``free_flight`` (a GammaFreeFlightActor on the world, the SPECT heads excluded) the
        angular acceptance (intersection + angle check against the heads, as the reference's
        free-flight recipe sets it, contrib/spect/spect_config.py:937-970) is applied by the
        free flight itself: its tolerance is returned in ``spec.ff_angle_tolerance`` (rad)."""
        if self.particle != "gamma":
            raise NotImplementedError(f"source '{self.name}': only gamma primaries are transported")
        if self.attached_to != "world":
            raise NotImplementedError(f"source '{self.name}': sources must be attached to the world")
        if self.weight not in (-1, 1) or self.weight_sigma > 0:
            raise NotImplementedError(f"source '{self.name}': primary weights are not supported")
        s = SourceSpec()
        p = self.position
        s.pos_type = {"point": C.GG_POS_POINT, "box": C.GG_POS_BOX, "sphere": C.GG_POS_SPHERE,
                      "disc": C.GG_POS_DISC}.get(p.type)
        if s.pos_type is None or p.confine:
            raise NotImplementedError(f"source '{self.name}': position type '{p.type}' / confine unsupported")
        s.translation = [float(x) for x in p.translation]
        s.rotation = np.asarray(p.rotation, dtype=np.float64)
        s.half_size = [float(x) / 2.0 for x in p.size]
        s.radius = float(p.radius)
        d = self.direction
        s.dir_type = {"iso": C.GG_DIR_ISO, "momentum": C.GG_DIR_MOMENTUM, "focused": C.GG_DIR_FOCUSED}.get(d.type)
        if s.dir_type is None:
            raise NotImplementedError(f"source '{self.name}': direction type '{d.type}' unsupported")
        s.theta = [float(x) for x in d.theta]
        s.phi = [float(x) for x in d.phi]
        s.momentum = [float(x) for x in d.momentum]
        s.focus = [float(x) for x in d.focus_point]
        aa = d.angular_acceptance
        s.ff_angle_tolerance = 0.0
        if aa.policy == "ForceDirection" and free_flight:
            # GateForcedDirectionManager: the direction is drawn in the cone about the target
            # head's axis with the cone's weight; here one source aims history h at head
            # h mod n_heads (the reference's one source copy per head, spect_config.py:986-1006)
            if s.dir_type != C.GG_DIR_ISO:
                raise ValueError("'ForceDirection' replaces an 'iso' direction")
            if not (0.0 <= float(aa.angle_tolerance_min) < float(aa.angle_tolerance_max)):
                raise ValueError("'ForceDirection' needs 0 <= angle_tolerance_min < angle_tolerance_max")
            s.dir_type = C.GG_DIR_FORCED
            s.fd_angle_min = float(aa.angle_tolerance_min) / u.rad
            s.fd_angle_max = float(aa.angle_tolerance_max) / u.rad
        elif aa.policy and free_flight:
            if aa.policy != "Rejection" or aa.skip_policy != "SkipEvents":
                raise NotImplementedError("angular acceptance with free flight: policy 'Rejection', 'SkipEvents'")
            if aa.enable_angle_check:
                if float(aa.angle_check_proximity_distance) != 0.0 or float(aa.angle_tolerance_min) != 0.0:
                    raise NotImplementedError("angular acceptance: angle_tolerance_max only (no proximity, "
                                              "no minimum)")
                s.ff_angle_tolerance = float(aa.angle_tolerance_max) / u.rad
            # the intersection check is the flight's own: a line that misses every head stops
        elif aa.policy:
            if aa.policy != "Rejection" or aa.skip_policy != "SkipEvents" or aa.enable_angle_check or \
                    not aa.enable_intersection_check:
                raise NotImplementedError("angular acceptance: only policy 'Rejection' with 'SkipEvents' and "
                                          "the intersection check is supported")
            if s.dir_type != C.GG_DIR_ISO:
                raise ValueError("'SkipEvents' needs an 'iso' direction (GateAcceptanceAngleManager)")
            for vname in aa.target_volumes:
                v = volumes[vname]
                if not isinstance(v, BoxVolume) or not np.allclose(v.rotation, np.eye(3)):
                    raise NotImplementedError("acceptance targets must be unrotated Box volumes")
                c = np.asarray(v.translation, dtype=np.float64)
                h = np.asarray(v.size, dtype=np.float64) / 2.0
                s.accept_boxes.append((tuple(c - h), tuple(c + h)))
            s.max_rejection = int(aa.max_rejection)
        e = self.energy
        if e.type == "mono":
            s.ene_type, s.mono = C.GG_ENE_MONO, float(e.mono)
        elif e.type == "range":
            s.ene_type, s.e_lo, s.e_hi = C.GG_ENE_RANGE, float(e.min_energy), float(e.max_energy)
        elif e.type == "spectrum_discrete":
            w = np.cumsum(np.asarray(e.spectrum_weights, dtype=np.float64))
            s.ene_type, s.spec_e, s.spec_cdf = C.GG_ENE_LINES, np.asarray(e.spectrum_energies, float), w / w[-1]
        elif e.type == "spectrum_histogram":
            if e.spectrum_histogram_interpolation not in (None, "None", "none"):
                raise NotImplementedError("spectrum_histogram: only interpolation None is supported")
            edges = np.asarray(e.spectrum_energy_bin_edges, dtype=np.float64)
            w = np.asarray(e.spectrum_weights, dtype=np.float64)
            if len(edges) != len(w) + 1:
                raise ValueError("spectrum_energy_bin_edges must have one more element than spectrum_weights")
            acc = np.cumsum(w * np.diff(edges))  # GateGenericSource.cpp:602-608
            s.ene_type, s.spec_e, s.spec_cdf = C.GG_ENE_HISTOGRAM, edges, acc / acc[-1]
        else:
            raise NotImplementedError(f"source '{self.name}': energy type '{e.type}' unsupported")
        return s



class VoxelSource(GenericSource):
    """Activity image source (opengate/sources/voxelsources.py:15-122): the activity image (.mhd path
    or image_io.Image, [z][y][x]) is centred on position.translation; emission points follow the
    3-level CDF of compute_image_3D_CDF (image.py:313-360) with a uniform jitter in the voxel."""

    type_name = "VoxelSource"
    user_info_defaults = dict(GenericSource.user_info_defaults, image=None)

    def to_spec(self, volumes, free_flight=False):
        p = self.position
        if p.type not in ("point", None) or p.confine:
            raise NotImplementedError("VoxelSource: position.type / confine are set by the image")
        s = GenericSource.to_spec(self, volumes, free_flight=free_flight)
        img = self.image
        if isinstance(img, (str, pathlib.Path)):
            img = image_io.read_mhd(img)
        if not isinstance(img, image_io.Image):
            raise ValueError(f"VoxelSource '{self.name}': set .image to an .mhd path or an image_io.Image")
        arr = np.asarray(img.array, dtype=np.float64)
        if not np.any(arr > 0):
            raise ValueError(f"VoxelSource '{self.name}': the activity image is empty")
        spacing = np.asarray(img.spacing, dtype=np.float64)
        size = np.array([arr.shape[2], arr.shape[1], arr.shape[0]], dtype=np.float64)
        corner = np.asarray(p.translation, dtype=np.float64) - size * spacing / 2.0
        s.set_activity_image(arr, spacing, corner)
        return s


def expected_number_of_events(activity, half_life, t0, t1):
    """Expected events of an activity source in [t0, t1] (GateVSource::GetExpectedNumberOfEvents,
    core/opengate_core/opengate_lib/GateVSource.cpp:127-141): round(A (t1 - t0)) without decay,
    round(A / lambda (exp(-lambda t0) - exp(-lambda t1))) with half-life; A in Bq, times in s."""
    if half_life is None or half_life <= 0:
        return int(round(activity * (t1 - t0)))
    lam = math.log(2.0) / half_life
    return int(round(activity / lam * (math.exp(-lam * t0) - math.exp(-lam * t1))))


def sample_number_of_events(activity, half_life, t0, t1, rng):
    """Events of an activity source in [t0, t1]: the reference draws decay times with exponential
    spacing at the (decaying) activity (GateVSource.cpp:55-92), a Poisson process whose count is
    Poisson with the expected value above (unrounded)."""
    if half_life is None or half_life <= 0:
        mu = activity * (t1 - t0)
    else:
        lam = math.log(2.0) / half_life
        mu = activity / lam * (math.exp(-lam * t0) - math.exp(-lam * t1))
    return int(rng.poisson(max(mu, 0.0)))


def activity_yield(source):
    """Activity factor of a spectrum_discrete source: the sum of the line weights
    (GateGenericSource.cpp:561-574 normalises the weights and multiplies the activity)."""
    if source.energy.type == "spectrum_discrete":
        return float(np.sum(np.asarray(source.energy.spectrum_weights, dtype=np.float64)))
    return 1.0


def events_per_run(source, run_timing_intervals, rng):
    """Primaries of `source` in each run: `n` (an int for every run, or one value per run) or the
    activity over each run interval (times in g4 units)."""
    runs = len(run_timing_intervals)
    if source.n:
        n = source.n
        if np.ndim(n) == 0:
            return [int(n)] * runs
        if len(n) != runs:
            raise ValueError(f"source '{source.name}': n has {len(n)} values for {runs} runs")
        return [int(x) for x in n]
    if source.activity:
        a = float(source.activity) / u.Bq * activity_yield(source)
        hl = float(source.half_life) / u.s if source.half_life and source.half_life > 0 else None
        return [sample_number_of_events(a, hl, t0 / u.s, t1 / u.s, rng) for t0, t1 in run_timing_intervals]
    raise ValueError(f"source '{source.name}': set n or activity")


# --------------------------------------------------------------------------- actors
class ActorOutput:
    """One output image of an actor (edep, dose, uncertainty ...)."""

    def __init__(self, actor, suffix, active=False, write_to_disk=True):
        self.actor = actor
        self.suffix = suffix
        self.active = active
        self.write_to_disk = write_to_disk
        self.image = None
        self.number_of_samples = 0

    def get_data(self):
        return self.image

    def get_output_path(self):
        """The actor's output_filename with the output's name inserted before the extension
        (``projection_1.mhd`` -> ``projection_1_counts.mhd``; actoroutput.py:1053-1058)."""
        base = self.actor.output_filename
        if base in (None, "auto", ""):
            base = f"{self.actor.name}.mhd"
        base = pathlib.Path(base)
        sim = self.actor.simulation
        return pathlib.Path(sim.output_dir) / base.parent / f"{base.stem}_{self.suffix}.mhd"


class DoseActor(GateObject):
    """Parameters as in VoxelDepositActor / DoseActor (doseactors.py:50-116, 317-440)."""

    type_name = "DoseActor"
    user_info_defaults = {"attached_to": "world", "size": [10, 10, 10], "spacing": [1.0, 1.0, 1.0],
                          "translation": [0.0, 0.0, 0.0], "rotation": np.eye(3), "repeated_volume_index": 0,
                          "hit_type": "random", "output_coordinate_system": "local", "output_filename": "auto",
                          "score_in": "material", "uncertainty_goal": None, "priority": 100,
                          "uncertainty_first_check_after_n_events": 1e4, "uncertainty_top_voxels_count": 10,
                          "uncertainty_voxel_edep_threshold": 0.7, "uncertainty_overshoot_factor_N_events": 1.05}

    def __init__(self, name, simulation=None, **kw):
        super().__init__(name, simulation, **kw)
        for suffix, active in (("edep", True), ("edep_squared", False), ("edep_uncertainty", False),
                               ("dose", False), ("dose_squared", False), ("dose_uncertainty", False),
                               ("density", False), ("counts", False)):
            object.__setattr__(self, suffix, ActorOutput(self, suffix, active))

    def check(self, image_volume, image):
        if self.attached_to != image_volume.name:
            raise NotImplementedError("the DoseActor must be attached to the ImageVolume")
        if self.uncertainty_goal is not None and not 0.0 < self.uncertainty_goal < 1.0:
            raise ValueError(f"Uncertainty goal must be > 0 and < 1, where 1 means 100%: {self.uncertainty_goal}")
        if self.score_in not in ("material", None):
            raise NotImplementedError("score_in other than 'material' is not supported")
        if self.hit_type not in ("random", "pre", "post", "middle"):
            raise ValueError(f"hit_type '{self.hit_type}'")
        if self.output_coordinate_system not in ("local", "global", "attached_to_image", None):
            raise ValueError(f"Illegal parameter 'output_coordinate_system': {self.output_coordinate_system}")
        if len(self.size) != 3 or min(int(v) for v in self.size) < 1 or min(float(v) for v in self.spacing) <= 0:
            raise ValueError(f"DoseActor '{self.name}': size must be 3 positive integers, spacing > 0")
        if self.counts.active:
            raise NotImplementedError("the DoseActor 'counts' output (steps per voxel) is not scored")

    def density_image(self, volume, image, material_db, spacing, origin, direction):
        """The 'density' output (DoseActor.create_density_image_from_image_volume,
        doseactors.py:530-542): the image volume's density map in g/cm3 (create_density_img,
        materials.py:294-324), resampled linearly onto the output image's grid by physical position
        with 0 outside when the two grids differ in size, spacing or origin (images_have_same_domain,
        image.py:506-520)."""
        rho = D.density_image(image.array, volume.voxel_materials, material_db)
        same = list(self.size) == list(image.size) and \
            all(math.isclose(a, b, rel_tol=1e-5) for a, b in zip(spacing, image.spacing)) and \
            all(math.isclose(a, b, rel_tol=1e-5) for a, b in zip(origin, image.origin))
        if same:
            return rho
        return D.resample_linear(rho, image.spacing, image.origin, self.size, spacing, origin,
                                 direction).astype(np.float32)

    def on_image_grid(self, image):
        """True when the dose grid is the image's own voxel grid."""
        return list(self.size) == list(image.size) and np.allclose(self.spacing, image.spacing) and \
            np.allclose(self.translation, 0.0)

    def scoring_grid(self, volume):
        """(dims, spacing, corner) in mm of the scoring grid: centred on the attached image volume
        plus `translation`, axis-aligned with it (GateDoseActor::BeginOfRunActionMasterThread ->
        AttachImageToVolume, GateHelpersImage.txx:20-58; the actor's `rotation` only orients the
        output images, as in the reference).  Deposits are scored at the interaction point: with
        electrons stopped at creation the step of a deposit has no length, so the hit types
        "random", "pre", "post" and "middle" all give that point."""
        size = np.array([int(v) for v in self.size], dtype=np.int64)
        sp = np.array([float(v) for v in self.spacing]) / u.mm
        centre = np.asarray(volume.translation, dtype=np.float64) / u.mm + np.asarray(self.translation) / u.mm
        return [int(v) for v in size], sp.tolist(), (centre - size * sp / 2.0).tolist()

    def output_geometry(self, volume, image):
        """(spacing, origin, direction) of the output images
        (VoxelDepositActor._update_output_coordinate_system, doseactors.py:170-232)."""
        from scipy.spatial.transform import Rotation

        size = np.array([int(v) for v in self.size], dtype=np.float64)
        sp = np.array([float(v) for v in self.spacing]) / u.mm
        origin = -size * sp / 2.0 + sp / 2.0
        rot = np.asarray(self.rotation, dtype=np.float64)
        origin_local = Rotation.from_matrix(rot).apply(origin) + np.asarray(self.translation) / u.mm
        cs = self.output_coordinate_system
        if cs is None:
            return sp, origin, np.eye(3)
        if cs == "local":
            return sp, origin_local, rot
        if cs == "attached_to_image":
            n_rot = np.asarray(image.direction, dtype=np.float64)
            n_size = np.array(image.size, dtype=np.float64)
            n_tr = np.asarray(image.origin) + Rotation.from_matrix(n_rot).apply((n_size - 1.0) * image.spacing / 2.0)
            return sp, Rotation.from_matrix(n_rot).apply(origin_local) + n_tr, n_rot @ rot
        # global: the attached image volume is an unrotated daughter of the world
        return sp, origin_local + np.asarray(volume.translation, dtype=np.float64) / u.mm, rot

    @property
    def number_of_samples(self):
        return self.edep.number_of_samples


class TLEDoseActor(DoseActor):
    """Track-length estimator dose (TLEDoseActor, opengate/actors/doseactors.py:722-776;
    GateTLEDoseActor, core/opengate_core/opengate_lib/GateTLEDoseActor.cpp): photons at or
    below the threshold score E * mu_en * track length in every voxel they cross instead of
    the energy their electrons deposit; photons at or below ``energy_min`` deposit their
    energy where they are and stop.  mu_en from the EPDL or NIST element tables of the
    reference (mass-fraction mixture, log-log interpolation)."""

    type_name = "TLEDoseActor"
    user_info_defaults = dict(DoseActor.user_info_defaults, energy_min=0.0, tle_threshold=np.inf,
                              tle_threshold_type="None", database="EPDL")

    def check(self, image_volume, image):
        super().check(image_volume, image)
        if self.tle_threshold_type not in ("None", "energy", "max range", "average range"):
            raise ValueError("You did not define a correct threshold type")
        if self.tle_threshold_type in ("max range", "average range"):
            raise NotImplementedError(
                f"tle_threshold_type '{self.tle_threshold_type}' needs electron CSDA ranges (G4EmCalculator), "
                "which the GPU path does not have; use 'None' or 'energy'")
        if self.database not in ("EPDL", "NIST"):
            raise ValueError(f"database must be 'EPDL' or 'NIST', not {self.database!r}")

    @property
    def threshold_energy(self):
        """Photon energy (MeV) at or below which the estimator scores (inf for type 'None')."""
        return np.inf if self.tle_threshold_type == "None" else float(self.tle_threshold)


class DigitizerProjectionActor(GateObject):
    """Projection of the singles of one SPECT head's crystal (GateDigitizerProjectionActor,
    core/opengate_core/opengate_lib/digitizer/GateDigitizerProjectionActor.cpp:127-223;
    opengate/actors/digitizers.py:1140-1395): counts [run * n_channels + channel][y][x] in the
    energy windows `channels` ({"name", "min", "max"}, [min, max)), singles = per-event crystal
    energy at the energy-winner position (GateDigiAdderInVolume EnergyWinnerPosition)."""

    type_name = "DigitizerProjectionActor"
    user_info_defaults = {"attached_to": None, "input_digi_collections": [], "channels": [],
                          "size": [128, 128], "spacing": [4.42 * u.mm, 4.42 * u.mm], "output_filename": "auto",
                          "write_to_disk": True, "detector_orientation_matrix": np.eye(3),
                          "priority": 100}

    def __init__(self, name, simulation=None, **kw):
        super().__init__(name, simulation, **kw)
        object.__setattr__(self, "counts", ActorOutput(self, "counts", True))
        # history-by-history squared counts (free flight: summed squared weights), written
        # when ``squared_counts.active`` is set, as in the reference
        sq = ActorOutput(self, "squared_counts", False)
        object.__setattr__(self, "squared_counts", sq)
        object.__setattr__(self, "counts_squared", sq)


class DigitizerEnergyWindowsActor(GateObject):
    """Energy windows of a head's singles (GateDigitizerEnergyWindowsActor::ApplyThreshold,
    core/opengate_core/opengate_lib/digitizer/GateDigitizerEnergyWindowsActor.cpp:116-132;
    opengate/actors/digitizers.py): `channels` = [{"name", "min", "max"}], [min, max).  A
    projection actor on the same crystal without channels of its own takes these."""

    type_name = "DigitizerEnergyWindowsActor"
    user_info_defaults = {"attached_to": None, "input_digi_collection": "Singles", "channels": [],
                          "output_filename": "auto", "write_to_disk": False, "priority": 90}


def check_channel_overlap(ch1, ch2):
    """True when two energy windows overlap (opengate/actors/arfactors.py:19-30)."""
    a0, a1, b0, b1 = float(ch1["min"]), float(ch1["max"]), float(ch2["min"]), float(ch2["max"])
    return b0 < a0 < b1 or b0 < a1 < b1 or a0 < b0 < a1 or a0 < b1 < a1


class ARFTrainingDatasetActor(GateObject):
    """Training rows of an ARF network (GateARFTrainingDatasetActor,
    core/opengate_core/opengate_lib/GateARFTrainingDatasetActor.cpp:76-137; arfactors.py:33-145):
    for photons reaching the detection plane `attached_to`, (E, Theta, Phi) at the plane and
    the energy window (1..n) their single ends in, 0 = none (kept with probability
    1 / russian_roulette).  The GPU path starts the photons on the plane with the source's
    energy range, directions uniform in theta up to `theta_max_deg` (default: the largest angle
    between the source disc and the plane) and phi, and tracks them through the head and the
    digitizer of the windows actor `energy_windows_actor`.  Rows go to `output_filename` (.npz,
    opengate_gb300.arf format)."""

    type_name = "ARFTrainingDatasetActor"
    user_info_defaults = {"attached_to": None, "energy_windows_actor": None, "russian_roulette": 1,
                          "plane_axis": [0, 1, 2], "attributes": [], "debug": False, "clear_every": 1e5,
                          "keep_zero_edep": False, "output_filename": "arf_training_dataset.npz",
                          "write_to_disk": True, "theta_max_deg": None, "priority": 100}

    def __init__(self, name, simulation=None, **kw):
        super().__init__(name, simulation, **kw)
        object.__setattr__(self, "rows", None)
        object.__setattr__(self, "number_of_samples", 0)
        object.__setattr__(self, "sampling", None)  # gg_arf_sampling of the last run

    def get_output_path(self):
        return pathlib.Path(self.simulation.output_dir) / pathlib.Path(self.output_filename)


class ARFActor(GateObject):
    """ARF detector (GateARFActor, core/opengate_core/opengate_lib/GateARFActor.cpp:60-113;
    opengate/actors/arfactors.py:147-453): photons reaching the plane `attached_to` are scored
    with the window probabilities of the network in `pth_filename` at the pixel where their line
    crosses the plane `distance_to_crystal` behind it.  Output `counts` (and `squared_counts`):
    [run * n_windows + window][y][x] float32, spacing (image_spacing, 1), origin as the
    projection actor's.  The network file is this library's (.npz from train_arf, not a garf .pth);
    photons outside its trained domain, or entering the head through a side, are tracked through
    the collimator and crystal instead and counted in the same image.  batch_size and
    verbose_batch have no effect (every photon is scored on the GPU); flip_plane,
    enable_hit_slice, plane_axis other than [0, 1, 2] and gpu_mode "cpu" raise."""

    type_name = "ARFActor"
    user_info_defaults = {"attached_to": None, "batch_size": 2e5, "pth_filename": None, "image_size": [128, 128],
                          "image_spacing": [4.41806 * u.mm, 4.41806 * u.mm], "distance_to_crystal": None,
                          "verbose_batch": False, "enable_hit_slice": False, "flip_plane": False,
                          "plane_axis": [0, 1, 2], "gpu_mode": "auto", "output_filename": "auto",
                          "write_to_disk": True, "priority": 100}

    def __init__(self, name, simulation=None, **kw):
        super().__init__(name, simulation, **kw)
        object.__setattr__(self, "counts", ActorOutput(self, "counts", True))
        sq = ActorOutput(self, "squared_counts", False)
        object.__setattr__(self, "squared_counts", sq)
        object.__setattr__(self, "counts_squared", sq)

    def check(self):
        if self.flip_plane:
            raise NotImplementedError(f"ARFActor '{self.name}': flip_plane")
        if self.enable_hit_slice:
            raise NotImplementedError(f"ARFActor '{self.name}': enable_hit_slice")
        if list(self.plane_axis) != [0, 1, 2]:
            raise NotImplementedError(f"ARFActor '{self.name}': plane_axis other than [0, 1, 2]")
        if self.gpu_mode not in ("auto", "gpu"):
            raise NotImplementedError(f"ARFActor '{self.name}': gpu_mode '{self.gpu_mode}' (the network runs "
                                      "on the GPU only)")
        if not self.pth_filename:
            raise ValueError(f"ARFActor '{self.name}': set pth_filename")


FWHM_TO_SIGMA = 1.0 / (2.0 * math.sqrt(2.0 * math.log(2.0)))

# singles kept on the device between two reads when a digitizer module writes its singles (48 B each)
SINGLES_LIST_CAPACITY = 1 << 22


class DigitizerAdderActor(GateObject):
    """Singles of a head crystal from its hits (DigitizerAdderActor; GateDigiAdderInVolume,
    digitizer/GateDigiAdderInVolume.cpp:29-88): energy sum per event, position of the
    energy winner or the energy-weighted centroid (``policy``)."""

    type_name = "DigitizerAdderActor"
    user_info_defaults = {"attached_to": None, "input_digi_collection": "Hits", "policy": "EnergyWinnerPosition",
                          "time_difference": False, "number_of_hits": False, "group_volume": None,
                          "skip_attributes": [], "clear_every": 1e5, "output_filename": "auto", "priority": 100,
                          "write_to_disk": True}

    def adder_policy(self):
        if self.policy not in C.ADDER_POLICIES:
            raise ValueError(f"policy '{self.policy}'")
        if self.group_volume is not None:
            raise NotImplementedError("the GPU path adds the hits of the whole crystal (group_volume None)")
        return self.policy


class DigitizerBlurringActor(GateObject):
    """Energy blurring of the singles of a head crystal (DigitizerBlurringActor,
    opengate/actors/digitizers.py:428-580; GateDigitizerBlurringActor.cpp:74-97):
    Gaussian (blur_sigma or blur_fwhm), InverseSquare (blur_resolution = FWHM/E at
    blur_reference_value) or Linear (+ blur_slope)."""

    type_name = "DigitizerBlurringActor"
    user_info_defaults = {"attached_to": None, "input_digi_collection": "Hits", "blur_attribute": None,
                          "skip_attributes": [], "clear_every": 1e5, "blur_method": "Gaussian", "blur_sigma": None,
                          "blur_fwhm": None, "blur_reference_value": 0, "blur_resolution": 0, "blur_slope": 0,
                          "output_filename": "auto", "priority": 100, "write_to_disk": True}

    def energy_blur(self):
        """Keyword arguments of SpectSpec.set_energy_blur (MeV), validated as the reference does."""
        if self.blur_attribute != "TotalEnergyDeposit":
            raise NotImplementedError("the GPU path blurs the singles' TotalEnergyDeposit only")
        m = self.blur_method
        if m == "Gaussian":
            if self.blur_fwhm is not None and self.blur_sigma is not None:
                raise ValueError("Error, use blur_sigma or blur_fwhm, not both")
            sigma = self.blur_fwhm * FWHM_TO_SIGMA if self.blur_fwhm is not None else self.blur_sigma
            if sigma is None:
                raise ValueError("Error, use blur_sigma or blur_fwhm")
            return dict(method="Gaussian", sigma=float(sigma) / u.MeV)
        if m not in ("InverseSquare", "Linear"):
            raise ValueError(f"blur_method '{m}'")
        if self.blur_reference_value is None or self.blur_reference_value < 0:
            raise ValueError("Error, use positive blur_reference_value")
        if self.blur_resolution is None or self.blur_resolution < 0:
            raise ValueError("Error, use positive blur_resolution")
        slope = 0.0 if self.blur_slope is None else float(self.blur_slope)
        if m == "Linear" and self.blur_slope is None:
            raise ValueError("Error, use positive blur_slope")
        return dict(method=m, resolution=float(self.blur_resolution),
                    reference=float(self.blur_reference_value) / u.MeV, slope=slope * u.MeV)


class DigitizerSpatialBlurringActor(GateObject):
    """Spatial blurring of the singles' position in the crystal (DigitizerSpatialBlurringActor,
    opengate/actors/digitizers.py:801-920; GateDigitizerSpatialBlurringActor.cpp:85-206)."""

    type_name = "DigitizerSpatialBlurringActor"
    user_info_defaults = {"attached_to": None, "attributes": [], "input_digi_collection": "Hits",
                          "skip_attributes": [], "clear_every": int(1e5), "blur_attribute": None, "blur_fwhm": None,
                          "blur_sigma": None, "keep_in_solid_limits": True, "use_truncated_Gaussian": True,
                          "output_filename": "auto", "priority": 100, "write_to_disk": True}

    def spatial_blur(self):
        """Keyword arguments of SpectSpec.set_spatial_blur (mm)."""
        if self.blur_attribute not in ("PostPosition", "PrePosition", "Position"):
            raise NotImplementedError("the GPU path blurs the singles' position only")
        if self.blur_fwhm is not None and self.blur_sigma is not None:
            raise ValueError("Error, use blur_sigma or blur_fwhm, not both")
        if self.blur_fwhm is not None:
            v = self.blur_fwhm
            sigma = [x * FWHM_TO_SIGMA for x in v] if hasattr(v, "__len__") else [v * FWHM_TO_SIGMA] * 3
        elif self.blur_sigma is not None:
            v = self.blur_sigma
            sigma = list(v) if hasattr(v, "__len__") else [v] * 3
        else:
            raise ValueError("Error, use blur_sigma or blur_fwhm")
        return dict(sigma=[float(x) / u.mm for x in sigma[:2]], keep_in_solid_limits=bool(self.keep_in_solid_limits),
                    truncated=bool(self.use_truncated_Gaussian))


class GammaFreeFlightActor(GateObject):
    """Free flight of gammas (GammaFreeFlightActor, opengate/actors/biasingactors.py:247-300;
    GateGammaFreeFlightOptrActor / GateGammaFreeFlightOptn): attached to the world with the
    SPECT heads as ``exclude_volumes``, photons do not interact outside the heads and carry
    the probability of reaching them as their weight; the projections become weighted sums.
    The primary (unscattered) component of the reference's free-flight SPECT recipe
    (contrib/spect/spect_config.py:937-970)."""

    type_name = "GammaFreeFlightActor"
    user_info_defaults = {"attached_to": "world", "exclude_volumes": [], "weight_cutoff": -1.0,
                          "energy_cutoff": 0.0, "bias_primary_only": True, "bias_only_once": False,
                          "particles": ["gamma"], "priority": 100}

    def check(self, head_volumes):
        if self.attached_to != "world":
            raise NotImplementedError("the GPU path applies free flight to the whole world (attached_to='world')")
        excluded = set(self.exclude_volumes)
        for h in head_volumes:
            if not ({h.name, h.crystal_name, f"{h.name}_collimator"} & excluded):
                raise NotImplementedError(f"free flight must exclude the SPECT head '{h.name}' (exclude_volumes)")


class ScatterSplittingFreeFlightActor(GateObject):
    """Scatter splitting with free flight (ScatterSplittingFreeFlightActor,
    opengate/actors/biasingactors.py:368-460; GateScatterSplittingFreeFlightOptrActor.cpp:200-420 and
    GateScatterSplittingFreeFlightOptn.cpp:69-149): attached to the world with the SPECT heads as
    ``exclude_volumes`` and ``kill_interacting_in_volumes``.  Photons are tracked analog outside the
    heads and die when they enter one; each Compton (up to ``max_compton_level``, the next one kills
    the photon) and each Rayleigh scattering is re-sampled ``compton_splitting_factor`` /
    ``rayleigh_splitting_factor`` times into copies of 1 / factor of the weight that fly freely to
    the heads.  The projections become weighted sums: the scattered component of the reference's
    free-flight SPECT recipe (contrib/spect/spect_config.py:937-1000); GammaFreeFlightActor gives
    the primary one.  Angular acceptance: the intersection check is always applied (a copy that
    misses every head is dropped); the angle check measures the angle to the axis of the head
    the copy enters (angle_tolerance_max; no proximity rule)."""

    type_name = "ScatterSplittingFreeFlightActor"
    user_info_defaults = {"attached_to": "world", "exclude_volumes": [], "kill_interacting_in_volumes": [],
                          "splitting_factor": 1, "compton_splitting_factor": -1, "rayleigh_splitting_factor": -1,
                          "max_compton_level": 10, "weight_cutoff": -1.0, "energy_cutoff": 0.0,
                          "particles": ["gamma"], "priority": 100, "debug": False}

    def __init__(self, name, simulation=None, **kw):
        super().__init__(name, simulation, **kw)
        object.__setattr__(self, "angular_acceptance", _default_angular_acceptance())

    def check(self, head_volumes):
        if self.attached_to != "world":
            raise NotImplementedError("the GPU path applies scatter splitting to the whole world (attached_to='world')")
        excluded, killed = set(self.exclude_volumes), set(self.kill_interacting_in_volumes)
        for h in head_volumes:
            names = {h.name, h.crystal_name, f"{h.name}_collimator"}
            if not names & excluded:
                raise NotImplementedError(f"scatter splitting must exclude the SPECT head '{h.name}' (exclude_volumes)")
            if not names & killed:
                raise NotImplementedError(
                    f"the SPECT head '{h.name}' must be a kill volume (kill_interacting_in_volumes)")
        aa = self.angular_acceptance
        if aa.policy not in (None, False, "Rejection"):
            raise NotImplementedError("angular acceptance: only the 'Rejection' policy (or none)")
        if aa.policy == "Rejection" and aa.enable_angle_check and (
                float(aa.angle_check_proximity_distance) != 0.0 or float(aa.angle_tolerance_min) != 0.0):
            raise NotImplementedError("angular acceptance: angle_tolerance_max only (no proximity, no minimum)")

    def factors(self):
        """(Compton factor, Rayleigh factor, angle tolerance in radians or 0)."""
        nc = int(self.compton_splitting_factor)
        nr = int(self.rayleigh_splitting_factor)
        nc = int(self.splitting_factor) if nc < 0 else nc
        nr = int(self.splitting_factor) if nr < 0 else nr
        aa = self.angular_acceptance
        tol = float(aa.angle_tolerance_max) / u.rad if aa.policy == "Rejection" and aa.enable_angle_check else 0.0
        return nc, nr, tol


class SimulationStatisticsActor(GateObject):
    type_name = "SimulationStatisticsActor"
    user_info_defaults = {"attached_to": "world", "track_types_flag": False, "output_filename": "auto"}

    def __init__(self, name, simulation=None, **kw):
        super().__init__(name, simulation, **kw)
        object.__setattr__(self, "counts", Box({"runs": 0, "events": 0, "tracks": 0, "steps": 0,
                                                "duration": 0.0, "pps": 0, "sps": 0}))

    def __str__(self):
        c = self.counts
        return (f"runs {c.runs}\nevents {c.events}\ntracks {c.tracks}\nsteps {c.steps}\n"
                f"duration {c.duration / u.s:.4f} s\nPPS {c.pps}")


# --------------------------------------------------------------------------- simulation
class Simulation:
    """Configuration object graph and run entry point (opengate/managers.py:1805)."""

    def __init__(self, name="simulation"):
        self.name = name
        self.output_dir = "."
        self.random_seed = "auto"
        self.random_engine = "MixMaxRng"  # accepted; the GPU path uses Philox4x32-10 streams
        self.number_of_threads = 1  # accepted; histories run on the GPU
        self.verbose_level = "INFO"
        self.run_timing_intervals = [[0, 1 * u.s]]
        self.device = 0  # CUDA device ordinal
        self.precision = 32  # transport arithmetic: 32 or 64
        self.batch = 0  # histories per tally batch, 0 = library default
        self.volume_manager = VolumeManager(self)
        self.physics_manager = PhysicsManager(self)
        self.sources = {}
        self.actors = {}
        self.last_seed = None

    # -- object graph -------------------------------------------------------
    @property
    def world(self):
        return self.volume_manager.world

    @property
    def volumes(self):
        return self.volume_manager.volumes

    def add_volume(self, volume_type, name):
        return self.volume_manager.add_volume(volume_type, name)

    def add_source(self, source_type, name):
        if name in self.sources:
            raise ValueError(f"a source named '{name}' already exists")
        cls = {"GenericSource": GenericSource, "VoxelSource": VoxelSource}.get(source_type)
        if cls is None:
            raise NotImplementedError(f"source type '{source_type}' is not supported by the GPU path")
        s = cls(name, self)
        self.sources[name] = s
        return s

    def add_actor(self, actor_type, name):
        if name in self.actors:
            raise ValueError(f"an actor named '{name}' already exists")
        cls = {"DoseActor": DoseActor, "TLEDoseActor": TLEDoseActor,
               "SimulationStatisticsActor": SimulationStatisticsActor,
               "DigitizerAdderActor": DigitizerAdderActor,
               "GammaFreeFlightActor": GammaFreeFlightActor,
               "ScatterSplittingFreeFlightActor": ScatterSplittingFreeFlightActor,
               "DigitizerBlurringActor": DigitizerBlurringActor,
               "DigitizerSpatialBlurringActor": DigitizerSpatialBlurringActor,
               "DigitizerProjectionActor": DigitizerProjectionActor,
               "DigitizerEnergyWindowsActor": DigitizerEnergyWindowsActor,
               "ARFActor": ARFActor, "ARFTrainingDatasetActor": ARFTrainingDatasetActor}.get(actor_type)
        if cls is None:
            raise NotImplementedError(f"actor type '{actor_type}' is not supported by the GPU path")
        a = cls(name, self)
        self.actors[name] = a
        return a

    def get_output_path(self, name):
        return pathlib.Path(self.output_dir) / name

    # -- run ---------------------------------------------------------------
    def _seed(self):
        if self.random_seed in (None, "auto"):
            return int.from_bytes(os.urandom(8), "little")
        return int(self.random_seed) & 0xFFFFFFFFFFFFFFFF

    def build_scene(self, extra_materials=(), free_flight=False):
        """(scene, image volume, HU image, material names by label, sources) for this configuration."""
        images = [v for v in self.volumes.values() if isinstance(v, ImageVolume)]
        if len(images) != 1:
            raise NotImplementedError("the GPU path transports through exactly one ImageVolume")
        vol = images[0]
        if vol.mother != "world" or not np.allclose(vol.rotation, np.eye(3)):
            raise NotImplementedError("the ImageVolume must be an unrotated daughter of the world")
        for v in self.volumes.values():
            if isinstance(v, BoxVolume) and v is not self.world and v.material != self.world.material:
                raise NotImplementedError(f"volume '{v.name}': only the image and virtual boxes in the world "
                                          "material are supported")
        hu = vol.load_image()
        db = self.volume_manager.material_database
        lut = M.material_to_label_lut(vol.material, vol.voxel_materials)
        names = sorted(lut, key=lut.get)
        labels = M.create_label_image(hu.array, vol.material, vol.voxel_materials, lut)
        if self.world.material not in names:
            names.append(self.world.material)
        for m in extra_materials:
            if m not in names:
                names.append(m)
        mats = [db.get(n) for n in names]
        pt = T.PhysicsTables(mats)
        spacing = hu.spacing
        size = np.array(hu.size, dtype=np.float64)
        corner = np.asarray(vol.translation, dtype=np.float64) - size * spacing / 2.0
        sources = [s for s in self.sources.values()]
        if not sources:
            raise ValueError("no source")
        specs = [s.to_spec(self.volumes, free_flight=free_flight) for s in sources]
        emax = max(sp.energy_bounds()[1] for sp in specs)
        self.physics_manager.check_supported(emax)
        half = [float(x) / 2.0 for x in self.world.size]
        scene = Scene(pt, labels, spacing, corner, half, names.index(self.world.material), specs[0])
        return scene, vol, hu, names, list(zip(sources, specs))

    def build_spect(self):
        """(scene, SpectSpec, sources, projection actors, head index per actor crystal) of a SPECT set-up."""
        from . import spect as S

        heads = [v for v in self.volumes.values() if isinstance(v, SpectHead)]
        if len(heads) > 2:
            raise NotImplementedError("at most two SPECT heads")
        h0 = heads[0]
        for h in heads[1:]:
            for k in ("collimator_type", "crystal_size", "radius", "step_angle_deg", "nb_angle", "gap"):
                if getattr(h, k) != getattr(h0, k):
                    raise NotImplementedError(f"SPECT heads must share '{k}'")
        runs = self.run_timing_intervals
        if h0.nb_angle not in (1, len(runs)):
            raise ValueError(f"rotate_gantry gave {h0.nb_angle} positions for {len(runs)} runs")
        step = h0.step_angle_deg if h0.nb_angle > 1 else 0.0
        projs = [a for a in self.actors.values() if isinstance(a, DigitizerProjectionActor)]
        arfs = [a for a in self.actors.values() if isinstance(a, ARFActor)]
        if projs and arfs:
            raise NotImplementedError("ARF detectors and projection actors in one simulation")
        if not projs and not arfs:
            raise ValueError("a SPECT simulation needs a DigitizerProjectionActor or an ARFActor")
        arf = None
        if arfs:
            # ARF detectors: the windows, adder and blurring are those the network was trained with
            from . import arf as ARF

            head_of = {h.name: i for i, h in enumerate(heads)}
            for a in arfs:
                a.check()
                if a.attached_to not in head_of:
                    raise ValueError(f"ARFActor '{a.name}' must be attached to a detection plane or head "
                                     f"({', '.join(head_of)})")
                if str(a.pth_filename) != str(arfs[0].pth_filename) or list(a.image_size) != \
                        list(arfs[0].image_size) or not np.allclose(a.image_spacing, arfs[0].image_spacing) or \
                        a.distance_to_crystal != arfs[0].distance_to_crystal:
                    raise NotImplementedError("ARF detectors must share the network, image size, spacing and "
                                              "distance to the crystal")
            model, params, meta = ARF.load_model(arfs[0].pth_filename)
            if meta["collimator_type"].lower() != str(h0.collimator_type).lower() or \
                    meta["crystal_size"] != str(h0.crystal_size):
                raise ValueError(f"network '{arfs[0].pth_filename}' was trained for a {meta['collimator_type']} "
                                 f"collimator and a {meta['crystal_size']} crystal, the heads have "
                                 f"{h0.collimator_type} / {h0.crystal_size}")
            if arfs[0].distance_to_crystal is not None:
                model.distance_to_crystal = float(arfs[0].distance_to_crystal) / u.mm
            arf = (model, params, meta)
            windows = [(float(a), float(b)) for a, b in np.asarray(meta["windows"])]
            size, spacing_in = arfs[0].image_size, arfs[0].image_spacing
        else:
            head_of = {h.crystal_name: i for i, h in enumerate(heads)}
            ewas = {a.attached_to: a for a in self.actors.values() if isinstance(a, DigitizerEnergyWindowsActor)}
            for a in projs:
                if a.attached_to not in head_of:
                    raise ValueError(f"projection actor '{a.name}' must be attached to a head crystal "
                                     f"({', '.join(head_of)})")
                if not a.channels and a.attached_to in ewas:
                    a.channels = ewas[a.attached_to].channels
                if a.channels != projs[0].channels or list(a.size) != list(projs[0].size) or \
                        not np.allclose(a.spacing, projs[0].spacing):
                    raise NotImplementedError("projection actors must share channels, size and spacing")
            channels = projs[0].channels
            windows = [(float(c["min"]) / u.MeV, float(c["max"]) / u.MeV) for c in channels]
            size, spacing_in = projs[0].size, projs[0].spacing
        housing = str(h0.housing)
        if any(str(h.housing) != housing for h in heads):
            raise NotImplementedError("heads with different housings")
        if arf is not None and str(arf[2].get("housing", "none")) != housing:
            raise ValueError(f"network '{arfs[0].pth_filename}' was trained for the housing "
                             f"'{arf[2].get('housing', 'none')}', the heads have '{housing}'")
        extra = [h0.collimator_material, h0.crystal_material] + list(S.HOUSING_MATERIALS.get(housing, ()))
        ffs = [a for a in self.actors.values() if isinstance(a, GammaFreeFlightActor)]
        sss = [a for a in self.actors.values() if isinstance(a, ScatterSplittingFreeFlightActor)]
        if len(ffs) + len(sss) > 1:
            raise NotImplementedError("one free-flight actor (GammaFreeFlightActor or ScatterSplittingFreeFlightActor)")
        scene, vol, hu, names, sources = self.build_scene(extra_materials=extra, free_flight=bool(ffs))
        coll = S.COLLIMATORS.get(str(h0.collimator_type).lower())
        if coll is None:
            raise NotImplementedError(f"collimator '{h0.collimator_type}'")
        spacing = [float(x) / u.mm for x in spacing_in]
        half_w = h0.half_width / u.mm if h0.half_width else None
        sp = S.SpectSpec(collimator=coll, crystal_thickness=S.CRYSTALS[h0.crystal_size], gap=h0.gap / u.mm,
                         radius=h0.radius / u.mm, n_heads=len(heads), n_runs=len(runs), windows=windows,
                         size=[int(x) for x in size], spacing=spacing,
                         step_angle_deg=step, collimator_material=names.index(h0.collimator_material),
                         crystal_material=names.index(h0.crystal_material),
                         head_start_deg=[h.start_angle_deg for h in heads])
        if half_w:
            sp.half_width = half_w
        sp.apply_housing(housing, names.index)
        sp.arf = arf
        # free flight (with ARF detectors too: the reference's recipes with ARF detectors)
        if ffs:
            ffs[0].check(heads)
            tols = {spec.ff_angle_tolerance for _, spec in sources}
            if len(tols) > 1:
                raise NotImplementedError("sources with different angle checks")
            sp.set_free_flight(float(ffs[0].weight_cutoff), float(ffs[0].energy_cutoff) / u.MeV,
                               angle_tolerance_max=tols.pop())
        if sss:
            ss = sss[0]
            ss.check(heads)
            nc, nr, tol = ss.factors()
            sp.set_scatter_splitting(nc, nr, int(ss.max_compton_level), float(ss.weight_cutoff),
                                     float(ss.energy_cutoff) / u.MeV, tol)
        if arf is not None:
            ARF.apply_head_meta(sp, arf[2])
            mods = [a.name for a in self.actors.values()
                    if isinstance(a, (DigitizerAdderActor, DigitizerBlurringActor, DigitizerSpatialBlurringActor))]
            if mods:
                raise NotImplementedError(f"with ARF detectors the digitizer is the network's own: remove {mods}")
            return scene, sp, sources, arfs, head_of
        # digitizer adder and blurring: one setting shared by every head's crystal
        def set_policy(policy):
            sp.adder_policy = policy

        for kind, setter, getter in ((DigitizerAdderActor, set_policy, "adder_policy"),
                                     (DigitizerBlurringActor, sp.set_energy_blur, "energy_blur"),
                                     (DigitizerSpatialBlurringActor, sp.set_spatial_blur, "spatial_blur")):
            mods = [a for a in self.actors.values() if isinstance(a, kind)]
            if not mods:
                continue
            for a in mods:
                if a.attached_to not in head_of:
                    raise ValueError(f"'{a.name}' must be attached to a head crystal ({', '.join(head_of)})")
            params = [getattr(a, getter)() for a in mods]
            if len({a.attached_to for a in mods}) != len(mods) or any(p != params[0] for p in params[1:]):
                raise NotImplementedError(f"one {kind.type_name} per head crystal, the same on every head")
            if isinstance(params[0], dict):
                setter(**params[0])
            else:
                setter(params[0])
        return scene, sp, sources, projs, head_of

    def _run_spect(self):
        """SPECT acquisition: heads + projection actors, one gantry position per run."""
        from .engine import SpectEngine

        t0 = time.perf_counter()
        scene, sp, sources, projs, head_of = self.build_spect()
        runs = self.run_timing_intervals
        spacing = sp.spacing
        seed = self._seed()
        self.last_seed = seed
        rng = np.random.default_rng(seed)
        plan = [events_per_run(src, runs, rng) for src, _ in sources]
        # a forced-direction source stands for one source copy per head: n_heads histories per event
        plan = [[k * sp.n_heads for k in p] if spec.dir_type == C.GG_DIR_FORCED else p
                for p, (_, spec) in zip(plan, sources)]
        writers = self._singles_writers(head_of) if sp.arf is None else {}
        eng = SpectEngine(scene, sp, device=self.device, precision=self.precision, batch=self.batch)
        singles = []
        try:
            if writers:
                eng.record_singles(SINGLES_LIST_CAPACITY)
            if sp.arf is not None:
                from .engine import ArfNetwork

                ArfNetwork(eng).set_model(sp.arf[0], sp.arf[1])
                eng.use_arf(True)
            first = 0
            for r in range(len(runs)):
                frames = np.ascontiguousarray(sp.frames(r), dtype=np.float64)
                eng._call("gg_spect_set_heads", r, C.ptr(frames, C.ctypes.c_double))
                for k, (src, spec) in enumerate(sources):
                    if len(sources) > 1 or k:
                        eng.set_source(spec)
                    # with a singles list, runs of at most capacity / n_heads histories (one single per
                    # head and history, scatter-split copies aside), each list read after its run
                    step = max(1, SINGLES_LIST_CAPACITY // sp.n_heads) if writers else max(plan[k][r], 1)
                    for a in range(0, plan[k][r], step):
                        m = min(step, plan[k][r] - a)
                        eng._call("gg_run", C.ctypes.c_uint64(m), C.ctypes.c_uint64(seed),
                                  C.ctypes.c_uint64(first + a))
                        if writers:
                            singles.append(eng.singles())
                    first += plan[k][r]
            if sp.arf is not None:
                # ARF detectors: network window weights plus the counts of the photons tracked instead
                counts = eng.projection()
                w, w2 = eng.arf_projection(squared=True)
                proj = (counts + w).astype(np.float32)
                proj2 = (counts + w2).astype(np.float32)
            elif sp.free_flight.enabled:
                proj, proj2 = eng.weighted_projection(squared=True)
            else:
                proj = eng.projection()
                proj2 = proj
            cnt = eng.counters()
        finally:
            eng.close()
        elapsed = time.perf_counter() - t0
        if writers:
            from . import root_io

            rec = np.concatenate(singles) if singles else np.zeros(0, dtype=C.SINGLE_DTYPE)
            # completion order is not reproducible: sort by history, head, then the values
            rec = rec[np.lexsort((rec["weight"], rec["a2"], rec["a1"], rec["energy"], rec["head"], rec["event_id"]))]
            for h, a in writers.items():
                path = pathlib.Path(self.output_dir) / (a.output_filename if a.output_filename not in
                                                        (None, "", "auto") else f"{a.name}.root")
                path.parent.mkdir(parents=True, exist_ok=True)
                root_io.write_tree(path, a.name, sp.singles_columns(rec[rec["head"] == h]))
                object.__setattr__(a, "singles", rec[rec["head"] == h])
        for a in projs:
            h = head_of[a.attached_to]
            sx, sy = spacing
            n0, n1 = (a.image_size if isinstance(a, ARFActor) else a.size)[:2]
            origin = [-n0 * sx / 2 + sx / 2, -n1 * sy / 2 + sy / 2, 0.0]
            img = image_io.Image(proj[h], [sx, sy, 1.0], origin)
            a.counts.image = img
            a.counts.number_of_samples = first
            a.counts_squared.image = image_io.Image(proj2[h].copy(), [sx, sy, 1.0], origin)
            a.counts_squared.number_of_samples = first
            if a.write_to_disk:
                path = a.counts.get_output_path()
                path.parent.mkdir(parents=True, exist_ok=True)
                image_io.write_mhd(path, img)
                if a.squared_counts.active:
                    image_io.write_mhd(a.squared_counts.get_output_path(), a.counts_squared.image)
        for a in self.actors.values():
            if isinstance(a, SimulationStatisticsActor):
                a.counts.runs = len(runs)
                a.counts.events = first
                a.counts.tracks = first
                a.counts.steps = cnt["woodcock_steps"] + cnt["world_steps"] + cnt["head_steps"]
                a.counts.duration = elapsed * u.s
                a.counts.pps = int(first / elapsed) if elapsed > 0 else 0
                a.counts.sps = int(a.counts.steps / elapsed) if elapsed > 0 else 0
        return cnt

    def _singles_writers(self, head_of):
        """{head index: actor} of the digitizer module whose singles collection goes to disk: the
        last of the chain adder -> energy blurring -> spatial blurring on each head crystal, as
        the GPU path applies them (the intermediate collections are not kept)."""
        last = {}
        for kind in (DigitizerAdderActor, DigitizerBlurringActor, DigitizerSpatialBlurringActor):
            for a in self.actors.values():
                if isinstance(a, kind) and a.attached_to in head_of:
                    last[head_of[a.attached_to]] = a
        return {h: a for h, a in last.items() if a.write_to_disk}

    def _arf_theta_max(self, actor, plane, source):
        """Largest angle (degrees) between the plane normal and a line from the source's disc to
        the plane: the angular domain of the training rows (capped to [1, 89] degrees)."""
        if actor.theta_max_deg is not None:
            return float(actor.theta_max_deg)
        pos = source.position
        if str(pos.type) not in ("disc", "point", "sphere"):
            return 85.0
        t = math.radians(plane.start_angle_deg)
        normal = np.array([math.sin(t), -math.cos(t), 0.0])
        centre = (plane.radius / u.mm) * normal
        src = np.asarray(pos.translation, dtype=np.float64) / u.mm
        depth = float(np.dot(src - centre, normal))
        if not depth > 0.0:
            return 85.0
        r = float(pos.radius) / u.mm if str(pos.type) != "point" else 0.0
        size = getattr(plane, "size", None)
        half_diag = 0.5 * math.hypot(size[0] / u.mm, size[1] / u.mm) if size is not None else plane.half_width
        lateral = float(np.linalg.norm((src - centre) - depth * normal))
        th = math.degrees(math.atan((r + lateral + half_diag) / depth))
        return float(min(max(th, 1.0), 89.0))

    def _run_arf_dataset(self):
        """ARF training rows (ARFTrainingDatasetActor): photons started on the detection plane,
        tracked through the head and the digitizer chain, one row per photon (class 0 rows
        Russian-rouletted), written to the actor's output file."""
        from . import arf as ARF
        from . import spect as S

        t0 = time.perf_counter()
        actors = [a for a in self.actors.values() if isinstance(a, ARFTrainingDatasetActor)]
        if len(actors) != 1:
            raise NotImplementedError("one ARFTrainingDatasetActor per simulation")
        act = actors[0]
        plane = self.volumes.get(act.attached_to)
        if not isinstance(plane, SpectHead):
            raise ValueError(f"ARFTrainingDatasetActor '{act.name}' must be attached to a detection plane "
                             "(add_detection_plane_for_arf) or a SPECT head")
        if list(act.plane_axis) != [0, 1, 2]:
            raise NotImplementedError("plane_axis other than [0, 1, 2]")
        ewa = self.actors.get(act.energy_windows_actor)
        if not isinstance(ewa, DigitizerEnergyWindowsActor):
            raise ValueError(f"The actor '{act.name}' has the user input energy_windows_actor="
                             f"{act.energy_windows_actor}, but no DigitizerEnergyWindowsActor of this name exists")
        chans = list(ewa.channels)
        for i, c1 in enumerate(chans):
            for j, c2 in enumerate(chans[i + 1:]):
                if check_channel_overlap(c1, c2):
                    raise ValueError(f"In the actor '{act.name}', the energy channels {i} and {i + 1 + j} overlap. "
                                     "This is not possible for ARF.")
        if not chans:
            raise ValueError(f"energy windows actor '{ewa.name}' has no channels")
        sources = list(self.sources.values())
        if len(sources) != 1 or sources[0].energy.type != "range":
            raise NotImplementedError("the ARF training dataset needs one GenericSource with energy.type 'range'")
        src = sources[0]
        e_min, e_max = float(src.energy.min_energy) / u.MeV, float(src.energy.max_energy) / u.MeV
        seed = self._seed()
        self.last_seed = seed
        rng = np.random.default_rng(seed)
        n = int(sum(events_per_run(src, self.run_timing_intervals, rng)))
        # head and digitizer: the plane's collimator / crystal, the windows, adder and blurring on its crystal
        sp = S.SpectSpec(collimator=S.COLLIMATORS[str(plane.collimator_type).lower()],
                         crystal_thickness=S.CRYSTALS[plane.crystal_size], gap=plane.gap / u.mm, n_heads=1,
                         n_runs=1, windows=[(float(c["min"]) / u.MeV, float(c["max"]) / u.MeV) for c in chans])
        sp.housing = str(plane.housing)  # recorded with the dataset; head_engine builds it
        # the digitizer modules on the windows actor's crystal (the plane's own, or that of a head
        # behind the plane as in the reference's set-up); the head geometry is the plane's
        for a in self.actors.values():
            if isinstance(a, (DigitizerAdderActor, DigitizerBlurringActor, DigitizerSpatialBlurringActor)):
                if a.attached_to != ewa.attached_to:
                    continue
                if isinstance(a, DigitizerAdderActor):
                    sp.adder_policy = a.adder_policy()
                elif isinstance(a, DigitizerBlurringActor):
                    sp.set_energy_blur(**a.energy_blur())
                else:
                    sp.set_spatial_blur(**a.spatial_blur())
        meta = ARF.head_meta(sp, plane.collimator_type, plane.crystal_size)
        theta_max = self._arf_theta_max(act, plane, src)
        size = getattr(plane, "size", None)
        half = [0.5 * float(size[0]) / u.mm, 0.5 * float(size[1]) / u.mm] if size is not None else [sp.half_width] * 2
        half = [min(h, sp.half_width) for h in half]
        from .engine import ArfNetwork

        eng, _ = ARF.head_engine(meta, device=self.device, precision=self.precision,
                                 collimator_material=plane.collimator_material,
                                 crystal_material=plane.crystal_material)
        with eng:
            smp = ArfNetwork.sampling(e_min, e_max, theta_max, half, float(act.russian_roulette))
            rows = ArfNetwork(eng).dataset(smp, n, seed)
            cnt = eng.counters()
        object.__setattr__(act, "rows", rows)
        object.__setattr__(act, "number_of_samples", n)
        object.__setattr__(act, "sampling", smp)
        if act.write_to_disk:
            ARF.save_dataset(act.get_output_path(), rows, meta, e_min, e_max, theta_max, act.russian_roulette)
        elapsed = time.perf_counter() - t0
        for a in self.actors.values():
            if isinstance(a, SimulationStatisticsActor):
                a.counts.runs = len(self.run_timing_intervals)
                a.counts.events = n
                a.counts.tracks = n
                a.counts.steps = cnt["head_steps"]
                a.counts.duration = elapsed * u.s
                a.counts.pps = int(n / elapsed) if elapsed > 0 else 0
        return cnt

    def run(self, start_new_process=False):
        from .engine import DoseEngine

        if any(isinstance(a, ARFTrainingDatasetActor) for a in self.actors.values()):
            return self._run_arf_dataset()
        if any(isinstance(v, SpectHead) for v in self.volumes.values()):
            return self._run_spect()
        t0 = time.perf_counter()
        scene, vol, hu, names, sources = self.build_scene()
        seed = self._seed()
        self.last_seed = seed
        rng = np.random.default_rng(seed)
        runs = self.run_timing_intervals
        plan = [events_per_run(src, runs, rng) for src, _ in sources]
        doses = [a for a in self.actors.values() if isinstance(a, DoseActor)]
        for a in doses:
            a.check(vol, hu)
        grids = {None if a.on_image_grid(hu) else tuple(map(tuple, a.scoring_grid(vol))) for a in doses}
        if len(grids) > 1:
            raise NotImplementedError("dose actors of one simulation must share their dose grid")
        grid = grids.pop() if grids else None
        if grid is not None and any(isinstance(a, TLEDoseActor) for a in doses):
            raise NotImplementedError("the TLEDoseActor scores on the image grid (size, spacing of the image)")
        if vol.dump_label_image:
            image_io.write_mhd(self.get_output_path(vol.dump_label_image),
                               image_io.Image(scene.labels, hu.spacing, hu.origin))
        goals = [a for a in doses if a.uncertainty_goal is not None]
        if len(goals) > 1:
            raise NotImplementedError("one DoseActor with an uncertainty goal")
        if goals and (len(sources) > 1 or len(runs) > 1):
            raise NotImplementedError("the uncertainty goal needs one source and one run")
        tles = [a for a in doses if isinstance(a, TLEDoseActor)]
        if tles and len(doses) > 1:
            raise NotImplementedError("a TLEDoseActor cannot share the run with another dose actor")
        eng = DoseEngine(scene, device=self.device, precision=self.precision, batch=self.batch)
        try:
            if grid is not None:
                eng.set_dose_grid(*grid, score_dose=True)
            if tles:
                eng.set_tle(tles[0].threshold_energy, float(tles[0].energy_min), tles[0].database)
            first = 0
            for r in range(len(runs)):
                for k, (src, spec) in enumerate(sources):
                    if len(sources) > 1:
                        eng.set_source(spec)
                    n = plan[k][r]
                    if not goals:
                        eng.run(n, seed, first)
                        first += n
                        continue
                    # uncertainty goal: GateDoseActor::EndOfEventAction (GateDoseActor.cpp:245-276)
                    g = goals[0]
                    n_next = int(g.uncertainty_first_check_after_n_events)
                    unc = 1.0
                    checks = []
                    while first < n:
                        todo = max(min(n_next, n) - first, 1)
                        eng.run(todo, seed, first)
                        first += todo
                        unc = D.compute_mean_uncertainty(eng.edep(), eng.edep_squared(), first,
                                                         g.uncertainty_voxel_edep_threshold,
                                                         g.uncertainty_top_voxels_count)
                        checks.append((first, unc))
                        object.__setattr__(g, "uncertainty_checks", checks)
                        if unc <= g.uncertainty_goal:
                            break
                        n_next = max(D.next_uncertainty_check(unc, g.uncertainty_goal, first,
                                                              g.uncertainty_overshoot_factor_N_events), first + 1)
                    object.__setattr__(g, "_uncertainty_reached", unc)
            edep, edep2, cnt = eng.edep(), eng.edep_squared(), eng.counters()
            if grid is not None:
                dsum, dsum2 = eng.dose_sum(), eng.dose_sum_squared()
        finally:
            eng.close()
        elapsed = time.perf_counter() - t0
        n_events = first
        rho = scene.voxel_density()
        for a in doses:
            spacing, origin, direction = a.output_geometry(vol, hu)
            if grid is None:
                dose = D.edep_to_dose(edep, rho, hu.spacing)
                dose2 = D.edep_to_dose(edep2, rho, hu.spacing, squared=True)
            else:
                dose = D.dose_sum_to_gy(dsum, grid[1])
                dose2 = D.dose_sum_to_gy(dsum2, grid[1], squared=True)
            data = {"edep": edep, "edep_squared": edep2,
                    "edep_uncertainty": D.variance_or_uncertainty(edep, edep2, n_events, "uncertainty"),
                    "dose": dose, "dose_squared": dose2,
                    "dose_uncertainty": D.variance_or_uncertainty(dose, dose2, n_events, "uncertainty")}
            if a.density.active:
                data["density"] = a.density_image(vol, hu, self.volume_manager.material_database,
                                                  spacing, origin, direction)
            for key, arr in data.items():
                out = getattr(a, key)
                out.image = image_io.Image(arr, spacing, origin, direction)
                out.number_of_samples = n_events
                if out.active and out.write_to_disk:
                    image_io.write_mhd(out.get_output_path(), out.image)
        for a in self.actors.values():
            if isinstance(a, SimulationStatisticsActor):
                a.counts.runs = len(runs)
                a.counts.events = n_events
                a.counts.tracks = n_events + cnt["secondaries"]
                a.counts.steps = cnt["woodcock_steps"] + cnt["world_steps"]
                a.counts.duration = elapsed * u.s
                a.counts.pps = int(n_events / elapsed) if elapsed > 0 else 0
                a.counts.sps = int(a.counts.steps / elapsed) if elapsed > 0 else 0
        return cnt
