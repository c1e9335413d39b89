"""SPECT heads, gantry positions and the projection digitizer.

The head model follows the parallel-hole heads of the reference
(contrib/spect/ge_discovery_nm670.py:125-164 add_spect_head, 464-490
lehr_collimator_repeater; contrib/spect/siemens_intevo.py:367-410 for the
medium-energy collimator): a lead collimator slab with hexagonal holes
(G4Polyhedra, "radius" = apothem) repeated on two offset rectangular
lattices, then the NaI crystal.  Shielding, cover and back compartment are
not modelled (their backscatter contribution to the low windows is left out).

Digitizer: per event and head the crystal deposits are summed and placed at
the energy-winner position (GateDigiAdderInVolume::Update, EnergyWinnerPosition),
classified into energy windows [lo, hi) (GateDigitizerEnergyWindowsActor::
ApplyThreshold) and counted in the projection pixel of that position on the
detector plane (GateDigitizerProjectionActor::ProcessSlice), slice = window +
run * n_windows.

Gantry: head h at run r sits at angle theta = start + r * step + h * 360/n_heads
about the z axis; its outward normal is (sin theta, -cos theta, 0) (theta = 0:
anterior, -y), e1 = (cos theta, sin theta, 0), e2 = (0, 0, 1), and the
collimator front face is at ``radius`` from the axis.
"""

import math

import numpy as np

from . import _capi as C

# parallel-hole collimators: (hole apothem, hole length, pitch between adjacent holes) in mm
LEHR = dict(hole_apothem=0.75, collimator_thickness=35.0, hole_pitch=1.7)  # 1.5 mm holes, 0.2 mm septa
MELP = dict(hole_apothem=1.47, collimator_thickness=40.6, hole_pitch=4.08)  # 2.94 mm holes, 1.14 mm septa
MEGP = dict(hole_apothem=1.5, collimator_thickness=58.0, hole_pitch=4.05)  # 3 mm holes, 1.05 mm septa
HEGP = dict(hole_apothem=2.0, collimator_thickness=66.0, hole_pitch=5.8)  # 4 mm holes, 1.8 mm septa
COLLIMATORS = {"lehr": LEHR, "melp": MELP, "megp": MEGP, "hegp": HEGP, "he": HEGP}
CRYSTALS = {"3/8": 9.525, "5/8": 15.875}  # NaI thickness, mm

# Housing of the NM670 head (ge_discovery_nm670.py:215-262 add_spect_box): the
# aluminium cover in front of the crystal, then behind it the TiO2 reflector,
# the Pyrex back compartment, what is left of the lead cover's 101.375 mm and
# the steel shielding's 10 mm behind the lead cover; the side rims shield.
HOUSING_MATERIALS = {"nm670": ("Aluminium", "TiO2", "Pyrex66", "Lead", "Steel")}


def housing_layers(kind, crystal_thickness):
    """(cover, back) of a housing kind ("none" or "nm670") as (thickness mm, material name)."""
    if kind in (None, "none"):
        return None, []
    if kind != "nm670":
        raise NotImplementedError(f"head housing '{kind}'")
    alu, reflector, backside, lead_cover, shielding = 1.3, 1.2, 80.0, 101.375, 111.375
    lead_back = lead_cover - (alu + crystal_thickness + reflector) - backside
    return (alu, "Aluminium"), [(reflector, "TiO2"), (backside, "Pyrex66"), (lead_back, "Lead"),
                                (shielding - lead_cover, "Steel")]


class SpectSpec:
    def __init__(self, collimator=LEHR, crystal_thickness=9.525, gap=0.0, radius=250.0, n_heads=2,
                 n_runs=60, start_angle_deg=0.0, step_angle_deg=6.0, windows=((0.126, 0.154), (0.108, 0.126)),
                 size=(128, 128), spacing=(4.42, 4.42), collimator_material=0, crystal_material=0,
                 head_start_deg=None):
        if n_heads not in (1, 2):
            raise ValueError("1 or 2 heads")
        if len(windows) > 8:
            raise ValueError("at most 8 energy windows")
        self.hole_apothem = float(collimator["hole_apothem"])
        self.collimator_thickness = float(collimator["collimator_thickness"])
        pitch = float(collimator["hole_pitch"])
        # adjacent holes at 30 degrees: lattice repeat (2 pitch cos 30, pitch)
        self.pitch_x = 2.0 * pitch * math.cos(math.radians(30.0))
        self.pitch_y = pitch
        self.crystal_thickness = float(crystal_thickness)
        self.gap = float(gap)
        self.radius = float(radius)
        self.n_heads = int(n_heads)
        self.n_runs = int(n_runs)
        self.start_angle = math.radians(start_angle_deg)
        self.step_angle = math.radians(step_angle_deg)
        self.windows = [(float(a), float(b)) for a, b in windows]
        self.size = [int(v) for v in size]
        self.spacing = [float(v) for v in spacing]
        self.half_width = 0.5 * max(self.size[0] * self.spacing[0], self.size[1] * self.spacing[1])
        self.collimator_material = int(collimator_material)
        self.crystal_material = int(crystal_material)
        # start angle of each head (default: evenly spread from start_angle_deg)
        self.head_start = None if head_start_deg is None else [math.radians(a) for a in head_start_deg]
        # digitizer: adder policy of the singles' position, blurring (off by default)
        self.adder_policy = "EnergyWinnerPosition"
        self.blur = C.BlurDesc()
        # free flight outside the heads (set_free_flight); off by default
        self.free_flight = C.FfDesc(C.FF_OFF, -1.0, 0.0, 0, 0, 0, 0.0)
        # housing slabs and side shielding (set_housing); none by default
        self.cover = None
        self.back = []
        self.shielded_sides = False
        self.housing = "none"

    def set_energy_blur(self, method, sigma=0.0, resolution=0.0, reference=0.0, slope=0.0):
        """DigitizerBlurringActor on the singles' energy (MeV): method "Gaussian" (sigma),
        "InverseSquare" (resolution = FWHM/E at reference) or "Linear" (+ slope per MeV)."""
        kinds = {"Gaussian": C.GG_BLUR_GAUSSIAN, "InverseSquare": C.GG_BLUR_INVERSE_SQUARE,
                 "Linear": C.GG_BLUR_LINEAR}
        if method not in kinds:
            raise ValueError(f"blur_method must be one of {tuple(kinds)}, not {method!r}")
        self.blur.energy_method = kinds[method]
        self.blur.energy_sigma = float(sigma)
        self.blur.energy_resolution = float(resolution)
        self.blur.energy_reference = float(reference)
        self.blur.energy_slope = float(slope)

    def set_free_flight(self, weight_cutoff=-1.0, energy_cutoff=0.0, enabled=True, angle_tolerance_max=0.0):
        """GammaFreeFlightActor on the world with the heads excluded: no interaction outside
        the heads, weights exp(-optical depth), weighted projections (MeV for the cutoff).
        angle_tolerance_max (radians, 0 = off): the angle check of the source's angular
        acceptance - photons whose line enters a head further off its axis are dropped."""
        self.free_flight = C.FfDesc(C.FF_PRIMARY if enabled else C.FF_OFF, float(weight_cutoff),
                                    float(energy_cutoff), 0, 0, 0, float(angle_tolerance_max))

    def set_scatter_splitting(self, compton_splitting, rayleigh_splitting, max_compton_level=10,
                              weight_cutoff=-1.0, energy_cutoff=0.0, angle_tolerance_max=0.0):
        """ScatterSplittingFreeFlightActor on the world, the heads excluded and kill volumes:
        analog photons outside the heads, every Compton (up to max_compton_level) and Rayleigh
        re-sampled into compton_splitting / rayleigh_splitting weighted copies that fly freely
        to the heads; the analog photons die at the heads.  Projections are weighted (the
        scattered component; the primary one comes from set_free_flight).  angle_tolerance_max
        (radians, 0 = off): copies entering a head further off its axis are dropped."""
        nc, nr, lvl = int(compton_splitting), int(rayleigh_splitting), int(max_compton_level)
        if not (0 <= nc <= C.MAX_SPLITTING and 0 <= nr <= C.MAX_SPLITTING):
            raise ValueError(f"splitting factors must be in [0, {C.MAX_SPLITTING}]")
        if lvl < 0:
            raise ValueError("max_compton_level must be >= 0")
        self.free_flight = C.FfDesc(C.FF_SCATTER, float(weight_cutoff), float(energy_cutoff), nc, nr, lvl,
                                    float(angle_tolerance_max))

    def set_spatial_blur(self, sigma, keep_in_solid_limits=True, truncated=False):
        """DigitizerSpatialBlurringActor on the crystal position: sigma (mm) along the
        projection axes (a scalar for both)."""
        sg = [float(sigma)] * 2 if not hasattr(sigma, "__len__") else [float(v) for v in list(sigma)[:2]]
        self.blur.spatial = 1
        self.blur.spatial_sigma[0], self.blur.spatial_sigma[1] = sg
        self.blur.keep_in_solid_limits = int(bool(keep_in_solid_limits))
        self.blur.truncated = int(bool(truncated))

    @property
    def n_windows(self):
        return len(self.windows)

    def desc(self):
        d = C.SpectDesc()
        d.half_width = self.half_width
        d.collimator_thickness = self.collimator_thickness
        d.gap = self.gap
        d.crystal_thickness = self.crystal_thickness
        d.hole_apothem = self.hole_apothem
        d.pitch_x = self.pitch_x
        d.pitch_y = self.pitch_y
        d.collimator_material = self.collimator_material
        d.crystal_material = self.crystal_material
        d.n_windows = self.n_windows
        for k, (lo, hi) in enumerate(self.windows):
            d.window_lo[k] = lo
            d.window_hi[k] = hi
        d.size[:] = self.size
        d.spacing[:] = self.spacing
        d.n_heads = self.n_heads
        d.n_runs = self.n_runs
        if self.adder_policy not in C.ADDER_POLICIES:
            raise NotImplementedError(f"adder policy '{self.adder_policy}'")
        d.adder_policy = C.ADDER_POLICIES[self.adder_policy]
        if self.cover is not None:
            d.n_cover = 1
            d.cover_thickness, d.cover_material = float(self.cover[0]), int(self.cover[1])
        d.n_back = len(self.back)
        for k, (t, m) in enumerate(self.back):
            d.back_thickness[k], d.back_material[k] = float(t), int(m)
        d.shielded_sides = 1 if self.shielded_sides else 0
        return d

    def set_housing(self, cover=None, back=(), shielded_sides=True):
        """Head housing (ge_discovery_nm670.py:215-262): ``cover`` = (thickness mm, material
        index) between the gap and the crystal, ``back`` = up to four (thickness mm, material
        index) layers behind the crystal, outwards; ``shielded_sides``: the head's side faces
        absorb (the shielding box's lead / steel rims).  Indices into the scene's material
        table."""
        back = [(float(t), int(m)) for t, m in back]
        if len(back) > 4:
            raise ValueError("at most four layers behind the crystal")
        for t, _ in ([cover] if cover is not None else []) + back:
            if not t > 0:
                raise ValueError("housing layers need a positive thickness")
        self.cover = None if cover is None else (float(cover[0]), int(cover[1]))
        self.back = back
        self.shielded_sides = bool(shielded_sides)

    def apply_housing(self, kind, index_of):
        """set_housing for a housing kind ("none" or "nm670"); index_of(name) -> material index."""
        cover, back = housing_layers(kind, self.crystal_thickness)
        if cover is None and not back:
            self.set_housing(None, (), shielded_sides=False)
            self.housing = "none"
            return
        self.set_housing((cover[0], index_of(cover[1])), [(t, index_of(m)) for t, m in back], shielded_sides=True)
        self.housing = kind

    def housing_depth(self):
        """Depth of the head box behind the collimator front face (mm)."""
        return (self.collimator_thickness + self.gap + (self.cover[0] if self.cover else 0.0) +
                self.crystal_thickness + sum(t for t, _ in self.back))

    def angle(self, run, head):
        if self.head_start is not None:
            return self.head_start[head] + run * self.step_angle
        return self.start_angle + run * self.step_angle + head * 2.0 * math.pi / self.n_heads

    def frames(self, run):
        """[n_heads][12]: front-face centre, outward normal, e1, e2 (float64)."""
        out = np.zeros((self.n_heads, 12))
        for h in range(self.n_heads):
            t = self.angle(run, h)
            u = np.array([math.sin(t), -math.cos(t), 0.0])
            e1 = np.array([math.cos(t), math.sin(t), 0.0])
            out[h] = np.concatenate([self.radius * u, u, e1, [0.0, 0.0, 1.0]])
        return out

    def crystal_depth(self):
        """Depth of the crystal's mid-plane behind the collimator front face (mm)."""
        return (self.collimator_thickness + self.gap + (self.cover[0] if self.cover else 0.0) +
                0.5 * self.crystal_thickness)

    def singles_columns(self, singles):
        """Columns of a singles list (C.SINGLE_DTYPE records) under the reference's digi
        attribute names (one column per value; PostPosition split into _X/_Y/_Z, mm, world
        frame, on the crystal's mid-plane of the record's head and gantry position)."""
        frames = self.all_frames()  # [run][head][12]
        f = frames[singles["run"], singles["head"]] if len(singles) else np.zeros((0, 12))
        pos = (f[:, 0:3] + self.crystal_depth() * f[:, 3:6] + singles["a1"][:, None] * f[:, 6:9]
               + singles["a2"][:, None] * f[:, 9:12])
        return {"EventID": singles["event_id"].astype(np.int64), "RunID": singles["run"].astype(np.int32),
                "HeadID": singles["head"].astype(np.int32),
                "TotalEnergyDeposit": singles["energy"].astype(np.float64),
                "PostPosition_X": pos[:, 0].copy(), "PostPosition_Y": pos[:, 1].copy(),
                "PostPosition_Z": pos[:, 2].copy(), "Weight": singles["weight"].astype(np.float64)}

    def all_frames(self):
        return np.ascontiguousarray(np.stack([self.frames(r) for r in range(self.n_runs)]))

    def projection_shape(self):
        """(head, run * window, y, x), the slice order of the reference's projection image."""
        return self.n_heads, self.n_runs * self.n_windows, self.size[1], self.size[0]


def voxel_cdfs(activity):
    """(cdf_z, cdf_y, cdf_x) float32 arrays of an activity image [z][y][x].

    Restates compute_image_3D_CDF (opengate/image.py:313-360): normalise the
    image, cumulative sums along x per (z, y) row (normalised when the row sum
    is not zero), along y of the x-sums per z slice, and along z of the xy-sums.
    """
    a = np.asarray(activity, dtype=np.float64)
    a = a / np.sum(a)
    sumx = a.sum(axis=2)
    sumxy = sumx.sum(axis=1)
    cdf_x = np.cumsum(a, axis=2)
    last = cdf_x[:, :, -1:]
    cdf_x = np.divide(cdf_x, last, out=cdf_x.copy(), where=last != 0)
    cdf_y = np.cumsum(sumx, axis=1)
    lasty = cdf_y[:, -1:]
    cdf_y = np.divide(cdf_y, lasty, out=cdf_y.copy(), where=lasty != 0)
    cdf_z = np.cumsum(sumxy) / np.sum(sumxy)
    return (np.ascontiguousarray(cdf_z, np.float32), np.ascontiguousarray(cdf_y, np.float32),
            np.ascontiguousarray(cdf_x, np.float32))


# ---------------------------------------------------------------------------
# projection noise and efficiency (contrib/spect/spect_helpers.py:374-387, 480-536, 582-591)
def compute_poisson_relative_uncertainty(counts):
    """sqrt(counts) / counts, 0 where counts == 0."""
    c = np.asarray(counts, dtype=np.float64)
    return np.divide(np.sqrt(c), c, out=np.zeros_like(c), where=c != 0)


def compute_history_by_history_relative_uncertainty(img, img_squared, n):
    """sqrt((sum x^2 / n - (sum x / n)^2) / (n - 1)) / (sum x / n), 0 where the mean is 0."""
    mean = np.asarray(img, dtype=np.float64) / n
    variance = (np.asarray(img_squared, dtype=np.float64) / n - mean * mean) / (n - 1)
    return np.divide(np.sqrt(variance), mean, out=np.zeros_like(variance), where=mean != 0)


def compute_efficiency(uncert, duration):
    """1 / (sigma^2 * T), 0 where sigma == 0."""
    u = np.asarray(uncert, dtype=np.float64)
    return np.divide(np.ones_like(u), u * u * duration, out=np.zeros_like(u), where=u != 0)


def compute_zscore(ref_counts, test_counts, var_ref, var_test):
    """(test - ref) / sqrt(var_ref + var_test) where both counts are non-zero."""
    ref = np.asarray(ref_counts, dtype=np.float64)
    test = np.asarray(test_counts, dtype=np.float64)
    both = (ref != 0) & (test != 0)
    return np.divide(test - ref, np.sqrt(np.asarray(var_ref) + np.asarray(var_test)), out=np.zeros_like(ref),
                     where=both)


def compute_speedup(ref_uncert, test_uncert, ref_duration, test_duration):
    """Efficiency ratio eff(test) / eff(ref), 0 where eff(ref) == 0."""
    e_ref = compute_efficiency(ref_uncert, ref_duration)
    e_test = compute_efficiency(test_uncert, test_duration)
    return np.divide(e_test, e_ref, out=np.zeros_like(e_test), where=e_ref != 0)


def mean_relative_uncertainty(counts, counts_squared, n, frac=0.1):
    """Mean history-by-history relative sigma over pixels above frac * max counts."""
    c = np.asarray(counts, dtype=np.float64)
    if not c.any():
        return None
    rel = compute_history_by_history_relative_uncertainty(c, counts_squared, n)
    sel = c > frac * c.max()
    return float(rel[sel].mean())
