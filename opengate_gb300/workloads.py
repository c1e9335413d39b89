"""Synthetic, seeded workloads for the photon-transport path.

* :func:`water_pencil` - 64^3 HU-0 water cube, 2 mm voxels, world of air,
  1 MeV pencil beam from the centre of the entrance face along +z.
* :func:`ct_phantom` - 256 x 256 x 160 int16 CT image, 1.2 mm voxels: air
  outside an elliptic-cylinder body (semi-axes 160 x 110 mm) of soft tissue
  N(40, 20^2), two ellipsoidal lungs N(-800, 50^2), spine and rib cylinders
  U(700, 1200), five fat ellipsoids N(-90, 15^2).  The ten-interval HU table
  in ``data/ct10_*.txt`` maps it to materials through the
  HounsfieldUnit_to_material restatement.  Source: point at 100 cm SSD
  (anterior, along +y), 10 x 10 cm field at the isocentre plane (angular
  acceptance box), 60-bin histogram spectrum on [0.1, 6] MeV with density
  proportional to E exp(-E / 1.5 MeV).

Every array is generated from a numpy seed, so a workload is reproducible
bit for bit on any machine.
"""

import math
import pathlib

import numpy as np

from . import _capi as C
from . import materials as M
from . import tables as T
from .scene import Scene, SourceSpec

DATA = pathlib.Path(__file__).resolve().parent / "data"
CT10_MATERIALS = DATA / "ct10_materials.txt"
CT10_DENSITIES = DATA / "ct10_densities.txt"


def world_air_materials():
    db = M.MaterialDatabase()
    return db


def water_pencil(n=64, spacing=2.0, energy=1.0):
    """Water cube, pencil beam.  Returns a Scene (materials: 0 G4_WATER, 1 G4_AIR)."""
    db = M.MaterialDatabase()
    mats = [db.get("G4_WATER"), db.get("G4_AIR")]
    pt = T.PhysicsTables(mats)
    labels = np.zeros((n, n, n), dtype=np.uint16)
    half = n * spacing / 2.0
    src = SourceSpec()
    src.pos_type = C.GG_POS_POINT
    src.translation = [0.0, 0.0, -half]
    src.dir_type = C.GG_DIR_MOMENTUM
    src.momentum = [0.0, 0.0, 1.0]
    src.ene_type = C.GG_ENE_MONO
    src.mono = energy
    return Scene(pt, labels, [spacing] * 3, [-half] * 3, [1000.0, 1000.0, 1000.0], 1, src)


def ct_hu_image(seed=20240611, shape=(160, 256, 256), spacing=1.2):
    """int16 HU array [nz][ny][nx] of the synthetic CT phantom."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    x = (np.arange(nx) + 0.5) * spacing - nx * spacing / 2
    y = (np.arange(ny) + 0.5) * spacing - ny * spacing / 2
    z = (np.arange(nz) + 0.5) * spacing - nz * spacing / 2
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    hu = np.full(shape, -1000.0, dtype=np.float32)
    body = (X / 160.0) ** 2 + (Y / 110.0) ** 2 <= 1.0
    hu[body] = rng.normal(40.0, 20.0, size=int(body.sum()))
    # five fat ellipsoids inside the body
    for _ in range(5):
        cx, cy = rng.uniform(-110, 110), rng.uniform(-70, 70)
        cz = rng.uniform(-70, 70)
        ax, ay, az = rng.uniform(10, 25, size=3)
        m = ((X - cx) / ax) ** 2 + ((Y - cy) / ay) ** 2 + ((Z - cz) / az) ** 2 <= 1.0
        m &= body
        hu[m] = rng.normal(-90.0, 15.0, size=int(m.sum()))
    # two lungs
    for sx in (-1.0, 1.0):
        m = ((X - sx * 65.0) / 45.0) ** 2 + ((Y + 5.0) / 60.0) ** 2 + ((Z - 10.0) / 75.0) ** 2 <= 1.0
        hu[m] = rng.normal(-800.0, 50.0, size=int(m.sum()))
    # spine: cylinder along z, posterior (+y)
    m = (X / 16.0) ** 2 + ((Y - 72.0) / 16.0) ** 2 <= 1.0
    hu[m] = rng.uniform(700.0, 1200.0, size=int(m.sum()))
    # ribs: thin cylinders along z on an ellipse around the lungs
    for ang in np.deg2rad([-150, -120, -60, -30, 30, 60, 120, 150]):
        rx, ry = 132.0 * math.cos(ang), 92.0 * math.sin(ang)
        m = ((X - rx) / 6.0) ** 2 + ((Y - ry) / 6.0) ** 2 <= 1.0
        m &= np.abs(Z - 10.0) <= 70.0
        hu[m] = rng.uniform(700.0, 1200.0, size=int(m.sum()))
    return np.clip(np.rint(hu), -1024, 3000).astype(np.int16)


def ct_materials(density_tolerance=0.05):
    """Material list (label order) for the CT phantom: label 0 = G4_AIR."""
    db = M.MaterialDatabase()
    vm, _ = M.hounsfield_unit_to_material(db, density_tolerance, CT10_MATERIALS, CT10_DENSITIES)
    lut = M.material_to_label_lut("G4_AIR", vm)
    names = sorted(lut, key=lut.get)
    return vm, lut, [db.get(n) for n in names]


def spectrum_e_exp(n_bins=60, e_lo=0.1, e_hi=6.0, kt=1.5):
    """60-bin histogram: edges and normalised cumulative of w_i dE_i, w ~ E exp(-E/kT)."""
    edges = np.linspace(e_lo, e_hi, n_bins + 1)
    centres = 0.5 * (edges[1:] + edges[:-1])
    w = centres * np.exp(-centres / kt)
    # GateGenericSource::InitializeEnergy (GateGenericSource.cpp:583-644):
    # accumulate weight x bin width, normalise to the total
    acc = np.cumsum(w * np.diff(edges))
    return edges, acc / acc[-1]


def ct_phantom(seed=20240611, shape=(160, 256, 256), spacing=1.2, ssd=1000.0, field=100.0,
               density_tolerance=0.05):
    hu = ct_hu_image(seed, shape, spacing)
    vm, lut, mats = ct_materials(density_tolerance)
    labels = M.create_label_image(hu, "G4_AIR", vm, lut)
    pt = T.PhysicsTables(mats)
    nz, ny, nx = shape
    corner = [-nx * spacing / 2, -ny * spacing / 2, -nz * spacing / 2]
    src = SourceSpec()
    src.pos_type = C.GG_POS_POINT
    sad = ssd + 110.0  # body surface at y = -110 mm, isocentre at the origin
    src.translation = [0.0, -sad, 0.0]
    # iso directions (G4 convention: direction = -(sin t cos p, sin t sin p, cos t)),
    # rotated so the cone axis is +y: theta measured from -z in the local frame;
    # use a rotation that maps local -z to +y.
    src.dir_type = C.GG_DIR_ISO
    half_diag = math.atan(math.hypot(field / 2, field / 2) / sad)
    src.theta = [math.pi / 2 - half_diag, math.pi / 2 + half_diag]
    src.phi = [3 * math.pi / 2 - half_diag, 3 * math.pi / 2 + half_diag]
    # acceptance: the field plane, a thin box at the isocentre depth scaled to
    # the first plane in front of the image (y just below the image face)
    y_plane = corner[1] - 1.0
    scale = (y_plane + sad) / sad
    hf = field / 2 * scale
    src.accept_boxes = [((-hf, y_plane - 0.5, -hf), (hf, y_plane + 0.5, hf))]
    src.ene_type = C.GG_ENE_HISTOGRAM
    src.spec_e, src.spec_cdf = spectrum_e_exp()
    air = 0
    return Scene(pt, labels, [spacing] * 3, corner, [1500.0, 1500.0, 1500.0], air, src), hu


def activity_phantom(hu, spacing=1.2, seed=424242, n_spheres=6, background=1.0):
    """Activity image [z][y][x] on the CT grid: uniform background in the body plus hot spheres.

    Spheres: radius 5-20 mm, contrast 4-10 x background, centres drawn inside the
    body (soft tissue) away from its edge.  Units: relative activity per voxel.
    """
    rng = np.random.default_rng(seed)
    nz, ny, nx = hu.shape
    x = (np.arange(nx) + 0.5) * spacing - nx * spacing / 2
    y = (np.arange(ny) + 0.5) * spacing - ny * spacing / 2
    z = (np.arange(nz) + 0.5) * spacing - nz * spacing / 2
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    body = (X / 160.0) ** 2 + (Y / 110.0) ** 2 <= 1.0
    act = np.where(body, background, 0.0)
    zmax = nz * spacing / 2 - 25.0
    for _ in range(n_spheres):
        r = rng.uniform(5.0, 20.0)
        c = rng.uniform(4.0, 10.0)
        while True:
            cx, cy, cz = rng.uniform(-120, 120), rng.uniform(-80, 80), rng.uniform(-zmax, zmax)
            if (cx / (160.0 - r - 10)) ** 2 + (cy / (110.0 - r - 10)) ** 2 <= 1.0:
                break
        m = (X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2 <= r * r
        act[m] = background * c
    return act


# radionuclide photon lines (MeV, yield per decay)
TC99M = ([0.1405], [0.89])
LU177 = ([0.1129, 0.2084], [0.062, 0.104])


def spect_phantom(shape=(160, 256, 256), spacing=1.2, nuclide=TC99M, collimator=None, n_runs=60,
                  windows=((0.126, 0.154), (0.108, 0.126)), density_tolerance=0.05, seed=20240611,
                  housing="none"):
    """SPECT workload: CT phantom as attenuation map, body + sphere activity, two heads.

    Returns (scene, spect_spec, activity).  Materials: the CT labels, then
    G4_Pb (collimator) and G4_SODIUM_IODIDE (crystal), then the housing's
    (housing="nm670": the NM670 shielding box's cover, reflector, back
    compartment, lead and steel, and shielded sides).
    """
    from . import spect as S

    hu = ct_hu_image(seed, shape, spacing)
    vm, lut, mats = ct_materials(density_tolerance)
    labels = M.create_label_image(hu, "G4_AIR", vm, lut)
    db = M.MaterialDatabase()
    n_ct = len(mats)
    hmats = list(S.HOUSING_MATERIALS.get(housing, ())) if housing not in (None, "none") else []
    mats = mats + [db.get("G4_Pb"), db.get("G4_SODIUM_IODIDE")] + [db.get(m) for m in hmats]
    pt = T.PhysicsTables(mats)
    nz, ny, nx = shape
    corner = [-nx * spacing / 2, -ny * spacing / 2, -nz * spacing / 2]
    act = activity_phantom(hu, spacing)
    src = SourceSpec()
    src.set_activity_image(act, [spacing] * 3, corner)
    src.dir_type = C.GG_DIR_ISO
    src.ene_type = C.GG_ENE_LINES
    e, w = nuclide
    src.spec_e = np.array(e, dtype=np.float64)
    src.spec_cdf = np.cumsum(w) / np.sum(w)
    scene = Scene(pt, labels, [spacing] * 3, corner, [1500.0] * 3, 0, src)
    sp = S.SpectSpec(collimator=collimator or S.LEHR, n_runs=n_runs, windows=windows,
                     step_angle_deg=360.0 / n_runs, collimator_material=n_ct, crystal_material=n_ct + 1)
    if hmats:
        sp.apply_housing(housing, lambda name: n_ct + 2 + hmats.index(name))
    return scene, sp, act


# Slab HU values of the batched workload: one per interval of the CT10 table
# (air, lung, fat, water, muscle, soft tissue, three bone densities)
SLAB_HU = (-1000, -800, -90, 0, 40, 60, 300, 700, 1200)


def batched_phantoms(n_sims=48, seed=20241203, sides=(32, 48, 64, 96, 128), spacing_range=(1.0, 3.0),
                     energy_range=(0.05, 2.0), primaries_range=(1e5, 1e7), density_tolerance=0.05):
    """Uneven simulations of one batched launch: (tables, [(Scene, n_primaries, seed), ...]).

    Each simulation: a cube of `side` voxels (drawn from `sides`) with spacing
    uniform in spacing_range, 1-4 slabs along z of HU drawn from SLAB_HU
    (through the CT10 HU -> material table), a monoenergetic disc beam (1 cm
    radius, +z, on the entrance face) with energy log-uniform in energy_range
    and primaries log-uniform in primaries_range.  All simulations share the
    material table and the 1 m air world.
    """
    rng = np.random.default_rng(seed)
    vm, lut, mats = ct_materials(density_tolerance)
    pt = T.PhysicsTables(mats)
    out = []
    for k in range(n_sims):
        side = int(rng.choice(sides))
        sp = float(rng.uniform(*spacing_range))
        n_slabs = int(rng.integers(1, 5))
        cuts = np.sort(rng.choice(np.arange(1, side), size=n_slabs - 1, replace=False)) if n_slabs > 1 else []
        hu = np.zeros((side, side, side), np.int16)
        edges = [0, *cuts, side]
        for a, b in zip(edges[:-1], edges[1:]):
            hu[a:b] = int(rng.choice(SLAB_HU))
        labels = M.create_label_image(hu, "G4_AIR", vm, lut)
        half = side * sp / 2.0
        src = SourceSpec()
        src.pos_type = C.GG_POS_DISC
        src.radius = 10.0
        src.translation = [0.0, 0.0, -half - 1.0]
        src.dir_type = C.GG_DIR_MOMENTUM
        src.momentum = [0.0, 0.0, 1.0]
        src.ene_type = C.GG_ENE_MONO
        src.mono = float(np.exp(rng.uniform(np.log(energy_range[0]), np.log(energy_range[1]))))
        n = int(np.exp(rng.uniform(np.log(primaries_range[0]), np.log(primaries_range[1]))))
        scene = Scene(pt, labels, [sp] * 3, [-half] * 3, [500.0] * 3, 0, src)
        out.append((scene, n, int(seed) * 1000 + k))
    return pt, out
