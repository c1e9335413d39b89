"""Host logic and oracle numerics against the reference's own outputs.

The fixtures under tests/golden/ were produced by tests/golden/make_golden.py,
which executes the reference's functions (HounsfieldUnit_to_material,
ImageVolume.create_label_image, calculate_variance,
get_variance_or_uncertainty, PhotonAttenuationEl) on these inputs.
"""

import json
import math
import pathlib

import numpy as np
import pytest

from opengate_gb300 import dose as D
from opengate_gb300 import materials as M
from opengate_gb300 import xsection as X

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
DATA = pathlib.Path(__file__).resolve().parents[1] / "opengate_gb300" / "data"


# ---- Philox / elementary functions (oracle) --------------------------------
PHILOX_KAT = [  # Random123 known-answer vectors for philox4x32, 10 rounds
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expected", PHILOX_KAT)
@pytest.mark.parametrize("precision", [32, 64])
def test_philox_known_answers(ctr, key, expected, precision):
    from oracle import oracle as O

    assert tuple(O.philox(ctr, key, precision)) == expected


@pytest.mark.parametrize("precision,ulps", [(32, 4), (64, 8)])
def test_elementary_functions_vs_libm(precision, ulps):
    from oracle import oracle as O

    dt = np.float32 if precision == 32 else np.float64
    eps = float(np.finfo(dt).eps)
    rng = np.random.default_rng(5)
    for x in np.concatenate([rng.uniform(1e-7, 1.0, 3000), np.geomspace(1e-3, 20, 500)]).astype(dt):
        ref = math.log(float(x))
        assert abs(O.math_fn("log", x, precision) - ref) <= ulps * eps * max(abs(ref), 1.0)
    for x in rng.uniform(-20, 0.4, 3000).astype(dt):
        ref = math.exp(float(x))
        assert abs(O.math_fn("exp", x, precision) - ref) <= ulps * eps * ref
    for f in rng.uniform(0, 1, 3000).astype(dt):
        s, c = O.sincos_turn(f, precision)
        assert abs(s - math.sin(2 * math.pi * float(f))) <= ulps * eps
        assert abs(c - math.cos(2 * math.pi * float(f))) <= ulps * eps


# ---- NIST attenuation ----------------------------------------------------------
def test_nist_mu_matches_reference_photon_attenuation():
    g = np.load(GOLDEN / "nist_mu.npz")
    for i, z in enumerate(g["z"]):
        np.testing.assert_allclose(X.nist_mu_rho(int(z), g["energy"]), g["mu_rho"][i], rtol=1e-12)
        np.testing.assert_allclose(X.nist_mu_rho(int(z), g["energy"], absorption=True), g["muen_rho"][i],
                                   rtol=1e-12)


def test_partial_cross_sections_sum_to_nist_total():
    """Compton + photo + Rayleigh + pair reproduces the NIST total (photo is the remainder)."""
    e = np.geomspace(2e-3, 19.0, 60)
    for z in (1, 6, 8, 20, 53, 82):
        p = X.element_partials(z, e)
        tot = p["compton"] + p["photo"] + p["rayleigh"] + p["pair"]
        # exact where the remainder is >= 0; where the Compton/pair parameterisations
        # exceed NIST the total is above it by at most 1.5 %
        assert np.all(tot >= p["nist_total"] * (1 - 1e-12))
        assert np.all(tot <= p["nist_total"] * 1.015)


# ---- HU -> material and label image ------------------------------------------------
def _hu_case(name):
    return json.loads((GOLDEN / f"{name}.json").read_text())


@pytest.mark.parametrize("name", ["hu_schneider_tol0.1", "hu_schneider_tol0.05", "hu_ct10_tol0.05",
                                  "hu_ct10_tol0.2"])
def test_hounsfield_unit_to_material_matches_reference(name):
    g = _hu_case(name)
    ref_data = pathlib.Path(__file__).resolve().parent / "golden"
    fm = DATA / g["materials_file"] if (DATA / g["materials_file"]).exists() else None
    fd = DATA / g["densities_file"] if (DATA / g["densities_file"]).exists() else None
    if fm is None:
        # Schneider tables: the same files ship in the reference; reconstruct them from
        # the fixture's created materials is not possible, so use the copies the
        # fixture generator read (kept as raw text next to the fixtures).
        fm = ref_data / g["materials_file"]
        fd = ref_data / g["densities_file"]
        if not fm.exists():
            pytest.skip("Schneider tables not present")
    db = M.MaterialDatabase()
    vm, created = M.hounsfield_unit_to_material(db, g["tolerance"], fm, fd)
    assert created == g["created"]
    assert len(vm) == len(g["voxel_materials"])
    for a, b in zip(vm, g["voxel_materials"]):
        assert a[0] == b[0] and a[1] == b[1] and a[2] == b[2]
    for name_, ref in g["materials"].items():
        m = db.get(name_)
        assert m.density == ref["density"]
        assert m.symbols == ref["elements"]
        np.testing.assert_allclose(m.fractions, ref["weights"], rtol=1e-12)


def test_read_voxel_materials_matches_reference(tmp_path):
    g = json.loads((GOLDEN / "read_voxel_materials.json").read_text())
    p = tmp_path / "vm.txt"
    p.write_text(g["input"])
    assert M.read_voxel_materials(p) == g["output"]


@pytest.mark.parametrize("case", ["schneider", "ct10", "gaps"])
def test_label_image_matches_reference(case):
    g = np.load(GOLDEN / "labels.npz")
    vm = json.loads(str(g[f"{case}_vm"]))
    default = str(g[f"{case}_default"])
    lut = M.material_to_label_lut(default, vm)
    assert lut == json.loads(str(g[f"{case}_lut"]))
    labels = M.create_label_image(g[f"{case}_hu"], default, vm, lut)
    assert labels.dtype == np.uint16
    assert np.array_equal(labels, g[f"{case}_labels"])


def test_overlapping_intervals_rejected():
    with pytest.raises(ValueError):
        M.material_to_label_lut("G4_AIR", [[0, 10, "G4_WATER"], [5, 20, "G4_Pb"]])


# ---- DoseActor statistics --------------------------------------------------------
def test_variance_and_uncertainty_match_reference():
    g = np.load(GOLDEN / "variance.npz")
    n = int(g["n"])
    np.testing.assert_array_equal(D.calculate_variance(g["edep"], g["edep2"], n), g["variance"])
    for q in ("variance", "std", "uncertainty"):
        np.testing.assert_array_equal(D.variance_or_uncertainty(g["edep"], g["edep2"], n, q), g[q + "_item"])


def test_uncertainty_edge_cases():
    v = np.array([1.0, 0.0, 2.0])
    assert np.all(D.variance_or_uncertainty(v, v, 1, "uncertainty") == 1.0)
    assert np.all(D.variance_or_uncertainty(v, None, 10, "uncertainty") == 0.0)


def test_dose_units():
    # 1 MeV in 1 g of water: 1.602176634e-13 J / 1e-3 kg
    edep = np.array([1.0])
    dens = np.array([1.0])
    dose = D.edep_to_dose(edep, dens, (10.0, 10.0, 10.0))  # 1 cm3 = 1 g
    assert dose[0] == pytest.approx(1.602176634e-10, rel=1e-15)
    d2 = D.edep_to_dose(edep, dens, (10.0, 10.0, 10.0), squared=True)
    assert d2[0] == pytest.approx(1.602176634e-10 ** 2, rel=1e-14)
