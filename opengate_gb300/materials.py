"""Materials, HU -> material conversion and label images.

Mirrors the reference's material handling for image volumes:

* :func:`read_voxel_materials` restates opengate/geometry/materials.py:14-58;
* :func:`hounsfield_unit_to_material` restates ``HounsfieldUnit_to_material``
  and its helpers (opengate/geometry/materials.py:61-230): HU intervals from a
  materials table, densities linearly interpolated from a density table,
  ``n = max(1, ddiff / tol)`` density bins per interval (one for air),
  ceil'ed when not 1, each bin a new material ``<name>_<k>`` with the
  interval's normalised element weights and the density at the bin centre;
* :func:`material_to_label_lut` and :func:`create_label_image` restate
  ``ImageVolume.create_material_to_label_lut`` / ``create_label_image``
  (opengate/geometry/volumes.py:1144-1243): label 0 is the volume's own
  material, the sorted intervals get labels 1.. in order of first appearance,
  gaps and values below the first interval map to label 0.

Densities are in g/cm3 throughout this module.
"""

import os

import numpy as np

from . import xsection

# Element-name spelling used by the Schneider-format tables (the reference's
# ``elements_name_symbol`` in opengate/definitions.py).
ELEMENT_NAME_SYMBOL = {
    "Hydrogen": "H", "Carbon": "C", "Nitrogen": "N", "Oxygen": "O", "Sodium": "Na",
    "Magnesium": "Mg", "Phosphor": "P", "Phosphorus": "P", "Sulfur": "S",
    "Chlorine": "Cl", "Argon": "Ar", "Potassium": "K", "Calcium": "Ca",
    "Titanium": "Ti", "Copper": "Cu", "Zinc": "Zn", "Silver": "Ag", "Tin": "Sn",
    "Iodine": "I", "Lead": "Pb", "Iron": "Fe", "Aluminium": "Al", "Aluminum": "Al",
    "Silicon": "Si", "Fluorine": "F", "Tungsten": "W",
}


class Material:
    """A material: density (g/cm3) and element mass fractions (normalised)."""

    def __init__(self, name, density, symbols, fractions):
        if density <= 0:
            raise ValueError(f"material {name}: density must be > 0")
        fr = np.asarray(fractions, dtype=np.float64)
        if len(symbols) != len(fr) or len(fr) == 0 or np.any(fr < 0) or fr.sum() <= 0:
            raise ValueError(f"material {name}: invalid composition")
        self.name = name
        self.density = float(density)
        self.symbols = list(symbols)
        self.fractions = fr / fr.sum()
        self.z = [xsection.z_of_symbol(s) for s in self.symbols]

    def composition_key(self):
        """Key identifying the element composition (not the density)."""
        return tuple((z, round(float(f), 12)) for z, f in sorted(zip(self.z, self.fractions)))

    def __repr__(self):
        comp = ", ".join(f"{s}:{f:.4f}" for s, f in zip(self.symbols, self.fractions))
        return f"Material({self.name}, {self.density} g/cm3, {comp})"


# NIST compound compositions (mass fractions) and densities for the materials
# this path uses; values follow the NIST material tables that Geant4's
# G4NistMaterialBuilder encodes.
_NIST = {
    "G4_Galactic": (1e-25, ["H"], [1.0]),
    "G4_AIR": (0.00120479, ["C", "N", "O", "Ar"], [0.000124, 0.755267, 0.231781, 0.012827]),
    "G4_WATER": (1.0, ["H", "O"], [0.111894, 0.888106]),
    "G4_Pb": (11.35, ["Pb"], [1.0]),
    "G4_W": (19.3, ["W"], [1.0]),
    "G4_Al": (2.699, ["Al"], [1.0]),
    "G4_Cu": (8.96, ["Cu"], [1.0]),
    "G4_SODIUM_IODIDE": (3.667, ["Na", "I"], [0.153373, 0.846627]),
    "G4_LUNG_ICRP": (1.04, ["H", "C", "N", "O", "Na", "P", "S", "Cl", "K"],
                     [0.105, 0.083, 0.023, 0.779, 0.002, 0.001, 0.002, 0.003, 0.002]),
    "G4_ADIPOSE_TISSUE_ICRP": (0.95, ["H", "C", "N", "O", "Na", "S", "Cl"],
                               [0.114, 0.598, 0.007, 0.278, 0.001, 0.001, 0.001]),
    "G4_MUSCLE_SKELETAL_ICRP": (1.05, ["H", "C", "N", "O", "Na", "P", "S", "Cl", "K"],
                                [0.102, 0.143, 0.034, 0.710, 0.001, 0.002, 0.003, 0.001, 0.004]),
    "G4_TISSUE_SOFT_ICRP": (1.03, ["H", "C", "N", "O", "Na", "P", "S", "Cl", "K"],
                            [0.105, 0.256, 0.027, 0.602, 0.001, 0.002, 0.003, 0.002, 0.002]),
    "G4_BONE_CORTICAL_ICRP": (1.92, ["H", "C", "N", "O", "Na", "Mg", "P", "S", "Ca"],
                              [0.034, 0.155, 0.042, 0.435, 0.001, 0.002, 0.103, 0.003, 0.225]),
    "G4_GLASS_PLATE": (2.4, ["O", "Na", "Si", "Ca"], [0.4598, 0.0964, 0.3365, 0.1073]),
    "G4_PLEXIGLASS": (1.19, ["H", "C", "O"], [0.080538, 0.599848, 0.319614]),
}


# Materials of the SPECT head housing as the reference's GateMaterials.db
# defines them (opengate/contrib/GateMaterials.db: Aluminium, TiO2, Pyrex66,
# Lead, Steel): density g/cm3, element mass fractions.
_GATE_DB = {
    "Aluminium": (2.6989, ["Al"], [1.0]),
    "TiO2": (4.23, ["Ti", "O"], [0.5993, 0.4007]),
    "Pyrex66": (1.478, ["O", "Si", "Na", "P", "B", "Al"], [0.5386, 0.3768, 0.0297, 0.0042, 0.0401, 0.0106]),
    "Lead": (11.4, ["Pb"], [1.0]),
    "Steel": (7.86, ["C", "Mn", "Fe"], [0.002, 0.005, 0.993]),
}


class MaterialDatabase:
    """Named materials: NIST built-ins plus user materials added by weights."""

    def __init__(self):
        self._user = {}

    def add_material_weights(self, name, symbols, weights, density):
        """Same role as MaterialDatabase.add_material_weights (materials.py:855)."""
        self._user[name] = Material(name, density, symbols, weights)

    def __contains__(self, name):
        return name in self._user or name in _NIST or name in _GATE_DB

    def get(self, name):
        if name in self._user:
            return self._user[name]
        if name in _NIST:
            d, s, f = _NIST[name]
            return Material(name, d, s, f)
        if name in _GATE_DB:
            d, s, f = _GATE_DB[name]
            return Material(name, d, s, f)
        raise KeyError(f"unknown material '{name}'")


# ---------------------------------------------------------------------------
# HU tables (opengate/geometry/materials.py)
# ---------------------------------------------------------------------------
def read_voxel_materials(filename, def_mat="G4_AIR"):
    """Read ``[start, stop, material]`` rows; fill gaps with ``def_mat`` (materials.py:14-58)."""
    rows = []
    state = 0
    with open(os.path.abspath(filename)) as f:
        for line in f:
            for word in line.split():
                if word[0] == "#":
                    break
                if state == 0:
                    start, state = float(word), 1
                elif state == 1:
                    stop, state = float(word), 2
                else:
                    rows.append([start, stop, word])
                    state = 0
    rows = sorted(rows)
    out = []
    prev = rows[0][0]
    for r in rows:
        if prev and prev > r[0]:
            raise ValueError(f"intervals are not disjoint: {prev} {r}")
        if r[0] > r[1]:
            raise ValueError(f"wrong interval {r}")
        if not prev or prev == r[0]:
            out.append([prev, r[1], r[2]])
        else:
            out.append([prev, r[0], def_mat])
            out.append([prev, r[1], r[2]])
        prev = r[1]
    return out


def hu_read_materials_table(file_mat):
    """Parse a Schneider-format materials table (materials.py:61-98)."""
    elements = ["HU"]
    materials = []
    section = None
    with open(os.path.abspath(file_mat)) as f:
        for line in f:
            cur = None
            for i, word in enumerate(line.split()):
                if word[0] == "#":
                    break
                if word == "[Elements]":
                    section = "element"
                    break
                if word == "[/Elements]":
                    elements.append("name")
                    section = "table"
                    break
                if section is None:
                    break
                if section == "element":
                    elements.append(word)
                    continue
                cur = cur if cur is not None else {}
                if i == 0:
                    cur[elements[i]] = int(word)
                elif i == len(elements) - 1:
                    cur[elements[i]] = word
                else:
                    cur[elements[i]] = float(word)
            if cur:
                materials.append(cur)
    return materials, elements


def hu_read_density_table(file_density):
    """Parse ``HU density`` rows (materials.py:101-113)."""
    out = []
    with open(os.path.abspath(file_density)) as f:
        for line in f:
            w = line.split()
            if not w or w[0][0] == "#":
                continue
            out.append({"HU": float(w[0]), "density": float(w[1])})
    return out


def hu_linear_interpolate_densities(hu, densities):
    """Piecewise-linear density at ``hu``, clamped at the table ends (materials.py:116-129)."""
    n = len(densities)
    i = 0
    while i < n and hu > densities[i]["HU"]:
        i += 1
    i -= 1
    if i < 0:
        return densities[0]["density"]
    if i >= n - 1:
        return densities[n - 1]["density"]
    a, b = densities[i], densities[i + 1]
    return ((hu - a["HU"]) / (b["HU"] - a["HU"])) * (b["density"] - a["density"]) + a["density"]


def hu_find_max_density_difference(hu_min, hu_max, d_min, d_max, densities):
    """Density span over table nodes inside [hu_min, hu_max] (materials.py:132-146)."""
    n = len(densities)
    i = 0
    while i < n and hu_min > densities[i]["HU"]:
        i += 1
    j = 0
    while j < n and hu_max > densities[j]["HU"]:
        j += 1
    j -= 1
    for x in range(i, j):
        d_min = min(d_min, densities[x]["density"])
        d_max = max(d_max, densities[x]["density"])
    return d_max - d_min


def hounsfield_unit_to_material(material_db, density_tolerance, file_mat, file_density):
    """Restatement of HounsfieldUnit_to_material (materials.py:149-230).

    ``density_tolerance`` is in g/cm3.  Returns ``(voxel_materials,
    created_material_names)`` and registers the new materials in
    ``material_db``.
    """
    materials, elements = hu_read_materials_table(file_mat)
    densities = hu_read_density_table(file_density)
    elems = elements[1:-1]
    symbols = [ELEMENT_NAME_SYMBOL[x] for x in elems]
    voxel_materials, created = [], []
    num = 0
    last = len(materials) - 1
    for i, mat in enumerate(materials):
        hu_min = mat["HU"]
        hu_max = hu_min + 1 if i == last else materials[i + 1]["HU"]
        if hu_max <= hu_min:
            raise ValueError(f"HU interval not valid: {mat}")
        dmin = hu_linear_interpolate_densities(hu_min, densities)
        dmax = hu_linear_interpolate_densities(hu_max, densities)
        ddiff = hu_find_max_density_difference(hu_min, hu_max, dmin, dmax, densities)
        n = max(1, ddiff / density_tolerance)
        if "Air" in mat["name"] or "AIR" in mat["name"]:
            n = 1
        htol = (hu_max - hu_min) / n
        if n != 1:
            n = int(np.ceil(n))
        for j in range(n):
            h1 = hu_min + j * htol
            h2 = min(hu_min + (j + 1) * htol, hu_max)
            d = hu_linear_interpolate_densities(h1 + (h2 - h1) / 2.0, densities)
            w_nz, s_nz = [], []
            for a, s in zip([mat[x] for x in elems], symbols):
                if a > 0:
                    w_nz.append(a)
                    s_nz.append(s)
            tot = sum(w_nz)
            w_nz = [w / tot for w in w_nz]
            name = f'{mat["name"]}_{num}'
            material_db.add_material_weights(name, s_nz, w_nz, d)
            voxel_materials.append([h1, h2, name])
            created.append(name)
            num += 1
    return voxel_materials, created


def material_to_label_lut(default_material, voxel_materials):
    """Material name -> label (volumes.py:1144-1168)."""
    lut = {default_material: 0}
    rows = sorted(voxel_materials, key=lambda r: r[0])
    lo = np.array([r[0] for r in rows])
    hi = np.array([r[1] for r in rows])
    if not (lo[1:] >= hi[:-1]).all():
        raise ValueError("overlapping intervals in voxel_materials")
    i = 1
    for r in rows:
        if r[2] not in lut:
            lut[r[2]] = i
            i += 1
    return lut


def create_label_image(hu, default_material, voxel_materials, lut=None):
    """uint16 label image from an HU array (volumes.py:1200-1243)."""
    if lut is None:
        lut = material_to_label_lut(default_material, voxel_materials)
    rows = sorted(voxel_materials, key=lambda r: r[0])
    bins = [r[0] for r in rows]
    extra = set(r[1] for r in rows).difference(bins)
    labels = [lut[r[2]] for r in rows]
    bins.extend(extra)
    labels.extend(len(extra) * [0])
    bins_sorted, labels_sorted = [], [0]
    for b, l in sorted(zip(bins, labels), key=lambda p: p[0]):
        bins_sorted.append(b)
        labels_sorted.append(l)
    return np.array(labels_sorted, dtype=np.uint16)[np.digitize(np.asarray(hu), bins=bins_sorted)]
