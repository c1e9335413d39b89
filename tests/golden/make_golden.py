"""Generate the golden fixtures in this directory from the reference's own code.

Run in a checkout that has the opengate sources (no Geant4 needed)::

    python tests/golden/make_golden.py /path/to/opengate

The opengate package cannot be imported without its compiled Geant4 core, so
this script lifts the pure-Python functions of the hot path out of the
reference sources with ``ast`` and executes them unchanged against small
stand-ins for ``itk`` (numpy arrays pass through) and ``opengate_core`` (not
used by these functions):

* opengate/geometry/materials.py: HU table readers and
  HounsfieldUnit_to_material (lines 14-230);
* opengate/geometry/volumes.py: ImageVolume.create_material_to_label_lut and
  ImageVolume.create_label_image (lines 1144-1243);
* opengate/utility.py: calculate_variance (lines 551-560);
* opengate/actors/dataitems.py:
  SingleItkImageWithVariance.get_variance_or_uncertainty (lines 1956-1993);
* opengate/data/PhotonAttenuation.py: PhotonAttenuationEl (NIST mu/rho);
* opengate/image.py: compute_image_3D_CDF (lines 313-360);
* opengate/contrib/spect/spect_helpers.py: projection noise and efficiency
  helpers (lines 374-387, 480-536, 582-591).

Outputs (small, committed): hu_*.json, labels.npz, variance.npz, nist_mu.npz,
voxel_cdf.npz, spect_metrics.npz.
"""

import ast
import json
import pathlib
import sys
import types

import numpy as np

OUT = pathlib.Path(__file__).resolve().parent


def _function_source(path, name, cls=None):
    tree = ast.parse(path.read_text())
    nodes = tree.body
    if cls is not None:
        nodes = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == cls).body
    node = next(n for n in nodes if isinstance(n, ast.FunctionDef) and n.name == name)
    return ast.get_source_segment(path.read_text(), node)


def _exec_functions(path, names, ns, cls=None):
    for name in names:
        src = _function_source(path, name, cls)
        exec(compile(src.replace("\n    ", "\n") if cls and src.startswith("    ") else src, str(path), "exec"), ns)
    return ns


class _FakeMaterialDB:
    def __init__(self):
        self.materials = {}

    def add_material_weights(self, name, elements, weights, density):
        self.materials[name] = {"elements": list(elements), "weights": [float(w) for w in weights],
                                "density": float(density)}


def _fatal(msg):
    raise RuntimeError(msg)


def hu_fixtures(ref):
    mat_py = ref / "opengate/geometry/materials.py"
    sys.path.insert(0, str(ref / "opengate"))
    defs_ns = {"np": np, "sys": sys}
    # elements_name_symbol lives in opengate/definitions.py (a plain dict literal)
    tree = ast.parse((ref / "opengate/definitions.py").read_text())
    for node in tree.body:
        if isinstance(node, ast.Assign) and node.targets[0].id == "elements_name_symbol":
            defs_ns["elements_name_symbol"] = ast.literal_eval(node.value)
    ns = {"np": np, "os": __import__("os"), "fatal": _fatal,
          "g4_units": types.SimpleNamespace(g_cm3=1.0),
          "elements_name_symbol": defs_ns["elements_name_symbol"]}
    _exec_functions(mat_py, ["read_voxel_materials", "HU_read_materials_table", "HU_read_density_table",
                             "HU_linear_interpolate_densities", "HU_find_max_density_difference",
                             "HounsfieldUnit_to_material"], ns)
    cases = {
        "hu_schneider_tol0.1": (ref / "opengate/data/Schneider2000MaterialsTable.txt",
                                ref / "opengate/data/Schneider2000DensitiesTable.txt", 0.1),
        "hu_schneider_tol0.05": (ref / "opengate/data/Schneider2000MaterialsTable.txt",
                                 ref / "opengate/data/Schneider2000DensitiesTable.txt", 0.05),
        "hu_ct10_tol0.05": (OUT.parent.parent / "opengate_gb300/data/ct10_materials.txt",
                            OUT.parent.parent / "opengate_gb300/data/ct10_densities.txt", 0.05),
        "hu_ct10_tol0.2": (OUT.parent.parent / "opengate_gb300/data/ct10_materials.txt",
                           OUT.parent.parent / "opengate_gb300/data/ct10_densities.txt", 0.2),
    }
    results = {}
    for key, (fm, fd, tol) in cases.items():
        db = _FakeMaterialDB()
        sim = types.SimpleNamespace(volume_manager=types.SimpleNamespace(material_database=db))
        vm, created = ns["HounsfieldUnit_to_material"](sim, tol, str(fm), str(fd))
        results[key] = {"tolerance": tol, "materials_file": fm.name, "densities_file": fd.name,
                        "voxel_materials": vm, "created": created, "materials": db.materials}
        (OUT / f"{key}.json").write_text(json.dumps(results[key], indent=1))
    # read_voxel_materials on a small text table with a gap
    tmp = OUT / "_voxel_materials_example.txt"
    tmp.write_text("# start stop material\n-1000 -500 G4_AIR\n-500 0 G4_LUNG_ICRP\n100 500 G4_WATER\n"
                   "500 2000 G4_BONE_CORTICAL_ICRP\n")
    vm = ns["read_voxel_materials"](str(tmp))
    (OUT / "read_voxel_materials.json").write_text(json.dumps({"input": tmp.read_text(), "output": vm}))
    tmp.unlink()
    return results


def label_fixtures(ref, hu_results):
    vol_py = ref / "opengate/geometry/volumes.py"
    ns = {"np": np, "fatal": _fatal}

    class _FakeImage(np.ndarray):
        def CopyInformation(self, other):
            pass

    ns["itk"] = types.SimpleNamespace(array_view_from_image=lambda im: np.asarray(im),
                                      image_from_array=lambda a: a.view(_FakeImage))
    for name in ("create_material_to_label_lut", "create_label_image"):
        src = _function_source(vol_py, name, cls="ImageVolume")
        src = "\n".join(line[4:] if line.startswith("    ") else line for line in src.splitlines())
        exec(compile(src, str(vol_py), "exec"), ns)
    rng = np.random.default_rng(7)
    out = {}
    cases = {
        "schneider": (hu_results["hu_schneider_tol0.1"]["voxel_materials"], "G4_AIR"),
        "ct10": (hu_results["hu_ct10_tol0.05"]["voxel_materials"], "G4_AIR"),
        "gaps": ([[-1000, -500, "G4_AIR"], [-400, 0, "G4_LUNG_ICRP"], [0, 300, "G4_WATER"],
                  [600, 1500, "G4_BONE_CORTICAL_ICRP"], [1500, 2500, "G4_WATER"]], "G4_Pb"),
    }
    for key, (vm, default) in cases.items():
        hu = rng.integers(-1100, 3100, size=(7, 11, 13)).astype(np.int16)
        hu.flat[:8] = [-1100, -1000, -999, 0, 300, 599, 1500, 3000]
        self = types.SimpleNamespace(material=default, voxel_materials=vm, material_to_label_lut=None,
                                     itk_image=hu, name="patient")
        self.create_material_to_label_lut = lambda material=None, voxel_materials=None, s=self: \
            ns["create_material_to_label_lut"](s, material, voxel_materials)
        lut = ns["create_material_to_label_lut"](self)
        self.material_to_label_lut = lut
        labels = np.asarray(ns["create_label_image"](self))
        out[f"{key}_hu"] = hu
        out[f"{key}_labels"] = labels.astype(np.uint16)
        out[f"{key}_lut"] = np.array(json.dumps(lut))
        out[f"{key}_vm"] = np.array(json.dumps(vm))
        out[f"{key}_default"] = np.array(default)
    np.savez_compressed(OUT / "labels.npz", **out)


def variance_fixtures(ref):
    ns = {"np": np}
    _exec_functions(ref / "opengate/utility.py", ["calculate_variance"], ns)
    src = _function_source(ref / "opengate/actors/dataitems.py", "get_variance_or_uncertainty",
                           cls="SingleItkImageWithVariance")
    src = "\n".join(line[4:] if line.startswith("    ") else line for line in src.splitlines())
    class _Img(np.ndarray):
        def CopyInformation(self, other):
            pass

    ns.update({"warning": lambda m: None, "fatal": _fatal,
               "itk_image_from_array": lambda a: np.asarray(a).view(_Img)})
    exec(compile(src, "dataitems.py", "exec"), ns)
    rng = np.random.default_rng(11)
    n = 1000
    edep = rng.gamma(0.3, 2.0, size=(6, 9, 10))
    edep[0, 0, :3] = 0.0
    edep2 = edep * edep / n + rng.gamma(0.5, 1.0, size=edep.shape) * edep
    edep2[0, 0, 3] = 0.0  # a voxel with variance below zero before clipping

    class _Item:
        def __init__(self, data, nos=None):
            self.data = data
            self.number_of_samples = nos

    def item_cls(data):
        return data

    me = types.SimpleNamespace(data=[_Item(edep.view(_Img), n), _Item(edep2.view(_Img))],
                               _data_item_classes=(item_cls,))
    out = {"edep": edep, "edep2": edep2, "n": np.array(n),
           "variance": ns["calculate_variance"](edep, edep2, n)}
    for q in ("variance", "std", "uncertainty"):
        out[q + "_item"] = np.asarray(ns["get_variance_or_uncertainty"](me, q))
    np.savez_compressed(OUT / "variance.npz", **out)


def nist_fixtures(ref):
    import importlib.util

    spec = importlib.util.spec_from_file_location("pa", ref / "opengate/data/PhotonAttenuation.py")
    pa = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pa)
    zs = np.array([1, 6, 7, 8, 11, 15, 20, 26, 53, 74, 82])
    es = np.geomspace(1.5e-3, 19.0, 40)
    mu = np.array([[pa.PhotonAttenuationEl(int(z), float(e), 1)[0] for e in es] for z in zs]).astype(np.float64)
    muen = np.array([[pa.PhotonAttenuationEl(int(z), float(e), 2)[0] for e in es] for z in zs]).astype(np.float64)
    np.savez_compressed(OUT / "nist_mu.npz", z=zs, energy=es, mu_rho=mu.reshape(len(zs), len(es)),
                        muen_rho=muen.reshape(len(zs), len(es)))


def voxel_cdf_fixtures(ref):
    """compute_image_3D_CDF (opengate/image.py:313-360) on an activity image with empty rows/slices."""
    ns = {"np": np, "itk": types.SimpleNamespace(array_from_image=lambda im: np.array(im))}
    _exec_functions(ref / "opengate/image.py", ["compute_image_3D_CDF"], ns)
    rng = np.random.default_rng(3)
    act = rng.gamma(0.6, 1.0, size=(6, 7, 9))
    act[2] = 0.0  # an empty z slice
    act[4, 3] = 0.0  # an empty row
    act[act < 0.2] = 0.0
    cdf_x, cdf_y, cdf_z = ns["compute_image_3D_CDF"](act)
    np.savez_compressed(OUT / "voxel_cdf.npz", activity=act, cdf_x=np.array(cdf_x), cdf_y=np.array(cdf_y),
                        cdf_z=np.array(cdf_z))


def spect_metric_fixtures(ref):
    """contrib/spect/spect_helpers.py: Poisson / history-by-history uncertainty, efficiency, z-score, speedup."""
    ns = {"np": np}
    _exec_functions(ref / "opengate/contrib/spect/spect_helpers.py",
                    ["compute_poisson_relative_uncertainty", "compute_efficiency",
                     "compute_history_by_history_relative_uncertainty", "compute_zscore", "compute_speedup"], ns)
    rng = np.random.default_rng(21)
    n = 5000
    counts = rng.poisson(3.0, size=(3, 8, 9)).astype(np.float64)
    counts2 = counts + rng.poisson(0.5, size=counts.shape) * counts  # multi-count events in some pixels
    test = rng.poisson(3.0, size=counts.shape).astype(np.float64)
    u_ref = ns["compute_history_by_history_relative_uncertainty"](counts, counts2, n)
    u_test = ns["compute_poisson_relative_uncertainty"](test)
    out = {"counts": counts, "counts2": counts2, "test": test, "n": np.array(n), "u_ref": u_ref, "u_test": u_test,
           "poisson": ns["compute_poisson_relative_uncertainty"](counts),
           "efficiency": ns["compute_efficiency"](u_ref, 12.5),
           "zscore": ns["compute_zscore"](counts, test, (u_ref * counts) ** 2, (u_test * test) ** 2),
           "speedup": ns["compute_speedup"](u_ref, u_test, 12.5, 0.8)}
    np.savez_compressed(OUT / "spect_metrics.npz", **out)


def main(ref):
    ref = pathlib.Path(ref)
    # the Schneider 2000 HU tables are inputs of the HU fixtures; keep copies of
    # these two data files next to the fixtures so the tests do not need the
    # opengate sources
    for name in ("Schneider2000MaterialsTable.txt", "Schneider2000DensitiesTable.txt"):
        (OUT / name).write_text((ref / "opengate/data" / name).read_text())
    hu = hu_fixtures(ref)
    label_fixtures(ref, hu)
    variance_fixtures(ref)
    nist_fixtures(ref)
    voxel_cdf_fixtures(ref)
    spect_metric_fixtures(ref)
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <root of the opengate source tree>")
    main(sys.argv[1])
