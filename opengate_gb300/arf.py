"""ARF files: training datasets and trained networks, and the training step.

The reference's ARF workflow has three steps
(opengate/contrib/spect/ge_discovery_nm670.py:994-1053,
opengate/actors/arfactors.py:33-453):

1. a simulation with an ``ARFTrainingDatasetActor`` writes, for photons
   crossing a detection plane in front of a SPECT head, the rows
   (E, Theta, Phi, window) of GateARFTrainingDatasetActor
   (core/opengate_core/opengate_lib/GateARFTrainingDatasetActor.cpp:76-137);
2. garf trains a network on those rows and saves it as a ``.pth`` file;
3. a simulation with an ``ARFActor`` loads the network and scores photons
   reaching the plane with their window probabilities.

Here step 2 is :func:`train_arf` on this library's tensor-core kernels
(``gg_arf_train_rows``) and the files are numpy archives of our own format:

* dataset (``.npz``): arrays ``E`` (MeV), ``Theta``, ``Phi`` (degrees),
  ``window`` (0 = no window, k = window k) - the reference's attribute names -
  plus the head and digitizer the rows were made with (collimator, crystal,
  energy windows, blurring) and the sampling domain (energy range, largest
  theta, Russian-roulette factor);
* network (``.npz``): the 35 600 parameters (layout of gg_arf_set_model),
  the input standardisation, the trained domain, the projection depth and
  the same head / digitizer description.

garf ``.pth`` files cannot be read (garf's network architecture and
pickled state are not part of this library); a ``.pth`` name raises.
"""

import pathlib

import numpy as np

from . import _capi as C

FORMAT_DATASET = "opengate_gb300.arf_dataset/1"
FORMAT_MODEL = "opengate_gb300.arf_model/1"

_BLUR_FIELDS = ("energy_method", "energy_sigma", "energy_resolution", "energy_reference", "energy_slope", "spatial",
                "keep_in_solid_limits", "truncated")


def _check_name(path, what):
    p = pathlib.Path(path)
    if p.suffix.lower() == ".pth":
        raise NotImplementedError(f"{what} '{p.name}': garf .pth files cannot be read or written by the GPU path; "
                                  "use a .npz file (opengate_gb300.arf format)")
    if p.suffix.lower() == ".root":
        raise NotImplementedError(f"{what} '{p.name}': ARF datasets are written as .npz files "
                                  "(E, Theta, Phi, window arrays)")
    return p


def head_meta(sp, collimator_type, crystal_size):
    """Description of the head and digitizer of a SpectSpec, stored with datasets and models."""
    b = sp.blur
    return {"collimator_type": str(collimator_type), "crystal_size": str(crystal_size), "gap": float(sp.gap),
            "housing": str(getattr(sp, "housing", "none")),
            "windows": np.asarray(sp.windows, dtype=np.float64).reshape(-1, 2),
            "adder_policy": str(sp.adder_policy),
            "blur": np.array([float(getattr(b, f)) for f in _BLUR_FIELDS] +
                             [float(b.spatial_sigma[0]), float(b.spatial_sigma[1])], dtype=np.float64)}


def apply_head_meta(sp, meta):
    """Sets the windows, adder policy and blurring of SpectSpec `sp` from a stored description."""
    sp.windows = [(float(a), float(b)) for a, b in np.asarray(meta["windows"]).reshape(-1, 2)]
    sp.adder_policy = str(meta["adder_policy"])
    vals = np.asarray(meta["blur"], dtype=np.float64)
    blur = C.BlurDesc()
    for f, v in zip(_BLUR_FIELDS, vals[: len(_BLUR_FIELDS)]):
        setattr(blur, f, int(v) if f in ("energy_method", "spatial", "keep_in_solid_limits", "truncated") else v)
    blur.spatial_sigma[0], blur.spatial_sigma[1] = float(vals[-2]), float(vals[-1])
    sp.blur = blur


def _meta_arrays(meta):
    return {"collimator_type": np.array(meta["collimator_type"]), "crystal_size": np.array(meta["crystal_size"]),
            "gap": np.float64(meta["gap"]), "housing": np.array(meta.get("housing", "none")),
            "windows": np.asarray(meta["windows"], dtype=np.float64),
            "adder_policy": np.array(meta["adder_policy"]), "blur": np.asarray(meta["blur"], dtype=np.float64)}


def _meta_from(z):
    return {"collimator_type": str(z["collimator_type"]), "crystal_size": str(z["crystal_size"]),
            "gap": float(z["gap"]), "housing": str(z["housing"]) if "housing" in z else "none",
            "windows": np.asarray(z["windows"]), "adder_policy": str(z["adder_policy"]),
            "blur": np.asarray(z["blur"])}


def save_dataset(path, rows, meta, e_min, e_max, theta_max_deg, russian_roulette):
    """Writes training rows [n][4] = (E MeV, theta deg, phi deg, window) with their head and domain."""
    p = _check_name(path, "ARF dataset")
    rows = np.asarray(rows, dtype=np.float32).reshape(-1, 4)
    p.parent.mkdir(parents=True, exist_ok=True)
    with open(p, "wb") as f:
        np.savez(f, format=np.array(FORMAT_DATASET), E=rows[:, 0], Theta=rows[:, 1], Phi=rows[:, 2],
                 window=rows[:, 3], e_min=np.float64(e_min), e_max=np.float64(e_max),
                 theta_max_deg=np.float64(theta_max_deg), russian_roulette=np.float64(russian_roulette),
                 **_meta_arrays(meta))
    return p


def load_dataset(path):
    """(rows [n][4] float32, meta, domain dict) of a dataset written by save_dataset."""
    p = _check_name(path, "ARF dataset")
    with np.load(p, allow_pickle=False) as z:
        if str(z["format"]) != FORMAT_DATASET:
            raise ValueError(f"{p}: not an ARF dataset of this library")
        rows = np.stack([z["E"], z["Theta"], z["Phi"], z["window"]], axis=1).astype(np.float32)
        dom = {k: float(z[k]) for k in ("e_min", "e_max", "theta_max_deg", "russian_roulette")}
        return np.ascontiguousarray(rows), _meta_from(z), dom


_MODEL_FIELDS = ("russian_roulette", "e_min", "e_max", "theta_max_deg", "distance_to_crystal")


def save_model(path, model, params, meta):
    """Writes a trained network (gg_arf_model + GG_ARF_N_PARAMS parameters) with its head description."""
    p = _check_name(path, "ARF model")
    params = np.ascontiguousarray(params, dtype=np.float32)
    if params.size != C.GG_ARF_N_PARAMS:
        raise ValueError(f"need {C.GG_ARF_N_PARAMS} parameters")
    p.parent.mkdir(parents=True, exist_ok=True)
    with open(p, "wb") as f:
        np.savez(f, format=np.array(FORMAT_MODEL), params=params, n_classes=np.int32(model.n_classes),
                 x_mean=np.array(list(model.x_mean), np.float32), x_std=np.array(list(model.x_std), np.float32),
                 **{k: np.float64(getattr(model, k)) for k in _MODEL_FIELDS}, **_meta_arrays(meta))
    return p


def load_model(path):
    """(gg_arf_model, params float32 [GG_ARF_N_PARAMS], meta) of a network written by save_model."""
    p = _check_name(path, "ARF model")
    with np.load(p, allow_pickle=False) as z:
        if str(z["format"]) != FORMAT_MODEL:
            raise ValueError(f"{p}: not an ARF network of this library")
        m = C.ArfModel()
        m.n_classes = int(z["n_classes"])
        m.x_mean[:] = [float(v) for v in z["x_mean"]]
        m.x_std[:] = [float(v) for v in z["x_std"]]
        for k in _MODEL_FIELDS:
            setattr(m, k, float(z[k]))
        params = np.ascontiguousarray(z["params"], dtype=np.float32)
        return m, params, _meta_from(z)


def head_spec(meta, n_runs=1, size=(128, 128), spacing=(4.42, 4.42), collimator_material=0, crystal_material=0,
              housing_index=None):
    """A one-head SpectSpec of the stored head description (housing_index(name) -> material
    index of the housing's materials, when it has one)."""
    from . import spect as S

    coll = S.COLLIMATORS.get(str(meta["collimator_type"]).lower())
    if coll is None:
        raise NotImplementedError(f"collimator '{meta['collimator_type']}'")
    sp = S.SpectSpec(collimator=coll, crystal_thickness=S.CRYSTALS[str(meta["crystal_size"])], gap=float(meta["gap"]),
                     n_heads=1, n_runs=n_runs, size=size, spacing=spacing, collimator_material=collimator_material,
                     crystal_material=crystal_material, windows=[tuple(w) for w in np.asarray(meta["windows"])])
    apply_head_meta(sp, meta)
    kind = str(meta.get("housing", "none"))
    if kind != "none":
        sp.apply_housing(kind, housing_index)
    return sp


def head_engine(meta, device=0, precision=32, world_material="G4_AIR", collimator_material="G4_Pb",
                crystal_material="G4_SODIUM_IODIDE"):
    """A SpectEngine holding only a head (a one-voxel world-material image stands in for the phantom):
    enough for the ARF dataset generation and for training."""
    from . import materials as M
    from . import tables as T
    from .engine import SpectEngine
    from .scene import Scene, SourceSpec

    from . import spect as S

    db = M.MaterialDatabase()
    hmats = list(S.HOUSING_MATERIALS.get(str(meta.get("housing", "none")), ()))
    names = [world_material, collimator_material, crystal_material] + hmats
    pt = T.PhysicsTables([db.get(n) for n in names])
    sp = head_spec(meta, collimator_material=1, crystal_material=2, housing_index=lambda m: 3 + hmats.index(m))
    src = SourceSpec()
    src.mono = 0.1
    scene = Scene(pt, np.zeros((1, 1, 1), np.uint16), [1.0] * 3, [-0.5] * 3, [2000.0] * 3, 0, src)
    return SpectEngine(scene, sp, device=device, precision=precision), sp


def train_arf(dataset_path, output_path, epochs=10, batch=8192, lr=2e-3, lr_final=1e-5, init_seed=1, device=0):
    """Trains the ARF network on a dataset file and writes the network file (the garf training step).

    Returns (gg_arf_model, loss per epoch)."""
    from .engine import ArfNetwork

    rows, meta, dom = load_dataset(dataset_path)
    eng, _ = head_engine(meta, device=device)
    with eng:
        net = ArfNetwork(eng)
        model, loss = net.train_rows(rows, dom["e_min"], dom["e_max"], dom["theta_max_deg"],
                                     dom["russian_roulette"], epochs=epochs, batch=batch, lr=lr, lr_final=lr_final,
                                     init_seed=init_seed)
        save_model(output_path, model, net.params(), meta)
    return model, loss


def arf_window_weights(counts_fallback, arf_weights):
    """Projection of an ARF detector: network window weights plus the counts of the photons
    tracked instead (outside the trained domain or entering through a side)."""
    return np.asarray(counts_fallback, dtype=np.float64) + np.asarray(arf_weights, dtype=np.float64)


__all__ = ["save_dataset", "load_dataset", "save_model", "load_model", "train_arf", "head_meta", "head_spec",
           "head_engine", "apply_head_meta"]
