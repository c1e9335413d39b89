"""ctypes binding of libgategpu.so (declarations in include/gate_gpu.h).

The shared library is built in-tree by ``opengate_gb300.build`` into
``opengate_gb300/_lib/libgategpu.so``.  Loading fails loudly when it is
missing: there is no CPU fallback for the transport path.
"""

import ctypes
import pathlib

import numpy as np

LIB_DIR = pathlib.Path(__file__).resolve().parent / "_lib"
LIB_PATH = LIB_DIR / "libgategpu.so"

GG_OK = 0
GG_ERR_ARG = 1
GG_ERR_CUDA = 2
GG_ERR_QUEUE_OVERFLOW = 3
GG_ERR_TIMEOUT = 4
GG_ERR_DOMAIN = 5
GG_ERR_STATE = 6
STATUS_NAMES = {0: "GG_OK", 1: "GG_ERR_ARG", 2: "GG_ERR_CUDA", 3: "GG_ERR_QUEUE_OVERFLOW",
                4: "GG_ERR_TIMEOUT", 5: "GG_ERR_DOMAIN", 6: "GG_ERR_STATE"}

GG_PREC_F32 = 32
GG_PREC_F64 = 64
GG_KERNEL_WAVEFRONT, GG_KERNEL_PHASED = 0, 1
GG_POS_POINT, GG_POS_BOX, GG_POS_SPHERE, GG_POS_DISC, GG_POS_VOXELS = 0, 1, 2, 3, 4
GG_DIR_ISO, GG_DIR_MOMENTUM, GG_DIR_FOCUSED, GG_DIR_FORCED = 0, 1, 2, 3
GG_ENE_MONO, GG_ENE_LINES, GG_ENE_HISTOGRAM, GG_ENE_RANGE = 0, 1, 2, 3
GG_IMG_EDEP, GG_IMG_EDEP_SQUARED, GG_IMG_DOSE, GG_IMG_DOSE_SQUARED = 0, 1, 2, 3
GG_N_COUNTERS = 16
COUNTER_NAMES = ["histories", "woodcock_steps", "real_interactions", "deposits", "tally_entries",
                 "list_overflows", "world_steps", "escaped", "skipped", "loop_capped",
                 "stack_overflow", "secondaries", "head_steps", "singles", "arf_photons", "arf_fallback"]

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u16p = ctypes.POINTER(ctypes.c_uint16)
_u64p = ctypes.POINTER(ctypes.c_uint64)


class TablesDesc(ctypes.Structure):
    _fields_ = [
        ("n_e", ctypes.c_int32), ("ln_emin", ctypes.c_float), ("inv_dln", ctypes.c_float),
        ("e_min", ctypes.c_float), ("e_max", ctypes.c_float), ("n_comp", ctypes.c_int32),
        ("sig", _f32p), ("cum", _f32p), ("ray_amax", _f32p), ("n_ray", ctypes.c_int32),
        ("ray_x2", _f32p), ("ray_cum", _f32p), ("n_mat", ctypes.c_int32), ("mat_comp", _i32p),
        ("mat_rho", _f32p),
    ]


GG_BLUR_NONE, GG_BLUR_GAUSSIAN, GG_BLUR_INVERSE_SQUARE, GG_BLUR_LINEAR = 0, 1, 2, 3


class BlurDesc(ctypes.Structure):
    _fields_ = [
        ("energy_method", ctypes.c_int32), ("energy_sigma", ctypes.c_double),
        ("energy_resolution", ctypes.c_double), ("energy_reference", ctypes.c_double),
        ("energy_slope", ctypes.c_double), ("spatial", ctypes.c_int32), ("spatial_sigma", ctypes.c_double * 2),
        ("keep_in_solid_limits", ctypes.c_int32), ("truncated", ctypes.c_int32),
    ]


FF_OFF, FF_PRIMARY, FF_SCATTER = 0, 1, 2
MAX_SPLITTING = 4096


class FfDesc(ctypes.Structure):
    _fields_ = [("enabled", ctypes.c_int32), ("weight_cutoff", ctypes.c_double), ("energy_cutoff", ctypes.c_double),
                ("compton_splitting", ctypes.c_int32), ("rayleigh_splitting", ctypes.c_int32),
                ("max_compton_level", ctypes.c_int32), ("angle_tolerance_max", ctypes.c_double)]


class TleDesc(ctypes.Structure):
    _fields_ = [
        ("enabled", ctypes.c_int32), ("threshold_energy", ctypes.c_double), ("energy_min", ctypes.c_double),
        ("muen", _f32p),
    ]


class DoseGridDesc(ctypes.Structure):
    _fields_ = [
        ("dims", ctypes.c_int32 * 3), ("spacing", ctypes.c_double * 3), ("corner", ctypes.c_double * 3),
        ("score_dose", ctypes.c_int32),
    ]


class VolumeDesc(ctypes.Structure):
    _fields_ = [
        ("dims", ctypes.c_int32 * 3), ("spacing", ctypes.c_double * 3),
        ("corner", ctypes.c_double * 3), ("labels", _u16p), ("majorant", _f32p),
    ]


class WorldDesc(ctypes.Structure):
    _fields_ = [("half_size", ctypes.c_double * 3), ("material", ctypes.c_int32)]


class SourceDesc(ctypes.Structure):
    _fields_ = [
        ("pos_type", ctypes.c_int32), ("translation", ctypes.c_double * 3),
        ("rotation", ctypes.c_double * 9), ("half_size", ctypes.c_double * 3),
        ("radius", ctypes.c_double), ("dir_type", ctypes.c_int32), ("theta", ctypes.c_double * 2),
        ("phi", ctypes.c_double * 2), ("momentum", ctypes.c_double * 3),
        ("focus", ctypes.c_double * 3), ("n_accept", ctypes.c_int32), ("accept_boxes", _f64p),
        ("max_rejection", ctypes.c_int32), ("ene_type", ctypes.c_int32), ("mono", ctypes.c_double),
        ("n_spec", ctypes.c_int32), ("spec_e", _f64p), ("spec_cdf", _f64p),
        ("e_lo", ctypes.c_double), ("e_hi", ctypes.c_double),
        ("vox_dims", ctypes.c_int32 * 3), ("vox_spacing", ctypes.c_double * 3),
        ("vox_corner", ctypes.c_double * 3), ("cdf_z", _f32p), ("cdf_y", _f32p), ("cdf_x", _f32p),
        ("fd_cos_min", ctypes.c_double), ("fd_cos_max", ctypes.c_double),
    ]


class SpectDesc(ctypes.Structure):
    _fields_ = [
        ("half_width", ctypes.c_double), ("collimator_thickness", ctypes.c_double), ("gap", ctypes.c_double),
        ("crystal_thickness", ctypes.c_double), ("hole_apothem", ctypes.c_double),
        ("pitch_x", ctypes.c_double), ("pitch_y", ctypes.c_double),
        ("collimator_material", ctypes.c_int32), ("crystal_material", ctypes.c_int32),
        ("n_windows", ctypes.c_int32), ("window_lo", ctypes.c_double * 8), ("window_hi", ctypes.c_double * 8),
        ("size", ctypes.c_int32 * 2), ("spacing", ctypes.c_double * 2), ("n_heads", ctypes.c_int32),
        ("n_runs", ctypes.c_int32), ("adder_policy", ctypes.c_int32),
        ("n_cover", ctypes.c_int32), ("cover_thickness", ctypes.c_double), ("cover_material", ctypes.c_int32),
        ("n_back", ctypes.c_int32), ("back_thickness", ctypes.c_double * 4), ("back_material", ctypes.c_int32 * 4),
        ("shielded_sides", ctypes.c_int32),
    ]


GG_ADDER_WINNER, GG_ADDER_CENTROID = 0, 1
ADDER_POLICIES = {"EnergyWinnerPosition": GG_ADDER_WINNER, "EnergyWeightedCentroidPosition": GG_ADDER_CENTROID}


class ArfSampling(ctypes.Structure):
    _fields_ = [
        ("e_min", ctypes.c_double),
        ("e_max", ctypes.c_double),
        ("cos_theta_max", ctypes.c_double),
        ("half_extent", ctypes.c_double * 2),
        ("russian_roulette", ctypes.c_double),
        ("theta_uniform", ctypes.c_int32),
    ]


class ArfModel(ctypes.Structure):
    _fields_ = [
        ("n_classes", ctypes.c_int32),
        ("x_mean", ctypes.c_float * 3),
        ("x_std", ctypes.c_float * 3),
        ("russian_roulette", ctypes.c_double),
        ("e_min", ctypes.c_double),
        ("e_max", ctypes.c_double),
        ("theta_max_deg", ctypes.c_double),
        ("distance_to_crystal", ctypes.c_double),
    ]


class ArfTrainOpts(ctypes.Structure):
    _fields_ = [
        ("n_samples", ctypes.c_uint64),
        ("seed", ctypes.c_uint64),
        ("init_seed", ctypes.c_uint64),
        ("batch", ctypes.c_int32),
        ("epochs", ctypes.c_int32),
        ("lr", ctypes.c_float),
        ("beta1", ctypes.c_float),
        ("beta2", ctypes.c_float),
        ("eps", ctypes.c_float),
        ("lr_final", ctypes.c_float),
    ]


class SimDescC(ctypes.Structure):
    _fields_ = [
        ("volume", VolumeDesc),
        ("source", SourceDesc),
        ("n_primaries", ctypes.c_uint64),
        ("seed", ctypes.c_uint64),
    ]


GG_ARF_N_PARAMS = 35600


class DeviceOpts(ctypes.Structure):
    _fields_ = [
        ("device", ctypes.c_int32), ("precision", ctypes.c_int32), ("block_size", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32), ("chunk", ctypes.c_int32), ("batch", ctypes.c_int64),
        ("refill_min", ctypes.c_int32), ("interact_min", ctypes.c_int32),
    ]


class AutotuneResult(ctypes.Structure):
    _fields_ = [("points", ctypes.c_int32), ("repeats", ctypes.c_int32), ("median_ms", ctypes.c_double),
                ("min_ms", ctypes.c_double), ("max_ms", ctypes.c_double), ("default_median_ms", ctypes.c_double)]


def ptr(arr, ctype):
    """Pointer to a contiguous numpy array (the caller keeps ``arr`` alive)."""
    if arr is None:
        return ctypes.cast(None, ctypes.POINTER(ctype))
    assert arr.flags["C_CONTIGUOUS"]
    return arr.ctypes.data_as(ctypes.POINTER(ctype))


# gg_single (include/gate_gpu.h): one record of the singles list
SINGLE_DTYPE = np.dtype([("event_id", np.uint64), ("head", np.int32), ("run", np.int32), ("energy", np.float64),
                         ("a1", np.float64), ("a2", np.float64), ("weight", np.float64)], align=True)
assert SINGLE_DTYPE.itemsize == 48


# Exported symbols and their prototypes: (name, restype, argtypes)
PROTOTYPES = [
    ("gg_create", ctypes.c_int, [ctypes.POINTER(DeviceOpts), ctypes.POINTER(ctypes.c_void_p)]),
    ("gg_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("gg_last_error", ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    ("gg_upload_tables", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(TablesDesc)]),
    ("gg_upload_volume", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(VolumeDesc)]),
    ("gg_set_world", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(WorldDesc)]),
    ("gg_set_source", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SourceDesc)]),
    ("gg_add_dose_tally", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("gg_reset_tally", ctypes.c_int, [ctypes.c_void_p]),
    ("gg_set_tle", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(TleDesc)]),
    ("gg_run", ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]),
    ("gg_synchronize", ctypes.c_int, [ctypes.c_void_p]),
    ("gg_set_transport_kernel", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("gg_set_dose_grid", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DoseGridDesc)]),
    ("gg_get_image", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _f64p, ctypes.c_size_t]),
    ("gg_get_image_device", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p),
                                           ctypes.POINTER(ctypes.c_size_t)]),
    ("gg_get_counters", ctypes.c_int, [ctypes.c_void_p, _u64p, ctypes.c_size_t]),
    ("gg_host_alloc", ctypes.c_void_p, [ctypes.c_size_t]),
    ("gg_host_free", ctypes.c_int, [ctypes.c_void_p]),
    ("gg_last_kernel_ms", ctypes.c_int,
     [ctypes.c_void_p, _f64p, _f64p, _f64p, ctypes.POINTER(ctypes.c_int32)]),
    ("gg_spect_setup", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SpectDesc)]),
    ("gg_spect_set_blur", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BlurDesc)]),
    ("gg_spect_set_free_flight", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FfDesc)]),
    ("gg_spect_set_heads", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _f64p]),
    ("gg_spect_run", ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, _f64p]),
    ("gg_get_projection", ctypes.c_int, [ctypes.c_void_p, _f64p, ctypes.c_size_t]),
    ("gg_spect_record_singles", ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    ("gg_spect_get_singles", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
    ("gg_arf_train", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ArfSampling), ctypes.POINTER(ArfTrainOpts), ctypes.POINTER(ArfModel), _f64p]),
    ("gg_arf_train_rows", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_uint64, ctypes.POINTER(ArfModel),
      ctypes.POINTER(ArfTrainOpts), ctypes.POINTER(ArfModel), _f64p]),
    ("gg_arf_set_model", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ArfModel), ctypes.POINTER(ctypes.c_float)]),
    ("gg_arf_get_params", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_size_t]),
    ("gg_arf_predict", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_uint64, ctypes.POINTER(ctypes.c_float)]),
    ("gg_arf_gradient", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_uint64, ctypes.POINTER(ctypes.c_float), _f64p]),
    ("gg_batch_setup", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SimDescC), ctypes.c_int32]),
    ("gg_batch_run", ctypes.c_int, [ctypes.c_void_p]),
    ("gg_batch_capture", ctypes.c_int, [ctypes.c_void_p]),
    ("gg_batch_replay", ctypes.c_int, [ctypes.c_void_p]),
    ("gg_batch_autotune", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DeviceOpts)]),
    ("gg_batch_autotune_result", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AutotuneResult)]),
    ("gg_batch_get_image", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, _f64p, ctypes.c_size_t]),
    ("gg_spect_use_arf", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("gg_last_stage_ms", ctypes.c_int, [ctypes.c_void_p, _f64p, _f64p, _f64p]),
    ("gg_get_arf_projection", ctypes.c_int, [ctypes.c_void_p, _f64p, _f64p, ctypes.c_size_t]),
    ("gg_arf_dataset", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ArfSampling), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
      ctypes.POINTER(ctypes.c_float), ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
    ("gg_dose_run_noalloc", ctypes.c_int,
     [ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(TablesDesc), ctypes.POINTER(VolumeDesc),
      ctypes.POINTER(WorldDesc), ctypes.POINTER(SourceDesc), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
      ctypes.c_void_p, ctypes.c_void_p, _u64p, ctypes.c_char_p, ctypes.c_size_t]),
]

# limits of gg_dose_run_noalloc (include/gate_gpu.h)
GG_NOALLOC_MAX_VOXELS = 1 << 20
GG_NOALLOC_BATCH = 65536

_lib = None


def load():
    """Load libgategpu.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build the CUDA extension first "
            "(python -c 'import opengate_gb300.build as b; b.build()')"
        )
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, res, args in PROTOTYPES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class GGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def check(lib, ctx, status):
    if status != GG_OK:
        buf = ctypes.create_string_buffer(1024)
        lib.gg_last_error(ctx, buf, len(buf))
        raise GGError(status, buf.value.decode(errors="replace"))
