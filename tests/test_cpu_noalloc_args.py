"""Argument checks of gg_dose_run_noalloc, which run before any CUDA call.

The no-allocation dose run must reject the same inputs as the allocating
path (gg_upload_tables / gg_upload_volume / gg_set_source): a bad majorant,
a negative or non-finite attenuation entry, decreasing spectrum weights, and
image dimensions whose product would wrap a 64-bit count.  Every case here
returns GG_ERR_ARG with a message and never reaches the GPU, so the tests run
without one.
"""

import ctypes

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import workloads as W
from opengate_gb300.scene import Scene, SourceSpec


def _call(scene, tables=None, volume=None, source=None):
    lib = C.load()
    err = ctypes.create_string_buffer(512)
    st = lib.gg_dose_run_noalloc(
        0, None, ctypes.byref(tables or scene.tables_desc), ctypes.byref(volume or scene.volume_desc),
        ctypes.byref(scene.world_desc), ctypes.byref(source or scene.source_desc), 1000, 1, 0,
        ctypes.c_void_p(16), None, None, err, len(err))
    return st, err.value.decode()


@pytest.fixture(scope="module")
def scene(built_lib):
    C._lib = None
    return W.water_pencil(n=8)


def test_noalloc_rejects_wrapping_dims(scene):
    v = C.VolumeDesc.from_buffer_copy(scene.volume_desc)
    v.dims[0], v.dims[1], v.dims[2] = 1 << 21, 1 << 21, 1 << 22  # product wraps to 0 in 64 bits
    st, msg = _call(scene, volume=v)
    assert st == C.GG_ERR_ARG and "at most" in msg


@pytest.mark.parametrize("bad", [0.0, -1.0, float("nan"), float("inf")])
def test_noalloc_rejects_bad_majorant(scene, bad):
    maj = np.array(scene.majorant, dtype=np.float32).copy()
    maj[len(maj) // 2] = bad
    v = C.VolumeDesc.from_buffer_copy(scene.volume_desc)
    v.majorant = maj.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    st, msg = _call(scene, volume=v)
    assert st == C.GG_ERR_ARG and "majorant" in msg


@pytest.mark.parametrize("bad", [-1e-3, float("nan"), float("inf")])
def test_noalloc_rejects_bad_attenuation(scene, bad):
    sig = np.array(scene.pt.sig, dtype=np.float32).copy()
    sig.flat[5] = bad
    t = C.TablesDesc.from_buffer_copy(scene.tables_desc)
    t.sig = sig.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    st, msg = _call(scene, tables=t)
    assert st == C.GG_ERR_ARG and "attenuation" in msg


def test_noalloc_rejects_decreasing_spectrum(built_lib):
    C._lib = None
    base = W.water_pencil(n=8)
    src = SourceSpec()
    src.ene_type = C.GG_ENE_HISTOGRAM
    src.spec_e = np.array([0.1, 0.2, 0.3, 0.4])
    src.spec_cdf = np.array([0.25, 0.75, 1.0])
    sc = Scene(base.pt, base.labels, base.spacing, base.corner, base.world_half, base.world_material, src)
    s = C.SourceDesc.from_buffer_copy(sc.source_desc)
    cdf = np.array([0.5, 0.3, 1.0])
    s.spec_cdf = cdf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    st, msg = _call(sc, source=s)
    assert st == C.GG_ERR_ARG and "cumulative" in msg
