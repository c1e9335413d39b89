"""The C-ABI library builds for sm_103a, loads, and exports what include/gate_gpu.h declares.

No compute call is made here (there is no GPU); the scene/host validation
paths are exercised instead.
"""

import ctypes
import pathlib
import re

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import workloads as W
from opengate_gb300.scene import Scene, SourceSpec

HEADER = pathlib.Path(__file__).resolve().parents[1] / "include" / "gate_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^(?:int|void\s*\*)\s*(gg_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_api():
    names = declared_functions()
    assert "gg_create" in names and "gg_run" in names and "gg_get_image" in names
    assert set(names) == {n for n, _, _ in C.PROTOTYPES}


def test_library_builds_loads_and_exports_every_symbol(built_lib):
    lib = ctypes.CDLL(str(built_lib))
    for name in declared_functions():
        assert hasattr(lib, name), name
    # no GPU here: context creation must fail cleanly with a message
    C._lib = None
    L = C.load()
    ctx = ctypes.c_void_p()
    st = L.gg_create(None, ctypes.byref(ctx))
    if st != C.GG_OK:
        buf = ctypes.create_string_buffer(256)
        L.gg_last_error(None, buf, 256)
        assert buf.value  # an explanatory message
    else:  # a GPU is visible after all
        L.gg_destroy(ctx)


def test_ctypes_struct_layout_matches_header(tmp_path):
    """sizeof / offsetof from gcc on include/gate_gpu.h equal the ctypes mirror."""
    import subprocess

    structs = {"gg_tables_desc": C.TablesDesc, "gg_volume_desc": C.VolumeDesc, "gg_spect_desc": C.SpectDesc,
               "gg_world_desc": C.WorldDesc, "gg_source_desc": C.SourceDesc, "gg_device_opts": C.DeviceOpts,
               "gg_arf_sampling": C.ArfSampling, "gg_sim_desc": C.SimDescC, "gg_arf_model": C.ArfModel,
               "gg_arf_train_opts": C.ArfTrainOpts, "gg_tle_desc": C.TleDesc,
               "gg_ff_desc": C.FfDesc, "gg_blur_desc": C.BlurDesc, "gg_dose_grid_desc": C.DoseGridDesc}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("  return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                               check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(out[cname]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(out[f"{cname}.{fname}"]) == getattr(py, fname).offset, f"{cname}.{fname}"


def test_scene_validation():
    base = W.water_pencil(n=4)
    bad = base.labels.copy()
    bad[0, 0, 0] = 7
    with pytest.raises(ValueError):
        Scene(base.pt, bad, base.spacing, base.corner, base.world_half, 1, base.source)
    src = SourceSpec()
    src.mono = 50.0  # above the 20 MeV table
    with pytest.raises(ValueError):
        Scene(base.pt, base.labels, base.spacing, base.corner, base.world_half, 1, src)
    with pytest.raises(ValueError):
        Scene(base.pt, base.labels[0], base.spacing, base.corner, base.world_half, 1, base.source)


def test_majorant_bounds_every_material():
    sc, _ = W.ct_phantom(shape=(16, 32, 32), spacing=9.6)
    present = np.unique(sc.labels)
    mu = sc.pt.sig[sc.pt.mat_comp[present]] * sc.pt.mat_rho[present, None]
    assert np.all(sc.majorant[None, :] >= mu)


def test_host_alloc_symbols_need_no_gpu_to_load(built_lib):
    """gg_host_alloc / gg_host_free are exported with their prototypes (calling them needs
    the CUDA runtime and a device: covered by the GPU tests)."""
    lib = C.load()
    assert lib.gg_host_alloc.restype is ctypes.c_void_p
    assert lib.gg_host_free(None) == 0  # NULL is a no-op
