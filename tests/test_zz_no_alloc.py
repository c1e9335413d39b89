"""gg_dose_run_noalloc: the dose run that allocates no device memory.

It is meant for callers that cannot call cudaMalloc while they work (the
call synchronises the whole device, and a caller whose memory is already
handed out by its own pool may have none to spare).  Its scratch lives in a
static device array shared by all calls, so this test calls it twice in a
row through the C ABI and requires each result to equal, bit for bit, what
the allocating entry point (gg_run through DoseEngine) gives for the same
seed, histories and batch size: the second call also shows that the state
left by the first is cleared.  This file is collected last on purpose.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _descs(scene):
    return (ctypes.byref(scene.tables_desc), ctypes.byref(scene.volume_desc), ctypes.byref(scene.world_desc),
            ctypes.byref(scene.source_desc))


def test_noalloc_matches_allocating_run_on_two_calls(built_lib):
    import torch

    from opengate_gb300 import _capi as C
    from opengate_gb300 import workloads as W
    from opengate_gb300.engine import DoseEngine

    lib = C.load()
    scene = W.water_pencil()  # 64^3 voxels, below GG_NOALLOC_MAX_VOXELS
    n = 150000
    seeds = (20240611, 777)
    expected = []
    with DoseEngine(scene, precision=32, batch=C.GG_NOALLOC_BATCH) as eng:
        for seed in seeds:
            eng.reset()
            eng.run(n, seed, 0)
            expected.append((eng.edep(), eng.edep_squared(), eng.counters()))

    d_edep = torch.empty(scene.n_voxels, dtype=torch.float64, device="cuda:0")
    d_edep2 = torch.empty(scene.n_voxels, dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    for seed, (e_ref, e2_ref, c_ref) in zip(seeds, expected):
        cnt = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
        err = ctypes.create_string_buffer(512)
        st = lib.gg_dose_run_noalloc(0, None, *_descs(scene), n, seed, 0, ctypes.c_void_p(d_edep.data_ptr()),
                                     ctypes.c_void_p(d_edep2.data_ptr()), C.ptr(cnt, ctypes.c_uint64), err,
                                     len(err))
        assert st == C.GG_OK, err.value.decode()
        edep = d_edep.cpu().numpy().reshape(scene.labels.shape)
        edep2 = d_edep2.cpu().numpy().reshape(scene.labels.shape)
        assert np.array_equal(edep, e_ref), f"edep differs in {int(np.sum(edep != e_ref))} voxels"
        assert np.array_equal(edep2, e2_ref)
        counters = {name: int(cnt[i]) for i, name in enumerate(C.COUNTER_NAMES)}
        assert counters == c_ref
        assert counters["histories"] == n and edep.sum() > 0


def test_noalloc_rejects_oversized_image(built_lib):
    from opengate_gb300 import _capi as C
    from opengate_gb300.scene import Scene

    lib = C.load()
    small = __import__("opengate_gb300.workloads", fromlist=["x"]).water_pencil(n=8)
    big = Scene(small.pt, np.zeros((128, 128, 65), np.uint16), small.spacing, small.corner, small.world_half,
                small.world_material, small.source)
    assert big.n_voxels > C.GG_NOALLOC_MAX_VOXELS
    err = ctypes.create_string_buffer(512)
    st = lib.gg_dose_run_noalloc(0, None, *_descs(big), 1000, 1, 0, ctypes.c_void_p(16), None, None, err, len(err))
    assert st == C.GG_ERR_ARG
    assert b"at most" in err.value


def _box_spectrum_source():
    """Box source, isotropic within a cone, 20-bin histogram spectrum, one acceptance box."""
    import math

    from opengate_gb300 import _capi as C
    from opengate_gb300.scene import SourceSpec

    s = SourceSpec()
    s.pos_type = C.GG_POS_BOX
    s.translation = [0.0, 0.0, -90.0]
    s.half_size = [10.0, 8.0, 2.0]
    s.dir_type = C.GG_DIR_ISO
    s.theta = [math.pi - 0.35, math.pi]  # iso convention: theta = pi is +z, into the cube
    s.phi = [0.0, 2.0 * math.pi]
    s.accept_boxes = [((-8.0, -8.0, -64.0), (8.0, 8.0, -60.0))]
    s.ene_type = C.GG_ENE_HISTOGRAM
    s.spec_e = np.linspace(0.05, 2.0, 21)
    w = np.exp(-np.linspace(0.05, 2.0, 20))
    s.spec_cdf = np.cumsum(w) / w.sum()
    return s


@pytest.mark.parametrize("squared", [True, False])
def test_noalloc_box_spectrum_acceptance_matches(built_lib, squared):
    """Histogram spectrum (host float staging of the n+1 edges), box positions,
    acceptance boxes, and the run without the squared image (d_edep2 = NULL)."""
    import torch

    from opengate_gb300 import _capi as C
    from opengate_gb300 import workloads as W
    from opengate_gb300.engine import DoseEngine
    from opengate_gb300.scene import Scene

    lib = C.load()
    base = W.water_pencil()
    scene = Scene(base.pt, base.labels, base.spacing, base.corner, base.world_half, base.world_material,
                  _box_spectrum_source())
    n, seed = 100000, 4242
    with DoseEngine(scene, precision=32, batch=C.GG_NOALLOC_BATCH, score_squared=squared) as eng:
        eng.run(n, seed, 0)
        e_ref, c_ref = eng.edep(), eng.counters()
        e2_ref = eng.edep_squared() if squared else None
    d_edep = torch.empty(scene.n_voxels, dtype=torch.float64, device="cuda:0")
    d_edep2 = torch.empty(scene.n_voxels, dtype=torch.float64, device="cuda:0") if squared else None
    torch.cuda.synchronize()
    for _ in range(2):
        cnt = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
        err = ctypes.create_string_buffer(512)
        st = lib.gg_dose_run_noalloc(0, None, *_descs(scene), n, seed, 0, ctypes.c_void_p(d_edep.data_ptr()),
                                     ctypes.c_void_p(d_edep2.data_ptr()) if squared else None,
                                     C.ptr(cnt, ctypes.c_uint64), err, len(err))
        assert st == C.GG_OK, err.value.decode()
        edep = d_edep.cpu().numpy().reshape(scene.labels.shape)
        assert np.array_equal(edep, e_ref), f"edep differs in {int(np.sum(edep != e_ref))} voxels"
        if squared:
            assert np.array_equal(d_edep2.cpu().numpy().reshape(scene.labels.shape), e2_ref)
        counters = {name: int(cnt[i]) for i, name in enumerate(C.COUNTER_NAMES)}
        assert counters == c_ref
        assert counters["skipped"] > 0 and edep.sum() > 0
