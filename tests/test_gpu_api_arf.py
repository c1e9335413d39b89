"""The reference's ARF workflow through the opengate-shaped API, on the GPU.

1. a training-dataset simulation (add_spect_head, add_digitizer_energy_windows,
   add_actor_for_arf_training_dataset, add_source_for_arf_training_dataset;
   contrib/spect/ge_discovery_nm670.py:994-1026) writes the rows file;
2. train_arf trains the network on those rows and writes the network file
   (the garf training step);
3. an acquisition with add_arf_detector on two heads loads the file and
   runs through Simulation.run().

The rows must equal the head engine's gg_arf_dataset rows for the same seed,
and the ARF images written by the acquisition must equal, value for value,
the tracked counts plus network weights of the same histories run directly
through the C ABI (gg_spect_use_arf).
"""

import numpy as np
import pytest

from .test_cpu_api_arf import LU177, _arf_sim, _dataset_sim

pytestmark = pytest.mark.gpu


def test_arf_train_save_load_acquire(tmp_path, built_lib):
    import ctypes

    from opengate_gb300 import _capi as C
    from opengate_gb300 import arf as ARF
    from opengate_gb300 import image_io
    from opengate_gb300 import units as U
    from opengate_gb300.engine import ArfNetwork, SpectEngine

    u = U.g4_units
    # 1. training dataset
    sim, plane, actor, src = _dataset_sim(tmp_path / "train", rr=20)
    sim.run_timing_intervals = [[0, 200 * u.s]]  # 1e5 Bq x 200 s: ~2e7 photons
    sim.random_seed = 123
    sim.run()
    path = actor.get_output_path()
    rows, meta, dom = ARF.load_dataset(path)
    assert len(rows) > 100_000 and abs(actor.number_of_samples - 20_000_000) < 30_000
    assert set(np.unique(rows[:, 3]).astype(int)) == {0, 1, 2, 3}
    smp = actor.sampling
    assert smp.e_min == pytest.approx(0.1) and smp.e_max == pytest.approx(0.23)
    assert smp.russian_roulette == 20.0 and 80.0 < dom["theta_max_deg"] <= 89.0
    eng, _ = ARF.head_engine(meta)
    with eng:
        again = ArfNetwork(eng).dataset(smp, actor.number_of_samples, 123)
    np.testing.assert_array_equal(rows, again)

    # 2. training (garf_train's step)
    model, loss = ARF.train_arf(path, tmp_path / "net.npz", epochs=3)
    assert np.all(np.isfinite(loss)) and loss[-1] < loss[0]
    assert model.n_classes == 4

    # 3. acquisition with ARF detectors
    acq, dets = _arf_sim(tmp_path / "acq", tmp_path / "net.npz", n=400_000, angles=2)
    for _, a in dets:
        a.squared_counts.active = True
    acq.random_seed = 777
    acq.run()
    scene, sp, sources, arfs, head_of = acq.build_spect()
    with SpectEngine(scene, sp) as e:
        ArfNetwork(e).set_model(sp.arf[0], sp.arf[1])
        e.use_arf(True)
        first = 0
        for r in range(sp.n_runs):
            frames = np.ascontiguousarray(sp.frames(r), dtype=np.float64)
            e._call("gg_spect_set_heads", r, C.ptr(frames, ctypes.c_double))
            e._call("gg_run", ctypes.c_uint64(400_000), ctypes.c_uint64(777), ctypes.c_uint64(first))
            first += 400_000
        counts = e.projection()
        w, w2 = e.arf_projection(squared=True)
        cnt = e.counters()
    assert cnt["arf_photons"] > 1000 and w.sum() > 0
    for plane_vol, a in dets:
        h = head_of[a.attached_to]
        got = image_io.read_mhd(a.counts.get_output_path()).array
        got2 = image_io.read_mhd(a.squared_counts.get_output_path()).array
        assert got.dtype == np.float32 and got.shape == (sp.n_runs * sp.n_windows, 64, 64)
        np.testing.assert_array_equal(got, (counts[h] + w[h]).astype(np.float32))
        np.testing.assert_array_equal(got2, (counts[h] + w2[h]).astype(np.float32))
    assert len(LU177) == sp.n_windows


@pytest.mark.parametrize("policy", ["Rejection", "ForceDirection"])
def test_free_flight_recipe_with_arf_detectors_through_the_api(tmp_path, built_lib, policy):
    """GammaFreeFlightActor + the source's angular acceptance (angle check 12 degrees, or the
    direction forced into the 12 degree cone of each head) + ARF detectors through
    Simulation.run(): the written images equal the weighted projection of the same histories
    run directly (free flight + gg_spect_use_arf)."""
    import ctypes

    from opengate_gb300 import _capi as C
    from opengate_gb300 import image_io
    from opengate_gb300.engine import ArfNetwork, SpectEngine

    from .test_cpu_api_arf import _ff_arf_sim, _model_file

    _model_file(tmp_path / "net.npz")
    n = 300_000
    sim, dets = _ff_arf_sim(tmp_path / "acq", tmp_path / "net.npz", deg=12.0, n=n)
    sim.sources["s"].direction.angular_acceptance.policy = policy
    for _, a in dets:
        a.squared_counts.active = True
    sim.random_seed = 4242
    sim.run()
    scene, sp, sources, arfs, head_of = sim.build_spect()
    assert sp.free_flight.enabled == C.FF_PRIMARY
    per_run = n * (sp.n_heads if policy == "ForceDirection" else 1)
    with SpectEngine(scene, sp) as e:
        ArfNetwork(e).set_model(sp.arf[0], sp.arf[1])
        e.use_arf(True)
        first = 0
        for r in range(sp.n_runs):
            frames = np.ascontiguousarray(sp.frames(r), dtype=np.float64)
            e._call("gg_spect_set_heads", r, C.ptr(frames, ctypes.c_double))
            e._call("gg_run", ctypes.c_uint64(per_run), ctypes.c_uint64(4242), ctypes.c_uint64(first))
            first += per_run
        counts = e.projection()
        w, w2 = e.arf_projection(squared=True)
        cnt = e.counters()
    assert counts.sum() == 0 and cnt["arf_photons"] > 100 and w.sum() > 0
    for _, a in dets:
        h = head_of[a.attached_to]
        got = image_io.read_mhd(a.counts.get_output_path()).array
        got2 = image_io.read_mhd(a.squared_counts.get_output_path()).array
        np.testing.assert_array_equal(got, w[h].astype(np.float32))
        np.testing.assert_array_equal(got2, w2[h].astype(np.float32))
