"""GPU vs oracle on the full-size benchmark geometries, not reduced stand-ins.

The other GPU tests run shrunken phantoms; here every case uses the real
geometry of a benchmark workload at a history count the oracle finishes in
seconds on the host's cores:

* CT phantom (256 x 256 x 160 voxels of 1.2 mm, 60-bin 0.1-6 MeV spectrum,
  10 x 10 cm field at 100 cm SSD): 1e6 histories in FP32, 1e5 in FP64,
  edep, edep^2 and every counter identical (GateDoseActor.cpp:180-243,
  359-397);
* Tc-99m / LEHR SPECT on the same phantom, 2 heads x 60 gantry positions,
  4e5 decays per position: every projection pixel and counter identical
  (GateDigitizerProjectionActor.cpp:127-223);
* Lu-177 / MELP SPECT, 2 heads x 120 positions, with a network trained on
  the GPU and the ARF detectors on: tracked counts and counters identical,
  network window weights within FP32 / BF16 rounding of the oracle's;
* the 48 uneven slab simulations of the batched launch, all in one run:
  the simulations with the fewest primaries (and the one cut by the
  batch boundary) each equal the oracle's run of that simulation alone,
  flushed at the same histories.
"""

import os

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import spect as S
from opengate_gb300 import workloads as W

pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.oracle")
THREADS = max(1, os.cpu_count() or 1)
LU177_WINDOWS = ((0.1872, 0.2288), (0.166, 0.187), (0.1017, 0.1243))


@pytest.fixture(scope="module")
def ct_scene(built_lib):
    scene, _ = W.ct_phantom()
    assert scene.labels.shape == (160, 256, 256)
    return scene


def _same_dose(g, o):
    (ea, e2a, ca), (eb, e2b, cb) = g, o
    assert ca == cb, {k: (ca[k], cb[k]) for k in ca if ca[k] != cb[k]}
    assert np.array_equal(ea, eb), f"edep differs in {int(np.sum(ea != eb))} voxels"
    assert np.array_equal(e2a, e2b), f"edep^2 differs in {int(np.sum(e2a != e2b))} voxels"


@pytest.mark.parametrize("precision,n", [(32, 1_000_000), (64, 100_000)])
def test_ct_phantom_full_grid_bit_exact(ct_scene, precision, n):
    from opengate_gb300.engine import DoseEngine

    seed = 20240611
    with DoseEngine(ct_scene, precision=precision) as eng:
        eng.run(n, seed)
        g = (eng.edep(), eng.edep_squared(), eng.counters())
    o = O.run_dose(ct_scene, n, seed, threads=THREADS, precision=precision)
    _same_dose(g, o)
    assert g[2]["histories"] == n and g[2]["skipped"] > 0
    assert g[2]["tally_entries"] > n // 2


def test_tc99m_lehr_full_acquisition_bit_exact(built_lib):
    from opengate_gb300.engine import SpectEngine

    scene, sp, _ = W.spect_phantom()
    assert scene.labels.shape == (160, 256, 256) and sp.n_runs == 60 and sp.n_heads == 2
    n_per_run, seed = 400_000, 31
    with SpectEngine(scene, sp) as eng:
        eng.run(n_per_run, seed)
        proj, cnt = eng.projection(), eng.counters()
    ref, rcnt = O.run_spect(scene, sp, n_per_run, seed, threads=THREADS)
    assert proj.shape == ref.shape == sp.projection_shape()
    assert ref.sum() > 1000
    np.testing.assert_array_equal(proj, ref)
    assert cnt == rcnt


def test_lu177_melp_trained_arf_full_acquisition(built_lib):
    from opengate_gb300.engine import ArfNetwork, SpectEngine

    scene, sp, _ = W.spect_phantom(nuclide=W.LU177, collimator=S.MELP, n_runs=120, windows=LU177_WINDOWS)
    assert sp.n_runs == 120 and sp.n_windows == 3
    n_per_run, seed = 10_000, 77
    with SpectEngine(scene, sp) as eng:
        net = ArfNetwork(eng)
        smp = ArfNetwork.sampling(0.1017, 0.21, 85.0, (200.0, 200.0), 40.0)
        model, loss = net.train(smp, 20_000_000, seed=8, epochs=4, batch=8192, lr=2e-3, lr_final=1e-5)
        assert np.all(np.isfinite(loss)) and loss[-1] < loss[0]
        params = net.params()
        eng.use_arf(True)
        eng.reset()
        eng.run(n_per_run, seed)
        counts, (arf, arf2), cnt = eng.projection(), eng.arf_projection(squared=True), eng.counters()
    ref, rarf, rarf2, rcnt = O.run_spect_arf(scene, sp, n_per_run, seed, model, params, threads=THREADS)
    np.testing.assert_array_equal(counts, ref)
    assert cnt == rcnt
    assert cnt["arf_photons"] > 10_000 and arf.sum() > 0
    nw = sp.n_windows
    for got, want in ((arf, rarf), (arf2, rarf2)):
        close = np.isclose(got, want, rtol=4e-3, atol=2e-6 * want.max())
        assert close.mean() > 0.999
        assert np.abs(got - want).max() < 0.02
        for w in range(nw):
            tot, rtot = got[:, w::nw].sum(), want[:, w::nw].sum()
            assert abs(tot - rtot) <= 2e-4 * rtot + 1e-6


def test_batched_48_simulations_full_set(built_lib):
    from opengate_gb300.engine import BatchEngine

    _, sims = W.batched_phantoms()
    assert len(sims) == 48
    batch = 1 << 26  # the context's default tally batch
    begins = np.cumsum([0] + [n for _, n, _ in sims])
    with BatchEngine(sims) as b:
        b.run()
        cnt = b.counters()
        # the six smallest simulations and the one the batch boundary cuts
        order = sorted(range(len(sims)), key=lambda k: sims[k][1])[:6]
        cut = [k for k in range(len(sims)) if begins[k] < batch < begins[k + 1]]
        picks = sorted(set(order + cut))
        got = {k: (b.image(k, C.GG_IMG_EDEP), b.image(k, C.GG_IMG_EDEP_SQUARED)) for k in picks}
    assert cnt["histories"] == int(begins[-1])
    for k in picks:
        scene, n, seed = sims[k]
        cuts = [c - int(begins[k]) for c in range(batch, int(begins[k + 1]), batch) if c > begins[k]]
        edges = [0, *cuts, n]
        e = np.zeros(scene.labels.shape)
        e2 = np.zeros(scene.labels.shape)
        for a, z in zip(edges[:-1], edges[1:]):  # the oracle flushed at the same histories as the batch
            ea, e2a, _ = O.run_dose(scene, z - a, seed, first=a, threads=THREADS)
            e = e + ea
            e2 = e2 + e2a
        assert np.array_equal(got[k][0], e), (k, int(np.sum(got[k][0] != e)))
        assert np.array_equal(got[k][1], e2), k
