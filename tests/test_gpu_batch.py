"""Batched simulations (one set of launches for many uneven dose simulations) on the GPU.

Every simulation of a batch must give exactly the images it gives when run
alone (same seed, histories from 0) - and therefore the oracle's - whatever
the batching, the CUDA-graph replay or the launch configuration chosen by the
autotuner.
"""

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import workloads as W

pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.oracle")


def small_batch(n_sims=5):
    _, sims = W.batched_phantoms(n_sims=n_sims, sides=(16, 24, 32), primaries_range=(2e4, 1e5), seed=7)
    return sims


def _images(b, k):
    return b.image(k, C.GG_IMG_EDEP), b.image(k, C.GG_IMG_EDEP_SQUARED)


def test_batched_simulations_equal_each_alone():
    from opengate_gb300.engine import BatchEngine, DoseEngine

    sims = small_batch()
    with BatchEngine(sims, batch=70_001) as b:
        b.run()
        got = [_images(b, k) for k in range(len(sims))]
        cnt = b.counters()
    total = {}
    begin = 0
    for k, (scene, n, seed) in enumerate(sims):
        # the batch flushes its tallies every 70 001 histories of the batch: the run
        # alone flushes at the same histories (same FP64 accumulation of edep^2)
        cuts = [c - begin for c in range(70_001, begin + n, 70_001) if c > begin]
        edges = [0, *cuts, n]
        with DoseEngine(scene) as e:
            for a, z in zip(edges[:-1], edges[1:]):
                e.run(z - a, seed, a)
            np.testing.assert_array_equal(got[k][0], e.edep())
            np.testing.assert_array_equal(got[k][1], e.edep_squared())
            for name, v in e.counters().items():
                total[name] = total.get(name, 0) + v
        begin += n
    assert cnt == total
    scene, n, seed = sims[1]
    e, e2, _ = O.run_dose(scene, n, seed, threads=8)
    np.testing.assert_array_equal(got[1][0], e)
    np.testing.assert_allclose(got[1][1], e2, rtol=1e-15, atol=0)


def test_graph_replay_and_autotune_keep_results():
    from opengate_gb300.engine import BatchEngine

    sims = small_batch(4)
    with BatchEngine(sims) as b:
        b.run()
        ref = [_images(b, k) for k in range(len(sims))]
        b.capture()  # a run of its own, discarded
        b.replay()
        for k in range(len(sims)):
            np.testing.assert_array_equal(_images(b, k)[0], ref[k][0])
            np.testing.assert_array_equal(_images(b, k)[1], ref[k][1])
        b.replay()  # replays accumulate
        np.testing.assert_array_equal(_images(b, 0)[0], 2 * ref[0][0])
        best = b.autotune()
        assert best.blocks_per_sm in (2, 3, 4) and best.chunk in (64, 256, 1024)
        res = b.autotune_result()
        assert res["points"] == 19 and res["repeats"] == 3
        assert res["min_ms"] <= res["median_ms"] <= res["max_ms"]
        assert res["median_ms"] <= res["default_median_ms"]
        b.run()
        for k in range(len(sims)):
            np.testing.assert_array_equal(_images(b, k)[0], ref[k][0])
