"""ARF detectors combined with free flight, GPU against the oracle.

The reference's ARF recipes run the primary component with free flight and
an angular acceptance at the source (contrib/spect/spect_config.py:937-970,
biasing/GateGammaFreeFlightOptn.cpp:34-83) and the scatter component with
scatter splitting; with ARF detectors every photon reaching a head face is
scored by the network (arfactors.py:349-453).  Here a photon (or split copy)
that reaches a face inside the trained domain adds its free-flight weight
times the network's window weights; the others are tracked through the head
with their weight.  Tracked counts and every counter must equal the
oracle's; the weighted projections agree within the FP32 / BF16 rounding of
the network (the tolerances of test_gpu_arf.py).
"""

import numpy as np
import pytest

from opengate_gb300 import workloads as W

from .test_gpu_arf import _model, random_params

pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.oracle")


def _setup(theta_max=12.0):
    scene, sp, _ = W.spect_phantom(shape=(40, 64, 64), spacing=4.8, n_runs=3)
    params = random_params(31, sp.n_windows + 1).astype(np.float32)
    model = _model(sp.n_windows + 1, rr=5.0)
    model.e_min, model.e_max, model.theta_max_deg, model.distance_to_crystal = 0.10, 0.16, theta_max, 39.8
    return scene, sp, model, params


def _run(scene, sp, model, params, n, seed):
    from opengate_gb300.engine import ArfNetwork, SpectEngine

    with SpectEngine(scene, sp) as eng:
        ArfNetwork(eng).set_model(model, params)
        eng.use_arf(True)
        eng.reset()
        eng.run(n, seed)
        return eng.projection(), *eng.arf_projection(squared=True), eng.counters()


def _compare(got, ref, nw):
    counts, w, w2, cnt = got
    rc, rw, rw2, rcnt = ref
    np.testing.assert_array_equal(counts, rc)
    assert cnt == rcnt, {k: (cnt[k], rcnt[k]) for k in cnt if cnt[k] != rcnt[k]}
    for a, b in ((w, rw), (w2, rw2)):
        close = np.isclose(a, b, rtol=4e-3, atol=2e-6 * max(b.max(), 1e-30))
        assert close.mean() > 0.999
        for k in range(nw):
            tot, rtot = a[:, k::nw].sum(), b[:, k::nw].sum()
            assert abs(tot - rtot) <= 2e-4 * rtot + 1e-6


@pytest.mark.parametrize("tol_deg", [10.0, 0.0])
def test_primary_free_flight_with_arf(tol_deg):
    scene, sp, model, params = _setup()
    sp.set_free_flight(angle_tolerance_max=np.radians(tol_deg))
    got = _run(scene, sp, model, params, 100_000, 17)
    ref = O.run_spect_arf_ff(scene, sp, 100_000, 17, model, params, threads=8)
    _compare(got, ref, sp.n_windows)
    cnt = got[3]
    assert cnt["arf_photons"] > 1000 and got[1].sum() > 0
    if tol_deg == 0.0:
        assert cnt["arf_fallback"] > 100  # outside the 12 degree domain: tracked with the weight


def test_scatter_splitting_with_arf():
    scene, sp, model, params = _setup(theta_max=30.0)
    sp.set_scatter_splitting(6, 2, max_compton_level=3, angle_tolerance_max=np.radians(25.0))
    got = _run(scene, sp, model, params, 30_000, 23)
    ref = O.run_spect_arf_ff(scene, sp, 30_000, 23, model, params, threads=8)
    _compare(got, ref, sp.n_windows)
    assert got[3]["arf_photons"] > 100


def test_forced_direction_with_arf():
    """ForceDirection + primary free flight + ARF detectors: each history's photon, aimed at
    its head within the cone, adds its cone weight x exp(-optical depth) x the window weights."""
    import math

    from opengate_gb300 import _capi as C

    scene, sp, model, params = _setup()
    sp.set_free_flight(angle_tolerance_max=math.radians(10.0))
    src = scene.source
    src.dir_type = C.GG_DIR_FORCED
    src.fd_angle_min, src.fd_angle_max = 0.0, math.radians(10.0)
    scene.set_source(src)
    got = _run(scene, sp, model, params, 40_000, 31)
    ref = O.run_spect_arf_ff(scene, sp, 40_000, 31, model, params, threads=8)
    _compare(got, ref, sp.n_windows)
    assert got[3]["arf_photons"] > 10_000
