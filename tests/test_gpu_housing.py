"""SPECT head housing on the GPU against the oracle, bit for bit.

The NM670 shielding box (contrib/spect/ge_discovery_nm670.py:215-262
add_spect_box) as slabs of the head stack: the aluminium entrance cover in
front of the crystal, the TiO2 reflector, the Pyrex back compartment, the
lead cover's and the steel shielding's backs behind it, and shielded side
faces.  Projections, weighted projections and every counter must equal the
oracle's for plain tracking, free flight and scatter splitting, in FP32 and
FP64; the housing must change the acquisition the way the physics says.
"""

import numpy as np
import pytest

from opengate_gb300 import spect as S
from opengate_gb300 import workloads as W

pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.oracle")

LU_WINDOWS = ((0.1872, 0.2288), (0.166, 0.187), (0.1017, 0.1243))


def _case(housing="nm670", n_runs=3):
    return W.spect_phantom(shape=(40, 64, 64), spacing=4.8, n_runs=n_runs, nuclide=W.LU177, collimator=S.MELP,
                           windows=LU_WINDOWS, housing=housing)


@pytest.mark.parametrize("precision", [32, 64])
def test_housing_projection_bit_exact(precision):
    from opengate_gb300.engine import SpectEngine

    scene, sp, _ = _case()
    assert sp.desc().n_back == 4 and sp.desc().n_cover == 1 and sp.desc().shielded_sides == 1
    n = 600_000
    with SpectEngine(scene, sp, precision=precision) as eng:
        eng.run(n, 13)
        proj, cnt = eng.projection(), eng.counters()
    ref, rcnt = O.run_spect(scene, sp, n, seed=13, threads=8, precision=precision)
    assert ref.sum() > 100
    np.testing.assert_array_equal(proj, ref)
    assert cnt == rcnt


def test_housing_free_flight_and_scatter_splitting_bit_exact():
    from opengate_gb300.engine import SpectEngine

    scene, sp, _ = _case()
    sp.set_free_flight(angle_tolerance_max=np.radians(40.0))
    with SpectEngine(scene, sp) as eng:
        eng.run(200_000, 17)
        w, w2 = eng.weighted_projection(squared=True)
        cnt = eng.counters()
    rw, rw2, rcnt = O.run_spect_ff(scene, sp, 200_000, seed=17, threads=8)
    np.testing.assert_array_equal(w, rw)
    np.testing.assert_array_equal(w2, rw2)
    assert cnt == rcnt and w.sum() > 0
    sp.set_scatter_splitting(6, 2, 3, angle_tolerance_max=np.radians(40.0))
    with SpectEngine(scene, sp) as eng:
        eng.run(40_000, 19)
        w, w2 = eng.weighted_projection(squared=True)
        cnt = eng.counters()
    rw, rw2, rcnt = O.run_spect_ff(scene, sp, 40_000, seed=19, threads=8)
    np.testing.assert_array_equal(w, rw)
    np.testing.assert_array_equal(w2, rw2)
    assert cnt == rcnt and w.sum() > 0


def test_housing_changes_the_acquisition_as_expected():
    """Shielded sides remove the photons that reached the crystal through a side face; the
    1.3 mm aluminium cover attenuates the 113 keV photopeak (mu/rho ~0.17 cm2/g: ~6 %)
    more than the 208 keV one (~3 %)."""
    from opengate_gb300.engine import SpectEngine

    n = 200_000_000
    tot = {}
    for kind in ("none", "sides", "nm670"):
        scene, sp, _ = _case("nm670" if kind == "nm670" else "none", n_runs=2)
        if kind == "sides":
            sp.set_housing(None, (), shielded_sides=True)
        with SpectEngine(scene, sp) as eng:
            eng.run(n, 23)
            p = eng.projection()
        tot[kind] = np.array([p[:, w::3].sum() for w in range(3)])
    assert np.all(tot["sides"] <= tot["none"])
    assert tot["sides"][2] < tot["none"][2] - 3 * np.sqrt(tot["none"][2] - tot["sides"][2] + 1)
    r113 = tot["nm670"][2] / tot["sides"][2]
    r208 = tot["nm670"][0] / tot["sides"][0]
    assert r113 < 0.97 and r208 < 1.01 and r113 < r208


def test_housing_and_dose_grid_arguments_are_checked():
    """gg_spect_setup refuses housing layers it cannot build (five back layers, a zero
    thickness, a material outside the table) and the context stays usable."""
    from opengate_gb300 import _capi as C
    from opengate_gb300.engine import SpectEngine

    scene, sp, _ = _case(n_runs=1)
    with SpectEngine(scene, sp) as eng:
        good = sp.desc()
        for mutate in (lambda d: setattr(d, "n_back", 5), lambda d: d.back_thickness.__setitem__(1, 0.0),
                       lambda d: d.back_material.__setitem__(0, 999), lambda d: setattr(d, "n_cover", 2)):
            d = sp.desc()
            mutate(d)
            with pytest.raises(C.GGError) as e:
                eng._call("gg_spect_setup", C.ctypes.byref(d))
            assert e.value.status == C.GG_ERR_ARG
        eng._call("gg_spect_setup", C.ctypes.byref(good))
        eng.run(1000, 3)
        assert eng.counters()["histories"] == 1000


@pytest.mark.parametrize("precision", [32, 64])
def test_forced_direction_free_flight_bit_exact(precision):
    """ForceDirection toward the heads (GateForcedDirectionManager.cpp) with primary free flight:
    history h aims at head h mod 2 within a 10 degree cone, weight (1 - cos 10 deg) / 2.
    Weighted projections, squares and counters equal the oracle's."""
    import math

    from opengate_gb300 import _capi as C
    from opengate_gb300.engine import SpectEngine

    scene, sp, _ = _case()
    sp.set_free_flight(angle_tolerance_max=math.radians(10.0))
    src = scene.source
    src.dir_type = C.GG_DIR_FORCED
    src.fd_angle_min, src.fd_angle_max = 0.0, math.radians(10.0)
    scene.set_source(src)
    n = 100_000
    with SpectEngine(scene, sp, precision=precision) as eng:
        eng.run(n, 29)
        w, w2 = eng.weighted_projection(squared=True)
        cnt = eng.counters()
    rw, rw2, rcnt = O.run_spect_ff(scene, sp, n, seed=29, threads=8, precision=precision)
    np.testing.assert_array_equal(w, rw)
    np.testing.assert_array_equal(w2, rw2)
    assert cnt == rcnt and w.sum() > 0


def test_forced_direction_needs_primary_free_flight():
    import math

    from opengate_gb300 import _capi as C
    from opengate_gb300.engine import SpectEngine

    scene, sp, _ = _case(n_runs=1)
    src = scene.source
    src.dir_type = C.GG_DIR_FORCED
    src.fd_angle_min, src.fd_angle_max = 0.0, math.radians(10.0)
    scene.set_source(src)
    with SpectEngine(scene, sp) as eng:
        with pytest.raises(C.GGError) as e:
            eng.run(1000, 3)
        assert e.value.status == C.GG_ERR_STATE
