"""SPECT projections on the GPU against the oracle, bit for bit.

Workload: a reduced CT phantom (40 x 64 x 64 voxels of 4.8 mm) with a body +
sphere activity image as voxel source, two heads, four gantry positions; the
full-size case is 160 x 256 x 256 voxels and 60 positions
(contrib/spect/ge_discovery_nm670.py geometry, Tc-99m/LEHR and Lu-177/MELP).
Counts are integers, so GPU and oracle must agree exactly for every pixel of
every head, run and energy window, and on every transport counter.
"""

import numpy as np
import pytest

from opengate_gb300 import spect as S
from opengate_gb300 import workloads as W

pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.oracle")

CASES = {
    "tc99m_lehr": (W.TC99M, S.LEHR, ((0.126, 0.154), (0.108, 0.126))),
    "lu177_melp": (W.LU177, S.MELP, ((0.1017, 0.1243), (0.1872, 0.2288), (0.166, 0.187))),
}


def _case(name, n_runs=4):
    nuc, coll, win = CASES[name]
    return W.spect_phantom(shape=(40, 64, 64), spacing=4.8, n_runs=n_runs, nuclide=nuc, collimator=coll,
                           windows=win)


def _gpu(scene, sp, n, seed, precision=32, **kw):
    from opengate_gb300.engine import SpectEngine

    with SpectEngine(scene, sp, precision=precision, **kw) as eng:
        eng.run(n, seed)
        return eng.projection(), eng.counters()


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("name", list(CASES))
def test_spect_projection_bit_exact(name, precision):
    scene, sp, _ = _case(name)
    n = 400_000
    proj, cnt = _gpu(scene, sp, n, seed=11, precision=precision)
    ref, rcnt = O.run_spect(scene, sp, n, seed=11, threads=8, precision=precision)
    assert proj.shape == ref.shape == sp.projection_shape()
    assert ref.sum() > 100
    np.testing.assert_array_equal(proj, ref)
    assert cnt == rcnt


def test_spect_independent_of_batching_and_launch_shape():
    scene, sp, _ = _case("tc99m_lehr", n_runs=2)
    a, ca = _gpu(scene, sp, 300_000, seed=3)
    b, cb = _gpu(scene, sp, 300_000, seed=3, batch=70_001, block_size=128, chunk=64)
    np.testing.assert_array_equal(a, b)
    assert ca == cb


def test_spect_reset_and_history_offset():
    """reset() clears the projection; `first` continues the history ids."""
    from opengate_gb300.engine import SpectEngine

    scene, sp, _ = _case("tc99m_lehr", n_runs=1)
    with SpectEngine(scene, sp) as eng:
        eng.run(200_000, 7)
        first = eng.projection()
        eng.reset()
        eng.run(200_000, 7)
        np.testing.assert_array_equal(eng.projection(), first)
        eng.reset()
        eng.run(100_000, 7, first=200_000)
        later = eng.projection()
    ref, _ = O.run_spect(scene, sp, 100_000, seed=7, first=200_000, threads=8)
    np.testing.assert_array_equal(later, ref)


def test_all_angles_in_one_call_equal_per_angle_calls():
    """gg_spect_run (one set of launches for every gantry position) == gg_spect_set_heads + gg_run per position."""
    from opengate_gb300.engine import SpectEngine

    scene, sp, _ = _case("tc99m_lehr", n_runs=3)
    with SpectEngine(scene, sp) as eng:
        eng.run(150_000, 13, first=1000)
        one = eng.projection()
        c_one = eng.counters()
        n_launch = eng.last_kernel_ms()[3]
        # one batch: the source stage, then phantom + head stage passes
        assert n_launch >= 3 and (n_launch - 1) % 2 == 0
    with SpectEngine(scene, sp) as eng:
        eng.run_per_angle(150_000, 13, first=1000)
        per = eng.projection()
        c_per = eng.counters()
    np.testing.assert_array_equal(one, per)
    assert c_one == c_per


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("truncated", [False, True])
def test_blurred_singles_bit_exact(precision, truncated):
    """Energy (inverse-square law, 6.3 % FWHM at 140.57 keV) and spatial (3 mm FWHM)
    blurring of the NM670 digitizer chain: the draws come from each history's own
    stream, so GPU and oracle still agree count for count."""
    scene, sp, _ = _case("tc99m_lehr")
    sp.set_energy_blur("InverseSquare", resolution=0.063, reference=0.14057)
    sp.set_spatial_blur(3.0 * 0.42466090014400953, keep_in_solid_limits=True, truncated=truncated)
    n = 400_000
    proj, cnt = _gpu(scene, sp, n, seed=21, precision=precision)
    ref, rcnt = O.run_spect(scene, sp, n, seed=21, threads=8, precision=precision)
    np.testing.assert_array_equal(proj, ref)
    assert cnt == rcnt
    # the blur moves counts: the unblurred acquisition of the same histories differs
    scene0, sp0, _ = _case("tc99m_lehr")
    plain, _ = _gpu(scene0, sp0, n, seed=21, precision=precision)
    assert not np.array_equal(plain, proj)
    assert abs(plain.sum() - proj.sum()) < 0.05 * plain.sum()


@pytest.mark.parametrize("precision", [32, 64])
def test_centroid_adder_bit_exact(precision):
    """EnergyWeightedCentroidPosition singles (the Intevo digitizer's adder)."""
    scene, sp, _ = _case("lu177_melp")
    sp.adder_policy = "EnergyWeightedCentroidPosition"
    n = 300_000
    proj, cnt = _gpu(scene, sp, n, seed=31, precision=precision)
    ref, rcnt = O.run_spect(scene, sp, n, seed=31, threads=8, precision=precision)
    np.testing.assert_array_equal(proj, ref)
    assert cnt == rcnt


@pytest.mark.parametrize("precision", [32, 64])
def test_free_flight_bit_exact(precision):
    """Free flight outside the heads: weighted projections (2^-32 fixed point) and
    their history-by-history squares identical to the oracle's."""
    scene, sp, _ = _case("tc99m_lehr")
    sp.set_free_flight(weight_cutoff=1e-4, energy_cutoff=0.01)
    n = 400_000
    from opengate_gb300.engine import SpectEngine

    with SpectEngine(scene, sp, precision=precision) as eng:
        eng.run(n, 41)
        w, w2 = eng.weighted_projection(squared=True)
        cnt = eng.counters()
        assert eng.projection().sum() == 0  # counts are not scored in free flight
    rw, rw2, rcnt = O.run_spect_ff(scene, sp, n, seed=41, threads=8, precision=precision)
    np.testing.assert_array_equal(w, rw)
    np.testing.assert_array_equal(w2, rw2)
    assert cnt == rcnt
    assert w.sum() > 0 and np.all(w2 <= w + 1e-12)  # weights <= 1


def test_free_flight_equals_analog_without_attenuation():
    """In vacuum nothing scatters outside the heads: the weighted free-flight projection
    and the analog counts estimate the same image in every window (free flight leaves
    out only what scatters outside the heads, which the reference simulates separately)."""
    from opengate_gb300 import materials as M
    from opengate_gb300 import tables as T
    from opengate_gb300.engine import SpectEngine
    from opengate_gb300.scene import Scene

    scene, sp, _ = _case("tc99m_lehr", n_runs=1)
    mats = list(scene.pt.materials)
    mats[0] = M.MaterialDatabase().get("G4_Galactic")  # label 0 and the world: vacuum
    vac = np.zeros_like(scene.labels)
    scene_air = Scene(T.PhysicsTables(mats), vac, scene.spacing, scene.corner, scene.world_half, 0,
                      scene.source)
    n = 60_000_000
    with SpectEngine(scene_air, sp) as eng:
        eng.run(n, 51)
        analog = eng.projection()
    sp.set_free_flight()
    with SpectEngine(scene_air, sp) as eng:
        eng.run(n, 52)
        ff, ff2 = eng.weighted_projection(squared=True)
    for k in range(sp.n_windows):
        a, f = analog[:, k].sum(), ff[:, k].sum()
        sigma = np.sqrt(a + ff2[:, k].sum())
        assert abs(a - f) < 4 * sigma + 1e-9, (k, a, f, sigma)
    assert analog[:, 0].sum() > 2000


@pytest.mark.parametrize("precision", [32, 64])
def test_scatter_splitting_bit_exact(precision):
    """Scatter splitting: analog photons outside the heads, each Compton / Rayleigh
    re-sampled into weighted copies on their own random streams, copies in free flight
    to the heads (angle check on).  Weighted projections, squares and counters identical
    to the oracle's."""
    scene, sp, _ = _case("tc99m_lehr")
    sp.set_scatter_splitting(8, 4, 3, weight_cutoff=1e-7, energy_cutoff=0.01, angle_tolerance_max=0.6)
    n = 60_000
    from opengate_gb300.engine import SpectEngine

    with SpectEngine(scene, sp, precision=precision) as eng:
        eng.run(n, 71)
        w, w2 = eng.weighted_projection(squared=True)
        cnt = eng.counters()
        assert eng.projection().sum() == 0
    rw, rw2, rcnt = O.run_spect_ff(scene, sp, n, seed=71, threads=8, precision=precision)
    np.testing.assert_array_equal(w, rw)
    np.testing.assert_array_equal(w2, rw2)
    assert cnt == rcnt
    assert w.sum() > 0 and w.max() < 1.0


@pytest.mark.parametrize("angle", [0.35, 0.0])
def test_scatter_splitting_one_head_bit_exact(angle):
    """One head, more Compton copies per request than a warp has lanes: the copies'
    scattering-angle test and head checks run over a single head axis, and the copies that
    can still reach it wait and are finished on full warps; with the angle check (0.35 rad)
    and without it (every live copy goes through the full check), weighted projections,
    squares and counters equal the oracle's."""
    scene, sp, _ = _case("tc99m_lehr", n_runs=2)
    sp.n_heads = 1
    sp.set_scatter_splitting(40, 6, 3, angle_tolerance_max=angle)
    n = 40_000
    from opengate_gb300.engine import SpectEngine

    with SpectEngine(scene, sp, precision=32) as eng:
        eng.run(n, 29)
        w, w2 = eng.weighted_projection(squared=True)
        cnt = eng.counters()
    assert w.shape[0] == 1
    rw, rw2, rcnt = O.run_spect_ff(scene, sp, n, seed=29, threads=8, precision=32)
    np.testing.assert_array_equal(w, rw)
    np.testing.assert_array_equal(w2, rw2)
    assert cnt == rcnt
    assert w.sum() > 0


def test_scatter_splitting_queue_overflow_repeats_the_pass():
    """Many copies per history and short batches: the head queue overflows, the phantom
    pass is repeated on fewer histories, and the result stays the oracle's, bit for bit
    (counters included: the overflowed pass leaves none behind)."""
    scene, sp, _ = _case("tc99m_lehr", n_runs=1)
    sp.set_scatter_splitting(64, 16, 5)
    n, batch = 24_000, 1024
    from opengate_gb300.engine import SpectEngine

    with SpectEngine(scene, sp, batch=batch) as eng:
        eng.run(n, 73)
        w, w2 = eng.weighted_projection(squared=True)
        cnt = eng.counters()
        launches = eng.last_kernel_ms()[3]
    nb = (n + batch - 1) // batch
    assert launches > 3 * nb  # generate + phantom + head per batch, plus the repeated / split passes
    rw, rw2, rcnt = O.run_spect_ff(scene, sp, n, seed=73, threads=8)
    np.testing.assert_array_equal(w, rw)
    np.testing.assert_array_equal(w2, rw2)
    assert cnt == rcnt


def test_free_flight_plus_scatter_splitting_equal_analog():
    """The reference's free-flight SPECT recipe: the primary (GammaFreeFlightActor) and
    the scattered (ScatterSplittingFreeFlightActor) weighted projections add up to the
    analog acquisition, window by window and head by head, within the statistics."""
    scene, sp, _ = _case("tc99m_lehr", n_runs=1)
    from opengate_gb300.engine import SpectEngine

    n_a, n_f, n_s = 400_000_000, 60_000_000, 12_000_000
    with SpectEngine(scene, sp) as eng:
        eng.run(n_a, 81)
        analog = eng.projection()
    sp.set_free_flight()
    with SpectEngine(scene, sp) as eng:
        eng.run(n_f, 82)
        ff, ff2 = eng.weighted_projection(squared=True)
    # the copies of one history are correlated: the scattered part's variance comes
    # from independent chunks of histories
    sp.set_scatter_splitting(20, 5, 1000)
    n_chunks = 12
    m = n_s // n_chunks
    shape = sp.projection_shape()
    axes = tuple(range(2, len(shape)))
    chunks = []
    with SpectEngine(scene, sp) as eng:
        prev = 0.0
        for k in range(n_chunks):
            eng.run(m, 83, first=k * m)
            cur, _ = eng.weighted_projection(squared=True)
            chunks.append((cur - prev).reshape(shape).sum(axis=axes))
            prev = cur
        ss = prev
    chunks = np.array(chunks)
    kf, ks = n_a / n_f, n_a / (m * n_chunks)
    a_t = analog.reshape(shape).sum(axis=axes)
    ss_t = ss.reshape(shape).sum(axis=axes) * ks
    e_t = ff.reshape(shape).sum(axis=axes) * kf + ss_t
    var_ss = ks * ks * n_chunks * chunks.var(axis=0, ddof=1)
    v_t = a_t + (ff2.reshape(shape).sum(axis=axes) * kf * kf) + var_ss
    z = (a_t - e_t) / np.sqrt(v_t)
    print("analog", a_t.tolist(), "primary + scatter", e_t.tolist(), "z", z.tolist())
    assert np.all(np.abs(z) < 4.5), (a_t, e_t, z)
    assert a_t.min() > 3000
    assert (ss * ks).reshape(shape).sum(axis=axes)[..., 1].min() > 0.3 * e_t[..., 1].min()
