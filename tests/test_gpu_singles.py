"""Singles list on the GPU (gg_spect_record_singles / gg_spect_get_singles) against the
oracle's, record for record, and the digitizer's ROOT output through the API.

The list is filled in completion order, so both sides are sorted before the
comparison; every field (history id, head, gantry position, blurred energy,
blurred crystal position, free-flight weight) must agree exactly.
"""

import numpy as np
import pytest

from opengate_gb300 import root_io
from opengate_gb300 import spect as S

from .test_cpu_singles import projection_of, small_case, sort_singles

pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.oracle")


def _gpu_singles(scene, sp, n, seed, precision, capacity=1 << 20):
    from opengate_gb300.engine import SpectEngine

    with SpectEngine(scene, sp, precision=precision) as eng:
        eng.record_singles(capacity)
        eng.run(n, seed)
        rec = eng.singles()
        again = eng.singles()  # read empties the list
        w = eng.weighted_projection() if sp.free_flight.enabled else None
        return rec, again, eng.projection(), w, eng.counters()


@pytest.mark.parametrize("precision", [32, 64])
def test_singles_list_bit_exact(precision):
    scene, sp, _ = small_case(n_runs=3)
    sp.set_energy_blur("InverseSquare", resolution=0.063, reference=0.14057)
    sp.set_spatial_blur(3.0 * 0.42466090014400953, keep_in_solid_limits=True, truncated=True)
    n = 1_000_000
    rec, again, proj, _, cnt = _gpu_singles(scene, sp, n, 17, precision)
    (rproj, rcnt), ref = O.with_singles(precision, 1 << 20,
                                        lambda: O.run_spect(scene, sp, n, 17, threads=8, precision=precision))
    assert len(again) == 0
    assert len(rec) == cnt["singles"] == len(ref) > 500
    np.testing.assert_array_equal(sort_singles(rec), sort_singles(ref))
    np.testing.assert_array_equal(proj, rproj)
    np.testing.assert_array_equal(projection_of(rec, sp, precision), proj)


def test_singles_list_with_scatter_splitting():
    """Weighted singles of the split copies keep their history's id."""
    scene, sp, _ = small_case(n_runs=2)
    sp.set_scatter_splitting(8, 4, 3, weight_cutoff=1e-7, energy_cutoff=0.01, angle_tolerance_max=0.6)
    n = 100_000
    rec, _, _, w, _ = _gpu_singles(scene, sp, n, 71, 32)
    (rw, _, _), ref = O.with_singles(32, 1 << 20, lambda: O.run_spect_ff(scene, sp, n, 71, threads=8))
    assert len(rec) == len(ref) > 50 and np.any(rec["weight"] != 1.0)
    np.testing.assert_array_equal(sort_singles(rec), sort_singles(ref))
    np.testing.assert_array_equal(w, rw)


def test_singles_list_overflow_and_no_effect_on_the_run():
    from opengate_gb300.engine import SpectEngine

    scene, sp, _ = small_case(n_runs=2)
    n = 300_000
    with SpectEngine(scene, sp) as eng:
        eng.run(n, 5)
        plain = eng.projection()
    with SpectEngine(scene, sp) as eng:
        eng.record_singles(8)
        eng.run(n, 5)
        with pytest.raises(RuntimeError, match="overflow"):
            eng.singles()
        np.testing.assert_array_equal(eng.projection(), plain)
        eng.record_singles(0)
        with pytest.raises(Exception):
            eng.singles()


def test_digitizer_writes_singles_root(tmp_path):
    """Simulation.run() with the NM670 digitizer chain writes each head's blurred singles as a
    ROOT tree named after the chain's last module, equal to the oracle's singles."""
    from .test_cpu_api_spect import spect_sim

    sim, heads = spect_sim(tmp_path, n_per_run=200_000, angles=2)
    sim.random_seed = 77
    sim.run()
    scene, sp, _, _, head_of = sim.build_spect()
    _, ref = O.with_singles(32, 1 << 20, lambda: O.run_spect(scene, sp, 200_000, 77, threads=8))
    ref = sort_singles(ref)
    total = 0
    for head, digi in heads:
        sb = [m for m in digi.modules if m.type_name == "DigitizerSpatialBlurringActor"][0]
        h = head_of[sb.attached_to]
        cols = root_io.read_tree(tmp_path / f"{sb.name}.root", sb.name)
        want = sp.singles_columns(ref[ref["head"] == h])
        assert list(cols) == list(want)
        for k in want:
            np.testing.assert_array_equal(cols[k], want[k])
        total += len(cols["EventID"])
    assert total == len(ref) > 50
