"""GPU transport vs the CPU oracle on the same seeded inputs (bit-exact).

The kernels and the oracle execute the same floating-point operation
sequence per history on the same Philox stream and tally in 64-bit fixed
point, so edep, edep-squared and every counter must be identical - not just
statistically compatible.
"""

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import workloads as W
from opengate_gb300.scene import Scene, SourceSpec

pytestmark = pytest.mark.gpu


def _gpu(scene, n, seed, precision=32, first=0, **opts):
    from opengate_gb300.engine import DoseEngine

    with DoseEngine(scene, precision=precision, **opts) as eng:
        eng.run(n, seed, first)
        return eng.edep(), eng.edep_squared(), eng.counters()


def _oracle(scene, n, seed, precision=32, first=0, batch=0):
    from oracle import oracle as O

    return O.run_dose(scene, n, seed, first=first, batch=batch, threads=4, precision=precision)


def _assert_same(a, b):
    ea, e2a, ca = a
    eb, e2b, cb = b
    assert ca == cb, {k: (ca[k], cb[k]) for k in ca if ca[k] != cb[k]}
    assert np.array_equal(ea, eb), f"edep differs in {int(np.sum(ea != eb))} voxels"
    assert np.array_equal(e2a, e2b), f"edep^2 differs in {int(np.sum(e2a != e2b))} voxels"


@pytest.fixture(scope="module")
def lib(built_lib):
    return C.load()


def small_ct():
    scene, _ = W.ct_phantom(shape=(40, 64, 64), spacing=4.8)
    return scene


@pytest.mark.parametrize("precision", [32, 64])
def test_water_pencil_bit_exact(lib, precision):
    sc = W.water_pencil()
    n = 20000 if precision == 32 else 5000
    g = _gpu(sc, n, 12345, precision=precision, batch=1 << 20)
    o = _oracle(sc, n, 12345, precision=precision, batch=1 << 20)
    _assert_same(g, o)
    assert g[2]["histories"] == n
    assert g[0].sum() > 0


@pytest.mark.parametrize("precision", [32, 64])
def test_ct_phantom_spectrum_bit_exact(lib, precision):
    sc = small_ct()
    n = 20000 if precision == 32 else 4000
    g = _gpu(sc, n, 777, precision=precision, first=1000, batch=7000)
    o = _oracle(sc, n, 777, precision=precision, first=1000, batch=7000)
    _assert_same(g, o)
    assert g[2]["skipped"] > 0  # the field acceptance rejected directions


def test_launch_shape_independence(lib):
    sc = small_ct()
    ref = _gpu(sc, 30000, 99, batch=10000)
    for opts in (dict(block_size=64, chunk=32), dict(block_size=128, blocks_per_sm=1, chunk=1024)):
        _assert_same(ref, _gpu(sc, 30000, 99, batch=10000, **opts))


@pytest.mark.parametrize("pos_type", [C.GG_POS_BOX, C.GG_POS_SPHERE, C.GG_POS_DISC, C.GG_POS_POINT])
def test_internal_sources_bit_exact(lib, pos_type):
    base = small_ct()
    src = SourceSpec()
    src.pos_type = pos_type
    src.translation = [10.0, -20.0, 5.0]
    src.half_size = [30.0, 20.0, 10.0]
    src.radius = 25.0
    th = np.deg2rad(30.0)
    src.rotation = np.array([[1, 0, 0], [0, np.cos(th), -np.sin(th)], [0, np.sin(th), np.cos(th)]])
    src.dir_type = C.GG_DIR_ISO
    src.ene_type = C.GG_ENE_LINES
    src.spec_e = np.array([0.1405, 0.3645, 2.5])
    src.spec_cdf = np.array([0.6, 0.9, 1.0])
    sc = Scene(base.pt, base.labels, base.spacing, base.corner, base.world_half, base.world_material, src)
    g = _gpu(sc, 10000, 4242, batch=1 << 20)
    o = _oracle(sc, 10000, 4242, batch=1 << 20)
    _assert_same(g, o)
    assert g[2]["secondaries"] > 0  # 2.5 MeV line converts sometimes


def test_focused_range_source_bit_exact(lib):
    base = small_ct()
    src = SourceSpec()
    src.pos_type = C.GG_POS_BOX
    src.translation = [0.0, 0.0, -400.0]
    src.half_size = [20.0, 20.0, 1.0]
    src.dir_type = C.GG_DIR_FOCUSED
    src.focus = [0.0, 10.0, 0.0]
    src.ene_type = C.GG_ENE_RANGE
    src.e_lo, src.e_hi = 0.05, 3.0
    sc = Scene(base.pt, base.labels, base.spacing, base.corner, base.world_half, base.world_material, src)
    _assert_same(_gpu(sc, 10000, 5, batch=1 << 20), _oracle(sc, 10000, 5, batch=1 << 20))


def test_reproducible_for_fixed_seed(lib):
    sc = small_ct()
    a = _gpu(sc, 20000, 31337, batch=1 << 20)
    b = _gpu(sc, 20000, 31337, batch=1 << 20)
    _assert_same(a, b)
    c = _gpu(sc, 20000, 31338, batch=1 << 20)
    assert not np.array_equal(a[0], c[0])


@pytest.mark.parametrize("precision", [32, 64])
def test_narrow_acceptance_bit_exact(lib, precision):
    """A field a tenth as wide: ~1 % of the directions are accepted, so the
    warp-cooperative acceptance loop deals many lanes to few histories per round; doses,
    rejection counts and everything else equal the oracle's sequential loop."""
    sc = small_ct()
    (lo, hi), = sc.source.accept_boxes
    c = [(a + b) / 2 for a, b in zip(lo, hi)]
    hx, hz = (hi[0] - lo[0]) / 20, (hi[2] - lo[2]) / 20  # a tenth of the field's half-width
    sc.source.accept_boxes = [((c[0] - hx, lo[1], c[2] - hz), (c[0] + hx, hi[1], c[2] + hz))]
    sc.set_source(sc.source)
    n = 6000 if precision == 32 else 2000
    g = _gpu(sc, n, 4242, precision=precision, batch=4096)
    o = _oracle(sc, n, 4242, precision=precision, batch=4096)
    _assert_same(g, o)
    assert g[2]["skipped"] > 20 * n


def test_acceptance_exhausted_fails_like_the_oracle(lib):
    """max_rejection = 2 with a ~1 % acceptance: both the GPU and the oracle stop with the
    domain error (GateSingleParticleSource gives up after max_rejection rejections)."""
    sc = small_ct()
    (lo, hi), = sc.source.accept_boxes
    c = [(a + b) / 2 for a, b in zip(lo, hi)]
    hx, hz = (hi[0] - lo[0]) / 20, (hi[2] - lo[2]) / 20  # a tenth of the field's half-width
    sc.source.accept_boxes = [((c[0] - hx, lo[1], c[2] - hz), (c[0] + hx, hi[1], c[2] + hz))]
    sc.set_source(sc.source)
    sc.source.max_rejection = 2
    sc.set_source(sc.source)
    with pytest.raises(Exception):
        _gpu(sc, 2000, 5, batch=4096)
    with pytest.raises(Exception):
        _oracle(sc, 2000, 5, batch=4096)


def test_images_into_pinned_buffers(lib):
    """edep / edep_squared into page-locked buffers (gg_host_alloc) equal the plain ones."""
    from opengate_gb300.engine import DoseEngine

    sc = W.water_pencil()
    with DoseEngine(sc, batch=1 << 20) as eng:
        eng.run(5000, 3)
        a, b = eng.edep(), eng.edep_squared()
        pa = eng.pinned_empty(sc.labels.shape)
        pb = eng.pinned_empty(sc.labels.shape)
        np.testing.assert_array_equal(eng.edep(pa), a)
        np.testing.assert_array_equal(eng.edep_squared(pb), b)
        assert pa.ctypes.data != a.ctypes.data


@pytest.mark.parametrize("precision", [32, 64])
def test_wavefront_and_phase_kernels_agree(lib, precision):
    """The block-phase kernel (default) and the compacted wavefront kernel run the same
    histories to the same edep, edep^2 and counters, on the CT phantom with its field
    source (acceptance loop, air gaps, pair production above 1.022 MeV)."""
    from opengate_gb300.engine import DoseEngine

    sc = small_ct()
    n = 40000 if precision == 32 else 8000
    out = []
    for kernel in (C.GG_KERNEL_PHASED, C.GG_KERNEL_WAVEFRONT):
        with DoseEngine(sc, precision=precision, batch=15000) as eng:
            eng.set_transport_kernel(kernel)
            eng.run(n, 2468, 17)
            out.append((eng.edep(), eng.edep_squared(), eng.counters()))
    _assert_same(out[0], out[1])
    assert out[0][2]["secondaries"] > 0 and out[0][2]["real_interactions"] > n


def test_wavefront_matches_oracle_and_launch_shapes(lib):
    """The wavefront kernel against the oracle directly, with small and large claim chunks."""
    from opengate_gb300.engine import DoseEngine

    sc = small_ct()
    ref = _oracle(sc, 30000, 99, batch=10000)
    for chunk in (32, 0):
        with DoseEngine(sc, precision=32, batch=10000, chunk=chunk) as eng:
            eng.set_transport_kernel(C.GG_KERNEL_WAVEFRONT)
            eng.run(30000, 99)
            _assert_same((eng.edep(), eng.edep_squared(), eng.counters()), ref)
