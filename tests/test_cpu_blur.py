"""Digitizer blurring (DigitizerBlurringActor / DigitizerSpatialBlurringActor) in the
oracle: the blurred singles follow the reference's laws (mean, standard deviation),
points outside the crystal are clamped or redrawn, and the erf of the truncated
redraw is within the published bound of its approximation."""

import math

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import spect as S

O = pytest.importorskip("oracle.oracle")
FWHM = 1.0 / (2.0 * math.sqrt(2.0 * math.log(2.0)))


def _blur(**kw):
    b = C.BlurDesc()
    for k, v in kw.items():
        if k == "spatial_sigma":
            b.spatial_sigma[0], b.spatial_sigma[1] = v
        else:
            setattr(b, k, v)
    return b


@pytest.mark.parametrize("precision", [32, 64])
def test_erf_approximation(precision):
    for x in np.linspace(-4, 4, 81):
        assert abs(O.erf(x, precision) - math.erf(x)) < (2e-7 if precision == 64 else 5e-7)


@pytest.mark.parametrize("e", [0.14057, 0.208, 0.113])
def test_inverse_square_energy_blur(e):
    # NM670 digitizer: FWHM/E = 6.3 % at 140.57 keV, scaling as 1/sqrt(E)
    b = _blur(energy_method=C.GG_BLUR_INVERSE_SQUARE, energy_resolution=0.063, energy_reference=0.14057)
    n = 200_000
    ee, _, _ = O.sample_blur(b, 100.0, e, 0.0, 0.0, n, seed=11)
    sigma = 0.063 * math.sqrt(0.14057 / e) * e * FWHM
    assert abs(ee.mean() - e) < 5 * sigma / math.sqrt(n)
    assert ee.std() == pytest.approx(sigma, rel=0.01)


def test_linear_and_gaussian_energy_blur():
    n = 200_000
    b = _blur(energy_method=C.GG_BLUR_LINEAR, energy_resolution=0.08, energy_reference=0.14, energy_slope=-0.2)
    ee, _, _ = O.sample_blur(b, 100.0, 0.2, 0.0, 0.0, n, seed=2)
    sigma = (-0.2 * (0.2 - 0.14) + 0.08) * 0.2 * FWHM
    assert ee.std() == pytest.approx(sigma, rel=0.01)
    b = _blur(energy_method=C.GG_BLUR_GAUSSIAN, energy_sigma=0.005)
    ee, _, _ = O.sample_blur(b, 100.0, 0.2, 0.0, 0.0, n, seed=3)
    assert ee.std() == pytest.approx(0.005, rel=0.01) and abs(ee.mean() - 0.2) < 1e-4


def test_spatial_blur_clamps_into_the_crystal():
    sg = 3.0 * FWHM  # NM670 digitizer: 3 mm FWHM
    b = _blur(spatial=1, spatial_sigma=(sg, sg), keep_in_solid_limits=1)
    n = 200_000
    _, x, y = O.sample_blur(b, 100.0, 0.14, 10.0, 99.0, n, seed=4)
    assert x.std() == pytest.approx(sg, rel=0.01) and abs(x.mean() - 10.0) < 0.02
    assert y.max() < 100.0 and y.min() > -100.0
    clamped = np.mean(y >= 100.0 - 1e-3)
    assert clamped == pytest.approx(0.5 * math.erfc(1.0 / (sg * math.sqrt(2.0))), abs=0.005)
    b.keep_in_solid_limits = 0
    _, _, y2 = O.sample_blur(b, 100.0, 0.14, 10.0, 99.0, n, seed=4)
    assert y2.max() > 100.0


def test_truncated_spatial_blur_redraws_inside():
    sg = 3.0 * FWHM
    b = _blur(spatial=1, spatial_sigma=(sg, sg), truncated=1)
    n = 100_000
    _, x, y = O.sample_blur(b, 100.0, 0.14, 0.0, 99.5, n, seed=5)
    assert y.max() <= 100.0 and y.min() >= -100.0
    assert x.std() == pytest.approx(sg, rel=0.02)  # far from the edges: plain Gaussian
    assert np.mean(y >= 100.0 - 1e-3) < 1e-3  # no pile-up at the edge


def test_spect_spec_blur_settings():
    sp = S.SpectSpec(n_runs=1)
    assert sp.blur.energy_method == C.GG_BLUR_NONE and sp.blur.spatial == 0
    sp.set_energy_blur("InverseSquare", resolution=0.063, reference=0.14057)
    sp.set_spatial_blur(3.0 * FWHM)
    assert sp.blur.energy_method == C.GG_BLUR_INVERSE_SQUARE and sp.blur.spatial == 1
    assert sp.blur.keep_in_solid_limits == 1 and sp.blur.truncated == 0
    with pytest.raises(ValueError):
        sp.set_energy_blur("Poisson")
