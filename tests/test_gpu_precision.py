"""Error of the FP32 transport against the FP64 build of the same kernels on the
same random stream.

Sampling and tables run in FP32; the tallies are integer fixed point flushed
into FP64 images in both builds.  The FP32 images are held to the statistical
criterion used between independent runs (integral edep within 0.3 %, at least
99 % of the voxels above 10 % of the maximum within 2 combined standard
deviations), although most histories of the two builds are identical.
"""

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import workloads as W
from opengate_gb300.dose import precision_error

pytestmark = pytest.mark.gpu

INTEGRAL_TOL = 3e-3
WITHIN_2SIGMA = 0.99


def _run(scene, n, seed, precision):
    from opengate_gb300.engine import DoseEngine

    with DoseEngine(scene, precision=precision) as e:
        e.run(n, seed, 0)
        return e.edep(), e.edep_squared()


@pytest.mark.parametrize("case", ["water_pencil", "ct_phantom"])
def test_fp32_against_fp64_same_stream(case):
    if case == "water_pencil":
        scene = W.water_pencil()
        n = 1_000_000
    else:
        scene, _ = W.ct_phantom()
        n = 2_000_000
    a, qa = _run(scene, n, 12345, 32)
    b, qb = _run(scene, n, 12345, 64)
    err = precision_error(a, qa, b, qb, n)
    assert err["integral_rel"] < INTEGRAL_TOL, err
    assert err["within_2sigma"] >= WITHIN_2SIGMA, err
    # the same stream: most voxels agree far better than the statistics
    assert err["median_z"] < 0.5, err


def test_batched_fp32_against_fp64():
    from opengate_gb300.engine import BatchEngine

    _, sims = W.batched_phantoms(n_sims=4, sides=(16, 24, 32), primaries_range=(5e4, 2e5), seed=11)
    imgs = {}
    for prec in (32, 64):
        with BatchEngine(sims, precision=prec) as b:
            b.run()
            imgs[prec] = [(b.image(k, C.GG_IMG_EDEP), b.image(k, C.GG_IMG_EDEP_SQUARED)) for k in range(len(sims))]
    for k, (_, n, _) in enumerate(sims):
        (a, qa), (b, qb) = imgs[32][k], imgs[64][k]
        err = precision_error(a, qa, b, qb, n)
        assert err["integral_rel"] < INTEGRAL_TOL, (k, err)
        assert err["within_2sigma"] >= WITHIN_2SIGMA, (k, err)
