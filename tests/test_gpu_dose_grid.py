"""DoseActor dose grids other than the image grid, GPU against the oracle bit for bit.

The tally grid is placed like the reference's (GateDoseActor::
BeginOfRunActionMasterThread -> AttachImageToVolume, GateHelpersImage.txx:20-58)
and every deposit is scored in the grid voxel of its interaction point
(GateDoseActor::GetVoxelPosition / SteppingAction, GateDoseActor.cpp:144-243),
dose as the sum of edep / density of the material there.  Cases: a grid twice
as coarse as the image, a grid offset so that part of it lies outside the
image, the image grid itself given as a dose grid (equal to the standard
path), and a rotated, translated DoseActor through Simulation.run().
"""

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import workloads as W

pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.oracle")


def _grid(dims, spacing, corner, dose=True):
    g = C.DoseGridDesc()
    g.dims[:] = dims
    g.spacing[:] = spacing
    g.corner[:] = corner
    g.score_dose = 1 if dose else 0
    return g


def _gpu(scene, g, n, seed, precision=32, batch=0):
    from opengate_gb300.engine import DoseEngine

    with DoseEngine(scene, precision=precision, batch=batch) as e:
        e.set_dose_grid(list(g.dims), list(g.spacing), list(g.corner), score_dose=bool(g.score_dose))
        e.run(n, seed)
        out = (e.edep(), e.edep_squared())
        if g.score_dose:
            out += (e.dose_sum(), e.dose_sum_squared())
        return out + (e.counters(),)


def _same(g, o):
    *ga, gc = g
    *oa, oc = o
    assert gc == oc, {k: (gc[k], oc[k]) for k in gc if gc[k] != oc[k]}
    for a, b in zip(ga, oa):
        if b is not None:
            assert np.array_equal(a, b), f"differs in {int(np.sum(a != b))} voxels"


@pytest.fixture(scope="module")
def ct(built_lib):
    scene, _ = W.ct_phantom(shape=(40, 64, 64), spacing=4.8)
    return scene


@pytest.mark.parametrize("precision", [32, 64])
def test_coarse_grid_bit_exact(ct, precision):
    g = _grid((32, 32, 20), (9.6, 9.6, 9.6), ct.corner)
    n = 30000 if precision == 32 else 6000
    got = _gpu(ct, g, n, 321, precision, batch=12000)
    ref = O.run_dose_grid(ct, g, n, 321, threads=8, precision=precision, batch=12000)
    _same(got, ref)
    assert got[2].sum() > 0 and got[0].sum() > 0


def test_offset_grid_partly_outside_bit_exact(ct):
    # shifted by 37 mm in x and 11 mm in z, finer than the image: part of it is outside
    corner = [ct.corner[0] + 37.0, ct.corner[1], ct.corner[2] - 11.0]
    g = _grid((40, 30, 25), (3.0, 4.0, 5.0), corner)
    got = _gpu(ct, g, 30000, 99)
    ref = O.run_dose_grid(ct, g, 30000, 99, threads=8)
    _same(got, ref)
    full = O.run_dose(ct, 30000, 99, threads=8)[0]
    assert 0 < got[0].sum() < full.sum()  # deposits outside the grid are not scored


def test_image_grid_as_dose_grid_equals_standard_path(ct):
    from opengate_gb300.engine import DoseEngine

    g = _grid(ct.dims_xyz, ct.spacing, ct.corner, dose=True)
    got = _gpu(ct, g, 20000, 5)
    with DoseEngine(ct) as e:
        e.run(20000, 5)
        std = (e.edep(), e.edep_squared(), e.counters())
    assert np.array_equal(got[0], std[0]) and np.array_equal(got[1], std[1]) and got[4] == std[2]
    ref = std[0] / ct.voxel_density()
    m = ref > 0.01 * ref.max()
    np.testing.assert_allclose(got[2][m], ref[m], rtol=1e-6)  # dose tally: 2^-32 fixed point


def test_rotated_translated_dose_actor_through_the_api(tmp_path, built_lib):
    from scipy.spatial.transform import Rotation

    import opengate_gb300 as gate

    from .test_cpu_api import water_sim

    u = gate.g4_units
    sim = water_sim(tmp_path, n=50_000)
    d = sim.actors["dose"]
    d.size = [16, 16, 40]
    d.spacing = [5 * u.mm, 5 * u.mm, 3 * u.mm]
    d.translation = [2 * u.mm, -4 * u.mm, 10 * u.mm]
    rot = Rotation.from_euler("x", 20, degrees=True).as_matrix()
    d.rotation = rot
    d.edep_squared.active = True
    d.dose_squared.active = True
    sim.run()
    scene, vol, hu, *_ = sim.build_scene()
    dims, sp, corner = d.scoring_grid(vol)
    g = _grid(dims, sp, corner)
    e, e2, ds, ds2, cnt = O.run_dose_grid(scene, g, 50_000, sim.last_seed, threads=8)
    np.testing.assert_array_equal(d.edep.get_data().array, e)
    np.testing.assert_array_equal(d.edep_squared.get_data().array, e2)
    from opengate_gb300 import dose as D

    np.testing.assert_array_equal(d.dose.get_data().array, D.dose_sum_to_gy(ds, sp))
    back = gate.read_mhd(d.dose.get_output_path())
    np.testing.assert_allclose(back.direction, rot, atol=1e-12)
    assert back.array.shape == (40, 16, 16)
