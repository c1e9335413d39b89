"""SPECT head model, digitizer and voxel source: oracle and host logic on the CPU.

The reference describes the collimator as hexagonal G4Polyhedra holes on two
offset rectangular lattices (contrib/spect/ge_discovery_nm670.py:464-490) and
scores projections with GateDigitizerProjectionActor; these tests check the
oracle's hole lattice against an independent numpy construction, the hole
traversal distance, a point source in air against the projection geometry
and the voxel-source CDFs against compute_image_3D_CDF (golden fixture).
"""

import math
import pathlib

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import materials as M
from opengate_gb300 import spect as S
from opengate_gb300 import tables as T
from opengate_gb300.scene import Scene, SourceSpec

O = pytest.importorskip("oracle.oracle")
GOLDEN = pathlib.Path(__file__).parent / "golden"
C30 = math.cos(math.radians(30.0))


def hex_metric(qx, qy):
    """max |q . n| over the three face normals (30, 90, 150 degrees) of a hole."""
    return np.maximum.reduce([np.abs(qy), np.abs(qy * 0.5 + qx * C30), np.abs(qy * 0.5 - qx * C30)])


def numpy_holes(sp, a1, a2):
    """Independent lattice search: nearest centre among both lattices' 3x3 neighbourhoods."""
    best = np.full(a1.shape, np.inf)
    for ox, oy in ((0.0, 0.0), (sp.pitch_x / 2, sp.pitch_y / 2)):
        i0 = np.floor((a1 - ox) / sp.pitch_x)
        j0 = np.floor((a2 - oy) / sp.pitch_y)
        for di in (-1, 0, 1, 2):
            for dj in (-1, 0, 1, 2):
                cx = (i0 + di) * sp.pitch_x + ox
                cy = (j0 + dj) * sp.pitch_y + oy
                best = np.minimum(best, hex_metric(a1 - cx, a2 - cy))
    return best


@pytest.mark.parametrize("coll", ["LEHR", "MELP"])
def test_hole_lattice_open_fraction(coll):
    sp = S.SpectSpec(collimator=getattr(S, coll))
    rng = np.random.default_rng(17)
    n = 20000
    a1 = rng.uniform(-200, 200, n)
    a2 = rng.uniform(-200, 200, n)
    inside = np.zeros(n, bool)
    for k in range(n):
        ins, cx, cy = O.find_hole(sp, a1[k], a2[k])
        inside[k] = ins
        if ins:
            assert hex_metric(a1[k] - cx, a2[k] - cy) <= sp.hole_apothem * (1 + 1e-5)
    metric = numpy_holes(sp, a1, a2)
    clear = np.abs(metric - sp.hole_apothem) > 1e-4  # points not on a wall within float32 rounding
    np.testing.assert_array_equal(inside[clear], metric[clear] <= sp.hole_apothem)
    # two hexagons of area 2 sqrt(3) apothem^2 per lattice cell pitch_x * pitch_y
    expect = 4.0 * math.sqrt(3.0) * sp.hole_apothem ** 2 / (sp.pitch_x * sp.pitch_y)
    sigma = math.sqrt(expect * (1 - expect) / n)
    assert abs(inside.mean() - expect) < 5 * sigma
    if coll == "LEHR":
        assert abs(expect - 0.7786) < 1e-3


def test_hex_exit_lands_on_wall():
    sp = S.SpectSpec()
    rng = np.random.default_rng(5)
    a = sp.hole_apothem
    for _ in range(500):
        while True:
            qx, qy = rng.uniform(-a / C30, a / C30), rng.uniform(-a, a)
            if hex_metric(qx, qy) < a:
                break
        phi = rng.uniform(0, 2 * math.pi)
        s = rng.uniform(0.05, 1.0)  # in-plane part of a unit direction
        d1, d2 = s * math.cos(phi), s * math.sin(phi)
        t = O.hex_exit(sp, qx, qy, d1, d2)
        assert t >= 0
        assert abs(hex_metric(qx + t * d1, qy + t * d2) - a) < 1e-4
        assert hex_metric(qx + 0.999 * t * d1, qy + 0.999 * t * d2) < a + 1e-6


def test_frames_are_orthonormal_and_face_the_axis():
    sp = S.SpectSpec(n_runs=7, step_angle_deg=360 / 7)
    fr = sp.all_frames()
    assert fr.shape == (7, 2, 12)
    for r in range(7):
        for h in range(2):
            c, u, e1, e2 = fr[r, h, :3], fr[r, h, 3:6], fr[r, h, 6:9], fr[r, h, 9:]
            np.testing.assert_allclose(np.linalg.norm(c), sp.radius)
            np.testing.assert_allclose(c / sp.radius, u, atol=1e-12)
            m = np.stack([u, e1, e2])
            np.testing.assert_allclose(m @ m.T, np.eye(3), atol=1e-12)
        np.testing.assert_allclose(fr[r, 0, 3:6], -fr[r, 1, 3:6], atol=1e-12)
    assert sp.projection_shape() == (2, 14, 128, 128)


def point_source_scene(pos, energy=0.1405):
    db = M.MaterialDatabase()
    mats = [db.get("G4_AIR"), db.get("G4_Pb"), db.get("G4_SODIUM_IODIDE")]
    pt = T.PhysicsTables(mats)
    src = SourceSpec()
    src.translation = list(pos)
    src.dir_type = C.GG_DIR_ISO
    src.ene_type = C.GG_ENE_MONO
    src.mono = energy
    return Scene(pt, np.zeros((2, 2, 2), np.uint16), [5.0] * 3, [-5.0] * 3, [1500.0] * 3, 0, src)


def test_point_source_in_air_projection():
    """Photopeak counts of a point source sit at its projection on each head."""
    pos = (30.0, 0.0, 20.0)
    scene = point_source_scene(pos)
    sp = S.SpectSpec(n_runs=1, collimator_material=1, crystal_material=2)
    n = 4_000_000
    proj, cnt = O.run_spect(scene, sp, n, seed=5, threads=8)
    assert cnt["histories"] == n and cnt["loop_capped"] == 0
    fr = sp.frames(0)
    half = 0.5 * sp.size[0] * sp.spacing[0]
    for h in range(2):
        peak = proj[h, 0]
        tot = peak.sum()
        # LEHR sensitivity with a 9.5 mm NaI crystal: about 1e-4 counts per 140 keV photon
        assert 6e-5 < tot / n < 1.4e-4
        j, i = np.indices(peak.shape)
        q = np.array(pos) - fr[h, :3]
        fx = (q @ fr[h, 6:9] + half) / sp.spacing[0] - 0.5
        fy = (q @ fr[h, 9:12] + half) / sp.spacing[1] - 0.5
        assert abs((peak * i).sum() / tot - fx) < 0.5
        assert abs((peak * j).sum() / tot - fy) < 0.5
        # in air almost nothing scatters into the 108-126 keV window
        assert proj[h, 1].sum() < 0.05 * tot


def test_voxel_cdfs_match_reference():
    g = np.load(GOLDEN / "voxel_cdf.npz")
    z, y, x = S.voxel_cdfs(g["activity"])
    assert z.dtype == np.float32 and y.shape == g["cdf_y"].shape and x.shape == g["cdf_x"].shape
    np.testing.assert_allclose(z, g["cdf_z"], rtol=0, atol=1e-7)
    np.testing.assert_allclose(y, g["cdf_y"], rtol=0, atol=1e-7)
    np.testing.assert_allclose(x, g["cdf_x"], rtol=0, atol=1e-7)


def test_voxel_source_follows_activity():
    """Oracle voxel source: emission points distribute like the activity image."""
    db = M.MaterialDatabase()
    pt = T.PhysicsTables([db.get("G4_WATER")])
    act = np.zeros((4, 5, 6))
    act[1, 2, 3] = 3.0
    act[3, 0, 0] = 1.0
    act[0, 4, 5] = 4.0
    src = SourceSpec()
    src.set_activity_image(act, [2.0, 3.0, 4.0], [-6.0, -7.5, -8.0])
    src.dir_type = C.GG_DIR_ISO
    scene = Scene(pt, np.zeros(act.shape, np.uint16), [2.0, 3.0, 4.0], [-6.0, -7.5, -8.0], [500.0] * 3, 0, src)
    pos, _, _, _ = O.sample_source(scene, 40000, seed=9)
    ix = np.floor((pos[:, 0] + 6.0) / 2.0).astype(int)
    iy = np.floor((pos[:, 1] + 7.5) / 3.0).astype(int)
    iz = np.floor((pos[:, 2] + 8.0) / 4.0).astype(int)
    keys, counts = np.unique(np.stack([iz, iy, ix], 1), axis=0, return_counts=True)
    got = {tuple(k): c / len(pos) for k, c in zip(keys, counts)}
    assert set(got) == {(1, 2, 3), (3, 0, 0), (0, 4, 5)}
    for k, p in ((1, 2, 3), 0.375), ((3, 0, 0), 0.125), ((0, 4, 5), 0.5):
        assert abs(got[k] - p) < 0.01


def test_projection_metrics_match_reference():
    g = np.load(GOLDEN / "spect_metrics.npz")
    n = int(g["n"])
    u_ref = S.compute_history_by_history_relative_uncertainty(g["counts"], g["counts2"], n)
    np.testing.assert_array_equal(u_ref, g["u_ref"])
    np.testing.assert_array_equal(S.compute_poisson_relative_uncertainty(g["test"]), g["u_test"])
    np.testing.assert_array_equal(S.compute_poisson_relative_uncertainty(g["counts"]), g["poisson"])
    np.testing.assert_array_equal(S.compute_efficiency(u_ref, 12.5), g["efficiency"])
    z = S.compute_zscore(g["counts"], g["test"], (u_ref * g["counts"]) ** 2, (g["u_test"] * g["test"]) ** 2)
    np.testing.assert_array_equal(z, g["zscore"])
    np.testing.assert_array_equal(S.compute_speedup(u_ref, g["u_test"], 12.5, 0.8), g["speedup"])


def test_nm670_housing_layers_and_validation():
    """The NM670 shielding box as slabs (ge_discovery_nm670.py:215-262): aluminium cover,
    TiO2 reflector, 80 mm Pyrex back compartment, the rest of the 101.375 mm lead cover and
    the 10 mm steel back; GateMaterials.db compositions; bad layers refused."""
    cover, back = S.housing_layers("nm670", S.CRYSTALS["3/8"])
    assert cover == (1.3, "Aluminium")
    assert [m for _, m in back] == ["TiO2", "Pyrex66", "Lead", "Steel"]
    assert sum(t for t, _ in back[:3]) + 1.3 + 9.525 == pytest.approx(101.375)
    assert back[3][0] == pytest.approx(10.0)
    _, back58 = S.housing_layers("nm670", S.CRYSTALS["5/8"])
    assert back58[2][0] == pytest.approx(101.375 - 1.3 - 15.875 - 1.2 - 80.0)
    assert S.housing_layers("none", 9.525) == (None, [])
    with pytest.raises(NotImplementedError):
        S.housing_layers("intevo", 9.525)
    db = M.MaterialDatabase()
    for name in S.HOUSING_MATERIALS["nm670"]:
        m = db.get(name)
        assert m.density > 1.0 and abs(m.fractions.sum() - 1.0) < 1e-12
    assert db.get("Steel").z == [6, 25, 26] and db.get("Lead").density == pytest.approx(11.4)
    sp = S.SpectSpec()
    sp.apply_housing("nm670", {n: 10 + k for k, n in enumerate(S.HOUSING_MATERIALS["nm670"])}.get)
    d = sp.desc()
    assert (d.n_cover, d.cover_material, d.n_back, d.shielded_sides) == (1, 10, 4, 1)
    assert list(d.back_material) == [11, 12, 13, 14]
    assert sp.housing_depth() == pytest.approx(35.0 + 1.3 + 9.525 + 1.2 + 80.0 + 9.35 + 10.0)
    with pytest.raises(ValueError):
        sp.set_housing(None, [(1.0, 1)] * 5)
    with pytest.raises(ValueError):
        sp.set_housing((0.0, 1), ())
    sp.apply_housing("none", None)
    d = sp.desc()
    assert (d.n_cover, d.n_back, d.shielded_sides, sp.housing) == (0, 0, 0, "none")


def test_shielded_sides_stop_side_entries_in_the_oracle():
    """A beam aimed at the side face of a head: with open sides photons reach the crystal
    through it and are counted; with shielded sides none is."""
    db = M.MaterialDatabase()
    pt = T.PhysicsTables([db.get("G4_AIR"), db.get("G4_Pb"), db.get("G4_SODIUM_IODIDE")])
    sp = S.SpectSpec(n_heads=1, n_runs=1, collimator_material=1, crystal_material=2,
                     windows=((0.126, 0.154),))
    fr = sp.frames(0)[0]
    u, e1 = fr[3:6], fr[6:9]
    # a point beside the head at the crystal's depth, aimed along e1 at the side face
    depth = sp.collimator_thickness + sp.gap + 0.5 * sp.crystal_thickness
    p = fr[:3] + depth * u - (sp.half_width + 20.0) * e1
    src = SourceSpec()
    src.translation = list(p)
    src.dir_type = C.GG_DIR_MOMENTUM
    src.momentum = list(e1)
    src.ene_type = C.GG_ENE_MONO
    src.mono = 0.1405
    scene = Scene(pt, np.zeros((2, 2, 2), np.uint16), [5.0] * 3, [-5.0] * 3, [1500.0] * 3, 0, src)
    open_proj, _ = O.run_spect(scene, sp, 20000, seed=3, threads=4)
    sp.set_housing(None, (), shielded_sides=True)
    shut_proj, cnt = O.run_spect(scene, sp, 20000, seed=3, threads=4)
    assert open_proj.sum() > 1000 and shut_proj.sum() == 0
    assert cnt["head_steps"] == 0 and cnt["escaped"] == 20000


def test_forced_direction_equals_angle_check_in_expectation():
    """ForceDirection (history h aimed at head h mod 2 within the cone, weight (1 - cos)/2) and
    the angle check by rejection on the same cone give the same expected weighted projection
    totals per head and window (oracle, primary free flight, Lu-177 / MELP / NM670 housing)."""
    from opengate_gb300 import workloads as W

    sc, sp, _ = W.spect_phantom(shape=(40, 64, 64), spacing=4.8, n_runs=1, nuclide=W.LU177, collimator=S.MELP,
                                windows=((0.1872, 0.2288), (0.1017, 0.1243)), housing="nm670")
    tol = math.radians(10.0)
    sp.set_free_flight(angle_tolerance_max=tol)
    n = 600_000
    w, w2, _ = O.run_spect_ff(sc, sp, n, seed=5, threads=8)
    src = sc.source
    src.dir_type = C.GG_DIR_FORCED
    src.fd_angle_min, src.fd_angle_max = 0.0, tol
    sc.set_source(src)
    m = 60_000  # per head
    wf, wf2, cnt = O.run_spect_ff(sc, sp, 2 * m, seed=6, threads=8)
    assert cnt["histories"] == 2 * m and cnt["skipped"] == 0
    for h in range(2):
        for k in range(2):
            a, va = w[h, k::2].sum() / n, w2[h, k::2].sum() / n ** 2
            b, vb = wf[h, k::2].sum() / m, wf2[h, k::2].sum() / m ** 2
            assert a > 0 and b > 0
            assert abs(a - b) < 4.0 * math.sqrt(va + vb), (h, k, a, b)
    # the forced estimate is far less noisy per history
    assert wf2[0, 0::2].sum() / wf[0, 0::2].sum() ** 2 * m < w2[0, 0::2].sum() / w[0, 0::2].sum() ** 2 * n
