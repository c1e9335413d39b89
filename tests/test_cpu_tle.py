"""Track-length estimator, host side and oracle: mu_en tables against the
element databases and published NIST values, the lookup's edge and range
behaviour, and the oracle's estimator against analog scoring."""

import math

import numpy as np
import pytest

from opengate_gb300 import mu_tables as M
from opengate_gb300 import workloads as W

WATER = ((1, 8), (0.111894, 0.888106))


def test_single_element_material_reproduces_element_rows():
    e, mu, muen = M.element_table("NIST", 8)
    t = M.MaterialMuTable([8], [1.0], "NIST")
    inner = e[1:-2]
    np.testing.assert_allclose(t.mu_en_over_rho(inner), muen[1:-2], rtol=1e-12)
    np.testing.assert_allclose(t.mu_over_rho(inner), mu[1:-2], rtol=1e-12)
    # between rows: log-log interpolation
    x = math.sqrt(e[3] * e[4])
    expect = math.exp(0.5 * (math.log(muen[3]) + math.log(muen[4])))
    assert float(t.mu_en_over_rho(x)) == pytest.approx(expect, rel=1e-12)


def test_water_mu_en_matches_published_nist_values():
    # Hubbell & Seltzer, water (liquid): mu_en/rho in cm2/g
    t = M.material_table(*WATER, "NIST")
    for e, ref in ((0.01, 4.944), (0.1, 0.02546), (0.5, 0.03299)):
        assert float(t.mu_en_over_rho(e)) == pytest.approx(ref, rel=5e-3)
    te = M.material_table(*WATER, "EPDL")
    assert float(te.mu_en_over_rho(0.1)) == pytest.approx(0.02546, rel=1e-2)


def test_absorption_edge_kept_twice():
    # lead K edge at 88.0 keV: the material table holds both sides of the jump
    t = M.MaterialMuTable([82], [1.0], "NIST")
    assert float(t.mu_over_rho(0.0879)) * 3 < float(t.mu_over_rho(0.0881))
    assert np.sum(np.diff(t.ln_e) == 0) >= 1


def test_lookup_above_the_table_keeps_the_second_last_row():
    # GateMuTable::GetMuEnOverRho: outside (or on) the last interval, the lower row
    t = M.material_table(*WATER, "NIST")
    last2 = math.exp(t.ln_muen[-2])
    assert float(t.mu_en_over_rho(1.0)) == pytest.approx(last2, rel=1e-12)
    assert float(t.mu_en_over_rho(5.0)) == pytest.approx(last2, rel=1e-12)


def test_unknown_database_raises():
    with pytest.raises(ValueError):
        M.element_table("XCOM", 8)


def test_muen_table_shape_and_units():
    sc = W.water_pencil(energy=0.3)
    tab = sc.pt.muen("NIST")
    assert tab.shape == (sc.pt.n_comp, 512) and tab.dtype == np.float32
    # 0.1 x mu_en/rho (mm^-1 per g/cm3) at 100 keV on the grid
    grid = np.exp(np.linspace(np.log(1e-3), np.log(20.0), 512))
    i = int(np.argmin(np.abs(grid - 0.1)))
    c = int(sc.pt.mat_comp[np.unique(sc.labels)[0]])
    assert tab[c, i] == pytest.approx(0.1 * float(M.material_table(*WATER, "NIST").mu_en_over_rho(grid[i])),
                                      rel=1e-3)


O = pytest.importorskip("oracle.oracle")


def test_oracle_tle_zero_threshold_is_analog():
    sc = W.water_pencil(energy=0.3)
    a = O.run_dose(sc, 5000, 3, threads=4)
    b = O.run_dose(sc, 5000, 3, threads=4, tle=sc.tle_desc(0.0, 0.0, "EPDL"))
    assert a[2] == b[2]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_oracle_tle_against_analog():
    from opengate_gb300.dose import mean_relative_uncertainty

    sc = W.water_pencil(energy=0.3)
    n = 100_000
    a, qa, _ = O.run_dose(sc, n, 7, threads=8)
    t, qt, ct = O.run_dose(sc, n, 8, threads=8, tle=sc.tle_desc(np.inf, 0.0, "EPDL"))
    assert t.sum() == pytest.approx(a.sum(), rel=0.02)
    assert mean_relative_uncertainty(t, qt, n) < mean_relative_uncertainty(a, qa, n) / 5
    # kill energy: photons at or below it stop and deposit all their energy on the spot
    # (none of it escapes any more), so fewer interactions and more energy in the image
    k, _, ck = O.run_dose(sc, n, 8, threads=8, tle=sc.tle_desc(np.inf, 0.2, "EPDL"))
    assert ck["real_interactions"] < ct["real_interactions"]
    assert k.sum() > 1.2 * t.sum()


def test_tle_actor_options():
    from opengate_gb300 import api

    sim = api.Simulation()
    a = sim.add_actor("TLEDoseActor", "tle")
    assert a.tle_threshold_type == "None" and a.database == "EPDL" and a.energy_min == 0.0
    assert a.threshold_energy == np.inf
    a.tle_threshold_type = "energy"
    a.tle_threshold = 0.2
    assert a.threshold_energy == 0.2
