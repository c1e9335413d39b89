"""Scatter splitting in the oracle (ScatterSplittingFreeFlightActor restatement),
cases whose answer is known without a GPU."""

import numpy as np
import pytest

from opengate_gb300 import materials as M
from opengate_gb300 import spect as S
from opengate_gb300 import tables as T
from opengate_gb300 import workloads as W
from opengate_gb300.scene import Scene

O = pytest.importorskip("oracle.oracle")


def _case():
    return W.spect_phantom(shape=(20, 32, 32), spacing=9.6, n_runs=1, nuclide=W.TC99M, collimator=S.LEHR,
                           windows=((0.126, 0.154), (0.108, 0.126)))


def test_no_scatter_outside_the_heads_no_copies():
    """In vacuum nothing scatters outside the heads: no copy, no weight, and every analog
    photon ends at a head (killed there) or leaves the world."""
    scene, sp, _ = _case()
    mats = list(scene.pt.materials)
    mats[0] = M.MaterialDatabase().get("G4_Galactic")
    vac = Scene(T.PhysicsTables(mats), np.zeros_like(scene.labels), scene.spacing, scene.corner, scene.world_half, 0,
                scene.source)
    sp.set_scatter_splitting(10, 10, 10)
    w, w2, cnt = O.run_spect_ff(vac, sp, 20_000, seed=5, threads=4)
    assert w.sum() == 0 and w2.sum() == 0
    assert cnt["real_interactions"] == 0 and cnt["head_steps"] == 0 and cnt["singles"] == 0
    assert cnt["escaped"] == cnt["histories"]


def test_factors_zero_or_level_zero_no_copies():
    scene, sp, _ = _case()
    sp.set_scatter_splitting(0, 0, 10)
    w, _, cnt = O.run_spect_ff(scene, sp, 20_000, seed=6, threads=4)
    assert w.sum() == 0 and cnt["real_interactions"] > 0 and cnt["head_steps"] == 0
    # level 0: the first Compton kills the photon without copies; no Rayleigh factor
    sp.set_scatter_splitting(5, 0, 0)
    w, _, cnt0 = O.run_spect_ff(scene, sp, 20_000, seed=6, threads=4)
    assert w.sum() == 0 and cnt0["real_interactions"] <= cnt["real_interactions"]


def test_copies_leave_the_analog_histories_alone():
    """The copies draw from their own random streams: the analog histories (stream 0)
    and their interactions do not depend on the splitting factors; more copies, more
    free flights."""
    scene, sp, _ = _case()
    sp.set_scatter_splitting(1, 1, 100)
    w1, _, c1 = O.run_spect_ff(scene, sp, 60_000, seed=7, threads=8)
    sp.set_scatter_splitting(8, 8, 100)
    w8, _, c8 = O.run_spect_ff(scene, sp, 60_000, seed=7, threads=8)
    assert w1.sum() > 0 and w8.sum() > 0
    # same analog histories (stream 0 untouched by the copies): same analog interactions
    assert c1["real_interactions"] == c8["real_interactions"]
    assert c8["world_steps"] > c1["world_steps"] and c8["singles"] > c1["singles"]
