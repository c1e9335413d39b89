"""ARF surrogate on the CPU: the FP64 network oracle and the training-row oracle.

The network oracle (oracle/arf_mlp.py) is itself checked against central
finite differences before it is used to judge the GPU gradients; the
training-row oracle (GateARFTrainingDatasetActor restated in oracle/gg_oracle.c)
is checked for determinism, its domain and its Russian roulette.
"""

import math

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import spect as S
from opengate_gb300 import workloads as W

O = pytest.importorskip("oracle.oracle")
M = pytest.importorskip("oracle.arf_mlp")


def random_params(seed, n_classes):
    rng = np.random.default_rng(seed)
    d = {}
    for k, shape in M.SHAPES.items():
        fan_in = shape[1] if len(shape) == 2 else 1
        d[k] = rng.uniform(-1, 1, size=shape) * (math.sqrt(6.0 / fan_in) if len(shape) == 2 else 0.1)
    d["W4"][n_classes:] = 0.0
    d["b4"][n_classes:] = 0.0
    return M.pack(d).astype(np.float32).astype(np.float64)


def random_rows(seed, n, n_classes):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(0.05, 0.25, n), rng.uniform(0, 30, n), rng.uniform(-180, 180, n),
                     rng.integers(0, n_classes, n)], axis=1).astype(np.float32)


MEAN, STD = [15.0, 0.0, 0.15], [8.66, 103.9, 0.0577]


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0, 3.0e38], dtype=np.float32)
    got = M.bf16(x)
    assert got[0] == 1.0
    assert got[1] == 1.0  # tie -> even mantissa
    assert got[2] == 1.0 + 4 * 2 ** -8  # tie -> even (up)
    assert got[3] == 1.0
    assert got[4] == -2.5 and got[5] == 0.0
    assert np.all(np.abs(M.bf16(np.linspace(-3, 3, 1001)) - np.linspace(-3, 3, 1001)) <= 2 ** -8 * 3)


def test_oracle_gradient_matches_finite_differences():
    n_classes = 4
    params = random_params(1, n_classes)
    rows = random_rows(2, 64, n_classes)
    loss, g = M.loss_and_grad(params, rows, MEAN, STD, n_classes, bf16_points=False)
    rng = np.random.default_rng(3)
    idx = []
    for name in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"):
        o, size = M.OFF[name]
        rows_used = n_classes if name in ("W4", "b4") else None
        lim = size if rows_used is None else (rows_used * (M.HID if name == "W4" else 1))
        idx += list(o + rng.integers(0, lim, 4))
    h = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += h
        p2[i] -= h
        l1, _ = M.loss_and_grad(p1, rows, MEAN, STD, n_classes, bf16_points=False)
        l2, _ = M.loss_and_grad(p2, rows, MEAN, STD, n_classes, bf16_points=False)
        fd = (l1 - l2) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])
    assert loss > 0


def test_bf16_emulation_stays_close_to_fp64():
    n_classes = 3
    params = random_params(5, n_classes)
    rows = random_rows(6, 256, n_classes)
    _, g64 = M.loss_and_grad(params, rows, MEAN, STD, n_classes, bf16_points=False)
    _, g16 = M.loss_and_grad(params, rows, MEAN, STD, n_classes, bf16_points=True)
    assert np.linalg.norm(g16 - g64) / np.linalg.norm(g64) < 3e-2


def test_arf_weights_undo_russian_roulette():
    p = np.array([[0.5, 0.25, 0.25], [0.0, 1.0, 0.0]])
    w = M.arf_weights(p, 3.0)
    np.testing.assert_allclose(w[0], [0.75, 0.125, 0.125])
    np.testing.assert_allclose(w[1], [0.0, 1.0, 0.0])


def _arf_case(rr=5.0):
    scene, sp, _ = W.spect_phantom(shape=(40, 64, 64), spacing=4.8, n_runs=1)
    a = C.ArfSampling()
    a.e_min, a.e_max = 0.05, 0.16
    a.cos_theta_max = math.cos(math.radians(20.0))
    a.half_extent[:] = [150.0, 150.0]
    a.russian_roulette = rr
    return scene, sp, a


def test_oracle_training_rows():
    scene, sp, a = _arf_case()
    rows, cnt = O.arf_dataset(scene.tables_desc, sp, a, 200_000, seed=7, threads=4)
    rows2, _ = O.arf_dataset(scene.tables_desc, sp, a, 200_000, seed=7, threads=1)
    np.testing.assert_array_equal(rows, rows2)  # independent of the thread split
    assert cnt["histories"] == 200_000 and cnt["loop_capped"] == 0
    e, th, ph, w = rows.T
    assert np.all((e >= 0.05) & (e <= 0.16))
    assert np.all((th >= 0) & (th <= 20.0 + 1e-4)) and np.all(np.abs(ph) <= 180.0)
    assert set(np.unique(w)) <= {0.0, 1.0, 2.0}
    # w = 0 rows kept with probability 1 / 5: the kept count agrees with the singles count
    n_detected = int((w > 0).sum())
    n_zero = int((w == 0).sum())
    expect = (200_000 - n_detected) / 5.0
    assert abs(n_zero - expect) < 5 * math.sqrt(expect)
    # photopeak detection needs a direction along the holes
    peak = (w == 1) & (e > 0.126)
    assert np.median(th[peak]) < 3.0
