"""Singles list and its ROOT output, on the CPU.

The ROOT writer (opengate_gb300.root_io) is checked by a structural read-back
that follows the TTree's streamed members, byte counts and basket seeks; the
oracle's singles list is checked against the oracle's own projection: every
single that falls in a window and on the detector adds one count to exactly
the pixel the projection counted (GateDigitizerProjectionActor.cpp:127-223).
"""

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import root_io
from opengate_gb300 import spect as S
from opengate_gb300 import workloads as W

O = pytest.importorskip("oracle.oracle")


def sort_singles(rec):
    """Records in a reproducible order (the list holds them in completion order)."""
    return rec[np.lexsort((rec["weight"], rec["a2"], rec["a1"], rec["energy"], rec["run"], rec["head"],
                           rec["event_id"]))]


def projection_of(rec, sp, precision=32):
    """Counts (or weights) of a singles list in the projection layout, with the pixel and
    window tests in the transport's arithmetic (gg_spect.cuh score_singles)."""
    f = np.float32 if precision == 32 else np.float64
    d = sp.desc()
    out = np.zeros(sp.projection_shape(), dtype=np.float64).reshape(sp.n_heads, sp.n_runs, sp.n_windows,
                                                                    sp.size[1], sp.size[0])
    fx = (f(rec["a1"]) + f(0.5 * sp.size[0] * sp.spacing[0])) * f(1.0 / sp.spacing[0])
    fy = (f(rec["a2"]) + f(0.5 * sp.size[1] * sp.spacing[1])) * f(1.0 / sp.spacing[1])
    on = (fx >= 0) & (fx < sp.size[0]) & (fy >= 0) & (fy < sp.size[1])
    e = f(rec["energy"])
    for k in range(sp.n_windows):
        m = on & (e >= f(d.window_lo[k])) & (e < f(d.window_hi[k]))
        np.add.at(out, (rec["head"][m], rec["run"][m], k, fy[m].astype(np.int64), fx[m].astype(np.int64)),
                  rec["weight"][m])
    return out.reshape(sp.projection_shape())


def small_case(n_runs=2):
    return W.spect_phantom(shape=(40, 64, 64), spacing=4.8, n_runs=n_runs, nuclide=W.TC99M, collimator=S.LEHR,
                           windows=((0.126, 0.154), (0.108, 0.126)))


def test_root_tree_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    n = 70_001
    cols = {"EventID": np.arange(n, dtype=np.int64) * 3, "TotalEnergyDeposit": rng.random(n),
            "HeadID": rng.integers(0, 2, n).astype(np.int32), "u32": rng.integers(0, 2**32, n).astype(np.uint32),
            "u64": rng.integers(0, 2**63, n).astype(np.uint64) * 2, "f32": rng.random(n).astype(np.float32)}
    path = tmp_path / "singles.root"
    root_io.write_tree(path, "Singles", cols, basket_entries=32_000)
    data = path.read_bytes()
    assert data[:4] == b"root" and len(data) > sum(a.nbytes for a in cols.values())
    back = root_io.read_tree(path, "Singles")
    assert list(back) == list(cols)
    for k, a in cols.items():
        assert back[k].dtype == a.dtype
        np.testing.assert_array_equal(back[k], a)
    with pytest.raises(KeyError):
        root_io.read_tree(path, "Hits")


def test_root_tree_edge_cases(tmp_path):
    root_io.write_tree(tmp_path / "empty.root", "Singles", {"a": np.zeros(0), "b": np.zeros(0, np.int32)})
    back = root_io.read_tree(tmp_path / "empty.root", "Singles")
    assert {k: len(v) for k, v in back.items()} == {"a": 0, "b": 0}
    one = {"x" * 300: np.array([1.5])}  # a name past the one-byte string length
    root_io.write_tree(tmp_path / "long.root", "T", one, basket_entries=1)
    np.testing.assert_array_equal(root_io.read_tree(tmp_path / "long.root", "T")["x" * 300], [1.5])
    with pytest.raises(ValueError):
        root_io.write_tree(tmp_path / "bad.root", "T", {"a": np.zeros(3), "b": np.zeros(4)})
    with pytest.raises(ValueError):
        root_io.write_tree(tmp_path / "bad.root", "T", {"a": np.zeros(3, np.complex128)})
    with pytest.raises(ValueError):
        root_io.write_tree(tmp_path / "bad.root", "T", {})


@pytest.mark.parametrize("blur", [False, True])
def test_oracle_singles_make_its_projection(blur):
    scene, sp, _ = small_case()
    if blur:
        sp.set_energy_blur("InverseSquare", resolution=0.063, reference=0.14057)
        sp.set_spatial_blur(3.0 * 0.42466090014400953, keep_in_solid_limits=True, truncated=False)
    n = 600_000
    (proj, cnt), rec = O.with_singles(32, 1 << 20, lambda: O.run_spect(scene, sp, n, 5, threads=8))
    assert len(rec) == cnt["singles"] > 200
    assert set(np.unique(rec["head"])) <= {0, 1} and set(np.unique(rec["run"])) <= {0, 1}
    assert np.all(rec["event_id"] < 2 * n) and np.all(rec["weight"] == 1.0)
    np.testing.assert_array_equal(projection_of(rec, sp), proj)
    # the list does not change the run
    proj2, cnt2 = O.run_spect(scene, sp, n, 5, threads=8)
    np.testing.assert_array_equal(proj2, proj)
    assert cnt2 == cnt


def test_oracle_singles_overflow_is_reported():
    scene, sp, _ = small_case(n_runs=1)
    with pytest.raises(RuntimeError, match="overflow"):
        O.with_singles(32, 10, lambda: O.run_spect(scene, sp, 400_000, 5, threads=4))


def test_singles_columns_on_the_crystal_plane():
    _, sp, _ = small_case()
    rec = np.zeros(4, dtype=C.SINGLE_DTYPE)
    rec["event_id"] = [7, 7, 9, 11]
    rec["head"] = [0, 1, 0, 1]
    rec["run"] = [0, 0, 1, 1]
    rec["a1"] = [0.0, 10.0, -5.0, 3.0]
    rec["a2"] = [0.0, -2.0, 4.0, 1.0]
    rec["energy"] = 0.14
    rec["weight"] = 1.0
    cols = sp.singles_columns(rec)
    assert list(cols) == ["EventID", "RunID", "HeadID", "TotalEnergyDeposit", "PostPosition_X", "PostPosition_Y",
                          "PostPosition_Z", "Weight"]
    f = sp.all_frames()[rec["run"], rec["head"]]
    pos = np.stack([cols["PostPosition_X"], cols["PostPosition_Y"], cols["PostPosition_Z"]], 1)
    rel = pos - f[:, 0:3]
    np.testing.assert_allclose(np.einsum("ij,ij->i", rel, f[:, 3:6]), sp.crystal_depth(), atol=1e-9)
    np.testing.assert_allclose(np.einsum("ij,ij->i", rel, f[:, 6:9]), rec["a1"], atol=1e-9)
    np.testing.assert_allclose(np.einsum("ij,ij->i", rel, f[:, 9:12]), rec["a2"], atol=1e-9)
