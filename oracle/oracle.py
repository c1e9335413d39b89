"""ctypes front-end of the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It runs a :class:`opengate_gb300.scene.Scene`
through ``libggo32.so`` / ``libggo64.so`` and returns the float64 edep and
edep-squared images plus the counters, in the same layout as the GPU path.
"""

import ctypes
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

from opengate_gb300 import _capi as C  # noqa: E402

from . import build_oracle  # noqa: E402

_libs = {}


def lib(precision=32):
    if precision not in _libs:
        build_oracle.build()
        L = ctypes.CDLL(str(HERE / "_build" / f"libggo{precision}.so"))
        pre = f"ggo{precision}_"
        fn = getattr(L, pre + "run_dose")
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.POINTER(C.TablesDesc), ctypes.POINTER(C.VolumeDesc),
                       ctypes.POINTER(C.WorldDesc), ctypes.POINTER(C.SourceDesc), ctypes.c_uint64,
                       ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                       ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                       ctypes.POINTER(ctypes.c_uint64)]
        fn = getattr(L, pre + "run_dose_tle")
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.POINTER(C.TablesDesc), ctypes.POINTER(C.VolumeDesc),
                       ctypes.POINTER(C.WorldDesc), ctypes.POINTER(C.SourceDesc), ctypes.POINTER(C.TleDesc),
                       ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                       ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                       ctypes.POINTER(ctypes.c_uint64)]
        for name in ("log", "exp"):
            f = getattr(L, pre + name)
            f.restype = ctypes.c_double
            f.argtypes = [ctypes.c_double]
        f = getattr(L, pre + "sincos_turn")
        f.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        f = getattr(L, pre + "philox")
        f.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3
        f = getattr(L, pre + "sample_compton")
        f.argtypes = [ctypes.c_double, ctypes.c_uint64, ctypes.c_int,
                      ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        descs = [ctypes.POINTER(C.TablesDesc), ctypes.POINTER(C.VolumeDesc), ctypes.POINTER(C.WorldDesc),
                 ctypes.POINTER(C.SourceDesc)]
        f = getattr(L, pre + "sample_source")
        f.restype = ctypes.c_int
        f.argtypes = descs + [ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_uint64)]
        f = getattr(L, pre + "sample_rayleigh")
        f.argtypes = [ctypes.POINTER(C.TablesDesc), ctypes.c_int, ctypes.c_double, ctypes.c_uint64, ctypes.c_int,
                      ctypes.POINTER(ctypes.c_double)]
        f = getattr(L, pre + "first_flight")
        f.restype = ctypes.c_int
        f.argtypes = descs + [ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
        _libs[precision] = L
    return _libs[precision]


def run_dose(scene, n, seed, first=0, batch=0, threads=1, precision=32, squared=True, tle=None):
    """Oracle run of histories [first, first + n): (edep, edep2 or None, counters dict).
    ``tle``: a gg_tle_desc (Scene.tle_desc) for the track-length estimator."""
    L = lib(precision)
    nv = scene.n_voxels
    edep = np.zeros(nv, dtype=np.float64)
    edep2 = np.zeros(nv, dtype=np.float64) if squared else None
    cnt = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
    descs = (ctypes.byref(scene.tables_desc), ctypes.byref(scene.volume_desc), ctypes.byref(scene.world_desc),
             ctypes.byref(scene.source_desc))
    outs = (C.ptr(edep, ctypes.c_double), C.ptr(edep2, ctypes.c_double), C.ptr(cnt, ctypes.c_uint64))
    if tle is not None:
        st = getattr(L, f"ggo{precision}_run_dose_tle")(*descs, ctypes.byref(tle), seed, first, n, batch, threads,
                                                        *outs)
    else:
        st = getattr(L, f"ggo{precision}_run_dose")(*descs, seed, first, n, batch, threads, *outs)
    if st != 0:
        raise RuntimeError(f"oracle run failed with status {st}")
    shape = scene.labels.shape
    counters = {name: int(cnt[i]) for i, name in enumerate(C.COUNTER_NAMES)}
    return edep.reshape(shape), (edep2.reshape(shape) if squared else None), counters


def run_dose_grid(scene, grid, n, seed, first=0, batch=0, threads=1, precision=32, squared=True):
    """Oracle run with the tally on its own grid (grid: a C.DoseGridDesc):
    (edep, edep2 or None, dose sum or None, dose2 or None, counters), grid shape [nz][ny][nx]."""
    L = lib(precision)
    fn = getattr(L, f"ggo{precision}_run_dose_grid")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(C.TablesDesc), ctypes.POINTER(C.VolumeDesc), ctypes.POINTER(C.WorldDesc),
                   ctypes.POINTER(C.SourceDesc), ctypes.POINTER(C.DoseGridDesc), ctypes.c_uint64, ctypes.c_uint64,
                   ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int] + [ctypes.POINTER(ctypes.c_double)] * 4 + \
        [ctypes.POINTER(ctypes.c_uint64)]
    shape = (grid.dims[2], grid.dims[1], grid.dims[0])
    nv = int(np.prod(shape))
    edep = np.zeros(nv)
    edep2 = np.zeros(nv) if squared else None
    dose = np.zeros(nv) if grid.score_dose else None
    dose2 = np.zeros(nv) if grid.score_dose and squared else None
    cnt = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
    descs = (ctypes.byref(scene.tables_desc), ctypes.byref(scene.volume_desc), ctypes.byref(scene.world_desc),
             ctypes.byref(scene.source_desc))
    st = fn(*descs, ctypes.byref(grid), seed, first, n, batch, threads,
            *(C.ptr(a, ctypes.c_double) for a in (edep, edep2, dose, dose2)), C.ptr(cnt, ctypes.c_uint64))
    if st != 0:
        raise RuntimeError(f"oracle run failed with status {st}")
    r = lambda a: None if a is None else a.reshape(shape)  # noqa: E731
    return r(edep), r(edep2), r(dose), r(dose2), {name: int(cnt[i]) for i, name in enumerate(C.COUNTER_NAMES)}


def philox(ctr, key, precision=32):
    L = lib(precision)
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    getattr(L, f"ggo{precision}_philox")(c, k, o)
    return list(o)


def math_fn(name, x, precision=32):
    return getattr(lib(precision), f"ggo{precision}_{name}")(float(x))


def sincos_turn(f, precision=32):
    s, c = ctypes.c_double(), ctypes.c_double()
    getattr(lib(precision), f"ggo{precision}_sincos_turn")(float(f), ctypes.byref(s), ctypes.byref(c))
    return s.value, c.value


def sample_compton(e, n, seed=1, precision=32):
    eps = np.zeros(n)
    cost = np.zeros(n)
    getattr(lib(precision), f"ggo{precision}_sample_compton")(
        float(e), seed, n, C.ptr(eps, ctypes.c_double), C.ptr(cost, ctypes.c_double))
    return eps, cost


def _descs(scene):
    return (ctypes.byref(scene.tables_desc), ctypes.byref(scene.volume_desc), ctypes.byref(scene.world_desc),
            ctypes.byref(scene.source_desc))


def sample_source(scene, n, seed=1, precision=32):
    """Primary positions, directions and energies of histories 0..n-1."""
    pos = np.zeros((n, 3))
    d = np.zeros((n, 3))
    e = np.zeros(n)
    cnt = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
    st = getattr(lib(precision), f"ggo{precision}_sample_source")(
        *_descs(scene), seed, n, C.ptr(pos, ctypes.c_double), C.ptr(d, ctypes.c_double),
        C.ptr(e, ctypes.c_double), C.ptr(cnt, ctypes.c_uint64))
    if st != 0:
        raise RuntimeError(f"source sampling failed with status {st}")
    return pos, d, e, {name: int(cnt[i]) for i, name in enumerate(C.COUNTER_NAMES)}


def sample_rayleigh(scene, comp, e, n, seed=1, precision=32):
    cost = np.zeros(n)
    getattr(lib(precision), f"ggo{precision}_sample_rayleigh")(
        ctypes.byref(scene.tables_desc), comp, float(e), seed, n, C.ptr(cost, ctypes.c_double))
    return cost


def first_flight(scene, n, seed=1, precision=32):
    """(transmitted, interacted) counts of the first flight through the image."""
    out = np.zeros(2, dtype=np.uint64)
    st = getattr(lib(precision), f"ggo{precision}_first_flight")(*_descs(scene), seed, n,
                                                                   C.ptr(out, ctypes.c_uint64))
    if st != 0:
        raise RuntimeError(f"first flight failed with status {st}")
    return int(out[0]), int(out[1])


def _with_blur(L, precision, spect, call):
    """Runs call() with the SPECT set-up's digitizer blurring installed in the oracle."""
    f = getattr(L, f"ggo{precision}_set_blur")
    f.argtypes = [ctypes.POINTER(C.BlurDesc)]
    f(ctypes.byref(getattr(spect, "blur", C.BlurDesc())))
    try:
        return call()
    finally:
        f(None)


def with_singles(precision, capacity, call):
    """Runs call() with a singles list of `capacity` records installed in the oracle:
    (call's result, C.SINGLE_DTYPE records in completion order).  Raises on overflow."""
    L = lib(precision)
    f = getattr(L, f"ggo{precision}_set_singles")
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
    count = getattr(L, f"ggo{precision}_singles_count")
    count.restype = ctypes.c_uint64
    buf = np.zeros(int(capacity), dtype=C.SINGLE_DTYPE)
    f(buf.ctypes.data_as(ctypes.c_void_p), int(capacity))
    try:
        res = call()
        n = int(count())
    finally:
        f(None, 0)
    if n > capacity:
        raise RuntimeError(f"oracle singles list overflow: {n} > {capacity}")
    return res, buf[:n]


def sample_blur(blur, half_w, e, a1, a2, n, seed=1, precision=32):
    """n blurred singles of one event: (energies, a1, a2) float64 arrays."""
    L = lib(precision)
    f = getattr(L, f"ggo{precision}_sample_blur")
    f.argtypes = [ctypes.POINTER(C.BlurDesc), ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                  ctypes.c_uint64, ctypes.c_uint64] + [ctypes.POINTER(ctypes.c_double)] * 3
    out = [np.empty(n) for _ in range(3)]
    f(ctypes.byref(blur), half_w, e, a1, a2, n, seed, *(C.ptr(o, ctypes.c_double) for o in out))
    return tuple(out)


def erf(x, precision=32):
    f = getattr(lib(precision), f"ggo{precision}_erf")
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_double]
    return f(float(x))


def run_spect(scene, spect, n_per_run, seed, first=0, threads=1, precision=32):
    """Oracle SPECT run: (projection counts [head][run*window][y][x] float64, counters)."""
    L = lib(precision)
    fn = getattr(L, f"ggo{precision}_run_spect")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(C.TablesDesc), ctypes.POINTER(C.VolumeDesc), ctypes.POINTER(C.WorldDesc),
                   ctypes.POINTER(C.SourceDesc), ctypes.POINTER(C.SpectDesc), ctypes.POINTER(ctypes.c_double),
                   ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    shape = spect.projection_shape()
    proj = np.zeros(int(np.prod(shape)), dtype=np.uint64)
    cnt = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
    desc = spect.desc()
    frames = spect.all_frames()
    st = _with_blur(L, precision, spect, lambda: fn(
        *_descs(scene), ctypes.byref(desc), C.ptr(frames, ctypes.c_double), seed, first, n_per_run, threads,
        C.ptr(proj, ctypes.c_uint64), C.ptr(cnt, ctypes.c_uint64)))
    if st != 0:
        raise RuntimeError(f"oracle SPECT run failed with status {st}")
    return proj.astype(np.float64).reshape(shape), {name: int(cnt[i]) for i, name in enumerate(C.COUNTER_NAMES)}


def run_spect_ff(scene, spect, n_per_run, seed, first=0, threads=1, precision=32):
    """Oracle SPECT run with free flight outside the heads (spect.free_flight):
    (weighted projection, its history-by-history squares, counters), projection layout."""
    L = lib(precision)
    fn = getattr(L, f"ggo{precision}_run_spect_ff")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(C.TablesDesc), ctypes.POINTER(C.VolumeDesc), ctypes.POINTER(C.WorldDesc),
                   ctypes.POINTER(C.SourceDesc), ctypes.POINTER(C.SpectDesc), ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(C.FfDesc), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                   ctypes.POINTER(ctypes.c_uint64)]
    shape = spect.projection_shape()
    n = int(np.prod(shape))
    wproj = np.zeros(n, dtype=np.uint64)
    wproj2 = np.zeros(2 * n, dtype=np.uint64)
    proj = np.zeros(n, dtype=np.uint64)
    cnt = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
    desc = spect.desc()
    frames = spect.all_frames()
    st = _with_blur(L, precision, spect, lambda: fn(
        *_descs(scene), ctypes.byref(desc), C.ptr(frames, ctypes.c_double), ctypes.byref(spect.free_flight), seed,
        first, n_per_run, threads, C.ptr(wproj, ctypes.c_uint64), C.ptr(wproj2, ctypes.c_uint64),
        C.ptr(proj, ctypes.c_uint64), C.ptr(cnt, ctypes.c_uint64)))
    if st != 0:
        raise RuntimeError(f"oracle SPECT free-flight run failed with status {st}")
    w = wproj.astype(np.float64) * 2.0 ** -32
    w2 = wproj2[1::2].astype(np.float64) * 2.0 ** -32 + wproj2[0::2].astype(np.float64) * 2.0 ** -64
    return w.reshape(shape), w2.reshape(shape), {name: int(cnt[i]) for i, name in enumerate(C.COUNTER_NAMES)}


def find_hole(spect, a1, a2, precision=32):
    L = lib(precision)
    f = getattr(L, f"ggo{precision}_find_hole")
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(C.SpectDesc), ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                  ctypes.POINTER(ctypes.c_double)]
    cx, cy = ctypes.c_double(), ctypes.c_double()
    d = spect.desc()
    inside = f(ctypes.byref(d), float(a1), float(a2), ctypes.byref(cx), ctypes.byref(cy))
    return bool(inside), cx.value, cy.value


def hex_exit(spect, qx, qy, d1, d2, precision=32):
    L = lib(precision)
    f = getattr(L, f"ggo{precision}_hex_exit")
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.POINTER(C.SpectDesc)] + [ctypes.c_double] * 4
    d = spect.desc()
    return f(ctypes.byref(d), float(qx), float(qy), float(d1), float(d2))


def arf_dataset(tables_desc, spect, sampling, n, seed, first=0, threads=8, precision=32):
    """Oracle ARF training rows: (rows [m][4] float32 = E, theta, phi, window, counters)."""
    L = lib(precision)
    fn = getattr(L, f"ggo{precision}_arf_dataset")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(C.TablesDesc), ctypes.POINTER(C.SpectDesc), ctypes.POINTER(C.ArfSampling),
                   ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                   ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    rows = np.zeros((max(n, 1), 4), dtype=np.float32)
    m = ctypes.c_uint64()
    cnt = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
    desc = spect.desc()
    st = _with_blur(L, precision, spect, lambda: fn(
        ctypes.byref(tables_desc), ctypes.byref(desc), ctypes.byref(sampling), seed, first, n, threads,
        C.ptr(rows, ctypes.c_float), ctypes.byref(m), C.ptr(cnt, ctypes.c_uint64)))
    if st != 0:
        raise RuntimeError(f"oracle ARF dataset failed with status {st}")
    return rows[: m.value].copy(), {name: int(cnt[i]) for i, name in enumerate(C.COUNTER_NAMES)}


def run_spect_arf(scene, spect, n_per_run, seed, model, params, first=0, threads=1, precision=32):
    """Oracle SPECT run with ARF detectors: (counts, arf_counts, arf_squared, counters), projection layout."""
    L = lib(precision)
    fn = getattr(L, f"ggo{precision}_run_spect_arf")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(C.TablesDesc), ctypes.POINTER(C.VolumeDesc), ctypes.POINTER(C.WorldDesc),
                   ctypes.POINTER(C.SourceDesc), ctypes.POINTER(C.SpectDesc), ctypes.POINTER(ctypes.c_double),
                   ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(C.ArfModel),
                   ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    shape = spect.projection_shape()
    n = int(np.prod(shape))
    proj = np.zeros(n, dtype=np.uint64)
    aproj = np.zeros(n, dtype=np.uint64)
    aproj2 = np.zeros(2 * n, dtype=np.uint64)
    cnt = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
    desc = spect.desc()
    frames = spect.all_frames()
    params = np.ascontiguousarray(params, dtype=np.float32)
    st = _with_blur(L, precision, spect, lambda: fn(
        *_descs(scene), ctypes.byref(desc), C.ptr(frames, ctypes.c_double), seed, first, n_per_run, threads,
        C.ptr(proj, ctypes.c_uint64), C.ptr(cnt, ctypes.c_uint64), ctypes.byref(model),
        C.ptr(params, ctypes.c_float), C.ptr(aproj, ctypes.c_uint64), C.ptr(aproj2, ctypes.c_uint64)))
    if st != 0:
        raise RuntimeError(f"oracle SPECT ARF run failed with status {st}")
    arf = aproj.astype(np.float64) * 2.0 ** -32
    arf2 = aproj2[1::2].astype(np.float64) * 2.0 ** -32 + aproj2[0::2].astype(np.float64) * 2.0 ** -64
    return (proj.astype(np.float64).reshape(shape), arf.reshape(shape), arf2.reshape(shape),
            {name: int(cnt[i]) for i, name in enumerate(C.COUNTER_NAMES)})


def run_spect_arf_ff(scene, spect, n_per_run, seed, model, params, first=0, threads=1, precision=32):
    """Oracle SPECT run with ARF detectors and free flight (spect.free_flight): (tracked counts,
    weighted projection of network weights x free-flight weights + weighted fallback singles,
    its history-by-history squares, counters), projection layout."""
    L = lib(precision)
    fn = getattr(L, f"ggo{precision}_run_spect_arf_ff")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(C.TablesDesc), ctypes.POINTER(C.VolumeDesc), ctypes.POINTER(C.WorldDesc),
                   ctypes.POINTER(C.SourceDesc), ctypes.POINTER(C.SpectDesc), ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(C.FfDesc), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(C.ArfModel),
                   ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    shape = spect.projection_shape()
    n = int(np.prod(shape))
    proj = np.zeros(n, dtype=np.uint64)
    aproj = np.zeros(n, dtype=np.uint64)
    aproj2 = np.zeros(2 * n, dtype=np.uint64)
    cnt = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
    desc = spect.desc()
    frames = spect.all_frames()
    params = np.ascontiguousarray(params, dtype=np.float32)
    st = _with_blur(L, precision, spect, lambda: fn(
        *_descs(scene), ctypes.byref(desc), C.ptr(frames, ctypes.c_double), ctypes.byref(spect.free_flight), seed,
        first, n_per_run, threads, C.ptr(proj, ctypes.c_uint64), C.ptr(cnt, ctypes.c_uint64), ctypes.byref(model),
        C.ptr(params, ctypes.c_float), C.ptr(aproj, ctypes.c_uint64), C.ptr(aproj2, ctypes.c_uint64)))
    if st != 0:
        raise RuntimeError(f"oracle SPECT ARF + free-flight run failed with status {st}")
    w = aproj.astype(np.float64) * 2.0 ** -32
    w2 = aproj2[1::2].astype(np.float64) * 2.0 ** -32 + aproj2[0::2].astype(np.float64) * 2.0 ** -64
    return (proj.astype(np.float64).reshape(shape), w.reshape(shape), w2.reshape(shape),
            {name: int(cnt[i]) for i, name in enumerate(C.COUNTER_NAMES)})
