"""GPU transport engine: one libgategpu context per simulation run.

This is the GB300 counterpart of the reference's SimulationEngine run phase
(opengate/engines.py:1554-1660): it pushes the scene to the device, runs the
requested histories in tally batches and fetches the float64 images, the way
DoseActor.EndOfRunActionMasterThread fetches them from C++
(opengate/actors/doseactors.py:662-715).
"""

import ctypes

import numpy as np

from . import _capi as C


class DoseEngine:
    """Drives libgategpu.so for one :class:`~opengate_gb300.scene.Scene`."""

    def __init__(self, scene, device=0, precision=32, block_size=0, blocks_per_sm=0, chunk=0, batch=0,
                 refill_min=0, interact_min=0, score_squared=True):
        self.lib = C.load()
        self.scene = scene
        opts = C.DeviceOpts(device, precision, block_size, blocks_per_sm, chunk, batch, refill_min, interact_min)
        ctx = ctypes.c_void_p()
        st = self.lib.gg_create(ctypes.byref(opts), ctypes.byref(ctx))
        C.check(self.lib, None, st)
        self.ctx = ctx
        self._pinned = []
        self.score_squared = score_squared
        self.upload()

    def _call(self, name, *args):
        C.check(self.lib, self.ctx, getattr(self.lib, name)(self.ctx, *args))

    def upload(self):
        s = self.scene
        self._call("gg_upload_tables", ctypes.byref(s.tables_desc))
        self._call("gg_upload_volume", ctypes.byref(s.volume_desc))
        self._call("gg_set_world", ctypes.byref(s.world_desc))
        self._call("gg_set_source", ctypes.byref(s.source_desc))
        self._call("gg_add_dose_tally", 1 if self.score_squared else 0)

    def set_source(self, source):
        """Switches to another source (tables, volume and tally are kept)."""
        self.scene.set_source(source)
        self._call("gg_set_source", ctypes.byref(self.scene.source_desc))

    def reset(self):
        self._call("gg_reset_tally")

    def set_transport_kernel(self, kind):
        """C.GG_KERNEL_PHASED (default) or C.GG_KERNEL_WAVEFRONT: same results, different speed."""
        self._call("gg_set_transport_kernel", int(kind))

    def set_tle(self, threshold_energy=float("inf"), energy_min=0.0, database="EPDL", enabled=True):
        """Track-length estimator of the dose tally (gg_set_tle); mu_en of the
        scene's compositions from ``database`` ("EPDL" or "NIST")."""
        if enabled:
            self._tle = self.scene.tle_desc(threshold_energy, energy_min, database)
        else:
            self._tle = C.TleDesc(0, 0.0, 0.0, None)
        self._call("gg_set_tle", ctypes.byref(self._tle))

    def run(self, n, seed, first=0):
        self._call("gg_run", ctypes.c_uint64(n), ctypes.c_uint64(seed), ctypes.c_uint64(first))

    def set_dose_grid(self, dims, spacing, corner, score_dose=True):
        """Dose tally on a grid of its own (gg_set_dose_grid): dims (nx, ny, nz), spacing and
        outer corner in mm (world); None: back to the image grid."""
        if dims is None:
            self._grid = None
            self._call("gg_set_dose_grid", None)
            return
        d = C.DoseGridDesc()
        d.dims[:] = [int(v) for v in dims]
        d.spacing[:] = [float(v) for v in spacing]
        d.corner[:] = [float(v) for v in corner]
        d.score_dose = 1 if score_dose else 0
        self._call("gg_set_dose_grid", ctypes.byref(d))
        self._grid = (int(dims[2]), int(dims[1]), int(dims[0]))

    def image_shape(self):
        """[nz][ny][nx] of the tally images: the dose grid's when set, else the image's."""
        return getattr(self, "_grid", None) or self.scene.labels.shape

    def image(self, which, out=None):
        """Image `which` [nz][ny][nx] (float64); into `out` when given (e.g. a pinned_empty
        buffer, reused between calls: the copy then runs at the link's DMA rate)."""
        shape = self.image_shape()
        n = int(np.prod(shape))
        if out is None:
            out = np.empty(shape, dtype=np.float64)
        if out.dtype != np.float64 or out.size != n or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of the image's size")
        self._call("gg_get_image", which, C.ptr(out, ctypes.c_double), out.size)
        return out.reshape(shape)

    def dose_sum(self):
        """Dose grid: sum of edep / rho per voxel (MeV cm3 / g), the DoseActor's dose before the
        division by the voxel volume."""
        return self.image(C.GG_IMG_DOSE)

    def dose_sum_squared(self):
        return self.image(C.GG_IMG_DOSE_SQUARED)

    def edep(self, out=None):
        return self.image(C.GG_IMG_EDEP, out)

    def edep_squared(self, out=None):
        return self.image(C.GG_IMG_EDEP_SQUARED, out)

    def image_device(self, which):
        """(device pointer, voxels) of an FP64 image on the context's device
        (gg_get_image_device): valid until the next run, reset or close."""
        ptr, n = ctypes.c_void_p(), ctypes.c_size_t()
        self._call("gg_get_image_device", int(which), ctypes.byref(ptr), ctypes.byref(n))
        return ptr.value, n.value

    def pinned_scene(self, scene):
        """A copy of `scene` whose label image lives in page-locked host memory owned by this
        engine (freed with it): uploads of it run at the host link's DMA rate."""
        import copy

        labels = self.pinned_empty(scene.labels.shape, np.uint16)
        labels[...] = scene.labels
        s = copy.copy(scene)
        s.labels = labels
        s._build_descs()
        return s

    def pinned_empty(self, shape, dtype=np.float64):
        """Uninitialised array in page-locked host memory (gg_host_alloc), freed with the
        engine."""
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        ptr = self.lib.gg_host_alloc(n)
        if not ptr:
            raise MemoryError(f"gg_host_alloc({n}) failed")
        self._pinned.append(ptr)
        buf = (ctypes.c_char * n).from_address(ptr)
        return np.frombuffer(buf, dtype=dtype).reshape(shape)

    def counters(self):
        out = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
        self._call("gg_get_counters", C.ptr(out, ctypes.c_uint64), out.size)
        return {name: int(out[i]) for i, name in enumerate(C.COUNTER_NAMES)}

    def last_kernel_ms(self):
        """(generate_ms, transport_ms, flush_ms, launches) of the last run."""
        g, t, f, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int32()
        self._call("gg_last_kernel_ms", ctypes.byref(g), ctypes.byref(t), ctypes.byref(f), ctypes.byref(n))
        return g.value, t.value, f.value, n.value

    def close(self):
        if self.ctx:
            self.lib.gg_destroy(self.ctx)
            self.ctx = None
        for ptr in getattr(self, "_pinned", []):
            self.lib.gg_host_free(ptr)
        self._pinned = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class SpectEngine(DoseEngine):
    """SPECT projections: heads + digitizer, one gg_run per gantry position.

    Mirrors a reference SPECT simulation with one run per angle
    (run_timing_intervals, contrib/spect/ge_discovery_nm670.py:1056-1080
    rotate_gantry): for run r the heads are placed with spect.frames(r) and
    n_per_run histories are simulated (history ids continue across runs).
    """

    def __init__(self, scene, spect, **kw):
        self.spect = spect
        super().__init__(scene, **kw)

    def upload(self):
        s = self.scene
        self._call("gg_upload_tables", ctypes.byref(s.tables_desc))
        self._call("gg_upload_volume", ctypes.byref(s.volume_desc))
        self._call("gg_set_world", ctypes.byref(s.world_desc))
        self._call("gg_set_source", ctypes.byref(s.source_desc))
        self._desc = self.spect.desc()
        self._call("gg_spect_setup", ctypes.byref(self._desc))
        self._call("gg_spect_set_blur", ctypes.byref(self.spect.blur))
        self._call("gg_spect_set_free_flight", ctypes.byref(self.spect.free_flight))

    def reset(self):
        self._call("gg_spect_setup", ctypes.byref(self._desc))
        self._call("gg_spect_set_blur", ctypes.byref(self.spect.blur))
        self._call("gg_spect_set_free_flight", ctypes.byref(self.spect.free_flight))

    def weighted_projection(self, squared=False):
        """Free-flight projection: summed single weights (and their history-by-history squares)."""
        return self.arf_projection(squared)

    def run(self, n_per_run, seed, first=0):
        """All gantry positions in one gg_spect_run call (one set of launches)."""
        frames = self.spect.all_frames()
        self._call("gg_spect_run", ctypes.c_uint64(n_per_run), ctypes.c_uint64(seed), ctypes.c_uint64(first),
                   C.ptr(frames, ctypes.c_double))
        self.kernel_ms = list(super().last_kernel_ms())

    def run_per_angle(self, n_per_run, seed, first=0):
        """Same histories as run(), one gg_spect_set_heads + gg_run per gantry position."""
        self.kernel_ms = [0.0, 0.0, 0.0, 0]
        for r in range(self.spect.n_runs):
            frames = np.ascontiguousarray(self.spect.frames(r), dtype=np.float64)
            self._call("gg_spect_set_heads", r, C.ptr(frames, ctypes.c_double))
            self._call("gg_run", ctypes.c_uint64(n_per_run), ctypes.c_uint64(seed),
                       ctypes.c_uint64(first + r * n_per_run))
            g, t, f, n = super().last_kernel_ms()
            self.kernel_ms = [self.kernel_ms[0] + g, self.kernel_ms[1] + t, self.kernel_ms[2] + f,
                              self.kernel_ms[3] + n]

    def last_kernel_ms(self):
        return tuple(self.kernel_ms)

    def last_stage_ms(self):
        """(phantom, head, ARF or scatter-splitting copies) stage device times of the last run, ms."""
        v = [ctypes.c_double() for _ in range(3)]
        self._call("gg_last_stage_ms", *(ctypes.byref(x) for x in v))
        return tuple(x.value for x in v)

    def use_arf(self, enable=True):
        """ARF detectors (a model must be set on the context, e.g. by ArfNetwork.train)."""
        self._call("gg_spect_use_arf", 1 if enable else 0)

    def arf_projection(self, squared=False):
        """ARF window weights (and their history-by-history squares) in the projection layout."""
        shape = self.spect.projection_shape()
        n = int(np.prod(shape))
        out = np.empty(n, dtype=np.float64)
        sq = np.empty(n, dtype=np.float64) if squared else None
        self._call("gg_get_arf_projection", C.ptr(out, ctypes.c_double), C.ptr(sq, ctypes.c_double), n)
        return (out.reshape(shape), sq.reshape(shape)) if squared else out.reshape(shape)

    def record_singles(self, capacity):
        """Keep the singles of the following runs in a device list of `capacity` records
        (0: off); see singles()."""
        self._call("gg_spect_record_singles", ctypes.c_uint64(int(capacity)))
        self._singles_cap = int(capacity)

    def singles(self):
        """The singles recorded since the last call (C.SINGLE_DTYPE records, completion order),
        then an empty list.  Raises if the list overflowed: its records would be a biased subset."""
        cap = getattr(self, "_singles_cap", 0)
        out = np.zeros(cap, dtype=C.SINGLE_DTYPE)
        n = ctypes.c_uint64()
        self._call("gg_spect_get_singles", out.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(cap),
                   ctypes.byref(n))
        if n.value > cap:
            raise RuntimeError(f"singles list overflow: {n.value} singles, capacity {cap} "
                               "(record_singles with a larger capacity)")
        return out[:n.value]

    def projection(self, out=None):
        """Counts (head, run * window, y, x); into `out` when given (e.g. pinned_empty)."""
        shape = self.spect.projection_shape()
        if out is None:
            out = np.empty(shape, dtype=np.float64)
        if out.dtype != np.float64 or out.size != int(np.prod(shape)) or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of the projection's size")
        self._call("gg_get_projection", C.ptr(out, ctypes.c_double), out.size)
        return out.reshape(shape)


class ArfNetwork:
    """ARF surrogate of a SPECT head on the context of a SpectEngine.

    Training rows come from the head transport (gg_arf_dataset); the network
    (3 -> 128 -> 128 -> 128 -> n_classes, BF16 tensor-core GEMMs) is trained
    on the GPU by gg_arf_train.  Mirrors the garf model the reference's
    ARFActor loads (opengate/actors/arfactors.py:299-331).
    """

    def __init__(self, engine):
        self.eng = engine
        self.model = None

    @staticmethod
    def sampling(e_min, e_max, theta_max_deg, half_extent, russian_roulette, theta_uniform=True):
        a = C.ArfSampling()
        a.theta_uniform = 1 if theta_uniform else 0
        a.e_min, a.e_max = float(e_min), float(e_max)
        a.cos_theta_max = float(np.cos(np.radians(theta_max_deg)))
        a.half_extent[:] = [float(half_extent[0]), float(half_extent[1])]
        a.russian_roulette = float(russian_roulette)
        return a

    def dataset(self, sampling, n, seed, first=0):
        rows = np.zeros((max(n, 1), 4), dtype=np.float32)
        m = ctypes.c_uint64()
        self.eng._call("gg_arf_dataset", ctypes.byref(sampling), ctypes.c_uint64(n), ctypes.c_uint64(seed),
                       ctypes.c_uint64(first), C.ptr(rows, ctypes.c_float), ctypes.c_uint64(n), ctypes.byref(m))
        return rows[: m.value].copy()

    def train(self, sampling, n_samples, seed, epochs=4, batch=8192, lr=1e-3, init_seed=1, beta1=0.9,
              beta2=0.999, eps=1e-8, lr_final=None):
        o = C.ArfTrainOpts()
        o.n_samples, o.seed, o.init_seed = int(n_samples), int(seed), int(init_seed)
        o.batch, o.epochs = int(batch), int(epochs)
        o.lr, o.beta1, o.beta2, o.eps = lr, beta1, beta2, eps
        o.lr_final = lr / 100.0 if lr_final is None else lr_final
        model = C.ArfModel()
        loss = np.zeros(epochs, dtype=np.float64)
        self.eng._call("gg_arf_train", ctypes.byref(sampling), ctypes.byref(o), ctypes.byref(model),
                       C.ptr(loss, ctypes.c_double))
        self.model = model
        return model, loss

    def train_rows(self, rows, e_min, e_max, theta_max_deg, russian_roulette, epochs=4, batch=8192, lr=1e-3,
                   init_seed=1, beta1=0.9, beta2=0.999, eps=1e-8, lr_final=None):
        """Trains on given rows [n][4] = (E MeV, theta deg, phi deg, class) (gg_arf_train_rows):
        the domain (energy range, largest theta, Russian roulette of class 0) sets the
        standardisation and the range where the network replaces tracking."""
        rows = np.ascontiguousarray(rows, dtype=np.float32).reshape(-1, 4)
        o = C.ArfTrainOpts()
        o.n_samples, o.seed, o.init_seed = len(rows), 0, int(init_seed)
        o.batch, o.epochs = int(batch), int(epochs)
        o.lr, o.beta1, o.beta2, o.eps = lr, beta1, beta2, eps
        o.lr_final = lr / 100.0 if lr_final is None else lr_final
        dom = C.ArfModel()
        dom.e_min, dom.e_max = float(e_min), float(e_max)
        dom.theta_max_deg, dom.russian_roulette = float(theta_max_deg), float(russian_roulette)
        model = C.ArfModel()
        loss = np.zeros(epochs, dtype=np.float64)
        self.eng._call("gg_arf_train_rows", C.ptr(rows, ctypes.c_float), ctypes.c_uint64(len(rows)),
                       ctypes.byref(dom), ctypes.byref(o), ctypes.byref(model), C.ptr(loss, ctypes.c_double))
        self.model = model
        return model, loss

    def set_model(self, model, params):
        params = np.ascontiguousarray(params, dtype=np.float32)
        if params.size != C.GG_ARF_N_PARAMS:
            raise ValueError(f"need {C.GG_ARF_N_PARAMS} parameters")
        self.eng._call("gg_arf_set_model", ctypes.byref(model), C.ptr(params, ctypes.c_float))
        self.model = model

    def params(self):
        out = np.zeros(C.GG_ARF_N_PARAMS, dtype=np.float32)
        self.eng._call("gg_arf_get_params", C.ptr(out, ctypes.c_float), out.size)
        return out

    def predict(self, rows):
        rows = np.ascontiguousarray(rows, dtype=np.float32)
        out = np.zeros((len(rows), self.model.n_classes), dtype=np.float32)
        self.eng._call("gg_arf_predict", C.ptr(rows, ctypes.c_float), ctypes.c_uint64(len(rows)),
                       C.ptr(out, ctypes.c_float))
        return out

    def gradient(self, rows):
        rows = np.ascontiguousarray(rows, dtype=np.float32)
        g = np.zeros(C.GG_ARF_N_PARAMS, dtype=np.float32)
        loss = ctypes.c_double()
        self.eng._call("gg_arf_gradient", C.ptr(rows, ctypes.c_float), ctypes.c_uint64(len(rows)),
                       C.ptr(g, ctypes.c_float), ctypes.byref(loss))
        return loss.value, g


class BatchEngine:
    """Many dose simulations in one set of launches (gg_batch_*): `sims` is a
    list of (Scene, n_primaries, seed) sharing one material table and world."""

    def __init__(self, sims, device=0, precision=32, batch=0, blocks_per_sm=0):
        self.lib = C.load()
        self.sims = sims
        opts = C.DeviceOpts(device, precision, 0, blocks_per_sm, 0, batch, 0, 0)
        ctx = ctypes.c_void_p()
        C.check(self.lib, None, self.lib.gg_create(ctypes.byref(opts), ctypes.byref(ctx)))
        self.ctx = ctx
        self._pinned = []
        self.upload()

    def _call(self, name, *args):
        C.check(self.lib, self.ctx, getattr(self.lib, name)(self.ctx, *args))

    def upload(self):
        first = self.sims[0][0]
        self._call("gg_upload_tables", ctypes.byref(first.tables_desc))
        self._call("gg_set_world", ctypes.byref(first.world_desc))
        arr = (C.SimDescC * len(self.sims))()
        for k, (scene, n, seed) in enumerate(self.sims):
            arr[k].volume = scene.volume_desc
            arr[k].source = scene.source_desc
            arr[k].n_primaries = int(n)
            arr[k].seed = int(seed)
        self._descs = arr  # the descriptors point into the scenes' arrays
        self._call("gg_batch_setup", arr, len(self.sims))

    @property
    def total_primaries(self):
        return int(sum(n for _, n, _ in self.sims))

    def run(self):
        self._call("gg_batch_run")

    def capture(self):
        self._call("gg_batch_capture")

    def replay(self):
        self._call("gg_batch_replay")

    def autotune(self):
        """Searches the launch configuration (gg_batch_autotune); returns the chosen options."""
        best = C.DeviceOpts()
        self._call("gg_batch_autotune", ctypes.byref(best))
        return best

    def autotune_result(self):
        """The last search: points timed, repeats per point, the winner's median / min / max
        device ms and the starting configuration's median."""
        r = C.AutotuneResult()
        self._call("gg_batch_autotune_result", ctypes.byref(r))
        return {k: getattr(r, k) for k, _ in r._fields_}

    def reset(self):
        self._call("gg_reset_tally")

    def image(self, k, which, out=None):
        """Image `which` of simulation k; into `out` when given (e.g. pinned_empty)."""
        scene = self.sims[k][0]
        if out is None:
            out = np.empty(scene.labels.shape, dtype=np.float64)
        if out.dtype != np.float64 or out.size != scene.n_voxels or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of the image's size")
        self._call("gg_batch_get_image", k, which, C.ptr(out, ctypes.c_double), out.size)
        return out.reshape(scene.labels.shape)

    pinned_empty = DoseEngine.pinned_empty
    pinned_scene = DoseEngine.pinned_scene

    def counters(self):
        out = np.zeros(C.GG_N_COUNTERS, dtype=np.uint64)
        self._call("gg_get_counters", C.ptr(out, ctypes.c_uint64), out.size)
        return {name: int(out[i]) for i, name in enumerate(C.COUNTER_NAMES)}

    def last_kernel_ms(self):
        g, t, f, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int32()
        self._call("gg_last_kernel_ms", ctypes.byref(g), ctypes.byref(t), ctypes.byref(f), ctypes.byref(n))
        return g.value, t.value, f.value, n.value

    def close(self):
        if self.ctx:
            self.lib.gg_destroy(self.ctx)
            self.ctx = None
        for ptr in getattr(self, "_pinned", []):
            self.lib.gg_host_free(ptr)
        self._pinned = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
