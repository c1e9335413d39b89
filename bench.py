"""Benchmark: primaries/s of voxelised photon transport with DoseActor scoring.

Workload (one step): the heterogeneous CT phantom - 256 x 256 x 160 int16 HU
image, 1.2 mm voxels, ten-interval HU table, point source at 100 cm SSD with a
10 x 10 cm field and a 60-bin E*exp(-E/1.5 MeV) spectrum on [0.1, 6] MeV -
1e8 primaries per step, FP32 transport, FP64 edep and edep-squared images
(history-by-history).  Inputs are synthetic and seeded.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  ``value`` is device-timed (CUDA events on
the launching stream, inputs resident); ``e2e`` goes through the C ABI with
host buffers (scene upload and image download inside the timed region).
``--impl reference`` times the CPU restatement of the path (the reference's
Geant4 stack cannot be installed here) on all host cores.
"""

import argparse
import copy
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "primaries/s at matched sigma (plain GPU transport, CT phantom dose)"
UNIT = "primaries/s"
PRIMARIES_PER_STEP = 100_000_000
TRANSPORT_DRAM_PER_PRIMARY = (478.16e6 + 200.48e6) / 3e6  # bytes, ncu capture of the dose workload
WORKLOAD = "ct_phantom_256x256x160_1.2mm_ssd100_field10x10_spectrum60_0.1-6MeV"

# SPECT acquisition: CT phantom as attenuation map, Tc-99m activity image,
# two LEHR heads at 25 cm, 60 gantry positions, 1e9 decays (0.89 photons each)
SPECT_METRIC = "primaries/s at matched sigma (plain GPU collimator tracking, SPECT projections)"
SPECT_DECAYS = 1_000_000_000
SPECT_YIELD = 0.89
SPECT_WORKLOAD = ("spect_tc99m_lehr_2heads_60angles_r250mm_128x128x4.42mm_windows126-154_108-126keV_"
                  "ct_phantom_256x256x160_1.2mm")

# Batched uneven simulations: 48 seeded slab phantoms (32-128 voxels, 1-3 mm),
# mono disc beams 50 keV-2 MeV, 1e5-1e7 primaries each, one set of launches per
# step (CUDA-graph replay, autotuned launch configuration)
BATCH_METRIC = "primaries/s at matched sigma (batched GPU: 48 uneven simulations in one launch sequence)"
BATCH_WORKLOAD = "batched_48_slab_phantoms_32-128vox_1-3mm_mono_0.05-2MeV_1e5-1e7_primaries"

# SPECT with ARF detectors: Lu-177 (113 keV 6.2 %, 208 keV 10.4 %), medium-energy
# collimator, 120 gantry positions, 1e10 decays; the network is trained on
# 2e8 photons of the plain collimator tracking, and the plain acquisition of
# the same decays is run beside it for the matched-sigma comparison
FF_METRIC = ("primaries/s (free-flight SPECT recipe: primary free-flight pass + scatter-splitting pass, "
             "SPECT projections)")
FF_DECAYS = 100_000_000
FF_SPLIT = (50, 10, 10000, 10.0)  # Compton, Rayleigh factors, max Compton level, angle tolerance (deg)
FF_CHUNKS = 8  # scatter pass in independent chunks: its variance (copies of a history are correlated)
FF_WORKLOAD = SPECT_WORKLOAD + "_freeflight_primary+scattersplit_c50_r10_aa10deg"
ARF_METRIC = "primaries/s at matched sigma (ARF GPU vs plain GPU collimator tracking, SPECT projections)"
ARF_DECAYS = 10_000_000_000
ARF_YIELD = 0.166
ARF_WINDOWS = ((0.1872, 0.2288), (0.166, 0.187), (0.1017, 0.1243))
ARF_TRAIN_SAMPLES = 200_000_000
ARF_WORKLOAD = ("spect_lu177_melp_2heads_120angles_r250mm_128x128x4.42mm_windows187-229_166-187_101-125keV_"
                "ct_phantom_256x256x160_1.2mm_arf_mlp3x128_bf16")


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                     "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5).stdout
                for line in out.strip().splitlines():
                    self.rows.append([x.strip() for x in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._th:
            self._th.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for name, v in zip(names, r[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws, use_cuda):
    if ws <= 1:
        return None
    import torch.distributed as dist

    dist.init_process_group("nccl" if use_cuda else "gloo")
    return dist


def dist_max(dist, value, use_cuda):
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device="cuda" if use_cuda else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def mean_relative_uncertainty(edep, edep2, n, frac=0.1):
    """Mean history-by-history relative sigma over voxels above frac * max edep."""
    mean = edep / n
    var = np.clip((edep2 / n - mean * mean) / (n - 1), 0, None)
    sel = edep > frac * edep.max()
    rel = np.sqrt(var[sel]) / mean[sel]
    return float(rel.mean()) if sel.any() else None


def cpu_sample(scene, threads, target_s=10.0, seed=424242):
    """Times the CPU restatement of the path on a bounded sample."""
    from oracle import oracle as O

    # each oracle call has a fixed cost (table conversion, tally allocation and
    # the final image flush); grow the sample until it dominates, then size the
    # timed sample from the marginal rate
    n = 200_000
    t_prev, n_prev = None, None
    while True:
        t0 = time.perf_counter()
        O.run_dose(scene, n, seed, threads=threads)
        dt = time.perf_counter() - t0
        if dt > 0.25 * target_s or n >= 5e7:
            break
        t_prev, n_prev = dt, n
        n *= 4
    rate = (n - n_prev) / max(dt - t_prev, 1e-6) if n_prev else n / dt
    n2 = int(min(max(n, rate * target_s), 4e8))
    t0 = time.perf_counter()
    O.run_dose(scene, n2, seed + 1, threads=threads)
    dt2 = time.perf_counter() - t0
    return n2 / dt2, n2, dt2


def spect_cpu_sample(scene, sp, threads, target_s=10.0, seed=424242):
    """Times the CPU restatement of the SPECT path on a bounded sample (all 60 positions)."""
    from oracle import oracle as O

    n_runs = sp.n_runs
    n = 2000
    t_prev, n_prev = None, None
    while True:
        t0 = time.perf_counter()
        O.run_spect(scene, sp, n, seed, threads=threads)
        dt = time.perf_counter() - t0
        if dt > 0.25 * target_s or n * n_runs >= 5e7:
            break
        t_prev, n_prev = dt, n
        n *= 4
    rate = (n - n_prev) * n_runs / max(dt - t_prev, 1e-6) if n_prev else n * n_runs / dt
    n2 = int(min(max(n, rate * target_s / n_runs), 4e8 / n_runs))
    t0 = time.perf_counter()
    O.run_spect(scene, sp, n2, seed + 1, threads=threads)
    dt2 = time.perf_counter() - t0
    return n2 * n_runs / dt2, n2 * n_runs, dt2


def grow_sample(run, target_s, n0, n_max):
    """Times run(n, seed) (the CPU restatement) on a bounded sample: grows n until
    a call takes a quarter of target_s (each call has a fixed set-up cost), then
    runs the size the marginal rate gives for target_s.  Returns (n / s, n, s)."""
    n, t_prev, n_prev = n0, None, None
    while True:
        t0 = time.perf_counter()
        run(n, 424242)
        dt = time.perf_counter() - t0
        if dt > 0.25 * target_s or n >= n_max:
            break
        t_prev, n_prev = dt, n
        n *= 4
    rate = (n - n_prev) / max(dt - t_prev, 1e-6) if n_prev else n / dt
    n2 = int(min(max(n, rate * target_s), n_max))
    t0 = time.perf_counter()
    run(n2, 424243)
    dt2 = time.perf_counter() - t0
    return n2 / dt2, n2, dt2


def reference_workload(args, threads):
    """(metric, workload, data, primaries per step, run(n, seed) in primaries, note) of
    the CPU restatement for the chosen workload, on the same configuration as --impl ours."""
    from oracle import oracle as O
    from opengate_gb300 import workloads as W

    if args.workload in ("spect", "spect_arf"):
        from opengate_gb300 import spect as S

        if args.workload == "spect":
            scene, sp, _ = W.spect_phantom()
            meta = (SPECT_METRIC, SPECT_WORKLOAD, int(SPECT_DECAYS * SPECT_YIELD))
        else:
            scene, sp, _ = W.spect_phantom(nuclide=W.LU177, collimator=S.MELP, n_runs=120, windows=ARF_WINDOWS)
            meta = (ARF_METRIC, ARF_WORKLOAD, int(ARF_DECAYS * ARF_YIELD))
        runs = sp.n_runs

        def run(n, seed):
            O.run_spect(scene, sp, max(n // runs, 1), seed, threads=threads)

        note = (f"plain collimator tracking over all {runs} positions" +
                (" (the reference's CPU method; the network is not part of its CPU path)"
                 if args.workload == "spect_arf" else ""))
        return meta + ("synthetic (seeded CT phantom + activity image)", run, note, 2000 * runs, int(4e8))
    if args.workload == "spect_ff":
        scene, sp_p, sp_s = spect_ff_specs()
        runs = sp_p.n_runs

        def run(n, seed):
            O.run_spect_ff(scene, sp_p, max(n // runs, 1), seed, threads=threads)
            O.run_spect_ff(scene, sp_s, max(n // runs, 1), seed + 1, threads=threads)

        return (FF_METRIC, FF_WORKLOAD, int(FF_DECAYS * SPECT_YIELD), "synthetic (seeded CT phantom + activity image)",
                run, f"primary free flight + scatter splitting over all {runs} positions", 200 * runs, int(4e8))
    if args.workload == "batched":
        _, sims = W.batched_phantoms(seed=args.seed)
        total = int(sum(k for _, k, _ in sims))

        def run(n, seed):
            # the same fraction of every simulation's primaries
            f = n / total
            for sc, k, sd in sims:
                O.run_dose(sc, max(int(k * f), 1), sd + seed, threads=threads)

        return (BATCH_METRIC, BATCH_WORKLOAD, total, "synthetic (seeded slab phantoms)", run,
                "every simulation, the same fraction of its primaries", 100_000, total)
    if args.workload == "tle":
        scene = W.water_pencil()
        tle = scene.tle_desc(np.inf, 0.0, "EPDL")

        def run(n, seed):
            O.run_dose(scene, n, seed, threads=threads, tle=tle)

        return ("primaries/s at matched sigma (TLE dose vs analog dose, 64^3 water, 1 MeV pencil)",
                "water_64x64x64_2mm_pencil_1MeV_tle_none_epdl", 10_000_000, "synthetic (uniform water phantom)",
                run, "track-length estimator", 50_000, int(2e8))
    scene, _ = W.ct_phantom()

    def run(n, seed):
        O.run_dose(scene, n, seed, threads=threads)

    return (METRIC, WORKLOAD, PRIMARIES_PER_STEP, "synthetic (seeded CT phantom)", run, "analog DoseActor",
            200_000, int(4e8))


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    metric, workload, n_step, data, run, note, n0, n_max = reference_workload(args, threads)
    t_all = time.perf_counter()
    for _ in range(args.warmup):
        grow_sample(run, 1.0, n0, n_max)
    rates, samples = [], []
    for _ in range(args.steps):
        r, n, dt = grow_sample(run, 8.0, n0, n_max)
        rates.append(r)
        samples.append(n)
    value = float(np.median(rates))
    line = {
        "impl": "reference", "metric": metric, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": n_step / value * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": data,
        "config": {"workload": workload, "primaries_per_step": n_step,
                   "note": f"CPU restatement of the path (C, pthreads), {note}; "
                           "Geant4/opengate_core not installable offline"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{int(np.median(samples))} primaries of the same workload per step, "
                                   f"{threads} host threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t_all,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours_spect(args, ws, rank, local, dist, use_cuda):
    import torch

    from opengate_gb300 import spect as S
    from opengate_gb300 import workloads as W
    from opengate_gb300.engine import SpectEngine

    scene, sp, _ = W.spect_phantom()
    n_step = args.primaries if args.primaries != PRIMARIES_PER_STEP else int(SPECT_DECAYS * SPECT_YIELD)
    n_per_run = n_step // sp.n_runs
    n = n_per_run * sp.n_runs
    eng = SpectEngine(scene, sp, device=local, precision=32, batch=args.batch)
    l2_flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    def first_of(step):
        return ((rank * (args.warmup + args.steps + 4)) + step) * n

    for w in range(args.warmup):
        eng.reset()
        eng.run(n_per_run, args.seed, first_of(w))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    dev_ms, launches = [], 0
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            l2_flush.zero_()
            torch.cuda.synchronize()
            eng.reset()
            eng.run(n_per_run, args.seed, first_of(args.warmup + k))
            tg, tt, tf, nl = eng.last_kernel_ms()
            dev_ms.append(tg + tt + tf)
            launches += nl
            if k == args.steps - 1:
                counters = eng.counters()
                transport_ms = tt
                stage_ms = {"generate": tg, "transport": tt, "flush": tf}
                ph_ms, hd_ms, _ = eng.last_stage_ms()
                stage_ms.update({"phantom_stage": ph_ms, "head_stage": hd_ms})
                launches_last = nl
        torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    total_ms = dist_max(dist, float(np.sum(dev_ms)), use_cuda)
    value = ws * n * args.steps / (total_ms / 1e3)
    proj = eng.projection()
    peak = proj[:, 0::sp.n_windows]  # photopeak window of every head and position
    sigma = S.mean_relative_uncertainty(peak, peak, n)  # one count per event: squared counts == counts

    # e2e through the C ABI with host buffers: scene + heads upload, all positions, projection download
    h2d = scene.labels.nbytes + scene._sig.nbytes + scene._cum.nbytes + scene._ray_amax.nbytes + \
        scene._ray_cum.nbytes + scene.majorant.nbytes + scene.source_desc_bytes() + sp.all_frames().nbytes
    d2h = int(np.prod(sp.projection_shape())) * 8
    out_p = eng.pinned_empty(sp.projection_shape())  # page-locked, reused every step
    torch.cuda.synchronize()
    e2e_t = []
    for k in range(max(1, min(args.steps, 3))):
        t1 = time.perf_counter()
        eng.upload()
        eng.run(n_per_run, args.seed, first_of(args.warmup + args.steps + k))
        eng.projection(out_p)
        e2e_t.append(time.perf_counter() - t1)
    e2e_s = dist_max(dist, float(np.mean(e2e_t)), use_cuda)

    peak_bw, peak_kind = measured_peaks()
    # dominant kernel: the phantom stage (label gathers of its Woodcock steps)
    bytes_alg = 32.0 * counters["woodcock_steps"]
    achieved = bytes_alg / (stage_ms["phantom_stage"] / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak_bw, "unit": "GB/s",
                "frac": achieved / peak_bw, "traffic": args.traffic, "peak_kind": peak_kind,
                "kernel": "k_spect_phantom<float> (phantom stage)",
                "bytes_alg_per_step": bytes_alg,
                "units": {"woodcock_steps": counters["woodcock_steps"], "head_steps": counters["head_steps"],
                          "singles": counters["singles"], "launches_per_step": launches_last},
                "stage_ms_per_step": stage_ms}
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        r, ns, dt = spect_cpu_sample(scene, sp, threads, target_s=args.cpu_seconds)
        cpu = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{ns} primaries over the 60 positions, {dt:.1f} s on {threads} host threads"}
    fp64 = None
    if rank == 0 and args.fp64_primaries > 0:
        fp64 = spect_fp64_error(scene, sp, max(1, args.fp64_primaries // sp.n_runs), args.seed, local, args.batch)
    if rank == 0:
        line = {
            "metric": SPECT_METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded CT phantom + activity image)",
            "config": {"workload": SPECT_WORKLOAD, "primaries_per_step": n, "decays_per_step": n / SPECT_YIELD,
                       "l2": "flushed between steps (256 MiB write)", "batch": args.batch,
                       "parallelism": f"replicas x{ws}, disjoint history ranges"},
            "sigma": {"mean_relative_uncertainty_peak_window_gt10pct_max": sigma, "primaries": n,
                      "counts_peak_window": float(peak.sum())},
            "fp64_error": fp64,
            "e2e": {"value": ws * n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
            "wall_s": wall,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()
    return 0


def spect_ff_specs():
    """(scene, primary free-flight spec, scatter-splitting spec) of the SPECT workload."""
    from opengate_gb300 import workloads as W

    scene, sp_p, _ = W.spect_phantom()
    sp_s = copy.deepcopy(sp_p)
    sp_p.set_free_flight()
    nc, nr, lvl, deg = FF_SPLIT
    sp_s.set_scatter_splitting(nc, nr, lvl, angle_tolerance_max=math.radians(deg))
    return scene, sp_p, sp_s


def run_ours_ff(args, ws, rank, local, dist, use_cuda):
    """The reference's free-flight SPECT recipe (contrib/spect/spect_config.py:937-1000): a
    primary pass (GammaFreeFlightActor) and a scatter pass (ScatterSplittingFreeFlightActor),
    whose weighted projections add up to the acquisition.  value: primaries/s of both passes
    on the same primaries; sigma: efficiency (1 / sigma^2 T) against the analog SPECT path."""
    import torch

    from opengate_gb300.engine import SpectEngine

    scene, sp_p, sp_s = spect_ff_specs()
    runs = sp_p.n_runs
    n_step = args.primaries if args.primaries != PRIMARIES_PER_STEP else int(FF_DECAYS * SPECT_YIELD)
    n_per_run = n_step // runs // FF_CHUNKS * FF_CHUNKS
    n = n_per_run * runs
    m = n_per_run // FF_CHUNKS
    eng_p = SpectEngine(scene, sp_p, device=local, precision=32, batch=args.batch)
    eng_s = SpectEngine(scene, sp_s, device=local, precision=32, batch=args.batch)
    l2_flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    def first_of(step):
        return ((rank * (args.warmup + args.steps + 4)) + step) * n

    parts = {}

    def step(first, keep=False):
        """Both passes; device ms, launches, (primary w, w2, scatter chunk projections) if keep."""
        ms, nl, chunks = 0.0, 0, []
        eng_p.reset()
        eng_s.reset()
        eng_p.run(n_per_run, args.seed, first)
        tg, tt, tf, k = eng_p.last_kernel_ms()
        ms, nl = ms + tg + tt + tf, nl + k
        parts["primary_pass"] = tg + tt + tf
        parts["scatter_phantom_stage"] = parts["scatter_head_stage"] = parts["scatter_copies"] = 0.0
        prev = 0.0
        for c in range(FF_CHUNKS):
            eng_s.run(m, args.seed + 1, first + c * m * runs)  # run r of a call: first + r * m
            tg, tt, tf, k = eng_s.last_kernel_ms()
            ms, nl = ms + tg + tt + tf, nl + k
            ph, hd, cp = eng_s.last_stage_ms()
            parts["scatter_phantom_stage"] += ph
            parts["scatter_head_stage"] += hd
            parts["scatter_copies"] += cp
            if keep:
                cur = eng_s.weighted_projection()
                chunks.append(cur - prev)
                prev = cur
        return ms, nl, chunks

    for w in range(args.warmup):
        step(first_of(w))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    dev_ms, launches = [], 0
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            l2_flush.zero_()
            torch.cuda.synchronize()
            ms, nl, _ = step(first_of(args.warmup + k))
            dev_ms.append(ms)
            launches += nl
        torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    total_ms = dist_max(dist, float(np.sum(dev_ms)), use_cuda)
    value = ws * n * args.steps / (total_ms / 1e3)
    # statistics of one more step: primary pass (w2: one photon, one single) + scatter chunks
    ms_s, _, chunks = step(first_of(args.warmup + args.steps), keep=True)
    cnt_s = eng_s.counters()
    ph_ms = parts["scatter_phantom_stage"]
    wp, wp2 = eng_p.weighted_projection(squared=True)
    nw = sp_p.n_windows
    # per-projection window totals (head, position, window): a photon of the primary pass
    # scores one single; the scatter pass's variance comes from its independent chunks
    ch = np.array(chunks).sum(axis=(3, 4))
    t_ff = wp.sum(axis=(2, 3)) + ch.sum(axis=0)
    v_ff = wp2.sum(axis=(2, 3)) + FF_CHUNKS * ch.var(axis=0, ddof=1)
    # analog SPECT path, same primaries (one count per single: variance = counts)
    sp_a = copy.deepcopy(sp_p)
    sp_a.set_free_flight(enabled=False)
    with SpectEngine(scene, sp_a, device=local, precision=32, batch=args.batch) as eng_a:
        eng_a.run(n_per_run, args.seed + 2, first_of(args.warmup + args.steps + 1))
        tg, tt, tf, _ = eng_a.last_kernel_ms()
        ms_a = tg + tt + tf
        t_a = eng_a.projection().sum(axis=(2, 3))

    def rel(t, v, w):
        tw, vw = t[:, w::nw], v[:, w::nw]
        sel = tw > 0
        return float((np.sqrt(vw[sel]) / tw[sel]).mean())

    sig = {}
    for w in range(nw):
        s_ff, s_a = rel(t_ff, v_ff, w), rel(t_a, t_a, w)
        sig[f"window_{w}"] = {"free_flight": s_ff, "analog": s_a, "ratio_totals": float(t_ff[:, w::nw].sum() /
                                                                                         t_a[:, w::nw].sum()),
                              "efficiency_gain_vs_analog": (s_a ** 2 * ms_a) / (s_ff ** 2 * ms_s)}

    # e2e through the C ABI with host buffers: uploads, both passes, weighted projections down
    h2d = 2 * (scene.labels.nbytes + scene._sig.nbytes + scene._cum.nbytes + scene._ray_amax.nbytes +
               scene._ray_cum.nbytes + scene.majorant.nbytes + scene.source_desc_bytes() + sp_p.all_frames().nbytes)
    d2h = 2 * 3 * int(np.prod(sp_p.projection_shape())) * 8
    torch.cuda.synchronize()
    e2e_t = []
    for k in range(max(1, min(args.steps, 2))):
        t1 = time.perf_counter()
        eng_p.upload()
        eng_s.upload()
        first = first_of(args.warmup + args.steps + 2 + k)
        eng_p.run(n_per_run, args.seed, first)
        eng_s.run(n_per_run, args.seed + 1, first)
        eng_p.weighted_projection(squared=True)
        eng_s.weighted_projection(squared=True)
        e2e_t.append(time.perf_counter() - t1)
    e2e_s = dist_max(dist, float(np.mean(e2e_t)), use_cuda)

    peak_bw, peak_kind = measured_peaks()
    bytes_alg = 32.0 * cnt_s["woodcock_steps"]
    achieved = bytes_alg / (ph_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak_bw, "unit": "GB/s",
                "frac": achieved / peak_bw, "traffic": args.traffic, "peak_kind": peak_kind,
                "kernel": "k_spect_phantom<float, 2, scatter splitting> (scatter pass, phantom stage)",
                "bytes_alg_per_step": bytes_alg,
                "note": "label gathers of the analog Woodcock steps only; the copies' free flights "
                        "(voxel walks of exp(-optical depth)) are latency-bound gathers not counted",
                "units": dict(cnt_s), "ms_per_step": dict(parts)}
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        from oracle import oracle as O

        threads = os.cpu_count() or 1

        def run(nn, seed):
            O.run_spect_ff(scene, sp_p, max(nn // runs, 1), seed, threads=threads)
            O.run_spect_ff(scene, sp_s, max(nn // runs, 1), seed + 1, threads=threads)

        r, ns, dt = grow_sample(run, args.cpu_seconds, 200 * runs, int(4e8))
        cpu = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{ns} primaries through both passes over the {runs} positions, {dt:.1f} s on "
                         f"{threads} host threads"}
    fp64 = None
    if rank == 0 and args.fp64_primaries > 0:
        npr = max(1, min(args.fp64_primaries, 10_000_000) // runs)
        fp64 = {"primary_pass": spect_fp64_error(scene, sp_p, npr, args.seed, local, args.batch, weighted=True),
                "scatter_pass": spect_fp64_error(scene, sp_s, max(1, npr // 10), args.seed, local, args.batch,
                                                 weighted=True)}
    if rank == 0:
        line = {
            "metric": FF_METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded CT phantom + activity image)",
            "config": {"workload": FF_WORKLOAD, "primaries_per_step": n, "decays_per_step": n / SPECT_YIELD,
                       "split": {"compton": FF_SPLIT[0], "rayleigh": FF_SPLIT[1], "max_compton_level": FF_SPLIT[2],
                                 "angle_tolerance_deg": FF_SPLIT[3]},
                       "l2": "flushed between steps (256 MiB write)", "batch": args.batch,
                       "parallelism": f"replicas x{ws}, disjoint history ranges"},
            "sigma": {"mean_relative_uncertainty_of_projection_totals": sig, "analog_ms": ms_a,
                      "free_flight_ms": ms_s, "primaries": n,
                      "method": f"per (head, position) window totals; efficiency 1 / (sigma^2 T); primary "
                                f"pass: history-by-history squares; scatter pass: variance of {FF_CHUNKS} "
                                f"independent chunks; analog: Poisson"},
            "fp64_error": fp64,
            "e2e": {"value": ws * n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
            "wall_s": wall,
        }
        print(json.dumps(line), flush=True)
    eng_p.close()
    eng_s.close()
    if dist:
        dist.destroy_process_group()
    return 0


def projection_sigma(tot, tot2, n, n_win):
    """(per-pixel sigma of the peak window as for the plain bench, mean relative
    uncertainty of the per-projection window totals)."""
    from opengate_gb300 import spect as S

    pix = S.mean_relative_uncertainty(tot[:, 0::n_win], tot2[:, 0::n_win], n)
    # per projection (head, position, window): totals and history-by-history squares
    t = tot.sum(axis=(2, 3))
    t2 = tot2.sum(axis=(2, 3))  # a history adds to one pixel of a projection at most
    rel = S.compute_history_by_history_relative_uncertainty(t, t2, n)
    return pix, float(rel[t > 0].mean())


def run_ours_arf(args, ws, rank, local, dist, use_cuda):
    import torch

    from opengate_gb300 import spect as S
    from opengate_gb300 import workloads as W
    from opengate_gb300.engine import ArfNetwork, SpectEngine

    scene, sp, _ = W.spect_phantom(nuclide=W.LU177, collimator=S.MELP, n_runs=120, windows=ARF_WINDOWS)
    n_step = args.primaries if args.primaries != PRIMARIES_PER_STEP else int(ARF_DECAYS * ARF_YIELD)
    n_per_run = n_step // sp.n_runs
    n = n_per_run * sp.n_runs
    nw = sp.n_windows
    eng = SpectEngine(scene, sp, device=local, precision=32, batch=min(args.batch, 1 << 26))
    net = ArfNetwork(eng)
    # training (not timed): rows from the plain head transport, theta uniform to 85 degrees
    smp = ArfNetwork.sampling(min(lo for lo, _ in ARF_WINDOWS), 0.21, 85.0, (200.0, 200.0), 40.0)
    t0 = time.perf_counter()
    model, loss = net.train(smp, args.arf_train_samples, seed=args.seed + 7, epochs=args.arf_epochs, batch=8192,
                            lr=2e-3, lr_final=1e-5)
    train_s = time.perf_counter() - t0
    l2_flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    def first_of(step):
        return ((rank * (args.warmup + args.steps + 8)) + step) * n

    def acquire(arf, step):
        eng.use_arf(arf)
        l2_flush.zero_()
        torch.cuda.synchronize()
        eng.reset()
        eng.run(n_per_run, args.seed, first_of(step))
        tg, tt, tf, nl = eng.last_kernel_ms()
        return tg + tt + tf, nl

    for w in range(args.warmup):
        acquire(True, w)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    dev_ms, launches = [], 0
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            ms, nl = acquire(True, args.warmup + k)
            dev_ms.append(ms)
            launches += nl
        torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    total_ms = dist_max(dist, float(np.sum(dev_ms)), use_cuda)
    value = ws * n * args.steps / (total_ms / 1e3)
    counters = eng.counters()
    ph_ms, hd_ms, arf_ms = eng.last_stage_ms()
    a_counts, (a_w, a_w2) = eng.projection(), eng.arf_projection(squared=True)
    tot_a, tot2_a = a_counts + a_w, a_counts + a_w2
    stage_ms = dict(zip(("generate", "transport", "flush"), eng.last_kernel_ms()[:3]))
    stage_ms.update({"phantom_stage": ph_ms, "head_stage": hd_ms, "arf_stage": arf_ms})
    # the plain acquisition of the same histories (last timed step) for the matched-sigma comparison
    plain_ms, _ = acquire(False, args.warmup + args.steps - 1)
    tot_p = eng.projection()
    sig_a = projection_sigma(tot_a, tot2_a, n, nw)
    sig_p = projection_sigma(tot_p, tot_p, n, nw)
    t_a = total_ms / args.steps
    gain_pix = (sig_p[0] ** 2 * plain_ms) / (sig_a[0] ** 2 * t_a)
    gain_proj = (sig_p[1] ** 2 * plain_ms) / (sig_a[1] ** 2 * t_a)
    win_ratio = [float(tot_a[:, k::nw].sum() / max(tot_p[:, k::nw].sum(), 1e-30)) for k in range(nw)]

    # e2e through the C ABI with host buffers: scene + heads + network upload, acquisition, projections download
    params = net.params()
    h2d = scene.labels.nbytes + scene._sig.nbytes + scene._cum.nbytes + scene._ray_amax.nbytes + \
        scene._ray_cum.nbytes + scene.majorant.nbytes + scene.source_desc_bytes() + sp.all_frames().nbytes + \
        params.nbytes
    d2h = 3 * int(np.prod(sp.projection_shape())) * 8
    torch.cuda.synchronize()
    e2e_t = []
    for k in range(max(1, min(args.steps, 2))):
        t1 = time.perf_counter()
        eng.upload()
        net.set_model(model, params)
        eng.use_arf(True)
        eng.run(n_per_run, args.seed, first_of(args.warmup + args.steps + 1 + k))
        eng.projection()
        eng.arf_projection(squared=True)
        e2e_t.append(time.perf_counter() - t1)
    e2e_s = dist_max(dist, float(np.mean(e2e_t)), use_cuda)
    fp64 = None
    if rank == 0 and args.fp64_primaries > 0:
        fp64 = spect_fp64_error(scene, sp, max(1, args.fp64_primaries // sp.n_runs), args.seed, local,
                                min(args.batch, 1 << 26), arf=(model, params))
    # the network's arithmetic: forward FLOP per scored photon
    flop_photon = 2.0 * (3 * 128 + 2 * 128 * 128 + 128 * 16)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    if rank == 0:
        line = {
            "metric": ARF_METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 transport, bf16 network (f32 accumulate)",
            "data": "synthetic (seeded CT phantom + activity image)",
            "config": {"workload": ARF_WORKLOAD, "primaries_per_step": n, "decays_per_step": n / ARF_YIELD,
                       "l2": "flushed between steps (256 MiB write)", "training_samples": args.arf_train_samples,
                       "parallelism": f"replicas x{ws}, disjoint history ranges"},
            "matched_sigma": {
                "plain_primaries_per_s": n / (plain_ms / 1e3),
                "plain_equivalent_primaries_per_s_pixel": value * sig_p[0] ** 2 / sig_a[0] ** 2,
                "plain_equivalent_primaries_per_s_projection": value * sig_p[1] ** 2 / sig_a[1] ** 2,
                "sigma_pixel": {"arf": sig_a[0], "plain": sig_p[0]},
                "sigma_projection_total": {"arf": sig_a[1], "plain": sig_p[1]},
                "efficiency_gain_pixel": gain_pix, "efficiency_gain_projection": gain_proj,
                "window_counts_arf_over_plain": win_ratio,
                "note": "efficiency = 1 / (sigma^2 T), contrib/spect/spect_helpers.py:480-488, 582-591"},
            "training": {"seconds": train_s, "loss_first_last": [float(loss[0]), float(loss[-1])],
                         "epochs": args.arf_epochs},
            "fp64_error": fp64,
            "e2e": {"value": ws * n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "kernel": "k_spect_phantom<float> (phantom stage, dominant)",
                         "achieved": 32.0 * counters["woodcock_steps"] / (ph_ms / 1e3) / 1e9,
                         "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                         "frac": 32.0 * counters["woodcock_steps"] / (ph_ms / 1e3) / 1e9 / peaks.get("hbm_gbs", 1.0),
                         "traffic": args.traffic, "bytes_alg_per_step": 32.0 * counters["woodcock_steps"]},
            "roofline_network": {"bound": "tensor", "kernel": "k_spect_arf<float> (ARF stage, network layers)",
                                 "flop_per_scored_photon": flop_photon,
                                 "scored_photons_per_step": counters["arf_photons"],
                                 "achieved": flop_photon * counters["arf_photons"] / (arf_ms / 1e3) / 1e12,
                                 "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
                                 "frac": flop_photon * counters["arf_photons"] / (arf_ms / 1e3) / 1e12 /
                                 peaks.get("bf16_tflops", 1.0),
                                 "note": "tcgen05.mma kind::f16 (M 128, N 128 / 16, K 16) BF16, FP32 accumulate "
                                         "in TMEM; arf_stage_ms includes the "
                                         "queue classification and the projection atomics"},
            "units": {k: counters[k] for k in ("woodcock_steps", "head_steps", "arf_photons", "arf_fallback", "singles")},
            "stage_ms_per_step": stage_ms,
            "cpu_baseline": None,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
            "wall_s": wall,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()
    return 0


def run_ours_batched(args, ws, rank, local, dist, use_cuda):
    import torch

    from opengate_gb300 import _capi as C
    from opengate_gb300 import workloads as W
    from opengate_gb300.engine import BatchEngine, DoseEngine

    _, sims = W.batched_phantoms(seed=args.seed + rank)
    n = int(sum(k for _, k, _ in sims))
    eng = BatchEngine(sims, device=local, precision=32)
    t0 = time.perf_counter()
    best = eng.autotune()
    tune_s = time.perf_counter() - t0
    eng.capture()
    l2_flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    def step():
        l2_flush.zero_()
        torch.cuda.synchronize()
        eng.reset()
        eng.replay()
        return eng.last_kernel_ms()[1]

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    dev_ms = []
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            dev_ms.append(step())
        torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    total_ms = dist_max(dist, float(np.sum(dev_ms)), use_cuda)
    value = ws * n * args.steps / (total_ms / 1e3)
    counters = eng.counters()
    # the same simulations one after another on one context (gg_run each), for comparison
    seq_ms = 0.0
    seq = DoseEngine(sims[0][0], device=local, precision=32)
    for scene, k, seed in sims:
        seq.scene = scene
        seq.upload()
        seq.run(k, seed, 0)
        g, t, f, _ = seq.last_kernel_ms()
        seq_ms += g + t + f
    seq.close()
    # e2e through the C ABI: descriptors + labels upload, one run, all images download
    h2d = sum(s.labels.nbytes + s.majorant.nbytes for s, _, _ in sims) + sims[0][0]._sig.nbytes
    d2h = 2 * sum(s.n_voxels for s, _, _ in sims) * 8
    # images into page-locked host buffers reused every step (gg_host_alloc)
    outs = [(eng.pinned_empty(sc.labels.shape), eng.pinned_empty(sc.labels.shape)) for sc, _, _ in sims]
    e2e_t = []
    for _ in range(3):
        eng.reset()
        t1 = time.perf_counter()
        eng.upload()
        eng.run()
        for k in range(len(sims)):
            eng.image(k, C.GG_IMG_EDEP, outs[k][0])
            eng.image(k, C.GG_IMG_EDEP_SQUARED, outs[k][1])
        e2e_t.append(time.perf_counter() - t1)
    e2e_s = dist_max(dist, float(np.mean(e2e_t)), use_cuda)
    peak_bw, peak_kind = measured_peaks()
    # counters of the last step (the tally and counters are reset before each replay)
    bytes_alg = 32.0 * counters["woodcock_steps"] + 64.0 * counters["tally_entries"]
    achieved = bytes_alg / (total_ms / args.steps / 1e3) / 1e9
    if rank == 0:
        line = {
            "metric": BATCH_METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded slab phantoms)",
            "config": {"workload": BATCH_WORKLOAD, "simulations": len(sims), "primaries_per_step": n,
                       "voxels": int(sum(s.n_voxels for s, _, _ in sims)),
                       "l2": "flushed between steps (256 MiB write)",
                       "launch": "CUDA graph replay of the batch (source, transport, flush per batch)",
                       "autotuned": {"blocks_per_sm": best.blocks_per_sm, "refill_min": best.refill_min,
                                     "interact_min": best.interact_min, "seconds": tune_s},
                       "parallelism": f"replicas x{ws}, independent batches"},
            "sequential": {"primaries_per_s": n / (seq_ms / 1e3), "note": "gg_run per simulation, same context"},
            "e2e": {"value": ws * n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak_bw, "unit": "GB/s",
                         "frac": achieved / peak_bw, "traffic": args.traffic, "peak_kind": peak_kind,
                         "kernel": "k_transport<float, MULTI> (batched transport)",
                         "bytes_alg_per_step": bytes_alg, "note": "graph replay time includes source and flush"},
            "cpu_baseline": None,
            "clocks": clk.summary(),
            "gpu_launches": int(len(dev_ms) * 3 * max(1, -(-n // (1 << 24)))),
            "wall_s": wall,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()
    return 0


def fp64_error(scene, n, seed, device, batch, tle=None):
    """Dose images of n histories in the FP32 and the FP64 build of the same
    kernels (same seed, same histories) and the error of the first against the
    second (opengate_gb300.dose.precision_error), with both builds' rates.
    tle: (threshold, kill energy, database) of the track-length estimator."""
    import torch
    from opengate_gb300.dose import precision_error
    from opengate_gb300.engine import DoseEngine

    imgs, rate = {}, {}
    for prec in (32, 64):
        with DoseEngine(scene, device=device, precision=prec, batch=batch) as e:
            if tle is not None:
                e.set_tle(*tle)
            e.run(n, seed, 0)
            torch.cuda.synchronize()
            tg, tt, tf, _ = e.last_kernel_ms()
            rate[prec] = n / ((tg + tt + tf) / 1e3)
            imgs[prec] = (e.edep(), e.edep_squared())
    err = precision_error(imgs[32][0], imgs[32][1], imgs[64][0], imgs[64][1], n)
    err.update({"primaries": n, "seed": seed, "voxels_gt": "10 % of max",
                "rate_f32": rate[32], "rate_f64": rate[64]})
    return err


def spect_fp64_error(scene, sp, n_per_run, seed, device, batch, arf=None, weighted=False):
    """Projections of the same histories from the FP32 and the FP64 build of the SPECT
    kernels (same seed) and the error of the first against the second
    (opengate_gb300.dose.precision_error over pixels > 10 % of max, per-pixel sigma
    from the history-by-history squares): analog counts (squares = counts), free
    flight (weights and their squares) or ARF detectors (tracked counts + network
    weights; `arf` = (model, params))."""
    import torch

    from opengate_gb300.dose import precision_error
    from opengate_gb300.engine import ArfNetwork, SpectEngine

    imgs, rate = {}, {}
    n = n_per_run * sp.n_runs
    for prec in (32, 64):
        with SpectEngine(scene, sp, device=device, precision=prec, batch=batch) as e:
            if arf is not None:
                ArfNetwork(e).set_model(*arf)
                e.use_arf(True)
                e.reset()
            e.run(n_per_run, seed)
            torch.cuda.synchronize()
            tg, tt, tf, _ = e.last_kernel_ms()
            rate[prec] = n / ((tg + tt + tf) / 1e3)
            if weighted:
                imgs[prec] = e.weighted_projection(squared=True)
            elif arf is not None:
                c = e.projection()
                w, w2 = e.arf_projection(squared=True)
                imgs[prec] = (c + w, c + w2)
            else:
                c = e.projection()
                imgs[prec] = (c, c)
    err = precision_error(imgs[32][0], imgs[32][1], imgs[64][0], imgs[64][1], n)
    err.update({"primaries": n, "seed": seed, "pixels_gt": "10 % of max", "rate_f32": rate[32],
                "rate_f64": rate[64]})
    return err


def run_ours_tle(args, ws, rank, local, dist, use_cuda):
    """Track-length estimator (TLEDoseActor) against analog scoring at matched sigma:
    64^3 water, 2 mm voxels, 1 MeV pencil beam on the entrance face (the small dose
    configuration), TLE threshold type "None", EPDL mu_en."""
    import torch

    from opengate_gb300 import workloads as W
    from opengate_gb300.engine import DoseEngine

    scene = W.water_pencil()
    n = args.primaries if args.primaries != PRIMARIES_PER_STEP else 10_000_000
    l2_flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    def first_of(step):
        return ((rank * (args.warmup + args.steps + 1)) + step) * n

    def timed(eng, steps, base):
        ms, launches = [], 0
        for k in range(steps):
            l2_flush.zero_()
            torch.cuda.synchronize()
            eng.reset()
            eng.run(n, args.seed, first_of(base + k))
            tg, tt, tf, nl = eng.last_kernel_ms()
            ms.append(tg + tt + tf)
            launches += nl
        return ms, launches

    tle = DoseEngine(scene, device=local, precision=32, batch=args.batch)
    tle.set_tle(np.inf, 0.0, "EPDL")
    timed(tle, args.warmup, 0)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        ms, launches = timed(tle, args.steps, args.warmup)
        torch.cuda.synchronize()
    total_ms = dist_max(dist, float(np.sum(ms)), use_cuda)
    value = ws * n * args.steps / (total_ms / 1e3)
    sig_t = mean_relative_uncertainty(tle.edep(), tle.edep_squared(), n)
    counters = tle.counters()
    stage = tle.last_kernel_ms()
    # e2e through the C ABI with host buffers: scene upload + estimator table, run, images back
    h2d = scene.labels.nbytes + scene._sig.nbytes + scene._cum.nbytes + scene._ray_amax.nbytes + \
        scene._ray_cum.nbytes + scene.majorant.nbytes + scene.pt.n_comp * 512 * 4
    d2h = 2 * scene.n_voxels * 8
    e2e_t = []
    for k in range(max(1, min(args.steps, 3))):
        t1 = time.perf_counter()
        tle.upload()
        tle.set_tle(np.inf, 0.0, "EPDL")
        tle.run(n, args.seed, first_of(args.warmup + args.steps + k))
        tle.edep(), tle.edep_squared()
        e2e_t.append(time.perf_counter() - t1)
    e2e_value = ws * n / dist_max(dist, float(np.mean(e2e_t)), use_cuda)
    tle.close()
    # analog scoring of the same histories
    ana = DoseEngine(scene, device=local, precision=32, batch=args.batch)
    timed(ana, args.warmup, 0)
    ams, _ = timed(ana, args.steps, args.warmup)
    sig_a = mean_relative_uncertainty(ana.edep(), ana.edep_squared(), n)
    ana.close()
    fp64 = None
    if rank == 0 and args.fp64_primaries > 0:
        fp64 = fp64_error(scene, min(n, args.fp64_primaries), args.seed, local, args.batch, tle=(np.inf, 0.0, "EPDL"))
    t_t, t_a = float(np.sum(ms)) / args.steps, float(np.sum(ams)) / args.steps
    gain = (sig_a ** 2 * t_a) / (sig_t ** 2 * t_t)
    peak, peak_kind = measured_peaks()
    bytes_alg = 32.0 * counters["woodcock_steps"] + 64.0 * counters["tally_entries"]
    achieved = bytes_alg / (stage[1] / 1e3) / 1e9
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        from oracle import oracle as O

        threads = os.cpu_count() or 1
        ns = 200_000
        t1 = time.perf_counter()
        O.run_dose(scene, ns, args.seed, threads=threads, tle=scene.tle_desc(np.inf, 0.0, "EPDL"))
        dt = time.perf_counter() - t1
        ns = max(ns, int(ns * args.cpu_seconds / max(dt, 1e-3)))
        t1 = time.perf_counter()
        O.run_dose(scene, ns, args.seed + 1, threads=threads, tle=scene.tle_desc(np.inf, 0.0, "EPDL"))
        dt = time.perf_counter() - t1
        cpu = {"value": ns / dt, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{ns} primaries of the same workload with the estimator, {dt:.1f} s on {threads} threads"}
    if rank == 0:
        line = {
            "metric": "primaries/s at matched sigma (TLE dose vs analog dose, 64^3 water, 1 MeV pencil)",
            "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (uniform water phantom)",
            "config": {"workload": "water_64x64x64_2mm_pencil_1MeV_tle_none_epdl", "primaries_per_step": n,
                       "tally": "fp64 edep + edep^2, history-by-history", "l2": "flushed between steps (256 MiB write)",
                       "parallelism": f"replicas x{ws}, disjoint history ranges"},
            "matched_sigma": {"sigma_tle": sig_t, "sigma_analog": sig_a, "ms_per_step_tle": t_t,
                              "ms_per_step_analog": t_a, "efficiency_gain": gain,
                              "analog_equivalent_primaries_per_s": value * gain,
                              "note": "efficiency = 1 / (sigma^2 T), sigma = mean relative uncertainty "
                                      "over voxels > 10 % of max"},
            "fp64_error": fp64,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_kind": peak_kind, "kernel": "k_transport<float> (estimator)",
                         "bytes_alg_per_step": bytes_alg,
                         "units": {"woodcock_steps": counters["woodcock_steps"],
                                   "tally_entries": counters["tally_entries"], "deposits": counters["deposits"]},
                         "stage_ms_per_step": {"generate": stage[0], "transport": stage[1], "flush": stage[2]}},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_ours(args):
    ws, rank, local = dist_env()
    import torch

    use_cuda = torch.cuda.is_available()
    if not use_cuda:
        raise RuntimeError("bench.py needs a CUDA GPU for --impl ours")
    torch.cuda.set_device(local)
    dist = dist_init(ws, use_cuda)
    if args.workload == "spect":
        return run_ours_spect(args, ws, rank, local, dist, use_cuda)
    if args.workload == "spect_arf":
        return run_ours_arf(args, ws, rank, local, dist, use_cuda)
    if args.workload == "batched":
        return run_ours_batched(args, ws, rank, local, dist, use_cuda)
    if args.workload == "tle":
        return run_ours_tle(args, ws, rank, local, dist, use_cuda)
    if args.workload == "spect_ff":
        return run_ours_ff(args, ws, rank, local, dist, use_cuda)
    from opengate_gb300 import _capi as C
    from opengate_gb300 import workloads as W
    from opengate_gb300.engine import DoseEngine

    scene, _ = W.ct_phantom()
    n = args.primaries
    eng = DoseEngine(scene, device=local, precision=32, batch=args.batch)
    l2_flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")
    # history ranges are disjoint across ranks and steps
    def first_of(step):
        return ((rank * (args.warmup + args.steps + 1)) + step) * n

    for w in range(args.warmup):
        eng.reset()
        eng.run(n, args.seed, first_of(w))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    dev_ms = []
    launches = 0
    counters = None
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            l2_flush.zero_()
            torch.cuda.synchronize()
            eng.reset()
            eng.run(n, args.seed, first_of(args.warmup + k))
            tg, tt, tf, nl = eng.last_kernel_ms()
            dev_ms.append(tg + tt + tf)
            launches += nl
            if k == args.steps - 1:
                counters = eng.counters()
                transport_ms = tt
                transport_launches = nl // 3
                stage_ms = {"generate": tg, "transport": tt, "flush": tf}
        torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    total_ms = dist_max(dist, float(np.sum(dev_ms)), use_cuda)
    value = ws * n * args.steps / (total_ms / 1e3)

    # sigma reached by one step (mean relative uncertainty, voxels > 10 % max)
    edep, edep2 = eng.edep(), eng.edep_squared()
    sigma = mean_relative_uncertainty(edep, edep2, n)

    # e2e through the C ABI with host buffers: scene upload (H2D), run, image download (D2H)
    h2d = scene.labels.nbytes + scene._sig.nbytes + scene._cum.nbytes + scene._ray_amax.nbytes + \
        scene._ray_cum.nbytes + scene.majorant.nbytes
    d2h = 2 * scene.n_voxels * 8
    # the images land in page-locked host buffers reused every step (gg_host_alloc)
    out_e = eng.pinned_empty(scene.labels.shape)
    out_e2 = eng.pinned_empty(scene.labels.shape)
    torch.cuda.synchronize()
    e2e_t = []
    for k in range(max(1, min(args.steps, 3))):
        t1 = time.perf_counter()
        eng.upload()
        eng.run(n, args.seed, first_of(args.warmup + args.steps + k))
        eng.edep(out_e), eng.edep_squared(out_e2)
        e2e_t.append(time.perf_counter() - t1)
    e2e_s = dist_max(dist, float(np.mean(e2e_t)), use_cuda)
    e2e_value = ws * n / e2e_s

    # roofline of the transport kernel: algorithmic bytes per launch
    peak, peak_kind = measured_peaks()
    bytes_alg = 32.0 * counters["woodcock_steps"] + 64.0 * counters["tally_entries"]
    achieved = bytes_alg / (transport_ms / 1e3) / 1e9
    # DRAM traffic of the transport kernel: an ncu capture of the same workload at 3e6
    # primaries (one launch: dram__bytes_read.sum 478.16 MB + dram__bytes_write.sum
    # 200.48 MB) scaled by primaries to this launch, unless measured and passed in
    traffic = args.traffic if args.traffic is not None else TRANSPORT_DRAM_PER_PRIMARY * n
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "traffic_note": None if args.traffic is not None else
                "ncu dram bytes of a 3e6-primary launch of this workload, scaled by primaries",
                "peak_kind": peak_kind, "kernel": "k_transport<float>",
                "bytes_alg_per_step": bytes_alg,
                "units": {"woodcock_steps": counters["woodcock_steps"], "tally_entries": counters["tally_entries"],
                          "transport_launches_per_step": transport_launches},
                "stage_ms_per_step": stage_ms}

    # error of the FP32 transport against the FP64 build on the same random stream (untimed)
    fp64 = None
    if rank == 0 and args.fp64_primaries > 0:
        fp64 = fp64_error(scene, args.fp64_primaries, args.seed, local, args.batch)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        r, ns, dt = cpu_sample(scene, threads, target_s=args.cpu_seconds)
        cpu = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{ns} primaries of the same workload, {dt:.1f} s on {threads} host threads"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded CT phantom)",
            "config": {"workload": WORKLOAD, "primaries_per_step": n, "tally": "fp64 edep + edep^2, history-by-history",
                       "l2": "flushed between steps (256 MiB write)", "batch": args.batch,
                       "parallelism": f"replicas x{ws}, disjoint history ranges"},
            "sigma": {"mean_relative_uncertainty_gt10pct_max": sigma, "primaries": n},
            "fp64_error": fp64,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
            "wall_s": wall,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dose", choices=["dose", "spect", "spect_arf", "batched", "tle", "spect_ff"],
                    help="dose: CT phantom DoseActor (default); spect: Tc-99m SPECT acquisition, 60 positions; "
                         "spect_arf: Lu-177 SPECT with ARF detectors vs plain tracking, 120 positions; "
                         "batched: 48 uneven dose simulations in one launch sequence; "
                         "tle: track-length estimator vs analog dose, 64^3 water, 1 MeV pencil; "
                         "spect_ff: free-flight SPECT recipe (primary + scatter splitting) on the spect workload")
    ap.add_argument("--primaries", type=int, default=PRIMARIES_PER_STEP)
    ap.add_argument("--arf-train-samples", type=int, default=ARF_TRAIN_SAMPLES)
    ap.add_argument("--arf-epochs", type=int, default=80)
    ap.add_argument("--batch", type=int, default=1 << 27)
    ap.add_argument("--seed", type=int, default=20240611)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--fp64-primaries", type=int, default=10_000_000,
                    help="histories of the FP32-vs-FP64 comparison of the dose workload (0: skip)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per transport launch from an ncu capture (reported as-is)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
