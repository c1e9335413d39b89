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
TRANSPORT_DRAM_PER_PRIMARY = (407.04e6 + 110.38e6) / 3e6  # bytes, ncu capture of the dose workload
# warp instructions per primary of the dose transport kernels and their active lanes per warp
# instruction (ncu captures of the same workload, 3e6 primaries: smsp__inst_executed.sum and
# smsp__thread_inst_executed_per_inst_executed.ratio; phase kernel, compacted wavefront kernel
# (the latter captured before the history lists moved to shared memory))
TRANSPORT_ISSUE = {"phased": (1.136376062e9 / 3e6, 8.60), "wavefront": (1.045618891e9 / 3e6, 14.12)}
WORKLOAD = "ct_phantom_256x256x160_1.2mm_ssd100_field10x10_spectrum60_0.1-6MeV"

# SPECT acquisition: CT phantom as attenuation map, Tc-99m activity image,
# two LEHR heads at 25 cm, 60 gantry positions, 1e9 decays (0.89 photons each)
SPECT_METRIC = "primaries/s at matched sigma (plain GPU collimator tracking, SPECT projections)"
SPECT_DECAYS = 1_000_000_000
SPECT_YIELD = 0.89
SPECT_HOUSING = "nm670"  # the NM670 shielding box: cover, reflector, back compartment, lead / steel, shielded sides
SPECT_WORKLOAD = ("spect_tc99m_lehr_nm670housing_2heads_60angles_r250mm_128x128x4.42mm_windows126-154_108-126keV_"
                  "ct_phantom_256x256x160_1.2mm")

# Batched uneven simulations: 48 seeded slab phantoms (32-128 voxels, 1-3 mm),
# mono disc beams 50 keV-2 MeV, 1e5-1e7 primaries each, one set of launches per
# step (CUDA-graph replay, autotuned launch configuration)
BATCH_METRIC = "primaries/s at matched sigma (batched GPU: 48 uneven simulations in one launch sequence)"
BATCH_WORKLOAD = "batched_48_slab_phantoms_32-128vox_1-3mm_mono_0.05-2MeV_1e5-1e7_primaries"

FF_METRIC = ("primaries/s (free-flight SPECT recipe: primary free-flight pass with forced directions + "
             "scatter-splitting pass on 1/4 of the primaries, SPECT projections)")
FF_DECAYS = 100_000_000
FF_SPLIT = (50, 10, 10000, 10.0)  # Compton, Rayleigh factors, max Compton level, angle tolerance (deg)
FF_CHUNKS = 8  # scatter pass in independent chunks: its variance (copies of a history are correlated)
FF_FORCED = (1.0 / 8, 20.0)  # primary pass: ForceDirection on this fraction of the decays per head, cone (deg)
FF_SCATTER_SHARE = 4  # the scatter pass runs 1 / 4 of the primaries
FF_WORKLOAD = SPECT_WORKLOAD + "_freeflight_forced20deg_1of8+scattersplit_c50_r10_aa10deg_1of4"

# SPECT with ARF detectors: Lu-177 (113 keV 6.2 %, 208 keV 10.4 %), medium-energy
# collimator, 120 gantry positions, 1e10 decays.  The ARF acquisition is the
# reference's recipe: a primary pass in free flight with the source's
# ForceDirection toward the heads (10 degree cones, on 1/32 of the decays per
# head) into the ARF detectors plus a scatter-splitting pass into the ARF
# detectors on 1/8 of the primaries; the network is trained on 2e8 photons of
# the plain collimator tracking, and the plain acquisition of as many decays is
# run beside it for the matched-sigma comparison
ARF_METRIC = ("primaries/s (ARF SPECT recipe: primary free-flight pass with forced directions toward the heads + "
              "scatter-splitting pass on 1/8 of the primaries, both into ARF detectors; SPECT projections)")
ARF_DECAYS = 10_000_000_000
ARF_YIELD = 0.166
ARF_WINDOWS = ((0.1872, 0.2288), (0.166, 0.187), (0.1017, 0.1243))
ARF_TRAIN_SAMPLES = 200_000_000
ARF_TRAIN_THETA_DEG = 85.0  # training photons on the detector face: incidence angle uniform up to this
ARF_PRIMARY_DEG = 10.0  # primary pass: angle tolerance of the source's angular acceptance
ARF_SPLIT = (10, 2, 10000, 10.0)  # scatter pass: Compton, Rayleigh factors, max Compton level, angle tolerance
ARF_SCATTER_SHARE = 8  # the scatter pass runs 1 / 8 of the primaries
ARF_FORCED = 1.0 / 32  # primary pass with ForceDirection on this fraction of the decays per head (0: rejection)
ARF_CHUNKS = 16  # ... in independent chunks (its variance)
ARF_SUMMARY_PRIMARIES = 600_000_000  # reduced comparison carried by the default (dose) line
ARF_WORKLOAD = ("spect_lu177_melp_nm670housing_2heads_120angles_r250mm_128x128x4.42mm_windows187-229_166-187_101-125keV_"
                "ct_phantom_256x256x160_1.2mm_arf_mlp3x128_bf16_freeflight_forced10deg_1of32+scattersplit_c10_r2_aa10deg_1of8")


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
            scene, sp, _ = W.spect_phantom(housing=SPECT_HOUSING)
            meta = (SPECT_METRIC, SPECT_WORKLOAD, int(SPECT_DECAYS * SPECT_YIELD))
        else:
            scene, sp, _ = W.spect_phantom(nuclide=W.LU177, collimator=S.MELP, n_runs=120, windows=ARF_WINDOWS,
                                           housing=SPECT_HOUSING)
            meta = (ARF_METRIC, ARF_WORKLOAD, int(ARF_DECAYS * ARF_YIELD))
        runs = sp.n_runs

        def run(n, seed):
            O.run_spect(scene, sp, max(n // runs, 1), seed, threads=threads)

        note = (f"plain collimator tracking over all {runs} positions" +
                (" (the reference's CPU method; the network is not part of its CPU path)"
                 if args.workload == "spect_arf" else ""))
        return meta + ("synthetic (seeded CT phantom + activity image)", run, note, 2000 * runs, int(4e8))
    if args.workload == "spect_ff":
        forced = (args.ff_forced, FF_FORCED[1])
        scene, scene_p, sp_p, sp_s = spect_ff_specs(forced)
        runs, heads = sp_p.n_runs, sp_p.n_heads

        def run(n, seed):  # the GPU step's composition for n primaries
            per = max(n // runs, 1)
            pr = max(heads, int(round(per * forced[0])) * heads) if forced[0] > 0 else per
            O.run_spect_ff(scene_p, sp_p, pr, seed, threads=threads)
            O.run_spect_ff(scene, sp_s, max(1, per // args.ff_scatter_share), seed + 1, threads=threads)

        return (FF_METRIC, FF_WORKLOAD, int(FF_DECAYS * SPECT_YIELD), "synthetic (seeded CT phantom + activity image)",
                run, f"primary free flight (forced directions) + scatter splitting over all {runs} positions",
                200 * runs, int(4e8))
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

    scene, sp, _ = W.spect_phantom(housing=SPECT_HOUSING)
    n_step = args.primaries if args.primaries != PRIMARIES_PER_STEP else int(SPECT_DECAYS * SPECT_YIELD)
    n_per_run = n_step // sp.n_runs
    n = n_per_run * sp.n_runs
    eng = SpectEngine(scene, sp, device=local, precision=32, batch=args.batch)
    l2_flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")
    if args.record_singles:  # the digitizer's singles list, read back after every step
        eng.record_singles(args.record_singles)
    n_singles = []

    def first_of(step):
        return ((rank * (args.warmup + args.steps + 4)) + step) * n

    for w in range(args.warmup):
        eng.reset()
        eng.run(n_per_run, args.seed, first_of(w))
        if args.record_singles:
            eng.singles()
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
            if args.record_singles:
                n_singles.append(len(eng.singles()))
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
                          "singles": counters["singles"], "launches_per_step": launches_last,
                          "singles_listed": n_singles[-1] if n_singles else None},
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


def spect_ff_specs(forced=FF_FORCED):
    """(scene, primary-pass scene, primary free-flight spec, scatter-splitting spec) of the
    SPECT workload; the primary-pass scene's source has ForceDirection toward the heads (the
    reference's setup_force_direction, test085_free_flight_spect_2b_fd: 20 degree cones) when
    `forced` is given."""
    from opengate_gb300 import _capi as C
    from opengate_gb300 import workloads as W

    scene, sp_p, _ = W.spect_phantom(housing=SPECT_HOUSING)
    sp_s = copy.deepcopy(sp_p)
    sp_p.set_free_flight()
    nc, nr, lvl, deg = FF_SPLIT
    sp_s.set_scatter_splitting(nc, nr, lvl, angle_tolerance_max=math.radians(deg))
    scene_p = scene
    if forced and forced[0] > 0:
        scene_p = copy.copy(scene)
        src = copy.copy(scene.source)
        src.dir_type = C.GG_DIR_FORCED
        src.fd_angle_min, src.fd_angle_max = 0.0, math.radians(forced[1])
        scene_p.set_source(src)
    return scene, scene_p, sp_p, sp_s


def run_ours_ff(args, ws, rank, local, dist, use_cuda):
    """The reference's free-flight SPECT recipe (contrib/spect/spect_config.py:937-1000): a
    primary pass (GammaFreeFlightActor) and a scatter pass (ScatterSplittingFreeFlightActor),
    whose weighted projections add up to the acquisition.  value: primaries/s of both passes
    on the same primaries; sigma: efficiency (1 / sigma^2 T) against the analog SPECT path."""
    import torch

    from opengate_gb300.engine import SpectEngine

    forced = (args.ff_forced, FF_FORCED[1])
    scene, scene_p, sp_p, sp_s = spect_ff_specs(forced)
    runs = sp_p.n_runs
    heads = sp_p.n_heads
    n_step = args.primaries if args.primaries != PRIMARIES_PER_STEP else int(FF_DECAYS * SPECT_YIELD)
    n_per_run = n_step // runs // FF_CHUNKS * FF_CHUNKS
    n = n_per_run * runs
    # scatter pass on 1 / share of the primaries, in FF_CHUNKS chunks
    m = max(1, n_per_run // args.ff_scatter_share // FF_CHUNKS)
    n_s = m * FF_CHUNKS * runs
    # primary pass: all primaries, or (ForceDirection) `forced` of them per head
    np_run = max(heads, int(round(n_per_run * forced[0])) * heads) if forced[0] > 0 else n_per_run
    n_pe = (np_run // heads if forced[0] > 0 else np_run) * runs  # decays per head it stands for
    eng_p = SpectEngine(scene_p, sp_p, device=local, precision=32, batch=args.batch)
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
        eng_p.run(np_run, args.seed, first)
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
    # both passes scaled to the n primaries of the analog acquisition
    sc_p, sc_s = n / n_pe, n / n_s
    ch = np.array(chunks).sum(axis=(3, 4))
    t_ff = wp.sum(axis=(2, 3)) * sc_p + ch.sum(axis=0) * sc_s
    v_ff = wp2.sum(axis=(2, 3)) * sc_p ** 2 + FF_CHUNKS * ch.var(axis=0, ddof=1) * sc_s ** 2
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
        eng_p.run(np_run, args.seed, first)
        eng_s.run(m * FF_CHUNKS, args.seed + 1, first)
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

        def run(nn, seed):  # the step's composition for nn primaries
            per = max(nn // runs, 1)
            pr = max(heads, int(round(per * forced[0])) * heads) if forced[0] > 0 else per
            O.run_spect_ff(scene_p, sp_p, pr, seed, threads=threads)
            O.run_spect_ff(scene, sp_s, max(1, per // args.ff_scatter_share), seed + 1, threads=threads)

        r, ns, dt = grow_sample(run, args.cpu_seconds, 200 * runs, int(4e8))
        cpu = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{ns} primaries through both passes over the {runs} positions, {dt:.1f} s on "
                         f"{threads} host threads"}
    fp64 = None
    if rank == 0 and args.fp64_primaries > 0:
        npr = max(1, min(args.fp64_primaries, 10_000_000) // runs)
        fp64 = {"primary_pass": spect_fp64_error(scene_p, sp_p, npr, args.seed, local, args.batch, weighted=True),
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
                       "primary_pass": {"forced_direction_share_per_head": forced[0] or None,
                                        "cone_deg": forced[1] if forced[0] > 0 else None,
                                        "histories": int(np_run * runs)},
                       "scatter_pass": {"share_of_primaries": 1.0 / args.ff_scatter_share, "histories": int(n_s)},
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


class ArfRecipe:
    """The ARF acquisition of the spect_arf workload, and the plain acquisition beside it.

    ARF acquisition, as the reference's free-flight and ARF recipes compose it
    (contrib/spect/spect_config.py:937-1000, actors/arfactors.py:349-453):
      * primary pass: free flight from the source with the angle check of the
        source's angular acceptance (biasing/GateGammaFreeFlightOptn.cpp:34-83);
        a photon that reaches a head face adds exp(-optical depth) x the
        network's window probabilities;
      * scatter pass, on 1 / ARF_SCATTER_SHARE of the primaries: scatter
        splitting (GateScatterSplittingFreeFlightOptrActor.cpp:291-420), the
        copies reaching a head scored by the network with their weight; run in
        ARF_CHUNKS independent chunks (the copies of a history are correlated,
        so its variance comes from the chunks).
    Plain acquisition: analog photons tracked through the collimator and
    crystal (counts).  The network is trained on rows of the plain head
    transport before either runs."""

    def __init__(self, local, seed, batch, train_samples, epochs, n_runs=120, primary_deg=ARF_PRIMARY_DEG,
                 split=ARF_SPLIT, share=ARF_SCATTER_SHARE, forced=0.0):
        from opengate_gb300 import spect as S
        from opengate_gb300 import workloads as W
        from opengate_gb300.engine import ArfNetwork, SpectEngine

        self.scene, self.sp, _ = W.spect_phantom(nuclide=W.LU177, collimator=S.MELP, n_runs=n_runs,
                                                 windows=ARF_WINDOWS, housing=SPECT_HOUSING)
        batch = min(batch, 1 << 26)
        self.plain = SpectEngine(self.scene, self.sp, device=local, precision=32, batch=batch)
        net = ArfNetwork(self.plain)
        # training rows: plain head transport of photons on the face, theta uniform to ARF_TRAIN_THETA_DEG
        smp = ArfNetwork.sampling(min(lo for lo, _ in ARF_WINDOWS), 0.21, ARF_TRAIN_THETA_DEG, (200.0, 200.0), 40.0)
        t0 = time.perf_counter()
        self.model, self.loss = net.train(smp, train_samples, seed=seed + 7, epochs=epochs, batch=8192, lr=2e-3,
                                          lr_final=1e-5)
        self.train_s = time.perf_counter() - t0
        self.params = net.params()
        self.sp_p = copy.deepcopy(self.sp)
        self.primary_deg, self.split, self.share, self.forced = primary_deg, tuple(split), share, float(forced)
        self.sp_p.set_free_flight(angle_tolerance_max=math.radians(primary_deg))
        scene_p = self.scene
        if self.forced > 0:
            # ForceDirection toward the heads (the reference's setup_force_direction): each
            # primary-pass history aims at one head within the cone, weight (1 - cos) / 2; the
            # pass simulates `forced` of the decays per head
            from opengate_gb300 import _capi as C

            scene_p = copy.copy(self.scene)
            src = copy.copy(self.scene.source)
            src.dir_type = C.GG_DIR_FORCED
            src.fd_angle_min, src.fd_angle_max = 0.0, math.radians(primary_deg)
            scene_p.set_source(src)
        nc, nr, lvl, deg = self.split
        self.sp_s = copy.deepcopy(self.sp)
        self.sp_s.set_scatter_splitting(nc, nr, lvl, angle_tolerance_max=math.radians(deg))
        self.scene_p = scene_p
        self.prim = SpectEngine(scene_p, self.sp_p, device=local, precision=32, batch=batch)
        self.scat = SpectEngine(self.scene, self.sp_s, device=local, precision=32, batch=batch)
        for e in (self.prim, self.scat):
            ArfNetwork(e).set_model(self.model, self.params)
            e.use_arf(True)
            e.reset()
        self.nw = self.sp.n_windows

    def scatter_per_run(self, n_per_run):
        return max(1, n_per_run // self.share // ARF_CHUNKS)

    def acquire(self, n_per_run, seed, first, keep=False):
        """One ARF acquisition (histories first .. first + n_per_run x positions): device ms,
        kernel launches, device ms per pass, and with keep the tallies for its statistics."""
        runs = self.sp.n_runs
        m = self.scatter_per_run(n_per_run)
        heads = self.sp.n_heads
        # primary-pass histories per run, and the decays they stand for per head
        np_run = max(heads, int(round(n_per_run * self.forced)) * heads) if self.forced > 0 else n_per_run
        self.prim.reset()
        self.prim.run(np_run, seed, first)
        tg, tt, tf, nl = self.prim.last_kernel_ms()
        parts = {"primary_pass": tg + tt + tf}
        ph, hd, arf = self.prim.last_stage_ms()
        parts.update({"primary_phantom_stage": ph, "primary_head_stage": hd, "primary_arf_stage": arf})
        ms = tg + tt + tf
        st = None
        if keep:
            wp, wp2 = self.prim.weighted_projection(squared=True)
            st = {"wp": wp, "wp2": wp2, "n_p": (np_run // heads if self.forced > 0 else np_run) * runs,
                  "n_s": m * ARF_CHUNKS * runs,
                  "counters_primary": self.prim.counters()}
            prev, s2, tot = 0.0, 0.0, []
        self.scat.reset()
        sc = {"scatter_pass": 0.0, "scatter_phantom_stage": 0.0, "scatter_head_stage": 0.0,
              "scatter_copies_and_arf": 0.0}
        for c in range(ARF_CHUNKS):
            self.scat.run(m, seed + 1, first + c * m * runs)  # run r of a call: first + r * m
            tg, tt, tf, k = self.scat.last_kernel_ms()
            ph, hd, cp = self.scat.last_stage_ms()
            ms, nl = ms + tg + tt + tf, nl + k
            sc["scatter_pass"] += tg + tt + tf
            sc["scatter_phantom_stage"] += ph
            sc["scatter_head_stage"] += hd
            sc["scatter_copies_and_arf"] += cp
            if keep:
                cur = self.scat.weighted_projection()
                d = cur - prev
                s2 = s2 + d * d
                tot.append(d.sum(axis=(2, 3)))
                prev = cur
        parts.update(sc)
        if keep:
            st.update({"ws": prev, "ws_c2": s2, "chunk_totals": np.array(tot), "counters_scatter": self.scat.counters()})
        return ms, nl, parts, st

    def estimate(self, st):
        """Per-primary projection of the ARF acquisition and the variance of that mean,
        per pixel and per projection total (head, position x window)."""
        n_p, n_s, j = st["n_p"], st["n_s"], ARF_CHUNKS
        mp = st["wp"] / n_p
        vp = np.maximum((st["wp2"] / n_p - mp * mp) / (n_p - 1), 0.0)
        # var(sum of j iid chunks) = j / (j - 1) * (sum c^2 - (sum c)^2 / j)
        vs = np.maximum(j / (j - 1) * (st["ws_c2"] - st["ws"] ** 2 / j), 0.0) / n_s ** 2
        m = mp + st["ws"] / n_s
        tp = st["wp"].sum(axis=(2, 3)) / n_p
        tvp = np.maximum((st["wp2"].sum(axis=(2, 3)) / n_p - tp * tp) / (n_p - 1), 0.0)
        ch = st["chunk_totals"]
        t = tp + ch.sum(axis=0) / n_s
        tvs = j * ch.var(axis=0, ddof=1) / n_s ** 2
        self.parts_var = (vp, vs, tvp, tvs)  # per-pass variances (allocation report)
        return m, vp + vs, t, tvp + tvs

    def compare(self, n_per_run, seed, first_arf, first_plain, arf_ms=None):
        """Matched-sigma comparison: one ARF acquisition and one plain acquisition of
        n_per_run histories per position.  Efficiency 1 / (sigma^2 T) per pixel of the
        peak window (mean relative sigma over pixels > 10 % of max) and per projection
        total (mean over projections, per window); window totals ARF / plain with their
        1-sigma statistical error."""
        import torch

        from opengate_gb300 import spect as S

        ms_a, _, parts, st = self.acquire(n_per_run, seed, first_arf, keep=True)
        if arf_ms is not None:
            ms_a = arf_ms
        self.plain.reset()
        torch.cuda.synchronize()
        self.plain.run(n_per_run, seed + 2, first_plain)
        tg, tt, tf, _ = self.plain.last_kernel_ms()
        ms_p = tg + tt + tf
        cp = self.plain.projection()
        n = n_per_run * self.sp.n_runs
        nw = self.nw
        m, v, t, tv = self.estimate(st)
        pk = m[:, 0::nw]
        sel = pk > 0.1 * pk.max()
        sig_a_pix = float((np.sqrt(v[:, 0::nw][sel]) / pk[sel]).mean())
        sig_p_pix = S.mean_relative_uncertainty(cp[:, 0::nw], cp[:, 0::nw], n)
        tp = cp.sum(axis=(2, 3))
        # the same pixels for both arms (peak-window pixels above 10 % of the primary pass's
        # maximum: its mean image is the least noisy), relative variances against the ARF mean
        # image; plain: Poisson variance of the counts
        mpk = st["wp"][:, 0::nw] / st["n_p"]
        mask = (mpk > 0.1 * mpk.max()) & (pk > 0)
        rv_a = float((v[:, 0::nw][mask] / pk[mask] ** 2).mean())
        rv_p = float((cp[:, 0::nw][mask] / float(n) ** 2 / pk[mask] ** 2).mean())
        out = {"arf_ms": ms_a, "plain_ms": ms_p, "primaries": n, "scatter_pass_primaries": st["n_s"],
               "arf_ms_per_pass": parts,
               "pixel_peak_window": {"sigma_arf": sig_a_pix, "sigma_plain": sig_p_pix,
                                     "efficiency_gain": (sig_p_pix ** 2 * ms_p) / (sig_a_pix ** 2 * ms_a),
                                     "method": "mean relative sigma over each arm's pixels > 10 % of its max "
                                               "(the reference's per-pixel figure)"},
               "pixel_peak_window_common_mask": {
                   "pixels": int(mask.sum()), "rel_var_arf": rv_a, "rel_var_plain": rv_p,
                   "efficiency_gain": (rv_p * ms_p) / (rv_a * ms_a),
                   "method": "mean relative variance over the same pixels (> 10 % of the primary pass's "
                             "max), both against the ARF mean image"},
               "projection_totals": {}, "window_totals_arf_over_plain": [], "window_ratio_sigma": []}
        for w in range(nw):
            ta, va, tpl = t[:, w::nw], tv[:, w::nw], tp[:, w::nw]
            ok = (ta > 0) & (tpl > 0)
            sa = float((np.sqrt(va[ok]) / ta[ok]).mean())
            spl = float((1.0 / np.sqrt(tpl[ok])).mean())
            out["projection_totals"][f"window_{w}"] = {
                "sigma_arf": sa, "sigma_plain": spl, "efficiency_gain": (spl ** 2 * ms_p) / (sa ** 2 * ms_a)}
            r = float(ta.sum() / (tpl.sum() / n))
            out["window_totals_arf_over_plain"].append(r)
            out["window_ratio_sigma"].append(r * math.sqrt(va.sum() / ta.sum() ** 2 + 1.0 / tpl.sum()))
        # allocation between the passes: each pass's share of the relative variance (peak-window
        # pixels; projection totals of window 0) and the efficiency of the best split of the
        # time between them, (sqrt(A t_p) + sqrt(B t_s))^-2 for variance shares A, B and pass
        # times t_p, t_s (variance of a pass ~ 1 / its primaries, time ~ its primaries)
        vp, vs, tvp, tvs = self.parts_var
        t_p, t_s = parts["primary_pass"], parts["scatter_pass"]
        alloc = {"primary_ms": t_p, "scatter_ms": t_s, "scatter_share": 1.0 / self.share}
        for key, (a_, b_, mm, sel_) in {"pixel_peak_window": (vp[:, 0::nw], vs[:, 0::nw], pk, sel),
                                         "projection_window_0": (tvp[:, 0::nw], tvs[:, 0::nw], t[:, 0::nw],
                                                                 t[:, 0::nw] > 0)}.items():
            a = float((a_[sel_] / mm[sel_] ** 2).mean())
            b = float((b_[sel_] / mm[sel_] ** 2).mean())
            best = (math.sqrt(a * t_p) + math.sqrt(b * t_s)) ** 2
            plain = (sig_p_pix ** 2 * ms_p) if key.startswith("pixel") else \
                out["projection_totals"]["window_0"]["sigma_plain"] ** 2 * ms_p
            alloc[key] = {"rel_var_primary": a, "rel_var_scatter": b,
                          "best_scatter_share": 1.0 / self.share * math.sqrt(b * t_p / max(a * t_s, 1e-300)),
                          "efficiency_gain_at_best_split": plain / best}
        out["allocation"] = alloc
        cnt = {f"primary_{k}": st["counters_primary"][k] for k in ("world_steps", "arf_photons", "arf_fallback")}
        cnt.update({f"scatter_{k}": st["counters_scatter"][k] for k in ("woodcock_steps", "arf_photons",
                                                                        "arf_fallback")})
        out["units"] = cnt
        out["method"] = ("ARF: primary pass history-by-history squares + scatter pass variance of "
                         f"{ARF_CHUNKS} independent chunks; plain: counts (Poisson); efficiency 1 / (sigma^2 T), "
                         "contrib/spect/spect_helpers.py:480-488")
        return out

    def close(self):
        for e in (self.prim, self.scat, self.plain):
            e.close()


def arf_options(args):
    split = list(ARF_SPLIT)
    split[3] = args.arf_scatter_deg
    return {"primary_deg": args.arf_primary_deg, "split": split, "share": args.arf_scatter_share,
            "forced": args.arf_forced}


def arf_summary(args, local):
    """A reduced spect_arf comparison for the default bench line (rank 0, untimed)."""
    r = ArfRecipe(local, args.seed, args.batch, args.arf_train_samples, args.arf_epochs, **arf_options(args))
    try:
        n_per_run = ARF_SUMMARY_PRIMARIES // r.sp.n_runs
        r.acquire(n_per_run // 8, args.seed, 0)  # warm-up
        out = r.compare(n_per_run, args.seed, 1 << 40, 1 << 41)
        out["training_seconds"] = r.train_s
        out["workload"] = ARF_WORKLOAD
        out["options"] = arf_options(args)
        return out
    finally:
        r.close()


def run_ours_arf(args, ws, rank, local, dist, use_cuda):
    import torch

    rec = ArfRecipe(local, args.seed, args.batch, args.arf_train_samples, args.arf_epochs, **arf_options(args))
    scene, sp = rec.scene, rec.sp
    n_step = args.primaries if args.primaries != PRIMARIES_PER_STEP else int(ARF_DECAYS * ARF_YIELD)
    n_per_run = n_step // sp.n_runs
    n = n_per_run * sp.n_runs
    l2_flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    def first_of(step):
        return ((rank * (args.warmup + args.steps + 8)) + step) * n

    for w in range(args.warmup):
        rec.acquire(n_per_run, args.seed, first_of(w))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    dev_ms, launches, parts = [], 0, None
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            l2_flush.zero_()
            torch.cuda.synchronize()
            ms, nl, parts, _ = rec.acquire(n_per_run, args.seed, first_of(args.warmup + k))
            dev_ms.append(ms)
            launches += nl
        torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    total_ms = dist_max(dist, float(np.sum(dev_ms)), use_cuda)
    value = ws * n * args.steps / (total_ms / 1e3)
    # statistics of one more acquisition (untimed: it reads the projections per chunk),
    # charged the timed steps' mean duration, and the plain acquisition of as many primaries
    cmp = rec.compare(n_per_run, args.seed, first_of(args.warmup + args.steps),
                      first_of(args.warmup + args.steps + 1), arf_ms=total_ms / args.steps)
    cnt_p = rec.prim.counters()

    # e2e through the C ABI with host buffers: scene + heads + network upload to both
    # passes' contexts, the acquisition, weighted projections down
    h2d = 2 * (scene.labels.nbytes + scene._sig.nbytes + scene._cum.nbytes + scene._ray_amax.nbytes +
               scene._ray_cum.nbytes + scene.majorant.nbytes + scene.source_desc_bytes() + sp.all_frames().nbytes +
               rec.params.nbytes)
    d2h = 2 * 3 * int(np.prod(sp.projection_shape())) * 8
    from opengate_gb300.engine import ArfNetwork

    torch.cuda.synchronize()
    e2e_t = []
    for k in range(max(1, min(args.steps, 2))):
        t1 = time.perf_counter()
        for e in (rec.prim, rec.scat):
            e.upload()
            ArfNetwork(e).set_model(rec.model, rec.params)
            e.use_arf(True)
        rec.acquire(n_per_run, args.seed, first_of(args.warmup + args.steps + 2 + k))
        rec.prim.weighted_projection(squared=True)
        rec.scat.weighted_projection(squared=True)
        e2e_t.append(time.perf_counter() - t1)
    e2e_s = dist_max(dist, float(np.mean(e2e_t)), use_cuda)
    fp64 = None
    if rank == 0 and args.fp64_primaries > 0:
        npr = max(1, args.fp64_primaries // sp.n_runs)
        fp64 = {"primary_pass": spect_fp64_error(rec.scene_p, rec.sp_p, npr, args.seed, local, min(args.batch, 1 << 26),
                                                 arf=(rec.model, rec.params), weighted=True),
                "scatter_pass": spect_fp64_error(scene, rec.sp_s, max(1, npr // 10), args.seed, local,
                                                 min(args.batch, 1 << 26), arf=(rec.model, rec.params),
                                                 weighted=True)}
    # the network's arithmetic: forward FLOP per scored photon
    flop_photon = 2.0 * (3 * 128 + 2 * 128 * 128 + 128 * 16)
    peak_bw, peak_kind = measured_peaks()
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    cnt_s = rec.scat.counters()
    bytes_alg = 32.0 * cnt_s["woodcock_steps"]
    ph_ms = parts["scatter_phantom_stage"]
    net_tf = flop_photon * cnt_p["arf_photons"] / (parts["primary_arf_stage"] / 1e3) / 1e12
    if rank == 0:
        line = {
            "metric": ARF_METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 transport, bf16 network (f32 accumulate)",
            "data": "synthetic (seeded CT phantom + activity image)",
            "config": {"workload": ARF_WORKLOAD, "primaries_per_step": n, "decays_per_step": n / ARF_YIELD,
                       "primary_pass_angle_tolerance_deg": rec.primary_deg,
                       "primary_pass_forced_direction_share": rec.forced or None,
                       "scatter_pass": {"share_of_primaries": 1.0 / rec.share, "chunks": ARF_CHUNKS,
                                        "compton": rec.split[0], "rayleigh": rec.split[1],
                                        "max_compton_level": rec.split[2], "angle_tolerance_deg": rec.split[3]},
                       "l2": "flushed between steps (256 MiB write)", "training_samples": args.arf_train_samples,
                       "parallelism": f"replicas x{ws}, disjoint history ranges"},
            "matched_sigma": cmp,
            "training": {"seconds": rec.train_s, "loss_first_last": [float(rec.loss[0]), float(rec.loss[-1])],
                         "epochs": args.arf_epochs},
            "fp64_error": fp64,
            "e2e": {"value": ws * n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "kernel": "k_spect_phantom<float, scatter splitting> (scatter pass)",
                         "achieved": bytes_alg / (ph_ms / 1e3) / 1e9, "peak": peak_bw, "unit": "GB/s",
                         "frac": bytes_alg / (ph_ms / 1e3) / 1e9 / peak_bw, "peak_kind": peak_kind,
                         "traffic": args.traffic, "bytes_alg_per_step": bytes_alg,
                         "note": "label gathers of the scatter pass's analog Woodcock steps"},
            "roofline_network": {"bound": "tensor", "kernel": "k_spect_arf<float> (ARF stage, network layers)",
                                 "flop_per_scored_photon": flop_photon,
                                 "scored_photons_per_step": cnt_p["arf_photons"] + cnt_s["arf_photons"],
                                 "achieved": net_tf, "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
                                 "frac": net_tf / peaks.get("bf16_tflops", 1.0),
                                 "note": "primary pass's ARF stage (network on its scored photons, the queue "
                                         "classification and the projection atomics included); tcgen05.mma "
                                         "kind::f16 (M 128, N 128 / 16, K 16) BF16, FP32 accumulate in TMEM"},
            "stage_ms_per_step": parts,
            "cpu_baseline": None,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
            "wall_s": wall,
        }
        print(json.dumps(line), flush=True)
    rec.close()
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
    tune = eng.autotune_result()
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
    # the label images from page-locked buffers as well
    eng.sims = [(eng.pinned_scene(sc), k, sd) for sc, k, sd in sims]
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
    # FP32 against the FP64 build on the same histories (untimed), per simulation
    fp64 = None
    if rank == 0 and args.fp64_primaries > 0:
        from opengate_gb300.dose import precision_error

        imgs = {}
        rate = {}
        for prec in (32, 64):
            with BatchEngine(sims, device=local, precision=prec) as e:
                e.run()
                g, t, f, _ = e.last_kernel_ms()
                rate[prec] = n / ((g + t + f) / 1e3)
                imgs[prec] = [(e.image(k, C.GG_IMG_EDEP), e.image(k, C.GG_IMG_EDEP_SQUARED)) for k in range(len(sims))]
        errs = [precision_error(a[0], a[1], b[0], b[1], k) for a, b, (_, k, _) in zip(imgs[32], imgs[64], sims)]
        fp64 = {"simulations": len(errs), "primaries": n,
                "integral_rel_max": max(e["integral_rel"] for e in errs),
                "within_2sigma_min": min(e.get("within_2sigma", 1.0) for e in errs),
                "rate_f32": rate[32], "rate_f64": rate[64], "voxels_gt": "10 % of max, per simulation"}
    if rank == 0:
        line = {
            "metric": BATCH_METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded slab phantoms)",
            "config": {"workload": BATCH_WORKLOAD, "simulations": len(sims), "primaries_per_step": n,
                       "voxels": int(sum(s.n_voxels for s, _, _ in sims)),
                       "l2": "flushed between steps (256 MiB write)",
                       "launch": "CUDA graph replay; per batch one source launch, one persistent transport "
                                 "launch taking the histories of all simulations from one device work counter "
                                 "(in-kernel binding of each history's simulation), one flush launch",
                       "autotuned": {"blocks_per_sm": best.blocks_per_sm, "refill_min": best.refill_min,
                                     "interact_min": best.interact_min, "claim_chunk": best.chunk,
                                     "batch_length": int(best.batch), "block_size": best.block_size,
                                     "search": tune, "seconds": tune_s},
                       "parallelism": f"replicas x{ws}, independent batches"},
            "sequential": {"primaries_per_s": n / (seq_ms / 1e3), "note": "gg_run per simulation, same context"},
            "fp64_error": fp64,
            "e2e": {"value": ws * n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak_bw, "unit": "GB/s",
                         "frac": achieved / peak_bw, "traffic": args.traffic, "peak_kind": peak_kind,
                         "kernel": "k_transport<float, MULTI> (batched transport)",
                         "bytes_alg_per_step": bytes_alg, "note": "graph replay time includes source and flush"},
            "cpu_baseline": None,
            "clocks": clk.summary(),
            "gpu_launches": int(len(dev_ms) * 3 * max(1, -(-n // max(1, int(best.batch))))),
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
    from opengate_gb300 import replicas as Rp
    from opengate_gb300 import workloads as W
    from opengate_gb300.engine import DoseEngine

    scene, _ = W.ct_phantom()
    n = args.primaries
    eng = DoseEngine(scene, device=local, precision=32, batch=args.batch)
    kernel = {"phased": C.GG_KERNEL_PHASED, "wavefront": C.GG_KERNEL_WAVEFRONT}[args.transport_kernel]
    eng.set_transport_kernel(kernel)
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
    dev_ms, merge_ms = [], []
    n_merged = n
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
            if ws > 1:
                # the replicas' images summed on the devices (NCCL all_reduce of the FP64
                # images in place), timed on torch's stream where the collective runs
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ev0.record()
                n_merged = Rp.merge_tallies_device(eng, (C.GG_IMG_EDEP, C.GG_IMG_EDEP_SQUARED), n)
                ev1.record()
                torch.cuda.synchronize()
                merge_ms.append(ev0.elapsed_time(ev1))
                dev_ms[-1] += merge_ms[-1]
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

    # sigma reached by one step (mean relative uncertainty, voxels > 10 % max); with
    # replicas, of the merged images of all ranks' histories
    edep, edep2 = eng.edep(), eng.edep_squared()
    sigma = mean_relative_uncertainty(edep, edep2, n_merged)

    # e2e through the C ABI with host buffers: scene upload (H2D), run, image download (D2H)
    h2d = scene.labels.nbytes + scene._sig.nbytes + scene._cum.nbytes + scene._ray_amax.nbytes + \
        scene._ray_cum.nbytes + scene.majorant.nbytes
    d2h = 2 * scene.n_voxels * 8
    # the label image comes from and the images land in page-locked host buffers reused every
    # step (gg_host_alloc), as a production caller keeps them
    out_e = eng.pinned_empty(scene.labels.shape)
    out_e2 = eng.pinned_empty(scene.labels.shape)
    eng.scene = eng.pinned_scene(scene)
    torch.cuda.synchronize()
    e2e_t = []
    for k in range(max(1, min(args.steps, 3))):
        t1 = time.perf_counter()
        eng.upload()
        eng.run(n, args.seed, first_of(args.warmup + args.steps + k))
        eng.edep(out_e), eng.edep_squared(out_e2)
        e2e_t.append(time.perf_counter() - t1)
    eng.scene = scene
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
                "peak_kind": peak_kind,
                "kernel": "k_transport<float>" if args.transport_kernel == "phased" else "k_wavefront<float>",
                "bytes_alg_per_step": bytes_alg,
                "units": {"woodcock_steps": counters["woodcock_steps"], "tally_entries": counters["tally_entries"],
                          "transport_launches_per_step": transport_launches},
                "stage_ms_per_step": stage_ms}

    # issue roofline of the transport kernel: warp instructions per second against the SMs'
    # issue peak (4 schedulers per SM, one warp instruction per cycle each, at the sampled clock)
    clk_summary = clk.summary()
    mhz = (clk_summary or {}).get("sm_mhz") or (clk_summary or {}).get("sm_max_mhz") or 2070.0
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    issue_peak = n_sm * 4 * mhz * 1e6
    inst_pp, lanes = TRANSPORT_ISSUE[args.transport_kernel]
    issue_ach = inst_pp * n / (transport_ms / 1e3)
    roofline_issue = {"bound": "issue", "achieved": issue_ach, "peak": issue_peak, "unit": "warp instructions/s",
                      "frac": issue_ach / issue_peak, "active_lanes_per_instruction": lanes,
                      "lane_weighted_frac": issue_ach / issue_peak * lanes / 32.0,
                      "note": "warp instructions per primary from an ncu capture of this kernel on this "
                              "workload (3e6 primaries) x primaries / CUDA-event transport time; peak = SMs x 4 "
                              "schedulers x the median sampled SM clock"}
    # error of the FP32 transport against the FP64 build on the same random stream (untimed)
    fp64 = None
    if rank == 0 and args.fp64_primaries > 0:
        fp64 = fp64_error(scene, args.fp64_primaries, args.seed, local, args.batch)

    # the spect_arf matched-sigma comparison at reduced size (untimed, separate contexts)
    arf = None
    if rank == 0 and ws == 1 and not args.no_arf_summary:
        eng.close()
        arf = arf_summary(args, local)

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
                       "transport_kernel": args.transport_kernel,
                       "l2": "flushed between steps (256 MiB write)", "batch": args.batch,
                       "parallelism": f"replicas x{ws}, disjoint history ranges"},
            "sigma": {"mean_relative_uncertainty_gt10pct_max": sigma, "primaries": n_merged},
            "replica_merge": {"ms_per_step": float(np.mean(merge_ms)) if merge_ms else None,
                              "method": "NCCL all_reduce of the FP64 edep and edep^2 device images, in the "
                                        "timed step (replicas.merge_tallies_device)"} if ws > 1 else None,
            "fp64_error": fp64,
            "spect_arf_efficiency": arf,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "roofline": roofline,
            "roofline_issue": roofline_issue,
            "cpu_baseline": cpu,
            "clocks": clk_summary,
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
    ap.add_argument("--arf-primary-deg", type=float, default=ARF_PRIMARY_DEG,
                    help="spect_arf: angle tolerance of the primary free-flight pass (degrees)")
    ap.add_argument("--arf-scatter-deg", type=float, default=ARF_SPLIT[3],
                    help="spect_arf: angle tolerance of the scatter-splitting copies (degrees)")
    ap.add_argument("--ff-forced", type=float, default=FF_FORCED[0],
                    help="spect_ff: primary pass with ForceDirection on this fraction of the decays per head "
                         "(0: all decays, no angle check)")
    ap.add_argument("--ff-scatter-share", type=int, default=FF_SCATTER_SHARE,
                    help="spect_ff: the scatter pass runs 1 / share of the primaries")
    ap.add_argument("--arf-forced", type=float, default=ARF_FORCED,
                    help="spect_arf: primary pass with ForceDirection toward the heads on this fraction of "
                         "the decays per head (0: angle check by rejection on all decays)")
    ap.add_argument("--arf-scatter-share", type=int, default=ARF_SCATTER_SHARE,
                    help="spect_arf: the scatter pass runs 1 / share of the primaries")
    ap.add_argument("--batch", type=int, default=1 << 27)
    ap.add_argument("--record-singles", type=int, default=0,
                    help="spect: keep the singles in a device list of this many records, read every step")
    ap.add_argument("--seed", type=int, default=20240611)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--transport-kernel", default="phased", choices=["phased", "wavefront"],
                    help="dose workload: the phase kernel (default) or the compacted wavefront kernel")
    ap.add_argument("--no-arf-summary", action="store_true",
                    help="dose workload: skip the reduced spect_arf comparison carried by its line")
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
