// gg_transport.cu - photon transport through a voxelised image with DoseActor scoring.
//
// Replaces, for photons in a voxelised volume, Geant4's stepping through the
// replica/parameterised voxels of ImageVolume
// (opengate/geometry/volumes.py:1093-1125, GateImageNestedParameterisation.cpp:47-75)
// and the scoring of GateDoseActor::SteppingAction / ScoreSquaredValue /
// FlushSquaredValues (core/opengate_core/opengate_lib/GateDoseActor.cpp:180-243, 359-397).
//
// Kernel design (one GB300, one process):
//   * persistent grid, one photon history per thread at a time; a warp claims
//     histories from a global counter in chunks (one atomic per chunk) and
//     hands them to its lanes as they finish (ballot + popc), so no lane idles
//     while work remains;
//   * Woodcock (delta) tracking against a per-energy majorant inside the image
//     box; analytic free flight in the world material outside it;
//   * the majorant, total attenuation rows and the label->(composition,
//     density) table are staged in shared memory; labels are read through the
//     read-only path (the image is L2-resident up to ~60 M voxels);
//   * every history keeps its deposits in a register list of (voxel, sum);
//     when the history ends each entry adds q = round(sum * 2^32) to the edep
//     tally (64-bit integer atomic) and q^2 to a 128-bit edep-squared tally:
//     the history-by-history squared sum of GateDoseActor, order independent
//     and therefore bit-reproducible;
//   * a second kernel flushes the per-batch fixed-point tallies into the
//     float64 images (and clears them), one voxel per thread, coalesced.
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_physics.cuh"
#include "gg_spect.cuh"

namespace gg {

// First step of a sampled primary in the source stage: a photon outside the
// image takes its first world flight here (dose; SPECT leaves it to the
// transport stage, whose world step also targets the heads).  Sets the
// record state; true when a world step was taken.
template <typename real>
__device__ __forceinline__ bool first_flight(const Scene<real> &s, RngAhead &g, Photon<real> &ph, uint32_t &state,
                                             uint32_t &steps, BlockCounters *bc) {
  if (ph.in_image) {
    state = kRecInImage;
    return false;
  }
  if (s.spect) {
    state = kRecWorld;
    return false;
  }
  steps = 1;
  real inf = gg_inf(real(0));
  real tin = ph.can_enter ? entry_distance(ph.pos, ph.dir, s.bmin, s.bmax) : inf;
  real wlo[3] = {-s.whalf[0], -s.whalf[1], -s.whalf[2]};
  real tout = exit_distance(ph.pos, ph.dir, wlo, s.whalf);
  int wm = s.world_mat;
  real mu = interp_row(s.sig + (size_t)s.mat_comp[wm] * s.n_e, ph.ei);
  mu = s.mat_rho[wm] * mu;
  real u = u01_open0<real>(g);
  real sd = -gg_log(u);
  sd = sd / mu;
  if (sd < tin && sd < tout) {
#pragma unroll
    for (int k = 0; k < 3; ++k) ph.pos[k] = ph.pos[k] + sd * ph.dir[k];
    state = kRecPendingWorld;
  } else if (tin <= tout) {
#pragma unroll
    for (int k = 0; k < 3; ++k) ph.pos[k] = ph.pos[k] + tin * ph.dir[k];
    state = kRecInImage;
  } else {
    atomicAdd(&bc->escaped, 1u);
  }
  return true;
}

template <typename real>
__device__ __forceinline__ void write_record(const Records<real> &rec, uint64_t i, const Photon<real> &ph,
                                             const RngAhead &g, uint32_t state, uint32_t steps, uint32_t sim) {
  rec.px[i] = ph.pos[0];
  rec.py[i] = ph.pos[1];
  rec.pz[i] = ph.pos[2];
  rec.dx[i] = ph.dir[0];
  rec.dy[i] = ph.dir[1];
  rec.dz[i] = ph.dir[2];
  rec.e[i] = ph.e;
  rec.flags[i] = state | (steps << 2);
  rec.rng_pos[i] = (g.blk << 3) | (uint32_t)g.idx;
  rec.rng_buf[i] = make_uint4(g.buf[0], g.buf[1], g.buf[2], g.buf[3]);
  rec.sim[i] = sim;
}

// Source stage: one thread per history.  Samples the primary
// (GateGenericSource::GeneratePrimaries order), places it, and performs the
// first transport iteration when the photon starts in the world (free flight
// to the image, to an air interaction, or out of the world).
// MULTI: batched simulations (Scene::sims): the thread's history picks its
// simulation, whose geometry, source and Philox key it then uses.  Without
// MULTI, isotropic directions with an acceptance loop are sampled by the
// warp together (warp_iso_direction_accepted).
template <typename real, bool MULTI>
__global__ void __launch_bounds__(256) k_generate(Scene<real> s, KernelArgs a) {
  __shared__ BlockCounters bc;
  if (threadIdx.x == 0) bc = BlockCounters{0, 0, 0, 0, 0, 0, 0, 0};
  __syncthreads();
  const uint64_t n = a.h_end - a.h_begin;
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool sampled = false, world_step = false;  // counted per block below
  // isotropic directions with an acceptance loop: the warp samples them together
  const bool warp_dirs = !MULTI && s.dir_type == GG_DIR_ISO && s.n_accept > 0;
  if (warp_dirs) {
    Records<real> rec = Records<real>::carve(a.records, a.rec_cap);
    RngAhead g;  // blocks made on demand: the warp's trials read the stream directly
    g.init(a.seed, a.h_begin + i, 0u);
    g.ahead = false;
    Photon<real> ph;
    const bool live = i < n;
    if (live) sample_position(s, g, ph, &bc);
    int st = warp_iso_direction_accepted(s, g, ph, live, &bc);
    if (live) {
      uint32_t state = kRecDead, steps = 0;
      if (st != GG_OK) {
        atomicOr(a.status, (unsigned int)st);
      } else {
        sample_energy(s, g, ph);
        sampled = true;
        start_photon(s, ph);
        world_step = first_flight(s, g, ph, state, steps, &bc);
      }
      write_record(rec, i, ph, g, state, steps, 0u);
    }
  } else if (i < n) {
    Records<real> rec = Records<real>::carve(a.records, a.rec_cap);
    RngAhead g;
    uint32_t sim = 0;
    if constexpr (MULTI) {
      const uint64_t h = a.h_begin + i;
      sim = (uint32_t)find_sim(s.sims, s.n_sims, h);
      const SimDesc<real> &d = s.sims[sim];
      bind_geometry(s, d, s.labels, s.sim_maj + (size_t)sim * s.n_e);
      bind_source(s, d);
      g.start(d.seed, h - d.h_begin, 0u);
    } else {
      g.start(a.seed, a.h_begin + i, 0u);
    }
    Photon<real> ph;
    if (s.dir_type == GG_DIR_FORCED) {  // the head (and run) the history's photon is aimed at
      const uint64_t h = a.h_begin + i;
      ph.run = s.run_base + (int)((h - s.run_first) / s.run_len);
      ph.head = (int)(h % (uint64_t)s.n_heads);
    }
    uint32_t state = kRecDead, steps = 0;
    int st = sample_primary(s, g, ph, &bc);
    if (st != GG_OK) {
      atomicOr(a.status, (unsigned int)st);
    } else {
      sampled = true;
      start_photon(s, ph);
      world_step = first_flight(s, g, ph, state, steps, &bc);
    }
    write_record(rec, i, ph, g, state, steps, sim);
  }
  const int n_hist = __syncthreads_count(sampled);
  const int n_world = __syncthreads_count(world_step);
  if (threadIdx.x == 0) {
    unsigned long long *cnt = a.counters;
    if (n_hist) atomicAdd(&cnt[GG_CNT_HISTORIES], (unsigned long long)n_hist);
    if (bc.skipped) atomicAdd(&cnt[GG_CNT_SKIPPED], (unsigned long long)bc.skipped);
    if (bc.escaped) atomicAdd(&cnt[GG_CNT_ESCAPED], (unsigned long long)bc.escaped);
    if (bc.loop_capped) atomicAdd(&cnt[GG_CNT_LOOP_CAPPED], (unsigned long long)bc.loop_capped);
    if (n_world) atomicAdd(&cnt[GG_CNT_WORLD_STEPS], (unsigned long long)n_world);
  }
}

// Transport stage.  Persistent grid; each lane carries one history at a time
// and is in one of the states kRefill (needs a history), kFly (next event is
// a flight) or kInteract (a collision is pending).  Every iteration the block
// picks ONE phase from counts of its lanes' states - refill when at least
// refill_min lanes per warp wait for a history, interact when at least
// interact_min collisions per warp are pending, otherwise fly - and only the
// lanes in that state execute it.  Expensive code (source-record loads, tally
// flushes, Compton sampling) therefore runs with many lanes active instead of
// one lane at a time, all warps of a block execute the same code region at
// the same time (the kernel is bound by instruction fetch, not arithmetic),
// and the order of operations inside each history, hence its result, is
// unchanged.
// MINB = resident blocks per SM the register budget is sized for.
// SPECT selects the head transport and projection scoring instead of the dose tally.
// DG: dose tally on a grid of its own (1: edep, 2: edep and dose), Scene::dgrid.
template <typename real, int MINB, bool SPECT, bool MULTI, bool TLE, int DG = 0>
__global__ void __launch_bounds__(256, MINB) k_transport(Scene<real> sg, KernelArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ BlockCounters bc;
  __shared__ BlockCounters bcd;  // counts of the dose list (DG 2), not reported
  __shared__ real sec_store[6 * 256];
  // ---- stage tables in shared memory --------------------------------------
  Scene<real> s = sg;
  {
    real *sh = reinterpret_cast<real *>(smem_raw);
    const int nsig = sg.n_comp * sg.n_e;
    real *ssig = sh;
    real *smaj = ssig + nsig;
    real *srho = smaj + sg.n_e;
    int *scomp = reinterpret_cast<int *>(srho + sg.n_mat);
    for (int i = threadIdx.x; i < nsig; i += blockDim.x) ssig[i] = sg.sig[i];
    for (int i = threadIdx.x; i < sg.n_e; i += blockDim.x) smaj[i] = sg.maj[i];
    for (int i = threadIdx.x; i < sg.n_mat; i += blockDim.x) {
      srho[i] = sg.mat_rho[i];
      scomp[i] = sg.mat_comp[i];
    }
    if (threadIdx.x == 0) bc = BlockCounters{0, 0, 0, 0, 0, 0, 0, 0};
    __syncthreads();
    s.sig = ssig;
    s.maj = smaj;
    s.mat_rho = srho;
    s.mat_comp = scomp;
  }
  const Records<real> rec = Records<real>::carve(args.records, args.rec_cap);
  Tally<real> t{args.acc_e, args.acc_e2};
  const Tally<real> td{args.acc_d, args.acc_d2};
  if constexpr (DG == 2) {
    if (threadIdx.x == 0) bcd = BlockCounters{0, 0, 0, 0, 0, 0, 0, 0};
  }
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  const uint64_t n_hist = args.h_end - args.h_begin;
  __shared__ uint64_t wpool[kBlock / 32][2];  // per warp: claimed histories not yet handed out
  uint64_t *pool = wpool[threadIdx.x >> 5];
  if (lane == 0) pool[0] = pool[1] = 0;
  __syncwarp();

  Photon<real> ph;
  ph.alive = 0;
  Secondary<real> sec;
  sec.base = sec_store;
  sec.stride = blockDim.x;
  sec.tid = threadIdx.x;
  sec.has = 0;
  // history lists after the tables: [list][vox | acc][kHistList][blockDim.x]
  HistList<real> l, ld;  // ld: dose list of the history (DG 2), same voxels as l
  {
    const int nt = (int)blockDim.x;
    unsigned char *lists = smem_raw + transport_smem_bytes<real>(sg.n_comp, sg.n_e, sg.n_mat);
    l.vox = reinterpret_cast<uint32_t *>(lists) + threadIdx.x;
    l.acc = reinterpret_cast<real *>(lists + (size_t)kHistList * nt * sizeof(uint32_t)) + threadIdx.x;
    l.stride = nt;
    l.n = 0;
    ld = l;
    if constexpr (DG == 2) {
      lists += hist_list_bytes<real>(1, nt);
      ld.vox = reinterpret_cast<uint32_t *>(lists) + threadIdx.x;
      ld.acc = reinterpret_cast<real *>(lists + (size_t)kHistList * nt * sizeof(uint32_t)) + threadIdx.x;
    }
  }
  Event<real> ev;
  ev.clear();
  Rng g;
  int state = kRefill;
  bool in_hist = false;
  int pmat = 0, pscored = 0;
  uint32_t pv = 0;
  unsigned int n_wood = 0, n_real = 0, n_dep = 0, n_world = 0, n_head = 0, n_singles = 0;

  for (;;) {
    // phase chosen per block: all warps run the same code region at the same
    // time (instruction-cache locality); thresholds are per warp
    const unsigned m_ref = __ballot_sync(0xffffffffu, state == kRefill);
    const int c_ref = __syncthreads_count(state == kRefill);
    const int c_fly = __syncthreads_count(state == kFly);
    const int c_int = __syncthreads_count(state == kInteract);
    if (c_ref + c_fly + c_int == 0) break;
    const int n_warps = (int)(blockDim.x >> 5);
    int phase;
    if (c_ref >= args.refill_min * n_warps || (c_fly + c_int) == 0) phase = kRefill;
    else if (c_int >= args.interact_min * n_warps || c_fly == 0) phase = kInteract;
    else phase = kFly;

    if (phase == kRefill) {
      const bool need = state == kRefill;
      if constexpr (SPECT) {
        if (need && in_hist) n_singles += score_singles(s, ev, ph.run, g);
      } else {
        // per-lane atomics: a warp-aggregated flush (same-voxel entries of the warp summed
        // first, __match_any_sync + shuffles) issued as many atomic instructions here and
        // made the transport 28 % slower, so it is not used
        if (need && in_hist) {
          hlist_flush(l, t, &bc);
          if constexpr (DG == 2) hlist_flush(ld, td, &bcd);
        }
      }
      if (need) in_hist = false;
      const uint64_t h = warp_pool_claim(pool, m_ref, lane, lt_mask, args.next, args.chunk);
      if (need) {
        if (h >= n_hist) {
          state = kDone;
        } else {
          const uint32_t f = rec.flags[h];
          const uint32_t rs = f & 3u;
          if (rs != kRecDead) {
            uint64_t hid = args.h_begin + h;
            uint64_t key = args.seed;
            if constexpr (MULTI) {
              // batched simulations: this history's geometry, majorant, tally and Philox stream
              const uint32_t k = rec.sim[h];
              const SimDesc<real> &d = sg.sims[k];
              bind_geometry(s, d, sg.labels, sg.sim_maj + (size_t)k * sg.n_e);
              t.acc_e = args.acc_e + d.vox_off;
              t.acc_e2 = args.acc_e2 ? args.acc_e2 + 2 * d.vox_off : nullptr;
              key = d.seed;
              hid = hid - d.h_begin;
            }
            ph.pos[0] = rec.px[h];
            ph.pos[1] = rec.py[h];
            ph.pos[2] = rec.pz[h];
            ph.dir[0] = rec.dx[h];
            ph.dir[1] = rec.dy[h];
            ph.dir[2] = rec.dz[h];
            set_energy(s, ph, rec.e[h]);
            ph.steps = (int)((f >> 2) & 1u);
            ph.alive = 1;
            ph.can_enter = 1;
            ph.in_head = 0;
            ph.exclude = -1;
            ph.w = s.s_fd_w;  // 1, or the forced direction's cone weight
            if constexpr (SPECT) {
              ev.clear();
              ph.run = s.run_base + (int)((hid - s.run_first) / s.run_len);
            }
            const uint32_t rp = rec.rng_pos[h];
            const uint4 b = rec.rng_buf[h];
            g.k0 = (uint32_t)key;
            g.k1 = (uint32_t)(key >> 32);
            g.stream = 0u;
            g.h0 = (uint32_t)hid;
            g.h1 = (uint32_t)(hid >> 32);
            g.blk = rp >> 3;
            g.idx = (int)(rp & 7u);
            g.buf[0] = b.x;
            g.buf[1] = b.y;
            g.buf[2] = b.z;
            g.buf[3] = b.w;
            if (rs == kRecInImage) {
              ph.in_image = 1;
              ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
              state = kFly;
            } else if (rs == kRecWorld) {
              ph.in_image = 0;
              state = kFly;
            } else {
              ph.in_image = 0;
              pmat = s.world_mat;
              pscored = 0;
              state = kInteract;
            }
            in_hist = true;
          }
        }
      }
    } else if (phase == kInteract) {
      if (state == kInteract) {
        if constexpr (DG > 0)
          state = do_interaction_grid<real, DG>(s, ph, g, &bc, pmat, pscored, l, ld, t, td, sec, n_dep, &bcd);
        else
          state = do_interaction<real, SPECT, TLE>(s, ph, g, &bc, pmat, pv, pscored, l, t, sec, n_dep, ev);
        if (state == kRefill && sec.has) {
          pop_secondary(s, ph, sec);
          state = kFly;
        }
      }
    } else {
      if (state == kFly) {
        state = flight<real, SPECT, TLE>(s, ph, g, &bc, pmat, pv, pscored, n_wood, n_real, n_world, n_head,
                                         TleScore<real>{&l, &t, &n_dep});
        if (state == kRefill && sec.has) {
          pop_secondary(s, ph, sec);
          state = kFly;
        }
      }
    }
  }
  // ---- counters -------------------------------------------------------------
  unsigned long long *cnt = args.counters;
  auto warp_add = [&](unsigned int v, int slot) {
    unsigned long long x = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0 && x) atomicAdd(&cnt[slot], x);
  };
  warp_add(n_wood, GG_CNT_WOODCOCK_STEPS);
  warp_add(n_real, GG_CNT_REAL_INTERACTIONS);
  warp_add(n_dep, GG_CNT_DEPOSITS);
  warp_add(n_world, GG_CNT_WORLD_STEPS);
  warp_add(n_head, GG_CNT_HEAD_STEPS);
  warp_add(n_singles, GG_CNT_SINGLES);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&cnt[GG_CNT_TALLY_ENTRIES], (unsigned long long)bc.tally_entries);
    atomicAdd(&cnt[GG_CNT_LIST_OVERFLOWS], (unsigned long long)bc.list_overflows);
    atomicAdd(&cnt[GG_CNT_ESCAPED], (unsigned long long)bc.escaped);
    atomicAdd(&cnt[GG_CNT_LOOP_CAPPED], (unsigned long long)bc.loop_capped);
    atomicAdd(&cnt[GG_CNT_STACK_OVERFLOW], (unsigned long long)bc.stack_overflow);
    atomicAdd(&cnt[GG_CNT_SECONDARIES], (unsigned long long)bc.secondaries);
  }
}

// Adds the per-batch fixed-point sums into the float64 images and clears them.
// scale multiplies the sums (1 for edep; 1 / rho_min for the dose tally, whose
// entries are edep * rho_min / rho), scale2 = scale^2 their squares.
__global__ void k_flush(unsigned long long *acc_e, unsigned long long *acc_e2, double *edep, double *edep2,
                        size_t n, double scale, double scale2) {
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    unsigned long long a = acc_e[i];
    if (a) {
      double v = (double)a * 2.3283064365386963e-10;
      v = v * scale;
      edep[i] += v;
      acc_e[i] = 0ull;
    }
    if (acc_e2) {
      const ulonglong2 b = reinterpret_cast<const ulonglong2 *>(acc_e2)[i];  // (low 32 bits, rest)
      if (b.x | b.y) {
        double lo = (double)b.x;
        lo = lo * 5.421010862427522e-20;  // 2^-64
        double hi = (double)b.y;
        hi = hi * 2.3283064365386963e-10;  // 2^-32
        double v = hi + lo;
        v = v * scale2;
        edep2[i] += v;
        reinterpret_cast<ulonglong2 *>(acc_e2)[i] = make_ulonglong2(0ull, 0ull);
      }
    }
  }
}


template <typename real>
size_t record_bytes(size_t cap) {
  return cap * (sizeof(uint4) + 7 * sizeof(real) + 3 * sizeof(uint32_t));
}

template <typename real>
cudaError_t launch_generate(const Scene<real> &s, const KernelArgs &a, cudaStream_t st) {
  uint64_t n = a.h_end - a.h_begin;
  unsigned int blocks = (unsigned int)((n + 255) / 256);
  if (s.n_sims > 0) k_generate<real, true><<<blocks, 256, 0, st>>>(s, a);
  else k_generate<real, false><<<blocks, 256, 0, st>>>(s, a);
  return cudaGetLastError();
}

template <typename real, int MINB, bool MULTI, bool TLE = false, int DG = 0>
static cudaError_t launch_transport_v(const Scene<real> &s, const KernelArgs &a, int grid, int block, size_t smem,
                                      cudaStream_t st) {
  static unsigned long long configured = 0;
  if (block <= 0 || block > kBlock) return cudaErrorInvalidValue;
  cudaError_t e = configure_smem(k_transport<real, MINB, false, MULTI, TLE, DG>, kTransportSmemMax, configured);
  if (e != cudaSuccess) return e;
  smem += hist_list_bytes<real>(DG == 2 ? 2 : 1, block);
  if (smem > (size_t)kTransportSmemMax) return cudaErrorInvalidValue;
  k_transport<real, MINB, false, MULTI, TLE, DG><<<grid, block, smem, st>>>(s, a);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_transport(const Scene<real> &s, const KernelArgs &a, int grid, int block, size_t smem,
                             int minb, cudaStream_t st) {
  // SPECT runs use the two-stage kernels of gg_spect.cu
  if (s.spect) return cudaErrorInvalidValue;
  if (s.dgrid) {
    // dose grid of its own (single simulations, analog scoring)
    if (s.muen || s.n_sims > 0) return cudaErrorInvalidValue;
    if (s.ddose) {
      if (minb <= 2) return launch_transport_v<real, 2, false, false, 2>(s, a, grid, block, smem, st);
      if (minb == 3) return launch_transport_v<real, 3, false, false, 2>(s, a, grid, block, smem, st);
      return launch_transport_v<real, 4, false, false, 2>(s, a, grid, block, smem, st);
    }
    if (minb <= 2) return launch_transport_v<real, 2, false, false, 1>(s, a, grid, block, smem, st);
    if (minb == 3) return launch_transport_v<real, 3, false, false, 1>(s, a, grid, block, smem, st);
    return launch_transport_v<real, 4, false, false, 1>(s, a, grid, block, smem, st);
  }
  if (s.muen) {
    // track-length estimator (single simulations only)
    if (s.n_sims > 0) return cudaErrorInvalidValue;
    if (minb <= 2) return launch_transport_v<real, 2, false, true>(s, a, grid, block, smem, st);
    if (minb == 3) return launch_transport_v<real, 3, false, true>(s, a, grid, block, smem, st);
    return launch_transport_v<real, 4, false, true>(s, a, grid, block, smem, st);
  }
  if (s.n_sims > 0) {
    if (minb <= 2) return launch_transport_v<real, 2, true>(s, a, grid, block, smem, st);
    if (minb == 3) return launch_transport_v<real, 3, true>(s, a, grid, block, smem, st);
    return launch_transport_v<real, 4, true>(s, a, grid, block, smem, st);
  }
  if (minb <= 2) return launch_transport_v<real, 2, false>(s, a, grid, block, smem, st);
  if (minb == 3) return launch_transport_v<real, 3, false>(s, a, grid, block, smem, st);
  return launch_transport_v<real, 4, false>(s, a, grid, block, smem, st);
}

cudaError_t launch_flush(unsigned long long *acc_e, unsigned long long *acc_e2, double *edep, double *edep2,
                         size_t n, int grid, cudaStream_t st, double scale) {
  k_flush<<<grid, 256, 0, st>>>(acc_e, acc_e2, edep, edep2, n, scale, scale * scale);
  return cudaGetLastError();
}

template <typename real>
cudaError_t occupancy_blocks(int block, size_t smem, int minb, int *bps) {
  smem += hist_list_bytes<real>(1, block);
  if (minb <= 2) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_transport<real, 2, false, false, false>, block, smem);
  if (minb == 3) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_transport<real, 3, false, false, false>, block, smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_transport<real, 4, false, false, false>, block, smem);
}

template size_t record_bytes<float>(size_t);
template size_t record_bytes<double>(size_t);
template cudaError_t launch_generate<float>(const Scene<float> &, const KernelArgs &, cudaStream_t);
template cudaError_t launch_generate<double>(const Scene<double> &, const KernelArgs &, cudaStream_t);
template cudaError_t launch_transport<float>(const Scene<float> &, const KernelArgs &, int, int, size_t, int,
                                             cudaStream_t);
template cudaError_t launch_transport<double>(const Scene<double> &, const KernelArgs &, int, int, size_t, int,
                                              cudaStream_t);
template cudaError_t occupancy_blocks<float>(int, size_t, int, int *);
template cudaError_t occupancy_blocks<double>(int, size_t, int, int *);

}  // namespace gg
