// gg_spect.cu - SPECT acquisition as a two-stage wavefront.
//
// A SPECT history crosses three very different kinds of geometry: the
// voxelised phantom (Woodcock steps and label gathers), the air of the world,
// and the heads (collimator hole lattice, crystal and the digitizer event).
// One kernel that carries all three keeps every warp's lanes spread over the
// three code paths.  Here the work is split by where the photon is:
//
//   * phantom stage: source records (or photons handed back by the head
//     stage) are tracked in the image and the world; a photon that reaches a
//     head box is written, with its RNG position and event, to the head queue
//     and its lane takes the next history;
//   * head stage: queued photons are tracked through collimator, gap and
//     crystal (and the world between the heads); the event is scored into the
//     projection when the photon dies; a photon that flies back into the
//     image is written to the return queue for another phantom pass.
//
// The host alternates the stages until the return queue stays empty.  Every
// photon executes the same operations in the same order as in a single
// kernel (the queues only change which lane runs them), so projections and
// counters equal those of the CPU oracle bit for bit.
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_physics.cuh"
#include "gg_queue.cuh"
#include "gg_spect.cuh"

namespace gg {

// Free-flight modes of the stages (Scene::ff).
constexpr int kFfOff = 0, kFfPrimary = 1, kFfScatter = 2;

// Phantom-stage flight: Woodcock step in the image (followed, when it leaves
// the image box, by the world step) or one world step; a photon whose world
// step ends at a head-box entry leaves the stage (kPush).  Primary free
// flight (FFM 1): one free flight to a head instead.  Scatter splitting
// (FFM 2): analog flights, and an analog photon that reaches a head is killed
// there (the heads are its kill volumes; only its split copies are detected).
template <typename real, int FFM>
__device__ __forceinline__ int phantom_flight(const Scene<real> &s, Photon<real> &ph, Rng &g, BlockCounters *bc,
                                              int &pmat, uint32_t &pv, int &pscored, unsigned int &n_wood,
                                              unsigned int &n_real, unsigned int &n_world) {
  if (++ph.steps > kStepCap) {
    atomicAdd(&bc->loop_capped, 1u);
    ph.alive = 0;
    return kRefill;
  }
  if constexpr (FFM == kFfPrimary) {  // free flight to a head: no interaction outside the heads
    // the checks here (cutoffs, angle, the head the line enters); the optical
    // depth of the photons that pass is walked by k_spect_walk, with full warps
    ++n_world;
    real tb;
    if (ff_target(s, ph, s.ss_cos, tb)) return kPush;
    atomicAdd(&bc->escaped, 1u);
    return kRefill;
  }
  if (ph.in_image) {
    const int r = image_flight(s, ph, g, pmat, pv, pscored, n_wood, n_real);
    if (r != kFly || ph.in_image) return r;
    // left the image box: the world step follows in the same iteration (same
    // flight count and draws as a separate phase)
    if (++ph.steps > kStepCap) {
      atomicAdd(&bc->loop_capped, 1u);
      ph.alive = 0;
      return kRefill;
    }
  }
  ++n_world;
  if (spect_world_flight(s, ph, g)) {
    pmat = s.world_mat;
    pscored = 0;
    return kInteract;
  }
  if (!ph.alive) {
    atomicAdd(&bc->escaped, 1u);
    return kRefill;
  }
  if constexpr (FFM == kFfScatter) {
    if (ph.in_head) {
      ph.alive = 0;
      atomicAdd(&bc->escaped, 1u);
      return kRefill;
    }
    return kFly;
  }
  return ph.in_head ? kPush : kFly;
}

// Head-stage flight: one step in a head, or one world step; a photon whose
// world step ends at the image-box entry leaves the stage (kPush).
template <typename real, bool FF>
__device__ __forceinline__ int head_stage_flight(const Scene<real> &s, Photon<real> &ph, Rng &g, BlockCounters *bc,
                                                 int &pmat, int &pscored, unsigned int &n_world,
                                                 unsigned int &n_head) {
  if (++ph.steps > kStepCap) {
    atomicAdd(&bc->loop_capped, 1u);
    ph.alive = 0;
    return kRefill;
  }
  if (ph.in_head) {
    ++n_head;
    int mat;
    if (head_flight(s, ph, g, mat)) {
      pmat = mat;
      pscored = ph.hreg == s.hreg_cr ? 2 : 3;
      return kInteract;
    }
    return ph.alive ? kFly : kRefill;  // (stopped by a shielded side)
  }
  ++n_world;
  if constexpr (FF) {  // free flight to another head (the image crossed on the way)
    if (ff_flight(s, ph, R<real>(-2))) return kFly;
    atomicAdd(&bc->escaped, 1u);
    return kRefill;
  }
  if (spect_world_flight(s, ph, g)) {
    pmat = s.world_mat;
    pscored = 0;
    return kInteract;
  }
  if (!ph.alive) {
    atomicAdd(&bc->escaped, 1u);
    return kRefill;
  }
  return ph.in_image ? kPush : kFly;
}

// Block counters and per-lane step counts into the global counters.
__device__ __forceinline__ void stage_counters(unsigned long long *cnt, const BlockCounters &bc, unsigned lane,
                                               unsigned int n_wood, unsigned int n_real, unsigned int n_world,
                                               unsigned int n_head, unsigned int n_singles) {
  auto warp_add = [&](unsigned int v, int slot) {
    unsigned long long x = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0 && x) atomicAdd(&cnt[slot], x);
  };
  warp_add(n_wood, GG_CNT_WOODCOCK_STEPS);
  warp_add(n_real, GG_CNT_REAL_INTERACTIONS);
  warp_add(n_world, GG_CNT_WORLD_STEPS);
  warp_add(n_head, GG_CNT_HEAD_STEPS);
  warp_add(n_singles, GG_CNT_SINGLES);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (bc.escaped) atomicAdd(&cnt[GG_CNT_ESCAPED], (unsigned long long)bc.escaped);
    if (bc.loop_capped) atomicAdd(&cnt[GG_CNT_LOOP_CAPPED], (unsigned long long)bc.loop_capped);
    if (bc.stack_overflow) atomicAdd(&cnt[GG_CNT_STACK_OVERFLOW], (unsigned long long)bc.stack_overflow);
    if (bc.secondaries) atomicAdd(&cnt[GG_CNT_SECONDARIES], (unsigned long long)bc.secondaries);
    if (bc.list_overflows) atomicAdd(&cnt[GG_CNT_LIST_OVERFLOWS], (unsigned long long)bc.list_overflows);
  }
}

// Whether a photon of direction d scattered by theta (cos, sin^2) can pass the
// angle check of some head (ff_target): over the azimuth, the largest cosine
// between the new direction and a head axis u is cos(theta - theta_u) =
// cos(theta) (d.u) + sin(theta) sqrt(1 - (d.u)^2).  A margin of 1e-4 on the
// cosine keeps every direction the full check would accept (rounding is far
// below it), so dropping the others changes no result.
template <typename real>
__device__ __forceinline__ bool cone_reachable(const Scene<real> &s, int run, const real d[3], real cost, real sint2,
                                               real cos_min) {
  const real sint = gg_sqrt(sint2 > R<real>(0) ? sint2 : R<real>(0));
  const real lim = cos_min - R<real>(1e-4);
  for (int h = 0; h < s.n_heads; ++h) {
    const HeadFrame<real> f = head_frame(s, run, h);
    const real c0 = dot3(d, f.u);
    real s0 = R<real>(1) - c0 * c0;
    s0 = gg_sqrt(s0 > R<real>(0) ? s0 : R<real>(0));
    real m = cost * c0;
    m = m + sint * s0;
    if (!(m < lim)) return true;
  }
  return false;
}

// Copies of one warp that passed the scattering-angle test and wait for the
// rest of their scattering and the head checks, kSplitPend at most: the copy
// index, the sampled (eps, 1 - cos, sin^2) of a Compton or (cos, -, -) of a
// Rayleigh scattering, and the words of the copy's stream drawn so far.
constexpr int kSplitPend = 64;
template <typename real>
struct SplitPending {
  uint64_t i[kSplitPend];
  real a[kSplitPend], b[kSplitPend], c[kSplitPend];
  uint32_t words[kSplitPend];
};

// Scatter splitting, the copies (GateScatterSplittingFreeFlightOptn.cpp:69-149):
// one thread per copy.  Request r of the phantom stage holds the photon
// before a Compton (or Rayleigh) interaction; its copy c re-samples that
// interaction from there on Philox stream 2 + base + c of the history, with
// 1 / n of the weight, and flies freely to a head: the intersection check of
// the angular acceptance is the flight itself (a copy that misses every head
// cannot be detected), the angle check comes before the optical depth.
// A copy whose line enters a head (past the checks) goes to the walk queue
// (q.out_q), where k_spect_walk computes its optical depth: the few copies
// that pass then walk the voxels with full warps.  Compton requests fill the
// buffer from the front and Rayleigh requests from the back; when together
// they overflowed it, nothing is done (the host repeats the pass on fewer
// histories).
// Most copies scatter away from every head: right after the rejection loop
// the scattering angle alone decides that (cone_reachable), and only the
// others draw their azimuth and meet the full check.  Those wait in a
// per-warp buffer until 32 of them fill the warp's lanes, so the azimuth,
// the rotation and the head checks run on full warps; each copy's arithmetic
// and draws are those of the plain sequence.
template <typename real>
__global__ void __launch_bounds__(256) k_spect_split(Scene<real> sg, KernelArgs args, StageArgs q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ BlockCounters bc;
  __shared__ SplitPending<real> pend_all[kBlock / 32];
  Scene<real> s = sg;
  stage_tables(sg, s, smem_raw, bc);
  const uint64_t n_c = *q.split_n, n_r = q.split_n[1];
  if (n_c + n_r > (uint64_t)q.split_cap) return;
  const uint64_t per_c = (uint64_t)s.ss_nc, per_r = (uint64_t)s.ss_nr;
  const uint64_t all_c = n_c * per_c, total = all_c + n_r * per_r;
  const SplitQueue<real> sq = SplitQueue<real>::carve(q.split_q, q.split_cap);
  const PQueue<real> out = PQueue<real>::carve(q.out_q, q.q_cap);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  SplitPending<real> &P = pend_all[threadIdx.x >> 5];
  int np = 0;  // copies waiting in P (the same in every lane of the warp)
  unsigned int n_world = 0;
  // copy i: its request, the photon before the interaction, its stream
  auto load_copy = [&](uint64_t i, Photon<real> &cp, Rng &gc, uint64_t &hid) {
    uint64_t r;
    uint32_t c, n;
    if (i < all_c) {
      r = i / per_c;
      c = (uint32_t)(i - r * per_c);
      n = (uint32_t)per_c;
    } else {
      const uint64_t j = i - all_c, rr = j / per_r;
      c = (uint32_t)(j - rr * per_r);
      r = (uint64_t)q.split_cap - 1 - rr;
      n = (uint32_t)per_r;
    }
    hid = sq.hid[r];
    cp.pos[0] = sq.px[r];
    cp.pos[1] = sq.py[r];
    cp.pos[2] = sq.pz[r];
    cp.dir[0] = sq.dx[r];
    cp.dir[1] = sq.dy[r];
    cp.dir[2] = sq.dz[r];
    cp.e = sq.e[r];  // the energy-grid state only where a sampling uses it (set_energy)
    cp.w = sq.w[r] / (real)n;
    cp.alive = 1;
    cp.run = sq.run[r];
    gc.init(args.seed, hid, 2u + sq.base[r] + c);
    return r;
  };
  // the waiting copies P[k0 + lane] (lane < cnt): the rest of the scattering,
  // the head checks, and the walk queue (every lane of the warp calls it)
  auto finish = [&](int k0, int cnt) {
    Photon<real> cp;
    Rng gc;
    uint64_t hid = 0;
    bool push = false;
    if ((int)lane < cnt) {
      const int k = k0 + (int)lane;
      const uint64_t i = P.i[k];
      load_copy(i, cp, gc, hid);
      // the stream after its first `w` words: the state an Rng reaches by drawing them
      const uint32_t w = P.words[k];
      if ((w & 3u) == 0u) {
        gc.blk = w >> 2;
        gc.idx = 4;
      } else {
        const uint4 b = philox_block(w >> 2, gc.stream, gc.h0, gc.h1, gc.k0, gc.k1);
        gc.buf[0] = b.x;
        gc.buf[1] = b.y;
        gc.buf[2] = b.z;
        gc.buf[3] = b.w;
        gc.blk = (w >> 2) + 1u;
        gc.idx = (int)(w & 3u);
      }
      if (i < all_c) compton_finish(s, cp, gc, P.a[k], P.b[k], P.c[k]);
      else rayleigh_finish(cp, gc, P.a[k]);
      if (cp.alive) {
        cp.exclude = -1;
        cp.steps = 0;
        cp.head = 0;
        cp.hreg = 0;
        ++n_world;
        real tb;
        push = ff_target(s, cp, s.ss_cos, tb) != 0;  // with the angle check of the angular acceptance
        if (!push) atomicAdd(&bc.escaped, 1u);
      }
    }
    const size_t kq = queue_claim(q.out_n, push, lane, lt_mask);
    if (push && kq < q.q_cap) {
      real v[kEvSlots];
      queue_put<real, true>(out, kq, cp, gc, hid, v, false);
    }
  };
  // the loop bound is the same for all threads of a block: queue claims stay warp-collective
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < total; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    bool wait = false;
    real a = R<real>(0), b = R<real>(0), c = R<real>(0);
    Rng gc;
    if (i < total) {
      Photon<real> cp;
      uint64_t hid;
      const uint64_t r = load_copy(i, cp, gc, hid);
      bool dead = false, out_of_cone;
      if (i < all_c) {
        compton_kn(cp.e, gc, &bc, a, b, c);
        // (below the energy cut the copy dies in compton_finish)
        dead = a * cp.e < s.e_min;
        out_of_cone = !dead && s.ss_cos > R<real>(-1) && !cone_reachable(s, cp.run, cp.dir, R<real>(1) - b, c, s.ss_cos);
      } else {
        set_energy(s, cp, cp.e);
        a = rayleigh_cost(s, sq.comp[r], cp, gc, &bc);
        out_of_cone = s.ss_cos > R<real>(-1) && !cone_reachable(s, cp.run, cp.dir, a, rayleigh_sint2(a), s.ss_cos);
      }
      if (out_of_cone) {  // a live copy that fails the head checks, as counted there
        ++n_world;
        atomicAdd(&bc.escaped, 1u);
      }
      wait = !dead && !out_of_cone;
    }
    const unsigned m = __ballot_sync(0xffffffffu, wait);
    if (wait) {
      const int k = np + __popc(m & lt_mask);
      P.i[k] = i;
      P.a[k] = a;
      P.b[k] = b;
      P.c[k] = c;
      P.words[k] = (gc.blk - 1u) * 4u + (uint32_t)gc.idx;  // (the loops drew at least one word)
    }
    np += __popc(m);
    __syncwarp();
    if (np >= 32) {
      finish(np - 32, 32);
      np -= 32;
      __syncwarp();
    }
  }
  if (np > 0) finish(0, np);
  stage_counters(args.counters, bc, lane, 0u, 0u, n_world, 0u, 0u);
}

// Label gathers in flight per lane in the walk kernel's optical depths.
constexpr int kWalkGroup = 8;

// Free flights that passed their checks (the copies of scatter splitting
// after the split kernel, the photons of primary free flight after the
// phantom stage): the whole ff_flight (its first part again, bit for bit the
// same, then the optical depth along the line), one photon per thread, so a
// warp walks 32 lines at once instead of one line among lanes that have
// finished; photons that reach their head go to the head queue.
template <typename real>
__global__ void __launch_bounds__(256) k_spect_walk(Scene<real> sg, KernelArgs args, StageArgs q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ BlockCounters bc;
  Scene<real> s = sg;
  stage_tables(sg, s, smem_raw, bc);
  const uint64_t n = min((uint64_t)*q.in_n, (uint64_t)q.q_cap);
  const PQueue<real> in = PQueue<real>::carve(q.in_q, q.q_cap);
  const PQueue<real> out = PQueue<real>::carve(q.out_q, q.q_cap);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    Photon<real> cp;
    Rng g;
    uint64_t hid = 0;
    bool push = false, has_ev = false;
    if (i < n) {
      hid = queue_get<real, true>(s, in, i, cp, g, args.seed, has_ev);
      push = ff_flight<real, kWalkGroup>(s, cp, s.ss_cos) != 0;
      if (!push) atomicAdd(&bc.escaped, 1u);
    }
    const size_t k = queue_claim(q.out_n, push, lane, lt_mask);
    if (push) {
      if (k < q.q_cap) {
        real v[kEvSlots];
        if (has_ev) load_event(in, i, v);
        queue_put<real, true>(out, k, cp, g, hid, v, has_ev);
      } else {
        atomicOr(args.status, kStatusQueueOverflow);
      }
    }
  }
  stage_counters(args.counters, bc, lane, 0u, 0u, 0u, 0u, 0u);
}

// Phantom stage.  Input: the batch's primary records (q.in_q == null) or the
// return queue; output: the head queue.  Persistent grid with the
// phase-batched lane loop of the dose transport kernel (refill / fly /
// interact, one phase per warp iteration).  FFM: free-flight mode (kFf*).
template <typename real, int MINB, int FFM>
__global__ void __launch_bounds__(256, MINB) k_spect_phantom(Scene<real> sg, KernelArgs args, StageArgs q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ BlockCounters bc;
  __shared__ real sec_store[6 * 256];
  Scene<real> s = sg;
  stage_tables(sg, s, smem_raw, bc);
  const bool from_queue = q.in_q != nullptr;
  const Records<real> rec = Records<real>::carve(args.records, args.rec_cap);
  PQueue<real> in{};
  if (from_queue) in = PQueue<real>::carve(q.in_q, q.q_cap);
  const PQueue<real> out = PQueue<real>::carve(q.out_q, q.q_cap);
  // a queue length above the capacity means entries were dropped (status
  // GG_ERR_QUEUE_OVERFLOW): never read past the capacity
  const uint64_t n_items = from_queue ? min((uint64_t)*q.in_n, (uint64_t)q.q_cap) : args.h_end - args.h_begin;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  __shared__ uint64_t wpool[kBlock / 32][2];  // per warp: claimed histories not yet handed out
  uint64_t *pool = wpool[threadIdx.x >> 5];
  if (lane == 0) pool[0] = pool[1] = 0;
  __syncwarp();

  Photon<real> ph;
  ph.alive = 0;
  ph.in_head = 0;
  ph.head = 0;
  ph.hreg = 0;
  Secondary<real> sec;
  sec.base = sec_store;
  sec.stride = blockDim.x;
  sec.tid = threadIdx.x;
  sec.has = 0;
  HistList<real> l{nullptr, nullptr, 0, 0};  // never scored here
  Tally<real> t{nullptr, nullptr};
  Event<real> ev_unused;
  Rng g;
  int state = kRefill;
  bool in_hist = false;
  // input-queue slot of the lane's photon | kHasEv when it carries an event
  // (read when the photon dies or leaves)
  __shared__ uint64_t sslot[kBlock];
  constexpr uint64_t kHasEv = 1ull << 63;
  sslot[threadIdx.x] = 0;
  int pmat = 0, pscored = 0;
  uint32_t pv = 0;
  unsigned int n_wood = 0, n_real = 0, n_dep = 0, n_world = 0, n_singles = 0;
  uint32_t nsplit = 0;  // split copies of the history so far
  int ncompt = 0;       // Compton interactions of the analog track

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
      if (need && in_hist && (sslot[threadIdx.x] & kHasEv)) {
        // a photon that came back from a head died here: score its event
        Event<real> ev;
        real v[kEvSlots];
        load_event(in, sslot[threadIdx.x] & ~kHasEv, v);
        event_from(v, ev);
        n_singles += score_singles(s, ev, ph.run, g);
      }
      if (need) in_hist = false;
      const uint64_t h = warp_pool_claim(pool, m_ref, lane, lt_mask, args.next, args.chunk);
      if (need) {
        if (h >= n_items) {
          state = kDone;
        } else if (from_queue) {
          bool has_ev;
          queue_get<real, FFM != kFfOff>(s, in, h, ph, g, args.seed, has_ev);
          sslot[threadIdx.x] = h | (has_ev ? kHasEv : 0ull);
          ph.in_head = 0;
          ph.in_image = 1;
          ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
          state = kFly;
          in_hist = true;
        } else {
          const uint64_t r = h + (args.h_begin - args.rec_first);  // record of the history
          const uint32_t f = rec.flags[r];
          const uint32_t rs = f & 3u;
          if (rs != kRecDead) {
            ph.pos[0] = rec.px[r];
            ph.pos[1] = rec.py[r];
            ph.pos[2] = rec.pz[r];
            ph.dir[0] = rec.dx[r];
            ph.dir[1] = rec.dy[r];
            ph.dir[2] = rec.dz[r];
            set_energy(s, ph, rec.e[r]);
            ph.steps = (int)((f >> 2) & 1u);
            ph.alive = 1;
            ph.can_enter = 1;
            ph.in_head = 0;
            ph.exclude = -1;
            ph.w = s.s_fd_w;  // 1, or the forced direction's cone weight
            const uint64_t hid = args.h_begin + h;
            ph.run = run_of(s, hid);
            sslot[threadIdx.x] = 0;
            nsplit = 0;
            ncompt = 0;
            rng_resume(g, args.seed, hid, rec.rng_pos[r], rec.rng_buf[r]);
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
      if constexpr (FFM == kFfScatter) {
        // GateScatterSplittingFreeFlightOptrActor.cpp:291-360: every Compton
        // up to the maximum level and every Rayleigh is split; the analog
        // photon goes on, and is killed after a Compton beyond the level
        const Photon<real> pre = ph;
        int kind = 0, n = 0;
        if (state == kInteract) {
          state = do_interaction<real, true>(s, ph, g, &bc, pmat, pv, pscored, l, t, sec, n_dep, ev_unused, &kind);
          if (kind == kCompton && s.ss_nc > 0) {
            if (++ncompt > s.ss_max) {
              ph.alive = 0;
              state = kRefill;
            } else {
              n = s.ss_nc;
            }
          } else if (kind == kRayleigh) {
            n = s.ss_nr;
          }
        }
        // the copies are made by the split kernel: one request per split interaction
        const bool req_c = n > 0 && kind == kCompton, req_r = n > 0 && kind == kRayleigh;
        const size_t kc = queue_claim(q.split_n, req_c, lane, lt_mask);
        const size_t kr = queue_claim(q.split_n + 1, req_r, lane, lt_mask);
        if (req_c || req_r) {
          // past the capacity the split kernel skips the whole buffer and the pass is repeated
          if (req_c ? kc < q.split_cap : kr < q.split_cap) {
            const size_t k = req_c ? kc : q.split_cap - 1 - kr;
            const SplitQueue<real> sq = SplitQueue<real>::carve(q.split_q, q.split_cap);
            sq.hid[k] = rng_history(g);
            sq.px[k] = pre.pos[0];
            sq.py[k] = pre.pos[1];
            sq.pz[k] = pre.pos[2];
            sq.dx[k] = pre.dir[0];
            sq.dy[k] = pre.dir[1];
            sq.dz[k] = pre.dir[2];
            sq.e[k] = pre.e;
            sq.w[k] = pre.w;
            sq.base[k] = nsplit;
            sq.comp[k] = s.mat_comp[pmat];
            sq.run[k] = ph.run;
          }
          nsplit += (uint32_t)n;
        }
        if (state == kRefill && sec.has) {
          pop_secondary(s, ph, sec);
          ncompt = 0;
          state = kFly;
        }
      } else if (state == kInteract) {
        state = do_interaction<real, true>(s, ph, g, &bc, pmat, pv, pscored, l, t, sec, n_dep, ev_unused);
        if (state == kRefill && sec.has) {
          pop_secondary(s, ph, sec);
          state = kFly;
        }
      }
    } else {
      if (state == kFly) {
        state = phantom_flight<real, FFM>(s, ph, g, &bc, pmat, pv, pscored, n_wood, n_real, n_world);
        if (state == kRefill && sec.has) {
          pop_secondary(s, ph, sec);
          state = kFly;
        }
      }
      const bool push = state == kPush;
      const size_t k = queue_claim(q.out_n, push, lane, lt_mask);
      if (push) {
        if (k < q.q_cap) {
          real v[kEvSlots];
          const uint64_t sl = sslot[threadIdx.x];
          const bool has_ev = (sl & kHasEv) != 0;
          if (has_ev) load_event(in, sl & ~kHasEv, v);
          queue_put<real, FFM != kFfOff>(out, k, ph, g, rng_history(g), v, has_ev);
        } else {
          atomicOr(args.status, kStatusQueueOverflow);
        }
        in_hist = false;
        state = kRefill;
      }
    }
  }
  stage_counters(args.counters, bc, lane, n_wood, n_real, n_world, 0u, n_singles);
}

// Head stage.  Input: the head queue; output: the return queue.  Each lane
// carries its photon's event in registers and scores it when the photon
// dies.
template <typename real, int MINB, bool FF>
__global__ void __launch_bounds__(256, MINB) k_spect_head(Scene<real> sg, KernelArgs args, StageArgs q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ BlockCounters bc;
  __shared__ real sec_store[6 * 256];
  Scene<real> s = sg;
  stage_tables(sg, s, smem_raw, bc);
  const PQueue<real> in = PQueue<real>::carve(q.in_q, q.q_cap);
  const PQueue<real> out = PQueue<real>::carve(q.out_q, q.q_cap);
  const uint64_t n_items = min((uint64_t)*q.in_n, (uint64_t)q.q_cap);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  __shared__ uint64_t wpool[kBlock / 32][2];  // per warp: claimed histories not yet handed out
  uint64_t *pool = wpool[threadIdx.x >> 5];
  if (lane == 0) pool[0] = pool[1] = 0;
  __syncwarp();

  Photon<real> ph;
  ph.alive = 0;
  ph.run = 0;
  Secondary<real> sec;
  sec.base = sec_store;
  sec.stride = blockDim.x;
  sec.tid = threadIdx.x;
  sec.has = 0;
  HistList<real> l{nullptr, nullptr, 0, 0};  // never scored here
  Tally<real> t{nullptr, nullptr};
  Event<real> ev;
  ev.clear();
  Rng g;
  int state = kRefill;
  bool in_hist = false;
  int pmat = 0, pscored = 0;
  uint32_t pv = 0;
  unsigned int n_dep = 0, n_world = 0, n_head = 0, n_singles = 0;

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
      if (need && in_hist) {
        n_singles += score_singles(s, ev, ph.run, g);
        in_hist = false;
      }
      const uint64_t h = warp_pool_claim(pool, m_ref, lane, lt_mask, args.next, args.chunk);
      if (need) {
        if (h >= n_items) {
          state = kDone;
        } else {
          bool has_ev;
          queue_get<real, FF>(s, in, h, ph, g, args.seed, has_ev);
          if (has_ev) {
            real v[kEvSlots];
            load_event(in, h, v);
            event_from(v, ev);
          } else {
            ev.clear();
          }
          ph.in_head = 1;
          ph.in_image = 0;
          state = kFly;
          in_hist = true;
        }
      }
    } else if (phase == kInteract) {
      if (state == kInteract) {
        state = do_interaction<real, true>(s, ph, g, &bc, pmat, pv, pscored, l, t, sec, n_dep, ev);
        if (state == kRefill && sec.has) {
          pop_secondary(s, ph, sec);
          state = kFly;
        }
      }
    } else {
      if (state == kFly) {
        state = head_stage_flight<real, FF>(s, ph, g, &bc, pmat, pscored, n_world, n_head);
        if (state == kRefill && sec.has) {
          pop_secondary(s, ph, sec);
          state = kFly;
        }
      }
      const bool push = state == kPush;
      const size_t k = queue_claim(q.out_n, push, lane, lt_mask);
      if (push) {
        if (k < q.q_cap) {
          real v[kEvSlots];
          event_to(ev, v);
          queue_put<real, FF>(out, k, ph, g, rng_history(g), v, true);
        } else {
          atomicOr(args.status, kStatusQueueOverflow);
        }
        in_hist = false;
        state = kRefill;
      }
    }
  }
  stage_counters(args.counters, bc, lane, 0u, 0u, n_world, n_head, n_singles);
}

// MINB / HMINB: register budgets (resident 256-thread blocks per SM) of the
// phantom and the head stage.
template <typename real, int MINB, int FFM = kFfOff, int HMINB = MINB>
static cudaError_t launch_stage_v(int stage, const Scene<real> &s, const KernelArgs &a, const StageArgs &q, int grid,
                                  int block, size_t smem, cudaStream_t st) {
  constexpr bool FF = FFM != kFfOff;
  static unsigned long long configured[2] = {0, 0};
  cudaError_t e = stage == 0 ? configure_smem(k_spect_phantom<real, MINB, FFM>, 200 * 1024, configured[0])
                             : configure_smem(k_spect_head<real, HMINB, FF>, 200 * 1024, configured[1]);
  if (e != cudaSuccess) return e;
  if (stage == 0) k_spect_phantom<real, MINB, FFM><<<grid, block, smem, st>>>(s, a, q);
  else k_spect_head<real, HMINB, FF><<<grid, block, smem, st>>>(s, a, q);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_spect_stage(int stage, const Scene<real> &s, const KernelArgs &a, const StageArgs &q, int grid,
                               int block, size_t smem, int minb, cudaStream_t st) {
  // free flight: one register budget (4 blocks of 256 threads per SM); a
  // smaller grid computed for another budget is a valid launch of it
  // the splitting loop keeps the photon before the interaction live: the
  // scatter-splitting phantom stage gets the 3-block register budget (80
  // registers, no spills; 15 % faster than 2 blocks at 90)
  if (s.ff == kFfScatter) return launch_stage_v<real, 3, kFfScatter, 4>(stage, s, a, q, grid, block, smem, st);
  if (s.ff) return launch_stage_v<real, 4, kFfPrimary>(stage, s, a, q, grid, block, smem, st);
  if (minb <= 2) return launch_stage_v<real, 2>(stage, s, a, q, grid, block, smem, st);
  if (minb == 3) return launch_stage_v<real, 3>(stage, s, a, q, grid, block, smem, st);
  return launch_stage_v<real, 4>(stage, s, a, q, grid, block, smem, st);
}

template <typename real, int MINB>
static cudaError_t stage_occupancy_v(int stage, int block, size_t smem, int *bps) {
  return stage == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_spect_phantom<real, MINB, kFfOff>, block, smem)
                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_spect_head<real, MINB, false>, block, smem);
}

template <typename real>
cudaError_t spect_stage_occupancy(int stage, int block, size_t smem, int minb, int *blocks_per_sm) {
  if (minb <= 2) return stage_occupancy_v<real, 2>(stage, block, smem, blocks_per_sm);
  if (minb == 3) return stage_occupancy_v<real, 3>(stage, block, smem, blocks_per_sm);
  return stage_occupancy_v<real, 4>(stage, block, smem, blocks_per_sm);
}

template <typename real>
cudaError_t launch_spect_split(const Scene<real> &s, const KernelArgs &a, const StageArgs &q, int block, size_t smem,
                               int n_sm, cudaStream_t st) {
  static unsigned long long configured = 0;
  cudaError_t e = configure_smem(k_spect_split<real>, 200 * 1024, configured);
  int bps = 1;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_spect_split<real>, block, smem);
  if (e != cudaSuccess) return e;
  if (bps < 1) bps = 1;
  k_spect_split<real><<<n_sm * bps, block, smem, st>>>(s, a, q);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_spect_walk(const Scene<real> &s, const KernelArgs &a, const StageArgs &q, int block, size_t smem,
                              int n_sm, cudaStream_t st) {
  static unsigned long long configured = 0;
  cudaError_t e = configure_smem(k_spect_walk<real>, 200 * 1024, configured);
  int bps = 1;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_spect_walk<real>, block, smem);
  if (e != cudaSuccess) return e;
  if (bps < 1) bps = 1;
  k_spect_walk<real><<<n_sm * bps, block, smem, st>>>(s, a, q);
  return cudaGetLastError();
}

template cudaError_t launch_spect_walk<float>(const Scene<float> &, const KernelArgs &, const StageArgs &, int,
                                              size_t, int, cudaStream_t);
template cudaError_t launch_spect_walk<double>(const Scene<double> &, const KernelArgs &, const StageArgs &, int,
                                               size_t, int, cudaStream_t);
template size_t split_bytes<float>(size_t);
template size_t split_bytes<double>(size_t);
template cudaError_t launch_spect_split<float>(const Scene<float> &, const KernelArgs &, const StageArgs &, int,
                                               size_t, int, cudaStream_t);
template cudaError_t launch_spect_split<double>(const Scene<double> &, const KernelArgs &, const StageArgs &, int,
                                                size_t, int, cudaStream_t);
template size_t queue_bytes<float>(size_t);
template size_t queue_bytes<double>(size_t);
template cudaError_t launch_spect_stage<float>(int, const Scene<float> &, const KernelArgs &, const StageArgs &, int,
                                               int, size_t, int, cudaStream_t);
template cudaError_t launch_spect_stage<double>(int, const Scene<double> &, const KernelArgs &, const StageArgs &,
                                                int, int, size_t, int, cudaStream_t);
template cudaError_t spect_stage_occupancy<float>(int, int, size_t, int, int *);
template cudaError_t spect_stage_occupancy<double>(int, int, size_t, int, int *);

}  // namespace gg
