// gg_wavefront.cu - dose transport as a per-block wavefront compacted by event type.
//
// The same transport as k_transport (GateImageNestedParameterisation::
// ComputeMaterial stepping and GateDoseActor scoring, see gg_transport.cu),
// scheduled differently.  Each 256-thread block owns 256 photon slots whose
// whole state - position, direction, energy index, Philox stream position,
// pending interaction, the history's voxel list and the waiting annihilation
// photon - lives in shared memory.  Slots wait in queues by their next event
// (flight step, Compton, other interaction, secondary pop, new history); a
// warp takes up to 32 slots of one queue, so its lanes run one code path, and
// the warps of a block work independently of each other (no block barrier).
//
// Each history still runs the exact operation sequence of k_transport and of
// the oracle: the first draw of an interaction (the process selection,
// select_kind) is taken at the end of the flight that found it, which is the
// same position of the stream; deposits go to the same per-history list and
// the same fixed-point tallies.  Results are bit-identical to k_transport.
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_physics.cuh"

namespace gg {

namespace {

enum : int { kWFly = 0, kWCompton = 1, kWOther = 2, kWPop = 3, kWRefill = 4, kWCodes = 5 };
constexpr int kWSlots = 256;  // slots per block = threads per block
// slot flags
enum : uint32_t { kFInImage = 1u, kFCanEnter = 2u, kFHasHist = 4u, kFSec = 8u };

// Structure-of-arrays views of the slots in shared memory.
template <typename real>
struct Slots {
  real *px, *py, *pz, *dx, *dy, *dz, *e, *fe, *mumax, *inv_mumax, *t_exit;
  real *hacc;  // [kHistList][kWSlots]
  real *sec;   // [6][kWSlots]: waiting annihilation photon (pos, dir)
  int *ie, *steps;
  uint32_t *flags, *rpos, *rb, *h0, *h1, *pv, *pend, *hn, *hvox;  // rb [4][S], hvox [kHistList][S]

  static constexpr size_t bytes() {
    // reals: 11 photon fields, the voxel-list sums, the secondary's 6; 32-bit words: ie, steps,
    // flags, rpos, h0, h1, pv, pend, hn, rb[4], the voxel-list indices
    return (size_t)kWSlots * ((11 + kHistList + 6) * sizeof(real) + (13 + kHistList) * 4);
  }
  __device__ static Slots carve(unsigned char *p) {
    Slots s;
    real *r = reinterpret_cast<real *>(p);
    real **rf[11] = {&s.px, &s.py, &s.pz, &s.dx, &s.dy, &s.dz, &s.e, &s.fe, &s.mumax, &s.inv_mumax, &s.t_exit};
    for (int i = 0; i < 11; ++i) *rf[i] = r + i * kWSlots;
    s.hacc = r + 11 * kWSlots;
    s.sec = s.hacc + kHistList * kWSlots;
    uint32_t *u = reinterpret_cast<uint32_t *>(s.sec + 6 * kWSlots);
    s.ie = reinterpret_cast<int *>(u);
    s.steps = reinterpret_cast<int *>(u + kWSlots);
    uint32_t **uf[6] = {&s.flags, &s.rpos, &s.h0, &s.h1, &s.pv, &s.pend};
    for (int i = 0; i < 6; ++i) *uf[i] = u + (2 + i) * kWSlots;
    s.hn = u + 8 * kWSlots;
    s.rb = u + 9 * kWSlots;  // 4 rows
    s.hvox = u + 13 * kWSlots;
    return s;
  }
};

template <typename real>
__device__ __forceinline__ void load_photon(const Slots<real> &S, int k, Photon<real> &ph) {
  ph.pos[0] = S.px[k];
  ph.pos[1] = S.py[k];
  ph.pos[2] = S.pz[k];
  ph.dir[0] = S.dx[k];
  ph.dir[1] = S.dy[k];
  ph.dir[2] = S.dz[k];
  ph.e = S.e[k];
  ph.ei.ie = S.ie[k];
  ph.ei.fe = S.fe[k];
  ph.mumax = S.mumax[k];
  ph.inv_mumax = S.inv_mumax[k];
  ph.t_exit = S.t_exit[k];
  const uint32_t f = S.flags[k];
  ph.in_image = (f & kFInImage) ? 1 : 0;
  ph.can_enter = (f & kFCanEnter) ? 1 : 0;
  ph.steps = S.steps[k];
  ph.alive = 1;
  ph.in_head = 0;
  ph.exclude = -1;
  ph.w = R<real>(1);
}

// flags keep the history / secondary bits of the slot
template <typename real>
__device__ __forceinline__ uint32_t photon_flags(const Photon<real> &ph, uint32_t f) {
  f &= ~(kFInImage | kFCanEnter);
  if (ph.in_image) f |= kFInImage;
  if (ph.can_enter) f |= kFCanEnter;
  return f;
}

template <typename real>
__device__ __forceinline__ void store_photon(const Slots<real> &S, int k, const Photon<real> &ph, uint32_t f) {
  S.px[k] = ph.pos[0];
  S.py[k] = ph.pos[1];
  S.pz[k] = ph.pos[2];
  S.dx[k] = ph.dir[0];
  S.dy[k] = ph.dir[1];
  S.dz[k] = ph.dir[2];
  S.e[k] = ph.e;
  S.ie[k] = ph.ei.ie;
  S.fe[k] = ph.ei.fe;
  S.mumax[k] = ph.mumax;
  S.inv_mumax[k] = ph.inv_mumax;
  S.t_exit[k] = ph.t_exit;
  S.flags[k] = photon_flags(ph, f);
  S.steps[k] = ph.steps;
}

template <typename real>
__device__ __forceinline__ void load_rng(const Slots<real> &S, int k, uint64_t key, Rng &g) {
  g.k0 = (uint32_t)key;
  g.k1 = (uint32_t)(key >> 32);
  g.stream = 0u;
  g.h0 = S.h0[k];
  g.h1 = S.h1[k];
  const uint32_t rp = S.rpos[k];
  g.blk = rp >> 3;
  g.idx = (int)(rp & 7u);
#pragma unroll
  for (int j = 0; j < 4; ++j) g.buf[j] = S.rb[j * kWSlots + k];
}

template <typename real>
__device__ __forceinline__ void store_rng(const Slots<real> &S, int k, const Rng &g) {
  S.rpos[k] = (g.blk << 3) | (uint32_t)g.idx;
#pragma unroll
  for (int j = 0; j < 4; ++j) S.rb[j * kWSlots + k] = g.buf[j];
}

// The voxel list of slot k, in place in the slot arrays.
template <typename real>
__device__ __forceinline__ void load_hist(const Slots<real> &S, int k, HistList<real> &l) {
  l.vox = S.hvox + k;
  l.acc = S.hacc + k;
  l.stride = kWSlots;
  l.n = (int)S.hn[k];
}

template <typename real>
__device__ __forceinline__ void store_hist(const Slots<real> &S, int k, const HistList<real> &l) {
  S.hn[k] = (uint32_t)l.n;
}

// pending interaction word: material | scored << 16 | kind << 24
__device__ __forceinline__ uint32_t pack_pending(int pmat, int pscored, int kind) {
  return (uint32_t)pmat | ((uint32_t)pscored << 16) | ((uint32_t)kind << 24);
}

__device__ __forceinline__ int code_of_kind(int kind) { return kind == kCompton ? kWCompton : kWOther; }

// Per-event work of one slot; returns the slot's next queue (-1: the batch
// is exhausted and the slot is done).  `h` is the history offset a refill
// item takes.
template <typename real>
__device__ __forceinline__ int wf_process(int code, int slot, uint64_t h, const Scene<real> &s, const Slots<real> &S,
                                          const Records<real> &rec, const Tally<real> &tally, uint64_t key,
                                          uint64_t h_begin, uint64_t n_hist, BlockCounters *bc, unsigned int &n_wood,
                                          unsigned int &n_real, unsigned int &n_dep, unsigned int &n_world) {
  unsigned int n_head = 0;
  if (code == kWFly) {
    // ---- one flight step (Woodcock in the image, or the world step) ----------
    Photon<real> ph;
    load_photon(S, slot, ph);
    Rng g;
    load_rng(S, slot, key, g);
    int pmat = 0, pscored = 0;
    uint32_t pv = 0;
    int nc;
    const int r = flight<real, false, false>(s, ph, g, bc, pmat, pv, pscored, n_wood, n_real, n_world, n_head);
    const uint32_t f = S.flags[slot];
    if (r == kInteract) {
      const int kind = select_kind(s, ph, pmat, g);
      S.pend[slot] = pack_pending(pmat, pscored, kind);
      S.pv[slot] = pv;
      nc = code_of_kind(kind);
    } else {
      nc = r == kFly ? kWFly : ((f & kFSec) ? kWPop : kWRefill);
    }
    S.px[slot] = ph.pos[0];
    S.py[slot] = ph.pos[1];
    S.pz[slot] = ph.pos[2];
    S.t_exit[slot] = ph.t_exit;
    S.flags[slot] = photon_flags(ph, f);
    S.steps[slot] = ph.steps;
    store_rng(S, slot, g);
    return nc;
  }
  if (code == kWCompton || code == kWOther) {
    // ---- the pending interaction (do_interaction of the dose path) -----------
    Photon<real> ph;
    load_photon(S, slot, ph);
    Rng g;
    load_rng(S, slot, key, g);
    HistList<real> l;
    load_hist(S, slot, l);
    uint32_t f = S.flags[slot];
    const uint32_t pd = S.pend[slot];
    const int pmat = (int)(pd & 0xffffu), pscored = (int)((pd >> 16) & 0xffu), kind = (int)(pd >> 24);
    Secondary<real> sec;
    sec.base = S.sec;
    sec.stride = kWSlots;
    sec.tid = slot;
    sec.has = (f & kFSec) ? 1 : 0;
    const real ed = apply_kind(s, ph, pmat, kind, g, bc, sec);
    if (pscored == 1) {
      deposit(l, tally, bc, S.pv[slot], ed, n_dep);
      if (ph.alive && ph.in_image) ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
    } else if (pscored == 0) {
      ph.can_enter = 1;
    }
    f = sec.has ? (f | kFSec) : (f & ~kFSec);
    store_photon(S, slot, ph, f);
    store_rng(S, slot, g);
    store_hist(S, slot, l);
    return ph.alive ? kWFly : (sec.has ? kWPop : kWRefill);
  }
  if (code == kWPop) {
    // ---- the waiting annihilation photon continues the history --------------
    Photon<real> ph;
    ph.can_enter = 1;  // start_photon sets it for a photon outside the image
    Secondary<real> sec;
    sec.base = S.sec;
    sec.stride = kWSlots;
    sec.tid = slot;
    sec.has = 1;
    pop_secondary(s, ph, sec);
    store_photon(S, slot, ph, S.flags[slot] & ~kFSec);
    return kWFly;
  }
  // ---- end of history: flush its voxel list, start history h -----------------
  if (S.flags[slot] & kFHasHist) {
    HistList<real> l;
    load_hist(S, slot, l);
    hlist_flush(l, tally, bc);
    S.hn[slot] = 0u;
  }
  if (h >= n_hist) {
    S.flags[slot] = 0u;
    return -1;  // the batch is exhausted: the slot is done
  }
  const uint32_t rf = rec.flags[h];
  const uint32_t rs = rf & 3u;
  if (rs == kRecDead) {
    S.flags[slot] = 0u;
    return kWRefill;  // no primary (source sampling failed): take another history
  }
  const uint64_t hid = h_begin + h;
  Photon<real> ph;
  ph.pos[0] = rec.px[h];
  ph.pos[1] = rec.py[h];
  ph.pos[2] = rec.pz[h];
  ph.dir[0] = rec.dx[h];
  ph.dir[1] = rec.dy[h];
  ph.dir[2] = rec.dz[h];
  set_energy(s, ph, rec.e[h]);
  ph.steps = (int)((rf >> 2) & 1u);
  ph.alive = 1;
  ph.can_enter = 1;
  ph.in_head = 0;
  ph.exclude = -1;
  ph.w = R<real>(1);
  Rng g;
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
  int nc;
  if (rs == kRecInImage) {
    ph.in_image = 1;
    ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
    nc = kWFly;
  } else if (rs == kRecWorld) {
    ph.in_image = 0;
    ph.t_exit = R<real>(0);
    nc = kWFly;
  } else {
    // a world interaction is pending: its process is the next draw
    ph.in_image = 0;
    ph.t_exit = R<real>(0);
    const int kind = select_kind(s, ph, s.world_mat, g);
    S.pend[slot] = pack_pending(s.world_mat, 0, kind);
    nc = code_of_kind(kind);
  }
  S.h0[slot] = g.h0;
  S.h1[slot] = g.h1;
  store_photon(S, slot, ph, kFHasHist);
  store_rng(S, slot, g);
  return nc;
}

constexpr uint32_t kWEmpty = 0xffffu;          // free entry of a queue ring
constexpr unsigned int kWSpinCap = 1u << 22;   // bounded waits (entry publication, the pool lock)
constexpr unsigned int kWIdleCap = 1u << 24;   // empty polls of a warp while other warps hold every slot

// Queue rings hold 16-bit slot indices, two per 32-bit word.  Entry i is
// written only while it is free and taken (read and freed) in one atomic
// step, so every appended slot is taken exactly once however the warps'
// appends and takes interleave around the ring (a queue is a bag: which
// taker gets which of its slots does not matter).  Both wait, boundedly, for
// the other side: a taker for an entry whose appender reserved it but has not
// written it yet, an appender for an entry whose taker has reserved but not
// yet freed it.  Returns the slot (put: the slot written), or -1 when the wait
// ran out.
__device__ __forceinline__ int ring_take(uint32_t *words, int i) {
  uint32_t *w = words + (i >> 1);
  const int sh = (i & 1) * 16;
  uint32_t old = *(volatile uint32_t *)w;
  for (unsigned int k = 0; k < kWSpinCap; ++k) {
    const uint32_t v = (old >> sh) & 0xffffu;
    if (v != kWEmpty) {
      const uint32_t prev = atomicCAS(w, old, old | (kWEmpty << sh));
      if (prev == old) return (int)v;
      old = prev;
    } else {
      __nanosleep(32);
      old = *(volatile uint32_t *)w;
    }
  }
  return -1;
}

__device__ __forceinline__ int ring_put(uint32_t *words, int i, int slot) {
  uint32_t *w = words + (i >> 1);
  const int sh = (i & 1) * 16;
  uint32_t old = *(volatile uint32_t *)w;
  for (unsigned int k = 0; k < kWSpinCap; ++k) {
    if (((old >> sh) & 0xffffu) == kWEmpty) {
      const uint32_t nw = (old & ~(0xffffu << sh)) | ((uint32_t)slot << sh);
      const uint32_t prev = atomicCAS(w, old, nw);
      if (prev == old) return slot;
      old = prev;
    } else {
      __nanosleep(32);
      old = *(volatile uint32_t *)w;
    }
  }
  return -1;
}

}  // namespace

// The wavefront transport of one tally batch (plain dose: single simulation,
// analog scoring).  Persistent grid of 256-thread blocks; the warps of a
// block share the block's slots through five ring queues in shared memory
// (one per next event) and never wait for each other at a barrier: a warp
// takes up to 32 slots from one queue (a queue holding a full warp's worth
// first, in the order refill, Compton, other, pop, flight; else the longest),
// runs that event for them, and appends each slot to the queue of its next
// event.  A slot's state is written before its queue entry is published
// (block-scope fences), and every wait for another warp is bounded: when one
// runs out the block stops and the status word reports it.
template <typename real, int MINB>
__global__ void __launch_bounds__(kWSlots, MINB) k_wavefront(Scene<real> sg, KernelArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ BlockCounters bc;
  __shared__ int q_head[kWCodes], q_tail[kWCodes];   // monotonic take / append counters
  __shared__ uint32_t q_ent[kWCodes][kWSlots / 2];   // rings of 16-bit slot indices
  __shared__ int live;                               // slots not done
  __shared__ int pool_lock;
  __shared__ unsigned long long pool_next, pool_end;  // the block's claimed, unused history offsets
  __shared__ unsigned int stop;                      // a bounded wait ran out
  // ---- tables in shared memory (as k_transport) ------------------------------
  Scene<real> s = sg;
  size_t table_bytes;
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
    s.sig = ssig;
    s.maj = smaj;
    s.mat_rho = srho;
    s.mat_comp = scomp;
    table_bytes = (sizeof(real) * ((size_t)nsig + sg.n_e + sg.n_mat) + sizeof(int) * (size_t)sg.n_mat + 15) &
                  ~(size_t)15;
  }
  const Slots<real> S = Slots<real>::carve(smem_raw + table_bytes);
  const int t = (int)threadIdx.x;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  // every slot starts in the refill queue, without a history
  S.flags[t] = 0u;
  S.hn[t] = 0u;
  if (t < kWSlots / 2) {
#pragma unroll
    for (int k = 0; k < kWCodes; ++k)
      q_ent[k][t] = k == kWRefill ? ((uint32_t)(2 * t) | ((uint32_t)(2 * t + 1) << 16)) : (kWEmpty | (kWEmpty << 16));
  }
  if (t < kWCodes) {
    q_head[t] = 0;
    q_tail[t] = t == kWRefill ? kWSlots : 0;
  }
  if (t == 0) {
    bc = BlockCounters{0, 0, 0, 0, 0, 0, 0, 0};
    live = kWSlots;
    pool_lock = 0;
    pool_next = 0;
    pool_end = 0;
    stop = 0u;
  }
  __syncthreads();

  const Records<real> rec = Records<real>::carve(args.records, args.rec_cap);
  const Tally<real> tally{args.acc_e, args.acc_e2};
  const uint64_t n_hist = args.h_end - args.h_begin;
  const uint64_t key = args.seed;
  const uint64_t chunk = (uint64_t)(args.chunk > 0 ? args.chunk : 256) * 16u;
  volatile int *vhead = q_head, *vtail = q_tail;
  unsigned int n_wood = 0, n_real = 0, n_dep = 0, n_world = 0;
  unsigned int idle = 0;

  for (;;) {
    if (*(volatile unsigned int *)&stop) break;
    // ---- choose a queue: a full warp's worth in priority order, else the longest
    int avail = 0;
    if (lane < kWCodes) avail = vtail[lane] - vhead[lane];
    const unsigned full = __ballot_sync(0xffffffffu, lane < kWCodes && avail >= 32);
    int code, have;
    if (full) {
      code = (full & (1u << kWRefill))    ? kWRefill
             : (full & (1u << kWCompton)) ? kWCompton
             : (full & (1u << kWOther))   ? kWOther
             : (full & (1u << kWPop))     ? kWPop
                                          : kWFly;
      have = 32;
    } else {
      int best = avail, bcode = (int)lane;
#pragma unroll
      for (int o = 4; o > 0; o >>= 1) {
        const int ob = __shfl_down_sync(0xffffffffu, best, o);
        const int oc = __shfl_down_sync(0xffffffffu, bcode, o);
        if (ob > best) best = ob, bcode = oc;
      }
      code = __shfl_sync(0xffffffffu, bcode, 0);
      have = __shfl_sync(0xffffffffu, best, 0);
    }
    if (have <= 0) {
      if (*(volatile int *)&live == 0 || *(volatile unsigned int *)&stop) break;
      if (++idle > kWIdleCap) {
        if (lane == 0) {
          atomicOr(&stop, 1u);
          atomicOr(args.status, kStatusWaitTimeout);
        }
        break;
      }
      __nanosleep(64);
      continue;
    }
    idle = 0;
    // ---- take up to 32 entries from the head of the queue ------------------
    int h0 = 0, n = 0;
    if (lane == 0) {
      const int hd = vhead[code];
      const int tl = vtail[code];
      n = min(32, tl - hd);
      if (n > 0 && atomicCAS(&q_head[code], hd, hd + n) != hd) n = 0;  // another warp took them: choose again
      h0 = hd;
    }
    n = __shfl_sync(0xffffffffu, n, 0);
    h0 = __shfl_sync(0xffffffffu, h0, 0);
    if (n <= 0) continue;
    int slot = -1;
    if ((int)lane < n) {
      slot = ring_take(q_ent[code], (h0 + (int)lane) & (kWSlots - 1));
      if (slot < 0) {
        atomicOr(&stop, 1u);
        atomicOr(args.status, kStatusWaitTimeout);
      }
      __threadfence_block();  // the slot's state is read after its entry
    }
    // ---- histories for refills: the block's pool, then a new chunk ----------
    uint64_t h = 0;
    if (code == kWRefill) {
      unsigned long long base_pool = 0, base_new = 0;
      int from_pool = 0;
      if (lane == 0) {
        unsigned int k = 0;
        while (atomicCAS(&pool_lock, 0, 1) != 0 && k < kWSpinCap) {
          __nanosleep(32);
          ++k;
        }
        if (k >= kWSpinCap) {
          atomicOr(&stop, 1u);
          atomicOr(args.status, kStatusWaitTimeout);
          from_pool = -1;
        } else {
          volatile unsigned long long *pn = &pool_next, *pe = &pool_end;
          const uint64_t a = *pe - *pn;
          base_pool = *pn;
          if (a >= (uint64_t)n) {
            from_pool = n;
            *pn = base_pool + (uint64_t)n;
          } else {
            const uint64_t need = (uint64_t)n - a;
            const uint64_t take = need > chunk ? need : chunk;
            base_new = atomicAdd(args.next, (unsigned long long)take);
            from_pool = (int)a;
            *pn = base_new + need;
            *pe = base_new + take;
          }
          __threadfence_block();
          atomicExch(&pool_lock, 0);
        }
      }
      from_pool = __shfl_sync(0xffffffffu, from_pool, 0);
      base_pool = __shfl_sync(0xffffffffu, base_pool, 0);
      base_new = __shfl_sync(0xffffffffu, base_new, 0);
      if (from_pool < 0) slot = -1;
      h = (int)lane < from_pool ? base_pool + lane : base_new + (uint64_t)((int)lane - from_pool);
    }
    // ---- the event, then the slot to its next queue --------------------------
    int nc = -1;
    if (slot >= 0)
      nc = wf_process(code, slot, h, s, S, rec, tally, key, args.h_begin, n_hist, &bc, n_wood, n_real, n_dep,
                      n_world);
    __threadfence_block();  // the slot's state is written before its entry
    const unsigned grp = __match_any_sync(0xffffffffu, nc);
    if (nc >= 0) {
      const int leader = __ffs(grp) - 1;
      int base = 0;
      if ((int)lane == leader) base = atomicAdd(&q_tail[nc], __popc(grp));
      base = __shfl_sync(grp, base, leader);
      if (ring_put(q_ent[nc], (base + __popc(grp & lt_mask)) & (kWSlots - 1), slot) < 0) {
        atomicOr(&stop, 1u);
        atomicOr(args.status, kStatusWaitTimeout);
      }
    } else if (slot >= 0) {
      atomicSub(&live, 1);
    }
    __syncwarp();
  }
  // ---- counters ---------------------------------------------------------------
  unsigned long long *cnt = args.counters;
  auto warp_add = [&](unsigned int v, int k) {
    unsigned long long x = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0 && x) atomicAdd(&cnt[k], x);
  };
  warp_add(n_wood, GG_CNT_WOODCOCK_STEPS);
  warp_add(n_real, GG_CNT_REAL_INTERACTIONS);
  warp_add(n_dep, GG_CNT_DEPOSITS);
  warp_add(n_world, GG_CNT_WORLD_STEPS);
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

template <typename real>
size_t wavefront_smem_bytes(int n_comp, int n_e, int n_mat) {
  return transport_smem_bytes<real>(n_comp, n_e, n_mat) + Slots<real>::bytes();
}

template <typename real, int MINB>
static cudaError_t launch_wavefront_v(const Scene<real> &s, const KernelArgs &a, int grid, size_t smem,
                                      cudaStream_t st) {
  static unsigned long long configured = 0;
  cudaError_t e = configure_smem(k_wavefront<real, MINB>, 220 * 1024, configured);
  if (e != cudaSuccess) return e;
  k_wavefront<real, MINB><<<grid, kWSlots, smem, st>>>(s, a);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_wavefront(const Scene<real> &s, const KernelArgs &a, int grid, size_t smem, int minb,
                             cudaStream_t st) {
  if (s.spect || s.muen || s.n_sims > 0) return cudaErrorInvalidValue;
  if (minb <= 2) return launch_wavefront_v<real, 2>(s, a, grid, smem, st);
  return launch_wavefront_v<real, 3>(s, a, grid, smem, st);
}

template <typename real>
cudaError_t wavefront_occupancy(size_t smem, int minb, int *bps) {
  static unsigned long long c2 = 0, c3 = 0;
  cudaError_t e = minb <= 2 ? configure_smem(k_wavefront<real, 2>, 220 * 1024, c2)
                            : configure_smem(k_wavefront<real, 3>, 220 * 1024, c3);
  if (e != cudaSuccess) return e;
  if (minb <= 2) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_wavefront<real, 2>, kWSlots, smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_wavefront<real, 3>, kWSlots, smem);
}

template size_t wavefront_smem_bytes<float>(int, int, int);
template size_t wavefront_smem_bytes<double>(int, int, int);
template cudaError_t launch_wavefront<float>(const Scene<float> &, const KernelArgs &, int, size_t, int,
                                             cudaStream_t);
template cudaError_t launch_wavefront<double>(const Scene<double> &, const KernelArgs &, int, size_t, int,
                                              cudaStream_t);
template cudaError_t wavefront_occupancy<float>(size_t, int, int *);
template cudaError_t wavefront_occupancy<double>(size_t, int, int *);

}  // namespace gg
