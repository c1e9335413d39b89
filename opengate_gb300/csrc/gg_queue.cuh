// gg_queue.cuh - photon queues between wavefront stages (device side).
//
// A queue entry is a photon in flight with everything needed to continue
// its history in another kernel: position, direction, energy, the history id
// and the position in its Philox stream, the step count, head state and the
// digitizer event of the history so far.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_physics.cuh"
#include "gg_spect.cuh"

namespace gg {

// Photons handed between the stages, SoA.  meta: bits 0-19 steps taken,
// bit 20 head, bits 21-22 head region, bit 23 event present, bits 24-26
// exclude + 1.  ev: esum[2], emax[2], wpos[2][2], w[2] of the history's
// event; w: the photon's weight (free flight).
constexpr int kEvSlots = 10;
template <typename real>
struct PQueue {
  uint4 *rng_buf;
  unsigned long long *hid;
  real *px, *py, *pz, *dx, *dy, *dz, *e, *w;
  real *ev[kEvSlots];
  uint32_t *rng_pos, *meta;
  uint32_t *stream;  // Philox stream of the photon (split copies; free flight only)

  __device__ __forceinline__ static PQueue carve(void *base, size_t cap) {
    PQueue q;
    unsigned char *p = reinterpret_cast<unsigned char *>(base);
    q.rng_buf = reinterpret_cast<uint4 *>(p);
    p += cap * sizeof(uint4);
    q.hid = reinterpret_cast<unsigned long long *>(p);
    p += cap * sizeof(unsigned long long);
    real **f[8] = {&q.px, &q.py, &q.pz, &q.dx, &q.dy, &q.dz, &q.e, &q.w};
    for (int i = 0; i < 8; ++i) {
      *f[i] = reinterpret_cast<real *>(p);
      p += cap * sizeof(real);
    }
    for (int i = 0; i < kEvSlots; ++i) {
      q.ev[i] = reinterpret_cast<real *>(p);
      p += cap * sizeof(real);
    }
    q.rng_pos = reinterpret_cast<uint32_t *>(p);
    p += cap * sizeof(uint32_t);
    q.meta = reinterpret_cast<uint32_t *>(p);
    p += cap * sizeof(uint32_t);
    q.stream = reinterpret_cast<uint32_t *>(p);
    return q;
  }
};

template <typename real>
size_t queue_bytes(size_t cap) {
  return cap * (sizeof(uint4) + sizeof(unsigned long long) + (8 + kEvSlots) * sizeof(real) + 3 * sizeof(uint32_t));
}

// Split requests of scatter splitting (phantom stage -> split kernel), SoA:
// the photon before the interaction (position, direction, energy, weight),
// its history, the stream offset of its first copy, the composition of the
// material (Rayleigh form factors) and the history's gantry position.
template <typename real>
struct SplitQueue {
  unsigned long long *hid;
  real *px, *py, *pz, *dx, *dy, *dz, *e, *w;
  uint32_t *base;
  int32_t *comp;
  int32_t *run;  // gantry position of the history

  __device__ __forceinline__ static SplitQueue carve(void *b, size_t cap) {
    SplitQueue q;
    unsigned char *p = reinterpret_cast<unsigned char *>(b);
    q.hid = reinterpret_cast<unsigned long long *>(p);
    p += cap * sizeof(unsigned long long);
    real **f[8] = {&q.px, &q.py, &q.pz, &q.dx, &q.dy, &q.dz, &q.e, &q.w};
    for (int i = 0; i < 8; ++i) {
      *f[i] = reinterpret_cast<real *>(p);
      p += cap * sizeof(real);
    }
    q.base = reinterpret_cast<uint32_t *>(p);
    p += cap * sizeof(uint32_t);
    q.comp = reinterpret_cast<int32_t *>(p);
    p += cap * sizeof(int32_t);
    q.run = reinterpret_cast<int32_t *>(p);
    return q;
  }
};

template <typename real>
size_t split_bytes(size_t cap) {
  return cap * (sizeof(unsigned long long) + 8 * sizeof(real) + 3 * sizeof(uint32_t));
}

constexpr uint32_t kMetaSteps = (1u << 20) - 1u;
// meta word above the step count: head (bit 20), head slab (3 bits from 21:
// up to kHeadRegions slabs), event flag (bit 24), exclude + 1 (from bit 25)
constexpr int kMetaHead = 20, kMetaReg = 21, kMetaEv = 24, kMetaExcl = 25;
static_assert(kHeadRegions <= 8, "the head slab index has 3 bits in the queue meta word");
static_assert(kStepCap <= (int)kMetaSteps, "the step count has 20 bits in the queue meta word");
constexpr int kPush = 4;  // lane state: photon leaves this stage through the output queue

// Tables of the block in shared memory (majorant, attenuation rows, label ->
// composition / density), as in the dose transport kernel.
template <typename real>
__device__ __forceinline__ void stage_tables(const Scene<real> &sg, Scene<real> &s, unsigned char *smem_raw,
                                             BlockCounters &bc) {
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

__device__ __forceinline__ void rng_resume(Rng &g, uint64_t seed, uint64_t hid, uint32_t rp, uint4 b,
                                           uint32_t stream = 0u) {
  g.k0 = (uint32_t)seed;
  g.k1 = (uint32_t)(seed >> 32);
  g.stream = stream;
  g.h0 = (uint32_t)hid;
  g.h1 = (uint32_t)(hid >> 32);
  g.blk = rp >> 3;
  g.idx = (int)(rp & 7u);
  g.buf[0] = b.x;
  g.buf[1] = b.y;
  g.buf[2] = b.z;
  g.buf[3] = b.w;
}

// The history of a resumed stream: its counter words (rng_resume sets both from it).
__device__ __forceinline__ uint64_t rng_history(const Rng &g) { return ((uint64_t)g.h1 << 32) | (uint64_t)g.h0; }

template <typename real>
__device__ __forceinline__ int run_of(const Scene<real> &s, uint64_t hid) {
  return s.run_base + (int)((hid - s.run_first) / s.run_len);
}

// Writes the lane's photon (and event) to slot k of the output queue; the
// weight only with free flight (FF), where it can differ from 1.
template <typename real, bool FF = true>
__device__ __forceinline__ void queue_put(const PQueue<real> &q, size_t k, const Photon<real> &ph, const Rng &g,
                                          uint64_t hid, const real ev[kEvSlots], bool has_ev) {
  q.rng_buf[k] = make_uint4(g.buf[0], g.buf[1], g.buf[2], g.buf[3]);
  q.rng_pos[k] = (g.blk << 3) | (uint32_t)g.idx;
  q.hid[k] = hid;
  q.px[k] = ph.pos[0];
  q.py[k] = ph.pos[1];
  q.pz[k] = ph.pos[2];
  q.dx[k] = ph.dir[0];
  q.dy[k] = ph.dir[1];
  q.dz[k] = ph.dir[2];
  q.e[k] = ph.e;
  if constexpr (FF) {
    q.w[k] = ph.w;
    q.stream[k] = g.stream;
  }
  if (has_ev) {
#pragma unroll
    for (int i = 0; i < kEvSlots; ++i) q.ev[i][k] = ev[i];
  }
  q.meta[k] = ((uint32_t)ph.steps & kMetaSteps) | ((uint32_t)ph.head << kMetaHead) |
              ((uint32_t)ph.hreg << kMetaReg) | ((has_ev ? 1u : 0u) << kMetaEv) |
              ((uint32_t)(ph.exclude + 1) << kMetaExcl);
}

// Reads slot k of an input queue into the lane (photon state as it was when
// it entered the queue: at a head-box entry in head-local coordinates, or at
// an image-box entry in world coordinates).
template <typename real, bool FF = true>
__device__ __forceinline__ uint64_t queue_get(const Scene<real> &s, const PQueue<real> &q, size_t k, Photon<real> &ph,
                                              Rng &g, uint64_t seed, bool &has_ev) {
  const uint64_t hid = q.hid[k];
  rng_resume(g, seed, hid, q.rng_pos[k], q.rng_buf[k], FF ? q.stream[k] : 0u);
  ph.pos[0] = q.px[k];
  ph.pos[1] = q.py[k];
  ph.pos[2] = q.pz[k];
  ph.dir[0] = q.dx[k];
  ph.dir[1] = q.dy[k];
  ph.dir[2] = q.dz[k];
  set_energy(s, ph, q.e[k]);
  if constexpr (FF) ph.w = q.w[k];
  else ph.w = R<real>(1);
  const uint32_t m = q.meta[k];
  ph.steps = (int)(m & kMetaSteps);
  ph.head = (int)((m >> kMetaHead) & 1u);
  ph.hreg = (int)((m >> kMetaReg) & 7u);
  has_ev = ((m >> kMetaEv) & 1u) != 0u;
  ph.exclude = (int)((m >> kMetaExcl) & 7u) - 1;
  ph.alive = 1;
  ph.can_enter = 1;
  ph.left_hole = 0;
  ph.run = run_of(s, hid);
  return hid;
}

// Per-warp slot allocation in an output queue for the lanes with `push` set;
// returns the lane's slot (meaningful only where push is set).
__device__ __forceinline__ size_t queue_claim(unsigned long long *count, bool push, unsigned lane, unsigned lt_mask) {
  const unsigned m = __ballot_sync(0xffffffffu, push);
  unsigned long long base = 0;
  if (m) {
    if (lane == (unsigned)(__ffs(m) - 1)) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
  }
  return (size_t)(base + __popc(m & lt_mask));
}

template <typename real>
__device__ __forceinline__ void load_event(const PQueue<real> &q, size_t k, real ev[kEvSlots]) {
#pragma unroll
  for (int i = 0; i < kEvSlots; ++i) ev[i] = q.ev[i][k];
}

template <typename real>
__device__ __forceinline__ void event_from(const real v[kEvSlots], Event<real> &ev) {
  ev.esum[0] = v[0];
  ev.esum[1] = v[1];
  ev.emax[0] = v[2];
  ev.emax[1] = v[3];
  ev.wpos[0][0] = v[4];
  ev.wpos[0][1] = v[5];
  ev.wpos[1][0] = v[6];
  ev.wpos[1][1] = v[7];
  ev.w[0] = v[8];
  ev.w[1] = v[9];
}

template <typename real>
__device__ __forceinline__ void event_to(const Event<real> &ev, real v[kEvSlots]) {
  v[0] = ev.esum[0];
  v[1] = ev.esum[1];
  v[2] = ev.emax[0];
  v[3] = ev.emax[1];
  v[4] = ev.wpos[0][0];
  v[5] = ev.wpos[0][1];
  v[6] = ev.wpos[1][0];
  v[7] = ev.wpos[1][1];
  v[8] = ev.w[0];
  v[9] = ev.w[1];
}

}  // namespace gg
