// gg_arf.cu - ARF (angular response function) training rows on the GPU.
//
// Replaces the ARF training-dataset simulation of the reference
// (GateARFTrainingDatasetActor, core/opengate_core/opengate_lib/
// GateARFTrainingDatasetActor.cpp:76-137, with the plane source of
// contrib/spect/ge_discovery_nm670.py:994-1027): photons start on the
// collimator front face of one head, are tracked through collimator and
// crystal by the same head transport as the SPECT head stage, and each gives
// the row (E, theta, phi, w) - energy and direction at the face, and the last
// energy window containing the event's crystal energy (+1; 0 = none).  Rows
// with w = 0 are kept with probability 1 / russian_roulette.
//
// Rows come out in sample order (bit-reproducible for a seed): one kernel
// tracks one sample per thread into a staging row and counts the kept rows of
// its block, one kernel turns the block counts into offsets, and one kernel
// compacts the kept rows.
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_physics.cuh"
#include "gg_spect.cuh"

namespace gg {

constexpr float kRadToDeg = 57.295779513082320876f;

template <typename real>
__global__ void __launch_bounds__(256) k_arf_sample(Scene<real> s, ArfArgs p) {
  __shared__ BlockCounters bc;
  __shared__ real sec_store[6 * 256];
  __shared__ unsigned int n_head, n_singles;
  if (threadIdx.x == 0) {
    bc = BlockCounters{0, 0, 0, 0, 0, 0, 0, 0};
    n_head = 0;
    n_singles = 0;
  }
  __syncthreads();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool keep = false;
  if (i < p.n) {
    Rng g;
    g.init(p.seed, p.first + i, 1u);
    Photon<real> ph;
    const real hx = (real)p.half_extent[0], hy = (real)p.half_extent[1];
    real u = R<real>(2) * u01<real>(g);
    u = u - R<real>(1);
    ph.pos[0] = u * hx;
    u = R<real>(2) * u01<real>(g);
    u = u - R<real>(1);
    ph.pos[1] = u * hy;
    ph.pos[2] = R<real>(0);
    real ct, st;
    if (p.theta_uniform) {
      const real f = u01<real>(g) * (real)p.theta_max_turn;
      gg_sincos_turn(f, st, ct);
    } else {
      real w = R<real>(1) - (real)p.cos_theta_max;
      w = u01<real>(g) * w;
      ct = R<real>(1) - w;
      real st2 = ct * ct;
      st2 = R<real>(1) - st2;
      st = gg_sqrt(st2 > R<real>(0) ? st2 : R<real>(0));
    }
    real sp, cp;
    gg_sincos_turn(u01<real>(g), sp, cp);
    ph.dir[0] = st * cp;
    ph.dir[1] = st * sp;
    ph.dir[2] = ct;
    real de = (real)p.e_max - (real)p.e_min;
    de = de * u01<real>(g);
    const real e = (real)p.e_min + de;
    float4 row;
    row.x = (float)e;
    row.y = acosf((float)ph.dir[2]) * kRadToDeg;
    row.z = atan2f((float)ph.dir[1], (float)ph.dir[0]) * kRadToDeg;
    set_energy(s, ph, e);
    ph.alive = 1;
    ph.in_head = 1;
    ph.in_image = 0;
    ph.head = 0;
    ph.hreg = 0;
    ph.left_hole = 0;
    ph.exclude = -1;
    ph.run = 0;
    ph.w = R<real>(1);
    ph.steps = 0;
    Secondary<real> sec;
    sec.base = sec_store;
    sec.stride = blockDim.x;
    sec.tid = threadIdx.x;
    sec.has = 0;
    HistList<real> l{nullptr, nullptr, 0, 0};  // never scored here
    Tally<real> t{nullptr, nullptr};
    Event<real> ev;
    ev.clear();
    unsigned int steps = 0, n_dep = 0;
    while (ph.alive && ph.in_head) {
      if (++ph.steps > kStepCap) {
        atomicAdd(&bc.loop_capped, 1u);
        break;
      }
      ++steps;
      int mat;
      if (head_flight(s, ph, g, mat))
        do_interaction<real, true>(s, ph, g, &bc, mat, 0u, ph.hreg == s.hreg_cr ? 2 : 3, l, t, sec, n_dep, ev);
    }
    atomicAdd(&n_head, steps);
    int label = 0;
    real ed = ev.esum[0];
    if (ed > R<real>(0)) {
      atomicAdd(&n_singles, 1u);
      if (s.eblur) ed = blur_energy(s, ed, g);  // the window the digitizer chain reports
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (k < s.n_win && ed >= s.wlo[k] && ed < s.whi[k]) label = k + 1;
    }
    row.w = (float)label;
    keep = true;
    if (label == 0) {
      const real r = u01<real>(g) * (real)p.russian_roulette;
      keep = r < R<real>(1);
    }
    if (!keep) row.w = -1.0f;
    p.stage[i] = row;
  }
  const int kept = __syncthreads_count(keep ? 1 : 0);
  if (threadIdx.x == 0) {
    p.block_count[blockIdx.x] = (unsigned int)kept;
    unsigned long long *cnt = p.counters;
    if (n_head) atomicAdd(&cnt[GG_CNT_HEAD_STEPS], (unsigned long long)n_head);
    if (n_singles) atomicAdd(&cnt[GG_CNT_SINGLES], (unsigned long long)n_singles);
    if (bc.loop_capped) atomicAdd(&cnt[GG_CNT_LOOP_CAPPED], (unsigned long long)bc.loop_capped);
  }
}

// Exclusive prefix of the per-block kept counts (one block; the counts of one
// call are at most a few ten thousand).
__global__ void k_arf_offsets(const unsigned int *block_count, unsigned long long *block_off, unsigned int n_blocks,
                              unsigned long long *total) {
  __shared__ unsigned long long part[1024];
  const unsigned int per = (n_blocks + blockDim.x - 1) / blockDim.x;
  const unsigned int b0 = threadIdx.x * per;
  unsigned long long sum = 0;
  for (unsigned int b = b0; b < b0 + per && b < n_blocks; ++b) sum += block_count[b];
  part[threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long run = *total;
    for (unsigned int k = 0; k < blockDim.x; ++k) {
      const unsigned long long v = part[k];
      part[k] = run;
      run += v;
    }
    *total = run;
  }
  __syncthreads();
  unsigned long long off = part[threadIdx.x];
  for (unsigned int b = b0; b < b0 + per && b < n_blocks; ++b) {
    block_off[b] = off;
    off += block_count[b];
  }
}

// Kept rows to their place: block offset + rank of the row inside its block.
__global__ void __launch_bounds__(256) k_arf_compact(const float4 *stage, const unsigned long long *block_off,
                                                     uint64_t n, float4 *rows, uint64_t capacity) {
  __shared__ unsigned int warp_base[8];
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float4 r = make_float4(0.f, 0.f, 0.f, -1.f);
  if (i < n) r = stage[i];
  const bool keep = i < n && r.w >= 0.0f;
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  if (lane == 0) warp_base[warp] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int run = 0;
    for (int k = 0; k < 8; ++k) {
      const unsigned int v = warp_base[k];
      warp_base[k] = run;
      run += v;
    }
  }
  __syncthreads();
  if (keep) {
    const uint64_t dst = block_off[blockIdx.x] + warp_base[warp] + __popc(m & ((1u << lane) - 1u));
    if (dst < capacity) rows[dst] = r;
  }
}

template <typename real>
cudaError_t launch_arf_dataset(const Scene<real> &s, const ArfArgs &p, float4 *rows, uint64_t capacity,
                               unsigned long long *total, cudaStream_t st) {
  const unsigned int blocks = (unsigned int)((p.n + 255) / 256);
  if (blocks == 0) return cudaSuccess;
  k_arf_sample<real><<<blocks, 256, 0, st>>>(s, p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_arf_offsets<<<1, 1024, 0, st>>>(p.block_count, p.block_off, blocks, total);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_arf_compact<<<blocks, 256, 0, st>>>(p.stage, p.block_off, p.n, rows, capacity);
  return cudaGetLastError();
}

template cudaError_t launch_arf_dataset<float>(const Scene<float> &, const ArfArgs &, float4 *, uint64_t,
                                               unsigned long long *, cudaStream_t);
template cudaError_t launch_arf_dataset<double>(const Scene<double> &, const ArfArgs &, float4 *, uint64_t,
                                                unsigned long long *, cudaStream_t);

}  // namespace gg
