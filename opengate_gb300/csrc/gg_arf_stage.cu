// gg_arf_stage.cu - ARF stage of the SPECT wavefront.
//
// Replaces GateARFActor::SteppingAction + ARFActor.apply /
// arf_build_image_from_projected_points (core/opengate_core/opengate_lib/
// GateARFActor.cpp:60-113, opengate/actors/arfactors.py:349-415): a photon
// that reaches a head's collimator face is not tracked through the head;
// the network gives its probability for every energy window, and the
// probabilities are added to the projection at the point where its line
// crosses the crystal plane (distance_to_crystal behind the face).
//
// Input is the head queue of the phantom stage.  Per photon:
//   * energy below every window: dropped (no window can be reached);
//   * entering through the collimator face, energy and angle inside the
//     trained domain, no crystal event yet: handled by the network;
//   * otherwise (side entry, outside the domain): copied to the fallback
//     queue, which the plain head stage tracks - the plain path both covers
//     and bounds what the network does not know.
// Each warpgroup of a CTA runs its own pipeline over tiles of 128 queued
// photons, one photon per thread (classify, network forward on tcgen05 from
// the CTA's shared weights - gg_mlp_tc.cuh -, softmax, scatter) with
// named-barrier synchronisation inside the group only, so the groups overlap
// one another's MMAs and epilogues.  Window weights are w_k = p_k / (RR p_0 +
// sum_k>0 p_k) (class 0 re-weighted by the Russian roulette of its training
// rows), times the photon's weight with free flight (the expected detection
// of a photon that got there with probability w), and go to fixed-point
// projection tallies (2^-32 units, with the exact
// square for the history-by-history variance), so projections are
// bit-reproducible.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_mlp.cuh"
#include "gg_mlp_tc.cuh"
#include "gg_physics.cuh"
#include "gg_queue.cuh"
#include "gg_spect.cuh"

namespace gg {

constexpr float kArfRadToDeg = 57.295779513082320876f;

template <typename real>
__device__ __forceinline__ void queue_copy(const PQueue<real> &in, size_t k, const PQueue<real> &out, size_t j) {
  out.rng_buf[j] = in.rng_buf[k];
  out.hid[j] = in.hid[k];
  out.px[j] = in.px[k];
  out.py[j] = in.py[k];
  out.pz[j] = in.pz[k];
  out.dx[j] = in.dx[k];
  out.dy[j] = in.dy[k];
  out.dz[j] = in.dz[k];
  out.e[j] = in.e[k];
  out.w[j] = in.w[k];
#pragma unroll
  for (int i = 0; i < kEvSlots; ++i) out.ev[i][j] = in.ev[i][k];
  out.rng_pos[j] = in.rng_pos[k];
  out.stream[j] = in.stream[k];
  out.meta[j] = in.meta[k];
}

enum : int { kArfNone = 0, kArfNet = 1, kArfFallback = 2 };

template <typename real>
__global__ void __launch_bounds__(kTcThreads, 1) k_spect_arf(Scene<real> s, ArfStageArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcNetSmem &sm = *reinterpret_cast<TcNetSmem *>(smem_raw);
  __shared__ unsigned int n_net, n_fb;
  if (threadIdx.x == 0) {
    n_net = 0;
    n_fb = 0;
  }
  const bool ready = tc_net_prepare(sm, a.params, a.wbf + kTcBf);

  const PQueue<real> in = PQueue<real>::carve(a.in_q, a.q_cap);
  const PQueue<real> out = PQueue<real>::carve(a.out_q, a.q_cap);
  const uint64_t n_items = min((uint64_t)*a.in_n, (uint64_t)a.q_cap);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int g = threadIdx.x >> 7, r = threadIdx.x & 127, bar = 1 + g;
  const size_t plane = (size_t)s.pny * s.pnx;
  uint32_t phase = 0;
  unsigned int my_net = 0, my_fb = 0;

  if (!ready && threadIdx.x == 0) atomicOr(a.status, kStatusWaitTimeout);
  for (;;) {
    if (!ready) break;
    // ---- claim a tile of 128 queued photons for the group ----
    if (r == 0) sm.claim[g] = atomicAdd(a.claim, (unsigned long long)kTcRows);
    named_bar(bar, kTcRows);
    const unsigned long long base = sm.claim[g];
    if (base >= n_items) break;
    // ---- classify (one photon per thread) ----
    const uint64_t k = base + r;
    int mode = kArfNone;
    float x0 = 0.f, x1 = 0.f, x2 = 0.f;
    float wph = 1.0f;  // the photon's free-flight weight (1 without free flight)
    long long p_off = -1;
    if (k < n_items) {
      const uint32_t meta = in.meta[k];
      const bool has_ev = ((meta >> kMetaEv) & 1u) != 0u;
      const real e = in.e[k];
      const real lz = in.pz[k];
      const real dz = in.dz[k];
      if (has_ev) {
        mode = kArfFallback;
      } else if (e < (real)a.e_detect_min) {
        mode = kArfNone;
      } else if (lz < (real)1e-3 && dz > (real)0 && e >= (real)a.e_min && e <= (real)a.e_max &&
                 dz >= (real)a.cos_theta_max) {
        mode = kArfNet;
        if (s.ff) wph = (float)in.w[k];
        const real dx = in.dx[k], dy = in.dy[k];
        const float th = acosf((float)dz) * kArfRadToDeg;
        const float ph = atan2f((float)dy, (float)dx) * kArfRadToDeg;
        x0 = (th - a.mean[0]) * a.inv_std[0];
        x1 = (ph - a.mean[1]) * a.inv_std[1];
        x2 = ((float)e - a.mean[2]) * a.inv_std[2];
        // the photon's line at the crystal plane (head-local)
        real t = (real)a.dc / dz;
        real u = in.px[k] + t * dx;
        real v = in.py[k] + t * dy;
        real fx = u + s.pix_half[0];
        fx = fx * s.inv_psp[0];
        real fy = v + s.pix_half[1];
        fy = fy * s.inv_psp[1];
        if (fx >= (real)0 && fx < (real)s.pnx && fy >= (real)0 && fy < (real)s.pny) {
          const int i = (int)fx, j = (int)fy;
          const int head = (int)((meta >> kMetaHead) & 1u);
          const int run = run_of(s, in.hid[k]);
          p_off = (long long)((((size_t)head * s.n_runs + run) * s.n_win) * plane + (size_t)j * s.pnx + i);
        }
      } else {
        mode = kArfFallback;
      }
    }
    const bool fb = mode == kArfFallback;
    const size_t slot = queue_claim(a.out_n, fb, lane, lt_mask);
    if (fb) {
      if (slot < a.q_cap) queue_copy(in, k, out, slot);
      else atomicOr(a.status, kStatusQueueOverflow);
      ++my_fb;
    }
    if (mode == kArfNet) ++my_net;
    // skip the network when no photon of the tile is scored
    if (!named_bar_any(bar, kTcRows, p_off >= 0)) continue;
    // ---- network (tensor cores) ----
    float p[16];
    if (!tc_net_forward(sm, g, r, phase, x0, x1, x2, p)) {
      if (r == 0) atomicOr(a.status, kStatusWaitTimeout);
      break;
    }
    // ---- window weights into the projection tallies ----
    if (p_off >= 0) {
      tc_softmax(p, a.n_classes);
      float norm = p[0] * a.rr;
#pragma unroll
      for (int c = 1; c < 16; ++c)
        if (c < a.n_classes) norm += p[c];
      const float inv = norm > 0.0f ? 1.0f / norm : 0.0f;
#pragma unroll
      for (int c = 1; c < 16; ++c) {
        if (c >= a.n_classes) break;
        const unsigned long long q = __float2ull_rn(((p[c] * inv) * wph) * 4294967296.0f);
        if (!q) continue;
        const size_t idx = (size_t)p_off + (size_t)(c - 1) * plane;
        atomicAdd(a.proj + idx, q);
        const unsigned long long lo = q * q;
        const unsigned long long rest = (__umul64hi(q, q) << 32) | (lo >> 32);
        if (lo & 0xffffffffull) atomicAdd(a.proj2 + 2 * idx, lo & 0xffffffffull);
        if (rest) atomicAdd(a.proj2 + 2 * idx + 1, rest);
      }
    }
  }
  if (my_net) atomicAdd(&n_net, my_net);
  if (my_fb) atomicAdd(&n_fb, my_fb);
  tc_net_teardown(sm);
  if (threadIdx.x == 0) {
    if (n_net) atomicAdd(&a.counters[GG_CNT_ARF_PHOTONS], (unsigned long long)n_net);
    if (n_fb) atomicAdd(&a.counters[GG_CNT_ARF_FALLBACK], (unsigned long long)n_fb);
  }
}

template <typename real>
cudaError_t launch_spect_arf(const Scene<real> &s, const ArfStageArgs &a, int grid, cudaStream_t st) {
  static unsigned long long configured = 0;
  cudaError_t e = configure_smem(k_spect_arf<real>, (int)sizeof(TcNetSmem), configured);
  if (e != cudaSuccess) return e;
  k_spect_arf<real><<<grid, kTcThreads, sizeof(TcNetSmem), st>>>(s, a);
  return cudaGetLastError();
}

template cudaError_t launch_spect_arf<float>(const Scene<float> &, const ArfStageArgs &, int, cudaStream_t);
template cudaError_t launch_spect_arf<double>(const Scene<double> &, const ArfStageArgs &, int, cudaStream_t);

}  // namespace gg
