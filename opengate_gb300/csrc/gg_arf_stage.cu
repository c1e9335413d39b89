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
// Each warp of a CTA runs its own pipeline over chunks of 32 queued photons
// (classify, layer 1 on the CUDA cores, layers 2-4 on the tensor cores from
// the CTA's shared weights, softmax, scatter) with warp-level
// synchronisation only.  Window weights are w_k = p_k / (RR p_0 +
// sum_k>0 p_k) (class 0 re-weighted by the Russian roulette of its training
// rows) and go to fixed-point projection tallies (2^-32 units, with the exact
// square for the history-by-history variance), so projections are
// bit-reproducible.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_mlp.cuh"
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
#pragma unroll
  for (int i = 0; i < 8; ++i) out.ev[i][j] = in.ev[i][k];
  out.rng_pos[j] = in.rng_pos[k];
  out.meta[j] = in.meta[k];
}

enum : int { kArfNone = 0, kArfNet = 1, kArfFallback = 2 };

constexpr int kArfWarps = 8;      // warps per CTA, each an independent 32-photon pipeline
constexpr int kArfRows = 32;      // photons per warp chunk

// Shared memory of the ARF stage: the network's weights once per CTA, and
// per warp two BF16 activation buffers (ping-pong between layers), the
// chunk's inputs and projection offsets.
struct ArfSmem {
  __nv_bfloat16 w2[kHid * kLds], w3[kHid * kLds], w4[kOutPad * kLds];
  float w1[kHid * 3], b1[kHid], b2[kHid], b3[kHid], b4[kOutPad];
  __nv_bfloat16 act[kArfWarps][2][kArfRows * kLds];
  float x[kArfWarps][kArfRows][3];
  long long pix[kArfWarps][kArfRows];  // projection offset of window 1, -1: not scored
};

// One hidden layer for the warp's 32 rows: out = bf16(relu(in W^T + b)).
__device__ __forceinline__ void arf_hidden(const __nv_bfloat16 *in, const __nv_bfloat16 *w, const float *b,
                                           __nv_bfloat16 *out) {
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float acc[2][8][4];
    zero_acc(acc);
    warp_gemm<2, 8, false, false>(acc, in, kLds, 0, w, kLds, 64 * half, kHid);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          int rr, cc;
          acc_pos(q, rr, cc);
          const int col = 64 * half + 8 * nt + cc;
          const float z = acc[mt][nt][q] + b[col];
          out[(16 * mt + rr) * kLds + col] = __float2bfloat16_rn(z > 0.0f ? z : 0.0f);
        }
  }
}

template <typename real>
__global__ void __launch_bounds__(kArfWarps * 32) k_spect_arf(Scene<real> s, ArfStageArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ArfSmem &sm = *reinterpret_cast<ArfSmem *>(smem_raw);
  __shared__ unsigned int n_net, n_fb;
  if (threadIdx.x == 0) {
    n_net = 0;
    n_fb = 0;
  }
  for (int e = threadIdx.x; e < kHid * kHid; e += blockDim.x) {
    const int row = e / kHid, col = e % kHid;
    sm.w2[row * kLds + col] = a.wbf[kBfW2 + e];
    sm.w3[row * kLds + col] = a.wbf[kBfW3 + e];
  }
  for (int e = threadIdx.x; e < kOutPad * kHid; e += blockDim.x) {
    const int row = e / kHid, col = e % kHid;
    sm.w4[row * kLds + col] = a.wbf[kBfW4 + e];
  }
  for (int e = threadIdx.x; e < kHid * 3; e += blockDim.x) sm.w1[e] = a.params[kOffW1 + e];
  for (int e = threadIdx.x; e < kHid; e += blockDim.x) {
    sm.b1[e] = a.params[kOffB1 + e];
    sm.b2[e] = a.params[kOffB2 + e];
    sm.b3[e] = a.params[kOffB3 + e];
  }
  for (int e = threadIdx.x; e < kOutPad; e += blockDim.x) sm.b4[e] = a.params[kOffB4 + e];
  __syncthreads();

  const PQueue<real> in = PQueue<real>::carve(a.in_q, a.q_cap);
  const PQueue<real> out = PQueue<real>::carve(a.out_q, a.q_cap);
  const uint64_t n_items = min((uint64_t)*a.in_n, (uint64_t)a.q_cap);
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  const size_t plane = (size_t)s.pny * s.pnx;
  __nv_bfloat16 *buf0 = sm.act[warp][0], *buf1 = sm.act[warp][1];
  float (*x)[3] = sm.x[warp];
  long long *pix = sm.pix[warp];
  unsigned int my_net = 0, my_fb = 0;

  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(a.claim, (unsigned long long)kArfRows);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n_items) break;
    // ---- classify the chunk (one photon per lane) ----
    const uint64_t k = base + lane;
    int mode = kArfNone;
    float x0 = 0.f, x1 = 0.f, x2 = 0.f;
    long long p_off = -1;
    if (k < n_items) {
      const uint32_t meta = in.meta[k];
      const bool has_ev = ((meta >> 23) & 1u) != 0u;
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
          const int head = (int)((meta >> 20) & 1u);
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
    x[lane][0] = x0;
    x[lane][1] = x1;
    x[lane][2] = x2;
    pix[lane] = p_off;
    // skip the network when no photon of the chunk is scored
    if (__ballot_sync(0xffffffffu, p_off >= 0) == 0u) continue;
    __syncwarp();
    // ---- layer 1 (CUDA cores) ----
    for (int e = lane; e < kArfRows * kHid; e += 32) {
      const int r = e / kHid, j = e % kHid;
      float z = sm.b1[j];
      z = fmaf(sm.w1[3 * j + 0], x[r][0], z);
      z = fmaf(sm.w1[3 * j + 1], x[r][1], z);
      z = fmaf(sm.w1[3 * j + 2], x[r][2], z);
      buf0[r * kLds + j] = __float2bfloat16_rn(z > 0.0f ? z : 0.0f);
    }
    __syncwarp();
    arf_hidden(buf0, sm.w2, sm.b2, buf1);
    __syncwarp();
    arf_hidden(buf1, sm.w3, sm.b3, buf0);
    __syncwarp();
    // ---- output layer + softmax, probabilities to buf1 (FP32 [32][16]) ----
    float *prob = reinterpret_cast<float *>(buf1);
    {
      float acc[2][2][4];
      zero_acc(acc);
      warp_gemm<2, 2, false, false>(acc, buf0, kLds, 0, sm.w4, kLds, 0, kHid);
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        float t[1][2][4];
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            int rr, cc;
            acc_pos(q, rr, cc);
            t[0][nt][q] = acc[mt][nt][q] + sm.b4[8 * nt + cc];
          }
        mlp_softmax(t, a.n_classes);
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            int rr, cc;
            acc_pos(q, rr, cc);
            prob[(16 * mt + rr) * kOutPad + 8 * nt + cc] = t[0][nt][q];
          }
      }
    }
    __syncwarp();
    // ---- window weights into the projection tallies ----
    if (p_off >= 0) {
      const float *pr = prob + lane * kOutPad;
      float norm = pr[0] * a.rr;
      for (int c = 1; c < a.n_classes; ++c) norm += pr[c];
      const float inv = norm > 0.0f ? 1.0f / norm : 0.0f;
      for (int c = 1; c < a.n_classes; ++c) {
        const unsigned long long q = __float2ull_rn((pr[c] * inv) * 4294967296.0f);
        if (!q) continue;
        const size_t idx = (size_t)p_off + (size_t)(c - 1) * plane;
        atomicAdd(a.proj + idx, q);
        const unsigned long long lo = q * q;
        const unsigned long long rest = (__umul64hi(q, q) << 32) | (lo >> 32);
        if (lo & 0xffffffffull) atomicAdd(a.proj2 + 2 * idx, lo & 0xffffffffull);
        if (rest) atomicAdd(a.proj2 + 2 * idx + 1, rest);
      }
    }
    __syncwarp();
  }
  if (my_net) atomicAdd(&n_net, my_net);
  if (my_fb) atomicAdd(&n_fb, my_fb);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (n_net) atomicAdd(&a.counters[GG_CNT_ARF_PHOTONS], (unsigned long long)n_net);
    if (n_fb) atomicAdd(&a.counters[GG_CNT_ARF_FALLBACK], (unsigned long long)n_fb);
  }
}

template <typename real>
cudaError_t launch_spect_arf(const Scene<real> &s, const ArfStageArgs &a, int grid, cudaStream_t st) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_spect_arf<real>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(ArfSmem));
    if (e != cudaSuccess) return e;
    configured = true;
  }
  k_spect_arf<real><<<grid, kArfWarps * 32, sizeof(ArfSmem), st>>>(s, a);
  return cudaGetLastError();
}

template cudaError_t launch_spect_arf<float>(const Scene<float> &, const ArfStageArgs &, int, cudaStream_t);
template cudaError_t launch_spect_arf<double>(const Scene<double> &, const ArfStageArgs &, int, cudaStream_t);

}  // namespace gg
