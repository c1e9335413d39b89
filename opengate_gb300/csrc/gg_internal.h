// gg_internal.h - declarations shared by the host API and the kernel translation units.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace gg {

// cudaFuncSetAttribute applies to the current device only: `done` remembers,
// one bit per device ordinal (< 64), on which devices a kernel's dynamic
// shared-memory limit has been raised: to `bytes`, or to what the block's
// opt-in limit leaves beside the kernel's static shared memory if less.
template <typename K>
inline cudaError_t configure_smem(K kernel, int bytes, unsigned long long &done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (done & bit)) return cudaSuccess;
  int optin = 0;
  cudaFuncAttributes fa;
  if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&fa, kernel)) != cudaSuccess) return e;
  const int room = optin - (int)fa.sharedSizeBytes;
  if (room < bytes) bytes = room;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done |= bit;
  return e;
}


template <typename real>
struct Scene;

// Arguments of one transport launch (one tally batch).
struct KernelArgs {
  uint64_t seed;
  uint64_t h_begin, h_end;          // histories [h_begin, h_end)
  unsigned long long *next;         // claim counter, zero at launch
  unsigned long long *acc_e;        // per-voxel fixed-point edep of this batch
  unsigned long long *acc_e2;       // per-voxel fixed-point edep^2 (or null)
  unsigned long long *counters;     // GG_N_COUNTERS slots
  unsigned int *status;             // OR of error codes raised by the kernel
  int chunk;                        // histories claimed per warp refill
  void *records;                    // primary records of the batch (k_generate -> k_transport)
  size_t rec_cap;                   // records capacity (histories per batch)
  uint64_t rec_first;               // history of record 0 (<= h_begin; a SPECT pass can start later)
  int refill_min;                   // lanes that must wait for a history before a refill phase
  int interact_min;                 // pending collisions that trigger an interaction phase
  unsigned long long *acc_d;        // dose grid: fixed-point sum(edep * rho_min / rho) (or null)
  unsigned long long *acc_d2;       // its history-by-history squares (or null)
};

// Bit of the kernel status word set when a stage queue overflowed (the low
// bits carry the source stage's GG_ERR_* code).
constexpr unsigned int kStatusQueueOverflow = 0x100u;
// Bit set when a bounded wait of a tensor-core kernel ran out (the kernel
// stopped early and freed its tensor memory).
constexpr unsigned int kStatusWaitTimeout = 0x200u;

// Queues of one SPECT stage launch (see gg_spect.cu).
struct StageArgs {
  void *in_q;                      // input queue (phantom stage: null = the batch's primary records)
  const unsigned long long *in_n;  // input queue length
  void *out_q;                     // output queue
  unsigned long long *out_n;       // output queue length (appended to)
  size_t q_cap;                    // capacity of each queue (entries)
  // scatter splitting: requests of the phantom stage for the split kernel
  // (Compton from the front, Rayleigh from the back of one buffer)
  void *split_q;
  unsigned long long *split_n;     // [Compton requests, Rayleigh requests]
  size_t split_cap;
};

// One launch of the ARF training-row generator (see gg_arf.cu).
struct ArfArgs {
  uint64_t seed, first, n;        // samples [first, first + n), Philox stream 1
  double e_min, e_max, cos_theta_max, half_extent[2], russian_roulette;
  int theta_uniform;              // theta = u theta_max instead of cos(theta) uniform
  double theta_max_turn;          // acos(cos_theta_max) / (2 pi)
  float4 *stage;                  // [n] row per sample (w = -1: dropped)
  unsigned int *block_count;      // [blocks] kept rows per block
  unsigned long long *block_off;  // [blocks] first output row of each block
  unsigned long long *counters;   // GG_N_COUNTERS slots
};

// One training step (or a prediction) of the ARF network (see gg_mlp.cu).
struct MlpTrainArgs {
  const float4 *rows;            // (E, theta, phi, class) rows
  uint64_t row0, n_rows;         // tile t reads rows (row0 + 128 t + r) % n_rows
  const float *params;           // FP32 parameters
  const __nv_bfloat16 *wbf;      // BF16 copies of W2, W3, W4
  float *partial;                // [tiles][kNParams] gradient of each tile
  float *loss_part;              // [tiles] loss sum of each tile
  float mean[3], inv_std[3];     // standardisation of (theta, phi, E)
  int n_classes;
  float inv_batch;               // 1 / rows in the step
  unsigned int *status;          // kStatusWaitTimeout when a tensor-core wait ran out
};

constexpr int kTrainRows = 128;  // rows per training tile (one CTA, MMA M)

struct MlpAdamArgs {
  const float *partial;
  int n_tiles;
  float *params;
  __nv_bfloat16 *wbf;
  float *m, *v;                  // Adam moments
  float *grad_out;               // summed gradient (or null)
  float lr, beta1, beta2, eps;   // lr = 0: gradient only, no update
  float c1, c2;                  // 1 / (1 - beta1^t), 1 / (1 - beta2^t)
  const float *loss_part;        // [n_tiles] tile loss sums, added to *loss_acc (or null)
  double *loss_acc;
};

// One launch of the ARF stage of the SPECT wavefront (see gg_arf_stage.cu).
struct ArfStageArgs {
  void *in_q;                      // head queue of the phantom stage
  const unsigned long long *in_n;
  void *out_q;                     // fallback queue for the plain head stage
  unsigned long long *out_n;
  size_t q_cap;
  const float *params;             // network
  const __nv_bfloat16 *wbf;
  float mean[3], inv_std[3];
  int n_classes;
  float rr;                        // class-0 Russian-roulette factor of the training rows
  double e_min, e_max, cos_theta_max;  // trained domain
  double e_detect_min;             // lowest window edge: photons below reach no window
  double dc;                       // collimator face -> crystal plane, mm
  unsigned long long *proj;        // fixed-point window weights, 2^-32 units, projection layout
  unsigned long long *proj2;       // their squares: (low 32 bits, rest) per pixel, 2^-64 / 2^-32 MeV^2 units
  unsigned long long *counters;
  unsigned int *status;
  unsigned long long *claim;       // chunk claim counter, zero at launch
};

size_t mlp_train_smem_bytes();
cudaError_t launch_mlp_train(const MlpTrainArgs &a, int n_tiles, cudaStream_t st);
cudaError_t launch_mlp_adam(const MlpAdamArgs &a, cudaStream_t st);
cudaError_t launch_mlp_to_bf16(const float *params, __nv_bfloat16 *wbf, cudaStream_t st);
size_t mlp_tc_smem_bytes();
cudaError_t launch_mlp_predict(const MlpTrainArgs &a, float *out, uint64_t n, int grid, unsigned int *status,
                               cudaStream_t st);
template <typename real>
cudaError_t launch_spect_arf(const Scene<real> &s, const ArfStageArgs &a, int grid, cudaStream_t st);

constexpr int kHistList = 8;     // entries of a history's voxel list
constexpr int kBlock = 256;      // most threads per block of the transport kernels
constexpr int kTransportSmemMax = 200 * 1024;  // dynamic shared memory of a transport block

// Shared memory of the transport kernels' tables: sigma rows, majorant, density
// and composition index per material, 16-byte aligned.
template <typename real>
__host__ __device__ inline size_t transport_smem_bytes(int n_comp, int n_e, int n_mat) {
  size_t b = sizeof(real) * ((size_t)n_comp * n_e + n_e + n_mat) + sizeof(int) * (size_t)n_mat;
  return (b + 15) & ~(size_t)15;
}

// Shared memory of `lists` per-history voxel lists of a block of `threads`
// (one column per thread).
template <typename real>
__host__ __device__ constexpr size_t hist_list_bytes(int lists, int threads = kBlock) {
  return (size_t)lists * kHistList * (size_t)threads * (sizeof(uint32_t) + sizeof(real));
}
// Rows of p.n samples appended to rows[*total ...] (capacity rows); *total advances on the device.
template <typename real>
cudaError_t launch_arf_dataset(const Scene<real> &s, const ArfArgs &p, float4 *rows, uint64_t capacity,
                               unsigned long long *total, cudaStream_t st);
template <typename real>
size_t queue_bytes(size_t cap);
// stage 0: phantom stage, 1: head stage
template <typename real>
cudaError_t launch_spect_stage(int stage, const Scene<real> &s, const KernelArgs &a, const StageArgs &q, int grid,
                               int block, size_t smem, int minb, cudaStream_t st);
template <typename real>
cudaError_t spect_stage_occupancy(int stage, int block, size_t smem, int minb, int *blocks_per_sm);
// Copies of scatter splitting (gg_spect.cu): the split requests of q.split_q
// into the walk queue (q.out_q / q.out_n); does nothing when the requests
// overflowed the buffer.
template <typename real>
cudaError_t launch_spect_split(const Scene<real> &s, const KernelArgs &a, const StageArgs &q, int block, size_t smem,
                               int n_sm, cudaStream_t st);
template <typename real>
size_t split_bytes(size_t cap);
// Free flights of the copies the split kernel queued (q.in_q / q.in_n) into
// the head queue (q.out_q / q.out_n).
template <typename real>
cudaError_t launch_spect_walk(const Scene<real> &s, const KernelArgs &a, const StageArgs &q, int block, size_t smem,
                              int n_sm, cudaStream_t st);
template <typename real>
size_t record_bytes(size_t cap);
template <typename real>
cudaError_t launch_generate(const Scene<real> &s, const KernelArgs &a, cudaStream_t st);
// minb selects the kernel variant compiled for that many resident blocks per SM
template <typename real>
cudaError_t launch_transport(const Scene<real> &s, const KernelArgs &a, int grid, int block, size_t smem,
                             int minb, cudaStream_t st);
template <typename real>
cudaError_t occupancy_blocks(int block, size_t smem, int minb, int *blocks_per_sm);
// Compacted wavefront dose transport (gg_wavefront.cu): 256-thread blocks,
// dynamic shared memory = tables + photon slots.
template <typename real>
size_t wavefront_smem_bytes(int n_comp, int n_e, int n_mat);
template <typename real>
cudaError_t launch_wavefront(const Scene<real> &s, const KernelArgs &a, int grid, size_t smem, int minb,
                             cudaStream_t st);
template <typename real>
cudaError_t wavefront_occupancy(size_t smem, int minb, int *blocks_per_sm);
// image += fixed point * 2^-32 * scale (squares: * scale^2), then clears the fixed-point sums
cudaError_t launch_flush(unsigned long long *acc_e, unsigned long long *acc_e2, double *edep, double *edep2,
                         size_t n, int grid, cudaStream_t st, double scale = 1.0);

}  // namespace gg
