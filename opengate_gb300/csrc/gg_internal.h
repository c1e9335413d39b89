// gg_internal.h - declarations shared by the host API and the kernel translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace gg {

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
  int refill_min;                   // lanes that must wait for a history before a refill phase
  int interact_min;                 // pending collisions that trigger an interaction phase
};

// Bit of the kernel status word set when a stage queue overflowed (the low
// bits carry the source stage's GG_ERR_* code).
constexpr unsigned int kStatusQueueOverflow = 0x100u;

// Queues of one SPECT stage launch (see gg_spect.cu).
struct StageArgs {
  void *in_q;                      // input queue (phantom stage: null = the batch's primary records)
  const unsigned long long *in_n;  // input queue length
  void *out_q;                     // output queue
  unsigned long long *out_n;       // output queue length (appended to)
  size_t q_cap;                    // capacity of each queue (entries)
};

template <typename real>
size_t transport_smem_bytes(int n_comp, int n_e, int n_mat);
template <typename real>
size_t queue_bytes(size_t cap);
// stage 0: phantom stage, 1: head stage
template <typename real>
cudaError_t launch_spect_stage(int stage, const Scene<real> &s, const KernelArgs &a, const StageArgs &q, int grid,
                               int block, size_t smem, int minb, cudaStream_t st);
template <typename real>
cudaError_t spect_stage_occupancy(int stage, int block, size_t smem, int minb, int *blocks_per_sm);
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
cudaError_t launch_flush(unsigned long long *acc_e, unsigned long long *acc_e2, double *edep, double *edep2,
                         size_t n, int grid, cudaStream_t st);

}  // namespace gg
