// gg_noalloc.cu - a dose run that allocates no device memory.
//
// Some callers cannot call cudaMalloc in the middle of their work: cudaMalloc
// and cudaFree synchronise the whole device, which a caller that keeps other
// streams busy (a reconstruction or treatment-planning loop calling the dose
// engine many times, a serving process sharing the GPU) cannot afford, and a
// caller whose device memory is already handed out by its own pool allocator
// may simply have nothing left for a second allocator.  For them
// gg_dose_run_noalloc runs the same three kernels as gg_run (source stage,
// transport, tally flush) with every scratch buffer - the copied scene
// inputs, the primary records, the fixed-point tallies, the claim counter,
// the counters and the status word - placed in one file-scope device array of
// GG_NOALLOC_SCRATCH_BYTES.  The caller passes the scene (host descriptors,
// as for gg_run) and the two output images (device pointers it owns).
//
// The array is static device memory: every GPU that loads the library
// reserves it until the process exits.  All calls share it, so it keeps the
// contents of the last call; each call clears the parts that must start at
// zero (tallies, counters, claim counter, status).  Calls whose GPU work
// overlaps (different host threads, or different streams without ordering
// between them) race on the array and give wrong results: serialise them.
//
// Host code cannot use the array's name as a device address (on the host it
// names a host-side shadow).  The first call on each device, with that device
// current, asks cudaGetSymbolAddress for the device address and keeps it; that
// first call should come before any stream capture on the device.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "../../include/gate_gpu.h"
#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_validate.h"

namespace {

constexpr size_t kScratchBytes = (size_t)GG_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// device address of g_noalloc_scratch, per device ordinal (set up on first use)
void *g_scratch_addr[kMaxDevices] = {nullptr};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Offsets of the regions inside the scratch array for one call.
struct Layout {
  size_t sig, cum, ray_amax, ray_x2, ray_cum, mat_rho, mat_comp, maj, spec_e, spec_cdf, acc_box;
  size_t labels, acc_e, acc_e2, records, counters, next, status, end;
};

Layout make_layout(int n_comp, int n_e, int n_ray, int n_mat, size_t n_vox) {
  Layout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o = align256(o + bytes);
    return at;
  };
  L.sig = take(sizeof(float) * (size_t)n_comp * n_e);
  L.cum = take(sizeof(float) * 3 * (size_t)n_comp * n_e);
  L.ray_amax = take(sizeof(float) * (size_t)n_comp * n_e);
  L.ray_x2 = take(sizeof(float) * (size_t)n_ray);
  L.ray_cum = take(sizeof(float) * (size_t)n_comp * n_ray);
  L.mat_rho = take(sizeof(float) * (size_t)n_mat);
  L.mat_comp = take(sizeof(int) * (size_t)n_mat);
  L.maj = take(sizeof(float) * (size_t)n_e);
  L.spec_e = take(sizeof(float) * (GG_NOALLOC_MAX_SPECTRUM + 1));
  L.spec_cdf = take(sizeof(float) * GG_NOALLOC_MAX_SPECTRUM);
  L.acc_box = take(sizeof(float) * 6 * GG_NOALLOC_MAX_ACCEPT);
  L.labels = take(sizeof(uint16_t) * n_vox);
  L.acc_e = take(8 * n_vox);
  L.acc_e2 = take(16 * n_vox);  // 128-bit edep^2 accumulator per voxel
  L.records = take(gg::record_bytes<float>((size_t)GG_NOALLOC_BATCH));
  L.counters = take(8 * GG_N_COUNTERS);
  L.next = take(8);
  L.status = take(4);
  L.end = o;
  return L;
}

int fail(char *err, size_t len, int code, const char *fmt, ...) {
  if (err && len) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, len, fmt, ap);
    va_end(ap);
  }
  return code;
}

// Device address of the scratch array on `device` (current); looked up once.
int scratch_address(int device, void **out, char *err, size_t len) {
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(err, len, GG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return GG_OK;
}

}  // namespace

extern "C" int gg_dose_run_noalloc(int32_t device, void *stream, const gg_tables_desc *t, const gg_volume_desc *v,
                                   const gg_world_desc *w, const gg_source_desc *src, uint64_t n_histories,
                                   uint64_t seed, uint64_t first_history, double *d_edep, double *d_edep2,
                                   uint64_t *counters, char *err, size_t err_len) {
  if (err && err_len) err[0] = 0;
  if (!t || !v || !w || !src || !d_edep)
    return fail(err, err_len, GG_ERR_ARG, "gg_dose_run_noalloc: null argument");
  if (device < 0 || device >= kMaxDevices) return fail(err, err_len, GG_ERR_ARG, "device ordinal out of range");
  // ---- size limits of the scratch array ----------------------------------
  if (t->n_e < 2 || t->n_e > GG_NOALLOC_MAX_ENERGIES || t->n_comp < 1 || t->n_comp > GG_NOALLOC_MAX_COMPOSITIONS ||
      t->n_ray < 2 || t->n_ray > GG_NOALLOC_MAX_RAYLEIGH || t->n_mat < 1 || t->n_mat > GG_NOALLOC_MAX_MATERIALS)
    return fail(err, err_len, GG_ERR_ARG,
                "table sizes beyond the no-allocation limits (n_e <= %d, n_comp <= %d, n_ray <= %d, n_mat <= %d)",
                GG_NOALLOC_MAX_ENERGIES, GG_NOALLOC_MAX_COMPOSITIONS, GG_NOALLOC_MAX_RAYLEIGH,
                GG_NOALLOC_MAX_MATERIALS);
  // the same checks as gg_upload_tables / gg_upload_volume / gg_set_source
  char msg[160];
  if (gg::check_tables(t, msg, sizeof(msg))) return fail(err, err_len, GG_ERR_ARG, "tables: %s", msg);
  if (!v->labels || !v->majorant) return fail(err, err_len, GG_ERR_ARG, "incomplete volume descriptor");
  for (int a = 0; a < 3; ++a)
    if (!(v->spacing[a] > 0) || !std::isfinite(v->spacing[a]) || !(w->half_size[a] > 0))
      return fail(err, err_len, GG_ERR_ARG, "spacing and world half sizes must be > 0");
  size_t n_vox = 0;
  if (gg::check_dims(v->dims, (size_t)GG_NOALLOC_MAX_VOXELS, &n_vox, msg, sizeof(msg)))
    return fail(err, err_len, GG_ERR_ARG, "the no-allocation run handles at most %u voxels: %s",
                (unsigned)GG_NOALLOC_MAX_VOXELS, msg);
  if (gg::check_majorant(v->majorant, t->n_e, msg, sizeof(msg))) return fail(err, err_len, GG_ERR_ARG, "%s", msg);
  // voxel (activity image) sources need their CDF arrays on the device: gg_run only
  if (src->pos_type < GG_POS_POINT || src->pos_type > GG_POS_DISC)
    return fail(err, err_len, GG_ERR_ARG, "position type %d not handled by the no-allocation run", src->pos_type);
  if (src->dir_type < GG_DIR_ISO || src->dir_type > GG_DIR_FOCUSED)
    return fail(err, err_len, GG_ERR_ARG, "direction type %d", src->dir_type);
  if (src->ene_type < GG_ENE_MONO || src->ene_type > GG_ENE_RANGE)
    return fail(err, err_len, GG_ERR_ARG, "energy type %d", src->ene_type);
  int n_spec_e = src->ene_type == GG_ENE_HISTOGRAM ? src->n_spec + 1 : src->n_spec;
  bool spectrum = src->ene_type == GG_ENE_LINES || src->ene_type == GG_ENE_HISTOGRAM;
  if (spectrum && (src->n_spec < 1 || src->n_spec > GG_NOALLOC_MAX_SPECTRUM || !src->spec_e || !src->spec_cdf))
    return fail(err, err_len, GG_ERR_ARG, "spectrum must have 1..%d entries", GG_NOALLOC_MAX_SPECTRUM);
  double elo = 0, ehi = 0;
  if (gg::check_source_energy(src, &elo, &ehi, msg, sizeof(msg)))
    return fail(err, err_len, GG_ERR_ARG, "source: %s", msg);
  if (src->n_accept < 0 || src->n_accept > GG_NOALLOC_MAX_ACCEPT || (src->n_accept && !src->accept_boxes))
    return fail(err, err_len, GG_ERR_ARG, "at most %d acceptance boxes", GG_NOALLOC_MAX_ACCEPT);
  if (w->material < 0 || w->material >= t->n_mat) return fail(err, err_len, GG_ERR_ARG, "bad world material");
  for (size_t i = 0; i < n_vox; ++i)
    if (v->labels[i] >= t->n_mat) return fail(err, err_len, GG_ERR_ARG, "label outside the material table");
  if (!(elo >= t->e_min) || !(ehi <= t->e_max))
    return fail(err, err_len, GG_ERR_DOMAIN, "source energies outside the tables");
  if (n_histories == 0) return GG_OK;

  Layout L = make_layout(t->n_comp, t->n_e, t->n_ray, t->n_mat, n_vox);
  if (L.end > kScratchBytes) return fail(err, err_len, GG_ERR_ARG, "scene does not fit the scratch array");

  int prev = 0;
  cudaGetDevice(&prev);
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(err, err_len, GG_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  int rc = GG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  void *base = nullptr;
  unsigned char *b = nullptr;
  do {
    if ((rc = scratch_address(device, &base, err, err_len))) break;
    b = (unsigned char *)base;
    // ---- inputs into the scratch array --------------------------------------
    size_t nce = (size_t)t->n_comp * t->n_e;
    float spec_e[GG_NOALLOC_MAX_SPECTRUM + 1], spec_cdf[GG_NOALLOC_MAX_SPECTRUM], boxes[6 * GG_NOALLOC_MAX_ACCEPT];
    int ns = spectrum ? src->n_spec : 0;
    for (int i = 0; i < (spectrum ? n_spec_e : 0); ++i) spec_e[i] = (float)src->spec_e[i];
    for (int i = 0; i < ns; ++i) spec_cdf[i] = (float)src->spec_cdf[i];
    for (int i = 0; i < 6 * src->n_accept; ++i) boxes[i] = (float)src->accept_boxes[i];
    struct {
      size_t off;
      const void *p;
      size_t bytes;
    } copies[] = {
        {L.sig, t->sig, 4 * nce},
        {L.cum, t->cum, 12 * nce},
        {L.ray_amax, t->ray_amax, 4 * nce},
        {L.ray_x2, t->ray_x2, 4 * (size_t)t->n_ray},
        {L.ray_cum, t->ray_cum, 4 * (size_t)t->n_comp * t->n_ray},
        {L.mat_rho, t->mat_rho, 4 * (size_t)t->n_mat},
        {L.mat_comp, t->mat_comp, 4 * (size_t)t->n_mat},
        {L.maj, v->majorant, 4 * (size_t)t->n_e},
        {L.spec_e, spec_e, 4 * (size_t)(spectrum ? n_spec_e : 0)},
        {L.spec_cdf, spec_cdf, 4 * (size_t)ns},
        {L.acc_box, boxes, 4 * 6 * (size_t)src->n_accept},
        {L.labels, v->labels, 2 * n_vox},
    };
    for (auto &c : copies) {
      if (!c.bytes) continue;
      if ((e = cudaMemcpyAsync(b + c.off, c.p, c.bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
    }
    if (e != cudaSuccess) {
      rc = fail(err, err_len, GG_ERR_CUDA, "copy of inputs: %s", cudaGetErrorString(e));
      break;
    }
    // ---- state that must start at zero ---------------------------------------
    size_t zero[][2] = {{L.acc_e, 8 * n_vox}, {L.acc_e2, 16 * n_vox}, {L.counters, 8 * GG_N_COUNTERS},
                        {L.status, 4}};
    for (auto &z : zero)
      if (e == cudaSuccess) e = cudaMemsetAsync(b + z[0], 0, z[1], st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_edep, 0, 8 * n_vox, st);
    if (e == cudaSuccess && d_edep2) e = cudaMemsetAsync(d_edep2, 0, 8 * n_vox, st);
    if (e != cudaSuccess) {
      rc = fail(err, err_len, GG_ERR_CUDA, "clearing scratch: %s", cudaGetErrorString(e));
      break;
    }
    // ---- scene over the scratch array (same conversions as gg_run) --------
    gg::Scene<float> s;
    memset(&s, 0, sizeof(s));
    s.n_e = t->n_e;
    s.n_comp = t->n_comp;
    s.n_ray = t->n_ray;
    s.n_mat = t->n_mat;
    s.ln_emin = t->ln_emin;
    s.inv_dln = t->inv_dln;
    s.e_min = t->e_min;
    s.sig = (const float *)(b + L.sig);
    s.cum = (const float *)(b + L.cum);
    s.ray_amax = (const float *)(b + L.ray_amax);
    s.ray_x2 = (const float *)(b + L.ray_x2);
    s.ray_cum = (const float *)(b + L.ray_cum);
    s.mat_rho = (const float *)(b + L.mat_rho);
    s.mat_comp = (const int *)(b + L.mat_comp);
    s.maj = (const float *)(b + L.maj);
    s.nx = v->dims[0];
    s.ny = v->dims[1];
    s.nz = v->dims[2];
    for (int a = 0; a < 3; ++a) {
      s.bmin[a] = (float)v->corner[a];
      s.bmax[a] = (float)(v->corner[a] + (double)v->dims[a] * v->spacing[a]);
      s.inv_sp[a] = (float)(1.0 / v->spacing[a]);
      s.whalf[a] = (float)w->half_size[a];
      s.s_t[a] = (float)src->translation[a];
      s.s_half[a] = (float)src->half_size[a];
      s.s_focus[a] = (float)src->focus[a];
    }
    s.labels = (const uint16_t *)(b + L.labels);
    s.world_mat = w->material;
    s.pos_type = src->pos_type;
    s.dir_type = src->dir_type;
    s.ene_type = src->ene_type;
    s.n_accept = src->n_accept;
    s.max_rejection = src->max_rejection;
    s.n_spec = src->n_spec;
    for (int i = 0; i < 9; ++i) s.s_rot[i] = (float)src->rotation[i];
    s.s_radius = (float)src->radius;
    s.s_cos_tmin = (float)cos(src->theta[0]);
    s.s_cos_tmax = (float)cos(src->theta[1]);
    s.s_phi0_turn = (float)(src->phi[0] / (2.0 * M_PI));
    s.s_dphi_turn = (float)((src->phi[1] - src->phi[0]) / (2.0 * M_PI));
    double mn = sqrt(src->momentum[0] * src->momentum[0] + src->momentum[1] * src->momentum[1] +
                     src->momentum[2] * src->momentum[2]);
    for (int a = 0; a < 3; ++a) s.s_mom[a] = (float)(mn > 0 ? src->momentum[a] / mn : 0.0);
    s.s_mono = (float)src->mono;
    s.s_elo = (float)src->e_lo;
    s.s_ehi = (float)src->e_hi;
    s.spec_e = (const float *)(b + L.spec_e);
    s.spec_cdf = (const float *)(b + L.spec_cdf);
    s.acc_box = (const float *)(b + L.acc_box);
    // ---- kernels: source stage, transport, flush per batch -------------------
    int n_sm = 0, bps = 0;
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device);
    size_t smem = gg::transport_smem_bytes<float>(t->n_comp, t->n_e, t->n_mat);
    if ((e = gg::occupancy_blocks<float>(256, smem, 3, &bps)) != cudaSuccess) {
      rc = fail(err, err_len, GG_ERR_CUDA, "occupancy: %s", cudaGetErrorString(e));
      break;
    }
    gg::KernelArgs a;
    memset(&a, 0, sizeof(a));
    a.seed = seed;
    a.next = (unsigned long long *)(b + L.next);
    a.acc_e = (unsigned long long *)(b + L.acc_e);
    a.acc_e2 = d_edep2 ? (unsigned long long *)(b + L.acc_e2) : nullptr;
    a.counters = (unsigned long long *)(b + L.counters);
    a.status = (unsigned int *)(b + L.status);
    a.chunk = 256;
    a.records = b + L.records;
    a.rec_cap = (size_t)GG_NOALLOC_BATCH;
    a.refill_min = 8;
    a.interact_min = 16;
    for (uint64_t h0 = first_history; h0 < first_history + n_histories && e == cudaSuccess;
         h0 += (uint64_t)GG_NOALLOC_BATCH) {
      a.h_begin = h0;
      a.rec_first = h0;
      a.h_end = h0 + (uint64_t)GG_NOALLOC_BATCH < first_history + n_histories ? h0 + (uint64_t)GG_NOALLOC_BATCH
                                                                            : first_history + n_histories;
      e = cudaMemsetAsync(a.next, 0, 8, st);
      if (e == cudaSuccess) e = gg::launch_generate<float>(s, a, st);
      if (e == cudaSuccess) e = gg::launch_transport<float>(s, a, n_sm * (bps > 0 ? bps : 1), 256, smem, 3, st);
      if (e == cudaSuccess) e = gg::launch_flush(a.acc_e, a.acc_e2, d_edep, d_edep2, n_vox, n_sm * 8, st);
    }
    if (e != cudaSuccess) {
      rc = fail(err, err_len, GG_ERR_CUDA, "transport: %s", cudaGetErrorString(e));
      break;
    }
    // status and counters through the caller's stream (no device-wide wait)
    unsigned int status = 0;
    unsigned long long cnt[GG_N_COUNTERS];
    e = cudaMemcpyAsync(&status, b + L.status, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && counters)
      e = cudaMemcpyAsync(cnt, b + L.counters, sizeof(cnt), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      rc = fail(err, err_len, GG_ERR_CUDA, "reading status: %s", cudaGetErrorString(e));
      break;
    }
    if (counters)
      for (int i = 0; i < GG_N_COUNTERS; ++i) counters[i] = cnt[i];
    if (status)
      rc = fail(err, err_len, GG_ERR_DOMAIN, "source sampling failed (angular acceptance exhausted max_rejection)");
  } while (false);
  cudaSetDevice(prev);
  return rc;
}
