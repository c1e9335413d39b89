// gg_api.cu - C ABI of libgategpu.so (declared in include/gate_gpu.h).
//
// A context owns one CUDA stream and every device buffer of one simulation:
// physics tables, label image, majorant, source spectra, the per-batch
// fixed-point tallies and the float64 edep / edep-squared images.  Host
// buffers passed in are copied; nothing is retained past a call.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gate_gpu.h"
#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_validate.h"
#include "gg_mlp.cuh"

namespace {

std::string g_create_error;

template <typename T>
void dfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

}  // namespace

struct gg_ctx {
  int device = 0;
  int precision = GG_PREC_F32;
  int block = 256;
  int blocks_per_sm = 0;
  int chunk = 256;
  // histories per batch: large batches keep the persistent grids and the SPECT
  // stage passes busy (2^24 made the 60-position Tc-99m acquisition ~20 % slower)
  int64_t batch = 1 << 26;
  int refill_min = 8;
  int interact_min = 16;
  // dose transport kernel of single simulations: the block-synchronous phase kernel (default,
  // also used for the track-length estimator and batches) or the compacted wavefront
  int transport_kernel = GG_KERNEL_PHASED;
  uint64_t last_batch = 0;  // histories per tally batch of the last run (after the overflow cap)
  int n_sm = 0;
  cudaStream_t stream = nullptr;
  std::string err;

  // tables (device, in working precision)
  int n_e = 0, n_comp = 0, n_ray = 0, n_mat = 0;
  float ln_emin = 0, inv_dln = 0, e_min = 0, e_max = 0;
  void *d_sig = nullptr, *d_cum = nullptr, *d_ray_amax = nullptr, *d_ray_cum = nullptr, *d_mat_rho = nullptr;
  // digitizer blurring (gg_spect_set_blur)
  gg_blur_desc blur{};
  // track-length estimator (gg_set_tle)
  void *d_muen = nullptr;
  bool tle = false;
  double tle_thr = 0.0, tle_emin = 0.0;
  void *d_ray_x2 = nullptr;
  int *d_mat_comp = nullptr;
  std::vector<int> h_mat_comp;
  std::vector<float> h_mat_rho;
  bool have_tables = false;

  // volume
  int dims[3] = {0, 0, 0};
  double spacing[3] = {0, 0, 0}, corner[3] = {0, 0, 0};
  uint16_t *d_labels = nullptr;
  size_t labels_cap = 0;  // voxels d_labels holds (kept across uploads of the same size or smaller)
  void *d_maj = nullptr;
  size_t n_vox = 0;
  bool have_volume = false;

  // world
  gg_world_desc world{};
  bool have_world = false;

  // source
  gg_source_desc src{};
  void *d_spec_e = nullptr, *d_spec_cdf = nullptr, *d_acc_box = nullptr;
  bool have_source = false;
  double src_emax = 0;
  void *d_cdf_z = nullptr, *d_cdf_y = nullptr, *d_cdf_x = nullptr;

  // SPECT
  gg_spect_desc spect{};
  bool have_spect = false;
  int spect_run = 0;
  std::vector<double> frames;  // [n_runs][n_heads][12], host copy
  void *d_frames = nullptr;    // same in working precision
  bool frames_dirty = true;
  uint64_t run_first = 0, run_len = 1;  // history h -> run run_base + (h - run_first) / run_len
  int run_base = 0;
  unsigned long long *d_proj = nullptr;
  size_t n_proj = 0;

  // tally
  unsigned long long *d_acc_e = nullptr, *d_acc_e2 = nullptr;
  double *d_edep = nullptr, *d_edep2 = nullptr;
  bool have_tally = false, squared = false;
  // dose tally on a grid of its own (gg_set_dose_grid): voxels of the tally images (the image
  // grid's n_vox when off), and the dose tally sum(edep * rho_min / rho)
  size_t n_tally = 0;
  bool dgrid_on = false, ddose = false;
  int ddims[3] = {0, 0, 0};
  double dspacing[3] = {0, 0, 0}, dcorner[3] = {0, 0, 0};
  float drho_min = 1.0f;
  unsigned long long *d_acc_d = nullptr, *d_acc_d2 = nullptr;
  double *d_dose = nullptr, *d_dose2 = nullptr;

  // run bookkeeping
  unsigned long long *d_counters = nullptr, *d_next = nullptr;
  unsigned int *d_status = nullptr;
  // singles list (gg_spect_record_singles): records and their count (0 capacity: off)
  gg::SingleRec *d_singles = nullptr;
  unsigned long long *d_n_singles = nullptr;
  uint64_t singles_cap = 0;
  void *d_records = nullptr;
  size_t rec_cap = 0;
  // SPECT stage queues (head queue, return queue) and their lengths
  void *d_queue[3] = {nullptr, nullptr, nullptr};  // head, return, ARF fallback
  size_t q_cap = 0;
  // ARF stage in the SPECT acquisition
  bool arf_on = false;
  // free flight outside the heads (gg_spect_set_free_flight): ff_mode
  // GG_FF_PRIMARY or GG_FF_SCATTER (split copies in free flight)
  bool ff_on = false;
  int ff_mode = GG_FF_OFF;
  double ff_wcut = -1.0, ff_ecut = 0.0;
  int ss_nc = 0, ss_nr = 0, ss_max = 0;
  double ss_cos = -2.0;
  // scatter splitting: histories per phantom pass whose copies fit the head
  // queue (lowered when a pass overflows), and the counters before a pass
  uint64_t ss_span = 0;
  unsigned long long *d_cnt_save = nullptr;
  void *d_split = nullptr;  // split requests (phantom stage -> split kernel)
  size_t split_cap = 0;
  unsigned long long *d_split_n = nullptr;
  unsigned long long *d_arf_proj = nullptr, *d_arf_proj2 = nullptr;
  size_t arf_proj_n = 0;
  unsigned long long *d_qn = nullptr;

  // ARF training rows (device): staging, block counts/offsets, rows, identity head frame
  float4 *d_arf_stage = nullptr, *d_arf_rows = nullptr;
  unsigned int *d_arf_bcount = nullptr;
  unsigned long long *d_arf_boff = nullptr, *d_arf_total = nullptr;
  uint64_t arf_rows_cap = 0, arf_n_rows = 0;
  void *d_frame_id = nullptr;

  // ARF network: FP32 parameters, BF16 weight copies, Adam moments, per-tile gradients
  float *d_params = nullptr, *d_adam_m = nullptr, *d_adam_v = nullptr, *d_grad = nullptr;
  float *d_partial = nullptr, *d_loss_part = nullptr;
  double *d_loss_acc = nullptr;
  __nv_bfloat16 *d_wbf = nullptr;
  int partial_tiles = 0;
  float4 *d_io_rows = nullptr;
  float *d_io_out = nullptr;
  size_t io_cap = 0;
  gg_arf_model arf{};
  bool have_arf = false;

  // batched simulations
  bool have_batch = false;
  int n_sims = 0;
  std::vector<uint64_t> sim_vox_off, sim_vox_n;
  uint64_t batch_total = 0;
  gg_autotune_result tune{};  // last gg_batch_autotune search
  void *d_sims = nullptr, *d_sim_maj = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<cudaEvent_t> ev;
  double last_generate_ms = 0, last_transport_ms = 0, last_flush_ms = 0;
  int last_launches = 0, last_stage_launches = 0, run_stage_launches = 0;
  // SPECT stage timing of the last run: events around each stage launch
  std::vector<cudaEvent_t> stage_ev;
  std::vector<int> stage_kind;  // 0 phantom, 1 head, 2 ARF, per event pair
  double stage_ms[3] = {0, 0, 0};

  int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  int cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return GG_OK;
    return fail(GG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
  size_t real_size() const { return precision == GG_PREC_F64 ? sizeof(double) : sizeof(float); }

  // Copies ordered with the context's kernels: the context stream is
  // non-blocking, so plain cudaMemcpy / cudaMemset (legacy stream) would not
  // wait for them.  Both return after the copy has completed.
  int h2d(void *dst, const void *src, size_t bytes, const char *what) {
    int st = cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream), what);
    return st ? st : cuda(cudaStreamSynchronize(stream), what);
  }
  int d2h(void *dst, const void *src, size_t bytes, const char *what) {
    int st = cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream), what);
    return st ? st : cuda(cudaStreamSynchronize(stream), what);
  }

  // Copies n floats to a new device array in working precision.
  int upload_real(void *&dst, const float *src, size_t n) {
    dfree(dst);
    if (n == 0) n = 1;
    int st = cuda(cudaMalloc(&dst, n * real_size()), "cudaMalloc");
    if (st) return st;
    if (!src) return cuda(cudaMemsetAsync(dst, 0, n * real_size(), stream), "cudaMemset");
    if (precision == GG_PREC_F64) {
      std::vector<double> tmp(src, src + n);
      st = h2d(dst, tmp.data(), n * sizeof(double), "cudaMemcpy");
    } else {
      st = h2d(dst, src, n * sizeof(float), "cudaMemcpy");
    }
    return st;
  }
  int upload_real_d(void *&dst, const double *src, size_t n) {
    std::vector<float> f;
    std::vector<double> d;
    dfree(dst);
    if (n == 0) n = 1;
    int st = cuda(cudaMalloc(&dst, n * real_size()), "cudaMalloc");
    if (st) return st;
    if (!src) return cuda(cudaMemsetAsync(dst, 0, n * real_size(), stream), "cudaMemset");
    if (precision == GG_PREC_F64) {
      return h2d(dst, src, n * sizeof(double), "cudaMemcpy");
    }
    f.resize(n);
    for (size_t i = 0; i < n; ++i) f[i] = (float)src[i];
    return h2d(dst, f.data(), n * sizeof(float), "cudaMemcpy");
  }

  void release() {
    dfree(d_sig); dfree(d_cum); dfree(d_ray_amax); dfree(d_ray_cum); dfree(d_mat_rho); dfree(d_mat_comp);
    dfree(d_muen);
    dfree(d_ray_x2);
    dfree(d_labels); dfree(d_maj); dfree(d_spec_e); dfree(d_spec_cdf); dfree(d_acc_box);
    dfree(d_acc_e); dfree(d_acc_e2); dfree(d_edep); dfree(d_edep2);
    dfree(d_acc_d); dfree(d_acc_d2); dfree(d_dose); dfree(d_dose2);
    dfree(d_counters); dfree(d_next); dfree(d_status); dfree(d_records); dfree(d_cnt_save);
    dfree(d_split); dfree(d_split_n);
    dfree(d_queue[0]); dfree(d_queue[1]); dfree(d_queue[2]); dfree(d_qn);
    dfree(d_arf_proj); dfree(d_arf_proj2);
    arf_proj_n = 0;
    dfree(d_arf_stage); dfree(d_arf_rows); dfree(d_arf_bcount); dfree(d_arf_boff); dfree(d_arf_total);
    dfree(d_frame_id);
    arf_rows_cap = 0;
    dfree(d_params); dfree(d_adam_m); dfree(d_adam_v); dfree(d_grad); dfree(d_partial); dfree(d_loss_part);
    dfree(d_loss_acc); dfree(d_wbf); dfree(d_io_rows); dfree(d_io_out);
    dfree(d_sims); dfree(d_sim_maj);
    dfree(d_singles); dfree(d_n_singles);
    singles_cap = 0;
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (graph) cudaGraphDestroy(graph);
    graph_exec = nullptr;
    graph = nullptr;
    partial_tiles = 0;
    io_cap = 0;
    q_cap = 0;
    dfree(d_cdf_z); dfree(d_cdf_y); dfree(d_cdf_x); dfree(d_proj); dfree(d_frames);
    rec_cap = 0;
    for (auto e : ev) cudaEventDestroy(e);
    ev.clear();
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }

  template <typename real>
  gg::Scene<real> scene() const {
    gg::Scene<real> s;
    memset(&s, 0, sizeof(s));
    s.n_e = n_e;
    s.n_comp = n_comp;
    s.n_ray = n_ray;
    s.n_mat = n_mat;
    s.ln_emin = (real)ln_emin;
    s.inv_dln = (real)inv_dln;
    s.e_min = (real)e_min;
    s.sig = (const real *)d_sig;
    s.cum = (const real *)d_cum;
    s.ray_amax = (const real *)d_ray_amax;
    s.ray_cum = (const real *)d_ray_cum;
    s.ray_x2 = (const real *)d_ray_x2;
    s.mat_rho = (const real *)d_mat_rho;
    s.mat_comp = d_mat_comp;
    s.maj = (const real *)d_maj;
    s.nx = dims[0];
    s.ny = dims[1];
    s.nz = dims[2];
    for (int a = 0; a < 3; ++a) {
      s.bmin[a] = (real)corner[a];
      s.bmax[a] = (real)(corner[a] + (double)dims[a] * spacing[a]);
      s.inv_sp[a] = (real)(1.0 / spacing[a]);
      s.sp[a] = (real)spacing[a];
      s.whalf[a] = (real)world.half_size[a];
    }
    s.muen = (tle && !have_spect && !have_batch) ? (const real *)d_muen : nullptr;
    if (dgrid_on && !have_spect && !have_batch) {
      s.dgrid = 1;
      s.dnx = ddims[0];
      s.dny = ddims[1];
      s.dnz = ddims[2];
      for (int a = 0; a < 3; ++a) {
        s.dcorner[a] = (real)dcorner[a];
        s.dinv_sp[a] = (real)(1.0 / dspacing[a]);
      }
      s.ddose = ddose ? 1 : 0;
      s.drho_min = (real)drho_min;
    }
    s.eblur = blur.energy_method;
    s.eb_sigma = (real)blur.energy_sigma;
    s.eb_res = (real)blur.energy_resolution;
    s.eb_ref = (real)blur.energy_reference;
    s.eb_slope = (real)blur.energy_slope;
    s.sblur = blur.spatial ? (blur.truncated ? 2 : 1) : 0;
    s.sb_keep = blur.keep_in_solid_limits;
    s.sb_sigma[0] = (real)blur.spatial_sigma[0];
    s.sb_sigma[1] = (real)blur.spatial_sigma[1];
    s.tle_thr = (real)tle_thr;
    s.tle_emin = (real)tle_emin;
    s.labels = d_labels;
    s.sims = have_batch ? (const gg::SimDesc<real> *)d_sims : nullptr;
    s.sim_maj = have_batch ? (const real *)d_sim_maj : nullptr;
    s.n_sims = have_batch ? n_sims : 0;
    s.world_mat = world.material;
    s.pos_type = src.pos_type;
    s.dir_type = src.dir_type;
    s.ene_type = src.ene_type;
    s.n_accept = src.n_accept;
    s.max_rejection = src.max_rejection;
    s.n_spec = src.n_spec;
    for (int a = 0; a < 3; ++a) {
      s.s_t[a] = (real)src.translation[a];
      s.s_half[a] = (real)src.half_size[a];
      s.s_focus[a] = (real)src.focus[a];
    }
    for (int i = 0; i < 9; ++i) s.s_rot[i] = (real)src.rotation[i];
    s.s_radius = (real)src.radius;
    s.s_cos_tmin = (real)cos(src.theta[0]);
    s.s_cos_tmax = (real)cos(src.theta[1]);
    s.s_phi0_turn = (real)(src.phi[0] / (2.0 * M_PI));
    s.s_dphi_turn = (real)((src.phi[1] - src.phi[0]) / (2.0 * M_PI));
    s.s_fd_cmin = (real)src.fd_cos_min;
    s.s_fd_cmax = (real)src.fd_cos_max;
    s.s_fd_w = src.dir_type == GG_DIR_FORCED ? (real)((src.fd_cos_min - src.fd_cos_max) / 2.0) : (real)1;
    double mn = sqrt(src.momentum[0] * src.momentum[0] + src.momentum[1] * src.momentum[1] +
                     src.momentum[2] * src.momentum[2]);
    for (int a = 0; a < 3; ++a) s.s_mom[a] = (real)(mn > 0 ? src.momentum[a] / mn : 0.0);
    s.s_mono = (real)src.mono;
    s.s_elo = (real)src.e_lo;
    s.s_ehi = (real)src.e_hi;
    s.spec_e = (const real *)d_spec_e;
    s.spec_cdf = (const real *)d_spec_cdf;
    s.acc_box = (const real *)d_acc_box;
    // voxel source (same conversions as the oracle)
    s.vnx = src.vox_dims[0];
    s.vny = src.vox_dims[1];
    s.vnz = src.vox_dims[2];
    for (int a = 0; a < 3; ++a) {
      s.v_org[a] = (real)(src.vox_corner[a] + 0.5 * src.vox_spacing[a]);
      s.v_sp[a] = (real)src.vox_spacing[a];
    }
    s.cdf_z = (const real *)d_cdf_z;
    s.cdf_y = (const real *)d_cdf_y;
    s.cdf_x = (const real *)d_cdf_x;
    // SPECT heads and digitizer
    s.spect = have_spect ? 1 : 0;
    if (have_spect) {
      const gg_spect_desc &sp = spect;
      s.n_heads = sp.n_heads;
      s.n_runs = sp.n_runs;
      s.n_win = sp.n_windows;
      s.pnx = sp.size[0];
      s.pny = sp.size[1];
      s.frames = (const real *)d_frames;
      s.run_first = run_first;
      s.run_len = run_len;
      s.run_base = run_base;
      s.half_w = (real)sp.half_width;
      s.centroid = sp.adder_policy == GG_ADDER_CENTROID ? 1 : 0;
      s.ff = ff_on ? ff_mode : GG_FF_OFF;
      s.ff_wcut = (real)ff_wcut;
      s.ff_ecut = (real)ff_ecut;
      s.ss_nc = ss_nc;
      s.ss_nr = ss_nr;
      s.ss_max = ss_max;
      s.ss_cos = (real)ss_cos;
      s.wproj = ff_on ? d_arf_proj : nullptr;
      s.wproj2 = ff_on ? d_arf_proj2 : nullptr;
      {
        // slab boundaries: running sums in double, each rounded once
        double z = 0.0;
        int k = 0;
        s.zb[0] = (real)0;
        auto slab = [&](double t, int m) {
          z = z + t;
          s.hmat[k] = m;
          s.zb[++k] = (real)z;
        };
        slab(sp.collimator_thickness, sp.collimator_material);
        slab(sp.gap, -1);
        if (sp.n_cover > 0) slab(sp.cover_thickness, sp.cover_material);
        s.hreg_cr = k;
        slab(sp.crystal_thickness, sp.crystal_material);
        for (int b = 0; b < sp.n_back; ++b) slab(sp.back_thickness[b], sp.back_material[b]);
        s.n_hreg = k;
        s.zend = s.zb[k];
        for (int j = k; j < gg::kHeadRegions; ++j) {
          s.hmat[j] = -1;
          s.zb[j + 1] = s.zend;
        }
        s.side_black = sp.shielded_sides ? 1 : 0;
      }
      s.apo = (real)sp.hole_apothem;
      s.px = (real)sp.pitch_x;
      s.py = (real)sp.pitch_y;
      s.hpx = (real)(0.5 * sp.pitch_x);
      s.hpy = (real)(0.5 * sp.pitch_y);
      s.inv_px = (real)(1.0 / sp.pitch_x);
      s.inv_py = (real)(1.0 / sp.pitch_y);
      s.mat_coll = sp.collimator_material;
      s.mat_cr = sp.crystal_material;
      for (int k = 0; k < sp.n_windows; ++k) {
        s.wlo[k] = (real)sp.window_lo[k];
        s.whi[k] = (real)sp.window_hi[k];
      }
      for (int a = 0; a < 2; ++a) {
        s.pix_half[a] = (real)(0.5 * sp.size[a] * sp.spacing[a]);
        s.inv_psp[a] = (real)(1.0 / sp.spacing[a]);
      }
      s.proj = d_proj;
      if (singles_cap) {
        s.singles = d_singles;
        s.n_singles_rec = d_n_singles;
        s.singles_cap = singles_cap;
      }
    }
    return s;
  }
};

// ARF chunk size: samples per k_arf_sample launch
static const uint64_t kArfChunk = 1ull << 22;

// Generates ARF training rows of n samples into c->d_arf_rows (capacity rows,
// reallocated when larger); c->arf_n_rows = rows produced (may exceed the
// capacity: only the first `capacity` are stored).
template <typename real>
static int arf_generate(gg_ctx *c, const gg_arf_sampling *a, uint64_t n, uint64_t seed, uint64_t first,
                        uint64_t capacity) {
  int st;
  if (!c->d_arf_stage) {
    const uint64_t blocks = kArfChunk / 256;
    if ((st = c->cuda(cudaMalloc(&c->d_arf_stage, kArfChunk * sizeof(float4)), "cudaMalloc ARF staging"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_arf_bcount, blocks * sizeof(unsigned int)), "cudaMalloc"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_arf_boff, blocks * sizeof(unsigned long long)), "cudaMalloc"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_arf_total, sizeof(unsigned long long)), "cudaMalloc"))) return st;
    static const double id[12] = {0, 0, 0, 0, 0, 1, 1, 0, 0, 0, 1, 0};
    if ((st = c->upload_real_d(c->d_frame_id, id, 12))) return st;
  }
  if (capacity > c->arf_rows_cap) {
    dfree(c->d_arf_rows);
    c->arf_rows_cap = 0;
    if ((st = c->cuda(cudaMalloc(&c->d_arf_rows, (capacity ? capacity : 1) * sizeof(float4)), "cudaMalloc ARF rows")))
      return st;
    c->arf_rows_cap = capacity;
  }
  gg::Scene<real> s = c->scene<real>();
  s.spect = 1;
  s.n_heads = 1;
  s.n_runs = 1;
  s.frames = (const real *)c->d_frame_id;
  s.run_base = 0;
  s.run_first = 0;
  s.run_len = 1;
  gg::ArfArgs p;
  p.seed = seed;
  p.e_min = a->e_min;
  p.e_max = a->e_max;
  p.cos_theta_max = a->cos_theta_max;
  p.half_extent[0] = a->half_extent[0];
  p.half_extent[1] = a->half_extent[1];
  p.russian_roulette = a->russian_roulette;
  p.theta_uniform = a->theta_uniform ? 1 : 0;
  p.theta_max_turn = std::acos(a->cos_theta_max) / (2.0 * M_PI);
  p.stage = c->d_arf_stage;
  p.block_count = c->d_arf_bcount;
  p.block_off = c->d_arf_boff;
  p.counters = c->d_counters;
  if ((st = c->cuda(cudaMemsetAsync(c->d_arf_total, 0, sizeof(unsigned long long), c->stream), "memset"))) return st;
  for (uint64_t done = 0; done < n; done += kArfChunk) {
    p.first = first + done;
    p.n = std::min<uint64_t>(kArfChunk, n - done);
    if ((st = c->cuda(gg::launch_arf_dataset<real>(s, p, c->d_arf_rows, capacity, c->d_arf_total, c->stream),
                      "ARF dataset launch")))
      return st;
  }
  unsigned long long total = 0;
  if ((st = c->cuda(cudaMemcpyAsync(&total, c->d_arf_total, sizeof(total), cudaMemcpyDeviceToHost, c->stream),
                    "ARF row count")))
    return st;
  if ((st = c->cuda(cudaStreamSynchronize(c->stream), "ARF dataset"))) return st;
  c->arf_n_rows = total;
  return GG_OK;
}

// ---- ARF network helpers -----------------------------------------------------
static int arf_alloc(gg_ctx *c, int tiles) {
  int st;
  if (!c->d_params) {
    if ((st = c->cuda(cudaMalloc(&c->d_params, gg::kNParams * sizeof(float)), "cudaMalloc ARF params"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_adam_m, gg::kNParams * sizeof(float)), "cudaMalloc"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_adam_v, gg::kNParams * sizeof(float)), "cudaMalloc"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_grad, gg::kNParams * sizeof(float)), "cudaMalloc"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_wbf, gg::kNBfAll * sizeof(__nv_bfloat16)), "cudaMalloc"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_loss_acc, 1024 * sizeof(double)), "cudaMalloc"))) return st;
  }
  if (tiles > c->partial_tiles) {
    dfree(c->d_partial);
    dfree(c->d_loss_part);
    c->partial_tiles = 0;
    if ((st = c->cuda(cudaMalloc(&c->d_partial, (size_t)tiles * gg::kNParams * sizeof(float)), "cudaMalloc")))
      return st;
    if ((st = c->cuda(cudaMalloc(&c->d_loss_part, (size_t)tiles * sizeof(float)), "cudaMalloc"))) return st;
    c->partial_tiles = tiles;
  }
  return GG_OK;
}

static int io_alloc(gg_ctx *c, size_t rows) {
  if (rows <= c->io_cap) return GG_OK;
  dfree(c->d_io_rows);
  dfree(c->d_io_out);
  c->io_cap = 0;
  int st;
  if ((st = c->cuda(cudaMalloc(&c->d_io_rows, rows * sizeof(float4)), "cudaMalloc"))) return st;
  if ((st = c->cuda(cudaMalloc(&c->d_io_out, rows * 16 * sizeof(float)), "cudaMalloc"))) return st;
  c->io_cap = rows;
  return GG_OK;
}

// splitmix64: the weight initialisation stream
static uint64_t splitmix64(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// He-uniform weights U(-sqrt(6 / fan_in), +sqrt(6 / fan_in)), zero biases,
// output rows >= n_classes zero.
static std::vector<float> arf_init_params(uint64_t seed, int n_classes) {
  std::vector<float> w(gg::kNParams, 0.0f);
  uint64_t st = seed;
  auto uni = [&](double lim) { return (float)(((double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0) * lim); };
  for (int e = 0; e < gg::kHid * 3; ++e) w[gg::kOffW1 + e] = uni(std::sqrt(6.0 / 3.0));
  for (int e = 0; e < gg::kHid * gg::kHid; ++e) w[gg::kOffW2 + e] = uni(std::sqrt(6.0 / gg::kHid));
  for (int e = 0; e < gg::kHid * gg::kHid; ++e) w[gg::kOffW3 + e] = uni(std::sqrt(6.0 / gg::kHid));
  for (int r = 0; r < n_classes; ++r)
    for (int k = 0; k < gg::kHid; ++k) w[gg::kOffW4 + r * gg::kHid + k] = uni(std::sqrt(6.0 / gg::kHid));
  return w;
}

static gg::MlpTrainArgs arf_args(const gg_ctx *c) {
  gg::MlpTrainArgs a{};
  a.params = c->d_params;
  a.wbf = c->d_wbf;
  a.partial = c->d_partial;
  a.loss_part = c->d_loss_part;
  for (int k = 0; k < 3; ++k) {
    a.mean[k] = c->arf.x_mean[k];
    a.inv_std[k] = 1.0f / c->arf.x_std[k];
  }
  a.n_classes = c->arf.n_classes;
  a.status = c->d_status;
  return a;
}

static int arf_model_check(gg_ctx *c, const gg_arf_model *m) {
  if (m->n_classes < 2 || m->n_classes > 9) return c->fail(GG_ERR_ARG, "ARF model: n_classes must be 2..9");
  for (int k = 0; k < 3; ++k)
    if (!(m->x_std[k] > 0.0f)) return c->fail(GG_ERR_ARG, "ARF model: x_std must be > 0");
  if (!(m->russian_roulette >= 1.0)) return c->fail(GG_ERR_ARG, "ARF model: russian_roulette must be >= 1");
  return GG_OK;
}

// ARF projection tallies (n pixels of the projection layout), zeroed.
static int arf_projection_alloc(gg_ctx *c, size_t n) {
  int st;
  if (n != c->arf_proj_n) {
    dfree(c->d_arf_proj);
    dfree(c->d_arf_proj2);
    c->arf_proj_n = 0;
    if ((st = c->cuda(cudaMalloc(&c->d_arf_proj, n * 8), "cudaMalloc ARF projection"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_arf_proj2, n * 16), "cudaMalloc ARF projection squared"))) return st;
    c->arf_proj_n = n;
  }
  if ((st = c->cuda(cudaMemsetAsync(c->d_arf_proj, 0, n * 8, c->stream), "memset"))) return st;
  return c->cuda(cudaMemsetAsync(c->d_arf_proj2, 0, n * 16, c->stream), "memset");
}

// ---- batched simulations -----------------------------------------------------
// Descriptor of one simulation with the same conversions as gg_ctx::scene()
// for a single simulation (so a batched simulation equals its run alone).
template <typename real>
static gg::SimDesc<real> sim_desc(const gg_sim_desc &d, uint64_t h_begin, uint64_t vox_off) {
  gg::SimDesc<real> o;
  memset(&o, 0, sizeof(o));
  o.h_begin = h_begin;
  o.n = d.n_primaries;
  o.seed = d.seed;
  o.vox_off = vox_off;
  const gg_volume_desc &v = d.volume;
  o.nx = v.dims[0];
  o.ny = v.dims[1];
  o.nz = v.dims[2];
  for (int a = 0; a < 3; ++a) {
    o.bmin[a] = (real)v.corner[a];
    o.bmax[a] = (real)(v.corner[a] + (double)v.dims[a] * v.spacing[a]);
    o.inv_sp[a] = (real)(1.0 / v.spacing[a]);
  }
  const gg_source_desc &src = d.source;
  o.pos_type = src.pos_type;
  o.dir_type = src.dir_type;
  o.ene_type = src.ene_type;
  for (int a = 0; a < 3; ++a) {
    o.s_t[a] = (real)src.translation[a];
    o.s_half[a] = (real)src.half_size[a];
    o.s_focus[a] = (real)src.focus[a];
  }
  for (int k = 0; k < 9; ++k) o.s_rot[k] = (real)src.rotation[k];
  o.s_radius = (real)src.radius;
  o.s_cos_tmin = (real)cos(src.theta[0]);
  o.s_cos_tmax = (real)cos(src.theta[1]);
  o.s_phi0_turn = (real)(src.phi[0] / (2.0 * M_PI));
  o.s_dphi_turn = (real)((src.phi[1] - src.phi[0]) / (2.0 * M_PI));
  double mn = sqrt(src.momentum[0] * src.momentum[0] + src.momentum[1] * src.momentum[1] +
                   src.momentum[2] * src.momentum[2]);
  for (int a = 0; a < 3; ++a) o.s_mom[a] = (real)(mn > 0 ? src.momentum[a] / mn : 0.0);
  o.s_mono = (real)src.mono;
  o.s_elo = (real)src.e_lo;
  o.s_ehi = (real)src.e_hi;
  return o;
}

template <typename real>
static int upload_sims(gg_ctx *c, const gg_sim_desc *sims, int n) {
  std::vector<gg::SimDesc<real>> h(n);
  uint64_t hb = 0;
  for (int k = 0; k < n; ++k) {
    h[k] = sim_desc<real>(sims[k], hb, c->sim_vox_off[k]);
    hb += sims[k].n_primaries;
  }
  dfree(c->d_sims);
  int st = c->cuda(cudaMalloc(&c->d_sims, n * sizeof(gg::SimDesc<real>)), "cudaMalloc simulations");
  if (st) return st;
  return c->h2d(c->d_sims, h.data(), n * sizeof(gg::SimDesc<real>), "upload simulations");
}

static void drop_graph(gg_ctx *c) {
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graph_exec = nullptr;
  c->graph = nullptr;
}

// (Re)allocates the tally images for the current tally grid: the dose grid
// when set, else the image grid (only once a volume is there); the dose
// tally only with gg_set_dose_grid(score_dose).
static int tally_alloc(gg_ctx *c) {
  size_t n = 0;
  if (c->dgrid_on) n = (size_t)c->ddims[0] * c->ddims[1] * c->ddims[2];
  else if (c->have_volume) n = c->n_vox;
  if (n != c->n_tally) {
    dfree(c->d_acc_e); dfree(c->d_acc_e2); dfree(c->d_edep); dfree(c->d_edep2);
    dfree(c->d_acc_d); dfree(c->d_acc_d2); dfree(c->d_dose); dfree(c->d_dose2);
    c->n_tally = n;
  }
  if (!n) return GG_OK;
  int st;
  if (!c->d_acc_e) {
    if ((st = c->cuda(cudaMalloc(&c->d_acc_e, n * 8), "cudaMalloc tally"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_edep, n * 8), "cudaMalloc edep"))) return st;
  }
  if (c->squared && !c->d_acc_e2) {
    if ((st = c->cuda(cudaMalloc(&c->d_acc_e2, n * 16), "cudaMalloc tally2"))) return st;  // 128-bit per voxel
    if ((st = c->cuda(cudaMalloc(&c->d_edep2, n * 8), "cudaMalloc edep2"))) return st;
  }
  if (c->dgrid_on && c->ddose && !c->d_acc_d) {
    if ((st = c->cuda(cudaMalloc(&c->d_acc_d, n * 8), "cudaMalloc dose tally"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_dose, n * 8), "cudaMalloc dose"))) return st;
  }
  if (c->dgrid_on && c->ddose && c->squared && !c->d_acc_d2) {
    if ((st = c->cuda(cudaMalloc(&c->d_acc_d2, n * 16), "cudaMalloc dose tally2"))) return st;
    if ((st = c->cuda(cudaMalloc(&c->d_dose2, n * 8), "cudaMalloc dose2"))) return st;
  }
  return GG_OK;
}

extern "C" {

int gg_create(const gg_device_opts *opts, gg_ctx **out) {
  if (!out) return GG_ERR_ARG;
  *out = nullptr;
  gg_ctx *c = new gg_ctx();
  if (opts) {
    c->device = opts->device;
    if (opts->precision) c->precision = opts->precision;
    if (opts->block_size) c->block = opts->block_size;
    if (opts->blocks_per_sm) c->blocks_per_sm = opts->blocks_per_sm;
    if (opts->chunk) c->chunk = opts->chunk;
    if (opts->batch) c->batch = opts->batch;
    if (opts->refill_min) c->refill_min = opts->refill_min;
    if (opts->interact_min) c->interact_min = opts->interact_min;
  }
  auto bail = [&](const std::string &m) {
    g_create_error = m;
    c->release();
    delete c;
    return m.rfind("arg", 0) == 0 ? GG_ERR_ARG : GG_ERR_CUDA;
  };
  if (c->precision != GG_PREC_F32 && c->precision != GG_PREC_F64) return bail("arg: precision must be 32 or 64");
  if (c->block <= 0 || c->block > 256 || c->block % 32) return bail("arg: block_size must be a multiple of 32 <= 256");
  if (c->chunk <= 0) return bail("arg: chunk must be > 0");
  if (c->batch <= 0) return bail("arg: batch must be > 0");
  if (c->refill_min < 1 || c->refill_min > 32 || c->interact_min < 1 || c->interact_min > 32)
    return bail("arg: refill_min and interact_min must be in 1..32");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return bail(std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (c->device < 0 || c->device >= ndev) return bail("arg: device ordinal out of range");
  if ((e = cudaSetDevice(c->device)) != cudaSuccess) return bail(cudaGetErrorString(e));
  cudaDeviceProp prop;
  if ((e = cudaGetDeviceProperties(&prop, c->device)) != cudaSuccess) return bail(cudaGetErrorString(e));
  c->n_sm = prop.multiProcessorCount;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(cudaGetErrorString(e));
  if ((e = cudaMalloc(&c->d_counters, GG_N_COUNTERS * sizeof(unsigned long long))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_next, sizeof(unsigned long long))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_status, sizeof(unsigned int))) != cudaSuccess)
    return bail(cudaGetErrorString(e));
  cudaMemsetAsync(c->d_counters, 0, GG_N_COUNTERS * sizeof(unsigned long long), c->stream);
  cudaMemsetAsync(c->d_status, 0, sizeof(unsigned int), c->stream);
  cudaStreamSynchronize(c->stream);
  *out = c;
  return GG_OK;
}

int gg_destroy(gg_ctx *ctx) {
  if (!ctx) return GG_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->release();
  delete ctx;
  return GG_OK;
}

int gg_last_error(const gg_ctx *ctx, char *buf, size_t len) {
  if (!buf || len == 0) return GG_ERR_ARG;
  const std::string &m = ctx ? ctx->err : g_create_error;
  size_t n = std::min(len - 1, m.size());
  memcpy(buf, m.data(), n);
  buf[n] = 0;
  return GG_OK;
}

int gg_upload_tables(gg_ctx *c, const gg_tables_desc *t) {
  if (!c || !t) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  char msg[160];
  if (gg::check_tables(t, msg, sizeof(msg))) return c->fail(GG_ERR_ARG, "gg_upload_tables: %s", msg);
  size_t nce = (size_t)t->n_comp * t->n_e;
  // tables plus the transport block's two per-history voxel lists
  size_t need = c->precision == GG_PREC_F64
                    ? gg::transport_smem_bytes<double>(t->n_comp, t->n_e, t->n_mat) + gg::hist_list_bytes<double>(2)
                    : gg::transport_smem_bytes<float>(t->n_comp, t->n_e, t->n_mat) + gg::hist_list_bytes<float>(2);
  if (need > (size_t)gg::kTransportSmemMax)
    return c->fail(GG_ERR_ARG, "gg_upload_tables: tables and voxel lists need %zu bytes of shared memory (max %d)",
                   need, gg::kTransportSmemMax);
  if (c->tle && (t->n_e != c->n_e || t->n_comp != c->n_comp)) c->tle = false;  // its table no longer fits
  c->n_e = t->n_e;
  c->n_comp = t->n_comp;
  c->n_ray = t->n_ray;
  c->n_mat = t->n_mat;
  c->ln_emin = t->ln_emin;
  c->inv_dln = t->inv_dln;
  c->e_min = t->e_min;
  c->e_max = t->e_max;
  int st;
  if ((st = c->upload_real(c->d_sig, t->sig, nce))) return st;
  if ((st = c->upload_real(c->d_cum, t->cum, 3 * nce))) return st;
  if ((st = c->upload_real(c->d_ray_amax, t->ray_amax, nce))) return st;
  if ((st = c->upload_real(c->d_ray_cum, t->ray_cum, (size_t)t->n_comp * t->n_ray))) return st;
  if ((st = c->upload_real(c->d_ray_x2, t->ray_x2, (size_t)t->n_ray))) return st;
  if ((st = c->upload_real(c->d_mat_rho, t->mat_rho, (size_t)t->n_mat))) return st;
  dfree(c->d_mat_comp);
  if ((st = c->cuda(cudaMalloc(&c->d_mat_comp, sizeof(int) * t->n_mat), "cudaMalloc"))) return st;
  if ((st = c->h2d(c->d_mat_comp, t->mat_comp, sizeof(int) * t->n_mat,
                    "cudaMemcpy")))
    return st;
  c->h_mat_comp.assign(t->mat_comp, t->mat_comp + t->n_mat);
  c->h_mat_rho.assign(t->mat_rho, t->mat_rho + t->n_mat);
  c->have_tables = true;
  return GG_OK;
}

// Device label image of n voxels: the allocation is kept when it is large
// enough (a re-upload of the same scene allocates nothing).
static int labels_alloc(gg_ctx *c, size_t n) {
  if (c->d_labels && c->labels_cap >= n) return GG_OK;
  dfree(c->d_labels);
  c->labels_cap = 0;
  int st = c->cuda(cudaMalloc(&c->d_labels, n * sizeof(uint16_t)), "cudaMalloc labels");
  if (!st) c->labels_cap = n;
  return st;
}

int gg_upload_volume(gg_ctx *c, const gg_volume_desc *v) {
  if (c) {
    c->have_batch = false;  // a single image replaces the batched simulations
    drop_graph(c);
  }
  if (!c || !v) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_tables) return c->fail(GG_ERR_STATE, "gg_upload_volume: upload the tables first");
  for (int a = 0; a < 3; ++a)
    if (!(v->spacing[a] > 0) || !std::isfinite(v->spacing[a]))
      return c->fail(GG_ERR_ARG, "gg_upload_volume: spacing must be finite and > 0");
  if (!v->labels || !v->majorant) return c->fail(GG_ERR_ARG, "gg_upload_volume: null labels or majorant");
  char msg[160];
  size_t n = 0;
  if (gg::check_dims(v->dims, (size_t)UINT32_MAX - 1, &n, msg, sizeof(msg)))
    return c->fail(GG_ERR_ARG, "gg_upload_volume: %s", msg);
  uint16_t lmax = 0;
  for (size_t i = 0; i < n; ++i) lmax = std::max(lmax, v->labels[i]);
  if ((int)lmax >= c->n_mat)
    return c->fail(GG_ERR_ARG, "gg_upload_volume: label %u outside the material table (%d)", lmax, c->n_mat);
  if (gg::check_majorant(v->majorant, c->n_e, msg, sizeof(msg))) return c->fail(GG_ERR_ARG, "gg_upload_volume: %s", msg);
  int st;
  if ((st = labels_alloc(c, n))) return st;
  if ((st = c->cuda(cudaMemcpyAsync(c->d_labels, v->labels, n * sizeof(uint16_t), cudaMemcpyHostToDevice, c->stream),
                    "cudaMemcpy labels")))
    return st;
  if ((st = c->upload_real(c->d_maj, v->majorant, (size_t)c->n_e))) return st;
  if (n != c->n_vox && !c->dgrid_on) {
    dfree(c->d_acc_e); dfree(c->d_acc_e2); dfree(c->d_edep); dfree(c->d_edep2);
    c->n_tally = 0;
    c->have_tally = false;
  }
  for (int a = 0; a < 3; ++a) {
    c->dims[a] = v->dims[a];
    c->spacing[a] = v->spacing[a];
    c->corner[a] = v->corner[a];
  }
  c->n_vox = n;
  c->have_volume = true;
  return c->cuda(cudaStreamSynchronize(c->stream), "upload volume");
}

int gg_set_world(gg_ctx *c, const gg_world_desc *w) {
  if (!c || !w) return GG_ERR_ARG;
  if (!c->have_tables) return c->fail(GG_ERR_STATE, "gg_set_world: upload the tables first");
  if (w->material < 0 || w->material >= c->n_mat) return c->fail(GG_ERR_ARG, "gg_set_world: bad material");
  for (int a = 0; a < 3; ++a)
    if (!(w->half_size[a] > 0)) return c->fail(GG_ERR_ARG, "gg_set_world: half sizes must be > 0");
  c->world = *w;
  c->have_world = true;
  return GG_OK;
}

int gg_set_source(gg_ctx *c, const gg_source_desc *s) {
  if (!c || !s) return GG_ERR_ARG;
  if (c->have_batch) return c->fail(GG_ERR_STATE, "gg_set_source: batched simulations carry their own sources");
  cudaSetDevice(c->device);
  if (!c->have_tables) return c->fail(GG_ERR_STATE, "gg_set_source: upload the tables first");
  if (s->pos_type < GG_POS_POINT || s->pos_type > GG_POS_VOXELS) return c->fail(GG_ERR_ARG, "gg_set_source: position type");
  if (s->dir_type < GG_DIR_ISO || s->dir_type > GG_DIR_FORCED) return c->fail(GG_ERR_ARG, "gg_set_source: direction type");
  if (s->dir_type == GG_DIR_FORCED &&
      !(s->fd_cos_min <= 1.0 && s->fd_cos_max >= -1.0 && s->fd_cos_max < s->fd_cos_min))
    return c->fail(GG_ERR_ARG, "gg_set_source: forced direction needs -1 <= cos(max angle) < cos(min angle) <= 1");
  if (s->ene_type < GG_ENE_MONO || s->ene_type > GG_ENE_RANGE) return c->fail(GG_ERR_ARG, "gg_set_source: energy type");
  if (s->n_accept < 0 || (s->n_accept > 0 && !s->accept_boxes)) return c->fail(GG_ERR_ARG, "gg_set_source: acceptance boxes");
  double elo = 0, ehi = 0;
  char msg[160];
  if (gg::check_source_energy(s, &elo, &ehi, msg, sizeof(msg))) return c->fail(GG_ERR_ARG, "gg_set_source: %s", msg);
  c->src_emax = ehi;
  if (!(elo >= c->e_min) || !(ehi <= c->e_max))
    return c->fail(GG_ERR_DOMAIN, "gg_set_source: energies [%g, %g] MeV outside the tables [%g, %g]", elo, ehi,
                   (double)c->e_min, (double)c->e_max);
  int st;
  int ne = s->ene_type == GG_ENE_HISTOGRAM ? s->n_spec + 1 : s->n_spec;
  if ((st = c->upload_real_d(c->d_spec_e, s->spec_e, s->spec_e ? (size_t)ne : 0))) return st;
  if ((st = c->upload_real_d(c->d_spec_cdf, s->spec_cdf, s->spec_cdf ? (size_t)s->n_spec : 0))) return st;
  if ((st = c->upload_real_d(c->d_acc_box, s->accept_boxes, (size_t)6 * s->n_accept))) return st;
  if (s->pos_type == GG_POS_VOXELS) {
    size_t nz = (size_t)s->vox_dims[2], ny = (size_t)s->vox_dims[1], nx = (size_t)s->vox_dims[0];
    if (!s->vox_dims[0] || !s->vox_dims[1] || !s->vox_dims[2] || s->vox_dims[0] < 0 || s->vox_dims[1] < 0 ||
        s->vox_dims[2] < 0 || !s->cdf_z || !s->cdf_y || !s->cdf_x)
      return c->fail(GG_ERR_ARG, "gg_set_source: voxel source needs dims and the three CDFs");
    for (int a = 0; a < 3; ++a)
      if (!(s->vox_spacing[a] > 0)) return c->fail(GG_ERR_ARG, "gg_set_source: voxel spacing must be > 0");
    if ((st = c->upload_real(c->d_cdf_z, s->cdf_z, nz))) return st;
    if ((st = c->upload_real(c->d_cdf_y, s->cdf_y, nz * ny))) return st;
    if ((st = c->upload_real(c->d_cdf_x, s->cdf_x, nz * ny * nx))) return st;
  }
  c->src = *s;
  c->src.cdf_z = c->src.cdf_y = c->src.cdf_x = nullptr;
  c->src.spec_e = nullptr;
  c->src.spec_cdf = nullptr;
  c->src.accept_boxes = nullptr;
  c->have_source = true;
  return GG_OK;
}

int gg_add_dose_tally(gg_ctx *c, int32_t score_squared) {
  if (!c) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_volume) return c->fail(GG_ERR_STATE, "gg_add_dose_tally: upload the volume first");
  c->squared = score_squared != 0;
  int st = tally_alloc(c);
  if (st) return st;
  c->have_tally = true;
  return gg_reset_tally(c);
}

int gg_set_dose_grid(gg_ctx *c, const gg_dose_grid_desc *d) {
  if (!c) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_tables) return c->fail(GG_ERR_STATE, "gg_set_dose_grid: upload the tables first");
  if (c->have_batch || c->have_spect)
    return c->fail(GG_ERR_STATE, "gg_set_dose_grid: dose grids are for single dose simulations");
  if (!d || d->dims[0] == 0) {
    c->dgrid_on = false;
    c->ddose = false;
  } else {
    char msg[160];
    size_t n = 0;
    if (gg::check_dims(d->dims, (size_t)UINT32_MAX - 1, &n, msg, sizeof(msg)))
      return c->fail(GG_ERR_ARG, "gg_set_dose_grid: %s", msg);
    for (int a = 0; a < 3; ++a)
      if (!(d->spacing[a] > 0) || !std::isfinite(d->spacing[a]) || !std::isfinite(d->corner[a]))
        return c->fail(GG_ERR_ARG, "gg_set_dose_grid: spacing must be finite and > 0, corner finite");
    c->dgrid_on = true;
    c->ddose = d->score_dose != 0;
    for (int a = 0; a < 3; ++a) {
      c->ddims[a] = d->dims[a];
      c->dspacing[a] = d->spacing[a];
      c->dcorner[a] = d->corner[a];
    }
    float rmin = c->h_mat_rho.empty() ? 1.0f : c->h_mat_rho[0];
    for (float r : c->h_mat_rho) rmin = std::min(rmin, r);
    c->drho_min = rmin;
  }
  int st = tally_alloc(c);
  if (st) return st;
  c->have_tally = c->d_acc_e != nullptr;
  return c->have_tally ? gg_reset_tally(c) : GG_OK;
}

int gg_spect_set_blur(gg_ctx *c, const gg_blur_desc *b) {
  if (!c || !b) return GG_ERR_ARG;
  if (b->energy_method < GG_BLUR_NONE || b->energy_method > GG_BLUR_LINEAR)
    return c->fail(GG_ERR_ARG, "gg_spect_set_blur: unknown energy blurring method %d", b->energy_method);
  if (b->energy_method == GG_BLUR_GAUSSIAN && !(b->energy_sigma >= 0))
    return c->fail(GG_ERR_ARG, "gg_spect_set_blur: energy sigma must be >= 0");
  if ((b->energy_method == GG_BLUR_INVERSE_SQUARE || b->energy_method == GG_BLUR_LINEAR) &&
      (!(b->energy_resolution >= 0) || !(b->energy_reference >= 0) || !std::isfinite(b->energy_slope)))
    return c->fail(GG_ERR_ARG, "gg_spect_set_blur: resolution and reference must be >= 0");
  if (b->spatial && (!(b->spatial_sigma[0] >= 0) || !(b->spatial_sigma[1] >= 0)))
    return c->fail(GG_ERR_ARG, "gg_spect_set_blur: spatial sigma must be >= 0");
  if (b->spatial && b->truncated && (!(b->spatial_sigma[0] > 0) || !(b->spatial_sigma[1] > 0)))
    return c->fail(GG_ERR_ARG, "gg_spect_set_blur: the truncated Gaussian needs sigma > 0");
  c->blur = *b;
  return GG_OK;
}

int gg_set_tle(gg_ctx *c, const gg_tle_desc *d) {
  if (!c || !d) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!d->enabled) {
    c->tle = false;
    return GG_OK;
  }
  if (!c->d_sig) return c->fail(GG_ERR_STATE, "gg_set_tle: upload the physics tables first");
  if (c->have_batch) return c->fail(GG_ERR_STATE, "gg_set_tle: batched simulations do not support the estimator");
  if (!d->muen) return c->fail(GG_ERR_ARG, "gg_set_tle: no mu_en table");
  if (std::isnan(d->threshold_energy) || !(d->energy_min >= 0) || !std::isfinite(d->energy_min))
    return c->fail(GG_ERR_ARG, "gg_set_tle: invalid threshold or kill energy");
  const size_t nce = (size_t)c->n_comp * c->n_e;
  for (size_t i = 0; i < nce; ++i)
    if (!(d->muen[i] >= 0) || !std::isfinite(d->muen[i]))
      return c->fail(GG_ERR_ARG, "gg_set_tle: mu_en table has a negative or non-finite entry");
  int st;
  if ((st = c->upload_real(c->d_muen, d->muen, nce))) return st;
  c->tle = true;
  c->tle_thr = d->threshold_energy;
  c->tle_emin = d->energy_min;
  return GG_OK;
}

int gg_reset_tally(gg_ctx *c) {
  if (!c) return GG_ERR_ARG;
  if (!c->have_tally) return c->fail(GG_ERR_STATE, "gg_reset_tally: no tally");
  cudaSetDevice(c->device);
  size_t n = c->n_tally;
  int st;
  if ((st = c->cuda(cudaMemsetAsync(c->d_acc_e, 0, n * 8, c->stream), "memset"))) return st;
  if ((st = c->cuda(cudaMemsetAsync(c->d_edep, 0, n * 8, c->stream), "memset"))) return st;
  if (c->d_acc_e2) {
    if ((st = c->cuda(cudaMemsetAsync(c->d_acc_e2, 0, n * 16, c->stream), "memset"))) return st;
    if ((st = c->cuda(cudaMemsetAsync(c->d_edep2, 0, n * 8, c->stream), "memset"))) return st;
  }
  if (c->d_acc_d) {
    if ((st = c->cuda(cudaMemsetAsync(c->d_acc_d, 0, n * 8, c->stream), "memset"))) return st;
    if ((st = c->cuda(cudaMemsetAsync(c->d_dose, 0, n * 8, c->stream), "memset"))) return st;
  }
  if (c->d_acc_d2) {
    if ((st = c->cuda(cudaMemsetAsync(c->d_acc_d2, 0, n * 16, c->stream), "memset"))) return st;
    if ((st = c->cuda(cudaMemsetAsync(c->d_dose2, 0, n * 8, c->stream), "memset"))) return st;
  }
  if ((st = c->cuda(cudaMemsetAsync(c->d_counters, 0, GG_N_COUNTERS * 8, c->stream), "memset"))) return st;
  return c->cuda(cudaMemsetAsync(c->d_status, 0, sizeof(unsigned int), c->stream), "memset");
}

static int upload_frames(gg_ctx *c) {
  if (!c->frames_dirty && c->d_frames) return GG_OK;
  int st = c->upload_real_d(c->d_frames, c->frames.data(), c->frames.size());
  if (st) return st;
  c->frames_dirty = false;
  return GG_OK;
}

// Records a start / end event of a stage launch (events are reused across runs).
static int stage_event(gg_ctx *c, int kind, bool start) {
  const size_t k = c->stage_kind.size() * 2 + (start ? 0 : 1);
  while (c->stage_ev.size() <= k) {
    cudaEvent_t e;
    int st = c->cuda(cudaEventCreate(&e), "cudaEventCreate");
    if (st) return st;
    c->stage_ev.push_back(e);
  }
  int st = c->cuda(cudaEventRecord(c->stage_ev[k], c->stream), "event");
  if (st) return st;
  if (!start) c->stage_kind.push_back(kind);
  return GG_OK;
}

// Adds the times of the recorded stage launches (stream synchronised) and forgets them.
static void stage_collect(gg_ctx *c) {
  for (size_t i = 0; i < c->stage_kind.size(); ++i) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c->stage_ev[2 * i], c->stage_ev[2 * i + 1]) == cudaSuccess)
      c->stage_ms[c->stage_kind[i]] += ms;
  }
  c->stage_kind.clear();
}

// Longest head queue of scatter splitting (entries).
static constexpr size_t kSsQueueMax = (size_t)1 << 26;

// SPECT transport of one batch: phantom stage on the primary records, head
// stage on the head queue, then phantom / head passes on the photons that
// flew back into the image until the return queue stays empty.
static int spect_stages(gg_ctx *c, gg::KernelArgs a, size_t smem, int minb) {
  int bps[2] = {0, 0};
  for (int stage = 0; stage < 2; ++stage) {
    cudaError_t e = c->precision == GG_PREC_F64
                        ? gg::spect_stage_occupancy<double>(stage, c->block, smem, minb, &bps[stage])
                        : gg::spect_stage_occupancy<float>(stage, c->block, smem, minb, &bps[stage]);
    if (e != cudaSuccess) return c->cuda(e, "occupancy");
    if (bps[stage] < 1) bps[stage] = 1;
  }
  unsigned long long *nh = c->d_qn, *nr = c->d_qn + 1, *nf = c->d_qn + 2;
  auto stage_run = [&](int stage, void *in_q, const unsigned long long *in_n, void *out_q,
                       unsigned long long *out_n) -> int {
    gg::StageArgs q{in_q, in_n, out_q, out_n, c->q_cap, c->d_split, c->d_split_n, c->split_cap};
    int st;
    if ((st = c->cuda(cudaMemsetAsync(out_n, 0, sizeof(unsigned long long), c->stream), "memset"))) return st;
    if ((st = c->cuda(cudaMemsetAsync(c->d_next, 0, 8, c->stream), "memset"))) return st;
    int grid = c->n_sm * bps[stage];
    if ((st = stage_event(c, stage, true))) return st;
    cudaError_t e = c->precision == GG_PREC_F64
                        ? gg::launch_spect_stage<double>(stage, c->scene<double>(), a, q, grid, c->block, smem, minb,
                                                         c->stream)
                        : gg::launch_spect_stage<float>(stage, c->scene<float>(), a, q, grid, c->block, smem, minb,
                                                        c->stream);
    if ((st = c->cuda(e, "SPECT stage launch"))) return st;
    return stage_event(c, stage, false);
  };
  // ARF stage between the phantom and the head stage: head queue -> network
  // (projection weights) + fallback queue for the head stage
  auto arf_run = [&]() -> int {
    int st;
    if ((st = c->cuda(cudaMemsetAsync(nf, 0, sizeof(unsigned long long), c->stream), "memset"))) return st;
    if ((st = c->cuda(cudaMemsetAsync(c->d_next, 0, sizeof(unsigned long long), c->stream), "memset"))) return st;
    gg::ArfStageArgs q{};
    q.claim = c->d_next;
    q.in_q = c->d_queue[0];
    q.in_n = nh;
    q.out_q = c->d_queue[2];
    q.out_n = nf;
    q.q_cap = c->q_cap;
    q.params = c->d_params;
    q.wbf = c->d_wbf;
    for (int k = 0; k < 3; ++k) {
      q.mean[k] = c->arf.x_mean[k];
      q.inv_std[k] = 1.0f / c->arf.x_std[k];
    }
    q.n_classes = c->arf.n_classes;
    q.rr = (float)c->arf.russian_roulette;
    q.e_min = c->arf.e_min;
    q.e_max = c->arf.e_max;
    q.cos_theta_max = std::cos(c->arf.theta_max_deg * (M_PI / 180.0));
    double lo = c->spect.window_lo[0];
    for (int k = 1; k < c->spect.n_windows; ++k) lo = std::min(lo, c->spect.window_lo[k]);
    q.e_detect_min = lo;
    q.dc = c->arf.distance_to_crystal;
    q.proj = c->d_arf_proj;
    q.proj2 = c->d_arf_proj2;
    q.counters = c->d_counters;
    q.status = c->d_status;
    if ((st = stage_event(c, 2, true))) return st;
    cudaError_t e = c->precision == GG_PREC_F64 ? gg::launch_spect_arf<double>(c->scene<double>(), q, c->n_sm, c->stream)
                                                : gg::launch_spect_arf<float>(c->scene<float>(), q, c->n_sm, c->stream);
    if ((st = c->cuda(e, "ARF stage launch"))) return st;
    return stage_event(c, 2, false);
  };
  auto head_pass = [&]() -> int {
    int st;
    if (c->arf_on) {
      if ((st = arf_run())) return st;
      return stage_run(1, c->d_queue[2], nf, c->d_queue[1], nr);
    }
    return stage_run(1, c->d_queue[0], nh, c->d_queue[1], nr);
  };
  const int per_pass = c->arf_on ? 3 : 2;
  int st;
  if (c->ff_on && c->ff_mode == GG_FF_SCATTER) {
    // scatter splitting: analog photons never return from the heads; the
    // phantom stage runs on spans of the batch whose copies fit the head
    // queue.  A span that overflowed scored nothing yet (only the head stage
    // scores), so it is repeated, shorter, after its counters are restored.
    if (!c->d_cnt_save &&
        (st = c->cuda(cudaMalloc(&c->d_cnt_save, GG_N_COUNTERS * sizeof(unsigned long long)), "cudaMalloc counters")))
      return st;
    // copies: split kernel (requests -> walk queue, the unused return queue),
    // then their free flights (walk queue -> head queue)
    auto split_run = [&]() -> int {
      gg::StageArgs q{nullptr, nullptr, c->d_queue[1], nr, c->q_cap, c->d_split, c->d_split_n, c->split_cap};
      int st2;
      if ((st2 = c->cuda(cudaMemsetAsync(nr, 0, sizeof(unsigned long long), c->stream), "memset"))) return st2;
      if ((st2 = stage_event(c, 2, true))) return st2;
      cudaError_t e = c->precision == GG_PREC_F64
                          ? gg::launch_spect_split<double>(c->scene<double>(), a, q, c->block, smem, c->n_sm, c->stream)
                          : gg::launch_spect_split<float>(c->scene<float>(), a, q, c->block, smem, c->n_sm, c->stream);
      if ((st2 = c->cuda(e, "split kernel launch"))) return st2;
      gg::StageArgs w{c->d_queue[1], nr, c->d_queue[0], nh, c->q_cap, nullptr, nullptr, 0};
      e = c->precision == GG_PREC_F64
              ? gg::launch_spect_walk<double>(c->scene<double>(), a, w, c->block, smem, c->n_sm, c->stream)
              : gg::launch_spect_walk<float>(c->scene<float>(), a, w, c->block, smem, c->n_sm, c->stream);
      if ((st2 = c->cuda(e, "walk kernel launch"))) return st2;
      return stage_event(c, 2, false);
    };
    const uint64_t h_end = a.h_end;
    uint64_t lo = a.h_begin;
    c->last_stage_launches = 0;
    while (lo < h_end) {
      if (c->ss_span == 0) c->ss_span = h_end - lo;
      a.h_begin = lo;
      a.h_end = lo + std::min<uint64_t>(c->ss_span, h_end - lo);
      if ((st = c->cuda(cudaMemcpyAsync(c->d_cnt_save, c->d_counters, GG_N_COUNTERS * sizeof(unsigned long long),
                                        cudaMemcpyDeviceToDevice, c->stream),
                        "save counters")))
        return st;
      if ((st = c->cuda(cudaMemsetAsync(c->d_split_n, 0, 2 * sizeof(unsigned long long), c->stream), "memset")))
        return st;
      if ((st = stage_run(0, nullptr, nullptr, c->d_queue[0], nh))) return st;
      if ((st = split_run())) return st;
      unsigned long long len[3] = {0, 0, 0};
      if ((st = c->cuda(cudaMemcpyAsync(len, c->d_split_n, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                        c->stream),
                        "split requests")) ||
          (st = c->cuda(cudaMemcpyAsync(len + 2, nr, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream),
                        "queue length")))
        return st;
      if ((st = c->cuda(cudaStreamSynchronize(c->stream), "SPECT phantom stage"))) return st;
      stage_collect(c);
      c->last_stage_launches += 3;
      // the head queue holds a subset of the walk queue
      const double fill = std::max((double)(len[0] + len[1]) / (double)c->split_cap, (double)len[2] / (double)c->q_cap);
      if (fill > 1.0) {
        const uint64_t span = a.h_end - a.h_begin;
        if (span == 1)
          return c->fail(GG_ERR_QUEUE_OVERFLOW, "SPECT stages: the split copies of one history overflow the queues");
        if ((st = c->cuda(cudaMemcpyAsync(c->d_counters, c->d_cnt_save, GG_N_COUNTERS * sizeof(unsigned long long),
                                          cudaMemcpyDeviceToDevice, c->stream),
                          "restore counters")))
          return st;
        // requests / copies per history of this span, with a margin
        c->ss_span = std::max<uint64_t>(1, std::min<uint64_t>(span / 2, (uint64_t)(0.85 * (double)span / fill)));
        continue;
      }
      if ((st = head_pass())) return st;
      c->last_stage_launches += c->arf_on ? 2 : 1;
      lo = a.h_end;
    }
    if ((st = c->cuda(cudaStreamSynchronize(c->stream), "SPECT head stage"))) return st;
    stage_collect(c);
    return GG_OK;
  }
  // primary free flight: the phantom stage checks the flights and queues the
  // photons that pass (third queue); their optical depths are walked by the
  // walk kernel, one photon per thread, into the head queue
  const bool ffp = c->ff_on && c->ff_mode == GG_FF_PRIMARY;
  auto phantom_pass = [&](void *in_q, const unsigned long long *in_n) -> int {
    if (!ffp) return stage_run(0, in_q, in_n, c->d_queue[0], nh);
    int st2;
    if ((st2 = stage_run(0, in_q, in_n, c->d_queue[2], nf))) return st2;
    if ((st2 = c->cuda(cudaMemsetAsync(nh, 0, sizeof(unsigned long long), c->stream), "memset"))) return st2;
    gg::StageArgs w{c->d_queue[2], nf, c->d_queue[0], nh, c->q_cap, nullptr, nullptr, 0};
    if ((st2 = stage_event(c, 0, true))) return st2;
    cudaError_t e = c->precision == GG_PREC_F64
                        ? gg::launch_spect_walk<double>(c->scene<double>(), a, w, c->block, smem, c->n_sm, c->stream)
                        : gg::launch_spect_walk<float>(c->scene<float>(), a, w, c->block, smem, c->n_sm, c->stream);
    if ((st2 = c->cuda(e, "walk kernel launch"))) return st2;
    return stage_event(c, 0, false);
  };
  const int per_phantom = ffp ? 2 : 1;
  if ((st = phantom_pass(nullptr, nullptr))) return st;
  if ((st = head_pass())) return st;
  c->last_stage_launches = per_pass + per_phantom - 1;
  for (int pass = 1;; ++pass) {
    unsigned long long back = 0;
    if ((st = c->cuda(cudaMemcpyAsync(&back, nr, sizeof(back), cudaMemcpyDeviceToHost, c->stream), "queue length")))
      return st;
    if ((st = c->cuda(cudaStreamSynchronize(c->stream), "SPECT stages"))) return st;
    stage_collect(c);
    if (back == 0) break;
    // a photon re-enters the image at most once per phantom / head pass; the
    // per-photon step cap ends every history, so this loop ends too
    if (pass > 100000) return c->fail(GG_ERR_DOMAIN, "SPECT stages: photons keep returning to the image");
    if ((st = phantom_pass(c->d_queue[1], nr))) return st;
    if ((st = head_pass())) return st;
    c->last_stage_launches += per_pass + per_phantom - 1;
  }
  return GG_OK;
}

// capturing: enqueue the launches only (no events, no host synchronisation),
// for a CUDA-graph capture of the stream
static int run_impl(gg_ctx *c, uint64_t n, uint64_t seed, uint64_t first, bool capturing = false) {
  size_t smem = c->precision == GG_PREC_F64 ? gg::transport_smem_bytes<double>(c->n_comp, c->n_e, c->n_mat)
                                            : gg::transport_smem_bytes<float>(c->n_comp, c->n_e, c->n_mat);
  // kernel variant: register budget for `minb` resident 256-thread blocks
  // batched simulations bind their geometry per history: more live registers, default 2 blocks / SM;
  // the track-length estimator's voxel walks: 3 (80 registers: 34.3 ms per 1e7 pencil primaries
  // against 36.5 at 4 blocks / SM)
  const bool tle_run = c->tle && !c->have_spect && !c->have_batch;
  int minb = c->blocks_per_sm > 0 ? std::min(c->blocks_per_sm, 4)
                                  : ((c->precision == GG_PREC_F64 || c->have_batch) ? 2 : (tle_run ? 3 : 4));
  int bps = 0;
  {
    // (occupancy_blocks counts one voxel list per thread; a dose grid scoring dose keeps two)
    const bool two_lists = c->dgrid_on && c->ddose && !c->have_spect && !c->have_batch;
    const size_t smem_occ = smem + (two_lists ? (c->precision == GG_PREC_F64 ? gg::hist_list_bytes<double>(1, c->block)
                                                                             : gg::hist_list_bytes<float>(1, c->block))
                                              : 0);
    cudaError_t e = c->precision == GG_PREC_F64 ? gg::occupancy_blocks<double>(c->block, smem_occ, minb, &bps)
                                                : gg::occupancy_blocks<float>(c->block, smem_occ, minb, &bps);
    if (e != cudaSuccess) return c->cuda(e, "occupancy");
    if (bps < 1) bps = 1;
  }
  int grid = c->n_sm * bps;
  // the compacted wavefront kernel: single dose simulations with analog scoring
  if (c->dgrid_on && c->tle && !c->have_spect && !c->have_batch)
    return c->fail(GG_ERR_STATE, "gg_run: the track-length estimator scores on the image grid (no dose grid)");
  if (!c->have_batch && c->src.dir_type == GG_DIR_FORCED &&
      !(c->have_spect && c->ff_on && c->ff_mode == GG_FF_PRIMARY))
    return c->fail(GG_ERR_STATE, "gg_run: a forced-direction source needs SPECT heads and primary free flight");
  const bool wave = !c->have_spect && !c->tle && !c->have_batch && !c->dgrid_on &&
                    c->transport_kernel == GG_KERNEL_WAVEFRONT;
  size_t wsmem = 0;
  int wgrid = 0, wminb = c->precision == GG_PREC_F64 ? 2 : 3;
  if (wave) {
    wsmem = c->precision == GG_PREC_F64 ? gg::wavefront_smem_bytes<double>(c->n_comp, c->n_e, c->n_mat)
                                        : gg::wavefront_smem_bytes<float>(c->n_comp, c->n_e, c->n_mat);
    if (wsmem > 220 * 1024)
      return c->fail(GG_ERR_ARG, "gg_run: tables and photon slots need %zu bytes of shared memory (max 220 KiB); "
                     "use the phase kernel (gg_set_transport_kernel)", wsmem);
    int wbps = 0;
    cudaError_t e = c->precision == GG_PREC_F64 ? gg::wavefront_occupancy<double>(wsmem, wminb, &wbps)
                                                : gg::wavefront_occupancy<float>(wsmem, wminb, &wbps);
    if (e != cudaSuccess) return c->cuda(e, "wavefront occupancy");
    if (wbps < 1) return c->fail(GG_ERR_CUDA, "gg_run: the wavefront kernel does not fit an SM");
    wgrid = c->n_sm * wbps;
  }
  // Histories per tally batch.  The fixed-point dose tallies cannot wrap within
  // a batch: a history deposits at most E_max in total, so over n histories a
  // voxel's edep^2 high word (units of 2^32 of (2^-32 MeV)^2) gains at most
  // n E_max^2 2^32 and its edep word n E_max 2^32; n <= 2^32 / E_max^2 (and
  // 2^32 / E_max) keeps both below 2^64.
  uint64_t batch = (uint64_t)c->batch;
  if (c->have_tally && !c->have_spect) {
    const double em = std::max(c->src_emax, 1e-6) * 1.001;
    const double lim = std::min(4294967296.0 / (em * em), 4294967296.0 / em);
    if ((double)batch > lim) batch = std::max<uint64_t>(1, (uint64_t)lim);
  }
  c->last_batch = batch;
  uint64_t nb = (n + batch - 1) / batch;
  size_t cap = (size_t)std::min<uint64_t>(n, batch);
  if (cap > c->rec_cap) {
    dfree(c->d_records);
    c->rec_cap = 0;
    size_t bytes = c->precision == GG_PREC_F64 ? gg::record_bytes<double>(cap) : gg::record_bytes<float>(cap);
    int st = c->cuda(cudaMalloc(&c->d_records, bytes), "cudaMalloc primary records");
    if (st) return st;
    c->rec_cap = cap;
  }
  // scatter splitting pushes several copies per history: a longer head queue
  // (the phantom passes adapt to it)
  const size_t q_need = c->ff_on && c->ff_mode == GG_FF_SCATTER ? std::max(cap, std::min(cap * 16, kSsQueueMax)) : cap;
  // the third queue: the ARF stage's fallback photons, and the walk queue of primary free flight
  const bool q3 = c->arf_on || (c->ff_on && c->ff_mode == GG_FF_PRIMARY);
  if (c->have_spect && (q_need > c->q_cap || (q3 && !c->d_queue[2]))) {
    for (int k = 0; k < 3; ++k) dfree(c->d_queue[k]);
    c->q_cap = 0;
    size_t qb = c->precision == GG_PREC_F64 ? gg::queue_bytes<double>(q_need) : gg::queue_bytes<float>(q_need);
    int st = c->cuda(cudaMalloc(&c->d_queue[0], qb), "cudaMalloc head queue");
    if (!st) st = c->cuda(cudaMalloc(&c->d_queue[1], qb), "cudaMalloc return queue");
    if (!st && q3) st = c->cuda(cudaMalloc(&c->d_queue[2], qb), "cudaMalloc ARF fallback / walk queue");
    if (!st && !c->d_qn) st = c->cuda(cudaMalloc(&c->d_qn, 3 * sizeof(unsigned long long)), "cudaMalloc queue lengths");
    if (st) return st;
    c->q_cap = q_need;
  }
  if (c->have_spect && c->ff_on && c->ff_mode == GG_FF_SCATTER && c->split_cap < q_need) {
    // split requests: one per split interaction (a few per history)
    dfree(c->d_split);
    c->split_cap = 0;
    size_t sb = c->precision == GG_PREC_F64 ? gg::split_bytes<double>(q_need) : gg::split_bytes<float>(q_need);
    int st = c->cuda(cudaMalloc(&c->d_split, sb), "cudaMalloc split requests");
    if (!st && !c->d_split_n)
      st = c->cuda(cudaMalloc(&c->d_split_n, 2 * sizeof(unsigned long long)), "cudaMalloc split lengths");
    if (st) return st;
    c->split_cap = q_need;
  }
  while (c->ev.size() < 3 * nb + 1) {
    cudaEvent_t e;
    int st = c->cuda(cudaEventCreate(&e), "cudaEventCreate");
    if (st) return st;
    c->ev.push_back(e);
  }
  gg::KernelArgs a{};
  a.seed = seed;
  a.next = c->d_next;
  a.acc_e = c->d_acc_e;
  a.acc_e2 = c->squared ? c->d_acc_e2 : nullptr;
  const bool dg = c->dgrid_on && !c->have_spect && !c->have_batch;
  a.acc_d = dg && c->ddose ? c->d_acc_d : nullptr;
  a.acc_d2 = dg && c->ddose && c->squared ? c->d_acc_d2 : nullptr;
  a.counters = c->d_counters;
  a.status = c->d_status;
  a.chunk = c->chunk;
  a.records = c->d_records;
  a.rec_cap = c->rec_cap;
  a.refill_min = c->refill_min;
  a.interact_min = c->interact_min;
  int flush_grid = c->n_sm * 8;
  c->run_stage_launches = 0;
  c->stage_ms[0] = c->stage_ms[1] = c->stage_ms[2] = 0;
  c->stage_kind.clear();
  int st;
  // per batch: [ev 3b] generate [ev 3b+1] transport [ev 3b+2] flush [ev 3b+3]
  for (uint64_t b = 0; b < nb; ++b) {
    a.h_begin = first + b * batch;
    a.h_end = std::min(first + n, a.h_begin + batch);
    a.rec_first = a.h_begin;
    if ((st = c->cuda(cudaMemsetAsync(c->d_next, 0, 8, c->stream), "memset"))) return st;
    if (!capturing && (st = c->cuda(cudaEventRecord(c->ev[3 * b], c->stream), "event"))) return st;
    cudaError_t e = c->precision == GG_PREC_F64 ? gg::launch_generate<double>(c->scene<double>(), a, c->stream)
                                                : gg::launch_generate<float>(c->scene<float>(), a, c->stream);
    if ((st = c->cuda(e, "generate launch"))) return st;
    if (!capturing && (st = c->cuda(cudaEventRecord(c->ev[3 * b + 1], c->stream), "event"))) return st;
    if (c->have_spect) {
      if ((st = spect_stages(c, a, smem, minb))) return st;
      c->run_stage_launches += c->last_stage_launches;
    } else if (wave) {
      e = c->precision == GG_PREC_F64
              ? gg::launch_wavefront<double>(c->scene<double>(), a, wgrid, wsmem, wminb, c->stream)
              : gg::launch_wavefront<float>(c->scene<float>(), a, wgrid, wsmem, wminb, c->stream);
      if ((st = c->cuda(e, "wavefront transport launch"))) return st;
    } else {
      e = c->precision == GG_PREC_F64
              ? gg::launch_transport<double>(c->scene<double>(), a, grid, c->block, smem, minb, c->stream)
              : gg::launch_transport<float>(c->scene<float>(), a, grid, c->block, smem, minb, c->stream);
      if ((st = c->cuda(e, "transport launch"))) return st;
    }
    if (!capturing && (st = c->cuda(cudaEventRecord(c->ev[3 * b + 2], c->stream), "event"))) return st;
    if (c->have_tally &&
        (st = c->cuda(gg::launch_flush(c->d_acc_e, a.acc_e2, c->d_edep, c->squared ? c->d_edep2 : nullptr,
                                       c->n_tally, flush_grid, c->stream),
                      "flush launch")))
      return st;
    if (a.acc_d &&
        (st = c->cuda(gg::launch_flush(a.acc_d, a.acc_d2, c->d_dose, a.acc_d2 ? c->d_dose2 : nullptr, c->n_tally,
                                       flush_grid, c->stream, 1.0 / (double)c->drho_min),
                      "dose flush launch")))
      return st;
  }
  if (capturing) return GG_OK;
  if ((st = c->cuda(cudaEventRecord(c->ev[3 * nb], c->stream), "event"))) return st;
  if ((st = c->cuda(cudaStreamSynchronize(c->stream), "transport"))) return st;
  double tg = 0, tt = 0, tf = 0;
  for (uint64_t b = 0; b < nb; ++b) {
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev[3 * b], c->ev[3 * b + 1]);
    tg += ms;
    cudaEventElapsedTime(&ms, c->ev[3 * b + 1], c->ev[3 * b + 2]);
    tt += ms;
    cudaEventElapsedTime(&ms, c->ev[3 * b + 2], c->ev[3 * b + 3]);
    tf += ms;
  }
  c->last_generate_ms = tg;
  c->last_transport_ms = tt;
  c->last_flush_ms = tf;
  c->last_launches = (int)(nb + (c->have_spect ? (uint64_t)c->run_stage_launches : nb) + (c->have_tally ? nb : 0));
  unsigned int status = 0;
  if ((st = c->d2h(&status, c->d_status, sizeof(status), "status"))) return st;
  if (status) {
    cudaMemsetAsync(c->d_status, 0, sizeof(unsigned int), c->stream);
    cudaStreamSynchronize(c->stream);
    if (status & gg::kStatusQueueOverflow)
      return c->fail(GG_ERR_QUEUE_OVERFLOW, "gg_run: a SPECT stage queue overflowed (photons were dropped)");
    if (status & gg::kStatusWaitTimeout)
      return c->fail(GG_ERR_TIMEOUT, "gg_run: a bounded wait ran out (ARF stage tensor cores, or the queues of "
                                     "the wavefront transport); the batch is incomplete");
    return c->fail(GG_ERR_DOMAIN, "gg_run: source sampling failed (angular acceptance exhausted max_rejection)");
  }
  return GG_OK;
}

int gg_run(gg_ctx *c, uint64_t n, uint64_t seed, uint64_t first) {
  if (!c) return GG_ERR_ARG;
  if (c->have_batch) return c->fail(GG_ERR_STATE, "gg_run: batched simulations run with gg_batch_run");
  cudaSetDevice(c->device);
  // SPECT heads are tracked for photons below the pair threshold only (no
  // secondary can be created inside a head)
  if (c->have_spect && !(c->src_emax < 2.0 * gg::kMC2))
    return c->fail(GG_ERR_DOMAIN, "gg_run: SPECT transport needs source energies below 1.022 MeV");
  if (!c->have_tables || !c->have_volume || !c->have_world || !c->have_source || !(c->have_tally || c->have_spect))
    return c->fail(GG_ERR_STATE, "gg_run: tables, volume, world, source and tally must be set first");
  if (n == 0) return GG_OK;
  if (first + n < first) return c->fail(GG_ERR_ARG, "gg_run: history range overflows");
  if (c->have_spect) {
    // every history of this call belongs to the run of the last gg_spect_set_heads
    c->run_base = c->spect_run;
    c->run_first = first;
    c->run_len = n;
    int st = upload_frames(c);
    if (st) return st;
  }
  return run_impl(c, n, seed, first);
}

int gg_set_transport_kernel(gg_ctx *c, int32_t kind) {
  if (!c) return GG_ERR_ARG;
  if (kind != GG_KERNEL_WAVEFRONT && kind != GG_KERNEL_PHASED)
    return c->fail(GG_ERR_ARG, "gg_set_transport_kernel: unknown kernel %d", kind);
  c->transport_kernel = kind;
  return GG_OK;
}

int gg_synchronize(gg_ctx *c) {
  if (!c) return GG_ERR_ARG;
  return c->cuda(cudaStreamSynchronize(c->stream), "synchronize");
}

int gg_get_image(gg_ctx *c, int32_t which, double *out, size_t n) {
  if (!c || !out) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_tally) return c->fail(GG_ERR_STATE, "gg_get_image: no tally");
  if (n != c->n_tally)
    return c->fail(GG_ERR_ARG, "gg_get_image: buffer has %zu voxels, image %zu", n, c->n_tally);
  double *src = nullptr;
  if (which == GG_IMG_EDEP) src = c->d_edep;
  else if (which == GG_IMG_EDEP_SQUARED) src = c->squared ? c->d_edep2 : nullptr;
  else if (which == GG_IMG_DOSE) src = c->dgrid_on && c->ddose ? c->d_dose : nullptr;
  else if (which == GG_IMG_DOSE_SQUARED) src = c->dgrid_on && c->ddose && c->squared ? c->d_dose2 : nullptr;
  if (!src) return c->fail(GG_ERR_ARG, "gg_get_image: image %d not scored", which);
  int st = c->cuda(cudaMemcpyAsync(out, src, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "download");
  if (st) return st;
  return c->cuda(cudaStreamSynchronize(c->stream), "download");
}

int gg_get_image_device(gg_ctx *c, int32_t which, void **ptr, size_t *n) {
  if (!c || !ptr || !n) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_tally) return c->fail(GG_ERR_STATE, "gg_get_image_device: no tally");
  double *src = nullptr;
  if (which == GG_IMG_EDEP) src = c->d_edep;
  else if (which == GG_IMG_EDEP_SQUARED) src = c->squared ? c->d_edep2 : nullptr;
  else if (which == GG_IMG_DOSE) src = c->dgrid_on && c->ddose ? c->d_dose : nullptr;
  else if (which == GG_IMG_DOSE_SQUARED) src = c->dgrid_on && c->ddose && c->squared ? c->d_dose2 : nullptr;
  if (!src) return c->fail(GG_ERR_ARG, "gg_get_image_device: image %d not scored", which);
  int st = c->cuda(cudaStreamSynchronize(c->stream), "gg_get_image_device");
  if (st) return st;
  *ptr = src;
  *n = c->n_tally;
  return GG_OK;
}

void *gg_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (bytes == 0 || cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}

int gg_host_free(void *p) {
  if (!p) return GG_OK;
  return cudaFreeHost(p) == cudaSuccess ? GG_OK : GG_ERR_CUDA;
}

int gg_get_counters(gg_ctx *c, uint64_t *out, size_t n) {
  if (!c || !out) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  unsigned long long tmp[GG_N_COUNTERS];
  int st = c->d2h(tmp, c->d_counters, sizeof(tmp), "counters");
  if (st) return st;
  for (size_t i = 0; i < n && i < GG_N_COUNTERS; ++i) out[i] = tmp[i];
  return GG_OK;
}

int gg_last_kernel_ms(gg_ctx *c, double *generate_ms, double *transport_ms, double *flush_ms,
                      int32_t *launches) {
  if (!c) return GG_ERR_ARG;
  if (generate_ms) *generate_ms = c->last_generate_ms;
  if (transport_ms) *transport_ms = c->last_transport_ms;
  if (flush_ms) *flush_ms = c->last_flush_ms;
  if (launches) *launches = c->last_launches;
  return GG_OK;
}

int gg_spect_setup(gg_ctx *c, const gg_spect_desc *sp) {
  if (!c || !sp) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_tables) return c->fail(GG_ERR_STATE, "gg_spect_setup: upload the tables first");
  if (sp->n_heads < 1 || sp->n_heads > 2) return c->fail(GG_ERR_ARG, "gg_spect_setup: 1 or 2 heads");
  if (sp->n_windows < 1 || sp->n_windows > 8) return c->fail(GG_ERR_ARG, "gg_spect_setup: 1..8 energy windows");
  if (sp->n_runs < 1 || sp->size[0] < 1 || sp->size[1] < 1 || !(sp->spacing[0] > 0) || !(sp->spacing[1] > 0))
    return c->fail(GG_ERR_ARG, "gg_spect_setup: runs, projection size and spacing must be > 0");
  if (!(sp->half_width > 0) || !(sp->collimator_thickness > 0) || !(sp->gap >= 0) || !(sp->crystal_thickness > 0) ||
      !(sp->hole_apothem > 0) || !(sp->pitch_x > 0) || !(sp->pitch_y > 0))
    return c->fail(GG_ERR_ARG, "gg_spect_setup: head dimensions must be > 0");
  if (!(2.0 * sp->hole_apothem < sp->pitch_y))
    return c->fail(GG_ERR_ARG, "gg_spect_setup: holes wider than their pitch would overlap");
  if (sp->collimator_material < 0 || sp->collimator_material >= c->n_mat || sp->crystal_material < 0 ||
      sp->crystal_material >= c->n_mat)
    return c->fail(GG_ERR_ARG, "gg_spect_setup: head materials outside the material table");
  if (sp->n_cover < 0 || sp->n_cover > 1 || sp->n_back < 0 || sp->n_back > 4)
    return c->fail(GG_ERR_ARG, "gg_spect_setup: housing: at most one cover and four back layers");
  if (sp->n_cover && (!(sp->cover_thickness > 0) || sp->cover_material < 0 || sp->cover_material >= c->n_mat))
    return c->fail(GG_ERR_ARG, "gg_spect_setup: housing cover needs a thickness > 0 and a table material");
  for (int b = 0; b < sp->n_back; ++b)
    if (!(sp->back_thickness[b] > 0) || sp->back_material[b] < 0 || sp->back_material[b] >= c->n_mat)
      return c->fail(GG_ERR_ARG, "gg_spect_setup: housing back layer %d needs a thickness > 0 and a table material", b);
  for (int k = 0; k < sp->n_windows; ++k)
    if (!(sp->window_hi[k] > sp->window_lo[k])) return c->fail(GG_ERR_ARG, "gg_spect_setup: empty window");
  size_t n = (size_t)sp->n_heads * sp->n_runs * sp->n_windows * sp->size[0] * sp->size[1];
  int st;
  if (n != c->n_proj) {
    dfree(c->d_proj);
    if ((st = c->cuda(cudaMalloc(&c->d_proj, n * 8), "cudaMalloc projections"))) return st;
    c->n_proj = n;
  }
  if ((st = c->cuda(cudaMemsetAsync(c->d_proj, 0, n * 8, c->stream), "memset projections"))) return st;
  if ((st = c->cuda(cudaMemsetAsync(c->d_counters, 0, GG_N_COUNTERS * 8, c->stream), "memset counters"))) return st;
  if ((c->arf_on || c->ff_on) && (st = arf_projection_alloc(c, n))) return st;
  c->spect = *sp;
  c->have_spect = true;
  c->spect_run = 0;
  c->frames.assign((size_t)sp->n_runs * sp->n_heads * 12, 0.0);
  c->frames_dirty = true;
  return c->cuda(cudaStreamSynchronize(c->stream), "spect setup");
}

static bool frames_valid(const double *frames, int n_heads) {
  for (int h = 0; h < n_heads; ++h) {
    const double *f = frames + 12 * h;
    for (int v = 1; v < 4; ++v) {
      double n2 = f[3 * v] * f[3 * v] + f[3 * v + 1] * f[3 * v + 1] + f[3 * v + 2] * f[3 * v + 2];
      if (!(std::fabs(n2 - 1.0) <= 1e-6)) return false;
    }
  }
  return true;
}

int gg_spect_set_heads(gg_ctx *c, int32_t run, const double *frames) {
  if (!c || !frames) return GG_ERR_ARG;
  if (!c->have_spect) return c->fail(GG_ERR_STATE, "gg_spect_set_heads: call gg_spect_setup first");
  if (run < 0 || run >= c->spect.n_runs) return c->fail(GG_ERR_ARG, "gg_spect_set_heads: run out of range");
  if (!frames_valid(frames, c->spect.n_heads))
    return c->fail(GG_ERR_ARG, "gg_spect_set_heads: axes must be unit vectors");
  std::copy(frames, frames + 12 * c->spect.n_heads, c->frames.begin() + (size_t)run * c->spect.n_heads * 12);
  c->frames_dirty = true;
  c->spect_run = run;
  return GG_OK;
}

int gg_spect_run(gg_ctx *c, uint64_t n_per_run, uint64_t seed, uint64_t first, const double *frames) {
  if (!c) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_spect) return c->fail(GG_ERR_STATE, "gg_spect_run: call gg_spect_setup first");
  const gg_spect_desc &sp = c->spect;
  if (frames) {
    for (int r = 0; r < sp.n_runs; ++r)
      if (!frames_valid(frames + (size_t)r * sp.n_heads * 12, sp.n_heads))
        return c->fail(GG_ERR_ARG, "gg_spect_run: run %d: axes must be unit vectors", r);
    std::copy(frames, frames + (size_t)sp.n_runs * sp.n_heads * 12, c->frames.begin());
    c->frames_dirty = true;
  }
  if (!(c->src_emax < 2.0 * gg::kMC2))
    return c->fail(GG_ERR_DOMAIN, "gg_spect_run: SPECT transport needs source energies below 1.022 MeV");
  if (!c->have_tables || !c->have_volume || !c->have_world || !c->have_source)
    return c->fail(GG_ERR_STATE, "gg_spect_run: tables, volume, world and source must be set first");
  if (n_per_run == 0) return GG_OK;
  const uint64_t n = n_per_run * (uint64_t)sp.n_runs;
  if (n / (uint64_t)sp.n_runs != n_per_run || first + n < first)
    return c->fail(GG_ERR_ARG, "gg_spect_run: history range overflows");
  c->run_base = 0;
  c->run_first = first;
  c->run_len = n_per_run;
  int st = upload_frames(c);
  if (st) return st;
  return run_impl(c, n, seed, first);
}

static_assert(sizeof(gg_single) == sizeof(gg::SingleRec) && offsetof(gg_single, energy) == offsetof(gg::SingleRec, energy) &&
                  offsetof(gg_single, weight) == offsetof(gg::SingleRec, weight),
              "gg_single and the device record must share their layout");

int gg_spect_record_singles(gg_ctx *c, uint64_t capacity) {
  if (!c) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (capacity > (1ull << 40) / sizeof(gg_single))
    return c->fail(GG_ERR_ARG, "gg_spect_record_singles: capacity above 2^40 bytes of records");
  int st;
  if (capacity != c->singles_cap) {
    dfree(c->d_singles);
    c->singles_cap = 0;
    if (capacity &&
        (st = c->cuda(cudaMalloc(&c->d_singles, capacity * sizeof(gg_single)), "cudaMalloc singles list")))
      return st;
  }
  if (!c->d_n_singles && (st = c->cuda(cudaMalloc(&c->d_n_singles, 8), "cudaMalloc singles count"))) return st;
  if ((st = c->cuda(cudaMemsetAsync(c->d_n_singles, 0, 8, c->stream), "clear singles count"))) return st;
  c->singles_cap = capacity;
  return c->cuda(cudaStreamSynchronize(c->stream), "singles list");
}

int gg_spect_get_singles(gg_ctx *c, gg_single *out, uint64_t out_capacity, uint64_t *n_recorded) {
  if (!c || !n_recorded || (out_capacity && !out)) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->singles_cap) return c->fail(GG_ERR_STATE, "gg_spect_get_singles: no singles list (gg_spect_record_singles)");
  unsigned long long n = 0;
  int st;
  if ((st = c->d2h(&n, c->d_n_singles, 8, "singles count"))) return st;
  *n_recorded = n;
  const uint64_t m = std::min<uint64_t>(std::min<uint64_t>(n, c->singles_cap), out_capacity);
  if (m && (st = c->d2h(out, c->d_singles, m * sizeof(gg_single), "download singles"))) return st;
  if ((st = c->cuda(cudaMemsetAsync(c->d_n_singles, 0, 8, c->stream), "clear singles count"))) return st;
  return c->cuda(cudaStreamSynchronize(c->stream), "singles list");
}

int gg_arf_dataset(gg_ctx *c, const gg_arf_sampling *a, uint64_t n, uint64_t seed, uint64_t first, float *rows,
                   uint64_t capacity, uint64_t *n_rows) {
  if (!c || !a || !n_rows || (capacity && !rows)) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_tables || !c->have_spect)
    return c->fail(GG_ERR_STATE, "gg_arf_dataset: upload the tables and call gg_spect_setup first");
  if (!(a->e_min > 0) || !(a->e_max >= a->e_min) || !(a->e_min >= c->e_min) || !(a->e_max <= c->e_max) ||
      !(a->e_max < 2.0 * gg::kMC2))
    return c->fail(GG_ERR_DOMAIN, "gg_arf_dataset: energies must lie in the tables and below 1.022 MeV");
  if (!(a->cos_theta_max >= 0.0 && a->cos_theta_max <= 1.0) || !(a->half_extent[0] >= 0) ||
      !(a->half_extent[1] >= 0) || !(a->russian_roulette >= 1.0))
    return c->fail(GG_ERR_ARG, "gg_arf_dataset: cos_theta_max in [0, 1], half extents >= 0, russian_roulette >= 1");
  int st = c->precision == GG_PREC_F64 ? arf_generate<double>(c, a, n, seed, first, capacity)
                                       : arf_generate<float>(c, a, n, seed, first, capacity);
  if (st) return st;
  *n_rows = c->arf_n_rows;
  const uint64_t m = std::min<uint64_t>(c->arf_n_rows, capacity);
  if (m) {
    st = c->d2h(rows, c->d_arf_rows, m * sizeof(float4), "download ARF rows");
    if (st) return st;
  }
  return GG_OK;
}

int gg_arf_set_model(gg_ctx *c, const gg_arf_model *m, const float *params) {
  if (!c || !m || !params) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  int st;
  if ((st = arf_model_check(c, m))) return st;
  if ((st = arf_alloc(c, 1))) return st;
  std::vector<float> w(params, params + gg::kNParams);
  for (int r = m->n_classes; r < gg::kOutPad; ++r) {
    for (int k = 0; k < gg::kHid; ++k) w[gg::kOffW4 + r * gg::kHid + k] = 0.0f;
    w[gg::kOffB4 + r] = 0.0f;
  }
  if ((st = c->h2d(c->d_params, w.data(), w.size() * sizeof(float), "upload")))
    return st;
  if ((st = c->cuda(gg::launch_mlp_to_bf16(c->d_params, c->d_wbf, c->stream), "ARF weights"))) return st;
  if ((st = c->cuda(cudaStreamSynchronize(c->stream), "ARF weights"))) return st;
  c->arf = *m;
  c->have_arf = true;
  return GG_OK;
}

int gg_arf_get_params(gg_ctx *c, float *params, size_t n) {
  if (!c || !params) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_arf) return c->fail(GG_ERR_STATE, "gg_arf_get_params: no ARF model");
  if (n != (size_t)gg::kNParams) return c->fail(GG_ERR_ARG, "gg_arf_get_params: need %d floats", gg::kNParams);
  return c->d2h(params, c->d_params, n * sizeof(float), "download");
}

// Reads and clears the status word after a tensor-core kernel.
static int check_tc_status(gg_ctx *c, const char *what) {
  unsigned int status = 0;
  int st;
  if ((st = c->d2h(&status, c->d_status, sizeof(status), "status"))) return st;
  if (!status) return GG_OK;
  cudaMemsetAsync(c->d_status, 0, sizeof(unsigned int), c->stream);
  cudaStreamSynchronize(c->stream);
  if (status & gg::kStatusWaitTimeout) return c->fail(GG_ERR_TIMEOUT, "%s: a tensor-core wait ran out", what);
  return c->fail(GG_ERR_DOMAIN, "%s: kernel status %u", what, status);
}

int gg_arf_predict(gg_ctx *c, const float *rows, uint64_t n, float *probs) {
  if (!c || (n && (!rows || !probs))) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_arf) return c->fail(GG_ERR_STATE, "gg_arf_predict: no ARF model");
  if (n == 0) return GG_OK;
  int st;
  if ((st = io_alloc(c, (size_t)n))) return st;
  if ((st = c->h2d(c->d_io_rows, rows, n * sizeof(float4), "upload"))) return st;
  gg::MlpTrainArgs a = arf_args(c);
  a.rows = c->d_io_rows;
  a.n_rows = n;
  // one CTA per SM (tensor memory and ~200 KB of shared memory each), four 128-row tiles at a time
  const uint64_t tiles = (n + 511) / 512;
  const int grid = (int)std::min<uint64_t>(tiles, (uint64_t)c->n_sm);
  if ((st = c->cuda(gg::launch_mlp_predict(a, c->d_io_out, n, grid, c->d_status, c->stream), "ARF predict")))
    return st;
  if ((st = c->d2h(probs, c->d_io_out, n * c->arf.n_classes * sizeof(float), "download"))) return st;
  return check_tc_status(c, "gg_arf_predict");
}

int gg_arf_gradient(gg_ctx *c, const float *rows, uint64_t n, float *grad, double *loss) {
  if (!c || !rows || !grad) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_arf) return c->fail(GG_ERR_STATE, "gg_arf_gradient: no ARF model");
  if (n == 0 || n % gg::kTrainRows || n > 65536)
    return c->fail(GG_ERR_ARG, "gg_arf_gradient: n must be a multiple of 128, <= 65536");
  const int tiles = (int)(n / gg::kTrainRows);
  int st;
  if ((st = arf_alloc(c, tiles)) || (st = io_alloc(c, (size_t)n))) return st;
  if ((st = c->h2d(c->d_io_rows, rows, n * sizeof(float4), "upload"))) return st;
  for (uint64_t i = 0; i < n; ++i)
    if (!(rows[4 * i + 3] >= 0.0f) || rows[4 * i + 3] >= (float)c->arf.n_classes)
      return c->fail(GG_ERR_ARG, "gg_arf_gradient: row %llu: class outside [0, n_classes)", (unsigned long long)i);
  gg::MlpTrainArgs a = arf_args(c);
  a.rows = c->d_io_rows;
  a.row0 = 0;
  a.n_rows = n;
  a.inv_batch = 1.0f / (float)n;
  if ((st = c->cuda(gg::launch_mlp_train(a, tiles, c->stream), "ARF gradient"))) return st;
  gg::MlpAdamArgs g{};
  g.partial = c->d_partial;
  g.n_tiles = tiles;
  g.params = c->d_params;
  g.wbf = c->d_wbf;
  g.grad_out = c->d_grad;
  g.lr = 0.0f;
  if ((st = c->cuda(gg::launch_mlp_adam(g, c->stream), "ARF gradient sum"))) return st;
  std::vector<float> lp(tiles);
  if ((st = c->d2h(grad, c->d_grad, gg::kNParams * sizeof(float), "download")))
    return st;
  if ((st = c->d2h(lp.data(), c->d_loss_part, tiles * sizeof(float), "download")))
    return st;
  if (loss) {
    double sum = 0.0;
    for (float v : lp) sum += v;
    *loss = sum / (double)n;
  }
  return check_tc_status(c, "gg_arf_gradient");
}

// The model of a training domain: classes = windows + 1, inputs standardised
// by the mean and standard deviation of uniform theta in [0, theta_max] deg,
// phi in [-180, 180) deg and E in [e_min, e_max].
static gg_arf_model arf_domain_model(const gg_ctx *c, double e_min, double e_max, double theta_max_deg,
                                     double russian_roulette) {
  gg_arf_model m{};
  m.n_classes = c->spect.n_windows + 1;
  const double th = theta_max_deg;
  m.x_mean[0] = (float)(0.5 * th);
  m.x_std[0] = (float)(th / std::sqrt(12.0));
  m.x_mean[1] = 0.0f;
  m.x_std[1] = (float)(360.0 / std::sqrt(12.0));
  m.x_mean[2] = (float)(0.5 * (e_min + e_max));
  m.x_std[2] = (float)((e_max - e_min) / std::sqrt(12.0));
  m.russian_roulette = russian_roulette;
  m.e_min = e_min;
  m.e_max = e_max;
  m.theta_max_deg = th;
  m.distance_to_crystal = c->spect.collimator_thickness + c->spect.gap +
                          (c->spect.n_cover > 0 ? c->spect.cover_thickness : 0.0) + 0.5 * c->spect.crystal_thickness;
  return m;
}

static int arf_check_opts(gg_ctx *c, const gg_arf_train_opts *o, const char *who) {
  if (o->batch < gg::kTrainRows || o->batch % gg::kTrainRows || o->batch > 65536 || o->epochs < 1 || o->epochs > 1024 ||
      !(o->lr > 0.0f))
    return c->fail(GG_ERR_ARG, "%s: batch a multiple of 128 (<= 65536), 1..1024 epochs, lr > 0", who);
  return GG_OK;
}

// Adam training of the network of model m on the n_rows rows in c->d_arf_rows.
static int arf_train_impl(gg_ctx *c, uint64_t n_rows, const gg_arf_model &m, const gg_arf_train_opts *o,
                          gg_arf_model *model_out, double *loss);

int gg_arf_train(gg_ctx *c, const gg_arf_sampling *smp, const gg_arf_train_opts *o, gg_arf_model *model_out,
                 double *loss) {
  if (!c || !smp || !o) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_tables || !c->have_spect)
    return c->fail(GG_ERR_STATE, "gg_arf_train: upload the tables and call gg_spect_setup first");
  int st;
  if ((st = arf_check_opts(c, o, "gg_arf_train"))) return st;
  if (o->n_samples == 0) return c->fail(GG_ERR_ARG, "gg_arf_train: samples > 0");
  // training rows on the device
  uint64_t n_rows = 0;
  {
    if (!(smp->e_min > 0) || !(smp->e_max > smp->e_min) || !(smp->e_min >= c->e_min) || !(smp->e_max <= c->e_max) ||
        !(smp->e_max < 2.0 * gg::kMC2) || !(smp->cos_theta_max >= 0.0 && smp->cos_theta_max < 1.0) ||
        !(smp->russian_roulette >= 1.0))
      return c->fail(GG_ERR_ARG, "gg_arf_train: invalid sampling");
    st = c->precision == GG_PREC_F64 ? arf_generate<double>(c, smp, o->n_samples, o->seed, 0, o->n_samples)
                                     : arf_generate<float>(c, smp, o->n_samples, o->seed, 0, o->n_samples);
    if (st) return st;
    n_rows = c->arf_n_rows;
    if (n_rows < (uint64_t)o->batch) return c->fail(GG_ERR_DOMAIN, "gg_arf_train: fewer rows than one batch");
  }
  const gg_arf_model m = arf_domain_model(c, smp->e_min, smp->e_max, std::acos(smp->cos_theta_max) * (180.0 / M_PI),
                                          smp->russian_roulette);
  return arf_train_impl(c, n_rows, m, o, model_out, loss);
}

int gg_arf_train_rows(gg_ctx *c, const float *rows, uint64_t n_rows, const gg_arf_model *domain,
                      const gg_arf_train_opts *o, gg_arf_model *model_out, double *loss) {
  if (!c || !rows || !domain || !o) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_tables || !c->have_spect)
    return c->fail(GG_ERR_STATE, "gg_arf_train_rows: upload the tables and call gg_spect_setup first");
  int st;
  if ((st = arf_check_opts(c, o, "gg_arf_train_rows"))) return st;
  if (n_rows < (uint64_t)o->batch) return c->fail(GG_ERR_DOMAIN, "gg_arf_train_rows: fewer rows than one batch");
  if (!(domain->e_min > 0) || !(domain->e_max > domain->e_min) || !(domain->theta_max_deg > 0) ||
      !(domain->theta_max_deg <= 90.0) || !(domain->russian_roulette >= 1.0))
    return c->fail(GG_ERR_ARG, "gg_arf_train_rows: domain needs 0 < e_min < e_max, 0 < theta_max <= 90, rr >= 1");
  const int n_classes = c->spect.n_windows + 1;
  for (uint64_t i = 0; i < n_rows; ++i) {
    const float *r = rows + 4 * i;
    if (!std::isfinite(r[0]) || !std::isfinite(r[1]) || !std::isfinite(r[2]) || !(r[3] >= 0.0f) ||
        !(r[3] < (float)n_classes) || r[3] != std::floor(r[3]))
      return c->fail(GG_ERR_ARG, "gg_arf_train_rows: row %llu: non-finite input or class outside [0, %d)",
                     (unsigned long long)i, n_classes);
  }
  if (n_rows > c->arf_rows_cap) {
    dfree(c->d_arf_rows);
    c->arf_rows_cap = 0;
    if ((st = c->cuda(cudaMalloc(&c->d_arf_rows, n_rows * sizeof(float4)), "cudaMalloc ARF rows"))) return st;
    c->arf_rows_cap = n_rows;
  }
  if ((st = c->h2d(c->d_arf_rows, rows, n_rows * sizeof(float4), "upload ARF rows"))) return st;
  const gg_arf_model m = arf_domain_model(c, domain->e_min, domain->e_max, domain->theta_max_deg,
                                          domain->russian_roulette);
  return arf_train_impl(c, n_rows, m, o, model_out, loss);
}

static int arf_train_impl(gg_ctx *c, uint64_t n_rows, const gg_arf_model &m, const gg_arf_train_opts *o,
                          gg_arf_model *model_out, double *loss) {
  int st;
  if ((st = arf_model_check(c, &m))) return st;
  std::vector<float> w0 = arf_init_params(o->init_seed, m.n_classes);
  if ((st = gg_arf_set_model(c, &m, w0.data()))) return st;
  const int tiles = o->batch / gg::kTrainRows;
  if ((st = arf_alloc(c, tiles))) return st;
  if ((st = c->cuda(cudaMemsetAsync(c->d_adam_m, 0, gg::kNParams * sizeof(float), c->stream), "memset"))) return st;
  if ((st = c->cuda(cudaMemsetAsync(c->d_adam_v, 0, gg::kNParams * sizeof(float), c->stream), "memset"))) return st;
  if ((st = c->cuda(cudaMemsetAsync(c->d_loss_acc, 0, 1024 * sizeof(double), c->stream), "memset"))) return st;
  gg::MlpTrainArgs a = arf_args(c);
  a.rows = c->d_arf_rows;
  a.n_rows = n_rows;
  a.inv_batch = 1.0f / (float)o->batch;
  gg::MlpAdamArgs g{};
  g.partial = c->d_partial;
  g.n_tiles = tiles;
  g.params = c->d_params;
  g.wbf = c->d_wbf;
  g.m = c->d_adam_m;
  g.v = c->d_adam_v;
  g.lr = o->lr;
  g.beta1 = o->beta1;
  g.beta2 = o->beta2;
  g.eps = o->eps;
  g.loss_part = c->d_loss_part;
  const uint64_t steps_per_epoch = (n_rows + (uint64_t)o->batch - 1) / (uint64_t)o->batch;
  const double total_steps = (double)steps_per_epoch * (double)o->epochs;
  const double decay = o->lr_final > 0.0f ? std::log((double)o->lr_final / (double)o->lr) : 0.0;
  uint64_t t = 0;
  for (int ep = 0; ep < o->epochs; ++ep) {
    g.loss_acc = c->d_loss_acc + ep;
    for (uint64_t k = 0; k < steps_per_epoch; ++k, ++t) {
      a.row0 = (t * (uint64_t)o->batch) % n_rows;
      if ((st = c->cuda(gg::launch_mlp_train(a, tiles, c->stream), "ARF train step"))) return st;
      g.lr = (float)((double)o->lr * std::exp(decay * (double)t / total_steps));
      g.c1 = (float)(1.0 / (1.0 - std::pow((double)o->beta1, (double)(t + 1))));
      g.c2 = (float)(1.0 / (1.0 - std::pow((double)o->beta2, (double)(t + 1))));
      if ((st = c->cuda(gg::launch_mlp_adam(g, c->stream), "ARF Adam step"))) return st;
    }
  }
  std::vector<double> lacc(o->epochs);
  if ((st = c->cuda(cudaMemcpyAsync(lacc.data(), c->d_loss_acc, o->epochs * sizeof(double), cudaMemcpyDeviceToHost,
                                    c->stream),
                    "download")))
    return st;
  if ((st = c->cuda(cudaStreamSynchronize(c->stream), "ARF training"))) return st;
  if ((st = check_tc_status(c, "gg_arf_train"))) return st;
  if (loss)
    for (int ep = 0; ep < o->epochs; ++ep) loss[ep] = lacc[ep] / ((double)steps_per_epoch * o->batch);
  if (model_out) *model_out = m;
  return GG_OK;
}

int gg_last_stage_ms(gg_ctx *c, double *phantom_ms, double *head_ms, double *arf_ms) {
  if (!c) return GG_ERR_ARG;
  if (phantom_ms) *phantom_ms = c->stage_ms[0];
  if (head_ms) *head_ms = c->stage_ms[1];
  if (arf_ms) *arf_ms = c->stage_ms[2];
  return GG_OK;
}

int gg_spect_use_arf(gg_ctx *c, int32_t enable) {
  if (!c) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!enable) {
    c->arf_on = false;
    return GG_OK;
  }
  if (!c->have_spect || !c->have_arf) return c->fail(GG_ERR_STATE, "gg_spect_use_arf: needs gg_spect_setup and an ARF model");
  if (c->arf.n_classes != c->spect.n_windows + 1)
    return c->fail(GG_ERR_ARG, "gg_spect_use_arf: the model has %d classes, the heads %d windows + 1", c->arf.n_classes,
                   c->spect.n_windows);
  c->arf_on = true;
  int st = arf_projection_alloc(c, c->n_proj);
  if (st) return st;
  return c->cuda(cudaStreamSynchronize(c->stream), "ARF projection");
}

int gg_spect_set_free_flight(gg_ctx *c, const gg_ff_desc *f) {
  if (!c || !f) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (f->enabled == GG_FF_OFF) {
    c->ff_on = false;
    c->ff_mode = GG_FF_OFF;
    return GG_OK;
  }
  if (f->enabled != GG_FF_PRIMARY && f->enabled != GG_FF_SCATTER)
    return c->fail(GG_ERR_ARG, "gg_spect_set_free_flight: unknown mode %d", f->enabled);
  if (!c->have_spect) return c->fail(GG_ERR_STATE, "gg_spect_set_free_flight: call gg_spect_setup first");
  if (std::isnan(f->weight_cutoff) || std::isnan(f->energy_cutoff))
    return c->fail(GG_ERR_ARG, "gg_spect_set_free_flight: invalid cutoff");
  if (std::isnan(f->angle_tolerance_max)) return c->fail(GG_ERR_ARG, "gg_spect_set_free_flight: invalid angle");
  if (f->enabled == GG_FF_SCATTER &&
      (f->compton_splitting < 0 || f->rayleigh_splitting < 0 || f->max_compton_level < 0 ||
       f->compton_splitting > GG_MAX_SPLITTING || f->rayleigh_splitting > GG_MAX_SPLITTING))
    return c->fail(GG_ERR_ARG, "gg_spect_set_free_flight: splitting factors must be in [0, %d], the level >= 0",
                   GG_MAX_SPLITTING);
  c->ff_on = true;
  c->ff_mode = f->enabled;
  c->ff_wcut = f->weight_cutoff;
  c->ff_ecut = f->energy_cutoff;
  c->ss_nc = f->enabled == GG_FF_SCATTER ? f->compton_splitting : 0;
  c->ss_nr = f->enabled == GG_FF_SCATTER ? f->rayleigh_splitting : 0;
  c->ss_max = f->enabled == GG_FF_SCATTER ? f->max_compton_level : 0;
  c->ss_cos = f->angle_tolerance_max > 0.0 ? std::cos(f->angle_tolerance_max) : -2.0;
  c->ss_span = 0;
  int st = arf_projection_alloc(c, c->n_proj);
  if (st) return st;
  return c->cuda(cudaStreamSynchronize(c->stream), "weighted projection");
}

int gg_get_arf_projection(gg_ctx *c, double *counts, double *squared, size_t n) {
  if (!c || !counts) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if ((!c->arf_on && !c->ff_on) || !c->d_arf_proj)
    return c->fail(GG_ERR_STATE, "gg_get_arf_projection: neither the ARF stage nor free flight is on");
  if (n != c->arf_proj_n) return c->fail(GG_ERR_ARG, "gg_get_arf_projection: buffer has %zu values, need %zu", n, c->arf_proj_n);
  std::vector<unsigned long long> tmp(n);
  int st = c->d2h(tmp.data(), c->d_arf_proj, n * 8, "download ARF projection");
  if (st) return st;
  for (size_t i = 0; i < n; ++i) counts[i] = (double)tmp[i] * 2.3283064365386963e-10;
  if (squared) {
    std::vector<unsigned long long> t2(2 * n);
    if ((st = c->d2h(t2.data(), c->d_arf_proj2, n * 16, "download ARF projection squared"))) return st;
    for (size_t i = 0; i < n; ++i) {
      double lo = (double)t2[2 * i];
      lo = lo * 5.421010862427522e-20;
      double hi = (double)t2[2 * i + 1];
      hi = hi * 2.3283064365386963e-10;
      squared[i] = hi + lo;
    }
  }
  return GG_OK;
}

int gg_batch_setup(gg_ctx *c, const gg_sim_desc *sims, int32_t n) {
  if (!c || !sims || n < 1) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_tables || !c->have_world)
    return c->fail(GG_ERR_STATE, "gg_batch_setup: upload the tables and set the world first");
  if (c->have_spect) return c->fail(GG_ERR_STATE, "gg_batch_setup: SPECT heads are set up on this context");
  if (c->dgrid_on) return c->fail(GG_ERR_STATE, "gg_batch_setup: a dose grid is set on this context");
  std::vector<uint64_t> off(n), nv(n);
  uint64_t total = 0, hist = 0;
  double emax = 0;
  for (int k = 0; k < n; ++k) {
    const gg_volume_desc &v = sims[k].volume;
    const gg_source_desc &src = sims[k].source;
    size_t m = 0;
    char msg[160];
    if (gg::check_dims(v.dims, (size_t)UINT32_MAX - 1, &m, msg, sizeof(msg)))
      return c->fail(GG_ERR_ARG, "sim %d: %s", k, msg);
    for (int a = 0; a < 3; ++a) {
      if (!(v.spacing[a] > 0)) return c->fail(GG_ERR_ARG, "sim %d: spacing must be > 0", k);
      if (!(std::fabs(v.corner[a]) + v.dims[a] * v.spacing[a] <= 2.0 * c->world.half_size[a]))
        return c->fail(GG_ERR_ARG, "sim %d: the image is not inside the world", k);
    }
    if (!v.labels || !v.majorant) return c->fail(GG_ERR_ARG, "sim %d: labels and majorant needed", k);
    uint16_t lmax = 0;  // (a branch-free reduction: the compiler vectorises it)
    for (uint64_t i = 0; i < m; ++i) lmax = std::max(lmax, v.labels[i]);
    if ((int)lmax >= c->n_mat) return c->fail(GG_ERR_ARG, "sim %d: label outside the material table", k);
    if (gg::check_majorant(v.majorant, c->n_e, msg, sizeof(msg))) return c->fail(GG_ERR_ARG, "sim %d: %s", k, msg);
    if (src.pos_type < GG_POS_POINT || src.pos_type > GG_POS_DISC || src.dir_type < GG_DIR_ISO ||
        src.dir_type > GG_DIR_FOCUSED || (src.ene_type != GG_ENE_MONO && src.ene_type != GG_ENE_RANGE) ||
        src.n_accept != 0)
      return c->fail(GG_ERR_ARG, "sim %d: batched sources are point/box/sphere/disc, mono or range, no acceptance", k);
    const double lo = src.ene_type == GG_ENE_MONO ? src.mono : src.e_lo;
    const double hi = src.ene_type == GG_ENE_MONO ? src.mono : src.e_hi;
    if (!(lo >= c->e_min) || !(hi <= c->e_max)) return c->fail(GG_ERR_DOMAIN, "sim %d: energies outside the tables", k);
    emax = std::max(emax, hi);
    off[k] = total;
    nv[k] = m;
    total += m;
    hist += sims[k].n_primaries;
  }
  drop_graph(c);
  // labels concatenated on the device (one copy per simulation, straight
  // from the caller's buffers), majorants per simulation; the element-wise
  // maximum serves as the context's majorant
  std::vector<float> maj(c->n_e, 0.0f), all_maj((size_t)n * c->n_e);
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < c->n_e; ++i) {
      maj[i] = std::max(maj[i], sims[k].volume.majorant[i]);
      all_maj[(size_t)k * c->n_e + i] = sims[k].volume.majorant[i];
    }
  int st;
  if ((st = labels_alloc(c, total))) return st;
  for (int k = 0; k < n; ++k)
    if ((st = c->cuda(cudaMemcpyAsync(c->d_labels + off[k], sims[k].volume.labels, nv[k] * sizeof(uint16_t),
                                      cudaMemcpyHostToDevice, c->stream),
                      "upload labels")))
      return st;
  if ((st = c->cuda(cudaStreamSynchronize(c->stream), "upload labels"))) return st;
  if ((st = c->upload_real(c->d_maj, maj.data(), (size_t)c->n_e))) return st;
  if ((st = c->upload_real(c->d_sim_maj, all_maj.data(), all_maj.size()))) return st;
  if (total != c->n_vox) {
    dfree(c->d_acc_e); dfree(c->d_acc_e2); dfree(c->d_edep); dfree(c->d_edep2);
    c->have_tally = false;
  }
  c->n_vox = total;
  c->dims[0] = c->dims[1] = c->dims[2] = 1;
  c->have_volume = true;
  c->sim_vox_off = off;
  c->sim_vox_n = nv;
  c->n_sims = n;
  c->batch_total = hist;
  st = c->precision == GG_PREC_F64 ? upload_sims<double>(c, sims, n) : upload_sims<float>(c, sims, n);
  if (st) return st;
  c->src = sims[0].source;
  c->src.spec_e = c->src.spec_cdf = nullptr;
  c->src.accept_boxes = nullptr;
  c->src.cdf_z = c->src.cdf_y = c->src.cdf_x = nullptr;
  c->src_emax = emax;
  c->have_source = true;
  c->have_batch = true;
  return gg_add_dose_tally(c, 1);
}

int gg_batch_run(gg_ctx *c) {
  if (!c) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_batch || !c->have_tally) return c->fail(GG_ERR_STATE, "gg_batch_run: call gg_batch_setup first");
  if (c->batch_total == 0) return GG_OK;
  return run_impl(c, c->batch_total, 0, 0);
}

int gg_batch_capture(gg_ctx *c) {
  if (!c) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_batch || !c->have_tally) return c->fail(GG_ERR_STATE, "gg_batch_capture: call gg_batch_setup first");
  int st;
  // one regular run first (buffers, kernel attributes, events), then discarded
  if ((st = gg_batch_run(c))) return st;
  if ((st = gg_reset_tally(c))) return st;
  if ((st = c->cuda(cudaStreamSynchronize(c->stream), "capture"))) return st;
  drop_graph(c);
  if ((st = c->cuda(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture"))) return st;
  int rc = run_impl(c, c->batch_total, 0, 0, true);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if ((st = c->cuda(e, "end capture"))) return st;
  c->graph = g;
  return c->cuda(cudaGraphInstantiate(&c->graph_exec, c->graph, 0), "graph instantiate");
}

int gg_batch_replay(gg_ctx *c) {
  if (!c) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->graph_exec) return c->fail(GG_ERR_STATE, "gg_batch_replay: call gg_batch_capture first");
  if (c->ev.empty()) return c->fail(GG_ERR_STATE, "gg_batch_replay: no events");
  int st;
  if ((st = c->cuda(cudaEventRecord(c->ev[0], c->stream), "event"))) return st;
  if ((st = c->cuda(cudaGraphLaunch(c->graph_exec, c->stream), "graph launch"))) return st;
  if ((st = c->cuda(cudaEventRecord(c->ev[1], c->stream), "event"))) return st;
  if ((st = c->cuda(cudaStreamSynchronize(c->stream), "graph replay"))) return st;
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
  c->last_generate_ms = 0;
  c->last_transport_ms = ms;
  c->last_flush_ms = 0;
  unsigned int status = 0;
  if ((st = c->d2h(&status, c->d_status, sizeof(status), "status"))) return st;
  if (status) return c->fail(GG_ERR_DOMAIN, "gg_batch_replay: kernel status %u", status);
  return GG_OK;
}

int gg_batch_autotune(gg_ctx *c, gg_device_opts *best) {
  if (!c) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_batch || !c->have_tally) return c->fail(GG_ERR_STATE, "gg_batch_autotune: call gg_batch_setup first");
  constexpr int kRep = 3;
  int st = GG_OK;
  // median / min / max of kRep device timings of the current configuration
  auto time_point = [&](double stats[3]) -> int {
    double t[kRep];
    for (int r = 0; r < kRep; ++r) {
      int s2;
      if ((s2 = gg_reset_tally(c)) || (s2 = gg_batch_run(c))) return s2;
      t[r] = c->last_generate_ms + c->last_transport_ms + c->last_flush_ms;
    }
    std::sort(t, t + kRep);
    stats[0] = t[kRep / 2];
    stats[1] = t[0];
    stats[2] = t[kRep - 1];
    ++c->tune.points;
    return GG_OK;
  };
  c->tune = gg_autotune_result{};
  c->tune.repeats = kRep;
  double cur[3];
  if ((st = time_point(cur))) return st;
  c->tune.default_median_ms = cur[0];
  double bst[3] = {cur[0], cur[1], cur[2]};
  // the starting configuration as run_impl resolves it (0 blocks per SM = its default)
  int bm = c->blocks_per_sm > 0 ? std::min(c->blocks_per_sm, 4) : (c->precision == GG_PREC_F64 || c->have_batch ? 2 : 4);
  int br = c->refill_min, bi = c->interact_min, bc = c->chunk;
  int64_t bb = c->batch;
  // stage 1: resident blocks per SM x phase thresholds
  const int minbs[3] = {2, 3, 4};
  const int thresholds[3][2] = {{8, 16}, {4, 8}, {12, 24}};
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      c->blocks_per_sm = minbs[a];
      c->refill_min = thresholds[b][0];
      c->interact_min = thresholds[b][1];
      double t[3];
      if ((st = time_point(t))) return st;
      if (t[0] < bst[0]) {
        std::copy(t, t + 3, bst);
        bm = minbs[a];
        br = thresholds[b][0];
        bi = thresholds[b][1];
      }
    }
  c->blocks_per_sm = bm;
  c->refill_min = br;
  c->interact_min = bi;
  // stage 2: per-warp claim chunk x batch length (all histories in one
  // generate / transport / flush sequence, or in 2 or 4)
  const int chunks[3] = {64, 256, 1024};
  const uint64_t tot = c->batch_total;
  const int64_t batches[3] = {(int64_t)tot, (int64_t)((tot + 1) / 2), (int64_t)((tot + 3) / 4)};
  const int64_t batch0 = c->batch;
  const int chunk0 = c->chunk;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      c->chunk = chunks[a];
      c->batch = std::max<int64_t>(1, batches[b]);
      double t[3];
      if ((st = time_point(t))) return st;
      if (t[0] < bst[0]) {
        std::copy(t, t + 3, bst);
        bc = chunks[a];
        bb = c->batch;
      }
    }
  if (bst[0] >= c->tune.default_median_ms) {  // nothing beat the starting point
    bc = chunk0;
    bb = batch0;
  }
  c->chunk = bc;
  c->batch = bb;
  c->tune.median_ms = bst[0];
  c->tune.min_ms = bst[1];
  c->tune.max_ms = bst[2];
  drop_graph(c);
  if ((st = gg_reset_tally(c))) return st;
  if (best) {
    best->device = c->device;
    best->precision = c->precision;
    best->block_size = c->block;
    best->blocks_per_sm = c->blocks_per_sm;
    best->chunk = c->chunk;
    best->batch = (int64_t)c->batch;
    best->refill_min = c->refill_min;
    best->interact_min = c->interact_min;
  }
  return c->cuda(cudaStreamSynchronize(c->stream), "autotune");
}

int gg_batch_autotune_result(gg_ctx *c, gg_autotune_result *out) {
  if (!c || !out) return GG_ERR_ARG;
  if (c->tune.points == 0) return c->fail(GG_ERR_STATE, "gg_batch_autotune_result: no search has run");
  *out = c->tune;
  return GG_OK;
}

int gg_batch_get_image(gg_ctx *c, int32_t sim, int32_t which, double *out, size_t n) {
  if (!c || !out) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_batch || !c->have_tally) return c->fail(GG_ERR_STATE, "gg_batch_get_image: no batch");
  if (sim < 0 || sim >= c->n_sims) return c->fail(GG_ERR_ARG, "gg_batch_get_image: simulation %d of %d", sim, c->n_sims);
  if (n != c->sim_vox_n[sim]) return c->fail(GG_ERR_ARG, "gg_batch_get_image: buffer has %zu voxels, image %llu", n,
                                             (unsigned long long)c->sim_vox_n[sim]);
  const double *src = which == GG_IMG_EDEP ? c->d_edep : (which == GG_IMG_EDEP_SQUARED ? c->d_edep2 : nullptr);
  if (!src) return c->fail(GG_ERR_ARG, "gg_batch_get_image: image %d", which);
  return c->d2h(out, src + c->sim_vox_off[sim], n * sizeof(double), "download");
}

int gg_get_projection(gg_ctx *c, double *out, size_t n) {
  if (!c || !out) return GG_ERR_ARG;
  cudaSetDevice(c->device);
  if (!c->have_spect) return c->fail(GG_ERR_STATE, "gg_get_projection: no SPECT heads");
  if (n != c->n_proj) return c->fail(GG_ERR_ARG, "gg_get_projection: buffer has %zu values, need %zu", n, c->n_proj);
  std::vector<unsigned long long> tmp(n);
  int st = c->d2h(tmp.data(), c->d_proj, n * 8, "download projections");
  if (st) return st;
  for (size_t i = 0; i < n; ++i) out[i] = (double)tmp[i];
  return GG_OK;
}

}  // extern "C"
