// gg_device.cuh - device-side numerics and photon physics of the transport kernels.
//
// Every function here is written as an explicit sequence of correctly rounded
// IEEE operations (the translation unit is compiled with -fmad=false, so no
// a*b+c is fused unless written as fma()), which makes one history's result
// reproducible bit for bit, independent of launch shape, and identical to a
// CPU evaluation of the same sequence.
//
// Physics (G4EmStandardPhysics option 0, as selected by
// physics_list_name = "G4EmStandardPhysics", opengate/physics.py:341-347):
//   * Compton: Klein-Nishina, composition + rejection sampling of the Geant4
//     Physics Reference Manual (Butcher & Messel), electron stopped at creation;
//   * photoelectric: absorption, local deposit (fluorescence off);
//   * Rayleigh: x^2 sampled from the tabulated form-factor cumulative,
//     accepted with (1 + cos^2)/2;
//   * pair: e- and e+ stopped at creation (min_ekine user limit,
//     opengate/physics.py:699-753), kinetic energy deposited, the positron
//     annihilates at rest into two back-to-back 511 keV photons.
#pragma once
#include <cstdint>

#include "../../include/gate_gpu.h"

namespace gg {

constexpr int kLoopCap = 1000;    // sampling-loop iteration cap
constexpr int kStepCap = 1000000; // per-photon step cap (termination guard)
constexpr int kHeadRegions = 8;   // SPECT head slabs: collimator, gap, cover, crystal, 4 back layers
constexpr double kMC2 = 0.51099895;
constexpr double kHcMevAngstrom = 12.398419843320026e-3;

template <typename real>
__device__ __forceinline__ real R(double x) {
  return static_cast<real>(x);
}

// ---------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon et al., SC'11)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1, uint32_t o[4]) {
  uint32_t c0 = c[0], c1 = c[1], c2 = c[2], c3 = c[3];
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t lo0 = 0xD2511F53u * c0;
    uint32_t hi0 = __umulhi(0xD2511F53u, c0);
    uint32_t lo1 = 0xCD9E8D57u * c2;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  o[0] = c0;
  o[1] = c1;
  o[2] = c2;
  o[3] = c3;
}

// One Philox block as a single out-of-line function: the generator is drawn
// from a dozen call sites and inlining the ten rounds at each of them would
// multiply the kernel's instruction footprint.
static __device__ __noinline__ uint4 philox_block(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                           uint32_t k1) {
  uint32_t c[4] = {c0, c1, c2, c3};
  uint32_t o[4];
  philox4x32_10(c, k0, k1, o);
  return make_uint4(o[0], o[1], o[2], o[3]);
}

// Stream of one history: key = seed, counter = (block, stream, history lo, hi).
struct Rng {
  uint32_t k0, k1;
  uint32_t blk, stream, h0, h1;
  uint32_t buf[4];
  int idx;

  __device__ __forceinline__ void init(uint64_t seed, uint64_t history, uint32_t s) {
    k0 = (uint32_t)seed;
    k1 = (uint32_t)(seed >> 32);
    blk = 0;
    stream = s;
    h0 = (uint32_t)history;
    h1 = (uint32_t)(history >> 32);
    idx = 4;
  }
  __device__ __forceinline__ uint32_t next() {
    if (idx == 4) {
      uint4 b = philox_block(blk, stream, h0, h1, k0, k1);
      buf[0] = b.x;
      buf[1] = b.y;
      buf[2] = b.z;
      buf[3] = b.w;
      blk += 1u;
      idx = 0;
    }
    // register-resident select instead of a dynamically indexed array
    uint32_t v = idx == 0 ? buf[0] : (idx == 1 ? buf[1] : (idx == 2 ? buf[2] : buf[3]));
    ++idx;
    return v;
  }
};

// The same stream with the next block computed ahead (the source stage: both
// first blocks of a history are generated while the warp is converged, so the
// divergent sampling loops draw without calling the generator).  State saved
// as (blk, idx, buf) is that of an Rng at the same point of the stream.
struct RngAhead : Rng {
  uint32_t nxt[4];
  bool ahead;

  // blocks 0 and 1 of the history: block 0 in buf, block 1 ahead
  __device__ __forceinline__ void start(uint64_t seed, uint64_t history, uint32_t s) {
    init(seed, history, s);
    const uint4 b0 = philox_block(0u, stream, h0, h1, k0, k1);
    const uint4 b1 = philox_block(1u, stream, h0, h1, k0, k1);
    buf[0] = b0.x;
    buf[1] = b0.y;
    buf[2] = b0.z;
    buf[3] = b0.w;
    nxt[0] = b1.x;
    nxt[1] = b1.y;
    nxt[2] = b1.z;
    nxt[3] = b1.w;
    blk = 1u;
    idx = 0;
    ahead = true;
  }
  __device__ __forceinline__ uint32_t next() {
    if (idx == 4) {
      if (ahead) {
        buf[0] = nxt[0];
        buf[1] = nxt[1];
        buf[2] = nxt[2];
        buf[3] = nxt[3];
        ahead = false;
      } else {
        const uint4 b = philox_block(blk, stream, h0, h1, k0, k1);
        buf[0] = b.x;
        buf[1] = b.y;
        buf[2] = b.z;
        buf[3] = b.w;
      }
      blk += 1u;
      idx = 0;
    }
    uint32_t v = idx == 0 ? buf[0] : (idx == 1 ? buf[1] : (idx == 2 ? buf[2] : buf[3]));
    ++idx;
    return v;
  }
};

template <typename real, typename G>
__device__ __forceinline__ real u01(G &g) {
  return (real)(g.next() >> 8) * R<real>(5.9604644775390625e-08);
}
template <typename real, typename G>
__device__ __forceinline__ real u01_open0(G &g) {
  return (real)((g.next() >> 8) + 1u) * R<real>(5.9604644775390625e-08);
}

// ---------------------------------------------------------------------------
// Elementary functions built from + - * / (A&S 4.1.27, 4.2.1, 4.3.65/66)
// ---------------------------------------------------------------------------
static __device__ __noinline__ float gg_log(float x) {
  uint32_t b = __float_as_uint(x);
  int e = (int)(b >> 23) - 127;
  uint32_t mb = (b & 0x007fffffu) | 0x3f800000u;
  if (mb > 0x3fb504f3u) {
    mb -= 0x00800000u;
    e += 1;
  }
  float m = __uint_as_float(mb);
  float num = m - 1.0f;
  float den = m + 1.0f;
  float s = num / den;
  float z = s * s;
  float p = (float)(1.0 / 11.0);
  p = p * z + (float)(1.0 / 9.0);
  p = p * z + (float)(1.0 / 7.0);
  p = p * z + (float)(1.0 / 5.0);
  p = p * z + (float)(1.0 / 3.0);
  float t = s * z;
  t = t * p;
  float u = s + t;
  float lm = u + u;
  float fe = (float)e;
  float lo = fe * 1.42860682030941723212e-06f;
  lo = lo + lm;
  float hi = fe * 0.693145751953125f;
  return hi + lo;
}

static __device__ __noinline__ double gg_log(double x) {
  uint64_t b = (uint64_t)__double_as_longlong(x);
  int e = (int)(b >> 52) - 1023;
  uint64_t mb = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;
  if (mb > 0x3ff6a09e667f3bcdull) {
    mb -= 0x0010000000000000ull;
    e += 1;
  }
  double m = __longlong_as_double((long long)mb);
  double num = m - 1.0;
  double den = m + 1.0;
  double s = num / den;
  double z = s * s;
  double p = 1.0 / 25.0;
  p = p * z + 1.0 / 23.0;
  p = p * z + 1.0 / 21.0;
  p = p * z + 1.0 / 19.0;
  p = p * z + 1.0 / 17.0;
  p = p * z + 1.0 / 15.0;
  p = p * z + 1.0 / 13.0;
  p = p * z + 1.0 / 11.0;
  p = p * z + 1.0 / 9.0;
  p = p * z + 1.0 / 7.0;
  p = p * z + 1.0 / 5.0;
  p = p * z + 1.0 / 3.0;
  double t = s * z;
  t = t * p;
  double u = s + t;
  double lm = u + u;
  double fe = (double)e;
  double lo = fe * 1.90821492927058770002e-10;
  lo = lo + lm;
  double hi = fe * 6.93147180369123816490e-01;
  return hi + lo;
}

__device__ __forceinline__ float gg_exp(float x) {
  if (x < -87.0f) return 0.0f;
  float t = x * 1.44269504088896340736f;
  t = t + 0.5f;
  int n = (int)t;
  if ((float)n > t) n = n - 1;
  float fn = (float)n;
  float r = x - fn * 0.693145751953125f;
  r = r - fn * 1.42860682030941723212e-06f;
  float p = (float)(1.0 / 5040.0);
  p = p * r + (float)(1.0 / 720.0);
  p = p * r + (float)(1.0 / 120.0);
  p = p * r + (float)(1.0 / 24.0);
  p = p * r + (float)(1.0 / 6.0);
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  float sc = __uint_as_float((uint32_t)(n + 127) << 23);
  return p * sc;
}

__device__ __forceinline__ double gg_exp(double x) {
  if (x < -708.0) return 0.0;
  double t = x * 1.44269504088896338700e+00;
  t = t + 0.5;
  int n = (int)t;
  if ((double)n > t) n = n - 1;
  double fn = (double)n;
  double r = x - fn * 6.93147180369123816490e-01;
  r = r - fn * 1.90821492927058770002e-10;
  double p = 1.0 / 6227020800.0;
  p = p * r + 1.0 / 479001600.0;
  p = p * r + 1.0 / 39916800.0;
  p = p * r + 1.0 / 3628800.0;
  p = p * r + 1.0 / 362880.0;
  p = p * r + 1.0 / 40320.0;
  p = p * r + 1.0 / 5040.0;
  p = p * r + 1.0 / 720.0;
  p = p * r + 1.0 / 120.0;
  p = p * r + 1.0 / 24.0;
  p = p * r + 1.0 / 6.0;
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  double sc = __longlong_as_double((long long)((uint64_t)(n + 1023) << 52));
  return p * sc;
}

// sin and cos of 2*pi*f, f in [0, 1): octant reduction on f (exact), Taylor
// series on [0, pi/4].
__device__ __forceinline__ void gg_sincos_turn(float f, float &sn, float &cs) {
  float t = f * 8.0f;
  int o = (int)t;
  if (o > 7) o = 7;
  float fr = t - (float)o;
  float a = (o & 1) ? (1.0f - fr) : fr;
  a = a * 0.785398163397448309616f;
  float z = a * a;
  float p = (float)(-1.0 / 39916800.0);
  p = p * z + (float)(1.0 / 362880.0);
  p = p * z + (float)(-1.0 / 5040.0);
  p = p * z + (float)(1.0 / 120.0);
  p = p * z + (float)(-1.0 / 6.0);
  float st = z * p;
  st = a * st;
  float s = a + st;
  float q = (float)(1.0 / 479001600.0);
  q = q * z + (float)(-1.0 / 3628800.0);
  q = q * z + (float)(1.0 / 40320.0);
  q = q * z + (float)(-1.0 / 720.0);
  q = q * z + (float)(1.0 / 24.0);
  q = q * z + (float)(-1.0 / 2.0);
  float ct = z * q;
  float c = 1.0f + ct;
  float ss = (o == 1 || o == 2 || o == 5 || o == 6) ? c : s;
  float cc = (o == 1 || o == 2 || o == 5 || o == 6) ? s : c;
  sn = (o >= 4) ? -ss : ss;
  cs = (o >= 2 && o <= 5) ? -cc : cc;
}

__device__ __forceinline__ void gg_sincos_turn(double f, double &sn, double &cs) {
  double t = f * 8.0;
  int o = (int)t;
  if (o > 7) o = 7;
  double fr = t - (double)o;
  double a = (o & 1) ? (1.0 - fr) : fr;
  a = a * 0.785398163397448309616;
  double z = a * a;
  double p = -1.0 / 121645100408832000.0;
  p = p * z + 1.0 / 355687428096000.0;
  p = p * z + -1.0 / 1307674368000.0;
  p = p * z + 1.0 / 6227020800.0;
  p = p * z + -1.0 / 39916800.0;
  p = p * z + 1.0 / 362880.0;
  p = p * z + -1.0 / 5040.0;
  p = p * z + 1.0 / 120.0;
  p = p * z + -1.0 / 6.0;
  double st = z * p;
  st = a * st;
  double s = a + st;
  double q = 1.0 / 2432902008176640000.0;
  q = q * z + -1.0 / 6402373705728000.0;
  q = q * z + 1.0 / 20922789888000.0;
  q = q * z + -1.0 / 87178291200.0;
  q = q * z + 1.0 / 479001600.0;
  q = q * z + -1.0 / 3628800.0;
  q = q * z + 1.0 / 40320.0;
  q = q * z + -1.0 / 720.0;
  q = q * z + 1.0 / 24.0;
  q = q * z + -1.0 / 2.0;
  double ct = z * q;
  double c = 1.0 + ct;
  double ss = (o == 1 || o == 2 || o == 5 || o == 6) ? c : s;
  double cc = (o == 1 || o == 2 || o == 5 || o == 6) ? s : c;
  sn = (o >= 4) ? -ss : ss;
  cs = (o >= 2 && o <= 5) ? -cc : cc;
}

__device__ __forceinline__ float gg_sqrt(float x) { return __fsqrt_rn(x); }
__device__ __forceinline__ double gg_sqrt(double x) { return __dsqrt_rn(x); }
__device__ __forceinline__ float gg_floor(float x) { return floorf(x); }
__device__ __forceinline__ double gg_floor(double x) { return floor(x); }
__device__ __forceinline__ uint64_t to_fixed(float v) { return __float2ull_rn(v * 4294967296.0f); }
__device__ __forceinline__ uint64_t to_fixed(double v) { return __double2ull_rn(v * 4294967296.0); }
__device__ __forceinline__ float gg_inf(float) { return __int_as_float(0x7f800000); }
__device__ __forceinline__ double gg_inf(double) { return __longlong_as_double(0x7ff0000000000000ll); }

// New direction: polar angle (cost, sint) and azimuth (cphi, sphi) measured
// around the old direction u.
template <typename real>
__device__ __forceinline__ void rotate_dir(real &ux, real &uy, real &uz, real cost, real sint, real cphi,
                                           real sphi) {
  real sx = sint * cphi;
  real sy = sint * sphi;
  real sz = cost;
  real p2 = ux * ux;
  p2 = p2 + uy * uy;
  real nx, ny, nz;
  if (p2 > R<real>(1e-20)) {
    real pp = gg_sqrt(p2);
    real inv = R<real>(1) / pp;
    real a = ux * uz;
    a = a * sx;
    a = a - uy * sy;
    a = a * inv;
    nx = a + ux * sz;
    real b = uy * uz;
    b = b * sx;
    b = b + ux * sy;
    b = b * inv;
    ny = b + uy * sz;
    real c = -pp * sx;
    nz = c + uz * sz;
  } else if (uz > R<real>(0)) {
    nx = sx;
    ny = sy;
    nz = sz;
  } else {
    nx = -sx;
    ny = sy;
    nz = -sz;
  }
  real n2 = nx * nx;
  n2 = n2 + ny * ny;
  n2 = n2 + nz * nz;
  real rn = R<real>(1) / gg_sqrt(n2);
  ux = nx * rn;
  uy = ny * rn;
  uz = nz * rn;
}

// ---------------------------------------------------------------------------
// Scene seen by a kernel; table pointers may point into shared memory.
// One simulation of a batched launch: many independent simulations (own
// image, source, seed and tally) share the tables, the world and one set of
// launches.  History h of the batch belongs to the simulation whose range
// [h_begin, h_begin + n) contains it; its Philox stream is (seed, h - h_begin),
// exactly the stream it gets when the simulation runs alone.
template <typename real>
struct SimDesc {
  uint64_t h_begin, n;  // history range in the batch
  uint64_t seed;        // Philox key
  uint64_t vox_off;     // first voxel in the concatenated labels and tallies
  int nx, ny, nz;
  int pos_type, dir_type, ene_type;
  real bmin[3], bmax[3], inv_sp[3];
  real s_t[3], s_half[3], s_mom[3], s_focus[3];
  real s_rot[9];
  real s_radius, s_mono, s_elo, s_ehi;
  real s_cos_tmin, s_cos_tmax, s_phi0_turn, s_dphi_turn;
};

// ---------------------------------------------------------------------------
// One single of the singles list (the C ABI's gg_single, same layout)
struct SingleRec {
  uint64_t event_id;
  int32_t head, run;
  double energy, a1, a2, weight;
};

template <typename real>
struct Scene {
  // tables
  int n_e, n_comp, n_ray, n_mat;
  real ln_emin, inv_dln, e_min;
  const real *sig, *cum, *ray_amax, *ray_x2, *ray_cum, *mat_rho, *maj;
  const int *mat_comp;
  // image
  int nx, ny, nz;
  real bmin[3], bmax[3], inv_sp[3], sp[3];
  const uint16_t *labels;
  // track-length estimator (muen = null: off): energy absorption per unit
  // density [n_comp][n_e], scored-photon energy threshold, kill energy
  const real *muen;
  real tle_thr, tle_emin;
  // dose tally on a grid of its own (dgrid 1; DoseActor size / spacing /
  // translation other than the image's): axis-aligned with the image box,
  // the voxel of a point p is floor((p - dcorner) * dinv_sp) when inside the
  // grid; ddose 1: also the dose tally sum(edep * drho_min / rho)
  int dgrid, dnx, dny, dnz, ddose;
  real dcorner[3], dinv_sp[3], drho_min;
  // batched simulations (n_sims > 0: labels is the concatenation of their
  // images, sim_maj their majorants [n_sims][n_e])
  const SimDesc<real> *sims;
  const real *sim_maj;
  int n_sims;
  // world
  real whalf[3];
  int world_mat;
  // source
  int pos_type, dir_type, ene_type, n_accept, max_rejection, n_spec;
  real s_t[3], s_rot[9], s_half[3], s_radius;
  real s_cos_tmin, s_cos_tmax, s_phi0_turn, s_dphi_turn;
  real s_mom[3], s_focus[3];
  real s_mono, s_elo, s_ehi;
  real s_fd_cmin, s_fd_cmax, s_fd_w;  // forced direction: cone cosines, initial weight (1 otherwise)
  const real *spec_e, *spec_cdf, *acc_box;
  // voxel source
  int vnx, vny, vnz;
  real v_org[3], v_sp[3];
  const real *cdf_z, *cdf_y, *cdf_x;
  // SPECT heads and digitizer (spect = 0: dose path)
  int spect, n_heads, n_win, pnx, pny, n_runs;
  // head frames [n_runs][n_heads][12] (front-face centre, outward normal, e1,
  // e2); history h belongs to run run_base + (h - run_first) / run_len
  const real *frames;
  uint64_t run_first, run_len;
  int run_base;
  // head slabs along the local w axis: region k = [zb[k], zb[k + 1]) of
  // material hmat[k] (-1 vacuum): 0 collimator (with the holes), 1 gap, the
  // optional entrance cover, the crystal (region hreg_cr, the only scored
  // one), the layers behind it; zend = zb[n_hreg] (the head box's depth);
  // side_black: the box's side faces absorb
  real half_w, zb[kHeadRegions + 1], zend, apo, px, py, hpx, hpy, inv_px, inv_py;
  int mat_coll, mat_cr, hmat[kHeadRegions], n_hreg, hreg_cr, side_black;
  real wlo[8], whi[8], pix_half[2], inv_psp[2];
  unsigned long long *proj;
  // digitizer blurring of the singles (GateDigitizerBlurringActor on the energy:
  // eblur 0 off, 1 Gaussian, 2 inverse square, 3 linear law; and
  // GateDigitizerSpatialBlurringActor on the crystal position: sblur 0 off,
  // 1 Gaussian (clamped into the crystal when sb_keep), 2 truncated Gaussian)
  int eblur, sblur, sb_keep;
  int centroid;  // adder policy: 0 EnergyWinnerPosition, 1 EnergyWeightedCentroidPosition
  // free flight outside the heads (GateGammaFreeFlightOptn, heads excluded):
  // ff = 1 on; weight / energy cutoffs; singles then add their weight (2^-32
  // fixed point, with history-by-history squares) to wproj / wproj2
  int ff;  // 0 off, 1 primary free flight, 2 scatter splitting (+ free flight of the copies)
  real ff_wcut, ff_ecut;
  int ss_nc, ss_nr, ss_max;  // splitting factors (Compton, Rayleigh), max Compton level
  real ss_cos;               // copies entering a head with a local dir z below this are dropped (-2: off)
  unsigned long long *wproj, *wproj2;
  real eb_sigma, eb_res, eb_ref, eb_slope, sb_sigma[2];
  // singles list (null: off): records appended at slot atomicAdd(n_singles_rec),
  // kept while the slot is below singles_cap
  SingleRec *singles;
  unsigned long long *n_singles_rec, singles_cap;
};

template <typename real>
struct EIdx {
  int ie;
  real fe;
};

template <typename real>
__device__ __forceinline__ real interp_row(const real *row, const EIdx<real> &ei) {
  real a = row[ei.ie];
  real d = row[ei.ie + 1] - a;
  d = ei.fe * d;
  return a + d;
}

template <typename real>
__device__ __forceinline__ EIdx<real> energy_index(const Scene<real> &s, real e) {
  EIdx<real> r;
  real le = gg_log(e);
  real t = le - s.ln_emin;
  t = t * s.inv_dln;
  int i = (int)t;
  if (i < 0) i = 0;
  if (i > s.n_e - 2) i = s.n_e - 2;
  r.ie = i;
  r.fe = t - (real)i;
  return r;
}

template <typename real>
__device__ __forceinline__ real exit_distance(const real p[3], const real d[3], const real lo[3],
                                              const real hi[3]) {
  real t = gg_inf(real(0));
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (d[a] > R<real>(0)) {
      real ta = (hi[a] - p[a]) / d[a];
      if (ta < t) t = ta;
    } else if (d[a] < R<real>(0)) {
      real ta = (lo[a] - p[a]) / d[a];
      if (ta < t) t = ta;
    }
  }
  if (t < R<real>(0)) t = R<real>(0);
  return t;
}

// exit_distance and the axis of the face it leaves through (the first axis
// reaching the minimum; -1 when no axis bounds the path)
template <typename real>
__device__ __forceinline__ real exit_distance_face(const real p[3], const real d[3], const real lo[3],
                                                   const real hi[3], int &face) {
  real t = gg_inf(real(0));
  face = -1;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (d[a] > R<real>(0)) {
      real ta = (hi[a] - p[a]) / d[a];
      if (ta < t) t = ta, face = a;
    } else if (d[a] < R<real>(0)) {
      real ta = (lo[a] - p[a]) / d[a];
      if (ta < t) t = ta, face = a;
    }
  }
  if (t < R<real>(0)) t = R<real>(0);
  return t;
}

template <typename real>
__device__ __forceinline__ real entry_distance(const real p[3], const real d[3], const real lo[3],
                                               const real hi[3]) {
  real inf = gg_inf(real(0));
  real tnear = -inf, tfar = inf;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (d[a] == R<real>(0)) {
      if (p[a] < lo[a] || p[a] > hi[a]) return inf;
    } else {
      real t1 = (lo[a] - p[a]) / d[a];
      real t2 = (hi[a] - p[a]) / d[a];
      if (t1 > t2) {
        real tmp = t1;
        t1 = t2;
        t2 = tmp;
      }
      if (t1 > tnear) tnear = t1;
      if (t2 < tfar) tfar = t2;
    }
  }
  if (tnear > tfar || tfar < R<real>(0)) return inf;
  return tnear > R<real>(0) ? tnear : R<real>(0);
}

// entry_distance and the axis of the face it enters through (the first axis
// reaching the largest near distance; -1 from inside or parallel to all)
template <typename real>
__device__ __forceinline__ real entry_distance_face(const real p[3], const real d[3], const real lo[3],
                                                    const real hi[3], int &face) {
  real inf = gg_inf(real(0));
  real tnear = -inf, tfar = inf;
  face = -1;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (d[a] == R<real>(0)) {
      if (p[a] < lo[a] || p[a] > hi[a]) return inf;
    } else {
      real t1 = (lo[a] - p[a]) / d[a];
      real t2 = (hi[a] - p[a]) / d[a];
      if (t1 > t2) {
        real tmp = t1;
        t1 = t2;
        t2 = tmp;
      }
      if (t1 > tnear) tnear = t1, face = a;
      if (t2 < tfar) tfar = t2;
    }
  }
  if (tnear > tfar || tfar < R<real>(0)) return inf;
  return tnear > R<real>(0) ? tnear : R<real>(0);
}

template <typename real>
__device__ __forceinline__ bool inside_box(const real p[3], const real lo[3], const real hi[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
    if (p[a] < lo[a] || p[a] > hi[a]) return false;
  return true;
}

template <typename real>
struct Photon {
  real pos[3], dir[3], e;
  real t_exit, mumax, inv_mumax;
  EIdx<real> ei;
  int alive, in_image, can_enter, steps;
  // SPECT: box not to re-enter before the next direction change (-1 none,
  // 0 image, 1 + h head h); head-local state while in_head
  int in_head, head, hreg, left_hole, exclude;
  int run;  // SPECT gantry position of the history
  real w;   // SPECT free flight: statistical weight (1 otherwise)
};

template <typename real>
struct EState {
  int ie;
  real fe, mumax, inv_mumax;
};

// Energy-grid position and majorant of energy e (out of line: it is reached
// from the source stage, every Compton scattering, pair conversion and
// secondary pop).
template <typename real>
static __device__ __noinline__ EState<real> energy_state(const real *maj, real ln_emin, real inv_dln, int n_e, real e) {
  EState<real> r;
  real le = gg_log(e);
  real t = le - ln_emin;
  t = t * inv_dln;
  int i = (int)t;
  if (i < 0) i = 0;
  if (i > n_e - 2) i = n_e - 2;
  r.ie = i;
  r.fe = t - (real)i;
  real a = maj[i];
  real d = maj[i + 1] - a;
  d = r.fe * d;
  real mm = a + d;
  r.mumax = mm;
  r.inv_mumax = R<real>(1) / mm;
  return r;
}

template <typename real>
__device__ __forceinline__ void set_energy(const Scene<real> &s, Photon<real> &ph, real e) {
  ph.e = e;
  EState<real> st = energy_state(s.maj, s.ln_emin, s.inv_dln, s.n_e, e);
  ph.ei.ie = st.ie;
  ph.ei.fe = st.fe;
  ph.mumax = st.mumax;
  ph.inv_mumax = st.inv_mumax;
}

template <typename real>
__device__ __forceinline__ void start_photon(const Scene<real> &s, Photon<real> &ph) {
  ph.steps = 0;
  ph.in_head = 0;
  ph.exclude = -1;
  if (inside_box(ph.pos, s.bmin, s.bmax)) {
    ph.in_image = 1;
    ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
  } else {
    ph.in_image = 0;
    ph.can_enter = 1;
  }
}

}  // namespace gg
