/*
 * gg_oracle.c - CPU oracle for the voxelised photon-transport path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of bench.py call it; the product path
 * (opengate_gb300 + libgategpu.so) never links, loads or calls it.
 *
 * It restates, in plain C and one history at a time, what the reference does
 * on this path:
 *   - primary generation: GateGenericSource::GeneratePrimaries and the SPS
 *     samplers (core/opengate_core/opengate_lib/GateGenericSource.cpp:209-262,
 *     312-664; GateSingleParticleSource.cpp:67-137 for the acceptance loop;
 *     GateSPSEneDistribution.cpp:116-159 for lines/histogram sampling);
 *   - the voxel lookup of GateImageNestedParameterisation::ComputeMaterial
 *     (GateImageNestedParameterisation.cpp:47-75) and the image index of
 *     GateDoseActor::GetVoxelPosition (GateDoseActor.cpp:144-178,
 *     GateHelpersImage.txx:60-92);
 *   - the photon physics of G4EmStandardPhysics as restated from the Geant4
 *     Physics Reference Manual (Klein-Nishina sampling of Butcher & Messel,
 *     photoelectric absorption with local deposit, Rayleigh from tabulated
 *     form factors, pair production with both leptons stopped at creation and
 *     the positron annihilating at rest into two 511 keV photons, the
 *     min_ekine user limit of opengate/physics.py:699-753);
 *   - DoseActor scoring: edep per voxel and the history-by-history squared sum
 *     (GateDoseActor.cpp:180-243 SteppingAction, 359-397 ScoreSquaredValue /
 *     FlushSquaredValues).
 *
 * The arithmetic is the same operation sequence the CUDA kernels execute
 * (float or double, no contraction of a*b+c, correctly rounded + - * / sqrt,
 * logarithm / exponential / sine-cosine built from those operations), with the
 * same counter-based Philox4x32-10 stream per history, so a GPU run and this
 * oracle agree bit for bit.  Tallies are 64-bit fixed point (2^-32 MeV and
 * 2^-32 MeV^2 units) per batch, flushed into float64 images, which makes the
 * totals independent of the order in which histories finish.
 *
 * Build: see oracle/build_oracle.py (gcc -O2 -ffp-contract=off, once with
 * -DGGO_DOUBLE for the FP64 variant).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/gate_gpu.h"

#ifdef GGO_DOUBLE
typedef double real;
#define R(x) ((double)(x))
#define GGO_PREFIX(name) ggo64_##name
#else
typedef float real;
#define R(x) ((float)(x))
#define GGO_PREFIX(name) ggo32_##name
#endif

#define HIST_LIST 8
#define LOOP_CAP 1000
#define STEP_CAP 1000000
#define MC2 0.51099895
#define HC_MEV_ANGSTROM 12.398419843320026e-3

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)                         */
/* ------------------------------------------------------------------------ */
static void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

typedef struct {
  uint32_t key[2];
  uint32_t ctr[4]; /* ctr[0] = block index, ctr[1] = stream, ctr[2..3] = history */
  uint32_t buf[4];
  int idx;
} rng_t;

static void rng_init(rng_t *g, uint64_t seed, uint64_t history, uint32_t stream) {
  g->key[0] = (uint32_t)seed;
  g->key[1] = (uint32_t)(seed >> 32);
  g->ctr[0] = 0;
  g->ctr[1] = stream;
  g->ctr[2] = (uint32_t)history;
  g->ctr[3] = (uint32_t)(history >> 32);
  g->idx = 4;
}

static uint32_t rng_u32(rng_t *g) {
  if (g->idx == 4) {
    philox4x32_10(g->ctr, g->key, g->buf);
    g->ctr[0] += 1u;
    g->idx = 0;
  }
  return g->buf[g->idx++];
}

/* uniform in [0, 1) with 24-bit resolution */
static real u01(rng_t *g) { return (real)(rng_u32(g) >> 8) * R(5.9604644775390625e-08); }
/* uniform in (0, 1] */
static real u01_open0(rng_t *g) { return (real)((rng_u32(g) >> 8) + 1u) * R(5.9604644775390625e-08); }

/* ------------------------------------------------------------------------ */
/* Elementary functions from + - * / (series of Abramowitz & Stegun 4.1.27,  */
/* 4.2.1, 4.3.65/66 after Cody-Waite style range reduction)                  */
/* ------------------------------------------------------------------------ */
#ifndef GGO_DOUBLE
static real ggo_log(real x) {
  uint32_t b;
  memcpy(&b, &x, 4);
  int e = (int)(b >> 23) - 127;
  uint32_t mb = (b & 0x007fffffu) | 0x3f800000u;
  if (mb > 0x3fb504f3u) {
    mb -= 0x00800000u;
    e += 1;
  }
  float m;
  memcpy(&m, &mb, 4);
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

static real ggo_exp(real x) {
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
  uint32_t sb = (uint32_t)(n + 127) << 23;
  float sc;
  memcpy(&sc, &sb, 4);
  return p * sc;
}

static void ggo_sincos_turn(real f, real *sn, real *cs) {
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
  switch (o) {
  case 0: *sn = s; *cs = c; break;
  case 1: *sn = c; *cs = s; break;
  case 2: *sn = c; *cs = -s; break;
  case 3: *sn = s; *cs = -c; break;
  case 4: *sn = -s; *cs = -c; break;
  case 5: *sn = -c; *cs = -s; break;
  case 6: *sn = -c; *cs = s; break;
  default: *sn = -s; *cs = c; break;
  }
}
#else
static real ggo_log(real x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  int e = (int)(b >> 52) - 1023;
  uint64_t mb = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;
  if (mb > 0x3ff6a09e667f3bcdull) {
    mb -= 0x0010000000000000ull;
    e += 1;
  }
  double m;
  memcpy(&m, &mb, 8);
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

static real ggo_exp(real x) {
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
  uint64_t sb = (uint64_t)(n + 1023) << 52;
  double sc;
  memcpy(&sc, &sb, 8);
  return p * sc;
}

static void ggo_sincos_turn(real f, real *sn, real *cs) {
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
  switch (o) {
  case 0: *sn = s; *cs = c; break;
  case 1: *sn = c; *cs = s; break;
  case 2: *sn = c; *cs = -s; break;
  case 3: *sn = s; *cs = -c; break;
  case 4: *sn = -s; *cs = -c; break;
  case 5: *sn = -c; *cs = -s; break;
  case 6: *sn = -c; *cs = s; break;
  default: *sn = -s; *cs = c; break;
  }
}
#endif

static real ggo_sqrt(real x) {
#ifdef GGO_DOUBLE
  return sqrt(x);
#else
  return sqrtf(x);
#endif
}

/* New direction from polar (cos t, sin t) and azimuth (cos p, sin p) around
   the old direction u: the rotation that takes the z axis onto u. */
static void rotate_dir(real u[3], real cost, real sint, real cphi, real sphi) {
  real sx = sint * cphi;
  real sy = sint * sphi;
  real sz = cost;
  real ux = u[0], uy = u[1], uz = u[2];
  real p2 = ux * ux;
  p2 = p2 + uy * uy;
  real nx, ny, nz;
  if (p2 > R(1e-20)) {
    real pp = ggo_sqrt(p2);
    real inv = R(1) / pp;
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
  } else if (uz > R(0)) {
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
  real rn = R(1) / ggo_sqrt(n2);
  u[0] = nx * rn;
  u[1] = ny * rn;
  u[2] = nz * rn;
}

/* ------------------------------------------------------------------------ */
/* Scene in working precision                                                */
/* ------------------------------------------------------------------------ */
typedef struct {
  /* tables */
  int n_e, n_comp, n_ray, n_mat;
  real ln_emin, inv_dln, e_min, e_max;
  real *sig, *cum, *ray_amax, *ray_x2, *ray_cum, *mat_rho;
  int *mat_comp;
  /* image */
  int nx, ny, nz;
  real bmin[3], bmax[3], inv_sp[3], sp[3];
  const uint16_t *labels;
  real *maj;
  /* dose tally on a grid of its own (gg_set_dose_grid): dgrid = 0 off */
  int dgrid, dnx, dny, dnz, ddose;
  real dcorner[3], dinv_sp[3], drho_min;
  /* track-length estimator (GateTLEDoseActor): tle = 0 off */
  int tle;
  real tle_thr, tle_emin;
  real *muen; /* [n_comp][n_e] */
  /* world */
  real whalf[3];
  int world_mat;
  /* source */
  gg_source_desc src;
  real s_t[3], s_rot[9], s_half[3], s_radius;
  real s_cos_tmin, s_cos_tmax, s_phi0_turn, s_dphi_turn;
  real s_fd_cmin, s_fd_cmax, s_fd_w; /* forced direction: cone cosines, initial weight (1 otherwise) */
  real s_mom[3], s_focus[3];
  real s_mono, s_elo, s_ehi;
  real *s_spec_e, *s_spec_cdf;
  real *acc_box;
  /* voxel source (GateSPSVoxelsPosDistribution) */
  int vnx, vny, vnz;
  real v_org[3], v_sp[3]; /* centre of voxel (0,0,0), spacing */
  real *cdf_z, *cdf_y, *cdf_x;
  /* SPECT heads and projection digitizer */
  int spect, n_heads, n_win, pnx, pny, n_runs, run;
  real hc[2][3], hu[2][3], he1[2][3], he2[2][3];
  /* head slabs along w: region k = [zb[k], zb[k + 1]) of material hmat[k]
     (-1 vacuum): collimator (holes), gap, optional cover, crystal (hreg_cr,
     the scored one), back layers; zend = zb[n_hreg]; side_black: the box's
     side faces absorb (gg_spect_desc.shielded_sides) */
  real half_w, zb[9], zend, apo, px, py, hpx, hpy, inv_px, inv_py;
  int mat_coll, mat_cr, hmat[8], n_hreg, hreg_cr, side_black;
  real wlo[8], whi[8], pix_half[2], inv_psp[2];
  uint64_t *proj; /* [head][run][window][pny][pnx], shared, atomics */
  /* digitizer blurring (gg_blur_desc): eblur 0 off / 1 Gaussian / 2 inverse
     square / 3 linear; sblur 0 off / 1 Gaussian (+ clamp) / 2 truncated */
  int eblur, sblur, sb_keep;
  int centroid; /* adder policy EnergyWeightedCentroidPosition */
  /* free flight outside the heads (gg_ff_desc) and its weighted projection */
  int ff; /* 0 off, 1 primary free flight, 2 scatter splitting */
  real ff_wcut, ff_ecut;
  int ss_nc, ss_nr, ss_max;
  real ss_cos; /* angle check: copies entering a head with local dir z below this are dropped */
  uint64_t *wproj, *wproj2;
  real eb_sigma, eb_res, eb_ref, eb_slope, sb_sigma[2];
  const struct arf_s *arf; /* ARF detector model, or NULL */
} scene_t;

typedef struct {
  int ie;
  real fe;
} eidx_t;

static real interp_row(const real *row, eidx_t ei) {
  real a = row[ei.ie];
  real d = row[ei.ie + 1] - a;
  d = ei.fe * d;
  return a + d;
}

static eidx_t energy_index(const scene_t *s, real e) {
  eidx_t r;
  real le = ggo_log(e);
  real t = le - s->ln_emin;
  t = t * s->inv_dln;
  int i = (int)t;
  if (i < 0) i = 0;
  if (i > s->n_e - 2) i = s->n_e - 2;
  r.ie = i;
  r.fe = t - (real)i;
  return r;
}

/* distance to leave box [lo, hi] from p along d (p assumed inside) */
static real exit_distance(const real p[3], const real d[3], const real lo[3], const real hi[3]) {
  real t = R(INFINITY);
  for (int a = 0; a < 3; ++a) {
    real ta;
    if (d[a] > R(0)) {
      ta = (hi[a] - p[a]) / d[a];
      if (ta < t) t = ta;
    } else if (d[a] < R(0)) {
      ta = (lo[a] - p[a]) / d[a];
      if (ta < t) t = ta;
    }
  }
  if (t < R(0)) t = R(0);
  return t;
}

/* exit_distance and the axis of the face it leaves through (first axis
   reaching the minimum, -1 if none) */
static real exit_distance_face(const real p[3], const real d[3], const real lo[3], const real hi[3], int *face) {
  real t = R(INFINITY);
  *face = -1;
  for (int a = 0; a < 3; ++a) {
    real ta;
    if (d[a] > R(0)) {
      ta = (hi[a] - p[a]) / d[a];
      if (ta < t) t = ta, *face = a;
    } else if (d[a] < R(0)) {
      ta = (lo[a] - p[a]) / d[a];
      if (ta < t) t = ta, *face = a;
    }
  }
  if (t < R(0)) t = R(0);
  return t;
}

/* entry_distance and the axis of the face it enters through */
static real entry_distance_face(const real p[3], const real d[3], const real lo[3], const real hi[3], int *face) {
  real tnear = -R(INFINITY), tfar = R(INFINITY);
  *face = -1;
  for (int a = 0; a < 3; ++a) {
    if (d[a] == R(0)) {
      if (p[a] < lo[a] || p[a] > hi[a]) return R(INFINITY);
    } else {
      real t1 = (lo[a] - p[a]) / d[a];
      real t2 = (hi[a] - p[a]) / d[a];
      if (t1 > t2) {
        real tmp = t1;
        t1 = t2;
        t2 = tmp;
      }
      if (t1 > tnear) tnear = t1, *face = a;
      if (t2 < tfar) tfar = t2;
    }
  }
  if (tnear > tfar || tfar < R(0)) return R(INFINITY);
  return tnear > R(0) ? tnear : R(0);
}

/* slab of head depth w: the inner bounds at or below it */
static int head_region(const scene_t *s, real w) {
  int k = 0;
  for (int j = 1; j < s->n_hreg; ++j) k += !(w < s->zb[j]);
  return k;
}

/* distance to enter box [lo, hi] from p along d; INFINITY if missed */
static real entry_distance(const real p[3], const real d[3], const real lo[3], const real hi[3]) {
  real tnear = -R(INFINITY), tfar = R(INFINITY);
  for (int a = 0; a < 3; ++a) {
    if (d[a] == R(0)) {
      if (p[a] < lo[a] || p[a] > hi[a]) return R(INFINITY);
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
  if (tnear > tfar || tfar < R(0)) return R(INFINITY);
  return tnear > R(0) ? tnear : R(0);
}

/* ------------------------------------------------------------------------ */
/* History state and tally                                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
  uint32_t vox[HIST_LIST];
  real acc[HIST_LIST];
  int n;
} hlist_t;

typedef struct {
  uint64_t *acc_e, *acc_e2; /* shared per batch, updated with atomics */
  uint64_t cnt[GG_N_COUNTERS];
  uint32_t ss_next; /* scatter splitting: copies of the current history so far */
  /* dose grid with the dose tally: sum(edep rho_min / rho), its squares, and
     the history's dose list (same voxels as its edep list) */
  uint64_t *acc_d, *acc_d2;
  hlist_t *ld;
} tally_t;

static uint64_t to_fixed(real v) {
  /* v * 2^32 is exact; round to nearest even */
#ifdef GGO_DOUBLE
  return (uint64_t)llrint(v * 4294967296.0);
#else
  return (uint64_t)llrintf(v * 4294967296.0f);
#endif
}

/* q = to_fixed(history's voxel sum) goes to acc_e[v]; q^2 (units 2^-64 MeV^2)
   is split into its low 32 bits, added to acc_e2[2v], and q^2 >> 32 (units
   2^-32 MeV^2), added to acc_e2[2v+1]; sum = acc_e2[2v+1] 2^-32 + acc_e2[2v] 2^-64. */
static void hlist_flush(hlist_t *l, tally_t *t) {
  for (int k = 0; k < l->n; ++k) {
    uint64_t q = to_fixed(l->acc[k]);
    size_t v = l->vox[k];
    __atomic_fetch_add(&t->acc_e[v], q, __ATOMIC_RELAXED);
    if (t->acc_e2) {
      unsigned __int128 sq = (unsigned __int128)q * q;
      __atomic_fetch_add(&t->acc_e2[2 * v], (uint64_t)sq & 0xffffffffu, __ATOMIC_RELAXED);
      __atomic_fetch_add(&t->acc_e2[2 * v + 1], (uint64_t)(sq >> 32), __ATOMIC_RELAXED);
    }
  }
  t->cnt[GG_CNT_TALLY_ENTRIES] += (uint64_t)l->n;
  l->n = 0;
}

/* The dose list of a history: flushed and filled like the edep list, into
   acc_d / acc_d2, without counting (the counters describe the edep list). */
static void dose_flush(hlist_t *l, tally_t *t) {
  for (int k = 0; k < l->n; ++k) {
    uint64_t q = to_fixed(l->acc[k]);
    size_t v = l->vox[k];
    __atomic_fetch_add(&t->acc_d[v], q, __ATOMIC_RELAXED);
    if (t->acc_d2) {
      unsigned __int128 sq = (unsigned __int128)q * q;
      __atomic_fetch_add(&t->acc_d2[2 * v], (uint64_t)sq & 0xffffffffu, __ATOMIC_RELAXED);
      __atomic_fetch_add(&t->acc_d2[2 * v + 1], (uint64_t)(sq >> 32), __ATOMIC_RELAXED);
    }
  }
  l->n = 0;
}

static void dose_deposit(hlist_t *l, tally_t *t, uint32_t v, real e) {
  if (!(e > R(0))) return;
  for (int k = 0; k < l->n; ++k) {
    if (l->vox[k] == v) {
      l->acc[k] = l->acc[k] + e;
      return;
    }
  }
  if (l->n == HIST_LIST) dose_flush(l, t);
  l->vox[l->n] = v;
  l->acc[l->n] = e;
  l->n++;
}

static void deposit(hlist_t *l, tally_t *t, uint32_t v, real e) {
  if (!(e > R(0))) return;
  t->cnt[GG_CNT_DEPOSITS]++;
  for (int k = 0; k < l->n; ++k) {
    if (l->vox[k] == v) {
      l->acc[k] = l->acc[k] + e;
      return;
    }
  }
  if (l->n == HIST_LIST) {
    t->cnt[GG_CNT_LIST_OVERFLOWS]++;
    hlist_flush(l, t);
  }
  l->vox[l->n] = v;
  l->acc[l->n] = e;
  l->n++;
}

typedef struct {
  real pos[3], dir[3], e; /* world frame; head-local frame while in_head */
  int alive, in_image, can_enter;
  real t_exit;
  eidx_t ei;
  real mumax, inv_mumax;
  /* SPECT: exclude = box not to re-enter before the next direction change
     (-1 none, 0 image, 1 + h head h); head, hreg (0 collimator, 1 gap,
     2 crystal) and left_hole while inside a head */
  int in_head, head, hreg, left_hole, exclude;
  /* ARF: visited_head = the photon was tracked in a head before (it then
     always stays with plain tracking); head_stage = it is being tracked with
     the heads since its last image entry (head-to-head flights skip the ARF) */
  int visited_head, head_stage;
  real w; /* free flight: statistical weight */
  int kind;   /* last interaction (KIND_*), set by interact */
  int ncompt; /* scatter splitting: Compton interactions of this track */
} photon_t;

enum { KIND_COMPTON = 1, KIND_PHOTO = 2, KIND_RAYLEIGH = 3, KIND_PAIR = 4 };

/* per-event crystal accumulation of each head (adder, EnergyWinnerPosition);
   wpos = head-local (a1, a2) of the energy winner */
typedef struct {
  real esum[2], emax[2], wpos[2][2];
  real w[2]; /* weight of each head's single (free flight) */
} event_t;

static void set_energy(const scene_t *s, photon_t *ph, real e) {
  ph->e = e;
  ph->ei = energy_index(s, e);
  real mm = interp_row(s->maj, ph->ei);
  ph->mumax = mm;
  ph->inv_mumax = R(1) / mm;
}

/* ------------------------------------------------------------------------ */
/* Interactions                                                              */
/* ------------------------------------------------------------------------ */
/* Klein-Nishina sampling, composition + rejection method of the Geant4
   Physics Reference Manual (G4KleinNishinaCompton). */
static void compton(const scene_t *s, photon_t *ph, rng_t *g, tally_t *t, real *edep_out) {
  real e = ph->e;
  real k = e * R(1.0 / MC2);
  real twok = R(2) * k;
  real eps0 = R(1) / (R(1) + twok);
  real eps0sq = eps0 * eps0;
  real alpha1 = -ggo_log(eps0);
  real alpha2 = R(1) - eps0sq;
  alpha2 = R(0.5) * alpha2;
  alpha2 = alpha1 + alpha2;
  real eps, epssq, onecost, sint2;
  int it = 0;
  for (;;) {
    real r0 = u01(g), r1 = u01(g), r2 = u01(g);
    if (alpha1 > alpha2 * r0) {
      eps = ggo_exp(-alpha1 * r1);
      epssq = eps * eps;
    } else {
      real w = R(1) - eps0sq;
      w = w * r1;
      epssq = eps0sq + w;
      eps = ggo_sqrt(epssq);
    }
    real ek = eps * k;
    onecost = (R(1) - eps) / ek;
    sint2 = onecost * (R(2) - onecost);
    real gr = eps * sint2;
    gr = gr / (R(1) + epssq);
    gr = R(1) - gr;
    if (gr >= r2) break;
    if (++it >= LOOP_CAP) {
      t->cnt[GG_CNT_LOOP_CAPPED]++;
      break;
    }
  }
  real e1 = eps * e;
  *edep_out = e - e1;
  real cost = R(1) - onecost;
  real sint = ggo_sqrt(sint2 > R(0) ? sint2 : R(0));
  real sp, cp;
  ggo_sincos_turn(u01(g), &sp, &cp);
  rotate_dir(ph->dir, cost, sint, cp, sp);
  if (e1 < s->e_min) {
    *edep_out = *edep_out + e1;
    ph->alive = 0;
  } else {
    set_energy(s, ph, e1);
  }
}

/* Rayleigh scattering: x^2 = (sin(theta/2)/lambda)^2 drawn from the
   tabulated form-factor cumulative (exact inversion of the piecewise-linear
   cumulative by bisection), x^2 beyond (E/hc)^2 rejected, then the angle kept
   with probability (1 + cos^2 theta)/2. */
static void rayleigh(const scene_t *s, int comp, photon_t *ph, rng_t *g, tally_t *t) {
  real k = ph->e * R(1.0 / HC_MEV_ANGSTROM);
  real x2max = k * k;
  real amax = interp_row(s->ray_amax + (size_t)comp * s->n_e, ph->ei);
  const real *cu = s->ray_cum + (size_t)comp * s->n_ray;
  const real *xn = s->ray_x2;
  real cost = R(1);
  int it = 0;
  for (;;) {
    if (++it > LOOP_CAP) {
      t->cnt[GG_CNT_LOOP_CAPPED]++;
      break;
    }
    real r = u01(g);
    real tt = r * amax;
    int lo = 0, hi = s->n_ray - 1;
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (cu[mid] <= tt) lo = mid;
      else hi = mid;
    }
    real den = cu[lo + 1] - cu[lo];
    real f = R(0);
    if (den > R(0)) {
      f = tt - cu[lo];
      f = f / den;
    }
    real d = xn[lo + 1] - xn[lo];
    d = f * d;
    real x2 = xn[lo] + d;
    if (x2 > x2max) continue;
    real q = R(2) * x2;
    q = q / x2max;
    cost = R(1) - q;
    real r2 = u01(g);
    real lhs = R(2) * r2;
    real rhs = cost * cost;
    rhs = R(1) + rhs;
    if (lhs <= rhs) break;
  }
  real st2 = cost * cost;
  st2 = R(1) - st2;
  real sint = ggo_sqrt(st2 > R(0) ? st2 : R(0));
  real sp, cp;
  ggo_sincos_turn(u01(g), &sp, &cp);
  rotate_dir(ph->dir, cost, sint, cp, sp);
}

static void iso_dir(rng_t *g, real d[3]) {
  real cost = R(2) * u01(g);
  cost = R(1) - cost;
  real st2 = cost * cost;
  st2 = R(1) - st2;
  real sint = ggo_sqrt(st2 > R(0) ? st2 : R(0));
  real sp, cp;
  ggo_sincos_turn(u01(g), &sp, &cp);
  d[0] = sint * cp;
  d[1] = sint * sp;
  d[2] = cost;
}

/* ------------------------------------------------------------------------ */
/* Source                                                                    */
/* ------------------------------------------------------------------------ */
static void rot_apply(const real m[9], const real v[3], real o[3]) {
  for (int i = 0; i < 3; ++i) {
    real a = m[3 * i] * v[0];
    a = a + m[3 * i + 1] * v[1];
    a = a + m[3 * i + 2] * v[2];
    o[i] = a;
  }
}

static int accept_dir(const scene_t *s, const real p[3], const real d[3]) {
  for (int b = 0; b < s->src.n_accept; ++b) {
    const real *bx = s->acc_box + 6 * b;
    if (entry_distance(p, d, bx, bx + 3) < R(INFINITY)) return 1;
  }
  return 0;
}

/* ForceDirection of the angular acceptance (GateForcedDirectionManager.cpp
   SampleDirectionWithinCone): history h aims at head h mod n_heads, about its
   axis a: u1 from the larger of |a_x|, |a_y|, u2 = a x u1 (normalised); phi
   uniform (first draw), cos(theta) uniform in [cos max, cos min]. */
static void forced_direction(const scene_t *s, uint64_t hid, rng_t *g, real d[3]) {
  const int head = (int)(hid % (uint64_t)s->n_heads);
  const real *a = s->hu[head];
  real u1[3], u2[3];
  const real ax = a[0] < R(0) ? -a[0] : a[0];
  const real ay = a[1] < R(0) ? -a[1] : a[1];
  if (ax > ay) {
    u1[0] = a[2];
    u1[1] = R(0);
    u1[2] = -a[0];
  } else {
    u1[0] = R(0);
    u1[1] = -a[2];
    u1[2] = a[1];
  }
  real n = u1[0] * u1[0];
  n = n + u1[1] * u1[1];
  n = n + u1[2] * u1[2];
  n = R(1) / ggo_sqrt(n);
  for (int k = 0; k < 3; ++k) u1[k] = u1[k] * n;
  u2[0] = a[1] * u1[2] - a[2] * u1[1];
  u2[1] = a[2] * u1[0] - a[0] * u1[2];
  u2[2] = a[0] * u1[1] - a[1] * u1[0];
  n = u2[0] * u2[0];
  n = n + u2[1] * u2[1];
  n = n + u2[2] * u2[2];
  n = R(1) / ggo_sqrt(n);
  for (int k = 0; k < 3; ++k) u2[k] = u2[k] * n;
  const real v = u01(g);
  real sp, cp;
  ggo_sincos_turn(v, &sp, &cp);
  real c = s->s_fd_cmin - s->s_fd_cmax;
  c = u01(g) * c;
  c = s->s_fd_cmax + c;
  real st = c * c;
  st = R(1) - st;
  st = ggo_sqrt(st > R(0) ? st : R(0));
  for (int k = 0; k < 3; ++k) {
    real t = cp * u1[k];
    const real t2 = sp * u2[k];
    t = t + t2;
    t = st * t;
    d[k] = a[k] * c;
    d[k] = d[k] + t;
  }
}

static void sample_direction(const scene_t *s, const real p[3], rng_t *g, real d[3], uint64_t hid) {
  if (s->src.dir_type == GG_DIR_FORCED) {
    forced_direction(s, hid, g, d);
  } else if (s->src.dir_type == GG_DIR_ISO) {
    real u = u01(g);
    real cost = s->s_cos_tmin - s->s_cos_tmax;
    cost = u * cost;
    cost = s->s_cos_tmin - cost;
    real st2 = cost * cost;
    st2 = R(1) - st2;
    real sint = ggo_sqrt(st2 > R(0) ? st2 : R(0));
    real f = s->s_dphi_turn * u01(g);
    f = s->s_phi0_turn + f;
    f = f - (real)floor((double)f);
    real sp, cp;
    ggo_sincos_turn(f, &sp, &cp);
    d[0] = -(sint * cp);
    d[1] = -(sint * sp);
    d[2] = -cost;
  } else if (s->src.dir_type == GG_DIR_MOMENTUM) {
    d[0] = s->s_mom[0];
    d[1] = s->s_mom[1];
    d[2] = s->s_mom[2];
  } else {
    real v[3];
    for (int a = 0; a < 3; ++a) v[a] = s->s_focus[a] - p[a];
    real n2 = v[0] * v[0];
    n2 = n2 + v[1] * v[1];
    n2 = n2 + v[2] * v[2];
    real rn = R(1) / ggo_sqrt(n2);
    for (int a = 0; a < 3; ++a) d[a] = v[a] * rn;
  }
}

static int sample_primary(const scene_t *s, rng_t *g, photon_t *ph, tally_t *t, uint64_t hid) {
  real loc[3] = {R(0), R(0), R(0)};
  int pt = s->src.pos_type;
  if (pt == GG_POS_BOX) {
    for (int a = 0; a < 3; ++a) {
      real u = R(2) * u01(g);
      u = u - R(1);
      loc[a] = u * s->s_half[a];
    }
  } else if (pt == GG_POS_SPHERE || pt == GG_POS_DISC) {
    int it = 0;
    for (;;) {
      real r2 = R(0);
      int na = (pt == GG_POS_SPHERE) ? 3 : 2;
      for (int a = 0; a < na; ++a) {
        real u = R(2) * u01(g);
        u = u - R(1);
        loc[a] = u * s->s_radius;
        r2 = r2 + loc[a] * loc[a];
      }
      real rr = s->s_radius * s->s_radius;
      if (r2 <= rr) break;
      if (++it >= LOOP_CAP) {
        t->cnt[GG_CNT_LOOP_CAPPED]++;
        break;
      }
    }
  }
  if (pt == GG_POS_VOXELS) {
    /* GateSPSVoxelsPosDistribution::VGenerateOne: z, then y | z, then x | z, y */
    int idx[3];
    const real *rows[3] = {s->cdf_z, NULL, NULL};
    int len[3] = {s->vnz, s->vny, s->vnx};
    for (int lev = 0; lev < 3; ++lev) {
      const real *c = lev == 0 ? s->cdf_z
                     : lev == 1 ? s->cdf_y + (size_t)idx[0] * s->vny
                                : s->cdf_x + ((size_t)idx[0] * s->vny + (size_t)idx[1]) * s->vnx;
      (void)rows;
      int k, it = 0;
      do {
        real p = u01_open0(g);
        int lo = 0, hi = len[lev];
        while (lo < hi) { /* lower_bound: first entry >= p */
          int mid = (lo + hi) >> 1;
          if (c[mid] < p) lo = mid + 1;
          else hi = mid;
        }
        k = lo;
        if (++it >= LOOP_CAP) {
          t->cnt[GG_CNT_LOOP_CAPPED]++;
          if (k >= len[lev]) k = len[lev] - 1;
          break;
        }
      } while (k >= len[lev]);
      idx[lev] = k;
    }
    int ind[3] = {idx[2], idx[1], idx[0]}; /* x, y, z */
    for (int a = 0; a < 3; ++a) {
      real x = (real)ind[a] * s->v_sp[a];
      x = s->v_org[a] + x;
      real j = u01(g) - R(0.5);
      j = j * s->v_sp[a];
      ph->pos[a] = x + j;
    }
  } else {
    real off[3];
    rot_apply(s->s_rot, loc, off);
    for (int a = 0; a < 3; ++a) ph->pos[a] = s->s_t[a] + off[a];
  }
  /* direction, with the acceptance loop of GateSingleParticleSource */
  int tries = 0;
  for (;;) {
    sample_direction(s, ph->pos, g, ph->dir, hid);
    if (s->src.n_accept == 0 || accept_dir(s, ph->pos, ph->dir)) break;
    t->cnt[GG_CNT_SKIPPED]++;
    if (++tries > s->src.max_rejection) return GG_ERR_DOMAIN;
  }
  /* energy */
  real e;
  int et = s->src.ene_type;
  if (et == GG_ENE_MONO) {
    e = s->s_mono;
  } else if (et == GG_ENE_RANGE) {
    real w = s->s_ehi - s->s_elo;
    w = w * u01(g);
    e = s->s_elo + w;
  } else {
    real p = u01(g);
    int i = 0;
    while (i < s->src.n_spec - 1 && p >= s->s_spec_cdf[i]) ++i;
    if (et == GG_ENE_LINES) {
      e = s->s_spec_e[i];
    } else {
      real a = s->s_spec_e[i];
      real w = s->s_spec_e[i + 1] - a;
      w = w * u01(g);
      e = a + w;
    }
  }
  ph->alive = 1;
  ph->can_enter = 1;
  ph->in_image = 0;
  ph->w = s->s_fd_w; /* 1, or the forced direction's cone weight */
  set_energy(s, ph, e);
  return GG_OK;
}

/* ------------------------------------------------------------------------ */
/* Transport of one history                                                  */
/* ------------------------------------------------------------------------ */
static int inside_box(const real p[3], const real lo[3], const real hi[3]) {
  for (int a = 0; a < 3; ++a)
    if (p[a] < lo[a] || p[a] > hi[a]) return 0;
  return 1;
}

static void start_photon(const scene_t *s, photon_t *ph) {
  ph->in_head = 0;
  ph->exclude = -1;
  ph->visited_head = 0;
  ph->head_stage = 0;
  if (inside_box(ph->pos, s->bmin, s->bmax)) {
    ph->in_image = 1;
    ph->t_exit = exit_distance(ph->pos, ph->dir, s->bmin, s->bmax);
  } else {
    ph->in_image = 0;
    ph->can_enter = 1;
  }
}

/* Interaction at ph->pos in material mat; returns the energy deposited
   locally (the caller scores it where a tally applies). */
static real interact(const scene_t *s, photon_t *ph, int mat, rng_t *g, tally_t *t, photon_t *sec,
                     int *has_sec) {
  int c = s->mat_comp[mat];
  const real *cu = s->cum + (size_t)c * 3 * s->n_e;
  real r = u01(g);
  real fc = interp_row(cu, ph->ei);
  if (r < fc) {
    real ed;
    ph->kind = KIND_COMPTON;
    compton(s, ph, g, t, &ed);
    return ed;
  }
  real fp = interp_row(cu + s->n_e, ph->ei);
  if (r < fp) {
    ph->kind = KIND_PHOTO;
    ph->alive = 0;
    return ph->e;
  }
  real fr = interp_row(cu + 2 * s->n_e, ph->ei);
  if (r < fr) {
    ph->kind = KIND_RAYLEIGH;
    rayleigh(s, c, ph, g, t);
    return R(0);
  }
  ph->kind = KIND_PAIR;
  /* pair: both leptons stopped at creation, positron annihilates at rest */
  real ekin = ph->e - R(2.0 * MC2);
  real d[3];
  iso_dir(g, d);
  if (!has_sec || *has_sec) {
    t->cnt[GG_CNT_STACK_OVERFLOW]++;
  } else {
    *sec = *ph;
    sec->ncompt = 0;
    sec->dir[0] = -d[0];
    sec->dir[1] = -d[1];
    sec->dir[2] = -d[2];
    set_energy(s, sec, R(MC2));
    *has_sec = 1;
  }
  ph->dir[0] = d[0];
  ph->dir[1] = d[1];
  ph->dir[2] = d[2];
  set_energy(s, ph, R(MC2));
  t->cnt[GG_CNT_SECONDARIES] += 2;
  return ekin;
}

/* ---- SPECT heads ------------------------------------------------------- */
#define C30 0.86602540378443864676 /* cos 30 degrees */

static real dot3(const real a[3], const real b[3]) {
  real r = a[0] * b[0];
  r = r + a[1] * b[1];
  r = r + a[2] * b[2];
  return r;
}

/* world -> head-local (a1 along e1, a2 along e2, w along the outward normal) */
static void to_local(const scene_t *s, int h, const real p[3], const real d[3], real lp[3], real ld[3]) {
  real q[3];
  for (int a = 0; a < 3; ++a) q[a] = p[a] - s->hc[h][a];
  lp[0] = dot3(q, s->he1[h]);
  lp[1] = dot3(q, s->he2[h]);
  lp[2] = dot3(q, s->hu[h]);
  ld[0] = dot3(d, s->he1[h]);
  ld[1] = dot3(d, s->he2[h]);
  ld[2] = dot3(d, s->hu[h]);
}

static void to_world(const scene_t *s, int h, const real lp[3], const real ld[3], real p[3], real d[3]) {
  for (int a = 0; a < 3; ++a) {
    real x = lp[0] * s->he1[h][a];
    x = s->hc[h][a] + x;
    x = x + lp[1] * s->he2[h][a];
    p[a] = x + lp[2] * s->hu[h][a];
    real y = ld[0] * s->he1[h][a];
    y = y + ld[1] * s->he2[h][a];
    d[a] = y + ld[2] * s->hu[h][a];
  }
}

/* Hole containing (a1, a2), if any: centres on two rectangular lattices of
   pitch (px, py), the second offset by half a pitch; a point is in a hole when
   its distance along each face normal (30, 90, 150 degrees) is <= apothem. */
static int find_hole(const scene_t *s, real a1, real a2, real *cx, real *cy) {
  for (int lat = 0; lat < 2; ++lat) {
    real ox = lat ? s->hpx : R(0), oy = lat ? s->hpy : R(0);
    real fx = a1 - ox;
    fx = fx * s->inv_px;
    fx = fx + R(0.5);
    fx = (real)floor((double)fx);
    real fy = a2 - oy;
    fy = fy * s->inv_py;
    fy = fy + R(0.5);
    fy = (real)floor((double)fy);
    real x = fx * s->px;
    x = x + ox;
    real y = fy * s->py;
    y = y + oy;
    real qx = a1 - x, qy = a2 - y;
    real t0 = qx * R(C30), t1 = qy * R(0.5);
    real n0 = t1 + t0, n2 = t1 - t0;
    if (fabs((double)qy) <= (double)s->apo && fabs((double)n0) <= (double)s->apo &&
        fabs((double)n2) <= (double)s->apo) {
      *cx = x;
      *cy = y;
      return 1;
    }
  }
  return 0;
}

/* distance to leave the hexagonal prism of a hole from q (relative to its
   centre) along (d1, d2) */
static real hex_exit(const scene_t *s, real qx, real qy, real d1, real d2) {
  real t0 = qx * R(C30), t1 = qy * R(0.5);
  real u0 = d1 * R(C30), u1 = d2 * R(0.5);
  real qn[3] = {t1 + t0, qy, t1 - t0};
  real dn[3] = {u1 + u0, d2, u1 - u0};
  real t = R(INFINITY);
  for (int k = 0; k < 3; ++k) {
    real tk;
    if (dn[k] > R(0)) {
      tk = s->apo - qn[k];
      tk = tk / dn[k];
      if (tk < t) t = tk;
    } else if (dn[k] < R(0)) {
      tk = -s->apo - qn[k];
      tk = tk / dn[k];
      if (tk < t) t = tk;
    }
  }
  return t < R(0) ? R(0) : t;
}

static void move(real p[3], const real d[3], real t) {
  for (int a = 0; a < 3; ++a) p[a] = p[a] + t * d[a];
}

/* leave the head box (to the world) or move to the next head region */
static void head_cross(const scene_t *s, photon_t *ph, int leave) {
  if (leave) {
    real p[3], d[3];
    to_world(s, ph->head, ph->pos, ph->dir, p, d);
    for (int a = 0; a < 3; ++a) {
      ph->pos[a] = p[a];
      ph->dir[a] = d[a];
    }
    ph->in_head = 0;
    ph->exclude = 1 + ph->head;
  } else {
    ph->hreg += ph->dir[2] > R(0) ? 1 : -1;
    ph->left_hole = 0;
  }
}

/* One step inside a head (photon in head-local coordinates). */
static void head_step(const scene_t *s, photon_t *ph, rng_t *g, tally_t *t, event_t *ev) {
  t->cnt[GG_CNT_HEAD_STEPS]++;
  real *l = ph->pos, *d = ph->dir;
  real lo[3] = {-s->half_w, -s->half_w, R(0)};
  real hi[3] = {s->half_w, s->half_w, s->zend};
  int face;
  real tbox = exit_distance_face(l, d, lo, hi, &face);
  real treg = R(INFINITY);
  if (d[2] > R(0)) {
    treg = s->zb[ph->hreg + 1] - l[2];
    treg = treg / d[2];
  } else if (d[2] < R(0)) {
    treg = s->zb[ph->hreg] - l[2];
    treg = treg / d[2];
  }
  if (treg < R(0)) treg = R(0);
  int leave = tbox <= treg;
  real tlim = leave ? tbox : treg;
  /* shielded sides: a photon that reaches a side face stops there */
  const int absorb = leave && s->side_black && face != 2;
  if (ph->hreg == 0 && !ph->left_hole) {
    real cx, cy;
    if (find_hole(s, l[0], l[1], &cx, &cy)) {
      real th = hex_exit(s, l[0] - cx, l[1] - cy, d[0], d[1]);
      ph->left_hole = 1;
      if (th < tlim) {
        move(l, d, th);
        return;
      }
      move(l, d, tlim);
      if (absorb) ph->alive = 0;
      else head_cross(s, ph, leave);
      return;
    }
  }
  ph->left_hole = 0;
  if (s->hmat[ph->hreg] < 0) { /* vacuum slab (the gap) */
    move(l, d, tlim);
    if (absorb) ph->alive = 0;
    else head_cross(s, ph, leave);
    return;
  }
  int mat = s->hmat[ph->hreg];
  real mu = interp_row(s->sig + (size_t)s->mat_comp[mat] * s->n_e, ph->ei);
  mu = s->mat_rho[mat] * mu;
  real u = u01_open0(g);
  real sd = -ggo_log(u);
  sd = sd / mu;
  if (sd >= tlim) {
    move(l, d, tlim);
    if (absorb) ph->alive = 0;
    else head_cross(s, ph, leave);
    return;
  }
  move(l, d, sd);
  if (ph->hreg == 0) {
    real cx, cy;
    if (find_hole(s, l[0], l[1], &cx, &cy)) return; /* null collision inside a hole */
  }
  real ed = interact(s, ph, mat, g, t, NULL, NULL);
  if (ph->hreg == s->hreg_cr && ed > R(0)) {
    int h = ph->head;
    ev->esum[h] = ev->esum[h] + ed;
    if (s->centroid) { /* EnergyWeightedCentroidPosition */
      ev->wpos[h][0] = ev->wpos[h][0] + ed * l[0];
      ev->wpos[h][1] = ev->wpos[h][1] + ed * l[1];
      ev->w[h] = ph->w; /* the last hit's weight */
    } else if (ed > ev->emax[h]) {
      ev->emax[h] = ed;
      ev->wpos[h][0] = l[0];
      ev->wpos[h][1] = l[1];
      ev->w[h] = ph->w; /* the winner hit's weight */
    }
  }
}

/* ---- ARF detector ------------------------------------------------------- */
/* The network of the ARF stage (3 -> 128 -> 128 -> 128 -> nc, softmax) in
   FP64, with W2, W3, W4 and the hidden activations rounded to bfloat16 where
   the GPU stores them; window weights p_k / (rr p_0 + sum_k>0 p_k) go to
   fixed-point projection tallies like the GPU's (2^-32 units). */
typedef struct arf_s {
  int nc;
  double w1[128 * 3], b1[128], w2[128 * 128], b2[128], w3[128 * 128], b3[128], w4[16 * 128], b4[16];
  float mean[3], inv[3];
  double rr;
  real emin, emax, ctmax, edet, dc;
  uint64_t *proj, *proj2;
} arf_t;

static double bf16r(double x) {
  float f = (float)x;
  uint32_t b;
  memcpy(&b, &f, 4);
  b = (b + 0x7FFFu + ((b >> 16) & 1u)) & 0xFFFF0000u;
  memcpy(&f, &b, 4);
  return (double)f;
}

static void arf_forward(const arf_t *a, const float x[3], double *p) {
  double h1[128], h2[128], h3[128];
  for (int j = 0; j < 128; ++j) {
    double z = a->b1[j] + a->w1[3 * j] * x[0] + a->w1[3 * j + 1] * x[1] + a->w1[3 * j + 2] * x[2];
    h1[j] = bf16r(z > 0 ? z : 0);
  }
  for (int j = 0; j < 128; ++j) {
    double z = a->b2[j];
    for (int i = 0; i < 128; ++i) z += a->w2[128 * j + i] * h1[i];
    h2[j] = bf16r(z > 0 ? z : 0);
  }
  for (int j = 0; j < 128; ++j) {
    double z = a->b3[j];
    for (int i = 0; i < 128; ++i) z += a->w3[128 * j + i] * h2[i];
    h3[j] = bf16r(z > 0 ? z : 0);
  }
  double mx = -INFINITY, sum = 0;
  for (int c = 0; c < a->nc; ++c) {
    double z = a->b4[c];
    for (int i = 0; i < 128; ++i) z += a->w4[128 * c + i] * h3[i];
    p[c] = z;
    if (z > mx) mx = z;
  }
  for (int c = 0; c < a->nc; ++c) {
    p[c] = exp(p[c] - mx);
    sum += p[c];
  }
  for (int c = 0; c < a->nc; ++c) p[c] /= sum;
}

/* A photon entering a head from the phantom side: plain tracking (returns),
   dropped, or scored by the network (photon ends). */
static void arf_at_head(const scene_t *s, photon_t *ph, tally_t *t) {
  const arf_t *a = s->arf;
  if (ph->visited_head) {
    t->cnt[GG_CNT_ARF_FALLBACK]++;
    return;
  }
  real e = ph->e, lz = ph->pos[2], dz = ph->dir[2];
  if (e < a->edet) {
    ph->alive = 0;
    ph->in_head = 0;
    return;
  }
  if (!(lz < (real)1e-3 && dz > R(0) && e >= a->emin && e <= a->emax && dz >= a->ctmax)) {
    t->cnt[GG_CNT_ARF_FALLBACK]++;
    return;
  }
  t->cnt[GG_CNT_ARF_PHOTONS]++;
  float th = acosf((float)dz) * 57.295779513082320876f;
  float phi = atan2f((float)ph->dir[1], (float)ph->dir[0]) * 57.295779513082320876f;
  float x[3] = {(th - a->mean[0]) * a->inv[0], (phi - a->mean[1]) * a->inv[1], ((float)e - a->mean[2]) * a->inv[2]};
  real tt = a->dc / dz;
  real u = ph->pos[0] + tt * ph->dir[0];
  real v = ph->pos[1] + tt * ph->dir[1];
  real fx = u + s->pix_half[0];
  fx = fx * s->inv_psp[0];
  real fy = v + s->pix_half[1];
  fy = fy * s->inv_psp[1];
  ph->alive = 0;
  ph->in_head = 0;
  if (!(fx >= R(0) && fx < (real)s->pnx && fy >= R(0) && fy < (real)s->pny)) return;
  int i = (int)fx, j = (int)fy;
  double p[16];
  arf_forward(a, x, p);
  double norm = a->rr * p[0];
  for (int c = 1; c < a->nc; ++c) norm += p[c];
  size_t plane = (size_t)s->pny * s->pnx;
  for (int c = 1; c < a->nc; ++c) {
    double w = norm > 0 ? p[c] / norm : 0.0;
    if (s->ff) w = w * (double)ph->w; /* free flight: the photon got here with probability w */
    uint64_t q = (uint64_t)llrint(w * 4294967296.0);
    if (!q) continue;
    size_t idx = ((((size_t)ph->head * s->n_runs + s->run) * s->n_win + (c - 1)) * plane) + (size_t)j * s->pnx + i;
    unsigned __int128 sq = (unsigned __int128)q * q;
    __atomic_fetch_add(&a->proj[idx], q, __ATOMIC_RELAXED);
    __atomic_fetch_add(&a->proj2[2 * idx], (uint64_t)sq & 0xffffffffu, __ATOMIC_RELAXED);
    __atomic_fetch_add(&a->proj2[2 * idx + 1], (uint64_t)(sq >> 32), __ATOMIC_RELAXED);
  }
}

/* World step with the image box and the head boxes as possible targets. */
static void ss_split(const scene_t *s, const photon_t *pre, photon_t *ph, int mat, const rng_t *g, tally_t *t);

static void spect_world_step(const scene_t *s, photon_t *ph, rng_t *g, tally_t *t, photon_t *sec,
                             int *has_sec) {
  t->cnt[GG_CNT_WORLD_STEPS]++;
  real tb = ph->exclude != 0 ? entry_distance(ph->pos, ph->dir, s->bmin, s->bmax) : R(INFINITY);
  int box = 0, bface = 2;
  real hlo[3] = {-s->half_w, -s->half_w, R(0)};
  real hhi[3] = {s->half_w, s->half_w, s->zend};
  for (int h = 0; h < s->n_heads; ++h) {
    if (ph->exclude == 1 + h) continue;
    real lp[3], ld[3];
    to_local(s, h, ph->pos, ph->dir, lp, ld);
    int f;
    real th = entry_distance_face(lp, ld, hlo, hhi, &f);
    if (th < tb) {
      tb = th;
      box = 1 + h;
      bface = f;
    }
  }
  real wlo[3] = {-s->whalf[0], -s->whalf[1], -s->whalf[2]};
  real tout = exit_distance(ph->pos, ph->dir, wlo, s->whalf);
  int wm = s->world_mat;
  real mu = interp_row(s->sig + (size_t)s->mat_comp[wm] * s->n_e, ph->ei);
  mu = s->mat_rho[wm] * mu;
  real u = u01_open0(g);
  real sd = -ggo_log(u);
  sd = sd / mu;
  if (sd < tb && sd < tout) {
    move(ph->pos, ph->dir, sd);
    const photon_t pre = *ph;
    interact(s, ph, wm, g, t, sec, has_sec);
    ph->exclude = -1;
    if (s->ff == 2) ss_split(s, &pre, ph, wm, g, t);
  } else if (tb <= tout) {
    move(ph->pos, ph->dir, tb);
    if (box == 0) {
      ph->in_image = 1;
      ph->t_exit = exit_distance(ph->pos, ph->dir, s->bmin, s->bmax);
      ph->head_stage = 0;
    } else if (s->side_black && bface != 2) {
      ph->alive = 0; /* stopped by the head's side shielding */
      t->cnt[GG_CNT_ESCAPED]++;
    } else {
      int h = box - 1;
      real lp[3], ld[3];
      to_local(s, h, ph->pos, ph->dir, lp, ld);
      for (int a = 0; a < 3; ++a) {
        ph->pos[a] = lp[a];
        ph->dir[a] = ld[a];
      }
      ph->in_head = 1;
      ph->head = h;
      ph->hreg = head_region(s, lp[2]);
      ph->left_hole = 0;
      /* (scatter splitting: the analog photon dies at the head, only its copies are scored) */
      if (s->arf && !ph->head_stage && s->ff != 2) arf_at_head(s, ph, t);
      if (ph->alive) {
        ph->visited_head = 1;
        ph->head_stage = 1;
      }
    }
  } else {
    ph->alive = 0;
    t->cnt[GG_CNT_ESCAPED]++;
  }
}

/* Singles of one event: energy windows and projection pixel per head. */
/* two standard normal deviates (Box & Muller 1958): sqrt(-2 ln u1) (cos, sin)(2 pi u2) */
static void normal_pair(rng_t *g, real *z0, real *z1) {
  const real u1 = u01_open0(g);
  const real u2 = u01(g);
  real r = ggo_log(u1);
  r = R(-2) * r;
  r = ggo_sqrt(r);
  real sn, cs;
  ggo_sincos_turn(u2, &sn, &cs);
  *z0 = r * cs;
  *z1 = r * sn;
}

#define FWHM_TO_SIGMA 0.42466090014400953

/* energy blurring of a single (GateDigitizerBlurringActor.cpp:74-97) */
static real blur_energy(const scene_t *s, real e, rng_t *g) {
  real sigma;
  if (s->eblur == 1) {
    sigma = s->eb_sigma;
  } else {
    real v;
    if (s->eblur == 2) {
      v = ggo_sqrt(s->eb_ref);
      const real q = ggo_sqrt(e);
      v = v / q;
      v = s->eb_res * v;
    } else {
      v = e - s->eb_ref;
      v = s->eb_slope * v;
      v = v + s->eb_res;
    }
    sigma = v * e;
    sigma = sigma * (real)FWHM_TO_SIGMA;
  }
  real z0, z1;
  normal_pair(g, &z0, &z1);
  const real d = sigma * z0;
  return e + d;
}

/* erf by Abramowitz & Stegun 7.1.26, odd extension */
static real erf_as(real x) {
  const real ax = x < R(0) ? -x : x;
  real t = R(0.3275911) * ax;
  t = R(1) + t;
  t = R(1) / t;
  real p = R(1.061405429) * t;
  p = p + R(-1.453152027);
  p = p * t;
  p = p + R(1.421413741);
  p = p * t;
  p = p + R(-0.284496736);
  p = p * t;
  p = p + R(0.254829592);
  p = p * t;
  real x2 = ax * ax;
  x2 = -x2;
  real y = p * ggo_exp(x2);
  y = R(1) - y;
  return x < R(0) ? -y : y;
}

/* redraw sigma of a truncated blur (GateDigitizerSpatialBlurringActor.cpp:158-206) */
static real trunc_sigma(real mu, real sigma, real lo, real hi) {
  const real inv_sqrt_2pi = R(0.39894228040143267794);
  const real inv_sqrt2 = R(0.70710678118654752440);
  real a = lo - mu;
  a = a / sigma;
  real b = hi - mu;
  b = b / sigma;
  real pa = R(-0.5) * a;
  pa = pa * a;
  pa = ggo_exp(pa) * inv_sqrt_2pi;
  real pb = R(-0.5) * b;
  pb = pb * b;
  pb = ggo_exp(pb) * inv_sqrt_2pi;
  real fa = erf_as(a * inv_sqrt2);
  fa = R(1) + fa;
  fa = R(0.5) * fa;
  real fb = erf_as(b * inv_sqrt2);
  fb = R(1) + fb;
  fb = R(0.5) * fb;
  const real z = fb - fa;
  real shift = pa - pb;
  shift = shift / z;
  real c = a * pa;
  c = c - b * pb;
  c = c / z;
  real var = R(1) - c;
  var = var - shift * shift;
  real s1 = sigma * ggo_sqrt(var);
  real delta = mu - lo;
  const real dh = hi - mu;
  delta = dh < delta ? dh : delta;
  delta = delta > R(0) ? delta : R(0);
  real dn = delta / s1;
  dn = dn > R(0.95) ? dn : R(0.95);
  if (dn < R(4)) {
    real corr = R(-0.86538264) * dn;
    corr = R(3.61070188) * ggo_exp(corr);
    s1 = s1 * corr;
  }
  return s1;
}

static real trunc_redraw(real mu, real p, real sigma, real lo, real hi, rng_t *g) {
  if (!(p > hi || p < lo)) return p;
  const real sg = trunc_sigma(mu, sigma, lo, hi);
  for (int k = 0; k < LOOP_CAP; ++k) {
    real z0, z1;
    normal_pair(g, &z0, &z1);
    p = sg * z0;
    p = mu + p;
    if (!(p > hi || p < lo)) return p;
  }
  return p < lo ? lo : hi;
}

/* spatial blurring of the crystal position (GateDigitizerSpatialBlurringActor.cpp:85-156) */
static void blur_position(const scene_t *s, real *a1, real *a2, rng_t *g) {
  real z0, z1;
  normal_pair(g, &z0, &z1);
  real p0 = s->sb_sigma[0] * z0;
  p0 = *a1 + p0;
  real p1 = s->sb_sigma[1] * z1;
  p1 = *a2 + p1;
  const real hi = s->half_w, lo = -s->half_w;
  if (s->sblur == 2) {
    p0 = trunc_redraw(*a1, p0, s->sb_sigma[0], lo, hi, g);
    p1 = trunc_redraw(*a2, p1, s->sb_sigma[1], lo, hi, g);
  } else if (s->sb_keep) {
    const real tiny = s->half_w * R(1e-6); /* just inside (FP32 keeps it inside) */
    if (p0 < lo) p0 = lo + tiny;
    if (p1 < lo) p1 = lo + tiny;
    if (p0 > hi) p0 = hi - tiny;
    if (p1 > hi) p1 = hi - tiny;
  }
  *a1 = p0;
  *a2 = p1;
}

/* singles list of the following SPECT runs (set_singles; the C ABI's
   gg_spect_record_singles): one gg_single per single at slot
   fetch_add(g_singles_n), kept below g_singles_cap */
static gg_single *g_singles;
static uint64_t g_singles_cap, g_singles_n;

void GGO_PREFIX(set_singles)(gg_single *buf, uint64_t cap) {
  g_singles = buf;
  g_singles_cap = buf ? cap : 0;
  g_singles_n = 0;
}

uint64_t GGO_PREFIX(singles_count)(void) { return g_singles_n; }

/* singles of one event: (blurring: head 0 before head 1, energy before
   position, from the history's stream,) windows and projection pixel */
static void score_singles(const scene_t *s, const event_t *ev, tally_t *t, rng_t *g) {
  for (int h = 0; h < s->n_heads; ++h) {
    real e = ev->esum[h];
    if (!(e > R(0))) continue;
    t->cnt[GG_CNT_SINGLES]++;
    real a1 = ev->wpos[h][0], a2 = ev->wpos[h][1];
    if (s->centroid) {
      a1 = a1 / e;
      a2 = a2 / e;
    }
    if (s->eblur) e = blur_energy(s, e, g);
    if (s->sblur) blur_position(s, &a1, &a2, g);
    if (g_singles) {
      const uint64_t slot = __atomic_fetch_add(&g_singles_n, 1, __ATOMIC_RELAXED);
      if (slot < g_singles_cap) {
        gg_single *r = &g_singles[slot];
        r->event_id = (uint64_t)g->ctr[2] | ((uint64_t)g->ctr[3] << 32);
        r->head = h;
        r->run = s->run;
        r->energy = (double)e;
        r->a1 = (double)a1;
        r->a2 = (double)a2;
        r->weight = s->ff ? (double)ev->w[h] : 1.0;
      }
    }
    real fx = a1 + s->pix_half[0];
    fx = fx * s->inv_psp[0];
    real fy = a2 + s->pix_half[1];
    fy = fy * s->inv_psp[1];
    if (!(fx >= R(0) && fx < (real)s->pnx && fy >= R(0) && fy < (real)s->pny)) continue;
    int i = (int)fx, j = (int)fy;
    /* free flight: the single's weight in 2^-32 units and its exact square */
    uint64_t q = 0, lo = 0, hi = 0;
    if (s->ff) {
      q = to_fixed(ev->w[h]);
      unsigned __int128 sq = (unsigned __int128)q * q;
      lo = (uint64_t)sq & 0xffffffffu;
      hi = (uint64_t)(sq >> 32);
    }
    for (int k = 0; k < s->n_win; ++k) {
      if (e >= s->wlo[k] && e < s->whi[k]) {
        size_t idx = ((((size_t)h * s->n_runs + s->run) * s->n_win + k) * s->pny + j) * s->pnx + i;
        if (!s->ff) {
          __atomic_fetch_add(&s->proj[idx], 1ull, __ATOMIC_RELAXED);
        } else if (q) {
          __atomic_fetch_add(&s->wproj[idx], q, __ATOMIC_RELAXED);
          if (lo) __atomic_fetch_add(&s->wproj2[2 * idx], lo, __ATOMIC_RELAXED);
          if (hi) __atomic_fetch_add(&s->wproj2[2 * idx + 1], hi, __ATOMIC_RELAXED);
        }
      }
    }
  }
}

static uint32_t voxel_of(const scene_t *s, const real p[3]) {
  int ix = (int)((p[0] - s->bmin[0]) * s->inv_sp[0]);
  int iy = (int)((p[1] - s->bmin[1]) * s->inv_sp[1]);
  int iz = (int)((p[2] - s->bmin[2]) * s->inv_sp[2]);
  ix = ix < 0 ? 0 : (ix >= s->nx ? s->nx - 1 : ix);
  iy = iy < 0 ? 0 : (iy >= s->ny ? s->ny - 1 : iy);
  iz = iz < 0 ? 0 : (iz >= s->nz ? s->nz - 1 : iz);
  return (uint32_t)ix + (uint32_t)s->nx * ((uint32_t)iy + (uint32_t)s->ny * (uint32_t)iz);
}

/* first boundary of a voxel walk along one axis: (bmin + k sp - p) / d for the
   next plane k in the direction of travel, and the distance between planes */
static void tle_first(const scene_t *s, int a, int i, real pa, real da, real *tn, real *td, int *st) {
  if (da > R(0)) {
    real b = (real)(i + 1) * s->sp[a];
    b = s->bmin[a] + b;
    b = b - pa;
    *tn = b / da;
    *td = s->sp[a] / da;
    *st = 1;
  } else if (da < R(0)) {
    real b = (real)i * s->sp[a];
    b = s->bmin[a] + b;
    b = b - pa;
    *tn = b / da;
    real q = -s->sp[a];
    *td = q / da;
    *st = -1;
  }
  if (*tn < R(0)) *tn = R(0);
}

/* Voxel walk (Amanatides-Woo) of the straight path [p, p + len d) inside the
   image: visit(ctx, v, m, length) for every voxel crossed, in order (ties:
   x, then y, then z). */
typedef void (*visit_fn)(void *ctx, uint32_t v, int m, real seg);

static void voxel_walk(const scene_t *s, const real p[3], const real d[3], real len, visit_fn visit, void *ctx) {
  const int n0 = s->nx, n1 = s->ny, n2 = s->nz;
  int i0 = (int)((p[0] - s->bmin[0]) * s->inv_sp[0]);
  int i1 = (int)((p[1] - s->bmin[1]) * s->inv_sp[1]);
  int i2 = (int)((p[2] - s->bmin[2]) * s->inv_sp[2]);
  i0 = i0 < 0 ? 0 : (i0 >= n0 ? n0 - 1 : i0);
  i1 = i1 < 0 ? 0 : (i1 >= n1 ? n1 - 1 : i1);
  i2 = i2 < 0 ? 0 : (i2 >= n2 ? n2 - 1 : i2);
  real tn0 = R(INFINITY), tn1 = R(INFINITY), tn2 = R(INFINITY);
  real td0 = R(INFINITY), td1 = R(INFINITY), td2 = R(INFINITY);
  int s0 = 0, s1 = 0, s2 = 0;
  tle_first(s, 0, i0, p[0], d[0], &tn0, &td0, &s0);
  tle_first(s, 1, i1, p[1], d[1], &tn1, &td1, &s1);
  tle_first(s, 2, i2, p[2], d[2], &tn2, &td2, &s2);
  real tc = R(0);
  const int cap = n0 + n1 + n2 + 3;
  for (int k = 0; k < cap; ++k) {
    int a;
    real tb;
    if (tn1 < tn0) {
      if (tn2 < tn1) a = 2, tb = tn2;
      else a = 1, tb = tn1;
    } else {
      if (tn2 < tn0) a = 2, tb = tn2;
      else a = 0, tb = tn0;
    }
    const real te = tb < len ? tb : len;
    const real seg = te - tc;
    if (seg > R(0)) {
      const uint32_t v = (uint32_t)i0 + (uint32_t)n0 * ((uint32_t)i1 + (uint32_t)n1 * (uint32_t)i2);
      visit(ctx, v, (int)s->labels[v], seg);
    }
    tc = te;
    if (!(tc < len)) break;
    if (a == 0) {
      i0 += s0;
      if (i0 < 0 || i0 >= n0) break;
      tn0 = tn0 + td0;
    } else if (a == 1) {
      i1 += s1;
      if (i1 < 0 || i1 >= n1) break;
      tn1 = tn1 + td1;
    } else {
      i2 += s2;
      if (i2 < 0 || i2 >= n2) break;
      tn2 = tn2 + td2;
    }
  }
}

typedef struct {
  const scene_t *s;
  real e;
  eidx_t ei;
  hlist_t *l;
  tally_t *t;
  real tau;
} walk_ctx_t;

static void tle_visit(void *c, uint32_t v, int m, real seg) {
  walk_ctx_t *w = (walk_ctx_t *)c;
  real mu = interp_row(w->s->muen + (size_t)w->s->mat_comp[m] * w->s->n_e, w->ei);
  mu = w->s->mat_rho[m] * mu;
  real ed = w->e * mu;
  ed = ed * seg;
  deposit(w->l, w->t, v, ed);
}

static void depth_visit(void *c, uint32_t v, int m, real seg) {
  (void)v;
  walk_ctx_t *w = (walk_ctx_t *)c;
  real mu = interp_row(w->s->sig + (size_t)w->s->mat_comp[m] * w->s->n_e, w->ei);
  mu = w->s->mat_rho[m] * mu;
  mu = mu * seg;
  w->tau = w->tau + mu;
}

/* Track-length estimator (GateTLEDoseActor::ScoreTLEDepositStep,
   GateTLEDoseActor.cpp:249-299): the straight path [p, p + len d) of a photon
   of energy e scores e * mu_en(E, material) * length in every voxel it
   crosses. */
static void tle_path(const scene_t *s, const real p[3], const real d[3], real len, real e, eidx_t ei,
                     hlist_t *l, tally_t *t) {
  walk_ctx_t c = {s, e, ei, l, t, R(0)};
  voxel_walk(s, p, d, len, tle_visit, &c);
}

/* optical depth of [p, p + len d) inside the image */
static real image_depth(const scene_t *s, const real p[3], const real d[3], real len, eidx_t ei) {
  walk_ctx_t c = {s, R(0), ei, NULL, NULL, R(0)};
  voxel_walk(s, p, d, len, depth_visit, &c);
  return c.tau;
}

/* Free flight outside the heads (GateGammaFreeFlightOptn, heads excluded): no
   interaction; straight to the nearest head entry (the head just left
   excluded) with the weight multiplied by exp(-optical depth); photons at or
   below a cutoff, missing every head, or (angle check of the angular
   acceptance, before the optical depth) entering it with a direction cosine
   to its axis below cos_min (-2: no check), stop. */
static void ff_step(const scene_t *s, photon_t *ph, tally_t *t, real cos_min) {
  t->cnt[GG_CNT_WORLD_STEPS]++;
  if (ph->e <= s->ff_ecut || ph->w <= s->ff_wcut) {
    ph->alive = 0;
    t->cnt[GG_CNT_ESCAPED]++;
    return;
  }
  if (cos_min > R(-1)) {
    /* no head axis within the angle tolerance: the check below fails too */
    int any = 0;
    for (int h = 0; h < s->n_heads; ++h)
      if (ph->exclude != 1 + h && !(dot3(ph->dir, s->hu[h]) < cos_min)) any = 1;
    if (!any) {
      ph->alive = 0;
      t->cnt[GG_CNT_ESCAPED]++;
      return;
    }
  }
  real tb = R(INFINITY);
  int box = 0, bface = 2;
  real cos_box = R(0);
  real hlo[3] = {-s->half_w, -s->half_w, R(0)};
  real hhi[3] = {s->half_w, s->half_w, s->zend};
  for (int h = 0; h < s->n_heads; ++h) {
    if (ph->exclude == 1 + h) continue;
    real lp[3], ld[3];
    to_local(s, h, ph->pos, ph->dir, lp, ld);
    int f;
    real th = entry_distance_face(lp, ld, hlo, hhi, &f);
    if (th < tb) {
      tb = th;
      box = 1 + h;
      cos_box = ld[2];
      bface = f;
    }
  }
  real wlo[3] = {-s->whalf[0], -s->whalf[1], -s->whalf[2]};
  const real tout = exit_distance(ph->pos, ph->dir, wlo, s->whalf);
  /* (a line into a shielded side face cannot be detected) */
  if (!(tb <= tout) || cos_box < cos_min || (s->side_black && bface != 2)) {
    ph->alive = 0;
    t->cnt[GG_CNT_ESCAPED]++;
    return;
  }
  const int wm = s->world_mat;
  real mu_air = interp_row(s->sig + (size_t)s->mat_comp[wm] * s->n_e, ph->ei);
  mu_air = s->mat_rho[wm] * mu_air;
  real l_air = tb;
  real tau = R(0);
  const real t0 = entry_distance(ph->pos, ph->dir, s->bmin, s->bmax);
  if (t0 < tb) {
    real p0[3];
    for (int a = 0; a < 3; ++a) p0[a] = ph->pos[a] + t0 * ph->dir[a];
    real lin = exit_distance(p0, ph->dir, s->bmin, s->bmax);
    const real rest = tb - t0;
    lin = lin < rest ? lin : rest;
    tau = image_depth(s, p0, ph->dir, lin, ph->ei);
    l_air = l_air - lin;
  }
  real ta = mu_air * l_air;
  tau = tau + ta;
  ph->w = ph->w * ggo_exp(-tau);
  if (ph->w <= s->ff_wcut) {
    ph->alive = 0;
    t->cnt[GG_CNT_ESCAPED]++;
    return;
  }
  move(ph->pos, ph->dir, tb);
  const int h = box - 1;
  real lp[3], ld[3];
  to_local(s, h, ph->pos, ph->dir, lp, ld);
  for (int a = 0; a < 3; ++a) {
    ph->pos[a] = lp[a];
    ph->dir[a] = ld[a];
  }
  ph->in_image = 0;
  ph->in_head = 1;
  ph->head = h;
  ph->hreg = head_region(s, lp[2]);
  ph->left_hole = 0;
  /* ARF detectors: a photon that reaches a head from the phantom is scored
     by the network with its weight, or tracked (the library's ARF stage) */
  if (s->arf && !ph->visited_head) arf_at_head(s, ph, t);
  if (ph->alive) ph->visited_head = 1;
}

/* Scatter splitting (GateScatterSplittingFreeFlightOptrActor.cpp:291-360 and
   GateScatterSplittingFreeFlightOptn.cpp:69-149), after an interaction of the
   analog photon outside the heads: each Compton up to max_compton_level and
   each Rayleigh is sampled again n times from the photon's state before it
   (pre); copy c of the history draws from Philox stream 2 + c, weighs
   pre->w / n, flies freely to a head (ff_step), is tracked there and scores
   its own event.  The Compton after the last level kills the analog photon
   (without copies). */
static void ss_split(const scene_t *s, const photon_t *pre, photon_t *ph, int mat, const rng_t *g, tally_t *t) {
  int n = 0;
  if (ph->kind == KIND_COMPTON && s->ss_nc > 0) {
    if (++ph->ncompt > s->ss_max) {
      ph->alive = 0;
      return;
    }
    n = s->ss_nc;
  } else if (ph->kind == KIND_RAYLEIGH) {
    n = s->ss_nr;
  }
  const uint64_t seed = (uint64_t)g->key[0] | ((uint64_t)g->key[1] << 32);
  const uint64_t hid = (uint64_t)g->ctr[2] | ((uint64_t)g->ctr[3] << 32);
  for (int c = 0; c < n; ++c) {
    rng_t gc;
    rng_init(&gc, seed, hid, 2u + t->ss_next++);
    photon_t cp = *pre;
    cp.w = pre->w / (real)n;
    if (ph->kind == KIND_COMPTON) {
      real ed;
      compton(s, &cp, &gc, t, &ed);
    } else {
      rayleigh(s, s->mat_comp[mat], &cp, &gc, t);
    }
    if (!cp.alive) continue;
    cp.exclude = -1;
    ff_step(s, &cp, t, s->ss_cos); /* with the angle check of the angular acceptance */
    event_t ev;
    memset(&ev, 0, sizeof(ev));
    int steps = 0;
    while (cp.alive) {
      if (++steps > STEP_CAP) {
        t->cnt[GG_CNT_LOOP_CAPPED]++;
        cp.alive = 0;
        break;
      }
      if (cp.in_head) head_step(s, &cp, &gc, t, &ev);
      else ff_step(s, &cp, t, R(-2));
    }
    score_singles(s, &ev, t, &gc);
  }
}

/* Voxel of point p in the dose grid; 0 outside (the library's dose_voxel). */
static int dose_voxel(const scene_t *s, const real p[3], uint32_t *v) {
  real f[3];
  for (int a = 0; a < 3; ++a) {
    real d = p[a] - s->dcorner[a];
    f[a] = d * s->dinv_sp[a];
  }
  if (!(f[0] >= R(0)) || !(f[1] >= R(0)) || !(f[2] >= R(0))) return 0;
  if (!(f[0] < (real)s->dnx) || !(f[1] < (real)s->dny) || !(f[2] < (real)s->dnz)) return 0;
  int ix = (int)f[0], iy = (int)f[1], iz = (int)f[2];
  if (ix >= s->dnx || iy >= s->dny || iz >= s->dnz) return 0;
  *v = (uint32_t)ix + (uint32_t)s->dnx * ((uint32_t)iy + (uint32_t)s->dny * (uint32_t)iz);
  return 1;
}

static void transport_photon(const scene_t *s, photon_t *ph, rng_t *g, tally_t *t, hlist_t *l,
                             photon_t *sec, int *has_sec, event_t *ev) {
  int steps = 0;
  while (ph->alive) {
    if (++steps > STEP_CAP) {
      /* termination guard: a photon never needs this many steps */
      t->cnt[GG_CNT_LOOP_CAPPED]++;
      ph->alive = 0;
      break;
    }
    if (s->ff == 1 && !ph->in_head) {
      ff_step(s, ph, t, ph->visited_head ? R(-2) : s->ss_cos);
      continue;
    }
    if (ph->in_image) {
      if (s->tle && ph->e <= s->tle_thr && ph->e <= s->tle_emin) {
        /* a scored photon at or below the kill energy stops in its voxel */
        deposit(l, t, voxel_of(s, ph->pos), ph->e);
        ph->alive = 0;
        break;
      }
      real u = u01_open0(g);
      real sd = -ggo_log(u);
      sd = sd * ph->inv_mumax;
      if (s->tle && ph->e <= s->tle_thr)
        tle_path(s, ph->pos, ph->dir, sd < ph->t_exit ? sd : ph->t_exit, ph->e, ph->ei, l, t);
      if (sd >= ph->t_exit) {
        for (int a = 0; a < 3; ++a) ph->pos[a] = ph->pos[a] + ph->t_exit * ph->dir[a];
        ph->in_image = 0;
        ph->can_enter = 0;
        ph->exclude = 0;
        continue;
      }
      ph->t_exit = ph->t_exit - sd;
      for (int a = 0; a < 3; ++a) ph->pos[a] = ph->pos[a] + sd * ph->dir[a];
      t->cnt[GG_CNT_WOODCOCK_STEPS]++;
      int ix = (int)((ph->pos[0] - s->bmin[0]) * s->inv_sp[0]);
      int iy = (int)((ph->pos[1] - s->bmin[1]) * s->inv_sp[1]);
      int iz = (int)((ph->pos[2] - s->bmin[2]) * s->inv_sp[2]);
      ix = ix < 0 ? 0 : (ix >= s->nx ? s->nx - 1 : ix);
      iy = iy < 0 ? 0 : (iy >= s->ny ? s->ny - 1 : iy);
      iz = iz < 0 ? 0 : (iz >= s->nz ? s->nz - 1 : iz);
      uint32_t v = (uint32_t)ix + (uint32_t)s->nx * ((uint32_t)iy + (uint32_t)s->ny * (uint32_t)iz);
      int m = s->labels[v];
      real mu = interp_row(s->sig + (size_t)s->mat_comp[m] * s->n_e, ph->ei);
      mu = s->mat_rho[m] * mu;
      real u2 = u01(g);
      if (u2 * ph->mumax >= mu) continue;
      t->cnt[GG_CNT_REAL_INTERACTIONS]++;
      const real e_pre = ph->e;
      const photon_t pre = *ph;
      real ed = interact(s, ph, m, g, t, sec, has_sec);
      /* electrons of a track-length-scored photon deposit nothing (GateTLEDoseActor.cpp:236-243) */
      if (s->dgrid) {
        uint32_t dv;
        if (dose_voxel(s, ph->pos, &dv)) {
          deposit(l, t, dv, ed);
          if (s->ddose) {
            real dd = ed * s->drho_min;
            dd = dd / s->mat_rho[m];
            dose_deposit(t->ld, t, dv, dd);
          }
        }
      } else if (!s->spect && !(s->tle && e_pre <= s->tle_thr)) {
        deposit(l, t, v, ed);
      }
      if (ph->alive && ph->in_image) ph->t_exit = exit_distance(ph->pos, ph->dir, s->bmin, s->bmax);
      if (s->ff == 2) ss_split(s, &pre, ph, m, g, t);
    } else if (ph->in_head) {
      head_step(s, ph, g, t, ev);
    } else if (s->spect) {
      spect_world_step(s, ph, g, t, sec, has_sec);
      if (s->ff == 2 && ph->alive && ph->in_head) {
        /* scatter splitting: the heads are kill volumes of the analog photon */
        ph->alive = 0;
        t->cnt[GG_CNT_ESCAPED]++;
      }
    } else {
      t->cnt[GG_CNT_WORLD_STEPS]++;
      real tin = ph->can_enter ? entry_distance(ph->pos, ph->dir, s->bmin, s->bmax) : R(INFINITY);
      real wlo[3] = {-s->whalf[0], -s->whalf[1], -s->whalf[2]};
      real tout = exit_distance(ph->pos, ph->dir, wlo, s->whalf);
      int wm = s->world_mat;
      real mu = interp_row(s->sig + (size_t)s->mat_comp[wm] * s->n_e, ph->ei);
      mu = s->mat_rho[wm] * mu;
      real u = u01_open0(g);
      real sd = -ggo_log(u);
      sd = sd / mu;
      if (sd < tin && sd < tout) {
        for (int a = 0; a < 3; ++a) ph->pos[a] = ph->pos[a] + sd * ph->dir[a];
        interact(s, ph, wm, g, t, sec, has_sec);
        ph->can_enter = 1;
      } else if (tin <= tout) {
        for (int a = 0; a < 3; ++a) ph->pos[a] = ph->pos[a] + tin * ph->dir[a];
        ph->in_image = 1;
        ph->t_exit = exit_distance(ph->pos, ph->dir, s->bmin, s->bmax);
      } else {
        ph->alive = 0;
        t->cnt[GG_CNT_ESCAPED]++;
      }
    }
  }
}

static int run_history(const scene_t *s, uint64_t seed, uint64_t h, tally_t *t) {
  rng_t g;
  rng_init(&g, seed, h, 0u);
  hlist_t l, ld;
  l.n = 0;
  ld.n = 0;
  t->ld = &ld;
  photon_t ph, sec;
  int has_sec = 0;
  event_t ev;
  memset(&ev, 0, sizeof(ev));
  int st = sample_primary(s, &g, &ph, t, h);
  if (st != GG_OK) return st;
  t->cnt[GG_CNT_HISTORIES]++;
  t->ss_next = 0;
  ph.ncompt = 0;
  start_photon(s, &ph);
  for (;;) {
    transport_photon(s, &ph, &g, t, &l, &sec, &has_sec, &ev);
    if (!has_sec) break;
    ph = sec;
    has_sec = 0;
    start_photon(s, &ph);
  }
  if (s->spect) {
    score_singles(s, &ev, t, &g);
  } else {
    hlist_flush(&l, t);
    if (s->dgrid && s->ddose) dose_flush(&ld, t);
  }
  t->ld = NULL;
  return GG_OK;
}

/* ------------------------------------------------------------------------ */
/* Scene set-up and driver                                                   */
/* ------------------------------------------------------------------------ */
static real *conv_f(const float *src, size_t n) {
  real *d = (real *)malloc(n * sizeof(real));
  for (size_t i = 0; i < n; ++i) d[i] = (real)src[i];
  return d;
}

static real *conv_d(const double *src, size_t n) {
  real *d = (real *)malloc((n ? n : 1) * sizeof(real));
  for (size_t i = 0; i < n; ++i) d[i] = (real)src[i];
  return d;
}

static void scene_free(scene_t *s) {
  free(s->sig); free(s->cum); free(s->ray_amax); free(s->ray_x2); free(s->ray_cum); free(s->mat_rho);
  free(s->mat_comp); free(s->maj); free(s->s_spec_e); free(s->s_spec_cdf); free(s->acc_box);
  free(s->cdf_z); free(s->cdf_y); free(s->cdf_x); free(s->muen);
}

static int scene_init(scene_t *s, const gg_tables_desc *tb, const gg_volume_desc *vol,
                      const gg_world_desc *w, const gg_source_desc *src) {
  memset(s, 0, sizeof(*s));
  s->n_e = tb->n_e; s->n_comp = tb->n_comp; s->n_ray = tb->n_ray; s->n_mat = tb->n_mat;
  s->ln_emin = (real)tb->ln_emin; s->inv_dln = (real)tb->inv_dln;
  s->e_min = (real)tb->e_min; s->e_max = (real)tb->e_max;
  s->sig = conv_f(tb->sig, (size_t)tb->n_comp * tb->n_e);
  s->cum = conv_f(tb->cum, (size_t)tb->n_comp * 3 * tb->n_e);
  s->ray_amax = conv_f(tb->ray_amax, (size_t)tb->n_comp * tb->n_e);
  s->ray_x2 = conv_f(tb->ray_x2, (size_t)tb->n_ray);
  s->ray_cum = conv_f(tb->ray_cum, (size_t)tb->n_comp * tb->n_ray);
  s->mat_rho = conv_f(tb->mat_rho, (size_t)tb->n_mat);
  s->mat_comp = (int *)malloc(sizeof(int) * tb->n_mat);
  for (int i = 0; i < tb->n_mat; ++i) s->mat_comp[i] = tb->mat_comp[i];
  s->nx = vol->dims[0]; s->ny = vol->dims[1]; s->nz = vol->dims[2];
  for (int a = 0; a < 3; ++a) {
    s->bmin[a] = (real)vol->corner[a];
    s->bmax[a] = (real)(vol->corner[a] + (double)vol->dims[a] * vol->spacing[a]);
    s->inv_sp[a] = (real)(1.0 / vol->spacing[a]);
    s->sp[a] = (real)vol->spacing[a];
    s->whalf[a] = (real)w->half_size[a];
  }
  s->labels = vol->labels;
  s->maj = conv_f(vol->majorant, (size_t)tb->n_e);
  s->world_mat = w->material;
  s->src = *src;
  for (int a = 0; a < 3; ++a) {
    s->s_t[a] = (real)src->translation[a];
    s->s_half[a] = (real)src->half_size[a];
    s->s_focus[a] = (real)src->focus[a];
  }
  for (int i = 0; i < 9; ++i) s->s_rot[i] = (real)src->rotation[i];
  s->s_radius = (real)src->radius;
  s->s_cos_tmin = (real)cos(src->theta[0]);
  s->s_cos_tmax = (real)cos(src->theta[1]);
  s->s_phi0_turn = (real)(src->phi[0] / (2.0 * M_PI));
  s->s_dphi_turn = (real)((src->phi[1] - src->phi[0]) / (2.0 * M_PI));
  s->s_fd_cmin = (real)src->fd_cos_min;
  s->s_fd_cmax = (real)src->fd_cos_max;
  s->s_fd_w = src->dir_type == GG_DIR_FORCED ? (real)((src->fd_cos_min - src->fd_cos_max) / 2.0) : R(1);
  double mn = sqrt(src->momentum[0] * src->momentum[0] + src->momentum[1] * src->momentum[1] +
                   src->momentum[2] * src->momentum[2]);
  for (int a = 0; a < 3; ++a) s->s_mom[a] = (real)(mn > 0 ? src->momentum[a] / mn : 0.0);
  s->s_mono = (real)src->mono;
  s->s_elo = (real)src->e_lo;
  s->s_ehi = (real)src->e_hi;
  int ns = src->n_spec;
  s->s_spec_e = conv_d(src->spec_e, (size_t)(src->ene_type == GG_ENE_HISTOGRAM ? ns + 1 : ns));
  s->s_spec_cdf = conv_d(src->spec_cdf, (size_t)ns);
  s->acc_box = conv_d(src->accept_boxes, (size_t)6 * src->n_accept);
  if (src->pos_type == GG_POS_VOXELS) {
    s->vnx = src->vox_dims[0];
    s->vny = src->vox_dims[1];
    s->vnz = src->vox_dims[2];
    for (int a = 0; a < 3; ++a) {
      s->v_org[a] = (real)(src->vox_corner[a] + 0.5 * src->vox_spacing[a]);
      s->v_sp[a] = (real)src->vox_spacing[a];
    }
    s->cdf_z = conv_f(src->cdf_z, (size_t)s->vnz);
    s->cdf_y = conv_f(src->cdf_y, (size_t)s->vnz * s->vny);
    s->cdf_x = conv_f(src->cdf_x, (size_t)s->vnz * s->vny * s->vnx);
  }
  return GG_OK;
}

/* n blurred singles of one event (energy e, crystal point a1, a2) on a crystal
   of half width half_w, sample i on the stream of history i (tests) */
void GGO_PREFIX(sample_blur)(const gg_blur_desc *b, double half_w, double e, double a1, double a2, uint64_t n,
                             uint64_t seed, double *out_e, double *out_a1, double *out_a2) {
  scene_t s;
  memset(&s, 0, sizeof(s));
  s.half_w = (real)half_w;
  s.eblur = b->energy_method;
  s.eb_sigma = (real)b->energy_sigma;
  s.eb_res = (real)b->energy_resolution;
  s.eb_ref = (real)b->energy_reference;
  s.eb_slope = (real)b->energy_slope;
  s.sblur = b->spatial ? (b->truncated ? 2 : 1) : 0;
  s.sb_keep = b->keep_in_solid_limits;
  s.sb_sigma[0] = (real)b->spatial_sigma[0];
  s.sb_sigma[1] = (real)b->spatial_sigma[1];
  for (uint64_t i = 0; i < n; ++i) {
    rng_t g;
    rng_init(&g, seed, i, 0u);
    real ee = (real)e, p = (real)a1, q = (real)a2;
    if (s.eblur) ee = blur_energy(&s, ee, &g);
    if (s.sblur) blur_position(&s, &p, &q, &g);
    out_e[i] = (double)ee;
    out_a1[i] = (double)p;
    out_a2[i] = (double)q;
  }
}

double GGO_PREFIX(erf)(double x) { return (double)erf_as((real)x); }

/* digitizer blurring of the following SPECT runs (set_blur) */
static gg_blur_desc g_blur;

void GGO_PREFIX(set_blur)(const gg_blur_desc *b) {
  if (b) g_blur = *b;
  else memset(&g_blur, 0, sizeof(g_blur));
}

static void spect_init(scene_t *s, const gg_spect_desc *sp) {
  s->spect = 1;
  s->centroid = sp->adder_policy == GG_ADDER_CENTROID;
  s->eblur = g_blur.energy_method;
  s->eb_sigma = (real)g_blur.energy_sigma;
  s->eb_res = (real)g_blur.energy_resolution;
  s->eb_ref = (real)g_blur.energy_reference;
  s->eb_slope = (real)g_blur.energy_slope;
  s->sblur = g_blur.spatial ? (g_blur.truncated ? 2 : 1) : 0;
  s->sb_keep = g_blur.keep_in_solid_limits;
  s->sb_sigma[0] = (real)g_blur.spatial_sigma[0];
  s->sb_sigma[1] = (real)g_blur.spatial_sigma[1];
  s->n_heads = sp->n_heads;
  s->n_runs = sp->n_runs;
  s->n_win = sp->n_windows;
  s->pnx = sp->size[0];
  s->pny = sp->size[1];
  s->half_w = (real)sp->half_width;
  {
    /* slab boundaries: running sums in double, each rounded once */
    double z = 0.0;
    int k = 0;
    s->zb[0] = R(0);
#define GGO_SLAB(t, m) (z = z + (t), s->hmat[k] = (m), s->zb[++k] = (real)z)
    GGO_SLAB(sp->collimator_thickness, sp->collimator_material);
    GGO_SLAB(sp->gap, -1);
    if (sp->n_cover > 0) GGO_SLAB(sp->cover_thickness, sp->cover_material);
    s->hreg_cr = k;
    GGO_SLAB(sp->crystal_thickness, sp->crystal_material);
    for (int b = 0; b < sp->n_back; ++b) GGO_SLAB(sp->back_thickness[b], sp->back_material[b]);
#undef GGO_SLAB
    s->n_hreg = k;
    s->zend = s->zb[k];
    for (int j = k; j < 8; ++j) {
      s->hmat[j] = -1;
      s->zb[j + 1] = s->zend;
    }
    s->side_black = sp->shielded_sides ? 1 : 0;
  }
  s->apo = (real)sp->hole_apothem;
  s->px = (real)sp->pitch_x;
  s->py = (real)sp->pitch_y;
  s->hpx = (real)(0.5 * sp->pitch_x);
  s->hpy = (real)(0.5 * sp->pitch_y);
  s->inv_px = (real)(1.0 / sp->pitch_x);
  s->inv_py = (real)(1.0 / sp->pitch_y);
  s->mat_coll = sp->collimator_material;
  s->mat_cr = sp->crystal_material;
  for (int k = 0; k < sp->n_windows; ++k) {
    s->wlo[k] = (real)sp->window_lo[k];
    s->whi[k] = (real)sp->window_hi[k];
  }
  for (int a = 0; a < 2; ++a) {
    s->pix_half[a] = (real)(0.5 * sp->size[a] * sp->spacing[a]);
    s->inv_psp[a] = (real)(1.0 / sp->spacing[a]);
  }
}

static void spect_set_heads(scene_t *s, int run, const double *frames) {
  s->run = run;
  for (int h = 0; h < s->n_heads; ++h) {
    for (int a = 0; a < 3; ++a) {
      s->hc[h][a] = (real)frames[12 * h + a];
      s->hu[h][a] = (real)frames[12 * h + 3 + a];
      s->he1[h][a] = (real)frames[12 * h + 6 + a];
      s->he2[h][a] = (real)frames[12 * h + 9 + a];
    }
  }
}

typedef struct {
  const scene_t *s;
  uint64_t seed, h0, h1;
  tally_t t;
  int status;
} worker_t;

static void *worker_main(void *arg) {
  worker_t *w = (worker_t *)arg;
  for (uint64_t h = w->h0; h < w->h1; ++h) {
    int st = run_history(w->s, w->seed, h, &w->t);
    if (st != GG_OK) {
      w->status = st;
      break;
    }
  }
  return NULL;
}

/* Runs histories [first, first + n) in batches of `batch`, adding the fixed
   point batch sums into the float64 images edep / edep2 (either may be
   NULL for the squared image), and adding to counters[GG_N_COUNTERS]. */
static int run_dose_impl(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                         const gg_source_desc *src, const gg_tle_desc *tle, const gg_dose_grid_desc *grid,
                         uint64_t seed, uint64_t first, uint64_t n, uint64_t batch, int n_threads, double *edep,
                         double *edep2, double *dose, double *dose2, uint64_t *counters) {
  scene_t s;
  scene_init(&s, tb, vol, w, src);
  double dscale = 1.0;
  if (grid && grid->dims[0] > 0) {
    s.dgrid = 1;
    s.dnx = grid->dims[0];
    s.dny = grid->dims[1];
    s.dnz = grid->dims[2];
    for (int a = 0; a < 3; ++a) {
      s.dcorner[a] = (real)grid->corner[a];
      s.dinv_sp[a] = (real)(1.0 / grid->spacing[a]);
    }
    s.ddose = grid->score_dose != 0 && dose != NULL;
    float rmin = tb->mat_rho[0];
    for (int m = 1; m < tb->n_mat; ++m)
      if (tb->mat_rho[m] < rmin) rmin = tb->mat_rho[m];
    s.drho_min = (real)rmin;
    dscale = 1.0 / (double)rmin;
  }
  if (tle && tle->enabled) {
    s.tle = 1;
    s.tle_thr = (real)tle->threshold_energy;
    s.tle_emin = (real)tle->energy_min;
    s.muen = conv_f(tle->muen, (size_t)tb->n_comp * tb->n_e);
  }
  size_t nv = s.dgrid ? (size_t)s.dnx * s.dny * s.dnz : (size_t)s.nx * s.ny * s.nz;
  uint64_t *acc_e = (uint64_t *)calloc(nv, sizeof(uint64_t));
  uint64_t *acc_e2 = edep2 ? (uint64_t *)calloc(2 * nv, sizeof(uint64_t)) : NULL;
  uint64_t *acc_d = s.ddose ? (uint64_t *)calloc(nv, sizeof(uint64_t)) : NULL;
  uint64_t *acc_d2 = s.ddose && dose2 ? (uint64_t *)calloc(2 * nv, sizeof(uint64_t)) : NULL;
  if (n_threads < 1) n_threads = 1;
  if (batch == 0) batch = n ? n : 1;
  {
    /* the library's cap on histories per batch (gg_api.cu run_impl): the
       fixed-point tallies cannot wrap, n <= 2^32 / E_max^2 and 2^32 / E_max */
    double em = src->mono;
    if (src->ene_type == GG_ENE_RANGE) em = src->e_hi;
    else if (src->ene_type == GG_ENE_LINES || src->ene_type == GG_ENE_HISTOGRAM) {
      const int ne = src->ene_type == GG_ENE_HISTOGRAM ? src->n_spec + 1 : src->n_spec;
      em = src->spec_e[0];
      for (int i = 1; i < ne; ++i)
        if (src->spec_e[i] > em) em = src->spec_e[i];
    }
    em = (em > 1e-6 ? em : 1e-6) * 1.001;
    double lim = 4294967296.0 / (em * em);
    if (4294967296.0 / em < lim) lim = 4294967296.0 / em;
    if ((double)batch > lim) batch = lim >= 1.0 ? (uint64_t)lim : 1;
  }
  worker_t *ws = (worker_t *)calloc((size_t)n_threads, sizeof(worker_t));
  pthread_t *th = (pthread_t *)calloc((size_t)n_threads, sizeof(pthread_t));
  int status = GG_OK;
  for (uint64_t b0 = first; b0 < first + n && status == GG_OK; b0 += batch) {
    uint64_t b1 = b0 + batch < first + n ? b0 + batch : first + n;
    uint64_t per = (b1 - b0 + (uint64_t)n_threads - 1) / (uint64_t)n_threads;
    for (int i = 0; i < n_threads; ++i) {
      ws[i].s = &s;
      ws[i].seed = seed;
      ws[i].h0 = b0 + per * (uint64_t)i < b1 ? b0 + per * (uint64_t)i : b1;
      ws[i].h1 = ws[i].h0 + per < b1 ? ws[i].h0 + per : b1;
      ws[i].t.acc_e = acc_e;
      ws[i].t.acc_e2 = acc_e2;
      ws[i].t.acc_d = acc_d;
      ws[i].t.acc_d2 = acc_d2;
      ws[i].status = GG_OK;
      if (n_threads > 1) pthread_create(&th[i], NULL, worker_main, &ws[i]);
      else worker_main(&ws[i]);
    }
    if (n_threads > 1)
      for (int i = 0; i < n_threads; ++i) pthread_join(th[i], NULL);
    for (int i = 0; i < n_threads; ++i)
      if (ws[i].status != GG_OK) status = ws[i].status;
    for (size_t v = 0; v < nv; ++v) {
      if (acc_e[v]) {
        edep[v] += (double)acc_e[v] * 2.3283064365386963e-10;
        acc_e[v] = 0;
      }
      if (acc_e2 && (acc_e2[2 * v] | acc_e2[2 * v + 1])) {
        double lo = (double)acc_e2[2 * v];
        lo = lo * 5.421010862427522e-20; /* 2^-64 */
        double hi = (double)acc_e2[2 * v + 1];
        hi = hi * 2.3283064365386963e-10; /* 2^-32 */
        edep2[v] += hi + lo;
        acc_e2[2 * v] = acc_e2[2 * v + 1] = 0;
      }
      /* dose tally: the library's k_flush with scale 1 / rho_min */
      if (acc_d && acc_d[v]) {
        double x = (double)acc_d[v] * 2.3283064365386963e-10;
        x = x * dscale;
        dose[v] += x;
        acc_d[v] = 0;
      }
      if (acc_d2 && (acc_d2[2 * v] | acc_d2[2 * v + 1])) {
        double lo = (double)acc_d2[2 * v];
        lo = lo * 5.421010862427522e-20;
        double hi = (double)acc_d2[2 * v + 1];
        hi = hi * 2.3283064365386963e-10;
        double x = hi + lo;
        x = x * (dscale * dscale);
        dose2[v] += x;
        acc_d2[2 * v] = acc_d2[2 * v + 1] = 0;
      }
    }
  }
  for (int i = 0; i < n_threads; ++i)
    for (int c = 0; c < GG_N_COUNTERS; ++c) counters[c] += ws[i].t.cnt[c];
  free(ws);
  free(th);
  free(acc_e);
  free(acc_e2);
  free(acc_d);
  free(acc_d2);
  scene_free(&s);
  return status;
}

int GGO_PREFIX(run_dose)(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                         const gg_source_desc *src, uint64_t seed, uint64_t first, uint64_t n,
                         uint64_t batch, int n_threads, double *edep, double *edep2,
                         uint64_t *counters) {
  return run_dose_impl(tb, vol, w, src, NULL, NULL, seed, first, n, batch, n_threads, edep, edep2, NULL, NULL,
                       counters);
}

/* run_dose with the tally on a grid of its own (gg_set_dose_grid): edep and,
   with grid->score_dose, the dose sum(edep / rho) (either squares may be NULL). */
int GGO_PREFIX(run_dose_grid)(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                              const gg_source_desc *src, const gg_dose_grid_desc *grid, uint64_t seed,
                              uint64_t first, uint64_t n, uint64_t batch, int n_threads, double *edep,
                              double *edep2, double *dose, double *dose2, uint64_t *counters) {
  return run_dose_impl(tb, vol, w, src, NULL, grid, seed, first, n, batch, n_threads, edep, edep2, dose, dose2,
                       counters);
}

/* run_dose with the track-length estimator of gg_set_tle. */
int GGO_PREFIX(run_dose_tle)(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                             const gg_source_desc *src, const gg_tle_desc *tle, uint64_t seed, uint64_t first,
                             uint64_t n, uint64_t batch, int n_threads, double *edep, double *edep2,
                             uint64_t *counters) {
  return run_dose_impl(tb, vol, w, src, tle, NULL, seed, first, n, batch, n_threads, edep, edep2, NULL, NULL,
                       counters);
}

/* SPECT projections: for each run r (gantry position, head frames
   frames[r][n_heads][12]) simulates histories [first + r * n_per_run,
   first + (r + 1) * n_per_run) and adds singles counts into proj
   ([head][run][window][pny][pnx], zeroed by the caller). */
static int run_spect_impl(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                          const gg_source_desc *src, const gg_spect_desc *sp, const double *frames,
                          uint64_t seed, uint64_t first, uint64_t n_per_run, int n_threads, uint64_t *proj,
                          uint64_t *counters, const arf_t *arf, const gg_ff_desc *ff, uint64_t *wproj,
                          uint64_t *wproj2) {
  scene_t s;
  scene_init(&s, tb, vol, w, src);
  spect_init(&s, sp);
  s.proj = proj;
  s.arf = arf;
  if (ff && ff->enabled) {
    s.ff = ff->enabled == 2 ? 2 : 1;
    s.ff_wcut = (real)ff->weight_cutoff;
    s.ff_ecut = (real)ff->energy_cutoff;
    if (s.ff == 2) {
      s.ss_nc = ff->compton_splitting;
      s.ss_nr = ff->rayleigh_splitting;
      s.ss_max = ff->max_compton_level;
    }
    /* angle check: the copies of scatter splitting, and primary free flights
       from the phantom (not the flights of photons leaving a head) */
    s.ss_cos = (real)(ff->angle_tolerance_max > 0.0 ? cos(ff->angle_tolerance_max) : -2.0);
    s.wproj = wproj;
    s.wproj2 = wproj2;
  }
  if (n_threads < 1) n_threads = 1;
  worker_t *ws = (worker_t *)calloc((size_t)n_threads, sizeof(worker_t));
  pthread_t *th = (pthread_t *)calloc((size_t)n_threads, sizeof(pthread_t));
  int status = GG_OK;
  for (int r = 0; r < sp->n_runs && status == GG_OK; ++r) {
    spect_set_heads(&s, r, frames + (size_t)r * sp->n_heads * 12);
    uint64_t b0 = first + (uint64_t)r * n_per_run, b1 = b0 + n_per_run;
    uint64_t per = (n_per_run + (uint64_t)n_threads - 1) / (uint64_t)n_threads;
    for (int i = 0; i < n_threads; ++i) {
      ws[i].s = &s;
      ws[i].seed = seed;
      ws[i].h0 = b0 + per * (uint64_t)i < b1 ? b0 + per * (uint64_t)i : b1;
      ws[i].h1 = ws[i].h0 + per < b1 ? ws[i].h0 + per : b1;
      ws[i].status = GG_OK;
      if (n_threads > 1) pthread_create(&th[i], NULL, worker_main, &ws[i]);
      else worker_main(&ws[i]);
    }
    if (n_threads > 1)
      for (int i = 0; i < n_threads; ++i) pthread_join(th[i], NULL);
    for (int i = 0; i < n_threads; ++i)
      if (ws[i].status != GG_OK) status = ws[i].status;
  }
  for (int i = 0; i < n_threads; ++i)
    for (int c = 0; c < GG_N_COUNTERS; ++c) counters[c] += ws[i].t.cnt[c];
  free(ws);
  free(th);
  scene_free(&s);
  return status;
}

/* ARF training rows (GateARFTrainingDatasetActor::SteppingAction /
   EndOfEventAction, core/opengate_core/opengate_lib/GateARFTrainingDatasetActor.cpp:76-137):
   sample i of [first, first + n) starts on the collimator front face of head 0
   (head-local frame = world frame), is tracked through the head until it is
   absorbed or leaves the head box, and gives the row (E, theta, phi, w) of
   its direction at the face: theta = acos(dz), phi = atan2(dy, dx) in
   degrees, w = last window containing the event's crystal energy + 1, 0 for
   none; w = 0 rows are kept with probability 1 / russian_roulette.  Rows are
   written in sample order to rows[4 * k]; *n_rows = rows written.  Philox
   stream 1 of history i. */
static int arf_sample(const scene_t *s, const gg_arf_sampling *a, uint64_t seed, uint64_t i, tally_t *t,
                      float row[4]) {
  rng_t g;
  rng_init(&g, seed, i, 1u);
  photon_t ph;
  memset(&ph, 0, sizeof(ph));
  real hx = (real)a->half_extent[0], hy = (real)a->half_extent[1];
  real u = R(2) * u01(&g);
  u = u - R(1);
  ph.pos[0] = u * hx;
  u = R(2) * u01(&g);
  u = u - R(1);
  ph.pos[1] = u * hy;
  ph.pos[2] = R(0);
  real ct, st;
  if (a->theta_uniform) {
    real f = u01(&g) * (real)(acos(a->cos_theta_max) / (2.0 * M_PI));
    ggo_sincos_turn(f, &st, &ct);
  } else {
    real w = R(1) - (real)a->cos_theta_max;
    w = u01(&g) * w;
    ct = R(1) - w;
    real st2 = ct * ct;
    st2 = R(1) - st2;
    st = ggo_sqrt(st2 > R(0) ? st2 : R(0));
  }
  real sp, cp;
  ggo_sincos_turn(u01(&g), &sp, &cp);
  ph.dir[0] = st * cp;
  ph.dir[1] = st * sp;
  ph.dir[2] = ct;
  real de = (real)a->e_max - (real)a->e_min;
  de = de * u01(&g);
  real e = (real)a->e_min + de;
  row[0] = (float)e;
  row[1] = (float)(acos((double)ph.dir[2]) * (180.0 / M_PI));
  row[2] = (float)(atan2((double)ph.dir[1], (double)ph.dir[0]) * (180.0 / M_PI));
  set_energy(s, &ph, e);
  ph.alive = 1;
  ph.in_head = 1;
  ph.head = 0;
  ph.hreg = 0;
  ph.left_hole = 0;
  ph.exclude = -1;
  event_t ev;
  memset(&ev, 0, sizeof(ev));
  int steps = 0;
  while (ph.alive && ph.in_head) {
    if (++steps > STEP_CAP) {
      t->cnt[GG_CNT_LOOP_CAPPED]++;
      break;
    }
    head_step(s, &ph, &g, t, &ev);
  }
  int label = 0;
  real ed = ev.esum[0];
  if (ed > R(0)) {
    t->cnt[GG_CNT_SINGLES]++;
    if (s->eblur) ed = blur_energy(s, ed, &g); /* the window the digitizer chain reports */
    for (int k = 0; k < s->n_win; ++k)
      if (ed >= s->wlo[k] && ed < s->whi[k]) label = k + 1;
  }
  row[3] = (float)label;
  if (label == 0) {
    real r = u01(&g) * (real)a->russian_roulette;
    if (!(r < R(1))) return 0;
  }
  return 1;
}

typedef struct {
  const scene_t *s;
  const gg_arf_sampling *a;
  uint64_t seed, i0, i1, first;
  float *rows;
  uint8_t *keep;
  tally_t t;
} arf_worker_t;

static void *arf_worker(void *arg) {
  arf_worker_t *w = (arf_worker_t *)arg;
  for (uint64_t i = w->i0; i < w->i1; ++i)
    w->keep[i - w->first] = (uint8_t)arf_sample(w->s, w->a, w->seed, i, &w->t, w->rows + 4 * (i - w->first));
  return NULL;
}

int GGO_PREFIX(arf_dataset)(const gg_tables_desc *tb, const gg_spect_desc *sp, const gg_arf_sampling *a,
                            uint64_t seed, uint64_t first, uint64_t n, int n_threads, float *rows,
                            uint64_t *n_rows, uint64_t *counters) {
  /* head-only scene: no image (one air voxel far away), identity head frame */
  static const uint16_t label0 = 0;
  gg_volume_desc vol;
  memset(&vol, 0, sizeof(vol));
  vol.dims[0] = vol.dims[1] = vol.dims[2] = 1;
  vol.spacing[0] = vol.spacing[1] = vol.spacing[2] = 1.0;
  vol.corner[0] = vol.corner[1] = vol.corner[2] = 1.0e6;
  vol.labels = &label0;
  float *maj = (float *)malloc((size_t)tb->n_e * sizeof(float));
  for (int k = 0; k < tb->n_e; ++k) maj[k] = 1.0f; /* the image is never entered */
  vol.majorant = maj;
  gg_world_desc wd;
  memset(&wd, 0, sizeof(wd));
  wd.half_size[0] = wd.half_size[1] = wd.half_size[2] = 2.0e6;
  gg_source_desc src;
  memset(&src, 0, sizeof(src));
  src.ene_type = GG_ENE_MONO;
  src.mono = a->e_max;
  scene_t s;
  scene_init(&s, tb, &vol, &wd, &src);
  gg_spect_desc one = *sp;
  one.n_heads = 1;
  one.n_runs = 1;
  spect_init(&s, &one);
  static const double frame[12] = {0, 0, 0, 0, 0, 1, 1, 0, 0, 0, 1, 0};
  spect_set_heads(&s, 0, frame);
  if (n_threads < 1) n_threads = 1;
  float *all = (float *)malloc((n ? n : 1) * 4 * sizeof(float));
  uint8_t *keep = (uint8_t *)calloc(n ? n : 1, 1);
  arf_worker_t *ws = (arf_worker_t *)calloc((size_t)n_threads, sizeof(arf_worker_t));
  pthread_t *th = (pthread_t *)calloc((size_t)n_threads, sizeof(pthread_t));
  uint64_t per = (n + (uint64_t)n_threads - 1) / (uint64_t)n_threads;
  for (int k = 0; k < n_threads; ++k) {
    ws[k].s = &s;
    ws[k].a = a;
    ws[k].seed = seed;
    ws[k].first = first;
    ws[k].i0 = first + (per * (uint64_t)k < n ? per * (uint64_t)k : n);
    ws[k].i1 = first + (per * (uint64_t)(k + 1) < n ? per * (uint64_t)(k + 1) : n);
    ws[k].rows = all;
    ws[k].keep = keep;
    if (n_threads > 1) pthread_create(&th[k], NULL, arf_worker, &ws[k]);
    else arf_worker(&ws[k]);
  }
  if (n_threads > 1)
    for (int k = 0; k < n_threads; ++k) pthread_join(th[k], NULL);
  uint64_t m = 0;
  for (uint64_t i = 0; i < n; ++i)
    if (keep[i]) {
      memcpy(rows + 4 * m, all + 4 * i, 4 * sizeof(float));
      ++m;
    }
  *n_rows = m;
  for (int k = 0; k < n_threads; ++k)
    for (int c = 0; c < GG_N_COUNTERS; ++c) counters[c] += ws[k].t.cnt[c];
  counters[GG_CNT_HISTORIES] += n;
  free(all);
  free(keep);
  free(ws);
  free(th);
  free(maj);
  scene_free(&s);
  return GG_OK;
}

int GGO_PREFIX(run_spect)(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                          const gg_source_desc *src, const gg_spect_desc *sp, const double *frames,
                          uint64_t seed, uint64_t first, uint64_t n_per_run, int n_threads, uint64_t *proj,
                          uint64_t *counters) {
  return run_spect_impl(tb, vol, w, src, sp, frames, seed, first, n_per_run, n_threads, proj, counters, NULL, NULL,
                        NULL, NULL);
}

/* run_spect with free flight outside the heads: weighted projection
   (2^-32 units) and its history-by-history squares (low 32 bits, rest). */
int GGO_PREFIX(run_spect_ff)(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                             const gg_source_desc *src, const gg_spect_desc *sp, const double *frames,
                             const gg_ff_desc *ff, uint64_t seed, uint64_t first, uint64_t n_per_run, int n_threads,
                             uint64_t *wproj, uint64_t *wproj2, uint64_t *proj, uint64_t *counters) {
  return run_spect_impl(tb, vol, w, src, sp, frames, seed, first, n_per_run, n_threads, proj, counters, NULL, ff,
                        wproj, wproj2);
}

/* SPECT with ARF detectors (the GPU's gg_spect_use_arf): as run_spect, with
   the network `params` (GG_ARF_N_PARAMS floats) of `model` applied where a
   photon reaches a head from the phantom side; window weights go to
   arf_proj / arf_proj2 (fixed point, 2^-32 and 2^-64 / 2^-32 units, zeroed by
   the caller). */
static arf_t *arf_make(const gg_spect_desc *sp, const gg_arf_model *m, const float *params, uint64_t *arf_proj,
                       uint64_t *arf_proj2) {
  arf_t *a = (arf_t *)calloc(1, sizeof(arf_t));
  a->nc = m->n_classes;
  const float *pw = params;
  for (int k = 0; k < 128 * 3; ++k) a->w1[k] = pw[k];
  pw += 128 * 3;
  for (int k = 0; k < 128; ++k) a->b1[k] = pw[k];
  pw += 128;
  for (int k = 0; k < 128 * 128; ++k) a->w2[k] = bf16r(pw[k]);
  pw += 128 * 128;
  for (int k = 0; k < 128; ++k) a->b2[k] = pw[k];
  pw += 128;
  for (int k = 0; k < 128 * 128; ++k) a->w3[k] = bf16r(pw[k]);
  pw += 128 * 128;
  for (int k = 0; k < 128; ++k) a->b3[k] = pw[k];
  pw += 128;
  for (int k = 0; k < 16 * 128; ++k) a->w4[k] = bf16r(pw[k]);
  pw += 16 * 128;
  for (int k = 0; k < 16; ++k) a->b4[k] = pw[k];
  for (int k = 0; k < 3; ++k) {
    a->mean[k] = m->x_mean[k];
    a->inv[k] = 1.0f / m->x_std[k];
  }
  a->rr = m->russian_roulette;
  a->emin = (real)m->e_min;
  a->emax = (real)m->e_max;
  a->ctmax = (real)cos(m->theta_max_deg * (M_PI / 180.0));
  double lo = sp->window_lo[0];
  for (int k = 1; k < sp->n_windows; ++k) lo = sp->window_lo[k] < lo ? sp->window_lo[k] : lo;
  a->edet = (real)lo;
  a->dc = (real)m->distance_to_crystal;
  a->proj = arf_proj;
  a->proj2 = arf_proj2;
  return a;
}

int GGO_PREFIX(run_spect_arf)(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                              const gg_source_desc *src, const gg_spect_desc *sp, const double *frames,
                              uint64_t seed, uint64_t first, uint64_t n_per_run, int n_threads, uint64_t *proj,
                              uint64_t *counters, const gg_arf_model *m, const float *params, uint64_t *arf_proj,
                              uint64_t *arf_proj2) {
  arf_t *a = arf_make(sp, m, params, arf_proj, arf_proj2);
  int st = run_spect_impl(tb, vol, w, src, sp, frames, seed, first, n_per_run, n_threads, proj, counters, a, NULL,
                          NULL, NULL);
  free(a);
  return st;
}

/* ARF detectors with free flight (gg_spect_use_arf + gg_spect_set_free_flight):
   network window weights times the free-flight weight and the weighted singles
   of the photons tracked instead go to the same weighted projection
   (arf_proj, arf_proj2), as in the library. */
int GGO_PREFIX(run_spect_arf_ff)(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                                 const gg_source_desc *src, const gg_spect_desc *sp, const double *frames,
                                 const gg_ff_desc *ff, uint64_t seed, uint64_t first, uint64_t n_per_run,
                                 int n_threads, uint64_t *proj, uint64_t *counters, const gg_arf_model *m,
                                 const float *params, uint64_t *arf_proj, uint64_t *arf_proj2) {
  arf_t *a = arf_make(sp, m, params, arf_proj, arf_proj2);
  int st = run_spect_impl(tb, vol, w, src, sp, frames, seed, first, n_per_run, n_threads, proj, counters, a, ff,
                          arf_proj, arf_proj2);
  free(a);
  return st;
}

/* ---- small exported probes for the unit tests ---- */
void GGO_PREFIX(philox)(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  philox4x32_10(ctr, key, out);
}
double GGO_PREFIX(log)(double x) { return (double)ggo_log((real)x); }
double GGO_PREFIX(exp)(double x) { return (double)ggo_exp((real)x); }
void GGO_PREFIX(sincos_turn)(double f, double *s, double *c) {
  real a, b;
  ggo_sincos_turn((real)f, &a, &b);
  *s = (double)a;
  *c = (double)b;
}
/* Samples n Klein-Nishina scatterings at energy e (MeV): writes E'/E and cos(theta). */
void GGO_PREFIX(sample_compton)(double e, uint64_t seed, int n, double *eps_out, double *cost_out) {
  scene_t s;
  memset(&s, 0, sizeof(s));
  static real maj2[2] = {R(1), R(1)};
  s.n_e = 2;
  s.maj = maj2;
  s.ln_emin = R(-10);
  s.inv_dln = R(0.01);
  s.e_min = R(0);
  tally_t t;
  memset(&t, 0, sizeof(t));
  for (int i = 0; i < n; ++i) {
    rng_t g;
    rng_init(&g, seed, (uint64_t)i, 0u);
    photon_t ph;
    memset(&ph, 0, sizeof(ph));
    ph.dir[2] = R(1);
    ph.alive = 1;
    set_energy(&s, &ph, (real)e);
    real ed;
    compton(&s, &ph, &g, &t, &ed);
    eps_out[i] = (double)ph.e / e;
    cost_out[i] = (double)ph.dir[2];
  }
}

/* Samples n primaries (history ids 0..n-1): position, direction, energy. */
int GGO_PREFIX(sample_source)(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                              const gg_source_desc *src, uint64_t seed, int n, double *pos, double *dir,
                              double *ene, uint64_t *counters) {
  scene_t s;
  scene_init(&s, tb, vol, w, src);
  tally_t t;
  memset(&t, 0, sizeof(t));
  int st = GG_OK;
  for (int i = 0; i < n && st == GG_OK; ++i) {
    rng_t g;
    rng_init(&g, seed, (uint64_t)i, 0u);
    photon_t ph;
    st = sample_primary(&s, &g, &ph, &t, (uint64_t)i);
    for (int a = 0; a < 3; ++a) {
      pos[3 * i + a] = (double)ph.pos[a];
      dir[3 * i + a] = (double)ph.dir[a];
    }
    ene[i] = (double)ph.e;
  }
  for (int c = 0; c < GG_N_COUNTERS; ++c) counters[c] += t.cnt[c];
  scene_free(&s);
  return st;
}

/* Samples n Rayleigh scatterings of a photon of energy e in composition comp;
   writes cos(theta). */
void GGO_PREFIX(sample_rayleigh)(const gg_tables_desc *tb, int comp, double e, uint64_t seed, int n,
                                 double *cost_out) {
  scene_t s;
  memset(&s, 0, sizeof(s));
  s.n_e = tb->n_e; s.n_comp = tb->n_comp; s.n_ray = tb->n_ray;
  s.ln_emin = (real)tb->ln_emin; s.inv_dln = (real)tb->inv_dln; s.e_min = (real)tb->e_min;
  s.ray_amax = conv_f(tb->ray_amax, (size_t)tb->n_comp * tb->n_e);
  s.ray_x2 = conv_f(tb->ray_x2, (size_t)tb->n_ray);
  s.ray_cum = conv_f(tb->ray_cum, (size_t)tb->n_comp * tb->n_ray);
  s.maj = conv_f(tb->sig, (size_t)tb->n_e); /* any positive row */
  tally_t t;
  memset(&t, 0, sizeof(t));
  for (int i = 0; i < n; ++i) {
    rng_t g;
    rng_init(&g, seed, (uint64_t)i, 0u);
    photon_t ph;
    memset(&ph, 0, sizeof(ph));
    ph.dir[2] = R(1);
    set_energy(&s, &ph, (real)e);
    rayleigh(&s, comp, &ph, &g, &t);
    cost_out[i] = (double)ph.dir[2];
  }
  free(s.ray_amax); free(s.ray_x2); free(s.ray_cum); free(s.maj);
}

/* First flight of n primaries: counts histories whose photon leaves the image
   box without a real interaction (out[0]) and those that interact in it
   (out[1]); primaries that never reach the image are not counted. */
int GGO_PREFIX(first_flight)(const gg_tables_desc *tb, const gg_volume_desc *vol, const gg_world_desc *w,
                             const gg_source_desc *src, uint64_t seed, int n, uint64_t *out) {
  scene_t s;
  scene_init(&s, tb, vol, w, src);
  tally_t t;
  memset(&t, 0, sizeof(t));
  out[0] = out[1] = 0;
  for (int i = 0; i < n; ++i) {
    rng_t g;
    rng_init(&g, seed, (uint64_t)i, 0u);
    photon_t ph;
    if (sample_primary(&s, &g, &ph, &t, (uint64_t)i) != GG_OK) { scene_free(&s); return GG_ERR_DOMAIN; }
    start_photon(&s, &ph);
    if (!ph.in_image) {
      real tin = entry_distance(ph.pos, ph.dir, s.bmin, s.bmax);
      if (!(tin < R(INFINITY))) continue;
      for (int a = 0; a < 3; ++a) ph.pos[a] = ph.pos[a] + tin * ph.dir[a];
      ph.in_image = 1;
      ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
    }
    for (;;) {
      real u = u01_open0(&g);
      real sd = -ggo_log(u);
      sd = sd * ph.inv_mumax;
      if (sd >= ph.t_exit) { out[0]++; break; }
      ph.t_exit = ph.t_exit - sd;
      for (int a = 0; a < 3; ++a) ph.pos[a] = ph.pos[a] + sd * ph.dir[a];
      int ix = (int)((ph.pos[0] - s.bmin[0]) * s.inv_sp[0]);
      int iy = (int)((ph.pos[1] - s.bmin[1]) * s.inv_sp[1]);
      int iz = (int)((ph.pos[2] - s.bmin[2]) * s.inv_sp[2]);
      ix = ix < 0 ? 0 : (ix >= s.nx ? s.nx - 1 : ix);
      iy = iy < 0 ? 0 : (iy >= s.ny ? s.ny - 1 : iy);
      iz = iz < 0 ? 0 : (iz >= s.nz ? s.nz - 1 : iz);
      uint32_t v = (uint32_t)ix + (uint32_t)s.nx * ((uint32_t)iy + (uint32_t)s.ny * (uint32_t)iz);
      int m = s.labels[v];
      real mu = interp_row(s.sig + (size_t)s.mat_comp[m] * s.n_e, ph.ei);
      mu = s.mat_rho[m] * mu;
      if (u01(&g) * ph.mumax < mu) { out[1]++; break; }
    }
  }
  scene_free(&s);
  return GG_OK;
}

/* Hole lattice probe: 1 and the hole centre when (a1, a2) lies in a hole. */
int GGO_PREFIX(find_hole)(const gg_spect_desc *sp, double a1, double a2, double *cx, double *cy) {
  scene_t s;
  memset(&s, 0, sizeof(s));
  spect_init(&s, sp);
  real x = 0, y = 0;
  int in = find_hole(&s, (real)a1, (real)a2, &x, &y);
  *cx = (double)x;
  *cy = (double)y;
  return in;
}

/* Distance from (qx, qy) (relative to a hole centre) to the hole wall along (d1, d2). */
double GGO_PREFIX(hex_exit)(const gg_spect_desc *sp, double qx, double qy, double d1, double d2) {
  scene_t s;
  memset(&s, 0, sizeof(s));
  spect_init(&s, sp);
  return (double)hex_exit(&s, (real)qx, (real)qy, (real)d1, (real)d2);
}
