// gg_spect.cuh - SPECT head transport and the projection digitizer (device side).
//
// Head model (local frame: a1 along e1, a2 along e2, w along the outward
// normal, collimator front face at w = 0): collimator slab with hexagonal
// vacuum holes on two offset rectangular lattices (faces normal to 30, 90,
// 150 degrees), vacuum gap, crystal.  In the collimator the photon is
// tracked with Woodcock steps against the collimator attenuation (points that
// land in a hole are null collisions) and crosses a hole it starts in
// analytically up to the hole wall.  Crystal interactions add to the event's
// per-head sum and energy-winner position (GateDigiAdderInVolume::Update,
// EnergyWinnerPosition, core/opengate_core/opengate_lib/digitizer/
// GateDigiAdderInVolume.cpp:29-77); at the end of the event each head's single
// is classified into the windows [lo, hi)
// (GateDigitizerEnergyWindowsActor.cpp:116-132) and counted in the detector
// pixel of its position (GateDigitizerProjectionActor.cpp:127-177).
#pragma once
#include "gg_device.cuh"

namespace gg {

constexpr double kCos30 = 0.86602540378443864676;

template <typename real>
__device__ __forceinline__ real dot3(const real a[3], const real b[3]) {
  real r = a[0] * b[0];
  r = r + a[1] * b[1];
  r = r + a[2] * b[2];
  return r;
}

// Frame of head h at gantry position `run`: 12 values c[3], u[3], e1[3], e2[3]
// loaded from the read-only frame table.
template <typename real>
struct HeadFrame {
  real c[3], u[3], e1[3], e2[3];
};

template <typename real>
__device__ __forceinline__ HeadFrame<real> head_frame(const Scene<real> &s, int run, int h) {
  const real *f = s.frames + ((size_t)run * s.n_heads + h) * 12;
  HeadFrame<real> r;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    r.c[a] = __ldg(f + a);
    r.u[a] = __ldg(f + 3 + a);
    r.e1[a] = __ldg(f + 6 + a);
    r.e2[a] = __ldg(f + 9 + a);
  }
  return r;
}

template <typename real>
__device__ __forceinline__ void to_local(const HeadFrame<real> &f, const real p[3], const real d[3], real lp[3],
                                         real ld[3]) {
  real q[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) q[a] = p[a] - f.c[a];
  lp[0] = dot3(q, f.e1);
  lp[1] = dot3(q, f.e2);
  lp[2] = dot3(q, f.u);
  ld[0] = dot3(d, f.e1);
  ld[1] = dot3(d, f.e2);
  ld[2] = dot3(d, f.u);
}

template <typename real>
__device__ __forceinline__ void to_world(const HeadFrame<real> &f, const real lp[3], const real ld[3], real p[3],
                                         real d[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    real x = lp[0] * f.e1[a];
    x = f.c[a] + x;
    x = x + lp[1] * f.e2[a];
    p[a] = x + lp[2] * f.u[a];
    real y = ld[0] * f.e1[a];
    y = y + ld[1] * f.e2[a];
    d[a] = y + ld[2] * f.u[a];
  }
}

template <typename real>
__device__ __forceinline__ real gg_fabs(real x) {
  return x < R<real>(0) ? -x : x;
}

template <typename real>
__device__ __forceinline__ bool find_hole(const Scene<real> &s, real a1, real a2, real &cx, real &cy) {
#pragma unroll
  for (int lat = 0; lat < 2; ++lat) {
    real ox = lat ? s.hpx : R<real>(0), oy = lat ? s.hpy : R<real>(0);
    real fx = a1 - ox;
    fx = fx * s.inv_px;
    fx = fx + R<real>(0.5);
    fx = gg_floor(fx);
    real fy = a2 - oy;
    fy = fy * s.inv_py;
    fy = fy + R<real>(0.5);
    fy = gg_floor(fy);
    real x = fx * s.px;
    x = x + ox;
    real y = fy * s.py;
    y = y + oy;
    real qx = a1 - x, qy = a2 - y;
    real t0 = qx * R<real>(kCos30), t1 = qy * R<real>(0.5);
    real n0 = t1 + t0, n2 = t1 - t0;
    if (gg_fabs(qy) <= s.apo && gg_fabs(n0) <= s.apo && gg_fabs(n2) <= s.apo) {
      cx = x;
      cy = y;
      return true;
    }
  }
  return false;
}

template <typename real>
__device__ __forceinline__ real hex_exit(const Scene<real> &s, real qx, real qy, real d1, real d2) {
  real t0 = qx * R<real>(kCos30), t1 = qy * R<real>(0.5);
  real u0 = d1 * R<real>(kCos30), u1 = d2 * R<real>(0.5);
  real qn[3] = {t1 + t0, qy, t1 - t0};
  real dn[3] = {u1 + u0, d2, u1 - u0};
  real t = gg_inf(real(0));
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    real tk;
    if (dn[k] > R<real>(0)) {
      tk = s.apo - qn[k];
      tk = tk / dn[k];
      if (tk < t) t = tk;
    } else if (dn[k] < R<real>(0)) {
      tk = -s.apo - qn[k];
      tk = tk / dn[k];
      if (tk < t) t = tk;
    }
  }
  return t < R<real>(0) ? R<real>(0) : t;
}

template <typename real>
__device__ __forceinline__ void move3(real p[3], const real d[3], real t) {
#pragma unroll
  for (int a = 0; a < 3; ++a) p[a] = p[a] + t * d[a];
}

// per-event crystal accumulation of each head; wpos = head-local (a1, a2) of
// the energy winner, which is also its position on the detector plane
template <typename real>
struct Event {
  real esum[2], emax[2], wpos[2][2];
  real w[2];  // weight of each head's single (free flight; 1 otherwise)
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      esum[h] = R<real>(0);
      emax[h] = R<real>(0);
      wpos[h][0] = wpos[h][1] = R<real>(0);
      w[h] = R<real>(1);
    }
  }
};

// Slab bound zb[k] and slab material hmat[k] for a k held in a register:
// selected over the constant indices (an indexed access would move the
// scene to local memory).
template <typename real>
__device__ __forceinline__ real head_zb(const Scene<real> &s, int k) {
  real z = s.zb[0];
#pragma unroll
  for (int j = 1; j <= kHeadRegions; ++j) z = k == j ? s.zb[j] : z;
  return z;
}

template <typename real>
__device__ __forceinline__ int head_mat(const Scene<real> &s, int k) {
  int m = s.hmat[0];
#pragma unroll
  for (int j = 1; j < kHeadRegions; ++j) m = k == j ? s.hmat[j] : m;
  return m;
}

// Slab of a head-local depth w: the number of inner bounds at or below w.
template <typename real>
__device__ __forceinline__ int head_region(const Scene<real> &s, real w) {
  int k = 0;
#pragma unroll
  for (int j = 1; j < kHeadRegions; ++j) k += (j < s.n_hreg && !(w < s.zb[j])) ? 1 : 0;
  return k;
}

template <typename real>
__device__ __forceinline__ void head_cross(const Scene<real> &s, Photon<real> &ph, bool leave) {
  if (leave) {
    real p[3], d[3];
    to_world(head_frame(s, ph.run, ph.head), ph.pos, ph.dir, p, d);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      ph.pos[a] = p[a];
      ph.dir[a] = d[a];
    }
    ph.in_head = 0;
    ph.exclude = 1 + ph.head;
  } else {
    ph.hreg += ph.dir[2] > R<real>(0) ? 1 : -1;
    ph.left_hole = 0;
  }
}

// Geometric part of one head step.  Returns true when the step continues
// with a sampled collision in material `mat` (collimator or crystal), after
// moving the photon to the tentative point; the caller then draws the
// interaction unless the point lies in a hole (null collision).
template <typename real>
__device__ __forceinline__ int head_flight(const Scene<real> &s, Photon<real> &ph, Rng &g, int &mat) {
  real *l = ph.pos, *d = ph.dir;
  real lo[3] = {-s.half_w, -s.half_w, R<real>(0)};
  real hi[3] = {s.half_w, s.half_w, s.zend};
  int face;
  real tbox = exit_distance_face(l, d, lo, hi, face);
  real treg = gg_inf(real(0));
  const real zlo = head_zb(s, ph.hreg), zhi = head_zb(s, ph.hreg + 1);
  if (d[2] > R<real>(0)) {
    treg = zhi - l[2];
    treg = treg / d[2];
  } else if (d[2] < R<real>(0)) {
    treg = zlo - l[2];
    treg = treg / d[2];
  }
  if (treg < R<real>(0)) treg = R<real>(0);
  bool leave = tbox <= treg;
  real tlim = leave ? tbox : treg;
  // shielded sides: a photon that reaches a side face of the box stops there
  const bool absorb = leave && s.side_black && face != 2;
  if (ph.hreg == 0 && !ph.left_hole) {
    real cx, cy;
    if (find_hole(s, l[0], l[1], cx, cy)) {
      real th = hex_exit(s, l[0] - cx, l[1] - cy, d[0], d[1]);
      ph.left_hole = 1;
      if (th < tlim) {
        move3(l, d, th);
        return 0;
      }
      move3(l, d, tlim);
      if (absorb) ph.alive = 0;
      else head_cross(s, ph, leave);
      return 0;
    }
  }
  ph.left_hole = 0;
  const int rm = head_mat(s, ph.hreg);
  if (rm < 0) {  // vacuum slab (the gap)
    move3(l, d, tlim);
    if (absorb) ph.alive = 0;
    else head_cross(s, ph, leave);
    return 0;
  }
  mat = rm;
  real mu = interp_row(s.sig + (size_t)s.mat_comp[mat] * s.n_e, ph.ei);
  mu = s.mat_rho[mat] * mu;
  real u = u01_open0<real>(g);
  real sd = -gg_log(u);
  sd = sd / mu;
  if (sd >= tlim) {
    move3(l, d, tlim);
    if (absorb) ph.alive = 0;
    else head_cross(s, ph, leave);
    return 0;
  }
  move3(l, d, sd);
  if (ph.hreg == 0) {
    real cx, cy;
    if (find_hole(s, l[0], l[1], cx, cy)) return 0;  // null collision inside a hole
  }
  return 1;
}

// World step with the image box and the head boxes as targets.  Returns
// 1 for an air interaction at the new position, 0 otherwise (ph.alive = 0
// when the photon left the world).
template <typename real>
__device__ __forceinline__ int spect_world_flight(const Scene<real> &s, Photon<real> &ph, Rng &g) {
  real inf = gg_inf(real(0));
  real tb = ph.exclude != 0 ? entry_distance(ph.pos, ph.dir, s.bmin, s.bmax) : inf;
  int box = 0, bface = 2;
  real hlo[3] = {-s.half_w, -s.half_w, R<real>(0)};
  real hhi[3] = {s.half_w, s.half_w, s.zend};
  for (int h = 0; h < s.n_heads; ++h) {
    if (ph.exclude == 1 + h) continue;
    real lp[3], ld[3];
    to_local(head_frame(s, ph.run, h), ph.pos, ph.dir, lp, ld);
    int f;
    real th = entry_distance_face(lp, ld, hlo, hhi, f);
    if (th < tb) {
      tb = th;
      box = 1 + h;
      bface = f;
    }
  }
  real wlo[3] = {-s.whalf[0], -s.whalf[1], -s.whalf[2]};
  real tout = exit_distance(ph.pos, ph.dir, wlo, s.whalf);
  int wm = s.world_mat;
  real mu = interp_row(s.sig + (size_t)s.mat_comp[wm] * s.n_e, ph.ei);
  mu = s.mat_rho[wm] * mu;
  real u = u01_open0<real>(g);
  real sd = -gg_log(u);
  sd = sd / mu;
  if (sd < tb && sd < tout) {
    move3(ph.pos, ph.dir, sd);
    return 1;
  }
  if (tb <= tout) {
    move3(ph.pos, ph.dir, tb);
    if (box == 0) {
      ph.in_image = 1;
      ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
    } else if (s.side_black && bface != 2) {
      ph.alive = 0;  // stopped by the head's side shielding
    } else {
      int h = box - 1;
      real lp[3], ld[3];
      to_local(head_frame(s, ph.run, h), ph.pos, ph.dir, lp, ld);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        ph.pos[a] = lp[a];
        ph.dir[a] = ld[a];
      }
      ph.in_head = 1;
      ph.head = h;
      ph.hreg = head_region(s, lp[2]);
      ph.left_hole = 0;
    }
    return 0;
  }
  ph.alive = 0;
  return 0;
}

// Free flight outside the heads (GateGammaFreeFlightOptn /
// GateGammaFreeFlightOptrActor with the heads as excluded volumes,
// biasing/GateGammaFreeFlightOptn.cpp:34-83, GateVBiasOptrActor.cpp:85-92):
// the photon does not interact in the world or the image; it flies straight
// to the nearest head entry (the head it just left excluded) and its weight
// is multiplied by the probability of getting there, exp(-optical depth)
// (air over the whole path, the voxels' attenuation inside the image box).
// Photons at or below the energy or weight cutoff, and photons whose line
// misses every head, stop; so do photons whose direction makes a cosine
// below cos_min with the axis of the head they would enter (angle check of
// the angular acceptance, before the optical depth is computed; -2: none).
// Returns 1 at a head entry (head-local state as spect_world_flight sets it),
// 0 when the photon stopped.  ff_target is its first part: the cutoffs, the
// head the line enters (1 + head, at distance tb) and the checks on it; 0
// when the photon stopped there.
template <typename real>
__device__ __forceinline__ int ff_target(const Scene<real> &s, Photon<real> &ph, real cos_min, real &tb_out) {
  if (ph.e <= s.ff_ecut || ph.w <= s.ff_wcut) {
    ph.alive = 0;
    return 0;
  }
  if (cos_min > R<real>(-1)) {
    // angle check first: no head axis within the tolerance means the test
    // below fails too (its cosine is the same dot product), without the
    // box intersections
    bool any = false;
    for (int h = 0; h < s.n_heads; ++h) {
      if (ph.exclude == 1 + h) continue;
      const HeadFrame<real> f = head_frame(s, ph.run, h);
      any = any || !(dot3(ph.dir, f.u) < cos_min);
    }
    if (!any) {
      ph.alive = 0;
      return 0;
    }
  }
  real tb = gg_inf(real(0));
  int box = 0, bface = 2;
  real cos_box = R<real>(0);
  real hlo[3] = {-s.half_w, -s.half_w, R<real>(0)};
  real hhi[3] = {s.half_w, s.half_w, s.zend};
  for (int h = 0; h < s.n_heads; ++h) {
    if (ph.exclude == 1 + h) continue;
    real lp[3], ld[3];
    to_local(head_frame(s, ph.run, h), ph.pos, ph.dir, lp, ld);
    int f;
    real th = entry_distance_face(lp, ld, hlo, hhi, f);
    if (th < tb) {
      tb = th;
      box = 1 + h;
      cos_box = ld[2];
      bface = f;
    }
  }
  real wlo[3] = {-s.whalf[0], -s.whalf[1], -s.whalf[2]};
  const real tout = exit_distance(ph.pos, ph.dir, wlo, s.whalf);
  // (a line into a shielded side face cannot be detected)
  if (!(tb <= tout) || cos_box < cos_min || (s.side_black && bface != 2)) {
    ph.alive = 0;
    return 0;
  }
  tb_out = tb;
  return box;
}

// Optical depth of a straight path through the image (gg_physics.cuh).
template <typename real, int GROUP = 1>
__device__ __forceinline__ real image_depth(const Scene<real> &s, const real p[3], const real d[3], real len,
                                           const EIdx<real> &ei);

template <typename real, int GROUP = 1>
__device__ __forceinline__ int ff_flight(const Scene<real> &s, Photon<real> &ph, real cos_min) {
  real tb;
  const int box = ff_target(s, ph, cos_min, tb);
  if (!box) return 0;
  const int wm = s.world_mat;
  real mu_air = interp_row(s.sig + (size_t)s.mat_comp[wm] * s.n_e, ph.ei);
  mu_air = s.mat_rho[wm] * mu_air;
  real l_air = tb;
  real tau = R<real>(0);
  const real t0 = entry_distance(ph.pos, ph.dir, s.bmin, s.bmax);
  if (t0 < tb) {
    real p0[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) p0[a] = ph.pos[a] + t0 * ph.dir[a];
    real lin = exit_distance(p0, ph.dir, s.bmin, s.bmax);
    const real rest = tb - t0;
    lin = lin < rest ? lin : rest;
    tau = image_depth<real, GROUP>(s, p0, ph.dir, lin, ph.ei);
    l_air = l_air - lin;
  }
  real ta = mu_air * l_air;
  tau = tau + ta;
  ph.w = ph.w * gg_exp(-tau);
  if (ph.w <= s.ff_wcut) {
    ph.alive = 0;
    return 0;
  }
  move3(ph.pos, ph.dir, tb);
  const int h = box - 1;
  real lp[3], ld[3];
  to_local(head_frame(s, ph.run, h), ph.pos, ph.dir, lp, ld);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    ph.pos[a] = lp[a];
    ph.dir[a] = ld[a];
  }
  ph.in_image = 0;
  ph.in_head = 1;
  ph.head = h;
  ph.hreg = head_region(s, lp[2]);
  ph.left_hole = 0;
  return 1;
}

// Two standard normal deviates from the history's stream (Box & Muller 1958):
// sqrt(-2 ln u1) (cos, sin)(2 pi u2), u1 in (0, 1].
template <typename real>
__device__ __forceinline__ void normal_pair(Rng &g, real &z0, real &z1) {
  const real u1 = u01_open0<real>(g);
  const real u2 = u01<real>(g);
  real r = gg_log(u1);
  r = R<real>(-2) * r;
  r = gg_sqrt(r);
  real sn, cs;
  gg_sincos_turn(u2, sn, cs);
  z0 = r * cs;
  z1 = r * sn;
}

// FWHM -> standard deviation, 1 / (2 sqrt(2 ln 2))
constexpr double kFwhmToSigma = 0.42466090014400953;

// Energy blurring of a single (GateDigitizerBlurringActor::GaussianBlur /
// InverseSquare / Linear, digitizer/GateDigitizerBlurringActor.cpp:74-97):
// sigma fixed, or FWHM/E = res sqrt(E_ref) / sqrt(E), or slope (E - E_ref) + res.
template <typename real>
__device__ __forceinline__ real blur_energy(const Scene<real> &s, real e, Rng &g) {
  real sigma;
  if (s.eblur == 1) {
    sigma = s.eb_sigma;
  } else {
    real v;
    if (s.eblur == 2) {
      v = gg_sqrt(s.eb_ref);
      const real q = gg_sqrt(e);
      v = v / q;
      v = s.eb_res * v;
    } else {
      v = e - s.eb_ref;
      v = s.eb_slope * v;
      v = v + s.eb_res;
    }
    sigma = v * e;
    sigma = sigma * (real)kFwhmToSigma;
  }
  real z0, z1;
  normal_pair(g, z0, z1);
  const real d = sigma * z0;
  return e + d;
}

// erf by Abramowitz & Stegun 7.1.26 (|error| < 1.5e-7), odd extension.
template <typename real>
__device__ __forceinline__ real erf_as(real x) {
  const real ax = x < R<real>(0) ? -x : x;
  real t = R<real>(0.3275911) * ax;
  t = R<real>(1) + t;
  t = R<real>(1) / t;
  real p = R<real>(1.061405429) * t;
  p = p + R<real>(-1.453152027);
  p = p * t;
  p = p + R<real>(1.421413741);
  p = p * t;
  p = p + R<real>(-0.284496736);
  p = p * t;
  p = p + R<real>(0.254829592);
  p = p * t;
  real x2 = ax * ax;
  x2 = -x2;
  real y = p * gg_exp(x2);
  y = R<real>(1) - y;
  return x < R<real>(0) ? -y : y;
}

// Standard deviation of the redraws of a truncated blur
// (GateDigitizerSpatialBlurringActor::ComputeTruncatedGaussianSigma and
// ComputeEdgeCorrectedSigma, GateDigitizerSpatialBlurringActor.cpp:158-206).
template <typename real>
__device__ __forceinline__ real trunc_sigma(real mu, real sigma, real lo, real hi) {
  const real inv_sqrt_2pi = R<real>(0.39894228040143267794);
  const real inv_sqrt2 = R<real>(0.70710678118654752440);
  real a = lo - mu;
  a = a / sigma;
  real b = hi - mu;
  b = b / sigma;
  real pa = R<real>(-0.5) * a;
  pa = pa * a;
  pa = gg_exp(pa) * inv_sqrt_2pi;
  real pb = R<real>(-0.5) * b;
  pb = pb * b;
  pb = gg_exp(pb) * inv_sqrt_2pi;
  real fa = erf_as(a * inv_sqrt2);
  fa = R<real>(1) + fa;
  fa = R<real>(0.5) * fa;
  real fb = erf_as(b * inv_sqrt2);
  fb = R<real>(1) + fb;
  fb = R<real>(0.5) * fb;
  const real z = fb - fa;
  real shift = pa - pb;
  shift = shift / z;
  real c = a * pa;
  c = c - b * pb;
  c = c / z;
  real var = R<real>(1) - c;
  var = var - shift * shift;
  real s1 = sigma * gg_sqrt(var);
  real delta = mu - lo;
  const real dh = hi - mu;
  delta = dh < delta ? dh : delta;
  delta = delta > R<real>(0) ? delta : R<real>(0);
  real dn = delta / s1;
  dn = dn > R<real>(0.95) ? dn : R<real>(0.95);
  if (dn < R<real>(4)) {
    real corr = R<real>(-0.86538264) * dn;
    corr = R<real>(3.61070188) * gg_exp(corr);
    s1 = s1 * corr;
  }
  return s1;
}

// Truncated blur of one coordinate: while outside [lo, hi], redraw around mu
// with the corrected sigma (at most kLoopCap draws, then clamped).
template <typename real>
__device__ __forceinline__ real trunc_redraw(real mu, real p, real sigma, real lo, real hi, Rng &g) {
  if (!(p > hi || p < lo)) return p;
  const real sg = trunc_sigma(mu, sigma, lo, hi);
  for (int k = 0; k < kLoopCap; ++k) {
    real z0, z1;
    normal_pair(g, z0, z1);
    p = sg * z0;
    p = mu + p;
    if (!(p > hi || p < lo)) return p;
  }
  return p < lo ? lo : hi;
}

// Spatial blurring of a single's crystal position (a1, a2) (GateDigitizerSpatialBlurringActor::
// BlurCurrentThreeVectorValue, GateDigitizerSpatialBlurringActor.cpp:85-156): the crystal
// spans |a| <= half_width; keep_in_solid_limits puts points outside just inside the edge.
template <typename real>
__device__ __forceinline__ void blur_position(const Scene<real> &s, real &a1, real &a2, Rng &g) {
  real z0, z1;
  normal_pair(g, z0, z1);
  real p0 = s.sb_sigma[0] * z0;
  p0 = a1 + p0;
  real p1 = s.sb_sigma[1] * z1;
  p1 = a2 + p1;
  const real hi = s.half_w, lo = -s.half_w;
  if (s.sblur == 2) {
    p0 = trunc_redraw(a1, p0, s.sb_sigma[0], lo, hi, g);
    p1 = trunc_redraw(a2, p1, s.sb_sigma[1], lo, hi, g);
  } else if (s.sb_keep) {
    // just inside the edge: 1e-6 of the half width (1 nm in the reference,
    // which FP32 would round back onto the edge)
    const real tiny = s.half_w * R<real>(1e-6);
    if (p0 < lo) p0 = lo + tiny;
    if (p1 < lo) p1 = lo + tiny;
    if (p0 > hi) p0 = hi - tiny;
    if (p1 > hi) p1 = hi - tiny;
  }
  a1 = p0;
  a2 = p1;
}

// Singles of one event: (blurring,) windows and projection pixel per head.
// Blurring draws come from the history's stream, head 0 before head 1,
// energy before position.
template <typename real>
__device__ __forceinline__ unsigned score_singles(const Scene<real> &s, const Event<real> &ev, int run, Rng &g) {
  unsigned n_singles = 0;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    if (h >= s.n_heads) break;
    real e = ev.esum[h];
    if (!(e > R<real>(0))) continue;
    ++n_singles;
    real a1 = ev.wpos[h][0], a2 = ev.wpos[h][1];
    if (s.centroid) {  // GateDigiAdderInVolume::Terminate: position sum / energy sum
      a1 = a1 / e;
      a2 = a2 / e;
    }
    if (s.eblur) e = blur_energy(s, e, g);
    if (s.sblur) blur_position(s, a1, a2, g);
    if (s.singles) {
      const unsigned long long slot = atomicAdd(s.n_singles_rec, 1ull);
      if (slot < s.singles_cap) {
        SingleRec r;
        r.event_id = (uint64_t)g.h0 | ((uint64_t)g.h1 << 32);
        r.head = h;
        r.run = run;
        r.energy = (double)e;
        r.a1 = (double)a1;
        r.a2 = (double)a2;
        r.weight = s.ff ? (double)ev.w[h] : 1.0;
        s.singles[slot] = r;
      }
    }
    real fx = a1 + s.pix_half[0];
    fx = fx * s.inv_psp[0];
    real fy = a2 + s.pix_half[1];
    fy = fy * s.inv_psp[1];
    if (!(fx >= R<real>(0) && fx < (real)s.pnx && fy >= R<real>(0) && fy < (real)s.pny)) continue;
    int i = (int)fx, j = (int)fy;
    // free flight: the single adds its weight in 2^-32 units, and the exact
    // square of that for the history-by-history variance (low 32 bits, rest)
    unsigned long long q = 0, lo = 0, rest = 0;
    if (s.ff) {
      q = (unsigned long long)to_fixed(ev.w[h]);
      lo = q * q;
      rest = (__umul64hi(q, q) << 32) | (lo >> 32);
      lo &= 0xffffffffull;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k < s.n_win && e >= s.wlo[k] && e < s.whi[k]) {
        size_t idx = ((((size_t)h * s.n_runs + run) * s.n_win + k) * s.pny + j) * s.pnx + i;
        if (!s.ff) {
          atomicAdd(s.proj + idx, 1ull);
        } else if (q) {
          atomicAdd(s.wproj + idx, q);
          if (lo) atomicAdd(s.wproj2 + 2 * idx, lo);
          if (rest) atomicAdd(s.wproj2 + 2 * idx + 1, rest);
        }
      }
    }
  }
  return n_singles;
}

}  // namespace gg
