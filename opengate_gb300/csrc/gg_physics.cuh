// gg_physics.cuh - device physics shared by the transport kernels: the
// per-history deposit list and fixed-point tallies, photon interactions
// (Compton, photoelectric, Rayleigh, pair), primary sampling, the primary
// records of the source stage, and the flight / interaction steps of the
// phase-batched transport loop.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gate_gpu.h"
#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_spect.cuh"

namespace gg {

// One history's voxel list: entry k at vox[k * stride], acc[k * stride] in
// shared memory (a column per thread of the block), so the list takes no
// registers across the transport loop.  Kernels that never score pass null
// arrays with n = 0.
template <typename real>
struct HistList {
  uint32_t *vox;
  real *acc;
  int stride;
  int n;
};

struct BlockCounters {
  unsigned int histories, tally_entries, list_overflows, escaped, skipped, loop_capped, stack_overflow,
      secondaries;
};

template <typename real>
struct Tally {
  unsigned long long *acc_e;
  unsigned long long *acc_e2;
};

// One history's entry: q = edep in units of 2^-32 MeV goes to acc_e[v]; its
// exact square q^2 (units of 2^-64 MeV^2, below 2^74) is split into its low
// 32 bits, added to acc_e2[2v], and the rest q^2 >> 32 (units of 2^-32 MeV^2),
// added to acc_e2[2v+1]: two reductions that need no return value.  The low
// word cannot overflow within a batch (fewer than 2^32 entries per voxel), so
// sum = acc_e2[2v+1] * 2^-32 + acc_e2[2v] * 2^-64 MeV^2 exactly; integer sums
// do not depend on the order of the atomics, and a voxel hit by one history
// has edep^2 == edep * edep exactly in these units.
template <typename real>
__device__ __forceinline__ void hlist_flush(HistList<real> &l, const Tally<real> &t, BlockCounters *bc) {
  for (int k = 0; k < l.n; ++k) {
    const unsigned long long q = (unsigned long long)to_fixed(l.acc[k * l.stride]);
    const uint32_t v = l.vox[k * l.stride];
    atomicAdd(&t.acc_e[v], q);
    if (t.acc_e2) {
      const unsigned long long lo = q * q;
      const unsigned long long hi = __umul64hi(q, q);
      atomicAdd(&t.acc_e2[2 * (size_t)v], lo & 0xffffffffull);
      atomicAdd(&t.acc_e2[2 * (size_t)v + 1], (hi << 32) | (lo >> 32));
    }
  }
  if (l.n) atomicAdd(&bc->tally_entries, (unsigned int)l.n);
  l.n = 0;
}

// Histories a warp has claimed from the launch's work counter and not yet
// handed out, [p[0], p[1]), kept in shared memory (one pair per warp) because
// only refills use them.  Every lane of the warp calls this with the ballot of
// the lanes that need a history; those get the next histories in lane order
// (the others a value they ignore), `chunk` more being claimed when the pool
// runs short.
__device__ __forceinline__ uint64_t warp_pool_claim(uint64_t *p, unsigned m_need, unsigned lane, unsigned lt_mask,
                                                    unsigned long long *next, int chunk) {
  const unsigned n_need = __popc(m_need);
  const unsigned rank = __popc(m_need & lt_mask);
  uint64_t pn = p[0];
  const uint64_t avail = p[1] - pn;
  uint64_t h;
  if (avail >= n_need) {
    h = pn + rank;
    pn += n_need;
    __syncwarp();
    if (lane == 0) p[0] = pn;
  } else {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(next, (unsigned long long)chunk);
    base = __shfl_sync(0xffffffffu, base, 0);
    h = rank < avail ? pn + rank : base + (rank - avail);
    __syncwarp();
    if (lane == 0) {
      p[0] = base + (n_need - avail);
      p[1] = base + (uint64_t)chunk;
    }
  }
  __syncwarp();
  return h;
}

template <typename real>
__device__ __forceinline__ void deposit(HistList<real> &l, const Tally<real> &t, BlockCounters *bc,
                                        uint32_t v, real e, unsigned int &n_dep) {
  if (!(e > R<real>(0))) return;
  ++n_dep;
  for (int k = 0; k < l.n; ++k) {
    if (l.vox[k * l.stride] == v) {
      real &a = l.acc[k * l.stride];
      a = a + e;
      return;
    }
  }
  if (l.n == kHistList) {
    atomicAdd(&bc->list_overflows, 1u);
    hlist_flush(l, t, bc);
  }
  l.vox[l.n * l.stride] = v;
  l.acc[l.n * l.stride] = e;
  l.n++;
}

// Klein-Nishina (G4KleinNishinaCompton sampling of the Physics Reference Manual)
// The rejection loop of the Klein-Nishina sampling: eps = E'/E, 1 - cos(theta)
// and sin^2(theta) of the scattering (3 draws per trial).
template <typename real>
__device__ __forceinline__ void compton_kn(real e, Rng &g, BlockCounters *bc, real &eps, real &onecost,
                                           real &sint2) {
  real k = e * R<real>(1.0 / kMC2);
  real twok = R<real>(2) * k;
  real eps0 = R<real>(1) / (R<real>(1) + twok);
  real eps0sq = eps0 * eps0;
  real alpha1 = -gg_log(eps0);
  real alpha2 = R<real>(1) - eps0sq;
  alpha2 = R<real>(0.5) * alpha2;
  alpha2 = alpha1 + alpha2;
  real epssq;
  int it = 0;
  for (;;) {
    real r0 = u01<real>(g);
    real r1 = u01<real>(g);
    real r2 = u01<real>(g);
    if (alpha1 > alpha2 * r0) {
      eps = gg_exp(-alpha1 * r1);
      epssq = eps * eps;
    } else {
      real w = R<real>(1) - eps0sq;
      w = w * r1;
      epssq = eps0sq + w;
      eps = gg_sqrt(epssq);
    }
    real ek = eps * k;
    onecost = (R<real>(1) - eps) / ek;
    sint2 = onecost * (R<real>(2) - onecost);
    real gr = eps * sint2;
    gr = gr / (R<real>(1) + epssq);
    gr = R<real>(1) - gr;
    if (gr >= r2) break;
    if (++it >= kLoopCap) {
      atomicAdd(&bc->loop_capped, 1u);
      break;
    }
  }
}

// The rest of a Compton scattering sampled by compton_kn: azimuth (one draw),
// new direction and energy; returns the energy given to the electron.
template <typename real>
__device__ __forceinline__ real compton_finish(const Scene<real> &s, Photon<real> &ph, Rng &g, real eps, real onecost,
                                               real sint2) {
  const real e = ph.e;
  real e1 = eps * e;
  real edep = e - e1;
  real cost = R<real>(1) - onecost;
  real sint = gg_sqrt(sint2 > R<real>(0) ? sint2 : R<real>(0));
  real sp, cp;
  gg_sincos_turn(u01<real>(g), sp, cp);
  rotate_dir(ph.dir[0], ph.dir[1], ph.dir[2], cost, sint, cp, sp);
  if (e1 < s.e_min) {
    edep = edep + e1;
    ph.alive = 0;
  } else {
    set_energy(s, ph, e1);
  }
  return edep;
}

template <typename real>
__device__ __forceinline__ real compton(const Scene<real> &s, Photon<real> &ph, Rng &g, BlockCounters *bc) {
  real eps, onecost, sint2;
  compton_kn(ph.e, g, bc, eps, onecost, sint2);
  return compton_finish(s, ph, g, eps, onecost, sint2);
}

// The rejection loop of the Rayleigh sampling (form-factor inversion, then
// the 1 + cos^2 acceptance): cos(theta) of the scattering.
template <typename real>
__device__ __forceinline__ real rayleigh_cost(const Scene<real> &s, int comp, const Photon<real> &ph, Rng &g,
                                              BlockCounters *bc) {
  real k = ph.e * R<real>(1.0 / kHcMevAngstrom);
  real x2max = k * k;
  real amax = interp_row(s.ray_amax + (size_t)comp * s.n_e, ph.ei);
  const real *cu = s.ray_cum + (size_t)comp * s.n_ray;
  const real *xn = s.ray_x2;
  real cost = R<real>(1);
  int it = 0;
  for (;;) {
    if (++it > kLoopCap) {
      atomicAdd(&bc->loop_capped, 1u);
      break;
    }
    real r = u01<real>(g);
    real tt = r * amax;
    // exact inversion of the piecewise-linear cumulative: bisection for the
    // node interval, then linear in x^2 inside it
    int lo = 0, hi = s.n_ray - 1;
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (cu[mid] <= tt) lo = mid;
      else hi = mid;
    }
    real den = cu[lo + 1] - cu[lo];
    real f = R<real>(0);
    if (den > R<real>(0)) {
      f = tt - cu[lo];
      f = f / den;
    }
    real d = xn[lo + 1] - xn[lo];
    d = f * d;
    real x2 = xn[lo] + d;
    if (x2 > x2max) continue;  // beyond the momentum transfer reachable at E
    real q = R<real>(2) * x2;
    q = q / x2max;
    cost = R<real>(1) - q;
    real r2 = u01<real>(g);
    real lhs = R<real>(2) * r2;
    real rhs = cost * cost;
    rhs = R<real>(1) + rhs;
    if (lhs <= rhs) break;
  }
  return cost;
}

template <typename real>
__device__ __forceinline__ real rayleigh_sint2(real cost) {
  real st2 = cost * cost;
  return R<real>(1) - st2;
}

// The rest of a Rayleigh scattering of cosine cost: azimuth (one draw) and new direction.
template <typename real>
__device__ __forceinline__ void rayleigh_finish(Photon<real> &ph, Rng &g, real cost) {
  const real st2 = rayleigh_sint2(cost);
  real sint = gg_sqrt(st2 > R<real>(0) ? st2 : R<real>(0));
  real sp, cp;
  gg_sincos_turn(u01<real>(g), sp, cp);
  rotate_dir(ph.dir[0], ph.dir[1], ph.dir[2], cost, sint, cp, sp);
}

template <typename real>
__device__ __forceinline__ void rayleigh(const Scene<real> &s, int comp, Photon<real> &ph, Rng &g,
                                         BlockCounters *bc) {
  rayleigh_finish(ph, g, rayleigh_cost(s, comp, ph, g, bc));
}

template <typename real>
__device__ __forceinline__ void iso_dir(Rng &g, real d[3]) {
  real cost = R<real>(2) * u01<real>(g);
  cost = R<real>(1) - cost;
  real st2 = cost * cost;
  st2 = R<real>(1) - st2;
  real sint = gg_sqrt(st2 > R<real>(0) ? st2 : R<real>(0));
  real sp, cp;
  gg_sincos_turn(u01<real>(g), sp, cp);
  d[0] = sint * cp;
  d[1] = sint * sp;
  d[2] = cost;
}

// interaction kinds (interact's `kind`)
enum : int { kCompton = 1, kPhoto = 2, kRayleigh = 3, kPair = 4 };

// One secondary slot per thread, in shared memory: after a pair conversion the
// photon continues as one 511 keV photon and the other waits here.  511 keV
// cannot convert again, so one slot always suffices.
template <typename real>
struct Secondary {
  real *base;  // [6][stride]: pos xyz, dir xyz
  int stride, tid;
  int has;
  __device__ __forceinline__ real &at(int k) { return base[k * stride + tid]; }
};

// Process of an interaction at energy index ph.ei in material `mat`: the
// first draw of the interaction against the cumulative fractions (Compton,
// + photoelectric, + Rayleigh; the rest is pair production).
template <typename real>
__device__ __forceinline__ int select_kind(const Scene<real> &s, const Photon<real> &ph, int mat, Rng &g) {
  int c = s.mat_comp[mat];
  const real *cu = s.cum + (size_t)c * 3 * s.n_e;
  real r = u01<real>(g);
  real fc = interp_row(cu, ph.ei);
  if (r < fc) return kCompton;
  real fp = interp_row(cu + s.n_e, ph.ei);
  if (r < fp) return kPhoto;
  real fr = interp_row(cu + 2 * s.n_e, ph.ei);
  if (r < fr) return kRayleigh;
  return kPair;
}

// The interaction of process `kind` (after select_kind).  Returns the energy
// deposited locally (scored by the caller when inside the image).
template <typename real>
__device__ __forceinline__ real apply_kind(const Scene<real> &s, Photon<real> &ph, int mat, int kind, Rng &g,
                                           BlockCounters *bc, Secondary<real> &sec) {
  if (kind == kCompton) return compton(s, ph, g, bc);
  if (kind == kPhoto) {
    ph.alive = 0;
    return ph.e;
  }
  if (kind == kRayleigh) {
    rayleigh(s, s.mat_comp[mat], ph, g, bc);
    return R<real>(0);
  }
  real ekin = ph.e - R<real>(2.0 * kMC2);
  real d[3];
  iso_dir(g, d);
  if (sec.has) {
    atomicAdd(&bc->stack_overflow, 1u);
  } else {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      sec.at(a) = ph.pos[a];
      sec.at(3 + a) = -d[a];
    }
    sec.has = 1;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) ph.dir[a] = d[a];
  set_energy(s, ph, R<real>(kMC2));
  atomicAdd(&bc->secondaries, 2u);
  return ekin;
}

// Interaction at ph.pos in material `mat`.  Returns the energy deposited
// locally (scored by the caller when inside the image).
template <typename real>
__device__ __forceinline__ real interact(const Scene<real> &s, Photon<real> &ph, int mat, Rng &g,
                                         BlockCounters *bc, Secondary<real> &sec, int *kind = nullptr) {
  const int k = select_kind(s, ph, mat, g);
  if (kind) *kind = k;
  return apply_kind(s, ph, mat, k, g, bc, sec);
}

template <typename real>
__device__ __forceinline__ void rot_apply(const real m[9], const real v[3], real o[3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    real a = m[3 * i] * v[0];
    a = a + m[3 * i + 1] * v[1];
    a = a + m[3 * i + 2] * v[2];
    o[i] = a;
  }
}

// Isotropic direction between the source's theta and phi bounds from two
// uniforms (GateSPSAngDistribution::GenerateIsotropicFlux).
template <typename real>
__device__ __forceinline__ void iso_direction(const Scene<real> &s, real u, real v, real d[3]) {
  real cost = s.s_cos_tmin - s.s_cos_tmax;
  cost = u * cost;
  cost = s.s_cos_tmin - cost;
  real st2 = cost * cost;
  st2 = R<real>(1) - st2;
  real sint = gg_sqrt(st2 > R<real>(0) ? st2 : R<real>(0));
  real f = s.s_dphi_turn * v;
  f = s.s_phi0_turn + f;
  f = f - gg_floor(f);
  real sp, cp;
  gg_sincos_turn(f, sp, cp);
  d[0] = -(sint * cp);
  d[1] = -(sint * sp);
  d[2] = -cost;
}

// Forced direction (GateForcedDirectionManager::SampleDirectionWithinCone):
// about the axis a of the history's head, u1 from the larger of |a_x|, |a_y|
// and u2 = a x u1 (both normalised); phi uniform (first draw), cos(theta)
// uniform in [cos max, cos min] (second draw).
template <typename real, typename G>
__device__ __forceinline__ void forced_direction(const Scene<real> &s, int run, int head, G &g, real d[3]) {
  const HeadFrame<real> f = head_frame(s, run, head);
  const real *a = f.u;
  real u1[3], u2[3];
  const real ax = a[0] < R<real>(0) ? -a[0] : a[0];
  const real ay = a[1] < R<real>(0) ? -a[1] : a[1];
  if (ax > ay) {
    u1[0] = a[2];
    u1[1] = R<real>(0);
    u1[2] = -a[0];
  } else {
    u1[0] = R<real>(0);
    u1[1] = -a[2];
    u1[2] = a[1];
  }
  real n = u1[0] * u1[0];
  n = n + u1[1] * u1[1];
  n = n + u1[2] * u1[2];
  n = R<real>(1) / gg_sqrt(n);
#pragma unroll
  for (int k = 0; k < 3; ++k) u1[k] = u1[k] * n;
  u2[0] = a[1] * u1[2] - a[2] * u1[1];
  u2[1] = a[2] * u1[0] - a[0] * u1[2];
  u2[2] = a[0] * u1[1] - a[1] * u1[0];
  n = u2[0] * u2[0];
  n = n + u2[1] * u2[1];
  n = n + u2[2] * u2[2];
  n = R<real>(1) / gg_sqrt(n);
#pragma unroll
  for (int k = 0; k < 3; ++k) u2[k] = u2[k] * n;
  const real v = u01<real>(g);
  real sp, cp;
  gg_sincos_turn(v, sp, cp);
  real c = s.s_fd_cmin - s.s_fd_cmax;
  c = u01<real>(g) * c;
  c = s.s_fd_cmax + c;
  real st = c * c;
  st = R<real>(1) - st;
  st = gg_sqrt(st > R<real>(0) ? st : R<real>(0));
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    real t = cp * u1[k];
    const real t2 = sp * u2[k];
    t = t + t2;
    t = st * t;
    d[k] = a[k] * c;
    d[k] = d[k] + t;
  }
}

template <typename real, typename G>
__device__ __forceinline__ void sample_direction(const Scene<real> &s, const real p[3], G &g, real d[3], int run = 0,
                                                 int head = 0) {
  if (s.dir_type == GG_DIR_FORCED) {
    forced_direction(s, run, head, g, d);
  } else if (s.dir_type == GG_DIR_ISO) {
    const real u = u01<real>(g);
    const real v = u01<real>(g);
    iso_direction(s, u, v, d);
  } else if (s.dir_type == GG_DIR_MOMENTUM) {
    d[0] = s.s_mom[0];
    d[1] = s.s_mom[1];
    d[2] = s.s_mom[2];
  } else {
    real v[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) v[a] = s.s_focus[a] - p[a];
    real n2 = v[0] * v[0];
    n2 = n2 + v[1] * v[1];
    n2 = n2 + v[2] * v[2];
    real rn = R<real>(1) / gg_sqrt(n2);
#pragma unroll
    for (int a = 0; a < 3; ++a) d[a] = v[a] * rn;
  }
}

template <typename real>
__device__ __forceinline__ bool accept_dir(const Scene<real> &s, const real p[3], const real d[3]) {
  for (int b = 0; b < s.n_accept; ++b) {
    const real *bx = s.acc_box + 6 * b;
    real lo[3] = {bx[0], bx[1], bx[2]};
    real hi[3] = {bx[3], bx[4], bx[5]};
    if (entry_distance(p, d, lo, hi) < gg_inf(real(0))) return true;
  }
  return false;
}

// Source position (GateSPSPosDistribution: point, box, sphere, disc, voxels).
template <typename real, typename G>
__device__ __forceinline__ void sample_position(const Scene<real> &s, G &g, Photon<real> &ph, BlockCounters *bc) {
  real loc[3] = {R<real>(0), R<real>(0), R<real>(0)};
  int pt = s.pos_type;
  if (pt == GG_POS_BOX) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      real u = R<real>(2) * u01<real>(g);
      u = u - R<real>(1);
      loc[a] = u * s.s_half[a];
    }
  } else if (pt == GG_POS_SPHERE || pt == GG_POS_DISC) {
    int it = 0;
    for (;;) {
      real r2 = R<real>(0);
      int na = (pt == GG_POS_SPHERE) ? 3 : 2;
      for (int a = 0; a < na; ++a) {
        real u = R<real>(2) * u01<real>(g);
        u = u - R<real>(1);
        real la = u * s.s_radius;
        if (a == 0) loc[0] = la;
        else if (a == 1) loc[1] = la;
        else loc[2] = la;
        r2 = r2 + la * la;
      }
      real rr = s.s_radius * s.s_radius;
      if (r2 <= rr) break;
      if (++it >= kLoopCap) {
        atomicAdd(&bc->loop_capped, 1u);
        break;
      }
    }
  }
  if (pt == GG_POS_VOXELS) {
    // GateSPSVoxelsPosDistribution::VGenerateOne: z, then y | z, then x | z, y;
    // lower_bound (first entry >= p) with p in (0, 1]
    int idx[3];
    const int len[3] = {s.vnz, s.vny, s.vnx};
#pragma unroll
    for (int lev = 0; lev < 3; ++lev) {
      const real *c = lev == 0   ? s.cdf_z
                      : lev == 1 ? s.cdf_y + (size_t)idx[0] * s.vny
                                 : s.cdf_x + ((size_t)idx[0] * s.vny + (size_t)idx[1]) * s.vnx;
      int k, it = 0;
      do {
        real p = u01_open0<real>(g);
        int lo = 0, hi = len[lev];
        while (lo < hi) {
          int mid = (lo + hi) >> 1;
          if (c[mid] < p) lo = mid + 1;
          else hi = mid;
        }
        k = lo;
        if (++it >= kLoopCap) {
          atomicAdd(&bc->loop_capped, 1u);
          if (k >= len[lev]) k = len[lev] - 1;
          break;
        }
      } while (k >= len[lev]);
      idx[lev] = k;
    }
    const int ind[3] = {idx[2], idx[1], idx[0]};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      real x = (real)ind[a] * s.v_sp[a];
      x = s.v_org[a] + x;
      real j = u01<real>(g) - R<real>(0.5);
      j = j * s.v_sp[a];
      ph.pos[a] = x + j;
    }
  } else {
    real off[3];
    rot_apply(s.s_rot, loc, off);
#pragma unroll
    for (int a = 0; a < 3; ++a) ph.pos[a] = s.s_t[a] + off[a];
  }
}

// Direction with the acceptance loop, one history.
template <typename real, typename G>
__device__ __forceinline__ int sample_direction_accepted(const Scene<real> &s, G &g, Photon<real> &ph,
                                                         BlockCounters *bc) {
  int tries = 0;
  for (;;) {
    sample_direction(s, ph.pos, g, ph.dir, ph.run, ph.head);
    if (s.n_accept == 0 || accept_dir(s, ph.pos, ph.dir)) break;
    atomicAdd(&bc->skipped, 1u);
    if (++tries > s.max_rejection) return GG_ERR_DOMAIN;
  }
  return GG_OK;
}

__device__ __forceinline__ uint32_t block_word(const uint4 &b, uint32_t w) {
  return w == 0 ? b.x : (w == 1 ? b.y : (w == 2 ? b.z : b.w));
}

// Words q and q + 1 (0-based counts of 32-bit draws) of a history's Philox
// stream: one block, or two when the pair straddles a block boundary.
__device__ __forceinline__ void stream_pair(const Rng &g, uint32_t q, uint32_t &x, uint32_t &y) {
  const uint4 b = philox_block(q >> 2, g.stream, g.h0, g.h1, g.k0, g.k1);
  x = block_word(b, q & 3u);
  if ((q & 3u) != 3u) {
    y = block_word(b, (q + 1u) & 3u);
  } else {
    const uint4 c = philox_block((q >> 2) + 1u, g.stream, g.h0, g.h1, g.k0, g.k1);
    y = c.x;
  }
}

// Isotropic directions with the acceptance loop for the histories of a warp
// together (every lane calls it; `need`: the lane's history wants a
// direction; its position is set and p0 words of its stream are drawn).
// Trial k of a history draws words p0 + 2k and p0 + 2k + 1, so trials can be
// evaluated out of order: each round deals the 32 lanes over the histories
// still waiting (lane l evaluates trial next + l / np of waiting history
// l % np) and every history takes its first accepted trial.  Results, draws
// and the rejection count per history equal those of
// sample_direction_accepted; the lanes stay converged instead of waiting for
// the warp's longest loop.  On return g stands after the accepted trial.
template <typename real>
__device__ __forceinline__ int warp_iso_direction_accepted(const Scene<real> &s, RngAhead &g, Photon<real> &ph,
                                                           bool need, BlockCounters *bc) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t p0 = (g.blk - 1u) * 4u + (uint32_t)g.idx;  // words drawn so far (Rng / RngAhead state)
  const uint32_t max_rej = (uint32_t)s.max_rejection;
  bool pending = need;
  uint32_t next = 0;  // first trial not yet evaluated
  int status = GG_OK;
  uint32_t k_acc = 0;
  for (;;) {
    const unsigned m = __ballot_sync(0xffffffffu, pending);
    if (m == 0u) break;
    const int np = __popc(m);
    const int r = (int)lane % np;
    const int owner = (int)__fns(m, 0u, r + 1);
    const uint32_t o_p0 = __shfl_sync(0xffffffffu, p0, owner);
    const uint32_t o_next = __shfl_sync(0xffffffffu, next, owner);
    Rng o = g;  // the owner's stream: key and counter words
    o.h0 = __shfl_sync(0xffffffffu, g.h0, owner);
    o.h1 = __shfl_sync(0xffffffffu, g.h1, owner);
    real op[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) op[a] = __shfl_sync(0xffffffffu, ph.pos[a], owner);
    const uint32_t q = o_p0 + 2u * (o_next + (uint32_t)((int)lane / np));
    uint32_t wu, wv;
    stream_pair(o, q, wu, wv);
    const real u = (real)(wu >> 8) * R<real>(5.9604644775390625e-08);
    const real v = (real)(wv >> 8) * R<real>(5.9604644775390625e-08);
    real d[3];
    iso_direction(s, u, v, d);
    const unsigned am = __ballot_sync(0xffffffffu, accept_dir(s, op, d));
    int src = (int)lane;
    bool won = false;
    if (pending) {
      const int rk = __popc(m & ((1u << lane) - 1u));  // this history's rank among the waiting ones
      unsigned grp = 0u;
      for (int l = rk; l < 32; l += np) grp |= 1u << l;
      const unsigned hits = am & grp;
      if (hits) {
        const int w = __ffs(hits) - 1;
        k_acc = next + (uint32_t)(w / np);
        src = w;
        won = true;
        pending = false;
        if (k_acc > max_rej) {
          status = GG_ERR_DOMAIN;
          k_acc = max_rej + 1u;
        }
      } else {
        next += (uint32_t)__popc(grp);
        if (next > max_rej) {
          status = GG_ERR_DOMAIN;
          k_acc = max_rej + 1u;
          pending = false;
        }
      }
    }
    // the winning lane's direction to the history's lane
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const real x = __shfl_sync(0xffffffffu, d[a], src);
      if (won) ph.dir[a] = x;
    }
  }
  if (!need) return GG_OK;
  if (k_acc) atomicAdd(&bc->skipped, k_acc);
  if (status != GG_OK) return status;
  // the stream after the accepted trial
  const uint32_t pe = p0 + 2u * (k_acc + 1u);
  g.ahead = false;
  if ((pe & 3u) == 0u) {
    g.blk = pe >> 2;
    g.idx = 4;
    g.buf[0] = g.buf[1] = g.buf[2] = g.buf[3] = 0u;
  } else {
    const uint4 b = philox_block(pe >> 2, g.stream, g.h0, g.h1, g.k0, g.k1);
    g.buf[0] = b.x;
    g.buf[1] = b.y;
    g.buf[2] = b.z;
    g.buf[3] = b.w;
    g.blk = (pe >> 2) + 1u;
    g.idx = (int)(pe & 3u);
  }
  return GG_OK;
}

template <typename real, typename G>
__device__ __forceinline__ void sample_energy(const Scene<real> &s, G &g, Photon<real> &ph) {
  real e;
  int et = s.ene_type;
  if (et == GG_ENE_MONO) {
    e = s.s_mono;
  } else if (et == GG_ENE_RANGE) {
    real w = s.s_ehi - s.s_elo;
    w = w * u01<real>(g);
    e = s.s_elo + w;
  } else {
    // first index with p < cdf[i] (the linear scan of
    // GateSPSEneDistribution::IndexForProbability), found by bisection on the
    // non-decreasing cumulative weights
    real p = u01<real>(g);
    int lo = 0, hi = s.n_spec - 1;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (p >= s.spec_cdf[mid]) lo = mid + 1;
      else hi = mid;
    }
    int i = lo;
    if (et == GG_ENE_LINES) {
      e = s.spec_e[i];
    } else {
      real a = s.spec_e[i];
      real w = s.spec_e[i + 1] - a;
      w = w * u01<real>(g);
      e = a + w;
    }
  }
  ph.alive = 1;
  ph.can_enter = 1;
  ph.in_image = 0;
  set_energy(s, ph, e);
}

// GateGenericSource::GeneratePrimaries order: position, direction (with the
// acceptance loop of GateSingleParticleSource::GenerateDirectionWithAA),
// energy.
template <typename real, typename G>
__device__ __forceinline__ int sample_primary(const Scene<real> &s, G &g, Photon<real> &ph, BlockCounters *bc) {
  sample_position(s, g, ph, bc);
  const int st = sample_direction_accepted(s, g, ph, bc);
  if (st != GG_OK) return st;
  sample_energy(s, g, ph);
  return GG_OK;
}

// Primary records written by k_generate and consumed by k_transport (SoA,
// one entry per history of the batch).  The state field says how the first
// transport iteration left the photon; the RNG position lets the transport
// kernel continue the history's Philox stream exactly where it stopped.
enum : uint32_t { kRecDead = 0, kRecInImage = 1, kRecPendingWorld = 2, kRecWorld = 3 };

template <typename real>
struct Records {
  uint4 *rng_buf;
  real *px, *py, *pz, *dx, *dy, *dz, *e;
  uint32_t *flags;    // bits 0-1 state, bit 2 steps already taken (0/1)
  uint32_t *rng_pos;  // block << 3 | index in buffer
  uint32_t *sim;      // simulation of the history (batched launches)

  __device__ __forceinline__ static Records carve(void *base, size_t cap) {
    Records r;
    unsigned char *p = reinterpret_cast<unsigned char *>(base);
    r.rng_buf = reinterpret_cast<uint4 *>(p);
    p += cap * sizeof(uint4);
    real **f[7] = {&r.px, &r.py, &r.pz, &r.dx, &r.dy, &r.dz, &r.e};
    for (int i = 0; i < 7; ++i) {
      *f[i] = reinterpret_cast<real *>(p);
      p += cap * sizeof(real);
    }
    r.flags = reinterpret_cast<uint32_t *>(p);
    p += cap * sizeof(uint32_t);
    r.rng_pos = reinterpret_cast<uint32_t *>(p);
    p += cap * sizeof(uint32_t);
    r.sim = reinterpret_cast<uint32_t *>(p);
    return r;
  }
};

// Lane states of the phase-batched transport loop.
enum : int { kDone = 0, kRefill = 1, kFly = 2, kInteract = 3 };

// Flight: one Woodcock tentative step in the image (followed, when it leaves
// the image box, by the world flight), or one free flight in the world.  A
// real collision is not handled here: the lane records it
// (material, voxel, scored) and waits in state kInteract until its warp runs
// an interaction phase.  Returns the lane's next state; kRefill means the
// photon died.
// pscored: what the pending interaction scores - 0 nothing (world), 1 the dose
// voxel pv, 2 the crystal of the current head, 3 nothing (collimator).
// Voxel of a point inside (or on the surface of) the image box.
template <typename real>
__device__ __forceinline__ uint32_t voxel_of(const Scene<real> &s, const real p[3]) {
  int ix = (int)((p[0] - s.bmin[0]) * s.inv_sp[0]);
  int iy = (int)((p[1] - s.bmin[1]) * s.inv_sp[1]);
  int iz = (int)((p[2] - s.bmin[2]) * s.inv_sp[2]);
  ix = ix < 0 ? 0 : (ix >= s.nx ? s.nx - 1 : ix);
  iy = iy < 0 ? 0 : (iy >= s.ny ? s.ny - 1 : iy);
  iz = iz < 0 ? 0 : (iz >= s.nz ? s.nz - 1 : iz);
  return (uint32_t)ix + (uint32_t)s.nx * ((uint32_t)iy + (uint32_t)s.ny * (uint32_t)iz);
}

// Voxel walk (Amanatides & Woo) of the straight path [p, p + len d) inside the
// image: visit(v, m, length) for every voxel v (material m) it crosses, in
// order; distance to the next boundary per axis, the nearest crossed first
// (ties: x, then y, then z).
template <typename real, typename Visit>
__device__ __forceinline__ void voxel_walk(const Scene<real> &s, const real p[3], const real d[3], real len,
                                           Visit &&visit) {
  const int n0 = s.nx, n1 = s.ny, n2 = s.nz;
  int i0 = (int)((p[0] - s.bmin[0]) * s.inv_sp[0]);
  int i1 = (int)((p[1] - s.bmin[1]) * s.inv_sp[1]);
  int i2 = (int)((p[2] - s.bmin[2]) * s.inv_sp[2]);
  i0 = i0 < 0 ? 0 : (i0 >= n0 ? n0 - 1 : i0);
  i1 = i1 < 0 ? 0 : (i1 >= n1 ? n1 - 1 : i1);
  i2 = i2 < 0 ? 0 : (i2 >= n2 ? n2 - 1 : i2);
  const real inf = gg_inf(real(0));
  real tn0 = inf, tn1 = inf, tn2 = inf, td0 = inf, td1 = inf, td2 = inf;
  int s0 = 0, s1 = 0, s2 = 0;
  // first boundary along one axis: (bmin + k sp - p) / d, k the next plane index
  auto first = [&](int a, int i, real pa, real da, real &tn, real &td, int &st) {
    if (da > R<real>(0)) {
      real b = (real)(i + 1) * s.sp[a];
      b = s.bmin[a] + b;
      b = b - pa;
      tn = b / da;
      td = s.sp[a] / da;
      st = 1;
    } else if (da < R<real>(0)) {
      real b = (real)i * s.sp[a];
      b = s.bmin[a] + b;
      b = b - pa;
      tn = b / da;
      td = -s.sp[a];
      td = td / da;
      st = -1;
    }
    if (tn < R<real>(0)) tn = R<real>(0);
  };
  first(0, i0, p[0], d[0], tn0, td0, s0);
  first(1, i1, p[1], d[1], tn1, td1, s1);
  first(2, i2, p[2], d[2], tn2, td2, s2);
  real tc = R<real>(0);
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
    if (seg > R<real>(0)) {
      const uint32_t v = (uint32_t)i0 + (uint32_t)n0 * ((uint32_t)i1 + (uint32_t)n1 * (uint32_t)i2);
      visit(v, (int)__ldg(s.labels + v), seg);
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

// Label gathers in flight per lane in the track-length estimator's walks.
constexpr int kTleGroup = 2;

template <typename real, int GROUP, typename Visit>
__device__ __forceinline__ void voxel_walk_grouped(const Scene<real> &s, const real p[3], const real d[3], real len,
                                                   Visit &&visit);

// Track-length estimator (GateTLEDoseActor::ScoreTLEDepositStep,
// core/opengate_core/opengate_lib/GateTLEDoseActor.cpp:249-299): the straight
// path [p, p + len d) of a photon of energy e (table index ei) scores
// e * mu_en(E, material) * length in every voxel it crosses.
template <typename real, int GROUP = kTleGroup>
__device__ __forceinline__ void tle_path(const Scene<real> &s, const real p[3], const real d[3], real len, real e,
                                         const EIdx<real> &ei, HistList<real> &l, const Tally<real> &t,
                                         BlockCounters *bc, unsigned int &n_dep) {
  voxel_walk_grouped<real, GROUP>(s, p, d, len, [&](uint32_t v, int m, real seg) {
    real mu = interp_row(s.muen + (size_t)s.mat_comp[m] * s.n_e, ei);
    mu = s.mat_rho[m] * mu;
    real ed = e * mu;
    ed = ed * seg;
    deposit(l, t, bc, v, ed, n_dep);
  });
}

// voxel_walk in groups of GROUP boundary crossings: the crossings of a group
// are computed first (voxel_walk's arithmetic, step for step), then their
// label gathers are issued together and visit() runs for each in walk order,
// so up to GROUP loads are in flight per lane instead of one and every
// visitor sees exactly voxel_walk's sequence.
template <typename real, int GROUP, typename Visit>
__device__ __forceinline__ void voxel_walk_grouped(const Scene<real> &s, const real p[3], const real d[3], real len,
                                                   Visit &&visit) {
  if constexpr (GROUP == 1) {
    voxel_walk(s, p, d, len, visit);
  } else {
    const int n0 = s.nx, n1 = s.ny, n2 = s.nz;
    int i0 = (int)((p[0] - s.bmin[0]) * s.inv_sp[0]);
    int i1 = (int)((p[1] - s.bmin[1]) * s.inv_sp[1]);
    int i2 = (int)((p[2] - s.bmin[2]) * s.inv_sp[2]);
    i0 = i0 < 0 ? 0 : (i0 >= n0 ? n0 - 1 : i0);
    i1 = i1 < 0 ? 0 : (i1 >= n1 ? n1 - 1 : i1);
    i2 = i2 < 0 ? 0 : (i2 >= n2 ? n2 - 1 : i2);
    const real inf = gg_inf(real(0));
    real tn[3] = {inf, inf, inf}, td[3] = {inf, inf, inf};
    int st[3] = {0, 0, 0};
    const int ii[3] = {i0, i1, i2};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const real da = d[a];
      if (da > R<real>(0)) {
        real b = (real)(ii[a] + 1) * s.sp[a];
        b = s.bmin[a] + b;
        b = b - p[a];
        tn[a] = b / da;
        td[a] = s.sp[a] / da;
        st[a] = 1;
      } else if (da < R<real>(0)) {
        real b = (real)ii[a] * s.sp[a];
        b = s.bmin[a] + b;
        b = b - p[a];
        tn[a] = b / da;
        td[a] = -s.sp[a];
        td[a] = td[a] / da;
        st[a] = -1;
      }
      if (tn[a] < R<real>(0)) tn[a] = R<real>(0);
    }
    real tn0 = tn[0], tn1 = tn[1], tn2 = tn[2];
    const real td0 = td[0], td1 = td[1], td2 = td[2];
    const int s0 = st[0], s1 = st[1], s2 = st[2];
    real tc = R<real>(0);
    const int cap = n0 + n1 + n2 + 3;
    int k = 0;
    bool go = true;
    while (go) {
      uint32_t vv[GROUP];
      real sg[GROUP];
      bool ok[GROUP];
#pragma unroll
      for (int j = 0; j < GROUP; ++j) {
        ok[j] = false;
        vv[j] = 0u;
        sg[j] = R<real>(0);
        if (go && k < cap) {
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
          if (seg > R<real>(0)) {
            vv[j] = (uint32_t)i0 + (uint32_t)n0 * ((uint32_t)i1 + (uint32_t)n1 * (uint32_t)i2);
            sg[j] = seg;
            ok[j] = true;
          }
          tc = te;
          ++k;
          if (!(tc < len)) {
            go = false;
          } else if (a == 0) {
            i0 += s0;
            if (i0 < 0 || i0 >= n0) go = false;
            tn0 = tn0 + td0;
          } else if (a == 1) {
            i1 += s1;
            if (i1 < 0 || i1 >= n1) go = false;
            tn1 = tn1 + td1;
          } else {
            i2 += s2;
            if (i2 < 0 || i2 >= n2) go = false;
            tn2 = tn2 + td2;
          }
        } else {
          go = false;
        }
      }
      int lab[GROUP];
#pragma unroll
      for (int j = 0; j < GROUP; ++j) lab[j] = ok[j] ? (int)__ldg(s.labels + vv[j]) : 0;
#pragma unroll
      for (int j = 0; j < GROUP; ++j)
        if (ok[j]) visit(vv[j], lab[j], sg[j]);
    }
  }
}

// Optical depth of the straight path [p, p + len d) inside the image:
// sum of mu(E, material) * length over the voxels it crosses (GROUP: label
// gathers in flight per lane, voxel_walk_grouped).
template <typename real, int GROUP>
__device__ __forceinline__ real image_depth(const Scene<real> &s, const real p[3], const real d[3], real len,
                                           const EIdx<real> &ei) {
  real tau = R<real>(0);
  voxel_walk_grouped<real, GROUP>(s, p, d, len, [&](uint32_t, int m, real seg) {
    real mu = interp_row(s.sig + (size_t)s.mat_comp[m] * s.n_e, ei);
    mu = s.mat_rho[m] * mu;
    mu = mu * seg;
    tau = tau + mu;
  });
  return tau;
}

// Scoring state handed to the flights of the track-length estimator.
template <typename real>
struct TleScore {
  HistList<real> *l;
  const Tally<real> *t;
  unsigned int *n_dep;
};

// One Woodcock tentative step of a photon inside the image box.  With TLE, a
// photon at or below the estimator's threshold first stops (depositing its
// energy in its voxel) when at or below the kill energy, else scores the
// path of the step.
template <typename real, bool TLE = false>
__device__ __forceinline__ int image_flight(const Scene<real> &s, Photon<real> &ph, Rng &g, int &pmat, uint32_t &pv,
                                            int &pscored, unsigned int &n_wood, unsigned int &n_real,
                                            BlockCounters *bc = nullptr, TleScore<real> sc = {nullptr, nullptr, nullptr}) {
  {
    if constexpr (TLE) {
      if (ph.e <= s.tle_thr && ph.e <= s.tle_emin) {
        deposit(*sc.l, *sc.t, bc, voxel_of(s, ph.pos), ph.e, *sc.n_dep);
        ph.alive = 0;
        return kRefill;
      }
    }
    real u = u01_open0<real>(g);
    real sd = -gg_log(u);
    sd = sd * ph.inv_mumax;
    if constexpr (TLE) {
      if (ph.e <= s.tle_thr)
        tle_path(s, ph.pos, ph.dir, sd < ph.t_exit ? sd : ph.t_exit, ph.e, ph.ei, *sc.l, *sc.t, bc, *sc.n_dep);
    }
    if (sd >= ph.t_exit) {
#pragma unroll
      for (int a = 0; a < 3; ++a) ph.pos[a] = ph.pos[a] + ph.t_exit * ph.dir[a];
      ph.in_image = 0;
      ph.can_enter = 0;
      ph.exclude = 0;
      return kFly;
    }
    ph.t_exit = ph.t_exit - sd;
#pragma unroll
    for (int a = 0; a < 3; ++a) ph.pos[a] = ph.pos[a] + sd * ph.dir[a];
    ++n_wood;
    const uint32_t v = voxel_of(s, ph.pos);
    int m = __ldg(s.labels + v);
    real mu = interp_row(s.sig + (size_t)s.mat_comp[m] * s.n_e, ph.ei);
    mu = s.mat_rho[m] * mu;
    real u2 = u01<real>(g);
    if (u2 * ph.mumax >= mu) return kFly;
    ++n_real;
    pmat = m;
    pv = v;
    pscored = 1;
    return kInteract;
  }
}

template <typename real, bool SPECT, bool TLE = false>
__device__ __forceinline__ int flight(const Scene<real> &s, Photon<real> &ph, Rng &g, BlockCounters *bc, int &pmat,
                                      uint32_t &pv, int &pscored, unsigned int &n_wood, unsigned int &n_real,
                                      unsigned int &n_world, unsigned int &n_head,
                                      TleScore<real> sc = {nullptr, nullptr, nullptr}) {
  if (++ph.steps > kStepCap) {
    atomicAdd(&bc->loop_capped, 1u);
    ph.alive = 0;
    return kRefill;
  }
  if (ph.in_image) {
    const int r = image_flight<real, TLE>(s, ph, g, pmat, pv, pscored, n_wood, n_real, bc, sc);
    if constexpr (SPECT) return r;
    if (r != kFly || ph.in_image) return r;
    // Left the image box: take the world step at once (the same flight
    // count and draws as a separate phase, one block iteration fewer).
    if (++ph.steps > kStepCap) {
      atomicAdd(&bc->loop_capped, 1u);
      ph.alive = 0;
      return kRefill;
    }
  }
  if constexpr (SPECT) {
    if (ph.in_head) {
      ++n_head;
      int mat;
      if (head_flight(s, ph, g, mat)) {
        pmat = mat;
        pscored = ph.hreg == s.hreg_cr ? 2 : 3;
        return kInteract;
      }
      return ph.alive ? kFly : kRefill;  // (stopped by a shielded side)
    }
    ++n_world;
    if (spect_world_flight(s, ph, g)) {
      pmat = s.world_mat;
      pscored = 0;
      return kInteract;
    }
    if (!ph.alive) {
      atomicAdd(&bc->escaped, 1u);
      return kRefill;
    }
    return kFly;
  }
  ++n_world;
  real inf = gg_inf(real(0));
  real tin = ph.can_enter ? entry_distance(ph.pos, ph.dir, s.bmin, s.bmax) : inf;
  real wlo[3] = {-s.whalf[0], -s.whalf[1], -s.whalf[2]};
  real tout = exit_distance(ph.pos, ph.dir, wlo, s.whalf);
  int wm = s.world_mat;
  real mu = interp_row(s.sig + (size_t)s.mat_comp[wm] * s.n_e, ph.ei);
  mu = s.mat_rho[wm] * mu;
  real u = u01_open0<real>(g);
  real sd = -gg_log(u);
  sd = sd / mu;
  if (sd < tin && sd < tout) {
#pragma unroll
    for (int a = 0; a < 3; ++a) ph.pos[a] = ph.pos[a] + sd * ph.dir[a];
    pmat = wm;
    pscored = 0;
    return kInteract;
  }
  if (tin <= tout) {
#pragma unroll
    for (int a = 0; a < 3; ++a) ph.pos[a] = ph.pos[a] + tin * ph.dir[a];
    ph.in_image = 1;
    ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
    return kFly;
  }
  ph.alive = 0;
  atomicAdd(&bc->escaped, 1u);
  return kRefill;
}

// A crystal hit of head H added to the event (GateDigiAdderInVolume::Update,
// digitizer/GateDigiAdderInVolume.cpp:29-72): energy sum, and either the
// energy-winner position or (s.centroid) the energy-weighted position sum.
template <typename real, int H>
__device__ __forceinline__ void event_add(const Scene<real> &s, Event<real> &ev, const Photon<real> &ph, real ed) {
  ev.esum[H] = ev.esum[H] + ed;
  if (s.centroid) {
    ev.wpos[H][0] = ev.wpos[H][0] + ed * ph.pos[0];
    ev.wpos[H][1] = ev.wpos[H][1] + ed * ph.pos[1];
    ev.w[H] = ph.w;  // the last hit's weight
  } else if (ed > ev.emax[H]) {
    ev.emax[H] = ed;
    ev.wpos[H][0] = ph.pos[0];
    ev.wpos[H][1] = ph.pos[1];
    ev.w[H] = ph.w;  // the winner hit's weight
  }
}

// With TLE, the energy a photon at or below the estimator's threshold gives
// to electrons is not scored (GateTLEDoseActor.cpp:236-243: secondaries of a
// track-length-scored photon deposit nothing); its path scores instead.
template <typename real, bool SPECT, bool TLE = false>
__device__ __forceinline__ int do_interaction(const Scene<real> &s, Photon<real> &ph, Rng &g, BlockCounters *bc,
                                              int pmat, uint32_t pv, int pscored, HistList<real> &l,
                                              const Tally<real> &t, Secondary<real> &sec, unsigned int &n_dep,
                                              Event<real> &ev, int *kind = nullptr) {
  const real e_pre = ph.e;
  real ed = interact(s, ph, pmat, g, bc, sec, kind);
  if (pscored == 1) {
    if constexpr (!SPECT) {
      if (!TLE || e_pre > s.tle_thr) deposit(l, t, bc, pv, ed, n_dep);
    }
    if (ph.alive && ph.in_image) ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
  } else if (pscored == 0) {
    ph.can_enter = 1;
    ph.exclude = -1;
  } else if constexpr (SPECT) {
    if (pscored == 2 && ed > R<real>(0)) {
      if (ph.head == 0) event_add<real, 0>(s, ev, ph, ed);
      else event_add<real, 1>(s, ev, ph, ed);
    }
  }
  return ph.alive ? kFly : kRefill;
}

// Voxel of point p in the dose grid (Scene::dgrid); false outside the grid.
template <typename real>
__device__ __forceinline__ bool dose_voxel(const Scene<real> &s, const real p[3], uint32_t &v) {
  real f[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    real d = p[a] - s.dcorner[a];
    f[a] = d * s.dinv_sp[a];
  }
  if (!(f[0] >= R<real>(0)) || !(f[1] >= R<real>(0)) || !(f[2] >= R<real>(0))) return false;
  if (!(f[0] < (real)s.dnx) || !(f[1] < (real)s.dny) || !(f[2] < (real)s.dnz)) return false;
  int ix = (int)f[0], iy = (int)f[1], iz = (int)f[2];
  if (ix >= s.dnx || iy >= s.dny || iz >= s.dnz) return false;
  v = (uint32_t)ix + (uint32_t)s.dnx * ((uint32_t)iy + (uint32_t)s.dny * (uint32_t)iz);
  return true;
}

// do_interaction of the dose path with the tally on its own grid
// (GateDoseActor::SteppingAction, GateDoseActor.cpp:180-243: the deposit is
// scored in the dose-grid voxel of the interaction point, when there is one;
// DG 2: also edep * rho_min / rho of the material there in the dose list ld).
template <typename real, int DG>
__device__ __forceinline__ int do_interaction_grid(const Scene<real> &s, Photon<real> &ph, Rng &g, BlockCounters *bc,
                                                   int pmat, int pscored, HistList<real> &l, HistList<real> &ld,
                                                   const Tally<real> &t, const Tally<real> &td,
                                                   Secondary<real> &sec, unsigned int &n_dep, BlockCounters *bcd) {
  const real ed = interact(s, ph, pmat, g, bc, sec);
  if (pscored == 1) {
    uint32_t dv;
    if (dose_voxel(s, ph.pos, dv)) {
      deposit(l, t, bc, dv, ed, n_dep);
      if constexpr (DG == 2) {
        real dd = ed * s.drho_min;
        dd = dd / s.mat_rho[pmat];
        unsigned int nd = 0;
        deposit(ld, td, bcd, dv, dd, nd);
      }
    }
    if (ph.alive && ph.in_image) ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
  } else if (pscored == 0) {
    ph.can_enter = 1;
    ph.exclude = -1;
  }
  return ph.alive ? kFly : kRefill;
}

template <typename real>
__device__ __forceinline__ void pop_secondary(const Scene<real> &s, Photon<real> &ph, Secondary<real> &sec) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    ph.pos[a] = sec.at(a);
    ph.dir[a] = sec.at(3 + a);
  }
  sec.has = 0;
  ph.alive = 1;
  set_energy(s, ph, R<real>(kMC2));
  start_photon(s, ph);
}

// Batched launches: the lane's scene geometry, source and tally pointers
// become those of simulation d (bound once per history; the rest of the
// transport code then runs unchanged).
template <typename real>
__device__ __forceinline__ void bind_geometry(Scene<real> &s, const SimDesc<real> &d, const uint16_t *labels_base,
                                              const real *maj) {
  s.maj = maj;  // the simulation's own majorant: its Woodcock steps equal those of a run alone
  s.nx = d.nx;
  s.ny = d.ny;
  s.nz = d.nz;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    s.bmin[a] = d.bmin[a];
    s.bmax[a] = d.bmax[a];
    s.inv_sp[a] = d.inv_sp[a];
  }
  s.labels = labels_base + d.vox_off;
}

template <typename real>
__device__ __forceinline__ void bind_source(Scene<real> &s, const SimDesc<real> &d) {
  s.pos_type = d.pos_type;
  s.dir_type = d.dir_type;
  s.ene_type = d.ene_type;
  s.n_accept = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    s.s_t[a] = d.s_t[a];
    s.s_half[a] = d.s_half[a];
    s.s_mom[a] = d.s_mom[a];
    s.s_focus[a] = d.s_focus[a];
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) s.s_rot[k] = d.s_rot[k];
  s.s_radius = d.s_radius;
  s.s_mono = d.s_mono;
  s.s_elo = d.s_elo;
  s.s_ehi = d.s_ehi;
  s.s_cos_tmin = d.s_cos_tmin;
  s.s_cos_tmax = d.s_cos_tmax;
  s.s_phi0_turn = d.s_phi0_turn;
  s.s_dphi_turn = d.s_dphi_turn;
}

// Simulation containing batch history h (binary search over the ranges).
template <typename real>
__device__ __forceinline__ int find_sim(const SimDesc<real> *sims, int n_sims, uint64_t h) {
  int lo = 0, hi = n_sims - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sims[mid].h_begin <= h) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

}  // namespace gg
