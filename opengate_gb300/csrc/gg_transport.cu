// gg_transport.cu - photon transport through a voxelised image with DoseActor scoring.
//
// Replaces, for photons in a voxelised volume, Geant4's stepping through the
// replica/parameterised voxels of ImageVolume
// (opengate/geometry/volumes.py:1093-1125, GateImageNestedParameterisation.cpp:47-75)
// and the scoring of GateDoseActor::SteppingAction / ScoreSquaredValue /
// FlushSquaredValues (core/opengate_core/opengate_lib/GateDoseActor.cpp:180-243, 359-397).
//
// Kernel design (one GB300, one process):
//   * persistent grid, one photon history per thread at a time; a warp claims
//     histories from a global counter in chunks (one atomic per chunk) and
//     hands them to its lanes as they finish (ballot + popc), so no lane idles
//     while work remains;
//   * Woodcock (delta) tracking against a per-energy majorant inside the image
//     box; analytic free flight in the world material outside it;
//   * the majorant, total attenuation rows and the label->(composition,
//     density) table are staged in shared memory; labels are read through the
//     read-only path (the image is L2-resident up to ~60 M voxels);
//   * every history keeps its deposits in a register list of (voxel, sum);
//     when the history ends each entry adds round(sum * 2^32) to the edep tally
//     and round(sum^2 * 2^32) to the edep-squared tally with 64-bit integer
//     atomics: the history-by-history squared sum of GateDoseActor, order
//     independent and therefore bit-reproducible;
//   * a second kernel flushes the per-batch fixed-point tallies into the
//     float64 images (and clears them), one voxel per thread, coalesced.
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_device.cuh"
#include "gg_internal.h"
#include "gg_spect.cuh"

namespace gg {

template <typename real>
struct HistList {
  uint32_t vox[kHistList];
  real acc[kHistList];
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
// exact square q^2 (units of 2^-64 MeV^2, up to 2^74) goes to the 128-bit
// accumulator acc_e2[2v] (low word) / acc_e2[2v+1] (high word), the carry out
// of the low word moving to the high word.  Integer sums do not depend on the
// order of the atomics, and a voxel hit by one history has edep^2 == edep * edep
// exactly in these units.
template <typename real>
__device__ __forceinline__ void hlist_flush(HistList<real> &l, const Tally<real> &t, BlockCounters *bc) {
#pragma unroll
  for (int k = 0; k < kHistList; ++k) {
    if (k < l.n) {
      const unsigned long long q = (unsigned long long)to_fixed(l.acc[k]);
      const uint32_t v = l.vox[k];
      atomicAdd(&t.acc_e[v], q);
      if (t.acc_e2) {
        const unsigned long long lo = q * q;
        unsigned long long hi = __umul64hi(q, q);
        const unsigned long long old = atomicAdd(&t.acc_e2[2 * (size_t)v], lo);
        hi += (old + lo < old) ? 1ull : 0ull;
        if (hi) atomicAdd(&t.acc_e2[2 * (size_t)v + 1], hi);
      }
    }
  }
  if (l.n) atomicAdd(&bc->tally_entries, (unsigned int)l.n);
  l.n = 0;
}

template <typename real>
__device__ __forceinline__ void deposit(HistList<real> &l, const Tally<real> &t, BlockCounters *bc,
                                        uint32_t v, real e, unsigned int &n_dep) {
  if (!(e > R<real>(0))) return;
  ++n_dep;
  bool found = false;
#pragma unroll
  for (int k = 0; k < kHistList; ++k) {
    if (!found && k < l.n && l.vox[k] == v) {
      l.acc[k] = l.acc[k] + e;
      found = true;
    }
  }
  if (found) return;
  if (l.n == kHistList) {
    atomicAdd(&bc->list_overflows, 1u);
    hlist_flush(l, t, bc);
  }
#pragma unroll
  for (int k = 0; k < kHistList; ++k) {
    if (k == l.n) {
      l.vox[k] = v;
      l.acc[k] = e;
    }
  }
  l.n++;
}

// Klein-Nishina (G4KleinNishinaCompton sampling of the Physics Reference Manual)
template <typename real>
__device__ __forceinline__ real compton(const Scene<real> &s, Photon<real> &ph, Rng &g, BlockCounters *bc) {
  real e = ph.e;
  real k = e * R<real>(1.0 / kMC2);
  real twok = R<real>(2) * k;
  real eps0 = R<real>(1) / (R<real>(1) + twok);
  real eps0sq = eps0 * eps0;
  real alpha1 = -gg_log(eps0);
  real alpha2 = R<real>(1) - eps0sq;
  alpha2 = R<real>(0.5) * alpha2;
  alpha2 = alpha1 + alpha2;
  real eps, epssq, onecost, sint2;
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
__device__ __forceinline__ void rayleigh(const Scene<real> &s, int comp, Photon<real> &ph, Rng &g,
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
  real st2 = cost * cost;
  st2 = R<real>(1) - st2;
  real sint = gg_sqrt(st2 > R<real>(0) ? st2 : R<real>(0));
  real sp, cp;
  gg_sincos_turn(u01<real>(g), sp, cp);
  rotate_dir(ph.dir[0], ph.dir[1], ph.dir[2], cost, sint, cp, sp);
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

// Interaction at ph.pos in material `mat`.  Returns the energy deposited
// locally (scored by the caller when inside the image).
template <typename real>
__device__ __forceinline__ real interact(const Scene<real> &s, Photon<real> &ph, int mat, Rng &g,
                                         BlockCounters *bc, Secondary<real> &sec) {
  int c = s.mat_comp[mat];
  const real *cu = s.cum + (size_t)c * 3 * s.n_e;
  real r = u01<real>(g);
  real fc = interp_row(cu, ph.ei);
  if (r < fc) return compton(s, ph, g, bc);
  real fp = interp_row(cu + s.n_e, ph.ei);
  if (r < fp) {
    ph.alive = 0;
    return ph.e;
  }
  real fr = interp_row(cu + 2 * s.n_e, ph.ei);
  if (r < fr) {
    rayleigh(s, c, ph, g, bc);
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

template <typename real>
__device__ __forceinline__ void sample_direction(const Scene<real> &s, const real p[3], Rng &g, real d[3]) {
  if (s.dir_type == GG_DIR_ISO) {
    real u = u01<real>(g);
    real cost = s.s_cos_tmin - s.s_cos_tmax;
    cost = u * cost;
    cost = s.s_cos_tmin - cost;
    real st2 = cost * cost;
    st2 = R<real>(1) - st2;
    real sint = gg_sqrt(st2 > R<real>(0) ? st2 : R<real>(0));
    real f = s.s_dphi_turn * u01<real>(g);
    f = s.s_phi0_turn + f;
    f = f - gg_floor(f);
    real sp, cp;
    gg_sincos_turn(f, sp, cp);
    d[0] = -(sint * cp);
    d[1] = -(sint * sp);
    d[2] = -cost;
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

// GateGenericSource::GeneratePrimaries order: position, direction (with the
// acceptance loop of GateSingleParticleSource::GenerateDirectionWithAA),
// energy.
template <typename real>
__device__ __forceinline__ int sample_primary(const Scene<real> &s, Rng &g, Photon<real> &ph, BlockCounters *bc) {
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
  int tries = 0;
  for (;;) {
    sample_direction(s, ph.pos, g, ph.dir);
    if (s.n_accept == 0 || accept_dir(s, ph.pos, ph.dir)) break;
    atomicAdd(&bc->skipped, 1u);
    if (++tries > s.max_rejection) return GG_ERR_DOMAIN;
  }
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
    return r;
  }
};

// Source stage: one thread per history.  Samples the primary
// (GateGenericSource::GeneratePrimaries order), places it, and performs the
// first transport iteration when the photon starts in the world (free flight
// to the image, to an air interaction, or out of the world).
template <typename real>
__global__ void __launch_bounds__(256) k_generate(Scene<real> s, KernelArgs a) {
  __shared__ BlockCounters bc;
  __shared__ unsigned int n_world;
  if (threadIdx.x == 0) {
    bc = BlockCounters{0, 0, 0, 0, 0, 0, 0, 0};
    n_world = 0;
  }
  __syncthreads();
  const uint64_t n = a.h_end - a.h_begin;
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    Records<real> rec = Records<real>::carve(a.records, a.rec_cap);
    Rng g;
    g.init(a.seed, a.h_begin + i, 0u);
    Photon<real> ph;
    uint32_t state = kRecDead, steps = 0;
    int st = sample_primary(s, g, ph, &bc);
    if (st != GG_OK) {
      atomicOr(a.status, (unsigned int)st);
    } else {
      atomicAdd(&bc.histories, 1u);
      start_photon(s, ph);
      if (ph.in_image) {
        state = kRecInImage;
      } else if (s.spect) {
        state = kRecWorld;  // the world step also targets the heads: left to the transport stage
      } else {
        steps = 1;
        atomicAdd(&n_world, 1u);
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
          for (int k = 0; k < 3; ++k) ph.pos[k] = ph.pos[k] + sd * ph.dir[k];
          state = kRecPendingWorld;
        } else if (tin <= tout) {
#pragma unroll
          for (int k = 0; k < 3; ++k) ph.pos[k] = ph.pos[k] + tin * ph.dir[k];
          state = kRecInImage;
        } else {
          atomicAdd(&bc.escaped, 1u);
        }
      }
    }
    rec.px[i] = ph.pos[0];
    rec.py[i] = ph.pos[1];
    rec.pz[i] = ph.pos[2];
    rec.dx[i] = ph.dir[0];
    rec.dy[i] = ph.dir[1];
    rec.dz[i] = ph.dir[2];
    rec.e[i] = ph.e;
    rec.flags[i] = state | (steps << 2);
    rec.rng_pos[i] = (g.blk << 3) | (uint32_t)g.idx;
    rec.rng_buf[i] = make_uint4(g.buf[0], g.buf[1], g.buf[2], g.buf[3]);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long *cnt = a.counters;
    if (bc.histories) atomicAdd(&cnt[GG_CNT_HISTORIES], (unsigned long long)bc.histories);
    if (bc.skipped) atomicAdd(&cnt[GG_CNT_SKIPPED], (unsigned long long)bc.skipped);
    if (bc.escaped) atomicAdd(&cnt[GG_CNT_ESCAPED], (unsigned long long)bc.escaped);
    if (bc.loop_capped) atomicAdd(&cnt[GG_CNT_LOOP_CAPPED], (unsigned long long)bc.loop_capped);
    if (n_world) atomicAdd(&cnt[GG_CNT_WORLD_STEPS], (unsigned long long)n_world);
  }
}

// Lane states of the phase-batched transport loop.
enum : int { kDone = 0, kRefill = 1, kFly = 2, kInteract = 3 };

// Flight: one Woodcock tentative step in the image, or one free flight in the
// world.  A real collision is not handled here: the lane records it
// (material, voxel, scored) and waits in state kInteract until its warp runs
// an interaction phase.  Returns the lane's next state; kRefill means the
// photon died.
// pscored: what the pending interaction scores - 0 nothing (world), 1 the dose
// voxel pv, 2 the crystal of the current head, 3 nothing (collimator).
template <typename real, bool SPECT>
__device__ __forceinline__ int flight(const Scene<real> &s, Photon<real> &ph, Rng &g, BlockCounters *bc, int &pmat,
                                      uint32_t &pv, int &pscored, unsigned int &n_wood, unsigned int &n_real,
                                      unsigned int &n_world, unsigned int &n_head) {
  if (++ph.steps > kStepCap) {
    atomicAdd(&bc->loop_capped, 1u);
    ph.alive = 0;
    return kRefill;
  }
  if (ph.in_image) {
    real u = u01_open0<real>(g);
    real sd = -gg_log(u);
    sd = sd * ph.inv_mumax;
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
    int ix = (int)((ph.pos[0] - s.bmin[0]) * s.inv_sp[0]);
    int iy = (int)((ph.pos[1] - s.bmin[1]) * s.inv_sp[1]);
    int iz = (int)((ph.pos[2] - s.bmin[2]) * s.inv_sp[2]);
    ix = ix < 0 ? 0 : (ix >= s.nx ? s.nx - 1 : ix);
    iy = iy < 0 ? 0 : (iy >= s.ny ? s.ny - 1 : iy);
    iz = iz < 0 ? 0 : (iz >= s.nz ? s.nz - 1 : iz);
    uint32_t v = (uint32_t)ix + (uint32_t)s.nx * ((uint32_t)iy + (uint32_t)s.ny * (uint32_t)iz);
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
  if constexpr (SPECT) {
    if (ph.in_head) {
      ++n_head;
      int mat;
      if (head_flight(s, ph, g, mat)) {
        pmat = mat;
        pscored = ph.hreg == 2 ? 2 : 3;
        return kInteract;
      }
      return kFly;
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

// The interaction a lane recorded during its last flight.
template <typename real, int H>
__device__ __forceinline__ void event_add(const Scene<real> &s, Event<real> &ev, const Photon<real> &ph, real ed) {
  ev.esum[H] = ev.esum[H] + ed;
  if (ed > ev.emax[H]) {
    real p[3], dd[3];
    to_world(s, H, ph.pos, ph.dir, p, dd);
    ev.emax[H] = ed;
    ev.wpos[H][0] = p[0];
    ev.wpos[H][1] = p[1];
    ev.wpos[H][2] = p[2];
  }
}

template <typename real, bool SPECT>
__device__ __forceinline__ int do_interaction(const Scene<real> &s, Photon<real> &ph, Rng &g, BlockCounters *bc,
                                              int pmat, uint32_t pv, int pscored, HistList<real> &l,
                                              const Tally<real> &t, Secondary<real> &sec, unsigned int &n_dep,
                                              Event<real> &ev) {
  real ed = interact(s, ph, pmat, g, bc, sec);
  if (pscored == 1) {
    if constexpr (!SPECT) deposit(l, t, bc, pv, ed, n_dep);
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

// Transport stage.  Persistent grid; each lane carries one history at a time
// and is in one of the states kRefill (needs a history), kFly (next event is
// a flight) or kInteract (a collision is pending).  Every iteration the warp
// picks ONE phase by ballot - refill when at least refill_min lanes wait for a
// history, interact when at least interact_min collisions are pending,
// otherwise fly - and only the lanes in that state execute it.  Expensive
// code (source-record loads, tally flushes, Compton sampling) therefore runs
// with many lanes active instead of one lane at a time, while the order of
// operations inside each history, and hence its result, is unchanged.
// MINB = resident blocks per SM the register budget is sized for.
// SPECT selects the head transport and projection scoring instead of the dose tally.
template <typename real, int MINB, bool SPECT>
__global__ void __launch_bounds__(256, MINB) k_transport(Scene<real> sg, KernelArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ BlockCounters bc;
  __shared__ real sec_store[6 * 256];
  // ---- stage tables in shared memory --------------------------------------
  Scene<real> s = sg;
  {
    real *sh = reinterpret_cast<real *>(smem_raw);
    const int nsig = sg.n_comp * sg.n_e;
    real *ssig = sh;
    real *smaj = ssig + nsig;
    real *srho = smaj + sg.n_e;
    int *scomp = reinterpret_cast<int *>(srho + sg.n_mat);
    for (int i = threadIdx.x; i < nsig; i += blockDim.x) ssig[i] = sg.sig[i];
    for (int i = threadIdx.x; i < sg.n_e; i += blockDim.x) smaj[i] = sg.maj[i];
    for (int i = threadIdx.x; i < sg.n_mat; i += blockDim.x) {
      srho[i] = sg.mat_rho[i];
      scomp[i] = sg.mat_comp[i];
    }
    if (threadIdx.x == 0) bc = BlockCounters{0, 0, 0, 0, 0, 0, 0, 0};
    __syncthreads();
    s.sig = ssig;
    s.maj = smaj;
    s.mat_rho = srho;
    s.mat_comp = scomp;
  }
  const Records<real> rec = Records<real>::carve(args.records, args.rec_cap);
  Tally<real> t{args.acc_e, args.acc_e2};
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  const uint64_t n_hist = args.h_end - args.h_begin;
  // warp-uniform pool of claimed history offsets [pool_next, pool_end)
  uint64_t pool_next = 0, pool_end = 0;

  Photon<real> ph;
  ph.alive = 0;
  Secondary<real> sec;
  sec.base = sec_store;
  sec.stride = blockDim.x;
  sec.tid = threadIdx.x;
  sec.has = 0;
  HistList<real> l;
  l.n = 0;
  Event<real> ev;
  ev.clear();
  Rng g;
  int state = kRefill;
  bool in_hist = false;
  int pmat = 0, pscored = 0;
  uint32_t pv = 0;
  unsigned int n_wood = 0, n_real = 0, n_dep = 0, n_world = 0, n_head = 0, n_singles = 0;

  for (;;) {
    const unsigned m_ref = __ballot_sync(0xffffffffu, state == kRefill);
    const unsigned m_fly = __ballot_sync(0xffffffffu, state == kFly);
    const unsigned m_int = __ballot_sync(0xffffffffu, state == kInteract);
    if ((m_ref | m_fly | m_int) == 0u) break;
    int phase;
    if (__popc(m_ref) >= args.refill_min || (m_fly | m_int) == 0u) phase = kRefill;
    else if (__popc(m_int) >= args.interact_min || m_fly == 0u) phase = kInteract;
    else phase = kFly;

    if (phase == kRefill) {
      const bool need = state == kRefill;
      if (need && in_hist) {
        if constexpr (SPECT) n_singles += score_singles(s, ev);
        else hlist_flush(l, t, &bc);
        in_hist = false;
      }
      const unsigned n_need = __popc(m_ref);
      const unsigned rank = __popc(m_ref & lt_mask);
      const uint64_t avail = pool_end - pool_next;
      uint64_t h;
      if (avail >= n_need) {
        h = pool_next + rank;
        pool_next += n_need;
      } else {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(args.next, (unsigned long long)args.chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        h = rank < avail ? pool_next + rank : base + (rank - avail);
        pool_next = base + (n_need - avail);
        pool_end = base + (uint64_t)args.chunk;
      }
      if (need) {
        if (h >= n_hist) {
          state = kDone;
        } else {
          const uint32_t f = rec.flags[h];
          const uint32_t rs = f & 3u;
          if (rs != kRecDead) {
            ph.pos[0] = rec.px[h];
            ph.pos[1] = rec.py[h];
            ph.pos[2] = rec.pz[h];
            ph.dir[0] = rec.dx[h];
            ph.dir[1] = rec.dy[h];
            ph.dir[2] = rec.dz[h];
            set_energy(s, ph, rec.e[h]);
            ph.steps = (int)((f >> 2) & 1u);
            ph.alive = 1;
            ph.can_enter = 1;
            ph.in_head = 0;
            ph.exclude = -1;
            if constexpr (SPECT) ev.clear();
            const uint64_t hid = args.h_begin + h;
            const uint32_t rp = rec.rng_pos[h];
            const uint4 b = rec.rng_buf[h];
            g.k0 = (uint32_t)args.seed;
            g.k1 = (uint32_t)(args.seed >> 32);
            g.stream = 0u;
            g.h0 = (uint32_t)hid;
            g.h1 = (uint32_t)(hid >> 32);
            g.blk = rp >> 3;
            g.idx = (int)(rp & 7u);
            g.buf[0] = b.x;
            g.buf[1] = b.y;
            g.buf[2] = b.z;
            g.buf[3] = b.w;
            if (rs == kRecInImage) {
              ph.in_image = 1;
              ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
              state = kFly;
            } else if (rs == kRecWorld) {
              ph.in_image = 0;
              state = kFly;
            } else {
              ph.in_image = 0;
              pmat = s.world_mat;
              pscored = 0;
              state = kInteract;
            }
            in_hist = true;
          }
        }
      }
    } else if (phase == kInteract) {
      if (state == kInteract) {
        state = do_interaction<real, SPECT>(s, ph, g, &bc, pmat, pv, pscored, l, t, sec, n_dep, ev);
        if (state == kRefill && sec.has) {
          pop_secondary(s, ph, sec);
          state = kFly;
        }
      }
    } else {
      if (state == kFly) {
        state = flight<real, SPECT>(s, ph, g, &bc, pmat, pv, pscored, n_wood, n_real, n_world, n_head);
        if (state == kRefill && sec.has) {
          pop_secondary(s, ph, sec);
          state = kFly;
        }
      }
    }
  }
  // ---- counters -------------------------------------------------------------
  unsigned long long *cnt = args.counters;
  auto warp_add = [&](unsigned int v, int slot) {
    unsigned long long x = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0 && x) atomicAdd(&cnt[slot], x);
  };
  warp_add(n_wood, GG_CNT_WOODCOCK_STEPS);
  warp_add(n_real, GG_CNT_REAL_INTERACTIONS);
  warp_add(n_dep, GG_CNT_DEPOSITS);
  warp_add(n_world, GG_CNT_WORLD_STEPS);
  warp_add(n_head, GG_CNT_HEAD_STEPS);
  warp_add(n_singles, GG_CNT_SINGLES);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&cnt[GG_CNT_TALLY_ENTRIES], (unsigned long long)bc.tally_entries);
    atomicAdd(&cnt[GG_CNT_LIST_OVERFLOWS], (unsigned long long)bc.list_overflows);
    atomicAdd(&cnt[GG_CNT_ESCAPED], (unsigned long long)bc.escaped);
    atomicAdd(&cnt[GG_CNT_LOOP_CAPPED], (unsigned long long)bc.loop_capped);
    atomicAdd(&cnt[GG_CNT_STACK_OVERFLOW], (unsigned long long)bc.stack_overflow);
    atomicAdd(&cnt[GG_CNT_SECONDARIES], (unsigned long long)bc.secondaries);
  }
}

// Adds the per-batch fixed-point sums into the float64 images and clears them.
__global__ void k_flush(unsigned long long *acc_e, unsigned long long *acc_e2, double *edep, double *edep2,
                        size_t n) {
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    unsigned long long a = acc_e[i];
    if (a) {
      edep[i] += (double)a * 2.3283064365386963e-10;
      acc_e[i] = 0ull;
    }
    if (acc_e2) {
      const ulonglong2 b = reinterpret_cast<const ulonglong2 *>(acc_e2)[i];  // (low, high)
      if (b.x | b.y) {
        double lo = (double)b.x;
        lo = lo * 5.421010862427522e-20;  // 2^-64
        edep2[i] += (double)b.y + lo;
        reinterpret_cast<ulonglong2 *>(acc_e2)[i] = make_ulonglong2(0ull, 0ull);
      }
    }
  }
}

template <typename real>
size_t transport_smem_bytes(int n_comp, int n_e, int n_mat) {
  size_t b = sizeof(real) * ((size_t)n_comp * n_e + n_e + n_mat) + sizeof(int) * (size_t)n_mat;
  return (b + 15) & ~(size_t)15;
}

template <typename real>
size_t record_bytes(size_t cap) {
  return cap * (sizeof(uint4) + 7 * sizeof(real) + 2 * sizeof(uint32_t));
}

template <typename real>
cudaError_t launch_generate(const Scene<real> &s, const KernelArgs &a, cudaStream_t st) {
  uint64_t n = a.h_end - a.h_begin;
  unsigned int blocks = (unsigned int)((n + 255) / 256);
  k_generate<real><<<blocks, 256, 0, st>>>(s, a);
  return cudaGetLastError();
}

template <typename real, int MINB, bool SPECT>
static cudaError_t launch_transport_v(const Scene<real> &s, const KernelArgs &a, int grid, int block, size_t smem,
                                      cudaStream_t st) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_transport<real, MINB, SPECT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  k_transport<real, MINB, SPECT><<<grid, block, smem, st>>>(s, a);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_transport(const Scene<real> &s, const KernelArgs &a, int grid, int block, size_t smem,
                             int minb, cudaStream_t st) {
  if (s.spect) {
    if (minb <= 2) return launch_transport_v<real, 2, true>(s, a, grid, block, smem, st);
    if (minb == 3) return launch_transport_v<real, 3, true>(s, a, grid, block, smem, st);
    return launch_transport_v<real, 4, true>(s, a, grid, block, smem, st);
  }
  if (minb <= 2) return launch_transport_v<real, 2, false>(s, a, grid, block, smem, st);
  if (minb == 3) return launch_transport_v<real, 3, false>(s, a, grid, block, smem, st);
  return launch_transport_v<real, 4, false>(s, a, grid, block, smem, st);
}

cudaError_t launch_flush(unsigned long long *acc_e, unsigned long long *acc_e2, double *edep, double *edep2,
                         size_t n, int grid, cudaStream_t st) {
  k_flush<<<grid, 256, 0, st>>>(acc_e, acc_e2, edep, edep2, n);
  return cudaGetLastError();
}

template <typename real, bool SPECT>
static cudaError_t occupancy_v(int block, size_t smem, int minb, int *bps) {
  if (minb <= 2) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_transport<real, 2, SPECT>, block, smem);
  if (minb == 3) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_transport<real, 3, SPECT>, block, smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k_transport<real, 4, SPECT>, block, smem);
}

template <typename real>
cudaError_t occupancy_blocks(int block, size_t smem, int minb, int *blocks_per_sm, bool spect) {
  return spect ? occupancy_v<real, true>(block, smem, minb, blocks_per_sm)
               : occupancy_v<real, false>(block, smem, minb, blocks_per_sm);
}

template size_t record_bytes<float>(size_t);
template size_t record_bytes<double>(size_t);
template cudaError_t launch_generate<float>(const Scene<float> &, const KernelArgs &, cudaStream_t);
template cudaError_t launch_generate<double>(const Scene<double> &, const KernelArgs &, cudaStream_t);
template size_t transport_smem_bytes<float>(int, int, int);
template size_t transport_smem_bytes<double>(int, int, int);
template cudaError_t launch_transport<float>(const Scene<float> &, const KernelArgs &, int, int, size_t, int,
                                             cudaStream_t);
template cudaError_t launch_transport<double>(const Scene<double> &, const KernelArgs &, int, int, size_t, int,
                                              cudaStream_t);
template cudaError_t occupancy_blocks<float>(int, size_t, int, int *, bool);
template cudaError_t occupancy_blocks<double>(int, size_t, int, int *, bool);

}  // namespace gg
