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

template <typename real>
__device__ __forceinline__ void hlist_flush(HistList<real> &l, const Tally<real> &t, BlockCounters *bc) {
#pragma unroll
  for (int k = 0; k < kHistList; ++k) {
    if (k < l.n) {
      real a = l.acc[k];
      real a2 = a * a;
      atomicAdd(&t.acc_e[l.vox[k]], (unsigned long long)to_fixed(a));
      if (t.acc_e2) atomicAdd(&t.acc_e2[l.vox[k]], (unsigned long long)to_fixed(a2));
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
  const real *inv = s.ray_inv + (size_t)comp * s.n_rinv;
  real cost;
  int it = 0;
  for (;;) {
    real r = u01<real>(g);
    real tt = r * amax;
    real pos = tt * (real)(s.n_rinv - 1);
    int j = (int)pos;
    if (j > s.n_rinv - 2) j = s.n_rinv - 2;
    real f = pos - (real)j;
    real d = inv[j + 1] - inv[j];
    d = f * d;
    real x2 = inv[j] + d;
    real q = R<real>(2) * x2;
    q = q / x2max;
    cost = R<real>(1) - q;
    if (cost < R<real>(-1)) cost = R<real>(-1);
    real r2 = u01<real>(g);
    real lhs = R<real>(2) * r2;
    real rhs = cost * cost;
    rhs = R<real>(1) + rhs;
    if (lhs <= rhs) break;
    if (++it >= kLoopCap) {
      atomicAdd(&bc->loop_capped, 1u);
      break;
    }
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

// One secondary slot: after a pair conversion the photon continues as one
// 511 keV photon and the other waits here.  511 keV cannot convert again,
// so one slot always suffices.
template <typename real>
struct Secondary {
  real pos[3], dir[3];
  int has;
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
      sec.pos[a] = ph.pos[a];
      sec.dir[a] = -d[a];
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
  real off[3];
  rot_apply(s.s_rot, loc, off);
#pragma unroll
  for (int a = 0; a < 3; ++a) ph.pos[a] = s.s_t[a] + off[a];
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
    real p = u01<real>(g);
    int i = 0;
    while (i < s.n_spec - 1 && p >= s.spec_cdf[i]) ++i;
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

// One transport event: a Woodcock tentative step in the image (with the
// interaction if it is real), or a free flight in the world.
template <typename real>
__device__ __forceinline__ void step(const Scene<real> &s, Photon<real> &ph, Rng &g, BlockCounters *bc,
                                     HistList<real> &l, const Tally<real> &t, Secondary<real> &sec,
                                     unsigned int &n_wood, unsigned int &n_real, unsigned int &n_dep,
                                     unsigned int &n_world) {
  if (++ph.steps > kStepCap) {
    atomicAdd(&bc->loop_capped, 1u);
    ph.alive = 0;
    return;
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
      return;
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
    if (u2 * ph.mumax >= mu) return;
    ++n_real;
    real ed = interact(s, ph, m, g, bc, sec);
    deposit(l, t, bc, v, ed, n_dep);
    if (ph.alive && ph.in_image) ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
  } else {
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
      interact(s, ph, wm, g, bc, sec);
      ph.can_enter = 1;
    } else if (tin <= tout) {
#pragma unroll
      for (int a = 0; a < 3; ++a) ph.pos[a] = ph.pos[a] + tin * ph.dir[a];
      ph.in_image = 1;
      ph.t_exit = exit_distance(ph.pos, ph.dir, s.bmin, s.bmax);
    } else {
      ph.alive = 0;
      atomicAdd(&bc->escaped, 1u);
    }
  }
}

template <typename real>
__global__ void __launch_bounds__(256) k_transport(Scene<real> sg, KernelArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ BlockCounters bc;
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
  Tally<real> t{args.acc_e, args.acc_e2};
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  const uint64_t n_hist = args.h_end - args.h_begin;
  // warp-uniform pool of claimed history offsets [pool_next, pool_end)
  uint64_t pool_next = 0, pool_end = 0;

  Photon<real> ph;
  ph.alive = 0;
  Secondary<real> sec;
  sec.has = 0;
  HistList<real> l;
  l.n = 0;
  Rng g;
  bool done = false, in_hist = false;
  unsigned int n_wood = 0, n_real = 0, n_dep = 0, n_world = 0;

  for (;;) {
    bool need = false;
    if (!done && !ph.alive) {
      if (sec.has) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          ph.pos[a] = sec.pos[a];
          ph.dir[a] = sec.dir[a];
        }
        sec.has = 0;
        ph.alive = 1;
        set_energy(s, ph, R<real>(kMC2));
        start_photon(s, ph);
      } else {
        if (in_hist) {
          hlist_flush(l, t, &bc);
          in_hist = false;
        }
        need = true;
      }
    }
    const unsigned need_mask = __ballot_sync(0xffffffffu, need);
    if (need_mask) {
      const unsigned n_need = __popc(need_mask);
      const unsigned rank = __popc(need_mask & lt_mask);
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
          done = true;
        } else {
          g.init(args.seed, args.h_begin + h, 0u);
          int st = sample_primary(s, g, ph, &bc);
          if (st != GG_OK) {
            atomicOr(args.status, (unsigned int)st);
            done = true;
          } else {
            atomicAdd(&bc.histories, 1u);
            in_hist = true;
            start_photon(s, ph);
          }
        }
      }
    }
    if (__all_sync(0xffffffffu, done)) break;
    if (!done && ph.alive) step(s, ph, g, &bc, l, t, sec, n_wood, n_real, n_dep, n_world);
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
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&cnt[GG_CNT_HISTORIES], (unsigned long long)bc.histories);
    atomicAdd(&cnt[GG_CNT_TALLY_ENTRIES], (unsigned long long)bc.tally_entries);
    atomicAdd(&cnt[GG_CNT_LIST_OVERFLOWS], (unsigned long long)bc.list_overflows);
    atomicAdd(&cnt[GG_CNT_ESCAPED], (unsigned long long)bc.escaped);
    atomicAdd(&cnt[GG_CNT_SKIPPED], (unsigned long long)bc.skipped);
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
      unsigned long long b = acc_e2[i];
      if (b) {
        edep2[i] += (double)b * 2.3283064365386963e-10;
        acc_e2[i] = 0ull;
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
cudaError_t launch_transport(const Scene<real> &s, const KernelArgs &a, int grid, int block, size_t smem,
                             cudaStream_t st) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_transport<real>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  k_transport<real><<<grid, block, smem, st>>>(s, a);
  return cudaGetLastError();
}

cudaError_t launch_flush(unsigned long long *acc_e, unsigned long long *acc_e2, double *edep, double *edep2,
                         size_t n, int grid, cudaStream_t st) {
  k_flush<<<grid, 256, 0, st>>>(acc_e, acc_e2, edep, edep2, n);
  return cudaGetLastError();
}

template <typename real>
cudaError_t occupancy_blocks(int block, size_t smem, int *blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_transport<real>, block, smem);
}

template size_t transport_smem_bytes<float>(int, int, int);
template size_t transport_smem_bytes<double>(int, int, int);
template cudaError_t launch_transport<float>(const Scene<float> &, const KernelArgs &, int, int, size_t,
                                             cudaStream_t);
template cudaError_t launch_transport<double>(const Scene<double> &, const KernelArgs &, int, int, size_t,
                                              cudaStream_t);
template cudaError_t occupancy_blocks<float>(int, size_t, int *);
template cudaError_t occupancy_blocks<double>(int, size_t, int *);

}  // namespace gg
