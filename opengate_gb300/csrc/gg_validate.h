// gg_validate.h - argument checks shared by every entry point that takes the
// scene descriptors (gg_upload_tables / gg_upload_volume / gg_set_source and
// the no-allocation dose run), so that both paths reject the same inputs.
// Each check returns nullptr when the input is valid, else a message naming
// what is wrong (written into `msg`).
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdio>

#include "../../include/gate_gpu.h"

namespace gg {

// Tables: sizes, energy grid, material -> composition / density, attenuation
// entries finite and >= 0, Rayleigh x^2 nodes increasing.
inline const char *check_tables(const gg_tables_desc *t, char *msg, size_t len) {
  if (t->n_e < 2 || t->n_comp < 1 || t->n_ray < 2 || t->n_mat < 1 || !t->sig || !t->cum || !t->ray_amax ||
      !t->ray_cum || !t->ray_x2 || !t->mat_comp || !t->mat_rho) {
    snprintf(msg, len, "incomplete table descriptor");
    return msg;
  }
  if (!(t->inv_dln > 0) || !(t->e_min > 0) || !(t->e_max > t->e_min) || !std::isfinite(t->e_max) ||
      !std::isfinite(t->inv_dln) || !std::isfinite(t->ln_emin)) {
    snprintf(msg, len, "invalid energy grid");
    return msg;
  }
  for (int m = 0; m < t->n_mat; ++m) {
    if (t->mat_comp[m] < 0 || t->mat_comp[m] >= t->n_comp) {
      snprintf(msg, len, "material %d refers to composition %d", m, t->mat_comp[m]);
      return msg;
    }
    if (!(t->mat_rho[m] > 0) || !std::isfinite(t->mat_rho[m])) {
      snprintf(msg, len, "material %d density must be finite and > 0", m);
      return msg;
    }
  }
  const size_t nce = (size_t)t->n_comp * t->n_e;
  for (size_t i = 0; i < nce; ++i)
    if (!(t->sig[i] >= 0) || !std::isfinite(t->sig[i])) {
      snprintf(msg, len, "attenuation table has a negative or non-finite entry");
      return msg;
    }
  for (int i = 1; i < t->n_ray; ++i)
    if (!(t->ray_x2[i] > t->ray_x2[i - 1])) {
      snprintf(msg, len, "Rayleigh x^2 nodes must increase");
      return msg;
    }
  return nullptr;
}

// Image dimensions: each > 0 and the voxel count at most max_voxels, checked
// before any product can wrap (every partial product stays <= max_voxels).
inline const char *check_dims(const int32_t dims[3], size_t max_voxels, size_t *n_vox, char *msg, size_t len) {
  size_t n = 1;
  for (int a = 0; a < 3; ++a) {
    if (dims[a] <= 0) {
      snprintf(msg, len, "dims must be > 0");
      return msg;
    }
    if ((size_t)dims[a] > max_voxels / n) {
      snprintf(msg, len, "image of %d x %d x %d voxels; at most %zu voxels", dims[0], dims[1], dims[2], max_voxels);
      return msg;
    }
    n *= (size_t)dims[a];
  }
  *n_vox = n;
  return nullptr;
}

// Woodcock majorant: finite and > 0 at every energy node.
inline const char *check_majorant(const float *maj, int n_e, char *msg, size_t len) {
  for (int i = 0; i < n_e; ++i)
    if (!(maj[i] > 0) || !std::isfinite(maj[i])) {
      snprintf(msg, len, "majorant must be finite and > 0");
      return msg;
    }
  return nullptr;
}

// Source energy distribution: non-empty spectra with finite energies and
// non-decreasing cumulative weights; returns the energy range in elo / ehi.
inline const char *check_source_energy(const gg_source_desc *s, double *elo, double *ehi, char *msg, size_t len) {
  if (s->ene_type == GG_ENE_MONO) {
    *elo = *ehi = s->mono;
  } else if (s->ene_type == GG_ENE_RANGE) {
    *elo = s->e_lo;
    *ehi = s->e_hi;
    if (!(s->e_hi >= s->e_lo)) {
      snprintf(msg, len, "energy range with e_hi < e_lo");
      return msg;
    }
  } else {
    if (s->n_spec < 1 || !s->spec_e || !s->spec_cdf) {
      snprintf(msg, len, "empty spectrum");
      return msg;
    }
    const int ne = s->ene_type == GG_ENE_HISTOGRAM ? s->n_spec + 1 : s->n_spec;
    *elo = *ehi = s->spec_e[0];
    for (int i = 0; i < ne; ++i) {
      if (!std::isfinite(s->spec_e[i])) {
        snprintf(msg, len, "spectrum energy %d is not finite", i);
        return msg;
      }
      *elo = std::fmin(*elo, s->spec_e[i]);
      *ehi = std::fmax(*ehi, s->spec_e[i]);
    }
    for (int i = 0; i < s->n_spec; ++i)
      if (!std::isfinite(s->spec_cdf[i]) || (i > 0 && s->spec_cdf[i] < s->spec_cdf[i - 1])) {
        snprintf(msg, len, "cumulative weights decrease or are not finite");
        return msg;
      }
  }
  return nullptr;
}

}  // namespace gg
