"""Cross-section and sampling tables handed to the transport kernels.

The tables are the data contract between the host and the CUDA kernels (and
the CPU oracle, which receives the very same float32 arrays):

* a log-spaced energy grid ``E_i = E_MIN * (E_MAX/E_MIN)^(i/(N_E-1))``;
* per composition ``c`` (a set of element mass fractions, shared by all
  materials with that composition whatever their density):
  - ``sig[c, i]``: total attenuation per unit density, mm^-1 per g/cm3
    (0.1 x the mass attenuation coefficient in cm2/g);
  - ``cum[c, k, i]``, k = 0, 1, 2: cumulative process fractions
    Compton, +photoelectric, +Rayleigh (pair takes the rest);
  - ``ray_amax[c, i]``: normalised cumulative of the Rayleigh form-factor
    law at the largest momentum transfer reachable at E_i;
  - ``ray_cum[c, j]``: normalised cumulative of F^2(x^2) dx^2 at the shared
    x^2 nodes ``ray_x2[j]`` (1/Angstrom^2), piecewise linear in between.
* per material ``m`` (label): its composition index and density.

Values between grid points are linear in ln(E).  The per-element partial
cross sections come from :mod:`opengate_gb300.xsection`.
"""

import functools

import numpy as np

from . import xsection

N_E = 512
E_MIN = 1e-3  # MeV; photons below are absorbed locally
E_MAX = 20.0  # MeV
N_RAY = 1024


def energy_grid():
    return np.exp(np.linspace(np.log(E_MIN), np.log(E_MAX), N_E))


def rayleigh_x2_nodes():
    """x^2 nodes (1/Angstrom^2) of the Rayleigh cumulative: 0, then log-spaced 1e-6..1e7."""
    return np.concatenate([[0.0], np.geomspace(1e-6, 1e7, N_RAY - 1)]).astype(np.float32).astype(np.float64)


@functools.lru_cache(maxsize=None)
def _element_partials_on_grid(z):
    p = xsection.element_partials(z, energy_grid())
    return {k: v.copy() for k, v in p.items()}


class CompositionTable:
    """Tables for one element composition."""

    def __init__(self, z_list, w_list):
        self.z_list = list(z_list)
        self.w_list = np.asarray(w_list, dtype=np.float64)
        parts = {k: np.zeros(N_E) for k in ("compton", "photo", "rayleigh", "pair")}
        for z, w in zip(self.z_list, self.w_list):
            p = _element_partials_on_grid(z)
            for k in parts:
                parts[k] += w * p[k]
        self.partials = parts  # cm2/g
        tot = parts["compton"] + parts["photo"] + parts["rayleigh"] + parts["pair"]
        self.mu_rho = tot
        with np.errstate(invalid="ignore", divide="ignore"):
            c0 = np.where(tot > 0, parts["compton"] / tot, 1.0)
            c1 = np.where(tot > 0, (parts["compton"] + parts["photo"]) / tot, 1.0)
            c2 = np.where(tot > 0, (parts["compton"] + parts["photo"] + parts["rayleigh"]) / tot, 1.0)
        # pair fraction exactly zero below threshold, and at the first grid
        # node above it, so that the linear interpolation inside the interval
        # that straddles 2 m_e c^2 cannot select a pair conversion below it
        below = energy_grid() <= 2.0 * xsection.ELECTRON_MASS_MEV
        below[1:] |= below[:-1]
        c2 = np.where(below, 1.0, c2)
        self.cum = np.stack([c0, c1, c2])
        # Rayleigh sampling tables: the cumulative of F^2 dx^2, piecewise linear in
        # x^2 between the nodes of rayleigh_x2_nodes(); the sampler inverts
        # exactly this piecewise-linear function, and ray_amax is evaluated on it
        x2n = rayleigh_x2_nodes()
        x2, a, _ = xsection.rayleigh_cumulative(self.z_list, self.w_list)
        cum = np.interp(x2n, np.concatenate([[0.0], x2]), np.concatenate([[0.0], a]))
        cum /= cum[-1]
        self.ray_cum = cum
        k2 = (energy_grid() / xsection.HC_MEV_ANGSTROM) ** 2
        self.ray_amax = np.interp(k2, x2n, cum)


class PhysicsTables:
    """All compositions needed by a simulation, plus per-material entries."""

    def __init__(self, materials):
        """``materials``: list of :class:`~opengate_gb300.materials.Material`; index = material id."""
        self.materials = list(materials)
        keys = []
        self.mat_comp = np.zeros(len(materials), dtype=np.int32)
        self.mat_rho = np.zeros(len(materials), dtype=np.float32)
        for m, mat in enumerate(materials):
            k = mat.composition_key()
            if k not in keys:
                keys.append(k)
            self.mat_comp[m] = keys.index(k)
            self.mat_rho[m] = np.float32(mat.density)
        self.comps = [CompositionTable([z for z, _ in k], [w for _, w in k]) for k in keys]
        nc = len(self.comps)
        self.sig = np.zeros((nc, N_E), dtype=np.float32)
        self.cum = np.zeros((nc, 3, N_E), dtype=np.float32)
        self.ray_amax = np.zeros((nc, N_E), dtype=np.float32)
        self.ray_cum = np.zeros((nc, N_RAY), dtype=np.float32)
        for c, ct in enumerate(self.comps):
            self.sig[c] = (0.1 * ct.mu_rho).astype(np.float32)
            self.cum[c] = ct.cum.astype(np.float32)
            self.ray_amax[c] = ct.ray_amax.astype(np.float32)
            self.ray_cum[c] = ct.ray_cum.astype(np.float32)

    @property
    def n_comp(self):
        return len(self.comps)

    def muen(self, database="EPDL"):
        """Energy absorption per unit density, mm^-1 per g/cm3 ([n_comp, N_E] float32):
        0.1 x mu_en/rho of each composition at the grid energies, from the
        material tables of :mod:`opengate_gb300.mu_tables` (the track-length
        estimator's data; linear in ln E between grid points like ``sig``)."""
        from . import mu_tables

        out = np.zeros((self.n_comp, N_E), dtype=np.float32)
        grid = energy_grid()
        for c, ct in enumerate(self.comps):
            t = mu_tables.material_table(tuple(int(z) for z in ct.z_list), tuple(float(w) for w in ct.w_list),
                                         database)
            out[c] = (0.1 * t.mu_en_over_rho(grid)).astype(np.float32)
        return out

    def mu_mm(self, material_index, energy):
        """Linear attenuation (1/mm) of a material at ``energy`` (float64, for checks)."""
        c = self.mat_comp[material_index]
        le = np.log(np.asarray(energy, dtype=np.float64))
        g = np.log(energy_grid())
        return float(self.mat_rho[material_index]) * np.interp(le, g, self.sig[c].astype(np.float64))

    def majorant(self, material_ids):
        """Per-energy majorant over ``material_ids`` (float32, inflated by 1e-6).

        Linear interpolation of a pointwise maximum dominates every interpolated
        member, so the interpolated majorant bounds each material's
        interpolated attenuation at any energy.
        """
        ids = np.unique(np.asarray(material_ids, dtype=np.int64))
        mu = self.sig[self.mat_comp[ids]].astype(np.float64) * self.mat_rho[ids, None].astype(np.float64)
        return (mu.max(axis=0) * (1.0 + 1e-6)).astype(np.float32)
