"""Attenuation and energy-absorption coefficients of materials (track-length estimator).

Restates the reference's mu / mu_en handler for the NIST and EPDL databases:

* element tables (GateMaterialMuHandler::InitElementTable,
  core/opengate_core/opengate_lib/GateMaterialMuHandler.cpp:265-296): raw
  rows (E MeV, mu/rho, mu_en/rho in cm2/g) per Z, an absorption edge being
  two rows with the same energy;
* material tables (GateMaterialMuHandler::ConstructMaterial, :159-263): the
  union of the element energies (an energy shared by two elements kept once,
  an edge pair of one element kept twice), and at each union energy the
  mass-fraction sum of the elements' values - the element's own value where
  it has that energy (below-edge value first, above-edge value at the second
  copy), else the log-log interpolation between its two neighbouring rows
  (``exp(ln ya + ln(yb/ya) / ln(xb/xa) * ln(x/xa))``, :103-106); stored as
  logarithms;
* lookup (GateMuTable::GetMuEnOverRho / GetMuOverRho,
  core/opengate_core/opengate_lib/GateMuTables.cpp:47-111): ln E, binary
  search for the bracketing rows, linear interpolation of the logarithms
  strictly inside, otherwise the lower row's value.

The element data come from ``data/mu_database.npz`` (see
``data/make_mu_database.py``).
"""

import functools
import math
import pathlib

import numpy as np

_DATA = pathlib.Path(__file__).with_name("data") / "mu_database.npz"
DATABASES = ("EPDL", "NIST")


@functools.lru_cache(maxsize=1)
def _raw():
    d = np.load(_DATA)
    return {k: d[k] for k in d.files}


@functools.lru_cache(maxsize=None)
def element_table(database, z):
    """(E, mu/rho, mu_en/rho) rows of element ``z`` in ``database``."""
    if database not in DATABASES:
        raise ValueError(f"mu/mu_en database must be one of {DATABASES}, not {database!r}")
    raw = _raw()
    count = raw[f"{database}_count"]
    if not 1 <= z < len(count):
        raise ValueError(f"element Z={z} is not in the {database} database")
    start = int(count[:z].sum())
    rows = raw[f"{database}_rows"][start:start + int(count[z])]
    return rows[:, 0].copy(), rows[:, 1].copy(), rows[:, 2].copy()


def _loglog(xa, xb, ya, yb, x):
    return math.exp(math.log(ya) + math.log(yb / ya) / math.log(xb / xa) * math.log(x / xa))


class MaterialMuTable:
    """Material table of one composition: ln E, ln mu/rho, ln mu_en/rho."""

    def __init__(self, z_list, w_list, database="EPDL"):
        tabs = [element_table(database, int(z)) for z in z_list]
        w = [float(x) for x in w_list]
        sizes = [len(t[0]) for t in tabs]
        n_el = len(tabs)
        # union energy grid
        energies = []
        index = [0] * n_el
        total = sum(sizes)
        i = 0
        while i < total:
            m = 0
            while index[m] >= sizes[m]:
                m += 1
            for j in range(m + 1, n_el):
                if index[j] < sizes[j] and tabs[j][0][index[j]] < tabs[m][0][index[m]]:
                    m = j
            e = tabs[m][0][index[m]]
            keep = True
            if energies and e == energies[-1]:
                keep = index[m] > 0 and tabs[m][0][index[m]] == tabs[m][0][index[m] - 1]
            if keep:
                energies.append(e)
                i += 1
            else:
                total -= 1
            index[m] += 1
        # values
        mu = np.zeros(len(energies))
        muen = np.zeros(len(energies))
        index = [0] * n_el
        for i, e in enumerate(energies):
            for j in range(n_el):
                ej, mj, aj = tabs[j]
                if index[j] < sizes[j] and ej[index[j]] < e:
                    index[j] += 1
                k = min(index[j], sizes[j] - 1)
                if ej[k] == e:
                    mu[i] += w[j] * mj[k]
                    muen[i] += w[j] * aj[k]
                    if i != len(energies) - 1 and k + 1 < sizes[j] and ej[k] == ej[k + 1]:
                        index[j] += 1
                else:
                    mu[i] += w[j] * _loglog(ej[k - 1], ej[k], mj[k - 1], mj[k], e)
                    muen[i] += w[j] * _loglog(ej[k - 1], ej[k], aj[k - 1], aj[k], e)
        self.ln_e = np.log(np.asarray(energies))
        self.ln_mu = np.log(mu)
        self.ln_muen = np.log(muen)

    def _lookup(self, table, energy):
        le = math.log(energy)
        lo, hi = 0, len(self.ln_e) - 1
        while hi - lo > 1:
            mid = (lo + hi) // 2
            if self.ln_e[mid] > le:
                hi = mid
            else:
                lo = mid
        e0, e1 = self.ln_e[lo], self.ln_e[hi]
        if e0 < le < e1:
            return math.exp(table[lo] + (table[hi] - table[lo]) * (le - e0) / (e1 - e0))
        return math.exp(table[lo])

    def mu_en_over_rho(self, energy):
        """cm2/g at ``energy`` MeV (scalar or array)."""
        return np.vectorize(lambda e: self._lookup(self.ln_muen, float(e)))(energy)

    def mu_over_rho(self, energy):
        return np.vectorize(lambda e: self._lookup(self.ln_mu, float(e)))(energy)


@functools.lru_cache(maxsize=None)
def material_table(z_tuple, w_tuple, database="EPDL"):
    return MaterialMuTable(z_tuple, w_tuple, database)
