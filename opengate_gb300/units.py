"""Geant4 / CLHEP unit system, so scripts written for opengate carry over.

Internal units are those of CLHEP: mm, ns, MeV, eplus, kelvin, mole, candela;
``g4_units.mm == 1``, ``g4_units.MeV == 1``.  Derived units follow the
CLHEP definitions (joule = MeV / e_SI * 1e-6, kg = joule s^2 / m^2, ...).
"""

import math


class _Units(dict):
    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e


def _build():
    u = _Units()
    u["mm"] = 1.0
    u["um"] = 1e-3
    u["nm"] = 1e-6
    u["cm"] = 10.0
    u["m"] = 1000.0
    u["km"] = 1e6
    u["mm2"] = 1.0
    u["cm2"] = 100.0
    u["mm3"] = 1.0
    u["cm3"] = 1000.0
    u["m3"] = 1e9
    u["mL"] = u["cm3"]
    u["L"] = 1e6
    u["rad"] = 1.0
    u["deg"] = math.pi / 180.0
    u["mrad"] = 1e-3
    u["sr"] = 1.0
    u["ns"] = 1.0
    u["s"] = 1e9
    u["ms"] = 1e6
    u["us"] = 1e3
    u["ps"] = 1e-3
    u["min"] = 60e9
    u["h"] = 3600e9
    u["second"] = u["s"]
    u["MeV"] = 1.0
    u["keV"] = 1e-3
    u["eV"] = 1e-6
    u["GeV"] = 1e3
    e_si = 1.602176634e-19
    u["eplus"] = 1.0
    u["joule"] = 1e-6 / e_si  # MeV per joule
    u["J"] = u["joule"]
    u["kg"] = u["joule"] * u["s"] ** 2 / u["m"] ** 2
    u["g"] = 1e-3 * u["kg"]
    u["mg"] = 1e-3 * u["g"]
    u["g_cm3"] = u["g"] / u["cm3"]
    u["kg_m3"] = u["kg"] / u["m3"]
    u["Gy"] = u["joule"] / u["kg"]
    u["mGy"] = 1e-3 * u["Gy"]
    u["Bq"] = 1.0 / u["s"]
    u["kBq"] = 1e3 * u["Bq"]
    u["MBq"] = 1e6 * u["Bq"]
    u["GBq"] = 1e9 * u["Bq"]
    u["Ci"] = 3.7e10 * u["Bq"]
    u["mCi"] = 1e-3 * u["Ci"]
    u["barn"] = 1e-22 * u["mm2"]
    return u


g4_units = _build()
