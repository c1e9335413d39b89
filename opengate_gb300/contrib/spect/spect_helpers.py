"""SPECT helpers (opengate/contrib/spect/spect_helpers.py counterparts).

Energy windows per radionuclide as in get_default_energy_windows
(spect_helpers.py:315-371); the noise and efficiency figures of merit are
those of opengate_gb300.spect.
"""

from ...units import g4_units as _u
from ...spect import (compute_efficiency, compute_history_by_history_relative_uncertainty,  # noqa: F401
                      compute_poisson_relative_uncertainty, compute_speedup, compute_zscore)

_keV = _u.keV

# (name, min keV, max keV); the first entry is the full-spectrum channel
_WINDOWS = {
    "lu177": [("spectrum", 3, 515), ("scatter1", 84.75, 101.7), ("peak113", 101.7, 124.3),
              ("scatter2", 124.3, 141.25), ("scatter3", 145.6, 187.2), ("peak208", 187.2, 228.8),
              ("scatter4", 228.8, 270.4)],
    "tc99m": [("spectrum", 3, 160), ("scatter", 108.58, 129.59), ("peak140", 129.59, 150.61)],
    "in111": [("spectrum_full", 3.0, 515.0), ("scatter_171_low", 138.4525, 158.4525),
              ("peak_171", 158.4525, 184.1475), ("scatter_171_high", 184.1475, 204.1475),
              ("scatter_245_low", 206.995, 226.995), ("peak_245", 226.995, 263.805),
              ("scatter_245_high", 263.805, 283.805)],
    "i123": [("spectrum", 3, 200), ("scatter_low", 125, 143.1), ("peak159", 143.1, 174.9),
             ("scatter_high", 174.9, 195)],
    "i131": [("spectrum", 3, 410), ("scatter_low", 285, 327.6), ("peak364", 327.6, 400.4)],
}
_ALIASES = {"177lu": "lu177", "lu177": "lu177", "tc99m": "tc99m", "111in": "in111", "in111": "in111",
            "123i": "i123", "i123": "i123", "131i": "i131", "i131": "i131"}


def get_default_energy_windows(radionuclide_name, spectrum_channel=False):
    n = radionuclide_name.lower()
    key = next((v for k, v in _ALIASES.items() if k in n), None)
    if key is None:
        raise ValueError(f"No default energy windows for {radionuclide_name}")
    ch = [{"name": name, "min": lo * _keV, "max": hi * _keV} for name, lo, hi in _WINDOWS[key]]
    return ch if spectrum_channel else ch[1:]
