"""DoseActor outputs: dose conversion, variance and uncertainty images.

Restates the reference's end-of-run arithmetic:

* :func:`calculate_variance` - opengate/utility.py:551-560:
  ``clip((sum_x2/N - (sum_x/N)^2) / (N - 1), 0)``;
* :func:`variance_or_uncertainty` - SingleItkImageWithVariance.
  get_variance_or_uncertainty (opengate/actors/dataitems.py:1956-1993): the
  variance, its square root, or the relative uncertainty std / (sum_x/N)
  (0 where sum_x = 0); all ones when N <= 1, zeros when the squared image is
  missing;
* :func:`edep_to_dose` - the dose path of GateDoseActor::SteppingAction
  (core/opengate_core/opengate_lib/GateDoseActor.cpp:196-217: dose += edep /
  density of the material at the deposit) and the unit conversion of
  DoseActor.EndOfRunActionMasterThread (opengate/actors/doseactors.py:686-696:
  divide by Gy x voxel volume, squared for the squared image).  When the dose
  grid is the image grid every deposit in a voxel sees that voxel's
  material, so the per-voxel division is exact.
"""

import numpy as np

# 1 MeV in joule (CODATA 2018, exact)
MEV_J = 1.602176634e-13


def calculate_variance(value, squared, n):
    return np.clip((squared / n - np.power(value / n, 2)) / (n - 1), 0, None)


def variance_or_uncertainty(value, squared, n, which):
    value = np.asarray(value, dtype=np.float64)
    if not n > 1:
        return np.ones_like(value)
    if squared is None:
        return np.zeros_like(value)
    out = calculate_variance(value, np.asarray(squared, dtype=np.float64), n)
    if which in ("std", "uncertainty"):
        out = np.sqrt(out)
    if which == "uncertainty":
        out = np.divide(out, value / n, out=np.zeros_like(out), where=value != 0)
    return out


def edep_to_dose(edep, density_g_cm3, spacing_mm, squared=False):
    """Dose image in Gy from an edep image in MeV (or its squared image).

    ``density_g_cm3`` is the per-voxel density (same shape as ``edep``).
    """
    voxel_kg = density_g_cm3 * 1e-3 * (spacing_mm[0] * spacing_mm[1] * spacing_mm[2] * 1e-3)
    scale = MEV_J / voxel_kg
    with np.errstate(divide="ignore", invalid="ignore"):
        out = np.where(voxel_kg > 0, edep * (scale * scale if squared else scale), 0.0)
    return out


def mean_relative_uncertainty(edep, edep2, n, threshold=0.1):
    """Mean relative uncertainty over voxels with edep above threshold * max."""
    unc = variance_or_uncertainty(edep, edep2, n, "uncertainty")
    sel = edep > threshold * edep.max()
    return float(unc[sel].mean()) if np.any(sel) else float("nan")
