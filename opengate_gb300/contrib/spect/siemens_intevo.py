"""Siemens Symbia Intevo heads on the opengate-shaped API
(opengate/contrib/spect/siemens_intevo.py counterparts): collimators lehr
(GE-like 1.5 mm holes here), melp (2.94 mm holes, 40.64 mm, 1.14 mm septa;
siemens_intevo.py:367-410) and he; crystal 3/8".  Placement as in
ge_discovery_nm670; the digitizer chain of siemens_intevo.add_digitizer
(siemens_intevo.py:729-800): energy-weighted centroid adder, inverse-square
energy blur of 9.9 % FWHM at 140.5 keV, 3.6 mm FWHM spatial blur."""

from ...units import g4_units as _u
from . import ge_discovery_nm670 as _nm670
from .ge_discovery_nm670 import add_spect_head as _add_head, get_default_size_and_spacing  # noqa: F401
from .ge_discovery_nm670 import rotate_gantry  # noqa: F401


def add_spect_head(sim, name="spect", collimator_type="lehr", debug=False):
    return _add_head(sim, name, collimator_type, debug=debug)


def add_digitizer(sim, crystal_name, name=None, size=None, spacing=None, channels=None, filename=None):
    return _nm670.add_digitizer(sim, crystal_name, name, size, spacing, channels, filename,
                                policy="EnergyWeightedCentroidPosition", resolution=0.099,
                                reference_energy=140.5 * _u.keV, spatial_fwhm=3.6 * _u.mm)
