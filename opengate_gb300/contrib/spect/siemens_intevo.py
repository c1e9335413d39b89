"""Siemens Symbia Intevo heads on the opengate-shaped API
(opengate/contrib/spect/siemens_intevo.py counterparts): collimators lehr
(GE-like 1.5 mm holes here), melp (2.94 mm holes, 40.64 mm, 1.14 mm septa;
siemens_intevo.py:367-410) and he; crystal 3/8".  Placement and digitizer
as in ge_discovery_nm670."""

from .ge_discovery_nm670 import add_digitizer, add_spect_head as _add_head, get_default_size_and_spacing  # noqa: F401
from .ge_discovery_nm670 import rotate_gantry  # noqa: F401


def add_spect_head(sim, name="spect", collimator_type="lehr", debug=False):
    return _add_head(sim, name, collimator_type, debug=debug)
