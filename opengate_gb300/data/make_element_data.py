"""Generate ``elements_nist.npz``: per-element photon attenuation data.

Run once in a checkout that has the opengate sources next to it::

    python opengate_gb300/data/make_element_data.py /path/to/opengate

It loads ``opengate/data/PhotonAttenuation.py`` (numpy/scipy only) and copies
its public NIST (Hubbell & Seltzer) arrays into a compact numpy archive:

* ``energy``: the 36-point energy grid, 1 keV - 20 MeV;
* ``mac``: mass attenuation coefficients, Z = 1..100, cm2/g;
* ``meac``: mass energy-absorption coefficients, Z = 1..92, cm2/g;
* ``edges``: absorption edges (Z, E, mac below/above, meac below/above);
* ``atomic_mass``: A = Z / (Z/A) from ``PropsEl``.

The package reads only the archive at run time.
"""

import importlib.util
import pathlib
import sys

import numpy as np


def main(ref_root):
    ref_root = pathlib.Path(ref_root)
    spec = importlib.util.spec_from_file_location(
        "photon_attenuation", ref_root / "opengate/data/PhotonAttenuation.py"
    )
    pa = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pa)
    n_el = pa.mac.shape[0]
    z_over_a = np.array([float(r[0]) for r in pa.PropsEl[:n_el]])
    symbols = np.array([str(r[2]) for r in pa.PropsEl[:n_el]])
    z = np.arange(1, n_el + 1, dtype=np.float64)
    out = pathlib.Path(__file__).with_name("elements_nist.npz")
    np.savez_compressed(
        out,
        energy=np.asarray(pa.energy, dtype=np.float64),
        mac=np.asarray(pa.mac, dtype=np.float64),
        meac=np.asarray(pa.meac, dtype=np.float64),
        edges=np.asarray(pa.edges, dtype=np.float64),
        atomic_mass=z / z_over_a,
        symbols=symbols,
    )
    print(f"wrote {out}: {n_el} elements x {pa.energy.size} energies, {len(pa.edges)} edges")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <root of the opengate source tree>")
    main(sys.argv[1])
