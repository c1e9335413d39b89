"""Generate ``mu_database.npz``: per-element attenuation and energy-absorption tables.

Run once in a checkout that has the opengate sources next to it::

    python opengate_gb300/data/make_mu_database.py /path/to/opengate

It reads the two public element databases that opengate's track-length
estimator uses (core/opengate_core/opengate_lib/GateMuDatabase.h: NIST,
Hubbell & Seltzer, Z = 1..92; EPDL97, Z = 1..100) - each a list of
(E MeV, mu/rho cm2/g, mu_en/rho cm2/g) rows per element, absorption edges as
two rows with the same energy - and stores, per database:

* ``<db>_count``: rows per element, index = Z (row 0 unused);
* ``<db>_rows``: all rows, elements in Z order, shape (sum(count), 3).

The package reads only the archive at run time.
"""

import pathlib
import re
import sys

import numpy as np


def _array(text, name):
    m = re.search(r"%s\s*\[\s*\d+\s*\]\s*=\s*\{([^}]*)\}" % re.escape(name), text)
    if not m:
        raise SystemExit(f"{name} not found")
    return np.array([float(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()])


def main(ref_root):
    src = pathlib.Path(ref_root) / "core/opengate_core/opengate_lib/GateMuDatabase.h"
    text = src.read_text()
    out = {}
    for db in ("NIST", "EPDL"):
        count = _array(text, f"{db}_mu_muen_data_energyNumber").astype(np.int32)
        rows = _array(text, f"{db}_mu_muen_data").reshape(-1, 3)
        if rows.shape[0] != int(count.sum()):
            raise SystemExit(f"{db}: {rows.shape[0]} rows, counts sum to {int(count.sum())}")
        out[f"{db}_count"] = count
        out[f"{db}_rows"] = rows
    dst = pathlib.Path(__file__).with_name("mu_database.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <root of the opengate source tree>")
    main(sys.argv[1])
