"""Combination of the free-flight SPECT passes (opengate/contrib/spect/spect_freeflight_helpers.py:6-141).

The reference's free-flight recipe runs one simulation per component (the primary pass with
GammaFreeFlightActor, the scatter pass with ScatterSplittingFreeFlightActor, ...), each writing
the weighted projection ``counts`` = sum(w) and ``squared_counts`` = sum(w^2) of its singles
over N_i primaries.  The components estimate disjoint parts of the acquisition, so their
per-primary means add, and so do the variances of those means:

    E_i = C_i / N_i,  V_i = (C2_i / N_i - E_i^2) / (N_i - 1)  (clamped at 0),
    counts = ref_n * sum_i E_i,  relative uncertainty = sqrt(sum_i V_i) / sum_i E_i.
"""

import pathlib

import numpy as np

from ... import image_io


def merge_freeflight_arrays(counts, squared_counts, num_events, ref_n):
    """(merged counts scaled to ref_n primaries, relative uncertainty) of component arrays;
    components with num_events <= 1 are skipped (no variance), as in the reference."""
    total, var = None, None
    for c, c2, n in zip(counts, squared_counts, num_events):
        if n <= 1:
            continue
        e = np.asarray(c, dtype=np.float64) / n
        e2 = np.asarray(c2, dtype=np.float64) / n
        v = (e2 - e * e) / (n - 1)
        v[v < 0] = 0
        total = e if total is None else total + e
        var = v if var is None else var + v
    if total is None:
        raise ValueError("merge_freeflight: no component with more than one event")
    rel = np.divide(np.sqrt(var), total, out=np.zeros_like(var), where=total != 0)
    return total * ref_n, rel


def merge_freeflight_uncertainty(folder, ref_n, subfolders, num_events, counts_filename="projection_0_counts.mhd",
                                 squared_counts_filename="projection_0_squared_counts.mhd",
                                 output_filename="relative_uncertainty_0_counts.mhd", verbose=False):
    """Reads folder/<subfolder>/<counts_filename> and <squared_counts_filename> of every
    component, writes the merged counts (folder/<counts_filename>) and the relative
    uncertainty (folder/<output_filename>); returns both images."""
    folder = pathlib.Path(folder)
    if len(subfolders) != len(num_events):
        raise ValueError(f"merge_freeflight: subfolders and num_events must have the same length "
                         f"{subfolders} {num_events}")
    counts, squared, ns, template = [], [], [], None
    for sub, n in zip(subfolders, num_events):
        if n <= 1:
            if verbose:
                print(f"Skipping {sub} with n={n} events (n > 1 required)")
            continue
        cp, sp = folder / sub / counts_filename, folder / sub / squared_counts_filename
        for p in (cp, sp):
            if not p.exists():
                raise FileNotFoundError(f"merge_freeflight: {p} does not exist")
        if verbose:
            print(f"Reading {sub} with {n} events")
        c = image_io.read_mhd(cp)
        if template is None:
            template = c
        counts.append(c.array)
        squared.append(image_io.read_mhd(sp).array)
        ns.append(n)
    total, rel = merge_freeflight_arrays(counts, squared, ns, ref_n)
    out_c = image_io.Image(total, template.spacing, template.origin)
    out_u = image_io.Image(rel, template.spacing, template.origin)
    image_io.write_mhd(folder / counts_filename, out_c)
    image_io.write_mhd(folder / output_filename, out_u)
    return out_c, out_u


def merge_freeflight_uncertainty_for_all_heads(folder, ref_n, subfolders, num_events, num_heads, verbose=False):
    """merge_freeflight_uncertainty for projection_<head>_counts.mhd of every head."""
    return [merge_freeflight_uncertainty(folder, ref_n, subfolders, num_events,
                                         counts_filename=f"projection_{h}_counts.mhd",
                                         squared_counts_filename=f"projection_{h}_squared_counts.mhd",
                                         output_filename=f"relative_uncertainty_{h}_counts.mhd", verbose=verbose)
            for h in range(num_heads)]
