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

:func:`precision_error` states the error of an FP32 build against the FP64
build of the same kernels on the same random stream.
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


def dose_sum_to_gy(dose_sum, spacing_mm, squared=False):
    """Dose image in Gy from the dose tally sum(edep / rho) in MeV cm3 / g of a dose grid
    (every deposit divided by the density where it happened, GateDoseActor.cpp:206-217),
    divided by the voxel volume (doseactors.py:686-696; squared for the squared image)."""
    scale = MEV_J / (spacing_mm[0] * spacing_mm[1] * spacing_mm[2] * 1e-6)
    return np.asarray(dose_sum, dtype=np.float64) * (scale * scale if squared else scale)


def mean_relative_uncertainty(edep, edep2, n, threshold=0.1):
    """Mean relative uncertainty over voxels with edep above threshold * max."""
    unc = variance_or_uncertainty(edep, edep2, n, "uncertainty")
    sel = edep > threshold * edep.max()
    return float(unc[sel].mean()) if np.any(sel) else float("nan")


def mean_of_highest_n(image, n):
    """Mean of the n largest voxel values (GateDoseActor::GetMeanOfHighestNValues,
    core/opengate_core/opengate_lib/GateDoseActor.cpp:401-430)."""
    v = np.asarray(image, dtype=np.float64).ravel()
    if v.size == 0 or n <= 0:
        return 0.0
    n = min(int(n), v.size)
    return float(np.partition(v, v.size - n)[v.size - n:].mean())


def compute_mean_uncertainty(edep, edep_squared, n_events, threshold=0.7, top_voxels=10):
    """Mean relative uncertainty of the voxels above threshold x (mean of the
    top_voxels largest edep) - the uncertainty-goal criterion of
    GateDoseActor::ComputeMeanUncertainty (GateDoseActor.cpp:261-317): events
    counted at least 2, per-voxel variance clipped at 0 and relative
    uncertainty at 1; 1 when no voxel qualifies."""
    e = np.asarray(edep, dtype=np.float64).ravel()
    e2 = np.asarray(edep_squared, dtype=np.float64).ravel()
    n = max(float(n_events), 2.0)
    sel = e > mean_of_highest_n(e, top_voxels) * threshold
    if not sel.any():
        return 1.0
    val = e[sel] / n
    unc = (e2[sel] / n - val * val) / (n - 1.0)
    unc = np.sqrt(np.clip(unc, 0.0, None)) / val
    unc = np.minimum(unc, 1.0)
    m = float(unc.mean())
    return m if m > 0 else 1.0


def next_uncertainty_check(current, goal, n_events, overshoot=1.05):
    """Events at which the next check happens (GateDoseActor.cpp:269-274)."""
    return int((current / goal) * (current / goal) * n_events * overshoot)


def precision_error(edep_a, edep2_a, edep_b, edep2_b, n, threshold=0.1):
    """Error of image ``a`` against image ``b``, both edep sums of the same ``n``
    histories on the same random stream (an FP32 build against the FP64 build of
    the same kernels).

    Histories follow the same draws until a rounding difference changes a
    decision, so most voxels agree to rounding and the rest differ by a few
    histories.  Reported over the voxels above ``threshold`` x max of ``b``:
    integral relative difference (all voxels), fraction of voxels within 2
    combined standard deviations of the sum (the statistical criterion applied
    to two independent runs), the largest and the median |a - b| / sigma, the
    median relative difference, and the fraction of voxels that are equal.
    """
    a = np.asarray(edep_a, dtype=np.float64).ravel()
    b = np.asarray(edep_b, dtype=np.float64).ravel()
    qa = np.asarray(edep2_a, dtype=np.float64).ravel()
    qb = np.asarray(edep2_b, dtype=np.float64).ravel()
    tb = float(b.sum())
    integral = abs(float(a.sum()) - tb) / tb if tb > 0 else 0.0
    mask = b > threshold * b.max() if b.size and b.max() > 0 else np.zeros(b.shape, bool)
    if not mask.any():
        return {"integral_rel": integral, "voxels": 0}
    # standard deviation of a sum of n history values: sqrt(n var) = sqrt(q - s^2 / n) * sqrt(n / (n - 1))
    f = n / (n - 1.0) if n > 1 else 1.0
    va = np.clip(qa[mask] - a[mask] ** 2 / n, 0, None) * f
    vb = np.clip(qb[mask] - b[mask] ** 2 / n, 0, None) * f
    sig = np.sqrt(va + vb)
    d = np.abs(a[mask] - b[mask])
    z = np.where(sig > 0, d / np.where(sig > 0, sig, 1.0), np.where(d > 0, np.inf, 0.0))
    rel = d / b[mask]
    return {
        "integral_rel": integral,
        "voxels": int(mask.sum()),
        "within_2sigma": float(np.mean(z <= 2.0)),
        "max_z": float(z.max()),
        "median_z": float(np.median(z)),
        "median_rel": float(np.median(rel)),
        "equal": float(np.mean(d == 0)),
    }


def density_image(hu, voxel_materials, material_db):
    """Density (g/cm3) of each voxel from its HU interval (opengate/geometry/materials.py:294-324
    create_density_img): voxels in [hu0, hu1) get the density of that interval's material, voxels
    in no interval 0; float32."""
    hu = np.asarray(hu)
    rho = np.zeros(hu.shape, dtype=np.float32)
    for hu0, hu1, name in voxel_materials:
        rho[(hu >= hu0) & (hu < hu1)] = np.float32(material_db.get(name).density)
    return rho


def resample_linear(img, src_spacing, src_origin, dst_dims, dst_spacing, dst_origin, dst_direction=None,
                    default=0.0):
    """Linear resampling of an axis-aligned image onto another image's grid by physical position
    (resample_itk_image_like, opengate/image.py:532-557: ITK ResampleImageFilter with the identity
    transform and LinearInterpolateImageFunction).  The output voxel (i, j, k) sits at
    p = dst_origin + dst_direction @ ((i, j, k) * dst_spacing); its continuous index in the source
    is c = (p - src_origin) / src_spacing.  A point with c outside [-0.5, n - 0.5) on any axis gets
    `default`; inside, trilinear weights over the eight neighbours, their indices clamped to the
    image.  img [z][y][x]; spacings, origins and dims in x, y, z order; returns [z][y][x] float64."""
    img = np.asarray(img, dtype=np.float64)
    n = np.array(img.shape[::-1], dtype=np.int64)
    dims = [int(v) for v in dst_dims]
    sp_s, o_s = np.asarray(src_spacing, np.float64), np.asarray(src_origin, np.float64)
    sp_d, o_d = np.asarray(dst_spacing, np.float64), np.asarray(dst_origin, np.float64)
    rot = np.eye(3) if dst_direction is None else np.asarray(dst_direction, np.float64).reshape(3, 3)
    flat = img.ravel()
    out = np.empty((dims[2], dims[1], dims[0]), dtype=np.float64)
    jj, ii = np.meshgrid(np.arange(dims[1]), np.arange(dims[0]), indexing="ij")
    for k in range(dims[2]):  # one output slice at a time keeps the work arrays small
        idx = np.stack([ii, jj, np.full_like(ii, k)], axis=-1) * sp_d
        c = (o_d + idx @ rot.T - o_s) / sp_s  # [y][x][3]
        ok = np.all((c >= -0.5) & (c < n - 0.5), axis=-1)
        i0 = np.floor(c).astype(np.int64)
        f = c - i0
        lo, hi = np.clip(i0, 0, n - 1), np.clip(i0 + 1, 0, n - 1)
        acc = np.zeros(ok.shape, dtype=np.float64)
        for bz in (0, 1):
            for by in (0, 1):
                for bx in (0, 1):
                    w = np.ones(ok.shape)
                    at = []
                    for a, b in ((0, bx), (1, by), (2, bz)):
                        w = w * (f[..., a] if b else 1.0 - f[..., a])
                        at.append(hi[..., a] if b else lo[..., a])
                    acc += w * flat[(at[2] * n[1] + at[1]) * n[0] + at[0]]
        acc[~ok] = default
        out[k] = acc
    return out
