"""Per-element photon cross sections for the G4EmStandardPhysics (option 0) processes.

The reference selects its photon physics by name (``physics_list_name =
"G4EmStandardPhysics"``, opengate/physics.py:341-347) and leaves every model to
Geant4 11.4.2, which is not part of the opengate sources.  The models of that
list, and the way this module restates each one, are:

* Compton scattering, G4KleinNishinaCompton: the empirical per-atom cross
  section published in the Geant4 Physics Reference Manual (section "Compton
  scattering", fit to the Storm-Israel / Hubbell data), restated in
  :func:`compton_per_atom`.
* Gamma conversion, G4BetheHeitler5D (cross section of G4BetheHeitlerModel):
  the parameterised per-atom formula of the Physics Reference Manual (section
  "Gamma conversion", valid above 1.5 MeV, quadratic threshold correction
  below), restated in :func:`pair_per_atom`.
* Rayleigh scattering, G4LivermoreRayleighModel: Livermore form factors are not
  available offline, so the coherent cross section and its angular law are
  computed from the independent-atom form factor of Slater-type orbitals
  (screening constants by Slater's rules), :func:`form_factor`.
* Photoelectric effect, G4LivermorePhotoElectricModel: the remainder of the
  NIST total attenuation coefficient (the data opengate ships in
  GateMuDatabase.h) after Compton, Rayleigh and pair, clamped at zero.

The total attenuation therefore reproduces the NIST tables wherever the
remainder is non-negative; the split between processes follows the published
parameterisations above.  Mass coefficients are in cm2/g, energies in MeV.
"""

import functools
import pathlib

import numpy as np

ELECTRON_MASS_MEV = 0.51099895
AVOGADRO = 6.02214076e23
BARN_CM2 = 1e-24
CLASSICAL_ELECTRON_RADIUS_CM = 2.8179403262e-13
HC_MEV_ANGSTROM = 12.398419843320026e-3  # h*c in MeV * Angstrom
BOHR_ANGSTROM = 0.529177210903

_DATA = pathlib.Path(__file__).with_name("data") / "elements_nist.npz"


@functools.lru_cache(maxsize=1)
def element_data():
    d = np.load(_DATA)
    return {k: d[k] for k in d.files}


def atomic_mass(z):
    return float(element_data()["atomic_mass"][z - 1])


def symbol(z):
    return str(element_data()["symbols"][z - 1])


def z_of_symbol(sym):
    syms = list(element_data()["symbols"])
    return syms.index(sym) + 1


def nist_mu_rho(z, energy, absorption=False):
    """NIST mass attenuation (or energy-absorption) coefficient of element ``z``.

    Restates the interpolation of ``PhotonAttenuationEl``
    (opengate/data/PhotonAttenuation.py:8556-8629): log-log PCHIP through the
    36-point grid; for Z > 10 the absorption edges are inserted as two points
    4 ulp either side of the edge energy, and near those points (the edge pair
    and its grid neighbours) the PCHIP value is blended with the log-log linear
    one using the linearly interpolated edge-marker weight.
    """
    from scipy.interpolate import interp1d, pchip_interpolate

    d = element_data()
    grid = d["energy"]
    y = (d["meac"] if absorption else d["mac"])[z - 1]
    lq = np.log(np.atleast_1d(np.asarray(energy, dtype=np.float64)))
    if z <= 10:
        return np.exp(pchip_interpolate(np.log(grid), np.log(y), lq))
    ed = d["edges"][d["edges"][:, 0] == z]
    e = ed[:, 1]
    dd = 4 * np.spacing(e)
    xx = np.concatenate([e - dd, e + dd])
    yy = np.concatenate([ed[:, 4], ed[:, 5]] if absorption else [ed[:, 2], ed[:, 3]])
    w = np.concatenate([np.zeros(len(grid)), np.ones(2 * len(e))])
    x = np.concatenate([np.log(grid), np.log(xx)])
    ly = np.concatenate([np.log(y), np.log(yy)])
    order = np.argsort(x, kind="stable")
    x, ly, w = x[order], ly[order], w[order]
    w = (np.convolve(w, [1, 1, 1], "same") > 0).astype(np.float64)

    def lin(xq, yp):
        out = interp1d(x, yp, kind="linear", bounds_error=False)(xq)
        out = np.where(xq < x[0], yp[0] + (xq - x[0]) * (yp[0] - yp[1]) / (x[0] - x[1]), out)
        return np.where(xq > x[-1], yp[-1] + (xq - x[-1]) * (yp[-1] - yp[-2]) / (x[-1] - x[-2]), out)

    b1 = lin(lq, ly)
    v = lin(lq, w)
    a = pchip_interpolate(x, ly, lq)
    return np.exp(a * (1 - v) + b1 * v)


def _per_atom_to_mass(z, sigma_barn):
    return sigma_barn * BARN_CM2 * AVOGADRO / atomic_mass(z)


# ---------------------------------------------------------------------------
# Compton: empirical cross section of the Geant4 Physics Reference Manual
# sigma(Z, E) = P1(Z) ln(1+2X)/X + (P2 + P3 X + P4 X^2)/(1 + a X + b X^2 + c X^3)
# with X = E / m_e c^2 and Pi(Z) = Z (d_i + e_i Z + f_i Z^2) in barn.
# Below T0 (15 keV, 40 keV for hydrogen) the value at T0 is extrapolated with
# exp(-y (c1 + c2 y)), y = ln(E/T0), matching the slope over [T0, T0 + 1 keV].
# ---------------------------------------------------------------------------
_KN_D = (2.7965e-1, -1.8300e-1, 6.7527, -1.9798e1)
_KN_E = (1.9756e-5, -1.0205e-2, -7.3913e-2, 2.7079e-2)
_KN_F = (-3.9178e-7, 6.8241e-5, 6.0480e-5, 3.0274e-4)
_KN_ABC = (20.0, 230.0, 440.0)


def _kn_fit(z, x):
    p = [z * (_KN_D[i] + _KN_E[i] * z + _KN_F[i] * z * z) for i in range(4)]
    a, b, c = _KN_ABC
    return p[0] * np.log1p(2.0 * x) / x + (p[1] + p[2] * x + p[3] * x * x) / (
        1.0 + a * x + b * x * x + c * x * x * x
    )


def compton_per_atom(z, energy):
    """Compton cross section per atom in barn."""
    energy = np.atleast_1d(np.asarray(energy, dtype=np.float64))
    t0 = 40e-3 if z < 1.5 else 15e-3
    x = np.maximum(energy, t0) / ELECTRON_MASS_MEV
    sig = _kn_fit(z, x)
    low = energy < t0
    if np.any(low):
        dt0 = 1e-3
        s0 = _kn_fit(z, np.array([t0 / ELECTRON_MASS_MEV]))[0]
        s1 = _kn_fit(z, np.array([(t0 + dt0) / ELECTRON_MASS_MEV]))[0]
        c1 = -t0 * (s1 - s0) / (s0 * dt0)
        c2 = 0.150 if z < 1.5 else 0.375 - 0.0556 * np.log(z)
        y = np.log(energy[low] / t0)
        sig = sig.copy()
        sig[low] = s0 * np.exp(-y * (c1 + c2 * y))
    return np.maximum(sig, 0.0)


# ---------------------------------------------------------------------------
# Pair production: parameterised Bethe-Heitler cross section of the Geant4
# Physics Reference Manual, sigma = (Z+1) Z [F1(X) + F2(X) Z + F3(X)/Z],
# X = ln(E / m_e c^2), Fi fifth-order polynomials (coefficients in microbarn),
# evaluated at max(E, 1.5 MeV) and scaled by ((E - 2m)/(1.5 MeV - 2m))^2 below.
# ---------------------------------------------------------------------------
_BH_A = (8.7842e2, -1.9625e3, 1.2949e3, -2.0028e2, 1.2575e1, -2.8333e-1)
_BH_B = (-1.0342e1, 1.7692e1, -8.2381, 1.3063, -9.0815e-2, 2.3586e-3)
_BH_C = (-4.5263e2, 1.1161e3, -8.6749e2, 2.1773e2, -2.0467e1, 6.5372e-1)
_BH_LIMIT = 1.5


def pair_per_atom(z, energy):
    """Pair-production cross section per atom in barn."""
    energy = np.atleast_1d(np.asarray(energy, dtype=np.float64))
    thr = 2.0 * ELECTRON_MASS_MEV
    e = np.maximum(energy, _BH_LIMIT)
    x = np.log(e / ELECTRON_MASS_MEV)
    powers = np.stack([x**k for k in range(6)])
    f1 = np.tensordot(_BH_A, powers, 1)
    f2 = np.tensordot(_BH_B, powers, 1)
    f3 = np.tensordot(_BH_C, powers, 1)
    sig = (z + 1.0) * z * (f1 + f2 * z + f3 / z) * 1e-6  # microbarn -> barn
    below = energy < _BH_LIMIT
    scale = np.where(below, ((energy - thr) / (_BH_LIMIT - thr)) ** 2, 1.0)
    sig = np.where(energy <= thr, 0.0, sig * scale)
    return np.maximum(sig, 0.0)


# ---------------------------------------------------------------------------
# Rayleigh: independent-atom form factor from Slater-type orbitals.
# ---------------------------------------------------------------------------
_AUFBAU = [
    (1, 0, 2), (2, 0, 2), (2, 1, 6), (3, 0, 2), (3, 1, 6), (4, 0, 2), (3, 2, 10),
    (4, 1, 6), (5, 0, 2), (4, 2, 10), (5, 1, 6), (6, 0, 2), (4, 3, 14), (5, 2, 10),
    (6, 1, 6), (7, 0, 2), (5, 3, 14), (6, 2, 10), (7, 1, 6),
]
_NSTAR = {1: 1.0, 2: 2.0, 3: 3.0, 4: 3.7, 5: 4.0, 6: 4.2, 7: 4.2}


def _slater_groups(z):
    """Return [(n, kind, count)] Slater groups in order; kind 'sp', 'd' or 'f'."""
    occ = {}
    left = z
    for n, l, cap in _AUFBAU:
        if left <= 0:
            break
        k = min(cap, left)
        left -= k
        kind = "sp" if l <= 1 else ("d" if l == 2 else "f")
        occ[(n, kind)] = occ.get((n, kind), 0) + k
    order = []
    for n in range(1, 8):
        for kind in ("sp", "d", "f"):
            if (n, kind) in occ:
                order.append((n, kind, occ[(n, kind)]))
    return order


def _slater_zeff(z):
    groups = _slater_groups(z)
    out = []
    for gi, (n, kind, cnt) in enumerate(groups):
        s = (cnt - 1) * (0.30 if n == 1 else 0.35)
        for gj, (n2, kind2, cnt2) in enumerate(groups):
            if gj >= gi:
                continue
            if kind == "sp":
                if n2 == n - 1:
                    s += 0.85 * cnt2
                elif n2 <= n - 2:
                    s += 1.00 * cnt2
                elif n2 == n:  # lower group of the same shell (never for sp)
                    s += 0.35 * cnt2
            else:
                s += 1.00 * cnt2
        out.append((n, cnt, max(z - s, 0.1)))
    return out


def form_factor(z, x):
    """Atomic form factor F(x, Z); x = sin(theta/2)/lambda in 1/Angstrom."""
    x = np.asarray(x, dtype=np.float64)
    q = 4.0 * np.pi * x  # momentum transfer, 1/Angstrom
    f = np.zeros_like(q)
    for n, cnt, zeff in _slater_zeff(z):
        ns = _NSTAR[n]
        m = 2.0 * ns
        beta = 2.0 * zeff / (ns * BOHR_ANGSTROM)
        phi = np.arctan2(q, beta)
        with np.errstate(invalid="ignore", divide="ignore"):
            g = beta ** (m + 1) * np.sin(m * phi) / (m * q * (beta * beta + q * q) ** (m / 2))
        g = np.where(q < 1e-12, 1.0, g)
        f += cnt * g
    return f


# x^2 grid for the Rayleigh tables (1/Angstrom^2)
RAYL_X2_MIN = 1e-8
RAYL_X2_MAX = 1e7
RAYL_NX2 = 2048


def rayleigh_x2_grid():
    return np.geomspace(RAYL_X2_MIN, RAYL_X2_MAX, RAYL_NX2)


def rayleigh_cumulative(z_list, w_list):
    """Cumulative integral of F^2(x^2) dx^2 for a mixture (per gram).

    Returns (x2 grid, A(x2)) with A(0) = 0, where the mixture weight of element Z
    is its number of atoms per gram, w_Z N_A / A_Z.
    """
    x2 = rayleigh_x2_grid()
    f2 = np.zeros_like(x2)
    for z, w in zip(z_list, w_list):
        f2 += w * AVOGADRO / atomic_mass(z) * form_factor(z, np.sqrt(x2)) ** 2
    # trapezoid on the log grid, plus the [0, x2_min] piece with F = F(0)
    seg = 0.5 * (f2[1:] + f2[:-1]) * np.diff(x2)
    a = np.concatenate([[f2[0] * x2[0]], f2[0] * x2[0] + np.cumsum(seg)])
    return x2, a, f2


def rayleigh_mass(z_list, w_list, energy):
    """Rayleigh mass attenuation coefficient (cm2/g) of a mixture.

    sigma = pi r_e^2 (2/k^2) int_0^{k^2} (1 + cos^2 theta) F^2(x^2) dx^2,
    cos theta = 1 - 2 x^2 / k^2, k = E / hc.
    """
    energy = np.atleast_1d(np.asarray(energy, dtype=np.float64))
    x2, a, f2 = rayleigh_cumulative(z_list, w_list)
    # first moment integrals for the cos^2 term on the same grid
    out = np.empty_like(energy)
    for i, e in enumerate(energy):
        k2 = (e / HC_MEV_ANGSTROM) ** 2
        sel = x2 <= k2
        xs = np.concatenate([[0.0], x2[sel], [k2]])
        fs = np.concatenate([[f2[0]], f2[sel], [np.interp(k2, x2, f2)]])
        c = 1.0 - 2.0 * xs / k2
        integrand = (1.0 + c * c) * fs
        integral = np.sum(0.5 * (integrand[1:] + integrand[:-1]) * np.diff(xs))
        out[i] = np.pi * CLASSICAL_ELECTRON_RADIUS_CM**2 * 2.0 / k2 * integral
    return out


def element_partials(z, energy):
    """Mass coefficients (cm2/g) of one element: dict compton, photo, rayleigh, pair."""
    energy = np.atleast_1d(np.asarray(energy, dtype=np.float64))
    comp = _per_atom_to_mass(z, compton_per_atom(z, energy))
    pair = _per_atom_to_mass(z, pair_per_atom(z, energy))
    rayl = rayleigh_mass([z], [1.0], energy)
    tot = nist_mu_rho(z, energy)
    photo = np.maximum(tot - comp - rayl - pair, 0.0)
    return {"compton": comp, "photo": photo, "rayleigh": rayl, "pair": pair, "nist_total": tot}
