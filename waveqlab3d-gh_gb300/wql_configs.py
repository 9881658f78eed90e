"""Seeded synthetic workloads in the reference's `.in` format.

The reference ships fixed input files and offline generators (Matlab
inputfile/*.m for fault and topography surfaces, python/vonKarman_3D.py for
random media) whose outputs it reads from disk.  This module generates the
same kinds of inputs from a seed, in memory, and returns `.in` text plus the
arrays for wql_scenario_create_ex:

  config 0  2 x 41^3 Cartesian, TPV5 slip-weakening, 200 steps (CPU-runnable)
  config 1  2 x 201^3 curvilinear, Gaussian-correlated topography, self-similar
            rough fault, aging-law rate and state, Gaussian overstress, 2000 steps
  config 2  2 x 401x201x201, 20-point PML on 5 sides, von Karman medium,
            Drucker-Prager viscoplasticity, depth-dependent stress, slip weakening
  upwind    2 x 76x101x151 Cartesian, upwind SBP-6, 12-point PML, locked
            interface, one moment-tensor point source (the block shapes of the
            reference's PML study with the upwind operators), optionally with
            the anelastic response
"""
import math

import numpy as np

RHO, CS, CP = 2.67, 3.464, 6.0


def _problem(name, problem, coupling, mesh, t_final, extra=""):
    return (f"&problem_list\n name = '{name}',\n problem = '{problem}',\n nblocks = 2,\n"
            f" t_final = {t_final!r},\n CFL = 0.5d0,\n coupling = '{coupling}',\n"
            f" type_of_mesh = '{mesh}',\n w_stride = 1,\n w_fault = F{extra} /\n")


def _block(b, n, a, bb, lqrs, rqrs, pml_l=None, pml_r=None, npml=0):
    s = (f"btp({b})%nqrs = {n[0]}, {n[1]}, {n[2]},\n"
         f"btp({b})%aqrs = {a[0]!r}, {a[1]!r}, {a[2]!r},\n"
         f"btp({b})%bqrs = {bb[0]!r}, {bb[1]!r}, {bb[2]!r},\n"
         f"btp({b})%rho_s_p = {RHO!r}, {CS!r}, {CP!r},\n"
         f"btp({b})%lqrs = {lqrs[0]}, {lqrs[1]}, {lqrs[2]},\n"
         f"btp({b})%rqrs = {rqrs[0]}, {rqrs[1]}, {rqrs[2]},\n")
    if pml_l is not None:
        tf = lambda v: "T" if v else "F"  # noqa: E731
        s += (f"btp({b})%pml_lqrs = {', '.join(tf(v) for v in pml_l)},\n"
              f"btp({b})%pml_rqrs = {', '.join(tf(v) for v in pml_r)},\n"
              f"btp({b})%npml = {npml},\n")
    return s


def dt_of(n, extent):
    """Time step of src/block.f90:437-452 (CFL 0.5)."""
    h = min(e / (k - 1) for e, k in zip(extent, n))
    return 0.5 * h / math.sqrt(CS * CS + CP * CP)


# ----------------------------------------------------------------- fields ----

def gaussian_surface(shape, spacing, corr_len, rms, seed):
    """Gaussian-correlated random surface (autocorrelation exp(-r^2/l^2)):
    white noise filtered in Fourier space by exp(-k^2 l^2 / 8), scaled to rms."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    k = [2 * np.pi * np.fft.fftfreq(n, d) for n, d in zip(shape, spacing)]
    K2 = sum(np.meshgrid(*[kk * kk for kk in k], indexing="ij"))
    f = np.real(np.fft.ifftn(np.fft.fftn(w) * np.exp(-K2 * corr_len ** 2 / 8.0)))
    f -= f.mean()
    return f * (rms / f.std())


def self_similar_surface(shape, spacing, alpha, lam_min, seed):
    """Self-similar (Hurst 1) rough surface: 2D power spectrum ~ k^-4, cut at
    k_max = 2 pi / lam_min, rms height = alpha * (longest side)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    k = [2 * np.pi * np.fft.fftfreq(n, d) for n, d in zip(shape, spacing)]
    K = np.sqrt(sum(np.meshgrid(*[kk * kk for kk in k], indexing="ij")))
    kmin = 2 * np.pi / max(n * d for n, d in zip(shape, spacing))
    amp = np.where((K > 0) & (K <= 2 * np.pi / lam_min), np.maximum(K, kmin) ** -2.0, 0.0)
    f = np.real(np.fft.ifftn(np.fft.fftn(w) * amp))
    f -= f.mean()
    L = max((n - 1) * d for n, d in zip(shape, spacing))
    return f * (alpha * L / f.std())


def von_karman(shape, spacing, corr_len, hurst, std, seed, kmax=None):
    """3D von Karman random field with PSD ~ (1 + k^2 a^2)^-(H + 3/2), unit
    variance scaled to `std`, cut at kmax (the method of
    python/vonKarman_3D.py, seeded)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape).astype(np.float64)
    k = [2 * np.pi * np.fft.fftfreq(n, d) for n, d in zip(shape, spacing)]
    K2 = sum(np.meshgrid(*[kk * kk for kk in k], indexing="ij", sparse=True))
    psd = (1.0 + K2 * corr_len ** 2) ** (-(hurst + 1.5))
    if kmax is not None:
        psd = np.where(K2 <= kmax * kmax, psd, 0.0)
    spec = np.fft.fftn(w) * np.sqrt(psd)
    spec.flat[0] = 0.0
    f = np.real(np.fft.ifftn(spec))
    return f * (std / f.std())


def nafe_drake_rho(cp):
    """Density from P velocity (the polynomial used by python/vonKarman_3D.py)."""
    return 1.6612 * cp - 0.4721 * cp ** 2 + 0.0671 * cp ** 3 - 0.0043 * cp ** 4 + 0.000106 * cp ** 5


# ---------------------------------------------------------------- configs ----

def config0(steps=200):
    """2 x 41^3 Cartesian blocks over 20 x 10 x 10 km, planar fault at x = 10 km,
    TPV5 slip weakening (IC:1283-1299, 1822-1831), CFL 0.5."""
    n = (41, 41, 41)
    dt = dt_of(n, (10.0, 10.0, 10.0))
    text = _problem("config0", "TPV5", "slip-weakening_friction", "cartesian", (steps + 0.5) * dt)
    text += "&block_list\n" + _block(1, n, (0.0, 0.0, -5.0), (10.0, 10.0, 5.0), (1, 2, 1), (0, 1, 1))
    text += _block(2, n, (10.0, 0.0, -5.0), (20.0, 10.0, 5.0), (0, 2, 1), (1, 1, 1)) + " /\n"
    return text, None


def config1(n=201, steps=2000, seed=2239):
    """2 x n^3 curvilinear blocks, (-15,0,-7.5)-(0,15,7.5) and (0,0,-7.5)-(15,15,7.5) km;
    seeded topography (l = 1 km, rms 150 m) on the y = 0 free surface, self-similar
    fault (alpha = 0.01, lambda_min = 200 m), aging-law rate and state with uniform
    a = 0.008, b = 0.012, V0 = 1e-6, f0 = 0.6, L = 0.02, Vini = 1e-12, stress
    (-120, 0, -120, 0, 75, 0) MPa and a 25 MPa Gaussian overstress (R = 1.5 km)
    at (y, z) = (7.5, 0) ramped over 1 s."""
    ext = 15.0
    h = ext / (n - 1)
    dt = dt_of((n, n, n), (ext, ext, ext))
    text = _problem("config1", "rs_param", "rate-and-state_friction", "curvilinear", (steps + 0.5) * dt)
    text += "&block_list\n" + _block(1, (n, n, n), (-ext, 0.0, -ext / 2), (0.0, ext, ext / 2), (1, 2, 1), (0, 1, 1))
    text += _block(2, (n, n, n), (0.0, 0.0, -ext / 2), (ext, ext, ext / 2), (0, 2, 1), (1, 1, 1)) + " /\n"
    text += ("&fault_list\n a = 0.008d0, b = 0.012d0, V0 = 1d-6, f0 = 0.6d0, L = 0.02d0, Vini = 1d-12,\n"
             " s0 = -120d0, 0d0, -120d0, 0d0, 75d0, 0d0,\n"
             " nuc_amp = 25d0, nuc_radius = 1.5d0, nuc_y = 7.5d0, nuc_z = 0d0, nuc_rise = 1d0 /\n")
    # topography over the whole x range (2n-1 points), split at the fault
    topo = gaussian_surface((2 * n - 1, n), (h, h), 1.0, 0.15, seed)
    topo0 = np.asfortranarray(topo[:n, :])       # (q, s) for block 1
    topo1 = np.asfortranarray(topo[n - 1:, :])   # block 2 shares the fault column
    # fault surface on (r, s); zero it near the free surface edge so the
    # interface and the topography meet consistently
    fault = self_similar_surface((n, n), (h, h), 0.01, 0.2, seed + 1)
    media = {
        "fault_offset": np.asfortranarray(fault).ravel(order="F"),
        "topo_offset": (topo0.ravel(order="F"), topo1.ravel(order="F")),
    }
    return text, media


def config2(nq=401, nrs=201, steps=3000, seed=2239, npml=20):
    """2 x nq x nrs x nrs blocks, (-20,0,-5)-(0,10,5) and (0,0,-5)-(20,10,5) km,
    20-point PML on the 5 non-free-surface outer sides, von Karman medium (a = 2 km,
    H = 0.2, 5 % on cp and cs, rho from cp), scec viscoplasticity (c = 1 MPa,
    friction 0.75, Tv = 0.03 s), TPV26 depth-dependent stress, linear slip weakening
    (the config-0 law with the TPV26 preset's fs 0.18, fd 0.12, Dc 0.3 m) and a
    20 MPa Gaussian overstress (R = 1.5 km) at 7.5 km depth."""
    ext = (20.0, 10.0, 10.0)
    h = ext[0] / (nq - 1)
    dt = dt_of((nq, nrs, nrs), ext)
    extra = ",\n response = 'plastic',\n plastic_model = 'scec'"
    text = _problem("config2", "sw_param", "slip-weakening_friction", "curvilinear", (steps + 0.5) * dt, extra)
    text += "&block_list\n" + _block(1, (nq, nrs, nrs), (-20.0, 0.0, -5.0), (0.0, 10.0, 5.0), (1, 2, 1), (0, 1, 1),
                                     (True, False, True), (False, True, True), npml)
    text += _block(2, (nq, nrs, nrs), (0.0, 0.0, -5.0), (20.0, 10.0, 5.0), (0, 2, 1), (1, 1, 1),
                   (False, False, True), (True, True, True), npml) + " /\n"
    # the linear slip-weakening law of config 0 with the TPV26 preset's own
    # parameters (src/Interface_Condition.f90:1378-1380): under the TPV26
    # stress (tau/sigma_n about 0.16) config 0's fs = 0.677, fd = 0.525 never slip
    text += ("&fault_list\n fs = 0.18d0, fd = 0.12d0, Dc = 0.3d0, stress_profile = 'TPV26',\n"
             " nuc_amp = 20d0, nuc_radius = 1.5d0, nuc_y = 7.5d0, nuc_z = 0d0, nuc_rise = 0d0 /\n"
             "&plastic_list\n cohesion = 1d0, friction = 0.75d0, Tv = 0.03d0 /\n")
    r = von_karman((2 * nq - 1, nrs, nrs), (h, h, h), 2.0, 0.2, 0.05, seed, kmax=np.pi / h)
    media = {"lam": [], "mu": [], "rho": []}
    for b in range(2):
        sl = r[:nq] if b == 0 else r[nq - 1:]
        cp = CP * (1.0 + sl)
        cs = CS * (1.0 + sl)
        rho = nafe_drake_rho(cp)
        mu = rho * cs * cs
        lam = rho * cp * cp - 2.0 * mu
        for key, val in (("lam", lam), ("mu", mu), ("rho", rho)):
            media[key].append(np.asfortranarray(val).ravel(order="F"))
    media = {k: tuple(v) for k, v in media.items()}
    return text, media


def upwind_pml12(steps=2000, nq=76, nr=101, ns=151, anelastic=False):
    """2 x nq x nr x ns Cartesian blocks, (0,0,0)-(15,20,30) and (15,0,0)-(30,20,30)
    km, the upwind SBP operators of order 6, a 12-point PML on every outer side
    but the y = 0 free surface, a locked interface at x = 15 km and one
    Cos-Bell moment-tensor source (M_xz = -10) at (5, 1.8, 5) km, order-4
    discrete delta.  anelastic: response = 'anelastic' with c = 2, weight_exp =
    0.6, fref = 1 Hz (the reference's PML study with attenuation)."""
    ext = (15.0, 20.0, 30.0)
    dt = dt_of((nq, nr, ns), ext)
    extra = ",\n fd_type = 'upwind',\n order = 6" + (",\n response = 'anelastic'" if anelastic else "")
    text = _problem("upwind_pml12", "TPV5", "locked", "cartesian", (steps + 0.5) * dt, extra)
    n = (nq, nr, ns)
    text += "&block_list\n" + _block(1, n, (0.0, 0.0, 0.0), (15.0, 20.0, 30.0), (1, 2, 1), (0, 1, 1),
                                     (True, False, True), (False, True, True), 12)
    text += _block(2, n, (15.0, 0.0, 0.0), (30.0, 20.0, 30.0), (0, 2, 1), (1, 1, 1),
                   (False, False, True), (True, True, True), 12) + " /\n"
    text += ("&moment_list\n use_moment_tensor = T,\n order = 4 /\n"
             "!---begin:tensor_listU---\n"
             "'Cos-Bell' 0d0 0.2d0 0d0 0d0 0d0 0d0 -10d0 0d0 5d0 1.8d0 5d0 0\n"
             "!---end:tensor_listU---\n"
             "!---begin:tensor_listV---\n!---end:tensor_listV---\n")
    if anelastic:
        text += "&anelastic_list\n c = 2d0,\n weight_exp = 0.6d0,\n fref = 1d0 /\n"
    return text, None


def updates_per_step(text):
    """Grid-point RK-stage updates per time step: sum of nq*nr*ns x 5 stages."""
    import re
    tot = 0
    for m in re.finditer(r"btp\(\d\)%nqrs\s*=\s*(\d+),\s*(\d+),\s*(\d+)", text):
        tot += int(m.group(1)) * int(m.group(2)) * int(m.group(3))
    return 5 * tot


# --------------------------------------------------- served point sources ----

def moment_tensor(strike, dip, rake, m0):
    """Moment tensor (XX, YY, ZZ, XY, XZ, YZ) of a double couple in the frame
    x = east, y = down, z = north, from strike/dip/rake in degrees (the
    Aki-Richards expressions in north-east-down, with the axes permuted)."""
    f, d, l = (np.radians(v) for v in (strike, dip, rake))
    nn = -m0 * (np.sin(d) * np.cos(l) * np.sin(2 * f) + np.sin(2 * d) * np.sin(l) * np.sin(f) ** 2)
    ne = m0 * (np.sin(d) * np.cos(l) * np.cos(2 * f) + 0.5 * np.sin(2 * d) * np.sin(l) * np.sin(2 * f))
    nd = -m0 * (np.cos(d) * np.cos(l) * np.cos(f) + np.cos(2 * d) * np.sin(l) * np.sin(f))
    ee = m0 * (np.sin(d) * np.cos(l) * np.sin(2 * f) - np.sin(2 * d) * np.sin(l) * np.cos(f) ** 2)
    ed = -m0 * (np.cos(d) * np.cos(l) * np.sin(f) - np.cos(2 * d) * np.sin(l) * np.cos(f))
    dd = m0 * np.sin(2 * d) * np.sin(l)
    return ee, dd, nn, ed, ne, nd


def config4_request(i, seed=4242, n_lo=96, n_hi=256, steps=100, medium=None):
    """Request i of the served stream: an n^3 grid (n uniform in n_lo..n_hi)
    as two blocks joined by a locked interface at x = 0, absorbing sides and
    a free surface at y = 0, a double-couple point source (strike 0-360,
    dip 10-90, rake -180-180, Mw 4-6 -> M0 = 10^(1.5 Mw + 9.1) N m, in
    MPa km^3 = 1e15 N m) with a Gaussian moment rate of rise time 0.1-0.5 s
    at 2-15 km depth, and 32 seeded stations on the free surface.  The
    domain is a cube of side max(depth + 5, 12) km.  `medium`, if given, is a
    von Karman perturbation field at least n^3, cropped to the grid."""
    rng = np.random.default_rng([seed, i])
    n = int(rng.integers(n_lo, n_hi + 1))
    depth = float(rng.uniform(2.0, 15.0))
    side = max(depth + 5.0, 12.0)
    strike, dip, rake = rng.uniform(0, 360), rng.uniform(10, 90), rng.uniform(-180, 180)
    mw = rng.uniform(4.0, 6.0)
    m0 = 10 ** (1.5 * mw + 9.1) / 1e15
    rise = rng.uniform(0.1, 0.5)
    w = 2.0 / rise
    t0 = 1.5 * rise
    mt = moment_tensor(strike, dip, rake, m0)
    h = side / (n - 1)
    nq1 = n // 2 + 1
    nq2 = n - nq1 + 1
    x1 = -h * (nq1 - 1)
    x2 = h * (nq2 - 1)
    # source inside block 1, off the grid points
    sx = float(rng.uniform(0.3, 0.7)) * x1
    sz = float(rng.uniform(-0.2, 0.2)) * side
    dt = 0.5 * h / math.sqrt(CS * CS + CP * CP)
    text = (f"&problem_list\n name = 'request{i}',\n problem = 'TPV5',\n nblocks = 2,\n"
            f" t_final = {(steps + 0.5) * dt!r},\n CFL = 0.5d0,\n coupling = 'locked',\n"
            f" type_of_mesh = 'cartesian',\n w_stride = 1,\n w_fault = F /\n")
    text += "&block_list\n" + _block(1, (nq1, n, n), (x1, 0.0, -side / 2), (0.0, side, side / 2), (1, 2, 1), (0, 1, 1))
    text += _block(2, (nq2, n, n), (0.0, 0.0, -side / 2), (x2, side, side / 2), (0, 2, 1), (1, 1, 1)) + " /\n"
    text += "&moment_list\n use_moment_tensor = T,\n order = 2 /\n"
    text += "!---begin:tensor_listU---\n"
    text += (f"'gaussian' {w!r} {t0!r} " + " ".join(repr(float(v)) for v in mt) +
             f" {sx!r} {depth!r} {sz!r} 0\n")
    text += "!---end:tensor_listU---\n"
    text += "&output_list\n output_seismograms = T /\n!---begin:station_list---\n"
    for k in range(32):
        text += f"{rng.uniform(x1, x2)!r} 0d0 {rng.uniform(-side / 2, side / 2)!r}\n"
    text += "!---end:station_list---\n"
    media = None
    if medium is not None:
        sl = medium[:n, :n, :n]
        media = {"lam": [], "mu": [], "rho": []}
        for b, (q0, nq) in enumerate(((0, nq1), (nq1 - 1, nq2))):
            p = sl[q0:q0 + nq]
            cp, cs = CP * (1.0 + p), CS * (1.0 + p)
            rho = nafe_drake_rho(cp)
            mu = rho * cs * cs
            lam = rho * cp * cp - 2.0 * mu
            for key, val in (("lam", lam), ("mu", mu), ("rho", rho)):
                media[key].append(np.asfortranarray(val).ravel(order="F"))
        media = {k: tuple(v) for k, v in media.items()}
    return text, media, n


def config4_medium(n=256, seed=4242, h=0.05):
    """One von Karman perturbation field (a = 2 km, H = 0.2, 5 %) that the
    requests crop to their size."""
    return von_karman((n, n, n), (h, h, h), 2.0, 0.2, 0.05, seed, kmax=np.pi / h)


# --------------------------------------------------- batched ensemble ----

def config3_scenario(i, seed=3131, n_lo=64, n_hi=160, steps=1500, medium=None, npml=10):
    """Member i of the batched ensemble: blocks of n^3 points (n^3 uniform in
    n_lo^3..n_hi^3), 15 km deep, slip weakening (fs 0.677, fd 0.525,
    Dc 0.4 m) under sigma_n = 120 MPa and tau_0 = fd*sigma_n + (fs - fd)*
    sigma_n/(1 + S) with S uniform in [0.5, 1.5], a nucleation patch
    (R = 1.5 km, just above peak strength) centred at a depth of 2-12 km
    and uniform along strike, a planar fault (Cartesian mesh) or a rough
    one (alpha 0.005-0.01, curvilinear mesh), a homogeneous or von Karman
    medium (cropped from `medium`), and npml-point PML on the five sides
    other than the free surface."""
    rng = np.random.default_rng([seed, i])
    n = int(np.floor(rng.uniform(n_lo ** 3, n_hi ** 3) ** (1.0 / 3.0)))
    h = 15.0 / (n - 1)
    ext = (n - 1) * h
    S = rng.uniform(0.5, 1.5)
    fs, fd, sn = 0.677, 0.525, 120.0
    tau0 = fd * sn + (fs - fd) * sn / (1.0 + S)
    ny = rng.uniform(2.0, 12.0)
    nz = rng.uniform(-0.35, 0.35) * ext
    rough = bool(rng.integers(0, 2))
    hetero = bool(rng.integers(0, 2)) and medium is not None
    mesh = "curvilinear" if rough else "cartesian"
    dt = dt_of((n, n, n), (ext, ext, ext))
    text = _problem(f"member{i}", "sw_param", "slip-weakening_friction", mesh, (steps + 0.5) * dt)
    text += "&block_list\n" + _block(1, (n, n, n), (-ext, 0.0, -ext / 2), (0.0, ext, ext / 2), (1, 2, 1), (0, 1, 1),
                                     (True, False, True), (False, True, True), npml)
    text += _block(2, (n, n, n), (0.0, 0.0, -ext / 2), (ext, ext, ext / 2), (0, 2, 1), (1, 1, 1),
                   (False, False, True), (True, True, True), npml) + " /\n"
    amp = (fs * sn - tau0) + 1.0
    text += (f"&fault_list\n fs = {fs}d0, fd = {fd}d0, Dc = 0.4d0,\n"
             f" s0 = -120d0, 0d0, -120d0, 0d0, {tau0!r}, 0d0,\n"
             f" nuc_amp = {amp!r}, nuc_radius = 1.5d0, nuc_y = {ny!r}, nuc_z = {nz!r}, nuc_rise = 0d0 /\n")
    media = {}
    if rough:
        alpha = rng.uniform(0.005, 0.01)
        fault = self_similar_surface((n, n), (h, h), alpha, max(2 * h, 0.2), seed + 7 * i + 1)
        media["fault_offset"] = np.asfortranarray(fault).ravel(order="F")
    if hetero:
        m = {"lam": [], "mu": [], "rho": []}
        for b in range(2):
            p = medium[b * (n - 1): b * (n - 1) + n, :n, :n] if medium.shape[0] >= 2 * n - 1 else medium[:n, :n, :n]
            cp, cs = CP * (1.0 + p), CS * (1.0 + p)
            rho = nafe_drake_rho(cp)
            mu = rho * cs * cs
            lam = rho * cp * cp - 2.0 * mu
            for key, val in (("lam", lam), ("mu", mu), ("rho", rho)):
                m[key].append(np.asfortranarray(val).ravel(order="F"))
        media.update({k: tuple(v) for k, v in m.items()})
    return text, (media or None), 2 * n ** 3
