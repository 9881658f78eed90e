"""Input-file helpers shared by the tests."""
import os
import re

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_in(prefix):
    with open(os.path.join(GOLDEN, prefix + ".in")) as f:
        return f.read()


def with_groups(text, extra):
    """Append namelist groups (e.g. "&gb300_list bc_penalty='weighted' /")."""
    return text + "\n" + extra + "\n"


def set_key(text, key, value):
    """Replace `key = ...` inside &problem_list (first occurrence)."""
    pat = re.compile(r"(^\s*%s\s*=\s*)([^,\n/]*)" % re.escape(key), re.M)
    new, n = pat.subn(lambda m: m.group(1) + value, text, count=1)
    assert n == 1, key
    return new


def write(tmp_path, name, text):
    p = os.path.join(str(tmp_path), name)
    with open(p, "w") as f:
        f.write(text)
    return p


def block_list(nq=21, extra1="", extra2=""):
    """&block_list of the truth/1 geometry with optional extra lines."""
    return f"""&block_list
btp(1)%nqrs = {nq}, {nq}, {nq},
btp(1)%aqrs = -3d0, 6d0, -1.5d0,
btp(1)%bqrs = 0d0, 9d0, 1.5d0,
btp(1)%rho_s_p = 2.67d0, 3.464d0, 6d0,
btp(1)%lqrs = 1, 2, 1,
btp(1)%rqrs = 0, 1, 1,
{extra1}
btp(2)%nqrs = {nq}, {nq}, {nq},
btp(2)%aqrs = 0d0, 6d0, -1.5d0,
btp(2)%bqrs = 3d0, 9d0, 1.5d0,
btp(2)%rho_s_p = 2.67d0, 3.464d0, 6d0,
btp(2)%lqrs = 0, 2, 1,
btp(2)%rqrs = 1, 1, 1,
{extra2} /
"""


def problem(problem="TPV5", coupling="slip-weakening_friction", mesh="cartesian", t_final="0.5d0",
            extra="", w_fault="T"):
    return f"""&problem_list
 name = 'gen',
 problem = '{problem}',
 nblocks = 2,
 t_final = {t_final},
 CFL = 0.5d0,
 coupling = '{coupling}',
 type_of_mesh = '{mesh}',
 w_stride = 1,
 w_fault = {w_fault}{extra} /
"""


PML_BLOCKS = dict(
    extra1="btp(1)%pml_lqrs = T, F, T,\nbtp(1)%pml_rqrs = F, T, T,\nbtp(1)%npml = 7,",
    extra2="btp(2)%pml_lqrs = F, F, T,\nbtp(2)%pml_rqrs = T, T, T,\nbtp(2)%npml = 7,")


def case_text(name):
    """Synthetic parity cases beyond the reference fixtures."""
    if name == "pml":
        return problem() + block_list(25, **PML_BLOCKS)
    if name == "pml_curv":
        return problem(mesh="curvilinear") + block_list(25, **PML_BLOCKS)
    if name == "plastic":
        return (problem("TPV26", extra=",\n response = 'plastic',\n plastic_model = 'scec'") +
                block_list() + "&plastic_list\n cohesion = 0.5d0,\n friction = 0.02d0,\n Tv = 0.03d0 /\n")
    if name == "rs":
        return problem("TPV101", "rate-and-state_friction") + block_list()
    if name == "rs_curv":
        return problem("TPV101", "rate-and-state_friction", "curvilinear") + block_list()
    if name == "locked":
        return problem("TPV5", "locked") + block_list()
    if name in ("rw", "rw_curv"):
        # problem 'rate-weakening': slip law with flash weakening and a
        # Gaussian stress pulse at (y, z) = (8, 0) switched on at t > 0
        return problem("rate-weakening", "rate-and-state_friction",
                       "curvilinear" if name == "rw_curv" else "cartesian") + block_list()
    if name in ("rw_plastic", "rw_plastic_curv"):
        # the reference's default plastic model (plastic_flow) with the
        # mu_beta_eta of its plasticity.in deck
        mbe = "btp({})%mu_beta_eta = 0.5735d0, 0.2867d0, 0.2775d0,"
        mesh = "curvilinear" if name.endswith("_curv") else "cartesian"
        return (problem("rate-weakening", "rate-and-state_friction", mesh, extra=",\n response = 'plastic'") +
                block_list(extra1=mbe.format(1), extra2=mbe.format(2)))
    if name.startswith(("an_", "an0_")):
        # anelastic response (GSLS memory variables, src/material.f90:11-142)
        c, wexp = ("2.0d0", "0.6d0") if not name.startswith("an0_") else ("5.0d0", "0d0")
        base = case_text(name.split("_", 1)[1])
        base = base.replace(" w_stride = 1,", " w_stride = 1,\n response = 'anelastic',", 1)
        return base + f"&anelastic_list\n c = {c},\n weight_exp = {wexp},\n fref = 1d0 /\n"
    if name.startswith(("up_", "up5_")):
        # the upwind operators of order 6 or 5 (fd_type = 'upwind')
        order = 5 if name.startswith("up5_") else 6
        return case_text(name.split("_", 1)[1]).replace(
            " w_stride = 1,", f" w_stride = 1,\n fd_type = 'upwind',\n order = {order},", 1)
    if name.startswith("linear_"):
        # linear friction coupling, tau = alpha v with alpha = 1e14
        # (src/Interface_Condition.f90:639-742, called at :366), around the
        # point sources of the moment-tensor cases
        return case_text(name.split("_", 1)[1]).replace("coupling = 'locked'", "coupling = 'linear_friction'", 1)
    if name in MT_CASES:
        mesh, order, mollify, lists = MT_CASES[name]
        extra = ",\n mollify_source = T" if mollify else ""
        return (problem("TPV5", "locked", mesh, extra=extra) + block_list() +
                f"&moment_list\n use_moment_tensor = T,\n order = {order} /\n" + lists)
    raise KeyError(name)


# moment-tensor point sources in a locked two-block domain: per-block lists
# (order 4, Gaussian moment rate, off-grid positions), a unified list across
# both blocks (order 2, mixed time functions), and a mollified source
_MT_U = ("!---begin:tensor_listU---\n"
         "'gaussian' 20d0 0.1d0 1d0 0.5d0 -0.7d0 0.3d0 -0.2d0 0.4d0 -1.63d0 7.31d0 0.22d0 0\n"
         "!---end:tensor_listU---\n"
         "!---begin:tensor_listV---\n"
         "'Brune' 15d0 0d0 0d0 0d0 0d0 1d0 0d0 0d0 1.21d0 7.74d0 -0.37d0 0\n"
         "!---end:tensor_listV---\n")
_MT_UNIFIED = ("! source_type duration t_init mXX mYY mZZ mXY mXZ mYZ x y z alpha\n"
               "!---begin:tensor_list---\n"
               "'gaussian' 25d0 0.08d0 0d0 0d0 0d0 0d0 1d0 0d0 -1.07d0 7.5d0 0.05d0 0\n"
               "'cosine' 0.2d0 0d0 0.5d0 0.5d0 0.5d0 0d0 0d0 0d0 1.52d0 6.93d0 0.31d0 0\n"
               "!---end:tensor_list---\n")
MT_CASES = {
    "mt4": ("cartesian", 4, False, _MT_U),
    "mt4_curv": ("curvilinear", 4, False, _MT_U),
    "mt2_unified": ("cartesian", 2, False, _MT_UNIFIED),
    "mt_mollified": ("cartesian", 2, True, _MT_U),
}


def _smooth_surface(seed, amp, nmodes=3):
    """A seeded smooth surface: a sum of sine products with wavelengths of
    1.5-4 km, evaluated at any resolution (for convergence studies)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    modes = [(rng.uniform(1.5, 4.0), rng.uniform(1.5, 4.0), rng.uniform(0, 2 * np.pi),
              rng.uniform(0, 2 * np.pi), rng.uniform(0.5, 1.0)) for _ in range(nmodes)]

    def f(a, b):
        out = 0.0
        for la, lb, pa, pb, w in modes:
            out = out + w * np.sin(2 * np.pi * a / la + pa) * np.sin(2 * np.pi * b / lb + pb)
        return amp * out / nmodes
    return f


def mms_case(n, t_final=0.15, mesh="curvilinear", seed=7):
    """Manufactured-solution problem (&mms_list, src/mms.f90) on two n^3
    blocks (-2,0,-1)-(0,2,1) and (0,0,-1)-(2,2,1) km with a locked interface,
    absorbing and free-surface outer boundaries.  Curvilinear: the fault and
    the y = 0 free surface are displaced by seeded smooth surfaces (up to
    about 0.1 km), blended across the blocks.  Returns (text, media)."""
    import numpy as np
    text = f"""&problem_list
 name = 'mms', problem = 'TPV5', nblocks = 2, t_final = {t_final!r}, CFL = 0.5d0,
 coupling = 'locked', type_of_mesh = '{mesh}', w_stride = 1, w_fault = F /
&block_list
btp(1)%nqrs = {n}, {n}, {n},
btp(1)%aqrs = -2d0, 0d0, -1d0,
btp(1)%bqrs = 0d0, 2d0, 1d0,
btp(1)%rho_s_p = 2.67d0, 3.464d0, 6d0,
btp(1)%lqrs = 1, 2, 1,
btp(1)%rqrs = 0, 1, 1,
btp(2)%nqrs = {n}, {n}, {n},
btp(2)%aqrs = 0d0, 0d0, -1d0,
btp(2)%bqrs = 2d0, 2d0, 1d0,
btp(2)%rho_s_p = 2.67d0, 3.464d0, 6d0,
btp(2)%lqrs = 0, 2, 1,
btp(2)%rqrs = 1, 1, 1 /
&mms_list
 use_mms = T, nt = 2d0, nx = 1d0, ny = 1d0, nz = 1d0 /
"""
    if mesh != "curvilinear":
        return text, None
    fault, topo = _smooth_surface(seed, 0.08), _smooth_surface(seed + 1, 0.06)
    h = 2.0 / (n - 1)
    y = np.arange(n) * h
    z = -1.0 + np.arange(n) * h
    Y, Z = np.meshgrid(y, z, indexing="xy")            # (s, r): r fastest when raveled
    X0, Z0 = np.meshgrid(-2.0 + np.arange(n) * h, z, indexing="xy")  # (s, q)
    X1, Z1 = np.meshgrid(np.arange(n) * h, z, indexing="xy")
    media = {"fault_offset": fault(Y, Z).ravel(),
             "topo_offset": (topo(X0, Z0).ravel(), topo(X1, Z1).ravel())}
    return text, media


def mms_relative_error(sim):
    """sqrt(sum (F - u_exact)^2 / sum u_exact^2) over both blocks and all
    nine components, from a scenario's or the oracle's mms_norms."""
    e2 = r2 = 0.0
    for b in range(2):
        e, r = sim.mms_norms(b)
        e2 += e.sum()
        r2 += r.sum()
    return (e2 / r2) ** 0.5


def topography_case(dirpath, n=21, amp=0.12, fault_amp=0.08, fault_file=True, seed=5):
    """truth/1's geometry (2 x n^3, x in [-3, 3], y in [6, 9], z in [-1.5, 1.5])
    with use_topography = T: a seeded smooth free surface read from
    topo_<b>.dat ('read_topo_from_memory', src/grid.f90:1394-1425: nq*ns rows
    of x y z, s fastest, y offset from ay) and, with fault_file, the fault
    surface from fault.dat ('read_from_memomry_fractal' under topography,
    src/grid.f90:1538-1676: nr*ns rows of x offset, y, z, r fastest), whose
    y runs from the topography's fault edge down to by.  Writes the files
    into dirpath and returns the .in text."""
    import numpy as np
    surf = _smooth_surface(seed, amp)
    bump = _smooth_surface(seed + 1, fault_amp)
    ay, by, az, bz = 6.0, 9.0, -1.5, 1.5
    z = az + (bz - az) * np.arange(n) / (n - 1)
    for b, (ax, bx) in enumerate(((-3.0, 0.0), (0.0, 3.0))):
        x = ax + (bx - ax) * np.arange(n) / (n - 1)
        with open(os.path.join(str(dirpath), f"topo_{b + 1}.dat"), "w") as f:
            for i in range(n):
                for k in range(n):
                    f.write(f"{float(x[i])!r} {float(surf(x[i], z[k]))!r} {float(z[k])!r}\n")
    if fault_file:
        with open(os.path.join(str(dirpath), "fault.dat"), "w") as f:
            for k in range(n):
                ytop = ay + surf(0.0, z[k])
                for j in range(n):
                    r = j / (n - 1)
                    y = ytop + (by - ytop) * r
                    f.write(f"{float(bump(y, z[k]) * r * (1 - r) * 4.0)!r} {float(y)!r} {float(z[k])!r}\n")
    prof = ("'read_from_memomry_fractal'", "'fault.dat'") if fault_file else ("'no_path'", "'none'")
    extra = {b: (f"btp({b})%lc = {1 if b == 1 else 0}d0,\nbtp({b})%rc = {0 if b == 1 else 1}d0,\n"
                 f"btp({b})%profile_type = {prof[0]},\nbtp({b})%profile_path = {prof[1]},\n"
                 f"btp({b})%topography_type = 'read_topo_from_memory',\n"
                 f"btp({b})%topography_path = 'topo_{b}.dat',") for b in (1, 2)}
    return (problem(mesh="curvilinear", extra=",\n use_topography = T") +
            block_list(n, extra1=extra[1], extra2=extra[2]))
