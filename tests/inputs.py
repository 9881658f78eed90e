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
    raise KeyError(name)
