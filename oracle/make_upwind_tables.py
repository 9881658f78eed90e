"""Generate the upwind SBP operator tables from the reference's source.

The reference defines its upwind operators (fd_type 'upwind', orders 2..9,
and 'upwind_drp', orders 3..7, 66, 679) as unrolled Fortran routines in
src/JU_xJU_yJU_z6.f90: JJU_x<order>_upwind(_drp) computes, at one point and
along each axis, the forward difference D+ of the velocities (the terms
`w*F%F(i, ..., 1:3)`) and the backward difference D- of the stress fluxes
(`w*X_x(i, ...)*G%J(i, ...)*F%F(i, ..., 4:n)`), with a case per closure row
(`if (x .eq. K)`, `if (x .eq. nx-K)`) and one interior case
(`if ((x .ge. A) .and. (x .le. nx-B))`); JJU_x<order>_interior_upwind(_drp)
differences the interior of the block with its cf/cb arrays.  The penalty
weights tau0 are set in src/block.f90:195-252.  This script reads those
routines and writes the operators as dense tables:

  oracle/upwind_tables.inc                     (the oracle's copy)
  waveqlab3d-gh_gb300/csrc/wql_upwind_tables.h (the library's copy)

Per operator: R closure rows per end; two sets of interior weights, D+ on
its offsets and D- on its offsets -- ip/im from the interior routine (the
block's interior) and bp/bm from the near-boundary routine's interior case
(the interior rows of points in the boundary shell); they agree except for
rounding of written-out decimals, but for upwind_drp 66 and 679 they are
different stencils.  For each axis the left rows (row r, point t) and the
right rows (row k at point n-1-k, point n-1-t) of both operators are stored
separately: the reference's order-8 and order-9 rows are not mirror images
of one another on every axis.  Every literal is read as double precision:
the reference compiles with -fdefault-real-8 / -r8 (src/CMakeLists.txt:24,
28), which promote unsuffixed real constants.

Usage:  python oracle/make_upwind_tables.py <reference checkout>
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OPS = [("upwind", o) for o in (2, 3, 4, 5, 6, 7, 8, 9)] + [("upwind_drp", o) for o in (3, 4, 5, 6, 7, 66, 679)]
RMAX, NCOL = 8, 13
NUM = r"\d+\.?\d*(?:[eEdD][+-]?\d+)?"


def fnum(s):
    return float(s.replace("d", "e").replace("D", "e"))


def rational(a, b):
    return fnum(a) / (fnum(b) if b else 1.0)


def routine(lines, name):
    start = None
    for i, l in enumerate(lines):
        if start is None and re.match(r"\s*subroutine\s+%s\s*\(" % name, l, re.I):
            start = i
        elif start is not None and re.match(r"\s*end\s+subroutine", l, re.I):
            return lines[start:i + 1]
    raise KeyError(name)


def cases(body):
    """(axis 0..2, 'v' or 's', condition, [(weight, index expression)]) for
    every statement J{q,r,s}_xU(1:3 | 4:9) = ... of a near-boundary routine."""
    out, cond, i = [], None, 0
    while i < len(body):
        l = body[i].split("!")[0]
        m = re.match(r"\s*if\s*\(\s*\(\s*\w\s*\.ge\.\s*(\d+)\s*\)\s*\.and\.\s*\(\s*\w\s*\.le\.\s*n\w\s*-\s*(\d+)\s*\)"
                     r"\s*\)\s*then", l)
        if m:
            cond = ("int", int(m.group(1)), int(m.group(2)))
        m = re.match(r"\s*if\s*\(\s*\w\s*\.eq\.\s*(\d+)\s*\)\s*then", l)
        if m:
            cond = ("left", int(m.group(1)))
        m = re.match(r"\s*if\s*\(\s*\w\s*\.eq\.\s*n\w\s*(?:-\s*(\d+))?\s*\)\s*then", l)
        if m:
            cond = ("right", int(m.group(1) or 0))
        m = re.match(r"\s*J([qrs])_xU\((1:3|4:9)\)\s*=", l)
        if m:
            axis = "qrs".index(m.group(1))
            txt = l.split("=", 1)[1]
            depth = txt.count("(") - txt.count(")")
            while depth > 0 or txt.rstrip().endswith("&"):
                i += 1
                seg = body[i].split("!")[0]
                txt += "\n" + seg
                depth += seg.count("(") - seg.count(")")
            pat = (r"(?:^|[\s(&])([+-]?)\s*(" + NUM + r")(?:_wp)?\s*(?:/\s*(" + NUM + r")(?:_wp)?)?\s*\*\s*"
                   r"(?:X_x\([^)]*\)\s*\*\s*G%J\([^)]*\)\s*\*\s*)?F%F\(([^)]*)\)")
            terms = []
            for t in re.finditer(pat, txt):
                sgn, a, b, ff = t.groups()
                w = rational(a, b)
                terms.append((-w if sgn == "-" else w, ff.split(",")[axis].strip()))
            out.append((axis, "v" if m.group(2) == "1:3" else "s", cond, terms))
        i += 1
    return out


def interior_operator(lines, name):
    """The interior routine's operator: its loop `do s = lo, hi` applies
    cf(s+k) to the velocities at x+s and cb(s+k) to the stresses at x+s-K.
    Returns ({offset: D+ weight}, {offset: D- weight})."""
    body = "\n".join(l.split("!")[0] for l in routine(lines, name))
    loop = re.search(r"do\s+s\s*=\s*(-?\d+)\s*,\s*(-?\d+)", body)
    slo, shi = int(loop.group(1)), int(loop.group(2))
    k0 = int(re.search(r"cfx\(s\s*\+\s*(\d+)\)", body).group(1))
    kb = int(re.search(r"cbx\(s\s*\+\s*(\d+)\)", body).group(1))
    sh = re.search(r"cbx\(s\s*\+\s*\d+\)\s*\*\s*\(?\s*F%F%F\(\s*x\s*\+\s*s\s*(?:-\s*(\d+))?\s*,", body)
    K = int(sh.group(1) or 0)
    arrays = {}
    for key in ("cf", "cb"):
        m = re.search(r"parameter\s*::\s*%s\s*\(1:(\d+)\)\s*=\s*\(/(.*?)/\)" % key, body, re.S)
        vals = []
        for t in re.finditer(r"([+-]?)\s*(" + NUM + r")(?:_wp)?\s*(?:/\s*(" + NUM + r")(?:_wp)?)?",
                             m.group(2).replace("&", " ")):
            sgn, a, b = t.groups()
            w = rational(a, b)
            vals.append(-w if sgn == "-" else w)
        assert len(vals) == int(m.group(1)), (name, key, vals)
        arrays[key] = vals
    assert len(arrays["cf"]) == shi - slo + 1 and k0 == 1 - slo and kb == k0, (name, slo, shi, k0, kb)
    return ({s: arrays["cf"][s - slo] for s in range(slo, shi + 1)},
            {s - K: arrays["cb"][s - slo] for s in range(slo, shi + 1)})


def tau0s(ref):
    text = open(os.path.join(ref, "src", "block.f90")).read()
    out = {}
    for m in re.finditer(r"B%fd_type\s*\.eq\.\s*'(\w+)'\s*\.and\.\s*B%order\s*\.eq\.\s*(\d+)\s*\)\s*then\s*"
                         r"B%tau0\s*=\s*(" + NUM + r")(?:_wp)?\s*(?:/\s*(" + NUM + r")(?:_wp)?)?", text):
        fd, o, a, b = m.groups()
        out[(fd, int(o))] = rational(a, b)
    return out


def operator(lines, fd, order):
    suffix = "upwind" if fd == "upwind" else "upwind_drp"
    name = "JJU_x%d_%s" % (order, suffix)
    cs = cases(routine(lines, name))
    ints = [c for c in cs if c[2][0] == "int"]
    lo, hi = ints[0][2][1], ints[0][2][2]
    R = lo - 1
    assert hi == R and R <= RMAX, (name, lo, hi)
    op = {"R": R, "lp": [], "lm": [], "rp": [], "rm": []}
    for axis in range(3):
        v, nv = "xyz"[axis], "n" + "xyz"[axis]
        rows = {k: [[0.0] * NCOL for _ in range(R)] for k in ("lp", "lm", "rp", "rm")}
        interior, seen = {}, set()
        for ax, kind, cond, terms in cs:
            if ax != axis or (kind, cond) in seen:
                continue
            seen.add((kind, cond))
            if cond[0] == "int":
                w = {}
                for wt, e in terms:
                    off = eval(e.replace(v, "0"))
                    w[off] = w.get(off, 0.0) + wt
                interior[kind] = w
            elif cond[0] == "left":
                tab = rows["lp" if kind == "v" else "lm"][cond[1] - 1]
                for wt, e in terms:
                    tab[int(e) - 1] += wt
            else:
                tab = rows["rp" if kind == "v" else "rm"][cond[1]]
                for wt, e in terms:
                    tab[-eval(e.replace(nv, "0"))] += wt
        for k in rows:
            op[k].append(rows[k])
        if axis == 0:
            op["bp"], op["bm"] = interior["v"], interior["s"]
        else:
            assert interior["v"] == op["bp"] and interior["s"] == op["bm"], (name, axis)
    op["ip"], op["im"] = interior_operator(lines, "JJU_x%d_interior_%s" % (order, suffix))
    return op


def emit(ops, taus, struct):
    def arr(v):
        return "{" + ", ".join(repr(float(x)) for x in v) + "}"

    def dense(d, lo, hi):
        return [d.get(o, 0.0) for o in range(lo, hi + 1)] + [0.0] * (NCOL - (hi - lo + 1))

    out = ["struct %s {" % struct,
           "  const char* fd_type;",
           "  int order;",
           "  double tau0;  // src/block.f90:195-252",
           "  int R;        // closure rows per end",
           "  // interior rows: D+ (velocities) on offsets plo .. plo+pn-1, D- (stress",
           "  // fluxes) on mlo .. mlo+mn-1; ip/im inside the block (the interior",
           "  // routine), bp/bm on the interior rows of points of the boundary shell",
           "  // (the near-boundary routine's interior case)",
           "  int plo, pn, mlo, mn;",
           "  double ip[%d], im[%d], bp[%d], bm[%d];" % (NCOL, NCOL, NCOL, NCOL),
           "  // closure rows per axis (q, r, s): left row r at point t; right row k",
           "  // (the point n-1-k) at point n-1-t",
           "  double lp[3][%d][%d], lm[3][%d][%d];" % (RMAX, NCOL, RMAX, NCOL),
           "  double rp[3][%d][%d], rm[3][%d][%d];" % (RMAX, NCOL, RMAX, NCOL),
           "};",
           "",
           "constexpr int k%sCount = %d;" % (struct, len(ops)),
           "inline const %s k%s[k%sCount] = {" % (struct, struct, struct)]
    for (fd, order), op in ops:
        plo = min(min(op["ip"]), min(op["bp"]))
        phi = max(max(op["ip"]), max(op["bp"]))
        mlo = min(min(op["im"]), min(op["bm"]))
        mhi = max(max(op["im"]), max(op["bm"]))

        def rows3(key):
            pad = [[0.0] * NCOL] * (RMAX - op["R"])
            return "{" + ", ".join("{" + ", ".join(arr(r) for r in op[key][a] + pad) + "}" for a in range(3)) + "}"
        out.append("    {\"%s\", %d, %r, %d, %d, %d, %d, %d,\n     %s,\n     %s,\n     %s,\n     %s,\n"
                   "     %s,\n     %s,\n     %s,\n     %s},"
                   % (fd, order, taus[(fd, order)], op["R"], plo, phi - plo + 1, mlo, mhi - mlo + 1,
                      arr(dense(op["ip"], plo, phi)), arr(dense(op["im"], mlo, mhi)),
                      arr(dense(op["bp"], plo, phi)), arr(dense(op["bm"], mlo, mhi)),
                      rows3("lp"), rows3("lm"), rows3("rp"), rows3("rm")))
    out.append("};")
    return "\n".join(out) + "\n"


def main(ref):
    lines = open(os.path.join(ref, "src", "JU_xJU_yJU_z6.f90")).read().split("\n")
    taus = tau0s(ref)
    ops = [((fd, o), operator(lines, fd, o)) for fd, o in OPS]
    head = ("// Upwind SBP operators of the reference (src/JU_xJU_yJU_z6.f90:815-16122 near the\n"
            "// boundaries, :16451-20922 inside; tau0 from src/block.f90:195-252), written by\n"
            "// oracle/make_upwind_tables.py from those routines.  Regenerate; do not edit.\n")
    with open(os.path.join(ROOT, "waveqlab3d-gh_gb300", "csrc", "wql_upwind_tables.h"), "w") as f:
        f.write("#pragma once\n" + head + "\nnamespace wql {\n\n" + emit(ops, taus, "UpwindTable") +
                "\n}  // namespace wql\n")
    with open(os.path.join(HERE, "upwind_tables.inc"), "w") as f:
        f.write(head + "// Included by oracle/wql_ref.cpp inside its anonymous namespace.\n\n" +
                emit(ops, taus, "UpTable"))
    for (fd, o), op in ops:
        print(fd, o, "R", op["R"], "tau0", taus[(fd, o)])


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/make_upwind_tables.py <reference checkout>")
    main(sys.argv[1])
