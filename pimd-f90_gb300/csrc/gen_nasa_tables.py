#!/usr/bin/env python3
"""Generate nasa_tables.h from the reference's nasa_mod.f90 data statements.

The Partridge-Schwenke monomer PES (245 terms) and dipole-moment surface (84 terms)
coefficient tables are published data; the force engine must use exactly the same
numbers as the reference, so they are extracted mechanically rather than retyped.

Source: pot_ttm/nasa_mod.f90:16-472 (data statements for idx, c5zA, cbasis, ccore,
crest, idxD, coefD and the scalar parameters).

Usage:  python gen_nasa_tables.py <path-to>/pot_ttm/nasa_mod.f90 > nasa_tables.h
Every literal is checked to carry a d/D exponent (double precision); a literal without
one would be a single-precision constant in Fortran and is rejected.
"""
import re
import sys


def _numbers(body):
    toks = [t.strip() for t in body.replace("&", " ").replace("\n", " ").split(",")]
    return [t for t in toks if t]


def _to_c_double(tok):
    t = tok.strip()
    if re.fullmatch(r"[+-]?\d+", t):
        return t + ".0"
    if not re.search(r"[dD]", t):
        raise ValueError("single-precision literal in a double table: %r" % tok)
    return t.replace("D", "e").replace("d", "e")


def parse(text):
    # drop comments
    lines = []
    for ln in text.splitlines():
        i = ln.find("!")
        lines.append(ln if i < 0 else ln[:i])
    src = "\n".join(lines)
    out = {}
    for m in re.finditer(r"data\s+([A-Za-z0-9_,():\s]+?)\s*/(.*?)/", src, re.S | re.I):
        names = m.group(1).strip()
        vals = _numbers(m.group(2))
        out[names.replace(" ", "")] = vals
    return out


def main():
    path = sys.argv[1]
    with open(path) as f:
        d = parse(f.read())
    idx = [d["idx(:,%d)" % c] for c in (1, 2, 3)]
    idxD = [d["idxD(1:84,%d)" % c] for c in (1, 2, 3)]
    for arr, n in ((idx, 245), (idxD, 84)):
        for col in arr:
            assert len(col) == n, (len(col), n)
    tables = {k: d["%s(1:245)" % k] for k in ("c5zA", "cbasis", "ccore", "crest")}
    for k, v in tables.items():
        assert len(v) == 245, (k, len(v))
    coefD = d["coefD(1:84)"]
    assert len(coefD) == 84
    scal_names = "reoh,thetae,b1,roh,alphaoh,deohA,phh1A,phh2".split(",")
    scal = dict(zip(scal_names, d["reoh,thetae,b1,roh,alphaoh,deohA,phh1A,phh2"]))
    scal.update(zip("f5z,fbasis,fcore,frest".split(","), d["f5z,fbasis,fcore,frest"]))
    scal["b1D"] = d["b1D"][0]
    scal.update(zip("a,b,c0,c1,c2".split(","), d["a,b,c0,c1,c2"]))

    w = sys.stdout.write
    w("// Generated by gen_nasa_tables.py from pot_ttm/nasa_mod.f90 (data statements).\n")
    w("// Partridge-Schwenke water monomer PES and dipole-moment surface coefficients.\n")
    w("// Do not edit by hand.\n#pragma once\n\n")
    for c in range(3):
        w("static const int PIMD_NASA_IDX%d[245] = {%s};\n" % (c + 1, ",".join(idx[c])))
    for c in range(3):
        w("static const int PIMD_NASA_IDXD%d[84] = {%s};\n" % (c + 1, ",".join(idxD[c])))
    for k in ("c5zA", "cbasis", "ccore", "crest"):
        w("static const double PIMD_NASA_%s[245] = {\n%s};\n" % (
            k.upper(), ",\n".join(_to_c_double(x) for x in tables[k])))
    w("static const double PIMD_NASA_COEFD[84] = {\n%s};\n" % ",\n".join(_to_c_double(x) for x in coefD))
    for k, v in scal.items():
        w("static const double PIMD_NASA_%s = %s;\n" % (k.upper(), _to_c_double(v)))


if __name__ == "__main__":
    main()
