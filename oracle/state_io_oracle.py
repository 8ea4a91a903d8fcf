"""Pure-Python restatement of PIMD-F90's configuration and checkpoint file formats.

TEST INFRASTRUCTURE ONLY: the checker for the engine library's file entry points
(pimd_read_config_header, pimd_read_xyz, pimd_write_xyz, pimd_save_image, pimd_load_image);
imported by tests/ and tests/golden/make_frames.py, never by the engine.

Each function follows the reference routine it names:
  read_header   read_and_initialize_all_nodes, InputOutput.f90:86-116
  read_xyz      read_coords_and_init, InputOutput.f90:422-446 (read_method 0 / 1)
  format_xyz    save_XYZ, InputOutput.f90:948-981
  format_image  save_checkpoint, InputOutput.f90:987-1024
  parse_image   load_checkpoint, InputOutput.f90:1030-1074, with PBCs, main_stuff.f90:107-125
Fortran edit descriptors are applied as fixed columns: '(a2,6(1x,f12.6))' puts the symbol in
columns 1-2 and field c in columns 4+13c .. 15+13c (1-based).
Parity status: these are format restatements (no arithmetic beyond the centring mean and the
PBC shift); they are pinned by the reference's own fixture files, which both readers must read
to the same numbers (tests/test_state_io.py).
"""
import math

import numpy as np


def _items(line):
    return line.replace(",", " ").replace("\t", " ").split()


def _real(s):
    return float(s.replace("d", "e").replace("D", "E"))


def _records_with_items(lines):
    for ln in lines:
        it = _items(ln)
        if it:
            yield it


def read_header(path):
    """(natoms, nbeads, time, box, records consumed before the atoms)."""
    with open(path) as f:
        lines = f.read().split("\n")
    if path.endswith(".img"):
        a = lines[0][:20].split()
        natoms, nbeads = int(a[0]), int(a[1])
        h = lines[1]
        time = _f_field(h, 0, 12, 6)
        box = np.array([_f_field(h, 14 + 13 * c, 12, 6) for c in range(3)])
        return natoms, nbeads, time, box, 2
    recs = [(i, _items(ln)) for i, ln in enumerate(lines) if _items(ln)]
    first = recs[0][1]
    if len(first) >= 4:
        return int(first[0]), 0, 0.0, np.array([_real(x) for x in first[1:4]]), recs[0][0] + 1
    if len(first) == 3:
        return int(recs[1][1][0]), 0, 0.0, np.array([_real(x) for x in first]), recs[1][0] + 1
    box = np.array([_real(x) for x in recs[1][1][:3]])
    return int(first[0]), 0, 0.0, box, recs[1][0] + 1


def read_xyz(path, read_method=1):
    """(box, RRc (Natoms, 3)); read_method 1 subtracts the mean accumulated in file order."""
    natoms, _, _, box, skip = read_header(path)
    with open(path) as f:
        lines = f.read().split("\n")[skip:]
    recs = _records_with_items(lines)
    N = natoms // 3
    RRc = np.zeros((natoms, 3))
    avg = [0.0, 0.0, 0.0]
    if read_method == 0:
        order = [3 * i for i in range(N)] + [3 * i + k for i in range(N) for k in (1, 2)]
    else:
        order = list(range(natoms))
    for i in order:
        it = next(recs)
        RRc[i] = [_real(x) for x in it[1:4]]
        if read_method == 1:
            for c in range(3):
                avg[c] = avg[c] + RRc[i, c]
    for c in range(3):
        avg[c] = avg[c] / natoms
        for i in range(natoms):
            RRc[i, c] = RRc[i, c] - avg[c]
    return box, RRc


def _fw(v, w=12, d=6):
    s = "%*.*f" % (w, d, v)
    return "*" * w if len(s) > w else s


def _f_field(rec, pos, w, d):
    s = rec[pos:pos + w].replace(" ", "")
    if not s:
        return 0.0
    if "." in s:
        return _real(s)
    m, _, e = s.upper().replace("D", "E").partition("E")
    return float(m) * 10.0 ** ((int(e) if e else 0) - d)


def format_xyz(RR):
    natoms = len(RR)
    out = ["%10d" % natoms, " "]
    for i in range(natoms):
        out.append(("O " if i % 3 == 0 else "H ") + "".join(" " + _fw(RR[i, c]) for c in range(3)))
    return "\n".join(out) + "\n"


def _ld(v):
    """gfortran list-directed REAL(8): one blank, then G25.17E3."""
    w, d, e = 25, 17, 3
    a = abs(v)
    if a == 0.0:
        k = 1
        fform = True
    else:
        ex = int(("%.*e" % (d - 1, a)).split("e")[1])
        fform = -1 <= ex < d
        k = ex + 1
    if fform:
        return " " + "%*.*f" % (w - e - 2, d - k, v) + " " * (e + 2)
    m, ex = ("%.*E" % (d - 1, v)).split("E")
    ex = int(ex)
    return " " + ("%s%s" % (m, "E%s%0*d" % ("-" if ex < 0 else "+", e, abs(ex)))).rjust(w)


def format_image(time, box, RRt, PPt, massO, massH, vxi_beads=None, vxi_global=None):
    P, natoms = RRt.shape[0], RRt.shape[1]
    out = ["%10d%10d" % (natoms, P), _fw(time) + "  " + _fw(box[0]) + " " + _fw(box[1]) + " " + _fw(box[2])]
    imass = (1.0 / massO, 1.0 / massH)
    for w in range(natoms // 3):
        for a in range(3):
            i = 3 * w + a
            for j in range(P):
                im = imass[0 if a == 0 else 1]
                out.append(("O " if a == 0 else "H ") + "".join(" " + _fw(RRt[j, i, c]) for c in range(3))
                           + "".join(" " + _fw(PPt[j, i, c] * im) for c in range(3)))
    if vxi_beads is not None:  # (3, P, natoms, 2) = vxi_beads(2, natoms, P, 3)
        for i in range(natoms):
            for j in range(P):
                for k in range(3):
                    out.append(_ld(vxi_beads[k, j, i, 0]) + _ld(vxi_beads[k, j, i, 1]))
    if vxi_global is not None:
        out.append("".join(_ld(v) for v in vxi_global))
    return "\n".join(out) + "\n"


def _anint(x):
    """Fortran ANINT: round half away from zero (a - floor(a) is exact for doubles)."""
    a = abs(x)
    f = math.floor(a)
    r = f + 1.0 if a - f >= 0.5 else float(f)
    return math.copysign(r, x)


def parse_image(path, massO, massH, vxi_beads=False, n_vxi_global=0):
    natoms, P, time, box, _ = read_header(path)
    with open(path) as f:
        lines = f.read().split("\n")
    RRt, PPt = np.zeros((P, natoms, 3)), np.zeros((P, natoms, 3))
    mass = (massO, massH)
    row = 2
    for w in range(natoms // 3):
        for a in range(3):
            i = 3 * w + a
            for j in range(P):
                rec = lines[row]
                row += 1
                vals = [_f_field(rec, 3 + 13 * c, 12, 6) for c in range(6)]
                RRt[j, i] = vals[:3]
                PPt[j, i] = [v * mass[0 if a == 0 else 1] for v in vals[3:]]
    recs = _records_with_items(lines[row:])
    out = {}
    if vxi_beads:
        vb = np.zeros((3, P, natoms, 2))
        for i in range(natoms):
            for j in range(P):
                for k in range(3):
                    it = next(recs)
                    vb[k, j, i] = [_real(it[0]), _real(it[1])]
        out["vxi_beads"] = vb
    if n_vxi_global:
        vals = []
        while len(vals) < n_vxi_global:
            vals += [_real(x) for x in next(recs)]
        out["vxi_global"] = np.array(vals[:n_vxi_global])
    cen = np.zeros((natoms, 3))
    for j in range(P):
        cen = cen + RRt[j]
    cen = cen / P
    boxi0 = 1.0 / box[0]
    for i in range(natoms):
        for c in range(3):
            x = cen[i, c] * boxi0
            shift = box[0] * _anint(x)
            cen[i, c] = cen[i, c] - shift
            for j in range(P):
                RRt[j, i, c] = RRt[j, i, c] - shift
    out.update(time=time, box=box, RRt=RRt, PPt=PPt, RRc=cen)
    return out
