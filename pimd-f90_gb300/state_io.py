"""Configuration and checkpoint files of PIMD-F90 (InputOutput.f90) through the C ABI.

  read_config_header(path)            read_and_initialize_all_nodes, InputOutput.f90:67-116
  read_xyz(path, read_method=1)       read_coords_and_init, InputOutput.f90:422-446
  write_xyz(path, RR, append=False)   save_XYZ, InputOutput.f90:948-981
  save_image(path, ...)               save_checkpoint, InputOutput.f90:987-1024
  load_image(path, ...)               load_checkpoint, InputOutput.f90:1030-1074

Arrays in the reference's layouts stored C-order: RR (Natoms, 3) is RR(3, Natoms), RRt
(P, Natoms, 3) is RRt(3, Natoms, P), vxi_beads (3, P, Natoms, 2) is vxi_beads(2, Natoms, P, 3).
Host-only calls: they need the built library but no GPU.
"""
import ctypes

import numpy as np

from .engine import PimdError, _f64, _p, load


def _b(path):
    return str(path).encode()


def read_config_header(path):
    """(natoms, nbeads, time, box) of an .xyz or .img file (nbeads = 0, time = 0 for .xyz)."""
    n, nb, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    box = np.zeros(3)
    rc = load().pimd_read_config_header(_b(path), ctypes.byref(n), ctypes.byref(nb), ctypes.byref(t), _p(box))
    if rc:
        raise PimdError("pimd_read_config_header(%s) failed (%d)" % (path, rc))
    return n.value, nb.value, t.value, box


def read_xyz(path, read_method=1):
    """(box, RRc) of an .xyz configuration; RRc (Natoms, 3), centred as the reference does."""
    natoms, _, _, box = read_config_header(path)
    RRc = np.zeros((natoms, 3))
    rc = load().pimd_read_xyz(_b(path), int(read_method), natoms, _p(RRc))
    if rc:
        raise PimdError("pimd_read_xyz(%s) failed (%d)" % (path, rc))
    return box, RRc


def write_xyz(path, RR, append=False):
    RR = _f64(RR)
    rc = load().pimd_write_xyz(_b(path), int(bool(append)), RR.shape[0], _p(RR))
    if rc:
        raise PimdError("pimd_write_xyz(%s) failed (%d)" % (path, rc))


def save_image(path, time, box, RRt, PPt, massO, massH, vxi_beads=None, vxi_global=None):
    RRt, PPt = _f64(RRt), _f64(PPt)
    P, natoms = RRt.shape[0], RRt.shape[1]
    vb = None if vxi_beads is None else _f64(vxi_beads)
    vg = None if vxi_global is None else _f64(vxi_global)
    rc = load().pimd_save_image(_b(path), natoms, P, float(time), _p(_f64(box)), _p(RRt), _p(PPt), float(massO),
                                float(massH), _p(vb), 0 if vb is None else vb.size, _p(vg),
                                0 if vg is None else vg.size)
    if rc:
        raise PimdError("pimd_save_image(%s) failed (%d)" % (path, rc))


def load_image(path, massO, massH, n_vxi_beads=False, n_vxi_global=0):
    """dict(time, box, RRt, PPt, RRc[, vxi_beads][, vxi_global]) of an .img image."""
    natoms, P, _, _ = read_config_header(path)
    t = ctypes.c_double()
    box = np.zeros(3)
    RRt, PPt, RRc = np.zeros((P, natoms, 3)), np.zeros((P, natoms, 3)), np.zeros((natoms, 3))
    vb = np.zeros((3, P, natoms, 2)) if n_vxi_beads else None
    vg = np.zeros(int(n_vxi_global)) if n_vxi_global else None
    rc = load().pimd_load_image(_b(path), natoms, P, float(massO), float(massH), ctypes.byref(t), _p(box), _p(RRt),
                                _p(PPt), _p(RRc), _p(vb), 0 if vb is None else vb.size, _p(vg),
                                0 if vg is None else vg.size)
    if rc:
        raise PimdError("pimd_load_image(%s) failed (%d)" % (path, rc))
    out = dict(time=t.value, box=box, RRt=RRt, PPt=PPt, RRc=RRc)
    if vb is not None:
        out["vxi_beads"] = vb
    if vg is not None:
        out["vxi_global"] = vg
    return out
