"""Python host mirror of PIMD-F90's hot-path interfaces over the C ABI (libpimd_gb300.so).

Names, argument order and meaning follow the reference:
  ForceEngine.pot_ttm(RR, RRc, t)            pot_ttm/pot_ttm.f90:3
  ForceEngine.full_bead_forces(RRt, RRc, t)  force_calc.f90:26-106 (all beads in one call)
  ForceEngine.nm_init / evolve_ring          NormalModes.f90:68, :34
Arrays are numpy float64 in the reference's layouts stored C-order: RR (Natoms, 3) is the
Fortran RR(3, Natoms); RRt (P, Natoms, 3) is RRt(3, Natoms, P).

The engine runs only on the GPU: if the shared library or a CUDA device is missing every
call raises; there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libpimd_gb300.so")

PIMD_FP64, PIMD_MIXED = 0, 1
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "neighbour list overflow", 4: "gammq did not converge",
          5: "out of device memory", 6: "call-order violation"}


# parameter vector of the differentiation form (include/pimd_gb300.h PIMD_TH_*)
THETA_NAMES = ["polar_M", "a_dd", "a_cc", "vdw_C", "vdw_D", "vdw_E", "dms1", "dms2", "dms3", "gamma_M", "nasa_f5z",
               "nasa_fbasis", "nasa_fcore", "nasa_frest"]


class PimdError(RuntimeError):
    pass


class Params(ctypes.Structure):
    _fields_ = [("pot_model", ctypes.c_int), ("natoms", ctypes.c_int), ("nbeads", ctypes.c_int),
                ("box", ctypes.c_double * 3), ("rc", ctypes.c_double), ("rc1", ctypes.c_double),
                ("eps_ewald", ctypes.c_double), ("alpha", ctypes.c_double), ("nmax", ctypes.c_int),
                ("polar_maxiter", ctypes.c_int), ("polar_sor", ctypes.c_double), ("polar_eps", ctypes.c_double),
                ("guess_initdip", ctypes.c_int), ("contraction", ctypes.c_int), ("precision", ctypes.c_int),
                ("device", ctypes.c_int)]


class MDParams(ctypes.Structure):
    _fields_ = [("delt", ctypes.c_double), ("massO", ctypes.c_double), ("massH", ctypes.c_double),
                ("langevin", ctypes.c_int), ("seed", ctypes.c_ulonglong)]


# every entry point of include/pimd_gb300.h with its ctypes signature
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_V = ctypes.c_void_p
SIGNATURES = {
    "pimd_create": [ctypes.POINTER(_V), ctypes.POINTER(Params)],
    "pimd_destroy": [_V],
    "pimd_set_stream": [_V, _V],
    "pimd_last_error": [_V],
    "pimd_ewald_info": [_V, _D, _I, _I],
    "pimd_pot_ttm": [_V, _D, _D, _D, _D, _D, _D, _D, _D, _D, ctypes.c_int],
    "pimd_pot_spc": [_V, _D, _D, _D, _D, _D, _D],
    "pimd_full_bead_forces": [_V, _D, _D, _D, _D, _D, _D, _D, _D, _D, ctypes.c_int],
    "pimd_full_bead_forces_device": [_V, _V, _V, _V, _V, _V, _V, _V, _V, _V, ctypes.c_int],
    "pimd_get_energies": [_V, ctypes.c_int, _D],
    "pimd_get_virial": [_V, ctypes.c_int, _D],
    "pimd_get_dipole_info": [_V, ctypes.c_int, _I, _D],
    "pimd_set_dipole_check": [_V, ctypes.c_int],
    "pimd_get_neighbors": [_V, ctypes.c_int, _I, ctypes.c_int, _I],
    "pimd_nm_init": [_V, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, _D, _D, _D, _D, _D, _D,
                     _D],
    "pimd_evolve_ring": [_V, _D, _D, ctypes.c_int, ctypes.c_double],
    "pimd_real2nm": [_V, _D, _D, ctypes.c_int],
    "pimd_nm2real": [_V, _D, _D, ctypes.c_int],
    "pimd_gen_rand_ring": [_V, _D, ctypes.c_double, ctypes.c_double, ctypes.c_int, _D],
    "pimd_gen_rand_ring_momenta": [_V, _D, ctypes.c_double, ctypes.c_double, ctypes.c_int, _D],

    "pimd_evolve_all_device": [_V, _V, _V, ctypes.c_double, ctypes.c_double],
    "pimd_langevin_init": [_V, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double],
    "pimd_langevin_nm_device": [_V, _V, _V, ctypes.c_double, ctypes.c_double, ctypes.c_ulonglong,
                                ctypes.c_ulonglong],
    "pimd_md_step_device": [_V, ctypes.POINTER(MDParams), _V, _V, _V, _V, _V, _V, ctypes.c_int, _V],
    "pimd_md_step": [_V, ctypes.POINTER(MDParams), _D, _D, _D, _D, _D, _D, ctypes.c_int, _D],
    "pimd_read_config_header": [ctypes.c_char_p, _I, _I, _D, _D],
    "pimd_read_xyz": [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _D],
    "pimd_write_xyz": [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _D],
    "pimd_save_image": [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, _D, _D, _D, ctypes.c_double,
                        ctypes.c_double, _D, ctypes.c_int, _D, ctypes.c_int],
    "pimd_load_image": [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, _D, _D, _D,
                        _D, _D, _D, ctypes.c_int, _D, ctypes.c_int],
    "pimd_checkpoint_write": [_V, ctypes.c_char_p, _D, _D, _D, ctypes.c_int, ctypes.c_ulonglong],
    "pimd_checkpoint_read": [_V, ctypes.c_char_p, _D, _D, _D, _I, ctypes.POINTER(ctypes.c_ulonglong)],
    "pimd_contracted_init": [_V, ctypes.c_int, ctypes.c_int],
    "pimd_contracted_step_device": [_V, ctypes.POINTER(MDParams), _V, _V, _V, _V, _V, _V, _V, ctypes.c_int, _V, _V,
                                    _V],
    "pimd_contracted_step": [_V, ctypes.POINTER(MDParams), _D, _D, _D, _D, _D, _D, _D, ctypes.c_int, _D, _D, _D],
    "pimd_geometry_reset": [_V],
    "pimd_geometry_accumulate_device": [_V, _V, _V],
    "pimd_geometry_report": [_V, _D, _D, _D, _D],
    "pimd_msd_init": [_V, ctypes.c_int],
    "pimd_msd_accumulate_device": [_V, _V],
    "pimd_msd_report": [_V, ctypes.c_double, _D, _I, _D],
    "pimd_spectra_init": [_V, ctypes.c_int, ctypes.c_double],
    "pimd_spectra_record_device": [_V, _V, _V],
    "pimd_ir_spectrum": [_V, ctypes.c_double, ctypes.c_double, _I, _D, _D],
    "pimd_dos": [_V, ctypes.c_double, _I, _D, _D],
    "pimd_set_thermostat": [_V, _V],
    "pimd_get_thermostat_state": [_V, _D, _D, _D],
    "pimd_set_thermostat_state": [_V, _D, ctypes.c_double, _D],
    "pimd_md_step_ex_device": [_V, ctypes.POINTER(MDParams), _V, _V, _V, _V, _V, _V, ctypes.c_int, _V],
    "pimd_md_step_ex": [_V, ctypes.POINTER(MDParams), _D, _D, _D, _D, _D, _D, ctypes.c_int, _D],
    "pimd_peak_flops": [ctypes.c_int, ctypes.c_int, _D],
    "pimd_set_graph": [_V, ctypes.c_int],
    "pimd_autotune": [_V, _V, _V],
    "pimd_get_theta": [_V, _D],
    "pimd_set_theta": [_V, _D],
    "pimd_pot_forward": [_V, _D, _D, _D, ctypes.c_int],
    "pimd_pot_backward": [_V, _D, _D, _D],
    "pimd_get_tuning": [_V, _I, ctypes.c_int],
    "pimd_set_tuning": [_V, _I, ctypes.c_int],
    "pimd_batch_create": [ctypes.POINTER(_V), ctypes.POINTER(Params), _V, ctypes.c_int, ctypes.POINTER(MDParams)],
    "pimd_batch_destroy": [_V],
    "pimd_batch_last_error": [_V],
    "pimd_batch_info": [_V, _I, _I],
    "pimd_batch_set_state": [_V, ctypes.c_int, _D, _D],
    "pimd_batch_get_state": [_V, ctypes.c_int, _D, _D, _D, _D],
    "pimd_batch_forces": [_V],
    "pimd_batch_autotune": [_V],
    "pimd_batch_step": [_V, ctypes.c_int],
    "pimd_batch_sync": [_V],
    "pimd_graph_info": [_V, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
    "pimd_neighbors_noalloc": [_V, ctypes.c_int, _D, ctypes.c_double, _V, ctypes.c_int, _V, _V],
    "pimd_timers_reset": [_V, ctypes.c_int],
    "pimd_launch_count": [_V],
    "pimd_timers_get": [_V, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, _D, ctypes.POINTER(ctypes.c_longlong)],
}

_lib = None


def load(path=LIB):
    """Load the engine library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise PimdError("libpimd_gb300.so not built: run __graft_entry__.build()")
        L = ctypes.CDLL(path)
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = {"pimd_last_error": ctypes.c_char_p, "pimd_batch_last_error": ctypes.c_char_p,
                         "pimd_launch_count": ctypes.c_longlong}.get(name, ctypes.c_int)
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_D) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def make_params(d, precision=PIMD_FP64, device=0):
    p = Params()
    p.pot_model = int(d["pot_model"])
    p.natoms = int(d["natoms"])
    p.nbeads = int(d.get("nbeads", 1))
    for i in range(3):
        p.box[i] = float(d["box"][i])
    p.rc = float(d["rc"])
    p.rc1 = float(d.get("rc1", 0.8 * d["rc"]))
    p.eps_ewald = float(d.get("eps_ewald", 1e-6))
    a = d.get("alpha")
    p.alpha = float(a) if a else 0.0
    p.nmax = int(d.get("nmax", 0) or 0)
    p.polar_maxiter = int(d.get("polar_maxiter", 15))
    p.polar_sor = float(d.get("polar_sor", 0.7))
    p.polar_eps = float(d.get("polar_eps", 1e-5))
    p.guess_initdip = int(d.get("guess_initdip", 0))
    p.contraction = int(d.get("contraction", 0))
    p.precision = int(d.get("precision", precision))
    p.device = int(d.get("device", device))
    return p


class Thermostat(ctypes.Structure):
    _fields_ = [("bead_thermostat", ctypes.c_int), ("global_thermostat", ctypes.c_int), ("tau", ctypes.c_double),
                ("temp", ctypes.c_double), ("centroid_thermostat", ctypes.c_int), ("tau_centroid", ctypes.c_double)]


MD_NOUT = 12
MD_OUT_NAMES = ("Upot", "virial", "virialc", "uk", "uk_mid", "K0", "sys_temp", "E_virial", "P_virial", "E_simple",
                "P_simple", "s_global")


class Replica(ctypes.Structure):
    _fields_ = [("natoms", ctypes.c_int), ("nbeads", ctypes.c_int), ("box", ctypes.c_double * 3),
                ("temp", ctypes.c_double)]


class ForceEngine:
    """One engine context: the reference's init_pot module state for P beads."""

    def __init__(self, params, precision=PIMD_FP64, device=0):
        L = load()
        self.params = dict(params)
        self._p = make_params(params, precision, device)
        h = _V()
        rc = L.pimd_create(ctypes.byref(h), ctypes.byref(self._p))
        if rc:
            raise PimdError("pimd_create failed (%d: %s)" % (rc, ERRORS.get(rc, "?")))
        self.h = h
        self.natoms = self._p.natoms
        self.nw = self.natoms // 3
        self.P = self._p.nbeads

    def close(self):
        if getattr(self, "h", None):
            load().pimd_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, rc, what):
        if rc:
            msg = load().pimd_last_error(self.h)
            raise PimdError("%s failed (%d: %s): %s" % (what, rc, ERRORS.get(rc, "?"), msg.decode() if msg else ""))

    def ewald_info(self):
        a = ctypes.c_double()
        nk = ctypes.c_int()
        hkl = (ctypes.c_int * 3)()
        self._check(load().pimd_ewald_info(self.h, ctypes.byref(a), ctypes.byref(nk), hkl), "ewald_info")
        return a.value, nk.value, tuple(hkl)

    def set_dipole_check(self, every):
        self._check(load().pimd_set_dipole_check(self.h, int(every)), "set_dipole_check")

    def energies(self, bead=0):
        U = np.zeros(4)
        self._check(load().pimd_get_energies(self.h, bead, _p(U)), "get_energies")
        n = ctypes.c_int()
        dd = ctypes.c_double()
        self._check(load().pimd_get_dipole_info(self.h, bead, ctypes.byref(n), ctypes.byref(dd)), "dipole_info")
        return dict(Umon=U[0], Uvdw=U[1], Uelec=U[2], Uind=U[3], niter=n.value, deltadip=dd.value)

    def neighbors(self, bead=0):
        """The O-O half neighbour list (npairs, 2) of the last force call."""
        n = ctypes.c_int()
        self._check(load().pimd_get_neighbors(self.h, bead, None, 0, ctypes.byref(n)), "get_neighbors")
        ij = np.zeros((max(1, n.value), 2), np.int32)
        self._check(load().pimd_get_neighbors(self.h, bead, ij.ctypes.data_as(_I), n.value, ctypes.byref(n)),
                    "get_neighbors")
        return ij[:n.value].copy()

    def virial(self, bead=0):
        v = np.zeros(9)
        self._check(load().pimd_get_virial(self.h, bead, _p(v)), "get_virial")
        return v.reshape(3, 3, order="F")

    def pot_ttm(self, RR, RRc, t=1):
        """pot_ttm(RR, RRc, En, dRR, virt, virialc, dip_momI, Edip_mom, chg, t)"""
        RR, RRc = _f64(RR), _f64(RRc)
        En, vc = ctypes.c_double(), ctypes.c_double()
        dRR = np.zeros_like(RR)
        virt = np.zeros(9)
        dI = np.zeros((self.nw, 3))
        dE = np.zeros((self.nw, 3))
        chg = np.zeros(self.natoms)
        rc = load().pimd_pot_ttm(self.h, _p(RR), _p(RRc), ctypes.byref(En), _p(dRR), _p(virt), ctypes.byref(vc),
                                 _p(dI), _p(dE), _p(chg), int(t))
        self._check(rc, "pot_ttm")
        out = dict(En=En.value, dRR=dRR, virt=virt.reshape(3, 3, order="F"), virialc=vc.value, dip_momI=dI,
                   Edip_mom=dE, chg=chg)
        out.update(self.energies(0))
        return out

    def pot_spc(self, RR):
        """pot_spc(RR, En, dRR, virt, dip_momI, chg) (pot_ttm/pot_spc.f90:1)"""
        RR = _f64(RR)
        En = ctypes.c_double()
        dRR = np.zeros_like(RR)
        virt = np.zeros(9)
        dI = np.zeros((self.nw, 3))
        chg = np.zeros(self.natoms)
        rc = load().pimd_pot_spc(self.h, _p(RR), ctypes.byref(En), _p(dRR), _p(virt), _p(dI), _p(chg))
        self._check(rc, "pot_spc")
        out = dict(En=En.value, dRR=dRR, virt=virt.reshape(3, 3, order="F"), dip_momI=dI, chg=chg)
        out.update(self.energies(0))
        return out

    def potential(self, RR, RRc, t=1):
        """force_calc.f90:112-170 dispatch on pot_model (one bead)."""
        if self._p.pot_model in (2, 3):
            return self.pot_ttm(RR, RRc, t)
        return self.pot_spc(RR)

    def full_bead_forces(self, RRt, RRc, t=1):
        RRt, RRc = _f64(RRt), _f64(RRc)
        P = self.P
        Upott, virialt, virialct = np.zeros(P), np.zeros(P), np.zeros(P)
        dRRt = np.zeros_like(RRt)
        dI = np.zeros((P, self.nw, 3))
        dE = np.zeros((P, self.nw, 3))
        chg = np.zeros(self.natoms)
        rc = load().pimd_full_bead_forces(self.h, _p(RRt), _p(RRc), _p(Upott), _p(dRRt), _p(virialt), _p(virialct),
                                          _p(dI), _p(dE), _p(chg), int(t))
        self._check(rc, "full_bead_forces")
        return dict(Upott=Upott, dRRt=dRRt, virialt=virialt, virialct=virialct, dip_momIt=dI, dip_momEt=dE, chg=chg,
                    Upot=Upott.sum(), virial=virialt.sum(), virialc=virialct.sum() / P)

    # ---- NormalModes.f90 / Langevin.f90 ------------------------------------------------
    def nm_init(self, P, omegan, delta, setNMfreq=0.0):
        A = [np.zeros(P) for _ in range(6)]
        C = np.zeros(P * P)
        rc = load().pimd_nm_init(self.h, P, omegan, delta, setNMfreq, *[_p(a) for a in A], _p(C))
        self._check(rc, "nm_init")
        return dict(A11=A[0], A12=A[1], A21=A[2], A22=A[3], omegalist=A[4], msf=A[5], C=C.reshape(P, P, order="F"))

    def evolve_ring(self, RR, PP, mass):
        RR, PP = _f64(RR).copy(), _f64(PP).copy()
        self._check(load().pimd_evolve_ring(self.h, _p(RR), _p(PP), RR.shape[0], float(mass)), "evolve_ring")
        return RR, PP

    def real2nm(self, A):
        A = _f64(A)
        out = np.zeros_like(A)
        self._check(load().pimd_real2nm(self.h, _p(A), _p(out), A.shape[0]), "real2nm")
        return out

    def nm2real(self, A):
        A = _f64(A)
        out = np.zeros_like(A)
        self._check(load().pimd_nm2real(self.h, _p(A), _p(out), A.shape[0]), "nm2real")
        return out

    def gen_rand_ring(self, mass, temp, P, xi=None):
        RR = np.zeros((P, 3))
        x = None if xi is None else _f64(xi)
        self._check(load().pimd_gen_rand_ring(self.h, _p(RR), float(mass), float(temp), int(P), _p(x)), "gen_rand_ring")
        return RR

    def gen_rand_ring_momenta(self, mass, temp, P, xi=None):
        PP = np.zeros((P, 3))
        x = None if xi is None else _f64(xi)
        self._check(load().pimd_gen_rand_ring_momenta(self.h, _p(PP), float(mass), float(temp), int(P), _p(x)),
                    "gen_rand_ring_momenta")
        return PP

    def langevin_init(self, delt2, centroid_thermostat, tau, temp_P):
        rc = load().pimd_langevin_init(self.h, float(delt2), int(centroid_thermostat), float(tau), float(temp_P))
        self._check(rc, "langevin_init")

    # ---- MD.f90 PIMD_VV --------------------------------------------------------------
    @staticmethod
    def md_params(delt, massO, massH, langevin=1, seed=12345):
        mp = MDParams()
        mp.delt = float(delt)
        mp.massO = float(massO)
        mp.massH = float(massH)
        mp.langevin = int(langevin)
        mp.seed = int(seed)
        return mp

    def md_step(self, mp, RRt, PPt, dRRt, t, xi1=None, xi2=None):
        """One PIMD_VV step on host arrays (updated in place); returns (Upot, virial, virialc, uk), RRc."""
        for a in (RRt, PPt, dRRt):
            assert a.dtype == np.float64 and a.flags.c_contiguous
        RRc = np.empty((self.natoms, 3))  # both written by the call
        out = np.empty(4)
        x1 = _f64(xi1) if xi1 is not None else None
        x2 = _f64(xi2) if xi2 is not None else None
        rc = load().pimd_md_step(self.h, ctypes.byref(mp), _p(RRt), _p(PPt), _p(dRRt), _p(RRc), _p(x1), _p(x2),
                                 int(t), _p(out))
        self._check(rc, "md_step")
        return out, RRc

    def set_thermostat(self, bead_thermostat=0, global_thermostat=0, tau=0.1, temp=300.0, centroid_thermostat=0,
                       tau_centroid=0.1):
        """Nose-Hoover chains of the MD step (bead_thermostat 2: on the normal modes; global)."""
        th = Thermostat(int(bead_thermostat), int(global_thermostat), float(tau), float(temp),
                        int(centroid_thermostat), float(tau_centroid))
        self._check(load().pimd_set_thermostat(self.h, ctypes.byref(th)), "set_thermostat")

    def thermostat_state(self, beads=False):
        vg = np.zeros(2)
        uk = ctypes.c_double()
        vb = np.zeros((3, self.P, self.natoms, 2)) if beads else None
        self._check(load().pimd_get_thermostat_state(self.h, _p(vg), ctypes.byref(uk), _p(vb)), "thermostat_state")
        return dict(vxi_global=vg, uk=uk.value, vxi_beads=vb)

    def set_thermostat_state(self, vxi_global=None, uk=0.0, vxi_beads=None):
        vg = None if vxi_global is None else _f64(vxi_global)
        vb = None if vxi_beads is None else _f64(vxi_beads)
        self._check(load().pimd_set_thermostat_state(self.h, _p(vg), float(uk), _p(vb)), "set_thermostat_state")

    def checkpoint_write(self, path, RRt, PPt, dRRt, t, seed):
        RRt, PPt, dRRt = _f64(RRt), _f64(PPt), _f64(dRRt)
        self._check(load().pimd_checkpoint_write(self.h, str(path).encode(), _p(RRt), _p(PPt), _p(dRRt), int(t),
                                                 int(seed)), "checkpoint_write")

    def checkpoint_read(self, path):
        """(RRt, PPt, dRRt, t, seed) of an exact restart file; the context takes its state."""
        shape = (self.P, self.natoms, 3)
        RRt, PPt, dRRt = np.zeros(shape), np.zeros(shape), np.zeros(shape)
        t, seed = ctypes.c_int(), ctypes.c_ulonglong()
        self._check(load().pimd_checkpoint_read(self.h, str(path).encode(), _p(RRt), _p(PPt), _p(dRRt),
                                                ctypes.byref(t), ctypes.byref(seed)), "checkpoint_read")
        return RRt, PPt, dRRt, t.value, seed.value

    def md_step_ex(self, mp, RRt, PPt, dRRt, t, xi1=None, xi2=None):
        """PIMD_VV on host arrays (in place) with the step's outputs and estimators by name."""
        for a in (RRt, PPt, dRRt):
            assert a.dtype == np.float64 and a.flags.c_contiguous
        RRc = np.zeros((self.natoms, 3))
        out = np.zeros(MD_NOUT)
        x1 = _f64(xi1) if xi1 is not None else None
        x2 = _f64(xi2) if xi2 is not None else None
        rc = load().pimd_md_step_ex(self.h, ctypes.byref(mp), _p(RRt), _p(PPt), _p(dRRt), _p(RRc), _p(x1), _p(x2),
                                    int(t), _p(out))
        self._check(rc, "md_step_ex")
        r = dict(zip(MD_OUT_NAMES, out.tolist()))
        r["RRc"] = RRc
        return r

    def contracted_init(self, mode, intra_timesteps=1):
        """Ring-polymer contraction with MTS (mode 0) or monomer PIMD (mode 1)."""
        self._check(load().pimd_contracted_init(self.h, int(mode), int(intra_timesteps)), "contracted_init")

    def contracted_step(self, mp, RRt, PPt, dRRt, dRRfast, t, xi1=None, xi2=None, dipoles=False):
        """One contracted / monomer-PIMD step on host arrays (in place); outputs by name."""
        for a in (RRt, PPt, dRRt) + (() if dRRfast is None else (dRRfast,)):
            assert a.dtype == np.float64 and a.flags.c_contiguous
        RRc = np.zeros((self.natoms, 3))
        out = np.zeros(MD_NOUT)
        dI = np.zeros((self.P, self.nw, 3)) if dipoles else None
        dE = np.zeros((self.P, self.nw, 3)) if dipoles else None
        x1 = _f64(xi1) if xi1 is not None else None
        x2 = _f64(xi2) if xi2 is not None else None
        rc = load().pimd_contracted_step(self.h, ctypes.byref(mp), _p(RRt), _p(PPt), _p(dRRt), _p(dRRfast), _p(RRc),
                                         _p(x1), _p(x2), int(t), _p(out), _p(dI), _p(dE))
        self._check(rc, "contracted_step")
        r = dict(zip(MD_OUT_NAMES, out.tolist()))
        r.update(RRc=RRc, dip_momIt=dI, dip_momEt=dE)
        return r

    # ---- run analyses (geometry_calculator, diffusion_calculator, spectral_properties) ---------
    def geometry_reset(self):
        self._check(load().pimd_geometry_reset(self.h), "geometry_reset")

    def geometry_accumulate_device(self, RRc_ptr, RRt_ptr):
        self._check(load().pimd_geometry_accumulate_device(self.h, RRc_ptr, RRt_ptr), "geometry_accumulate")

    def geometry_report(self):
        out, hc, hb, acc = np.zeros(14), np.zeros((80, 2)), np.zeros((80, 2)), np.zeros(176)
        self._check(load().pimd_geometry_report(self.h, _p(out), _p(hc), _p(hb), _p(acc)), "geometry_report")
        return dict(report=out, hist_centroid=hc, hist_beads=hb, accumulator=acc)

    def msd_init(self, num_timesteps):
        self._check(load().pimd_msd_init(self.h, int(num_timesteps)), "msd_init")

    def msd_accumulate_device(self, RRc_ptr):
        self._check(load().pimd_msd_accumulate_device(self.h, RRc_ptr), "msd_accumulate")

    def msd_report(self, timestep):
        n = ctypes.c_int()
        out = np.zeros(4)
        aMS = np.zeros(100000)
        self._check(load().pimd_msd_report(self.h, float(timestep), _p(aMS), ctypes.byref(n), _p(out)), "msd_report")
        return dict(aMS=aMS[:n.value].copy(), D=out[0], errD=out[1], slope=out[2], intercept=out[3])

    def spectra_init(self, max_steps, massH):
        self._check(load().pimd_spectra_init(self.h, int(max_steps), float(massH)), "spectra_init")

    def spectra_record_device(self, dip_ptr, PPt_ptr):
        self._check(load().pimd_spectra_record_device(self.h, dip_ptr or None, PPt_ptr or None), "spectra_record")

    def ir_spectrum(self, timestep, temp, npoints=350):
        n = ctypes.c_int(int(npoints))
        f, v = np.zeros(npoints), np.zeros(npoints)
        self._check(load().pimd_ir_spectrum(self.h, float(timestep), float(temp), ctypes.byref(n), _p(f), _p(v)),
                    "ir_spectrum")
        return f[:n.value].copy(), v[:n.value].copy()

    def dos(self, timestep, npoints=350):
        n = ctypes.c_int(int(npoints))
        f, v = np.zeros(npoints), np.zeros(npoints)
        self._check(load().pimd_dos(self.h, float(timestep), ctypes.byref(n), _p(f), _p(v)), "dos")
        return f[:n.value].copy(), v[:n.value].copy()

    def md_step_ex_device(self, mp, RRt, PPt, dRRt, RRc, t, out, xi1=0, xi2=0):
        """pimd_md_step_ex_device on device buffers given as raw pointers (ints), stream-ordered."""
        rc = load().pimd_md_step_ex_device(self.h, ctypes.byref(mp), RRt, PPt, dRRt, RRc, xi1 or None, xi2 or None,
                                           int(t), out)
        self._check(rc, "md_step_ex_device")

    def md_step_device(self, mp, RRt, PPt, dRRt, RRc, t, out4, xi1=0, xi2=0):
        """PIMD_VV on device buffers given as raw pointers (ints), stream-ordered."""
        rc = load().pimd_md_step_device(self.h, ctypes.byref(mp), RRt, PPt, dRRt, RRc, xi1 or None, xi2 or None,
                                        int(t), out4)
        self._check(rc, "md_step_device")

    def set_graph(self, enable=True):
        """Run md_step/md_step_device as a captured CUDA graph (dipole loop on the device)."""
        self._check(load().pimd_set_graph(self.h, int(enable)), "set_graph")

    def graph_info(self):
        c, n = ctypes.c_longlong(), ctypes.c_longlong()
        self._check(load().pimd_graph_info(self.h, ctypes.byref(c), ctypes.byref(n)), "graph_info")
        return c.value, n.value

    def set_stream(self, stream_ptr):
        self._check(load().pimd_set_stream(self.h, stream_ptr), "set_stream")

    # ---- dans_timer-style phase timers ----------------------------------------------------
    def timers_reset(self, enable=True):
        self._check(load().pimd_timers_reset(self.h, int(enable)), "timers_reset")

    def timers(self):
        L = load()
        n = L.pimd_timers_get(self.h, -1, None, 0, None, None)
        out = {}
        buf = ctypes.create_string_buffer(64)
        for i in range(n):
            ms = ctypes.c_double()
            cnt = ctypes.c_longlong()
            L.pimd_timers_get(self.h, i, buf, 64, ctypes.byref(ms), ctypes.byref(cnt))
            out[buf.value.decode()] = (ms.value, cnt.value)
        return out

    # ---- differentiation form ----------------------------------------------------------
    def get_theta(self):
        th = np.zeros(len(THETA_NAMES))
        self._check(load().pimd_get_theta(self.h, _p(th)), "get_theta")
        return th

    def set_theta(self, theta):
        self._check(load().pimd_set_theta(self.h, _p(_f64(theta))), "set_theta")

    def pot_forward(self, RRt, RRc, t=1):
        """Energies Upott (P,) of all beads, recording the dipole iterations for pot_backward."""
        RRt, RRc = _f64(RRt), _f64(RRc)
        U = np.zeros(self.P)
        self._check(load().pimd_pot_forward(self.h, _p(RRt), _p(RRc), _p(U), int(t)), "pot_forward")
        return U

    def pot_backward(self, ebar):
        """dE/dRRt (P, Natoms, 3) and dE/dtheta for E = sum_k ebar[k] Upot_k of the last forward."""
        ebar = _f64(ebar)
        g = np.zeros((self.P, self.natoms, 3))
        dth = np.zeros(len(THETA_NAMES))
        self._check(load().pimd_pot_backward(self.h, _p(ebar), _p(g), _p(dth)), "pot_backward")
        return g, dth

    # ---- autotuner ---------------------------------------------------------------------
    def autotune(self, RRt_ptr=None, RRc_ptr=None):
        """Pick the fastest launch shapes on the current (or given device) positions."""
        self._check(load().pimd_autotune(self.h, RRt_ptr, RRc_ptr), "autotune")
        return self.tuning()

    # pimd_get_tuning / pimd_set_tuning order; qd_tc is a report only (tensor-core force pass in use)
    TUNING_ORDER = ("sf_tiled", "sf_groups", "ff_regs", "max_slices", "nbr_block", "wave_shapes", "sf_tc", "ff_tc",
                    "dd_overlap", "x_cache", "pdl", "loop_unroll", "ewald_overlap", "dd_otf", "qd_tc", "l2_keep",
                    "dd_async", "dd_pev", "dd_jpev", "nbr_overlap")
    TUNING_REPORTS = ("qd_tc",)
    TUNING_KEYS = TUNING_ORDER[:14] + TUNING_ORDER[15:]

    def tuning(self):
        n = len(self.TUNING_ORDER)
        k = (ctypes.c_int * n)()
        self._check(load().pimd_get_tuning(self.h, k, n), "get_tuning")
        return {name: k[i] for i, name in enumerate(self.TUNING_ORDER)}

    def set_tuning(self, **knobs):
        """Set launch-shape knobs by name (the keys of tuning()); the others keep their values."""
        cur = self.tuning()
        unknown = set(knobs) - set(self.TUNING_KEYS)
        if unknown:
            raise ValueError("unknown tuning knobs: %s" % sorted(unknown))
        cur.update({k: int(v) for k, v in knobs.items()})
        n = len(self.TUNING_ORDER)
        k = (ctypes.c_int * n)(*[cur[name] for name in self.TUNING_ORDER])
        self._check(load().pimd_set_tuning(self.h, k, n), "set_tuning")
        return self.tuning()


class ReplicaBatch:
    """Independent ring polymers of uneven sizes stepped together (one CUDA graph per step).

    replicas: list of dicts with natoms, nbeads, box (3,), temp. common: engine parameters
    shared by all (pot_model, rc, rc1, eps_ewald or alpha/nmax, polar settings)."""

    def __init__(self, common, replicas, delt, massO, massH, langevin=1, seed=12345, precision=PIMD_FP64, device=0):
        L = load()
        p = make_params(dict(dict(natoms=3, nbeads=1, box=(1.0, 1.0, 1.0)), **common), precision, device)
        arr = (Replica * len(replicas))()
        for i, r in enumerate(replicas):
            arr[i].natoms = int(r["natoms"])
            arr[i].nbeads = int(r["nbeads"])
            for c in range(3):
                arr[i].box[c] = float(r["box"][c])
            arr[i].temp = float(r["temp"])
        mp = ForceEngine.md_params(delt, massO, massH, langevin, seed)
        h = _V()
        rc = L.pimd_batch_create(ctypes.byref(h), ctypes.byref(p), ctypes.cast(arr, _V), len(replicas), ctypes.byref(mp))
        if rc:
            raise PimdError("pimd_batch_create failed (%d: %s)" % (rc, ERRORS.get(rc, "?")))
        self.h = h
        self.replicas = [dict(r) for r in replicas]

    def close(self):
        if getattr(self, "h", None):
            load().pimd_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, rc, what):
        if rc:
            msg = load().pimd_batch_last_error(self.h)
            raise PimdError("%s failed (%d: %s): %s" % (what, rc, ERRORS.get(rc, "?"), msg.decode() if msg else ""))

    def groups(self):
        n = ctypes.c_int()
        g = (ctypes.c_int * len(self.replicas))()
        self._check(load().pimd_batch_info(self.h, ctypes.byref(n), g), "batch_info")
        return n.value, list(g)

    def set_state(self, r, RRt, PPt):
        self._check(load().pimd_batch_set_state(self.h, r, _p(_f64(RRt)), _p(_f64(PPt))), "batch_set_state")

    def get_state(self, r):
        rep = self.replicas[r]
        shape = (rep["nbeads"], rep["natoms"], 3)
        R, P, G, o = np.zeros(shape), np.zeros(shape), np.zeros(shape), np.zeros(4)
        self._check(load().pimd_batch_get_state(self.h, r, _p(R), _p(P), _p(G), _p(o)), "batch_get_state")
        return R, P, G, o

    def forces(self):
        self._check(load().pimd_batch_forces(self.h), "batch_forces")

    def autotune(self):
        self._check(load().pimd_batch_autotune(self.h), "batch_autotune")

    def step(self, nsteps=1):
        self._check(load().pimd_batch_step(self.h, int(nsteps)), "batch_step")

    def sync(self):
        self._check(load().pimd_batch_sync(self.h), "batch_sync")
