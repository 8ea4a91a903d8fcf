"""ctypes binding of the CPU FP64 oracle (pimd_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, always as the checker or the timed CPU baseline, never by the engine.
Parity status: unpinned by the reference's own outputs (no Fortran compiler to build the
reference); pinned by physics known-answer tests.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build(force=False):
    """Compile the oracle with the host compiler: IEEE double, no FMA contraction."""
    src = os.path.join(HERE, "pimd_oracle.cpp")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", src, "-o", LIB]
    subprocess.check_call(cmd)
    return LIB


class Params(ctypes.Structure):
    _fields_ = [("pot_model", ctypes.c_int), ("natoms", ctypes.c_int), ("box", ctypes.c_double * 3),
                ("rc", ctypes.c_double), ("rc1", ctypes.c_double), ("eps_ewald", ctypes.c_double),
                ("alpha", ctypes.c_double), ("nmax", ctypes.c_int), ("polar_maxiter", ctypes.c_int),
                ("polar_sor", ctypes.c_double), ("polar_eps", ctypes.c_double),
                ("guess_initdip", ctypes.c_int), ("contraction", ctypes.c_int), ("nbeads", ctypes.c_int),
                ("shared_history", ctypes.c_int)]


class MDParams(ctypes.Structure):
    _fields_ = [("delt", ctypes.c_double), ("massO", ctypes.c_double), ("massH", ctypes.c_double),
                ("setNMfreq", ctypes.c_double), ("langevin", ctypes.c_int),
                ("centroid_thermostat", ctypes.c_int), ("tau_centroid", ctypes.c_double),
                ("temp", ctypes.c_double)]


def make_params(d):
    p = Params()
    p.pot_model = int(d["pot_model"])
    p.natoms = int(d["natoms"])
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
    p.nbeads = int(d.get("nbeads", 1))
    p.shared_history = int(d.get("shared_history", 0))
    return p


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        D = ctypes.POINTER(ctypes.c_double)
        I = ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.POINTER(Params)]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_ewald_info.argtypes = [ctypes.c_void_p, D, I, I]
        L.orc_kvectors.argtypes = [ctypes.c_void_p, I, D, D]
        L.orc_pot_ttm.argtypes = [ctypes.c_void_p, ctypes.c_int, D, D, D, D, D, D, D, D, D, ctypes.c_int]
        L.orc_pot_spc.argtypes = [ctypes.c_void_p, D, D, D, D, D, D]
        L.orc_energies.argtypes = [ctypes.c_void_p, D, I, D]
        L.orc_neighbors.argtypes = [ctypes.c_void_p, D, I, ctypes.c_int]
        L.orc_neighbors.restype = ctypes.c_int
        L.orc_full_bead_forces.argtypes = [ctypes.POINTER(Params), ctypes.c_int, D, D, D, D, D, D, D, D, D,
                                           ctypes.c_int]
        L.orc_nm_init.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, D, D, D, D, D,
                                  D, D]
        L.orc_evolve_ring.argtypes = [ctypes.c_int, D, D, D, D, D, D, D, D, ctypes.c_double]
        L.orc_langevin_init.argtypes = [ctypes.c_int, D, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, D, D]
        L.orc_langevin_nm.argtypes = [ctypes.c_int, ctypes.c_int, D, D, D, D, ctypes.c_double, ctypes.c_double,
                                      D, D]
        L.orc_calc_uk.restype = ctypes.c_double
        L.orc_calc_uk.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, D,
                                  ctypes.c_double, D, D]
        L.orc_pimd_vv_step.argtypes = [ctypes.c_void_p, ctypes.POINTER(MDParams), ctypes.c_int, D, D, D, D, D, D,
                                       ctypes.c_int, D, D, D, D]
        L.orc_pool_create.restype = ctypes.c_void_p
        L.orc_pool_create.argtypes = [ctypes.POINTER(Params), ctypes.c_int]
        L.orc_pool_destroy.argtypes = [ctypes.c_void_p]
        L.orc_pool_forces.argtypes = [ctypes.c_void_p, D, D, D, D, D, D, ctypes.c_int]
        L.orc_pimd_vv_step_pool.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(MDParams),
                                            ctypes.c_int, D, D, D, D, D, D, ctypes.c_int, D, D, D, D]
        L.orc_real2nm.argtypes = [ctypes.c_int, D, D, D]
        L.orc_nm2real.argtypes = [ctypes.c_int, D, D, D]
        L.orc_gen_rand_ring.argtypes = [ctypes.c_int, D, D, D, ctypes.c_double, ctypes.c_double, D, D]
        L.orc_gen_rand_ring_momenta.argtypes = [ctypes.c_int, D, D, ctypes.c_double, ctypes.c_double, D, D]
        L.orc_contracted_step.argtypes = [ctypes.c_void_p, ctypes.POINTER(MDParams), ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, D, D, D, D, D, D,
                                          D, D, D, D, ctypes.c_int, D, D, D]
        F = ctypes.POINTER(ctypes.c_float)
        L.orc_geometry_accumulate.argtypes = [D, ctypes.c_int, ctypes.c_int, D, D, D]
        L.orc_geometry_report.argtypes = [D, ctypes.c_int, D]
        L.orc_msd_step.argtypes = [D, ctypes.c_int, ctypes.c_int, D, D]
        L.orc_msd_report.argtypes = [D, ctypes.c_int, ctypes.c_double, D]
        L.orc_four1.argtypes = [F, ctypes.c_int, ctypes.c_int]
        L.orc_ir_spectrum.argtypes = [F, ctypes.c_int, D, ctypes.c_double, ctypes.c_double, I, D, D]
        L.orc_dos.argtypes = [F, ctypes.c_int, ctypes.c_int, ctypes.c_double, I, D, D]
        L.orc_nose_hoover.argtypes = [D, D, D, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_double]
        L.orc_estimators.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 7 + [D]
        L.orc_ring_k0.restype = ctypes.c_double
        L.orc_ring_k0.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, D]
        L.orc_pimd_vv_step_ex.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(MDParams), ctypes.c_int,
                                          ctypes.c_int, ctypes.c_double, ctypes.c_int, D, D, D, D, D, D, D, D, D,
                                          ctypes.c_int, D]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """One reference 'rank': the module state of init_pot plus one pot_ttm/pot_spc at a time."""

    def __init__(self, params):
        self.params = dict(params)
        self._p = make_params(params)
        self.h = lib().orc_create(ctypes.byref(self._p))
        self.natoms = self._p.natoms
        self.nw = self.natoms // 3

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def ewald_info(self):
        a = ctypes.c_double()
        nk = ctypes.c_int()
        hkl = (ctypes.c_int * 3)()
        lib().orc_ewald_info(self.h, ctypes.byref(a), ctypes.byref(nk), hkl)
        return a.value, nk.value, tuple(hkl)

    def kvectors(self):
        _, nk, _ = self.ewald_info()
        hkl = np.zeros((nk, 3), np.int32)
        kv = np.zeros((nk, 3))
        Ak = np.zeros(nk)
        lib().orc_kvectors(self.h, hkl.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(kv), _p(Ak))
        return hkl, kv, Ak

    def energies(self):
        U = np.zeros(4)
        it = ctypes.c_int()
        dd = ctypes.c_double()
        lib().orc_energies(self.h, _p(U), ctypes.byref(it), ctypes.byref(dd))
        return dict(Umon=U[0], Uvdw=U[1], Uelec=U[2], Uind=U[3], niter=it.value, deltadip=dd.value)

    def neighbors(self, RR):
        """All (i, j) O-O pairs of find_neigh in the reference's order, shape (npairs, 2)."""
        RR = _f64(RR)
        cap = self.nw * (self.nw - 1) // 2 + 1
        ij = np.zeros((cap, 2), np.int32)
        n = lib().orc_neighbors(self.h, _p(RR), ij.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), cap)
        return ij[:n].copy()

    def pot_ttm(self, RR, RRc, t=1, bead=0):
        RR, RRc = _f64(RR), _f64(RRc)
        En, vc = ctypes.c_double(), ctypes.c_double()
        dRR = np.zeros_like(RR)
        virt = np.zeros(9)
        dI = np.zeros((self.nw, 3))
        dE = np.zeros((self.nw, 3))
        chg = np.zeros(self.natoms)
        lib().orc_pot_ttm(self.h, bead, _p(RR), _p(RRc), ctypes.byref(En), _p(dRR), _p(virt), ctypes.byref(vc),
                          _p(dI), _p(dE), _p(chg), int(t))
        out = dict(En=En.value, dRR=dRR, virt=virt.reshape(3, 3, order="F"), virialc=vc.value, dip_momI=dI,
                   Edip_mom=dE, chg=chg)
        out.update(self.energies())
        return out

    def pot_spc(self, RR):
        RR = _f64(RR)
        En = ctypes.c_double()
        dRR = np.zeros_like(RR)
        virt = np.zeros(9)
        dI = np.zeros((self.nw, 3))
        chg = np.zeros(self.natoms)
        lib().orc_pot_spc(self.h, _p(RR), ctypes.byref(En), _p(dRR), _p(virt), _p(dI), _p(chg))
        out = dict(En=En.value, dRR=dRR, virt=virt.reshape(3, 3, order="F"), dip_momI=dI, chg=chg)
        out.update(self.energies())
        return out

    def potential(self, RR, RRc, t=1, bead=0):
        if self._p.pot_model in (2, 3):
            return self.pot_ttm(RR, RRc, t, bead)
        return self.pot_spc(RR)


def full_bead_forces(params, RRt, RRc, t=1, nthreads=None):
    """force_calc.f90:26-106 over all beads, one bead per worker thread at a time."""
    p = make_params(params)
    P = p.nbeads
    na = p.natoms
    RRt, RRc = _f64(RRt), _f64(RRc)
    assert RRt.shape == (P, na, 3)
    Upott, virialt, virialct = np.zeros(P), np.zeros(P), np.zeros(P)
    dRRt = np.zeros_like(RRt)
    dI = np.zeros((P, na // 3, 3))
    dE = np.zeros((P, na // 3, 3))
    chg = np.zeros(na)
    nthreads = nthreads or os.cpu_count() or 1
    lib().orc_full_bead_forces(ctypes.byref(p), int(nthreads), _p(RRt), _p(RRc), _p(Upott), _p(dRRt),
                               _p(virialt), _p(virialct), _p(dI), _p(dE), _p(chg), int(t))
    return dict(Upott=Upott, dRRt=dRRt, virialt=virialt, virialct=virialct, dip_momIt=dI, dip_momEt=dE, chg=chg,
                Upot=Upott.sum(), virial=virialt.sum(), virialc=virialct.sum() / P)


def nm_init(P, omegan, delta, setNMfreq=0.0):
    A = [np.zeros(P) for _ in range(6)]
    C = np.zeros(P * P)
    lib().orc_nm_init(P, omegan, delta, setNMfreq, *[_p(a) for a in A], _p(C))
    return dict(A11=A[0], A12=A[1], A21=A[2], A22=A[3], omegalist=A[4], msf=A[5], C=C.reshape(P, P, order="F"))


def evolve_ring(nm, RR, PP, mass):
    """RR, PP: (P, 3) one atom's beads; returns updated copies."""
    P = RR.shape[0]
    RR, PP = _f64(RR).copy(), _f64(PP).copy()
    C = np.asfortranarray(nm["C"]).ravel(order="F")
    C = np.ascontiguousarray(C)
    lib().orc_evolve_ring(P, _p(nm["A11"]), _p(nm["A12"]), _p(nm["A21"]), _p(nm["A22"]), _p(nm["msf"]), _p(C),
                          _p(RR), _p(PP), float(mass))
    return RR, PP


def langevin_init(nm, delt2, centroid_thermostat, tau, temp_P):
    P = len(nm["omegalist"])
    c1, c2 = np.zeros(P), np.zeros(P)
    lib().orc_langevin_init(P, _p(nm["omegalist"]), delt2, int(centroid_thermostat), tau, temp_P, _p(c1), _p(c2))
    return c1, c2


def langevin_nm(nm, c1, c2, massO, massH, PPt, xi):
    """PPt (P, Natoms, 3); xi (Natoms, P, 3) standard normals. Returns updated copy."""
    P, na, _ = PPt.shape
    PPt = _f64(PPt).copy()
    C = np.ascontiguousarray(np.asfortranarray(nm["C"]).ravel(order="F"))
    lib().orc_langevin_nm(P, na, _p(C), _p(nm["msf"]), _p(c1), _p(c2), massO, massH, _p(PPt), _p(_f64(xi)))
    return PPt


def calc_uk(nm, massO, massH, PPt, setNMfreq=0.0):
    P, na, _ = PPt.shape
    C = np.ascontiguousarray(np.asfortranarray(nm["C"]).ravel(order="F"))
    return lib().orc_calc_uk(P, na, massO, massH, _p(_f64(PPt)), setNMfreq, _p(C), _p(nm["msf"]))


class Pool:
    """Host-core bead pool: bead k always on worker k % nthreads (an MPI rank per thread)."""

    def __init__(self, params, nthreads=None):
        self._p = make_params(params)
        self.nthreads = int(nthreads or os.cpu_count() or 1)
        self.h = lib().orc_pool_create(ctypes.byref(self._p), self.nthreads)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_pool_destroy(self.h)
            self.h = None

    def forces(self, RRt, RRc, t=1):
        P = self._p.nbeads
        RRt, RRc = _f64(RRt), _f64(RRc)
        U, v, vc = np.zeros(P), np.zeros(P), np.zeros(P)
        dRRt = np.zeros_like(RRt)
        lib().orc_pool_forces(self.h, _p(RRt), _p(RRc), _p(U), _p(dRRt), _p(v), _p(vc), int(t))
        return dict(Upott=U, dRRt=dRRt, virialt=v, virialct=vc)


def pimd_vv_step(orc, md, RRt, PPt, dRRt, xi1=None, xi2=None, t=1, pool=None):
    """MD.f90:35-110 one velocity-Verlet PIMD step; arrays (P, Natoms, 3) updated in place.
    With a Pool the force call is spread over its worker threads."""
    mp = MDParams()
    mp.delt = md["delt"]
    mp.massO = md["massO"]
    mp.massH = md["massH"]
    mp.setNMfreq = md.get("setNMfreq", 0.0)
    mp.langevin = int(md.get("langevin", 1))
    mp.centroid_thermostat = int(md.get("centroid_thermostat", 0))
    mp.tau_centroid = md.get("tau_centroid", 0.1)
    mp.temp = md["temp"]
    P = RRt.shape[0]
    RRc = np.zeros(RRt.shape[1:])
    U, v, vc, uk = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    x1 = _p(_f64(xi1)) if xi1 is not None else None
    x2 = _p(_f64(xi2)) if xi2 is not None else None
    lib().orc_pimd_vv_step_pool(orc.h, pool.h if pool is not None else None, ctypes.byref(mp), P, _p(RRt), _p(PPt),
                                _p(dRRt), _p(RRc), x1, x2, int(t), ctypes.byref(U), ctypes.byref(v),
                                ctypes.byref(vc), ctypes.byref(uk))
    return dict(Upot=U.value, virial=v.value, virialc=vc.value, uk=uk.value, RRc=RRc)


MD_NOUT = 12
MD_OUT_NAMES = ("Upot", "virial", "virialc", "uk", "uk_mid", "K0", "sys_temp", "E_virial", "P_virial", "E_simple",
                "P_simple", "s_global")


def _md_params(md):
    mp = MDParams()
    mp.delt = md["delt"]
    mp.massO = md["massO"]
    mp.massH = md["massH"]
    mp.setNMfreq = md.get("setNMfreq", 0.0)
    mp.langevin = int(md.get("langevin", 1))
    mp.centroid_thermostat = int(md.get("centroid_thermostat", 0))
    mp.tau_centroid = md.get("tau_centroid", 0.1)
    mp.temp = md["temp"]
    return mp


def thermostat_state(P, natoms, uk=0.0):
    """The reference's initial chain state (InputOutput.f90:397-404): vxi_global = 1, vxi_beads = 0
    (layout (3, P, natoms, 2) = vxi_beads(2, natoms, P, 3)), and the module variable uk."""
    return dict(vxi_global=np.ones(2), uk=float(uk), vxi_beads=np.zeros((3, P, natoms, 2)))


def pimd_vv_step_ex(orc, md, RRt, PPt, dRRt, state, t=1, xi1=None, xi2=None, bead_thermostat=0, global_thermostat=0,
                    tau=0.1, pool=None):
    """PIMD_VV (MD.f90:35-110) with bead thermostat 0 none / 1 Langevin_NM (xi1, xi2) / 2 Nose-Hoover
    on the normal modes, and the global chain thermostat; arrays updated in place, state (chain
    velocities, uk) updated in place. Returns the 12 outputs of the step by name."""
    mp = _md_params(md)
    P = RRt.shape[0]
    RRc = np.zeros(RRt.shape[1:])
    out = np.zeros(MD_NOUT)
    vg = state["vxi_global"]
    vb = state["vxi_beads"]
    assert vg.dtype == np.float64 and vg.flags.c_contiguous and vb.flags.c_contiguous
    uk = ctypes.c_double(state["uk"])
    x1 = _p(_f64(xi1)) if xi1 is not None else None
    x2 = _p(_f64(xi2)) if xi2 is not None else None
    lib().orc_pimd_vv_step_ex(orc.h, pool.h if pool is not None else None, ctypes.byref(mp), int(bead_thermostat),
                              int(global_thermostat), float(tau), P, _p(RRt), _p(PPt), _p(dRRt), _p(RRc), x1, x2,
                              _p(vg), ctypes.byref(uk), _p(vb), int(t), _p(out))
    state["uk"] = uk.value
    r = dict(zip(MD_OUT_NAMES, out.tolist()))
    r["RRc"] = RRc
    return r


def nose_hoover(uk, vxi, tau, delt2, L, temp):
    """Nose_Hoover.f90:33-112 half step: returns (s, uk); vxi (2,) updated in place."""
    s, u = ctypes.c_double(), ctypes.c_double(uk)
    lib().orc_nose_hoover(ctypes.byref(s), ctypes.byref(u), _p(vxi), float(tau), float(delt2), int(L), float(temp))
    return s.value, u.value


def estimators(natoms, P, volume, omegan, Upot, virial, virialc, uk, K0):
    e = np.zeros(5)
    lib().orc_estimators(int(natoms), int(P), float(volume), float(omegan), float(Upot), float(virial),
                         float(virialc), float(uk), float(K0), _p(e))
    return dict(zip(("sys_temp", "E_virial", "P_virial", "E_simple", "P_simple"), e.tolist()))


def ring_k0(massO, massH, RRt):
    """estimators.f90:57-73: K0 = sum over beads, atoms, components of m (r_k - r_(k-1))^2."""
    RRt = _f64(RRt)
    return lib().orc_ring_k0(RRt.shape[0], RRt.shape[1], float(massO), float(massH), _p(RRt))


def _colmajor(C):
    return np.asfortranarray(C).ravel(order="F")


def real2nm(nm, A):
    """NormalModes.f90:308-324 for one atom: A (P, 3) -> (P, 3)."""
    A = _f64(A)
    out = np.zeros_like(A)
    lib().orc_real2nm(A.shape[0], _p(_f64(_colmajor(nm["C"]))), _p(A), _p(out))
    return out


def nm2real(nm, A):
    """NormalModes.f90:327-341 for one atom."""
    A = _f64(A)
    out = np.zeros_like(A)
    lib().orc_nm2real(A.shape[0], _p(_f64(_colmajor(nm["C"]))), _p(A), _p(out))
    return out


def gen_rand_ring(nm, mass, temp, xi):
    """NormalModes.f90:224-250 with unit normals xi (P, 3)."""
    P = len(nm["msf"])
    RR = np.zeros((P, 3))
    lib().orc_gen_rand_ring(P, _p(_f64(_colmajor(nm["C"]))), _p(_f64(nm["omegalist"])), _p(_f64(nm["msf"])),
                            float(mass), float(temp), _p(_f64(xi)), _p(RR))
    return RR


def gen_rand_ring_momenta(nm, mass, temp, xi):
    """NormalModes.f90:257-275 with unit normals xi (P, 3)."""
    P = len(nm["msf"])
    PP = np.zeros((P, 3))
    lib().orc_gen_rand_ring_momenta(P, _p(_f64(_colmajor(nm["C"]))), _p(_f64(nm["msf"])), float(mass), float(temp),
                                    _p(_f64(xi)), _p(PP))
    return PP


def contracted_step(orc_c, md, mode, intra, RRt, PPt, dRRt, dRRfast, state, t=1, xi1=None, xi2=None,
                    bead_thermostat=0, global_thermostat=0, tau=0.1, dipoles=False):
    """contracted_MD (mode 0, MD.f90:276-449) / monomer_PIMD (mode 1, MD.f90:117-265); orc_c is a
    one-bead Oracle of the centroid (contraction=1 in mode 0). Arrays updated in place."""
    mp = _md_params(md)
    P, na = RRt.shape[0], RRt.shape[1]
    RRc = np.zeros(RRt.shape[1:])
    out = np.zeros(MD_NOUT)
    uk = ctypes.c_double(state["uk"])
    x1 = _p(_f64(xi1)) if xi1 is not None else None
    x2 = _p(_f64(xi2)) if xi2 is not None else None
    dI = np.zeros((P, na // 3, 3)) if dipoles else None
    dE = np.zeros((P, na // 3, 3)) if dipoles else None
    lib().orc_contracted_step(orc_c.h, ctypes.byref(mp), int(mode), int(intra), int(bead_thermostat),
                              int(global_thermostat), float(tau), P, _p(RRt), _p(PPt), _p(dRRt), _p(dRRfast), _p(RRc),
                              x1, x2, _p(state["vxi_global"]), ctypes.byref(uk), _p(state["vxi_beads"]), int(t),
                              _p(out), _p(dI), _p(dE))
    state["uk"] = uk.value
    r = dict(zip(MD_OUT_NAMES, out.tolist()))
    r.update(RRc=RRc, dip_momIt=dI, dip_momEt=dE)
    return r


def _pf(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class Geometry:
    """geometry_calculator.f90: calc_geometry per frame, write_out_geometry / write_out_histogram."""

    def __init__(self, natoms, P, box):
        self.acc = np.zeros(176)
        self.natoms, self.P, self.box = natoms, P, _f64(box)

    def accumulate(self, RRc, RRt):
        lib().orc_geometry_accumulate(_p(self.acc), self.natoms, self.P, _p(self.box), _p(_f64(RRc)), _p(_f64(RRt)))

    def report(self):
        out = np.zeros(14)
        lib().orc_geometry_report(_p(self.acc), self.P, _p(out))
        return out


class MSD:
    """diffusion_calculator.f90: calc_diff_RMSD per frame and write_out_diffusion."""

    def __init__(self, natoms, num_timesteps, box):
        self.ntimes = int(np.floor(np.float32(num_timesteps) / np.float32(20)))
        self.natoms = natoms
        self.st = np.zeros(2 + self.ntimes + 1 + 2 * natoms)
        self.box = _f64(box)

    def step(self, RRc):
        lib().orc_msd_step(_p(self.st), self.natoms, self.ntimes, _p(self.box), _p(_f64(RRc)))

    def report(self, timestep):
        out = np.zeros(4)
        aMS = self.st[2:2 + self.ntimes].copy()
        lib().orc_msd_report(_p(aMS), self.ntimes, float(timestep), _p(out))
        return dict(aMS=aMS, D=out[0], errD=out[1], slope=out[2], intercept=out[3])


def four1(z, isign):
    """four1.f on a complex64 array (in place on a copy)."""
    d = np.ascontiguousarray(np.asarray(z, np.complex64)).view(np.float32).copy()
    lib().orc_four1(_pf(d), len(d) // 2, int(isign))
    return d.view(np.complex64)


def ir_spectrum(dip, box, timestep, temp, npoints=350):
    """spectral_properties.f90 calc_infrared_spectrum; dip (tread, 3) float32 total dipoles (Debye)."""
    d = np.ascontiguousarray(dip, np.float32)
    n = ctypes.c_int(npoints)
    f, v = np.zeros(npoints), np.zeros(npoints)
    lib().orc_ir_spectrum(_pf(d), d.shape[0], _p(_f64(box)), float(timestep), float(temp), ctypes.byref(n), _p(f),
                          _p(v))
    return f[:n.value], v[:n.value]


def dos(hvel, timestep, npoints=350):
    """spectral_properties.f90 calc_DOS; hvel (nhyd, tread, 3) float32."""
    h = np.ascontiguousarray(hvel, np.float32)
    n = ctypes.c_int(npoints)
    f, v = np.zeros(npoints), np.zeros(npoints)
    lib().orc_dos(_pf(h), h.shape[1], h.shape[0], float(timestep), ctypes.byref(n), _p(f), _p(v))
    return f[:n.value], v[:n.value]
