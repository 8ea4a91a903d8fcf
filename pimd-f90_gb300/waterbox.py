"""Seeded synthetic water boxes and free ring-polymer initial conditions.

The workloads are the reference's benchmark configurations: N water molecules on a jittered
cubic-ish lattice in a periodic box spanning [-L/2, L/2]^3, uniform random orientations
(Shoemake quaternions), rigid initial monomer geometry, and P beads drawn from the free
ring-polymer distribution around each atom (NormalModes.f90:224-250 gen_rand_ring) with
momenta from the free-ring momentum distribution (NormalModes.f90:257-275), both at T*P.

Arrays follow the reference's Fortran layouts, stored C-order:
  RRt, PPt: (P, Natoms, 3)  == Fortran RRt(3, Natoms, P)
  RRc:      (Natoms, 3)     == Fortran RRc(3, Natoms)
Atoms are ordered O H H O H H ... (read_method 1 of the reference).
"""
import math

import numpy as np

KB_AMU = 0.831447148       # consts.f90: KB_amuA2ps2perK, amu*A^2/ps^2/K
HBAR = 6.35077993041       # consts.f90: hbar in amu*A^2/ps
BASE_SEED = 20261203

# name -> (pot_model, N, L, P, Rc, nmax, r_OH, theta_HOH_deg)
CONFIGS = {
    "qspcfw_32x8": dict(pot_model=4, nw=32, L=9.865, P=8, rc=4.9, nmax=7, alpha=3.0 / 4.9,
                        roh=1.0, theta=112.0, index=1),
    "ttm21f_128x32": dict(pot_model=2, nw=128, L=15.66, P=32, rc=7.8, nmax=9, alpha=None,
                          roh=0.9572, theta=104.52, index=2),
    "ttm3f_512x32": dict(pot_model=3, nw=512, L=24.86, P=32, rc=9.0, nmax=12, alpha=None,
                         roh=0.9572, theta=104.52, index=3),
    "ttm3f_4096x32": dict(pot_model=3, nw=4096, L=49.72, P=32, rc=9.0, nmax=24, alpha=None,
                          roh=0.9572, theta=104.52, index=5),
}


def ewald_alpha_eps(rc, eps=1.0e-6):
    """ewald.f90:312-313: alpha = sqrt(-ln eps)/Rc."""
    return math.sqrt(-math.log(eps)) / rc


def lattice_dims(n):
    """Near-cubic lattice (nx >= ny >= nz, each within 2 of ceil(n^(1/3))) with the fewest
    sites >= n: 32 -> 4x4x2, 128 -> 6x6x4, 512 -> 8x8x8, 4096 -> 16x16x16."""
    c = int(math.ceil(n ** (1.0 / 3.0) - 1e-9))
    best = None
    for nx in range(max(1, c - 2), c + 1):
        for ny in range(max(1, c - 2), nx + 1):
            for nz in range(max(1, c - 2), ny + 1):
                tot = nx * ny * nz
                if tot >= n and (best is None or tot < best[0]):
                    best = (tot, (nx, ny, nz))
    return best[1]


def _shoemake(rng, n):
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], axis=1)
    x, y, z, w = q.T
    Rm = np.empty((n, 3, 3))
    Rm[:, 0, 0] = 1 - 2 * (y * y + z * z)
    Rm[:, 0, 1] = 2 * (x * y - z * w)
    Rm[:, 0, 2] = 2 * (x * z + y * w)
    Rm[:, 1, 0] = 2 * (x * y + z * w)
    Rm[:, 1, 1] = 1 - 2 * (x * x + z * z)
    Rm[:, 1, 2] = 2 * (y * z - x * w)
    Rm[:, 2, 0] = 2 * (x * z - y * w)
    Rm[:, 2, 1] = 2 * (y * z + x * w)
    Rm[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return Rm


def centroid_box(nw, L, roh, theta_deg, seed, jitter=0.3):
    """Centroid coordinates RRc (Natoms, 3) of nw molecules in a cube of side L."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = lattice_dims(nw)
    grid = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    if len(grid) > nw:
        grid = grid[np.sort(rng.choice(len(grid), nw, replace=False))]
    cell = np.array([L / nx, L / ny, L / nz])
    O = (grid + 0.5) * cell - L / 2 + rng.uniform(-jitter, jitter, size=(nw, 3))
    th = math.radians(theta_deg)
    body = np.array([[0.0, 0.0, 0.0],
                     [roh * math.sin(th / 2), 0.0, roh * math.cos(th / 2)],
                     [-roh * math.sin(th / 2), 0.0, roh * math.cos(th / 2)]])
    Rm = _shoemake(rng, nw)
    atoms = O[:, None, :] + np.einsum("nij,aj->nai", Rm, body)
    return atoms.reshape(3 * nw, 3)


def nm_matrices(P, omegan, delta=0.0, setNMfreq=0.0):
    """NormalModes.f90:68-218 InitNormalModes (C, omegalist, mass scale factors)."""
    l = (P - 2) // 2 if P % 2 == 0 else (P - 1) // 2
    C = np.zeros((P, P))
    for i in range(1, P + 1):
        C[0, i - 1] = math.sqrt(1.0 / P)
        for k in range(1, l + 1):
            C[k, i - 1] = math.sqrt(2.0 / P) * math.cos(k * i * 2.0 * math.pi / P)
            C[k + l, i - 1] = math.sqrt(2.0 / P) * math.sin(k * i * 2.0 * math.pi / P)
        if P % 2 == 0:
            C[2 * l + 1, i - 1] = math.sqrt(1.0 / P) * (-1) ** i
    om = np.zeros(P)
    ks = list(range(1, l + 1)) * 2 + ([l + 1] if P % 2 == 0 else [])
    for idx, k in enumerate(ks):
        ratio = float(np.float32(np.float32(abs(k)) / np.float32(P)))
        om[idx + 1] = 2 * omegan * math.sin(math.pi * ratio)
    msf = np.ones(P)
    return C, om, msf


def ring_polymer(RRc, P, T, massO, massH, seed):
    """Beads around centroids: gen_rand_ring at T (NormalModes.f90:224-250) and momenta from
    gen_rand_ring_momenta at T*P (NormalModes.f90:257-275). Returns RRt, PPt (P, Natoms, 3)."""
    rng = np.random.default_rng(seed + 7919)
    na = RRc.shape[0]
    omegan = KB_AMU * T * P / HBAR
    C, om, msf = nm_matrices(P, omegan)
    mass = np.where(np.arange(na) % 3 == 0, massO, massH)
    RRtr = np.zeros((na, P, 3))
    for j in range(P):
        if om[j] != 0.0:
            std = np.sqrt((omegan * HBAR) / (mass * msf[j] * om[j] ** 2))
            RRtr[:, j, :] = rng.standard_normal((na, 3)) * std[:, None]
    # NM2real: RR(:, j) = sum_k C(k, j) RRtr(:, k)
    RRt = np.einsum("kj,akc->jac", C, RRtr) + RRc[None, :, :]
    PPtr = rng.standard_normal((na, P, 3)) * np.sqrt(KB_AMU * mass[:, None, None] * msf[None, :, None] * T * P)
    PPt = np.einsum("kj,akc->jac", C, PPtr)
    return np.ascontiguousarray(RRt), np.ascontiguousarray(PPt)


def make_config(name, massO=15.9994, massH=1.008, T=300.0, P=None, nw=None, seed=None):
    """Build one benchmark workload. Returns a dict with params and arrays."""
    c = dict(CONFIGS[name])
    if P is not None:
        c["P"] = P
    L = c["L"]
    if nw is not None and nw != c["nw"]:
        L = (nw * 29.96) ** (1.0 / 3.0)
        c["nw"] = nw
        c["L"] = L
    seed = BASE_SEED + c["index"] if seed is None else seed
    RRc = centroid_box(c["nw"], L, c["roh"], c["theta"], seed)
    RRt, PPt = ring_polymer(RRc, c["P"], T, massO, massH, seed)
    alpha = c["alpha"] if c["alpha"] is not None else ewald_alpha_eps(c["rc"])
    params = dict(pot_model=c["pot_model"], natoms=3 * c["nw"], box=(L, L, L), rc=c["rc"], rc1=0.8 * c["rc"],
                  eps_ewald=1.0e-6, alpha=alpha, nmax=c["nmax"], polar_maxiter=100, polar_sor=0.7,
                  polar_eps=1.0e-8, guess_initdip=0, contraction=0, nbeads=c["P"])
    RRc_true = RRt.mean(axis=0)
    return dict(name=name, params=params, RRt=RRt, PPt=PPt, RRc=RRc_true, T=T, massO=massO, massH=massH)
