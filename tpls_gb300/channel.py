"""Seeded channel workloads (the two-layer stratified channel of the
benchmark configurations) built with the reference's own initial-condition
routine for the base flow.

Two geometries:

* ``"cubic"`` (default): cubic cells dx = dy = dz = 1/nz, Lz = 1,
  Lx = nx dz, Ly = ny dz (the grid of twophase_initialisation_wave.F90:66-75);
* ``"box"``: the 2*pi x pi x 1 channel, dx = 2 pi/nx, dy = pi/ny, dz = 1/nz
  (dx, dy and dz all differ on grids such as 37x19x23).

Inlet/outlet in x, periodic y, no-slip walls in z (the reference's boundary
conditions).  Two layers: mu_minus = m below the interface (phi < 0),
mu_plus = 1 above; viscosity (mu)/Re.

Long runs use cubic cells: the reference's redistancing (levelset.f90) uses
one spacing h = dx for every direction (the Godunov gradient and the inlet
row z = k h - h/2, levelset.f90:168-177), so on the 2*pi x pi x 1 box
(dx = 4.7 dz at 256x128x192) it drives phi towards a distance function
stretched 4.7 times in z; the interface band collapses and the reference's
algorithm diverges (NaN near step 85 at 256x128x192).  A few steps on the
box are well-defined arithmetic, which the parity tests check.

* phi = z - h(x, y) on every p-grid point including ghosts, with cell
  centres x_i = (i-1/2)dx, y_j = (j-1/2)dy, z_k = (k-1/2)dz;
* u(z) from twophase_initialisation_wave.F90:79-122 (10000 sweeps, dpdl=-1)
  on every u point, plus seeded uniform noise of +-1e-3 on the interior u, v
  and w points (w stays 0 on the walls); u_inlet(k) = u(z_k);
* p = -x with x = i*dx - dx/2 (twophase_initialisation_wave.F90:145-154),
  p_old = 0 (main_ns_hybrid.F90:423);
* smooth_width = 1.5 dx, scap = 1, height = 0.5,
  dt = min(0.2 dx / max u, 0.5 sqrt(dx^3 / (2 pi))) (CFL 0.2; the capillary
  bound is below it only for slow, low-Re instances).

Noise comes from SplitMix64(seed) in Fortran order over u, then v, then w;
interface modes from numpy's PCG64(seed).  There is no public dataset for
this path: these synthetic fields are the workload.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .api import Params, base_profile

SEED0 = 20261203
GAMMA = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """n consecutive SplitMix64 outputs (uint64) starting after `offset`."""
    with np.errstate(over="ignore"):
        idx = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * GAMMA
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
        return z ^ (z >> np.uint64(31))


def uniform_pm(seed: int, n: int, amp: float, offset: int = 0) -> np.ndarray:
    u53 = (splitmix64(seed, n, offset) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return (2.0 * u53 - 1.0) * amp


@dataclass
class Workload:
    name: str
    nx: int
    ny: int
    nz: int
    m: float          # viscosity ratio mu_lower / mu_upper
    re: float
    r: float          # density ratio (no reference semantics; recorded only)
    amp_max: float
    modes: int        # 0 = the single-mode interface of the 64x32x48 case
    steps: int
    seed: int
    # > 0: interface modes limited to wavelengths >= this length (kx, ky <=
    # L / min_wavelength; ky = 0 when Ly is shorter), for the batched and
    # served instances whose boxes can be narrow
    min_wavelength: float = 0.0


WORKLOADS = {
    "A": Workload("A: 64x32x48 FP64, m=2, Re=100, 1-mode interface", 64, 32, 48, 2.0, 100.0, 1.0, 0.05, 0, 100,
                  SEED0 + 0),
    "B": Workload("B: 256x128x192 FP64, m=2, Re=200, 4-mode interface", 256, 128, 192, 2.0, 200.0, 1.0, 0.05, 4,
                  200, SEED0 + 1),
    "C": Workload("C: 512x256x256 FP32-mixed, m=20, Re=500, 4-mode interface", 512, 256, 256, 20.0, 500.0, 10.0,
                  0.08, 4, 500, SEED0 + 2),
    # profiling case: the physics of B on a grid whose sweep working set
    # (~200 MB of coefficient records) exceeds the 129 MB L2 while the whole
    # channel stays near 1.5 GB on the device
    "M": Workload("M: 192x96x144 FP64 profiling case, m=2, Re=200, 4-mode interface", 192, 96, 144, 2.0, 200.0,
                  1.0, 0.05, 4, 200, SEED0 + 5),
}


def interface_height(w: Workload, x: np.ndarray, y: np.ndarray, Lx: float, Ly: float) -> np.ndarray:
    if w.modes == 0:
        return 0.5 + w.amp_max * np.sin(2.0 * np.pi * x / Lx) * np.cos(2.0 * np.pi * y / Ly)
    rng = np.random.default_rng(w.seed)
    if w.min_wavelength > 0.0:
        kxm = max(1, min(4, int(Lx // w.min_wavelength)))
        kym = min(4, int(Ly // w.min_wavelength))
        kx = rng.integers(1, kxm + 1, size=w.modes)
        ky = rng.integers(1, kym + 1, size=w.modes) if kym >= 1 else np.zeros(w.modes, dtype=np.int64)
    else:
        kx = rng.integers(1, 5, size=w.modes)
        ky = rng.integers(1, 5, size=w.modes)
    amp = rng.uniform(0.0, w.amp_max, size=w.modes)
    th = rng.uniform(0.0, 2.0 * np.pi, size=w.modes)
    h = np.full(np.broadcast(x, y).shape, 0.5)
    for q in range(w.modes):
        h = h + amp[q] * np.cos(2.0 * np.pi * kx[q] * x / Lx + 2.0 * np.pi * ky[q] * y / Ly + th[q])
    return h


def make_case(w: Workload | str, *, nx: int | None = None, ny: int | None = None, nz: int | None = None,
              mom: int = 30, levelset: int = 10, p_rtol: float = 1e-5, p_maxits: int = 200,
              precision: int = 0, fp64_parts: int = 0, mg_fp32: int = 0, idm: str = "lsm",
              epn: float | None = None, pe: float = 1000.0, max_iteration_dim: int = 18,
              geometry: str = "cubic", profile=None, flags: int = 0):
    """Returns (params, u_inlet, state) for a workload, optionally resized.

    state maps TPLS field names (tpls_gb300.api.STATE_FIELDS subset) to
    Fortran-ordered arrays; fields not given start at zero.  `profile` is
    the base-state routine (the signature of api.base_profile; default: the
    library's host code)."""
    if isinstance(w, str):
        w = WORKLOADS[w]
    nx = nx or w.nx
    ny = ny or w.ny
    nz = nz or w.nz
    dz = 1.0 / nz
    if geometry == "cubic":
        dx = dy = dz
        Lx, Ly = nx * dx, ny * dy
    elif geometry == "box":
        Lx, Ly = 2.0 * np.pi, np.pi
        dx, dy = Lx / nx, Ly / ny
    else:
        raise ValueError(f"unknown geometry {geometry!r}")
    sw = 1.5 * dx
    mu_minus, mu_plus = w.m, 1.0
    uz = (profile or base_profile)(nz, dz, w.re, -1.0, mu_minus, mu_plus, 0.5, sw)
    umax = float(np.max(np.abs(uz)))
    # CFL 0.2 on the base flow, and half the capillary limit of the explicit
    # surface-tension term, sqrt(rho dx^3 / (2 pi sigma)) with rho = 1 and
    # sigma = scap = 1 (binding only for slow, low-Re instances)
    dt = min(0.2 * dx / umax, 0.5 * np.sqrt(dx ** 3 / (2.0 * np.pi)))
    params = Params(dx=dx, dy=dy, dz=dz, dt=dt, re=w.re, mu_plus=mu_plus, mu_minus=mu_minus, height=0.5,
                    scap=1.0, smooth_width=sw, mom_u=mom, mom_v=mom, mom_w=mom, levelset=levelset,
                    p_rtol=p_rtol, p_maxits=p_maxits, precision=precision, fp64_parts=fp64_parts,
                    mg_fp32=mg_fp32, idm=1 if idm == "dim" else 0, max_iteration_dim=max_iteration_dim,
                    epn=(1.5 * dz if epn is None else epn), pe=pe, flags=flags)
    xi = (np.arange(nx + 2) - 0.5) * dx
    yj = (np.arange(ny + 2) - 0.5) * dy
    zk = (np.arange(nz + 2) - 0.5) * dz
    h = interface_height(w, xi[:, None], yj[None, :], Lx, Ly)
    # the same phi = z - h for both interface methods, as the reference's
    # initial-condition program writes it (create_initial_conditions_program.F90)
    phi = np.asfortranarray(zk[None, None, :] - h[:, :, None])
    u = np.asfortranarray(np.broadcast_to(uz[None, None, :], (nx + 2, ny + 2, nz)).copy())
    v = np.zeros((nx + 2, ny + 2, nz), order="F")
    wv = np.zeros((nx + 2, ny + 2, nz + 1), order="F")
    off = 0
    n = (nx - 1) * ny * nz
    u[1:nx, 1:ny + 1, :] += uniform_pm(w.seed, n, 1e-3, off).reshape((nx - 1, ny, nz), order="F")
    off += n
    n = nx * ny * nz
    v[1:nx + 1, 1:ny + 1, :] += uniform_pm(w.seed, n, 1e-3, off).reshape((nx, ny, nz), order="F")
    off += n
    n = nx * ny * (nz - 1)
    wv[1:nx + 1, 1:ny + 1, 1:nz] += uniform_pm(w.seed, n, 1e-3, off).reshape((nx, ny, nz - 1), order="F")
    for a in (u, v, wv):  # periodic y rows
        a[:, 0, :] = a[:, ny, :]
        a[:, ny + 1, :] = a[:, 1, :]
    xp = np.arange(nx + 2) * dx - dx / 2.0
    pres = np.asfortranarray(np.broadcast_to(-xp[:, None, None], (nx + 2, ny + 2, nz + 2)).copy())
    state = {"PHI2": phi, "U2": u, "V2": v, "W2": wv, "PRES": pres,
             "PRES_OLD": np.zeros_like(pres, order="F")}
    if params.idm == 1:
        # the diffuse-interface iteration starts from phi3; the harness seeds it
        # with the initial phi (the reference's driver starts it at 0)
        state["PHI3"] = phi.copy(order="F")
        state["CONVPREV_PHI"] = np.zeros_like(phi, order="F")
    return params, np.ascontiguousarray(uz), state
