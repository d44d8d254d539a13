"""Known-answer tests that pin the CPU oracle to the mathematics of the
reference routines (the reference ships no golden vectors for this path).
CPU only."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle.oracle import Oracle, weno5
from tpls_gb300.api import Params
from tpls_gb300.channel import make_case

from _util import relmax


def _params(nx, ny, nz, dx=None, dy=None, dz=None, **kw):
    dx = dx or 2 * np.pi / nx
    dy = dy or np.pi / ny
    dz = dz or 1.0 / nz
    base = dict(dx=dx, dy=dy, dz=dz, dt=1e-3, re=100.0, mu_plus=1.0, mu_minus=2.0, height=0.5, scap=1.0,
                smooth_width=1.5 * dx)
    base.update(kw)
    return Params(**base)


# --- weno.f90:175-215 -------------------------------------------------------
def test_weno5_exact_for_quadratic_cell_averages():
    rng = np.random.default_rng(1)
    for _ in range(50):
        a, b, c = rng.normal(size=3)
        x = np.arange(-2, 3, dtype=float)
        avg = a + b * x + c * (x * x + 1.0 / 12.0)  # cell averages of a+bx+cx^2
        face = a + b * 0.5 + c * 0.25               # point value at x = 1/2
        assert abs(weno5(*avg) - face) <= 1e-12 * (1 + abs(face))
        # mirrored stencil (upwind from the right) gives the same face value
        assert abs(weno5(*avg[::-1][:5]) - (a - b * 0.5 + c * 0.25)) <= 1e-12 * (1 + abs(face))


def test_weno5_fifth_order_on_smooth_data():
    errs = []
    for h in (0.2, 0.1, 0.05):
        x = np.arange(-2, 3) * h + 0.3
        avg = (np.cos(x - h / 2) - np.cos(x + h / 2)) / h  # cell averages of sin
        errs.append(abs(weno5(*avg) - np.sin(0.3 + h / 2)))
    assert errs[0] / errs[1] > 20 and errs[1] / errs[2] > 20


# --- advect_phi.f90 ---------------------------------------------------------
def test_advect_constant_phi_divergence_free_velocity_gives_zero():
    nx, ny, nz = 12, 8, 10
    p = _params(nx, ny, nz)
    o = Oracle(nx, ny, nz, p, np.ones(nz))
    phi = np.full(o.shape("p"), 0.3, order="F")
    u = np.full(o.shape("uv"), 1.0, order="F")
    v = np.full(o.shape("uv"), 0.5, order="F")
    w = np.zeros(o.shape("w"), order="F")
    conv = o.do_advect_phi(phi, u, v, w, p.dx, p.dy, p.dz)
    assert np.max(np.abs(conv)) < 1e-12
    assert np.all(conv[0, :, :] == 0) and np.all(conv[:, :, 0] == 0)  # zero outside the interior


def test_advect_linear_phi_uniform_u_gives_u_dphidx():
    # phi = x, u = 1: WENO5 is exact for linear data, so conv = d(u phi)/dx = 1
    nx, ny, nz = 12, 8, 10
    p = _params(nx, ny, nz)
    o = Oracle(nx, ny, nz, p, np.ones(nz))
    x = (np.arange(nx + 2) - 0.5) * p.dx
    phi = np.asfortranarray(np.broadcast_to(x[:, None, None], o.shape("p")).copy())
    u = np.full(o.shape("uv"), 1.0, order="F")
    v = np.zeros(o.shape("uv"), order="F")
    w = np.zeros(o.shape("w"), order="F")
    conv = o.do_advect_phi(phi, u, v, w, p.dx, p.dy, p.dz)
    c = conv[:, 1:ny + 1, 1:nz + 1]
    # WENO faces (3 <= i <= nx-2) are exact for linear data; faces 0..2 and
    # nx-1..nx are first-order upwind (weno.f90:45-76), so the cells where
    # the two kinds meet see x_{3+1/2} - x_2 and x_{nx-1} - x_{nx-3/2}.
    exact = [i for i in range(1, nx + 1) if i not in (3, nx - 1)]
    np.testing.assert_allclose(c[exact], 1.0, rtol=1e-12)
    np.testing.assert_allclose(c[3], 1.5, rtol=1e-12)
    np.testing.assert_allclose(c[nx - 1], 0.5, rtol=1e-12)


# --- levelset.f90 / two_phase_levelset.f90 ------------------------------------
def test_redistancing_keeps_planar_signed_distance():
    # with h = dx = dz the signed distance z - height is a fixed point
    nx, ny, nz = 10, 6, 12
    h = 1.0 / nz
    p = _params(nx, ny, nz, dx=h, dz=h)
    o = Oracle(nx, ny, nz, p, np.ones(nz))
    k = np.arange(nz + 2)
    z = k * h - 0.5 * h
    phi = np.asfortranarray(np.broadcast_to((z - 0.5)[None, None, :], o.shape("p")).copy())
    zero = o.zeros("p")
    phi3, err = o.do_tpls(phi, zero, zero, zero, 10, 0.5, h, h, 1e-3)
    r = (slice(0, nx + 2), slice(1, ny + 1), slice(0, nz + 2))
    assert relmax(phi3, phi, r) < 1e-13
    assert err < 1e-26


def test_levelset_status_marks_interface_cells():
    nx, ny, nz = 8, 6, 10
    h = 1.0 / nz
    p = _params(nx, ny, nz, dx=h, dz=h)
    o = Oracle(nx, ny, nz, p, np.ones(nz))
    z = np.arange(nz + 2) * h - 0.5 * h
    phi = np.asfortranarray(np.broadcast_to((z - 0.52)[None, None, :], o.shape("p")).copy())
    D, ist, sgn = o.get_levelset_status(phi, h)
    kint = np.where(ist[3, 3, :] == 1)[0]
    assert list(kint) == [5, 6]  # the two cells straddling z = 0.52
    np.testing.assert_allclose(D[3, 3, kint], phi[3, 3, kint], rtol=1e-12)
    assert sgn[3, 3, 1] == -1 and sgn[3, 3, nz] == 1 and sgn[0, 3, 3] == 0


def test_csf_zero_for_flat_interface():
    nx, ny, nz = 8, 6, 10
    p = _params(nx, ny, nz)
    o = Oracle(nx, ny, nz, p, np.ones(nz))
    z = (np.arange(nz + 2) - 0.5) * p.dz
    phi = np.asfortranarray(np.broadcast_to((z - 0.5)[None, None, :], o.shape("p")).copy())
    fx, fy, fz = o.get_csf(phi, p.dx, p.dy, p.dz, 1.0, p.smooth_width)
    for f in (fx, fy, fz):
        assert np.max(np.abs(f[:, 1:ny + 1, :])) < 1e-9


# --- momentum_allflux.f90:474 ----------------------------------------------------
def test_heaviside_viscosity_limits_and_symmetry():
    nx, ny, nz = 6, 4, 6
    p = _params(nx, ny, nz)
    o = Oracle(nx, ny, nz, p, np.ones(nz))
    sw = p.smooth_width
    vals = np.linspace(-2 * sw, 2 * sw, (nx + 2) * (ny + 2) * (nz + 2))
    phi = np.asfortranarray(vals.reshape(o.shape("p"), order="F"))
    va = o.get_viscosity(phi, sw, p.re, p.mu_minus, p.mu_plus)
    mu = va[1:nx + 3, 2:ny + 2, :]  # x 0..nx+1, rows 1..ny
    ph = phi[:, 1:ny + 1, :]
    assert np.all(mu[ph < -sw] == p.mu_minus / p.re)
    assert np.all(mu[ph > sw] == p.mu_plus / p.re)
    Hm = (p.mu_minus / p.re - mu) / ((p.mu_minus - p.mu_plus) / p.re)  # = H(phi)
    phi_m = -phi
    va2 = o.get_viscosity(np.asfortranarray(phi_m), sw, p.re, p.mu_minus, p.mu_plus)
    Hm2 = (p.mu_minus / p.re - va2[1:nx + 3, 2:ny + 2, :]) / ((p.mu_minus - p.mu_plus) / p.re)
    np.testing.assert_allclose(Hm + Hm2, 1.0, atol=1e-13)
    # periodic augmentation rows -1, 0 and ny+1, ny+2
    np.testing.assert_array_equal(va[1:nx + 3, 0, :], va[1:nx + 3, ny, :])
    np.testing.assert_array_equal(va[1:nx + 3, ny + 3, :], va[1:nx + 3, 3, :])


# --- jacobi / sor ---------------------------------------------------------------
@pytest.mark.parametrize("comp", [0, 1, 2])
def test_sweeps_converge_to_the_helmholtz_solution(comp):
    """Many outer iterations of Jacobi + red-black SOR reach a fixed point of
    the Jacobi operator (the Crank-Nicolson Helmholtz solution)."""
    nx, ny, nz = 10, 6, 8
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz)
    o = Oracle(nx, ny, nz, params, uin)
    va = o.get_viscosity(st["PHI2"], params.smooth_width, params.re, params.mu_minus, params.mu_plus)
    kind = "w" if comp == 2 else "uv"
    rng = np.random.default_rng(7)
    rhs = np.asfortranarray(rng.normal(size=o.shape(kind)))
    dt = params.dt * 50  # stiffer system than the workload's
    x3, xo, err = o.momentum(comp, rhs, va, st["PRES"], 600, params.dx, params.dy, params.dz, dt)
    assert err < 1e-24
    j = np.array(x3, order="F")
    xin = np.array(x3, order="F")
    o.exchange2d(xin)
    [o.do_jacobi_u, o.do_jacobi_v, o.do_jacobi_w][comp](j, xin, rhs, va, params.dx, params.dy, params.dz, dt)
    iend = nx - 1 if comp == 0 else nx
    k0 = 1 if comp == 2 else 0
    r = (slice(1, iend + 1), slice(1, ny + 1), slice(k0, (nz - 1 if comp == 2 else nz - 1) + 1))
    assert relmax(j, x3, r) < 1e-12


def test_sor_odd_sweep_is_column_sequential():
    """For odd iteration_time the colouring is mod(j+flg,2) in every plane:
    relaxing a column upward must equal the plane-by-plane reference order."""
    nx, ny, nz = 8, 5, 7
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz)
    o = Oracle(nx, ny, nz, params, uin)
    va = o.get_viscosity(st["PHI2"], params.smooth_width, params.re, params.mu_minus, params.mu_plus)
    rng = np.random.default_rng(3)
    x = np.asfortranarray(rng.normal(size=o.shape("uv")))
    rhs = np.asfortranarray(rng.normal(size=o.shape("uv")))
    ref = np.array(x, order="F")
    o.do_sor_v(ref, rhs, va, params.dx, params.dy, params.dz, params.dt, 1, 3)
    # restatement with an explicit column march
    mine = np.array(x, order="F")
    ax, ay, az = (params.dt / d ** 2 for d in (params.dx, params.dy, params.dz))
    V = va[1:, 1:, :]  # index viscosity_aug from 0 like the p-grid
    for i0 in range(1, nx + 1):
        for jj in range(1, ny + 1):
            if (i0 - 1) % 2 != (jj + 1) % 2:
                continue
            for k in range(nz):
                c = mine
                mpx = (V[i0, jj + 1, k + 1] + V[i0, jj, k + 1] + V[i0 + 1, jj + 1, k + 1] + V[i0 + 1, jj, k + 1]) / 4
                mmx = (V[i0, jj + 1, k + 1] + V[i0, jj, k + 1] + V[i0 - 1, jj + 1, k + 1] + V[i0 - 1, jj, k + 1]) / 4
                mpy, mmy = V[i0, jj + 1, k + 1], V[i0, jj, k + 1]
                mpz = (V[i0, jj + 1, k + 1] + V[i0, jj, k + 1] + V[i0, jj + 1, k + 2] + V[i0, jj, k + 2]) / 4
                mmz = (V[i0, jj + 1, k + 1] + V[i0, jj, k + 1] + V[i0, jj + 1, k] + V[i0, jj, k]) / 4
                zm = -2 * c[i0, jj, 0] + c[i0, jj, 1] / 3 if k == 0 else c[i0, jj, k - 1]
                zp = -2 * c[i0, jj, nz - 1] + c[i0, jj, nz - 2] / 3 if k == nz - 1 else c[i0, jj, k + 1]
                diag = 1 + ax / 2 * (mpx + mmx) + ay / 2 * (mpy + mmy) + az / 2 * (mpz + mmz)
                res = (1 / diag) * (ax / 2 * (mpx * c[i0 + 1, jj, k] + mmx * c[i0 - 1, jj, k])
                                    + ay / 2 * (mpy * c[i0, jj + 1, k] + mmy * c[i0, jj - 1, k])
                                    + az / 2 * (mpz * zp + mmz * zm) + rhs[i0, jj, k])
                c[i0, jj, k] = c[i0, jj, k] + 1.2 * (res - c[i0, jj, k])
    assert relmax(mine, ref) < 1e-13


# --- pressure_solver.F90 -------------------------------------------------------------
def _reduced_apply(p, cx, cy, cz):
    """symmetric interior operator with Neumann x/z and periodic y"""
    pe = np.pad(p, ((1, 1), (0, 0), (1, 1)), mode="edge")
    lap = (cx * (2 * p - pe[:-2, :, 1:-1] - pe[2:, :, 1:-1]) +
           cy * (2 * p - np.roll(p, 1, axis=1) - np.roll(p, -1, axis=1)) +
           cz * (2 * p - pe[1:-1, :, :-2] - pe[1:-1, :, 2:]))
    return lap


def _petsc_system(nx, ny, nz, dx, dy, dz, dt, rhs_p, u3, u_inlet):
    """pressure_solver.F90:234-441 restated with scipy: the matrix and RHS
    PETSc is handed, in PETSc's (i=y, j=x, k=z) numbering."""
    gx, gy, gz = ny, nx, nz  # global_dim_x/y/z
    nI, nJ, nK = gx, gy + 2, gz + 2

    def idx(i, j, k):
        return i + nI * (j + nJ * k)

    rows, cols, vals = [], [], []
    b = np.zeros(nI * nJ * nK)
    for k in range(nK):
        for j in range(nJ):
            for i in range(nI):
                r = idx(i, j, k)
                if (j == 0 and k == 0) or (j == gy + 1 and k == 0):
                    ent = [(idx(i, j, k), 1 / dz), (idx(i, j, k + 1), -1 / dz)]
                elif (j == 0 and k == gz + 1) or (j == gy + 1 and k == gz + 1):
                    ent = [(idx(i, j, k), -1 / dz), (idx(i, j, k - 1), 1 / dz)]
                elif j == 0:
                    ent = [(idx(i, j, k), 1 / dy), (idx(i, j + 1, k), -1 / dy)]
                elif j == gy + 1:
                    ent = [(idx(i, j, k), -1 / dy), (idx(i, j - 1, k), 1 / dy)]
                elif k == 0:
                    ent = [(idx(i, j, k), 1 / dz), (idx(i, j, k + 1), -1 / dz)]
                elif k == gz + 1:
                    ent = [(idx(i, j, k), -1 / dz), (idx(i, j, k - 1), 1 / dz)]
                else:
                    ent = [(idx(i, j, k - 1), -1 / dz ** 2), (idx((i - 1) % nI, j, k), -1 / dx ** 2),
                           (idx(i, j - 1, k), -1 / dy ** 2), (idx(i, j, k), 2 * (1 / dx ** 2 + 1 / dy ** 2 + 1 / dz ** 2)),
                           (idx(i, j + 1, k), -1 / dy ** 2), (idx((i + 1) % nI, j, k), -1 / dx ** 2),
                           (idx(i, j, k + 1), -1 / dz ** 2)]
                for cidx, v in ent:
                    rows.append(r)
                    cols.append(cidx)
                    vals.append(v)
                b[r] = -rhs_p[j, i + 1, k]
                if j == 0 and 1 <= k <= gz:
                    b[r] = (dx / dt) * (u_inlet[k - 1] - u3[0, i, k - 1]) / dy
    A = sp.csr_matrix((vals, (rows, cols)), shape=(b.size, b.size))
    return A, b, idx


def test_pressure_oracle_solves_the_petsc_system():
    nx, ny, nz = 10, 6, 8
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz)
    o = Oracle(nx, ny, nz, params, uin)
    rng = np.random.default_rng(11)
    rhs_p = o.zeros("p")
    rhs_p[1:nx + 1, 1:ny + 1, 1:nz + 1] = rng.normal(size=(nx, ny, nz))
    o.exchange2d(rhs_p)
    u3 = np.asfortranarray(rng.normal(size=o.shape("uv")))
    pres_old = np.asfortranarray(rng.normal(size=o.shape("p")))
    p, _, rnorm, _ = o.pressure_solve(pres_old, rhs_p, u3, uin, params.dx, params.dy, params.dz, params.dt)
    A, b, idx = _petsc_system(nx, ny, nz, params.dx, params.dy, params.dz, params.dt, rhs_p, u3, uin)
    x = np.zeros(b.size)
    for k in range(nz + 2):
        for j in range(nx + 2):
            for i in range(ny):
                x[idx(i, j, k)] = p[j, i + 1, k]
    r = A @ x - b
    interior = np.zeros(b.size, bool)
    for k in range(1, nz + 1):
        for j in range(1, nx + 1):
            for i in range(ny):
                interior[idx(i, j, k)] = True
    scale = np.max(np.abs(b))
    # ghost rows satisfied exactly; interior rows off by one constant (the
    # compatibility projection of the singular system)
    assert np.max(np.abs(r[~interior])) < 1e-10 * scale
    ri = r[interior]
    assert np.max(np.abs(ri - ri.mean())) < 1e-9 * scale
    # constant fixed by the initial guess's interior mean
    assert abs(p[1:nx + 1, 1:ny + 1, 1:nz + 1].mean() - pres_old[1:nx + 1, 1:ny + 1, 1:nz + 1].mean()) < 1e-12
    # periodic y rows
    np.testing.assert_array_equal(p[:, 0, :], p[:, ny, :])


def test_pressure_oracle_manufactured_solution():
    nx, ny, nz = 12, 8, 10
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz)
    o = Oracle(nx, ny, nz, params, uin)
    rng = np.random.default_rng(5)
    pt = rng.normal(size=(nx, ny, nz))
    pt -= pt.mean()
    cx, cy, cz = 1 / params.dy ** 2, 1 / params.dx ** 2, 1 / params.dz ** 2
    b = _reduced_apply(pt, cx, cy, cz)
    rhs_p = o.zeros("p")
    rhs_p[1:nx + 1, 1:ny + 1, 1:nz + 1] = -b
    u3 = o.zeros("uv")
    u3[0, :, :] = uin[None, :]  # no inlet flux
    p, _, _, _ = o.pressure_solve(o.zeros("p"), rhs_p, u3, uin, params.dx, params.dy, params.dz, params.dt)
    assert relmax(p[1:nx + 1, 1:ny + 1, 1:nz + 1], pt) < 1e-11


def test_projection_makes_divergence_uniform():
    """After the solve and get_uvw_pres, get_source_pres is one constant on
    every interior cell (the compatibility residual of the singular system).
    Needs dx == dy: compute_matrix puts 1/dy^2 on the physical-x neighbours
    and 1/dx^2 on the physical-y ones (pressure_solver.F90:394-421)."""
    nx, ny, nz = 16, 8, 10
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz)
    o = Oracle(nx, ny, nz, params, uin)
    rng = np.random.default_rng(9)
    u3 = np.asfortranarray(st["U2"] + 1e-2 * rng.normal(size=o.shape("uv")))
    v3 = np.asfortranarray(1e-2 * rng.normal(size=o.shape("uv")))
    w3 = np.asfortranarray(1e-2 * rng.normal(size=o.shape("w")))
    w3[:, :, 0] = 0
    w3[:, :, nz] = 0
    u3[0, :, :] = u3[1, :, :]
    for a in (u3, v3, w3):
        o.exchange2d(a)
    d = params
    rhs = o.get_source_pres(u3, v3, w3, d.dx, d.dy, d.dz, d.dt)
    p, _, _, _ = o.pressure_solve(o.zeros("p"), rhs, u3, uin, d.dx, d.dy, d.dz, d.dt)
    o.get_uvw_pres(u3, v3, w3, p, d.dx, d.dy, d.dz, d.dt, uin)
    for a in (u3, v3, w3):
        o.exchange2d(a)
    div = o.get_source_pres(u3, v3, w3, d.dx, d.dy, d.dz, d.dt)[1:nx + 1, 1:ny + 1, 1:nz + 1]
    assert np.max(np.abs(div - div.mean())) < 1e-9 * np.max(np.abs(rhs))


def test_oracle_step_is_deterministic_and_finite():
    params, uin, st = make_case("A", nx=16, ny=8, nz=12)
    outs = []
    for _ in range(2):
        o = Oracle(16, 8, 12, params, uin)
        o.set_state(st)
        o.step(2)
        outs.append(o.get_state())
    for k in outs[0]:
        assert np.all(np.isfinite(outs[0][k])), k
        np.testing.assert_array_equal(outs[0][k], outs[1][k])


def _dim_oracle(nx=24, ny=10, nz=14):
    params, uin, _ = make_case("A", nx=nx, ny=ny, nz=nz, idm="dim")
    return params, Oracle(nx, ny, nz, params, uin)


def test_dim_keeps_a_uniform_concentration_away_from_the_inlet():
    """cahn_hilliard_solver.f90 dim on a uniform C with no advection and no
    history: the bulk and Laplacian terms vanish, so C stays exactly c0
    except where the inlet profile has reached; each SOR iteration widens
    that reach by two cells (grad^2 of grad^2)."""
    p, o = _dim_oracle()
    nx, ny, nz = o.nx, o.ny, o.nz
    c0 = 0.3
    C = np.full((nx + 2, ny + 2, nz + 2), c0, order="F")
    zero = np.zeros_like(C, order="F")
    its = 3
    new, cprev = o.dim(C, C, zero, zero, C, its, p.epn, p.pe, p.height, p.dx, p.dy, p.dz, p.dt)
    far = new[2 * its + 2:nx + 1, 1:ny + 1, 1:nz + 1]
    assert np.array_equal(far, np.full_like(far, c0))
    assert np.all(cprev[1:nx + 1, 1:ny + 1, 1:nz + 1] == 0.0)
    # the inlet column carries the reference's tanh profile
    z = (np.arange(1, nz + 1) - 0.5) * p.dz
    prof = 0.5 + 0.5 * np.tanh((z - p.height) / (2.0 * np.sqrt(2.0) * p.epn))
    assert np.allclose(new[0, 1:ny + 1, 1:nz + 1], prof[None, :], rtol=0, atol=1e-15)


def test_dim_clamps_to_the_unit_interval_and_steps_stay_finite():
    """The update clamps C^{n+1} to [0, 1] (cahn_hilliard_solver.f90:311-312);
    whole diffuse-interface steps of the oracle stay finite with phi = C - 0.5
    inside [-0.5, 0.5] on the interior."""
    p, o = _dim_oracle()
    nx, ny, nz = o.nx, o.ny, o.nz
    rng = np.random.default_rng(3)
    C = np.asfortranarray(rng.uniform(-0.2, 1.2, size=(nx + 2, ny + 2, nz + 2)))
    zero = np.zeros_like(C, order="F")
    new, _ = o.dim(C, C, zero, zero, C, 2, p.epn, p.pe, p.height, p.dx, p.dy, p.dz, p.dt)
    inner = new[1:nx + 1, 1:ny + 1, 1:nz + 1]
    assert inner.min() >= 0.0 and inner.max() <= 1.0
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz, idm="dim")
    o2 = Oracle(nx, ny, nz, params, uin)
    o2.set_state(st)
    o2.step(3)
    phi = o2.get_field("PHI2")
    assert np.isfinite(phi).all()
    inter = phi[1:nx + 1, 1:ny + 1, 1:nz + 1]
    assert inter.min() >= -0.5 and inter.max() <= 0.5
    assert np.isfinite(o2.get_field("U2")).all()
