"""Generate the golden fixtures of the CPU oracle (tests/golden/oracle_*.npz).

The Fortran reference cannot be built on these machines and ships no golden
vectors for the per-timestep path, so these fixtures pin the oracle itself:
its output on seeded inputs for every routine of the path and for one whole
step, on a small even grid and a small odd one (odd ny takes the unfused
periodic-row paths).  tests/test_golden.py regenerates the outputs and
compares; the GPU parity tests compare the CUDA path with the same oracle.

Inputs are not stored: the seeded two-layer channel of tpls_gb300.channel
(workload A resized) stepped once by the oracle gives realistic fields with
non-zero histories, and the sweep inputs are drawn from numpy's PCG64 with
fixed seeds.  Regenerate only when the oracle's arithmetic is meant to
change, and say why in the commit:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

CASES = {"even": (12, 6, 8), "odd": (9, 5, 7)}
STEP_FIELDS = ("PHI2", "U2", "V2", "W2", "PRES")
STAT_KEYS = ("err_phi", "err_u", "err_v", "err_w", "liquid_volume")


def fixture_path(case: str) -> Path:
    return HERE / f"oracle_{case}.npz"


def _sweep_inputs(o, comp: int, seed: int):
    kind = "w" if comp == 2 else "uv"
    rng = np.random.default_rng(seed)
    x = np.asfortranarray(rng.normal(size=o.shape(kind)))
    xo = np.asfortranarray(rng.normal(size=o.shape(kind)))
    rhs = np.asfortranarray(rng.normal(size=o.shape(kind)))
    o.exchange2d(x)
    o.exchange2d(xo)
    return x, xo, rhs


def compute(case: str) -> dict:
    """Every recorded output of the oracle for one case, by name."""
    from oracle.oracle import Oracle
    from tpls_gb300.channel import make_case
    nx, ny, nz = CASES[case]
    p, uin, st = make_case("A", nx=nx, ny=ny, nz=nz)
    o = Oracle(nx, ny, nz, p, uin)
    o.set_state(st)
    o.step(1)  # realistic fields and non-zero AB3 histories
    s = o.get_state()
    out: dict = {}
    out["advect.conv2_phi"] = o.do_advect_phi(*(np.array(s[k], order="F") for k in ("PHI2", "U2", "V2", "W2")),
                                              p.dx, p.dy, p.dz)
    phi3, err = o.do_tpls(s["PHI2"], s["CONV0_PHI"], s["CONV1_PHI"], o.get_field("CONV2_PHI"), p.levelset,
                          p.height, p.dx, p.dz, p.dt)[:2]
    out["do_tpls.phi3"] = phi3
    out["do_tpls.err"] = np.array(err)
    D, ist, sgn = o.get_levelset_status(s["PHI2"], p.dx)
    out["status.D"], out["status.istatus"], out["status.sign"] = D, ist, sgn
    ri, rerr = o.do_levelset_iteration(s["PHI2"], np.array(s["PHI2"], order="F"), D, ist, sgn, p.dx, p.height)
    out["ls_iteration.phi"], out["ls_iteration.err"] = ri, np.array(rerr)
    for name, a in zip(("fx", "fy", "fz"), o.get_csf(s["PHI2"], p.dx, p.dy, p.dz, p.scap, p.smooth_width)):
        out["csf." + name] = a
    va = o.get_viscosity(s["PHI2"], p.smooth_width, p.re, p.mu_minus, p.mu_plus)
    out["viscosity.aug"] = va
    for which, f in (("conv", o.get_conv_all), ("diff", o.get_diffusion_all)):
        for comp, a in zip("uvw", f(va, s["U2"], s["V2"], s["W2"], p.dx, p.dy, p.dz)):
            out[f"{which}.{comp}"] = a
    for comp in range(3):
        x, xo, rhs = _sweep_inputs(o, comp, 10 + comp)
        [o.do_jacobi_u, o.do_jacobi_v, o.do_jacobi_w][comp](x, xo, rhs, va, p.dx, p.dy, p.dz, p.dt)
        out[f"jacobi.{comp}"] = x
        for flg in (0, 1):
            for it in (1, 2):
                x, _, rhs = _sweep_inputs(o, comp, 20 + comp)
                [o.do_sor_u, o.do_sor_v, o.do_sor_w][comp](x, rhs, va, p.dx, p.dy, p.dz, p.dt, flg, it)
                out[f"sor.{comp}.{flg}.{it}"] = x
    u3, v3, w3 = (o.get_field(k) for k in ("U3", "V3", "W3"))
    out["source.rhs_p"] = o.get_source_pres(u3, v3, w3, p.dx, p.dy, p.dz, p.dt)
    pres = o.pressure_solve(o.get_field("PRES_OLD"), o.get_field("RHS_P"), u3, uin, p.dx, p.dy, p.dz, p.dt)[0]
    out["pressure.pres"] = pres
    uo, vo, wo = (np.array(a, order="F") for a in (u3, v3, w3))
    o.get_uvw_pres(uo, vo, wo, pres, p.dx, p.dy, p.dz, p.dt, uin)
    out["project.u"], out["project.v"], out["project.w"] = uo, vo, wo
    o.set_state(s)
    o.step(1)
    for k in STEP_FIELDS:
        out["step." + k] = o.get_field(k)
    st2 = o.stats()
    out["step.stats"] = np.array([st2[k] for k in STAT_KEYS])
    return out


def main() -> None:
    from oracle.oracle import set_threads
    set_threads(1)
    for case in CASES:
        out = compute(case)
        np.savez_compressed(fixture_path(case), **out)
        print(f"{fixture_path(case).name}: {len(out)} arrays, {fixture_path(case).stat().st_size} bytes")


if __name__ == "__main__":
    main()
