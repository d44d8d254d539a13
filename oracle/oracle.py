"""Python binding of the CPU oracle (oracle/tpls_oracle.c).

TEST INFRASTRUCTURE ONLY -- the parity oracle and the CPU baseline.  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it; the
product package never imports it.  PARITY UNPINNED: the Fortran reference
cannot be built on these machines and ships no golden vectors for this path;
the oracle is pinned by the mathematical known-answer tests in
tests/test_oracle_kats.py and by the committed golden fixtures it produced
(tests/golden/).

Methods mirror tpls_gb300.api.TplsGpu (same names, arguments and layouts),
so parity tests call both the same way.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_ROOT = Path(__file__).resolve().parent
ORACLE_LIB = _ROOT / "_build" / "liboracle.so"
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_lib = None


def load():
    global _lib
    if _lib is None:
        if not ORACLE_LIB.exists():
            raise RuntimeError(f"oracle library {ORACLE_LIB} not built (tpls_gb300.build.build_oracle())")
        _lib = C.CDLL(str(ORACLE_LIB))
        _lib.orc_weno5.restype = C.c_double
        _lib.orc_weno5.argtypes = [C.c_double] * 5
        _lib.orc_create.restype = C.c_void_p
        _lib.orc_destroy.argtypes = [C.c_void_p]
        _lib.orc_set_field.argtypes = [C.c_void_p, C.c_int, _DP]
        _lib.orc_get_field.argtypes = [C.c_void_p, C.c_int, _DP]
        _lib.orc_step.argtypes = [C.c_void_p, C.c_int]
        _lib.orc_get_stats.argtypes = [C.c_void_p, C.c_void_p]
    return _lib


def set_threads(n: int) -> None:
    """OpenMP threads of the oracle (results do not depend on it, except the
    summation order of the logged residuals)."""
    os.environ["OMP_NUM_THREADS"] = str(n)
    try:
        gomp = C.CDLL("libgomp.so.1")
        gomp.omp_set_num_threads(int(n))
    except OSError:
        pass


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.f_contiguous
    return a.ctypes.data_as(_DP)


def weno5(v1, v2, v3, v4, v5) -> float:
    return load().orc_weno5(v1, v2, v3, v4, v5)


def base_profile(nz, dz, re, dpdl, mu_minus, mu_plus, height, smooth_width) -> np.ndarray:
    """twophase_initialisation_wave.F90:79-122 base velocity u(z) (nz values);
    same arguments as tpls_gb300.api.base_profile."""
    lib = load()
    out = np.zeros(int(nz))
    lib.orc_base_profile(int(nz), C.c_double(dz), C.c_double(re), C.c_double(dpdl), C.c_double(mu_minus),
                         C.c_double(mu_plus), C.c_double(height), C.c_double(smooth_width),
                         out.ctypes.data_as(_DP))
    return out


class Oracle:
    """CPU restatement of one channel (single MPI rank semantics)."""

    def __init__(self, nx, ny, nz, params, u_inlet):
        from tpls_gb300.api import TplsParams  # struct layout shared with the C ABI
        self.lib = load()
        self.nx, self.ny, self.nz = nx, ny, nz
        self.params = params
        self._cp = params.to_c()
        self.u_inlet = np.ascontiguousarray(u_inlet, dtype=np.float64)
        self.ctx = self.lib.orc_create(nx, ny, nz, C.byref(self._cp), self.u_inlet.ctypes.data_as(_DP))
        if not self.ctx:
            raise ValueError("oracle: unsupported grid size")
        self._TplsParams = TplsParams

    def close(self):
        if self.ctx:
            self.lib.orc_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self, kind):
        from tpls_gb300.api import shape_of
        return shape_of(kind, self.nx, self.ny, self.nz)

    def zeros(self, kind):
        return np.zeros(self.shape(kind), order="F")

    # -- whole-step driver ------------------------------------------------
    def set_field(self, name, a):
        from tpls_gb300.api import F, FIELD_KIND
        a = np.asfortranarray(a, dtype=np.float64)
        assert a.shape == self.shape(FIELD_KIND[name])
        self.lib.orc_set_field(self.ctx, F[name], _p(a))

    def get_field(self, name):
        from tpls_gb300.api import F, FIELD_KIND
        out = self.zeros(FIELD_KIND[name])
        self.lib.orc_get_field(self.ctx, F[name], _p(out))
        return out

    def set_state(self, state):
        for k, v in state.items():
            self.set_field(k, v)

    def get_state(self):
        from tpls_gb300.api import DIM_STATE_FIELDS, IDM_DIM, STATE_FIELDS
        names = STATE_FIELDS + (DIM_STATE_FIELDS if self.params.idm == IDM_DIM else [])
        return {k: self.get_field(k) for k in names}

    def step(self, nsteps=1):
        self.lib.orc_step(self.ctx, int(nsteps))
        return 0

    def stats(self):
        from tpls_gb300.api import TplsStats
        st = TplsStats()
        self.lib.orc_get_stats(self.ctx, C.byref(st))
        return st.as_dict()

    # -- single routines ----------------------------------------------------
    def do_advect_phi(self, phi2, u2, v2, w2, dx, dy, dz):
        conv = self.zeros("p")
        self.lib.orc_do_advect_phi(self.nx, self.ny, self.nz, _p(phi2), _p(u2), _p(v2), _p(w2), _p(conv),
                                   C.c_double(dx), C.c_double(dy), C.c_double(dz))
        return conv

    def dim(self, phi, phi_old, conv2_phi, conv_prev_phi, phi_new, max_iteration_dim, epn, pe, height, dx,
            dy, dz, dt):
        """cahn_hilliard_solver.f90:41 dim -> (phi_new, conv_prev_phi) (copies)."""
        phi_new = np.array(phi_new, order="F", copy=True)
        conv_prev_phi = np.array(conv_prev_phi, order="F", copy=True)
        self.lib.orc_dim(self.nx, self.ny, self.nz, C.c_double(dx), C.c_double(dy), C.c_double(dz),
                         C.c_double(dt), C.c_double(epn), C.c_double(pe), _p(phi), _p(phi_old), _p(conv2_phi),
                         _p(conv_prev_phi), _p(phi_new), C.c_double(height), int(max_iteration_dim))
        return phi_new, conv_prev_phi

    def do_tpls(self, phi2, conv0_phi, conv1_phi, conv2_phi, max_iteration_levelset, height, dx, dz, dt,
                phi3=None):
        phi3 = self.zeros("p") if phi3 is None else phi3
        err = C.c_double(0.0)
        self.lib.orc_do_tpls(self.nx, self.ny, self.nz, _p(phi2), _p(phi3), _p(conv0_phi), _p(conv1_phi),
                             _p(conv2_phi), int(max_iteration_levelset), C.c_double(height), C.c_double(dx),
                             C.c_double(dz), C.c_double(dt), C.byref(err))
        return phi3, err.value

    def get_levelset_status(self, phi, h):
        D, sgn = self.zeros("p"), self.zeros("p")
        ist = np.zeros(self.shape("p"), dtype=np.int32, order="F")
        self.lib.orc_get_levelset_status(self.nx, self.ny, self.nz, _p(phi), _p(D),
                                         ist.ctypes.data_as(_IP), _p(sgn), C.c_double(h))
        return D, ist, sgn

    def do_levelset_iteration(self, phi, phi_reinit, D, istatus, sgn, h, height):
        err = C.c_double(0.0)
        self.lib.orc_do_levelset_iteration(self.nx, self.ny, self.nz, _p(phi), _p(phi_reinit), _p(D),
                                           istatus.ctypes.data_as(_IP), _p(sgn), C.c_double(h),
                                           C.c_double(height), C.byref(err))
        return phi_reinit, err.value

    def get_csf(self, fi, dx, dy, dz, scap, smooth_width, fx=None, fy=None, fz=None):
        fx = self.zeros("p") if fx is None else fx
        fy = self.zeros("p") if fy is None else fy
        fz = self.zeros("p") if fz is None else fz
        self.lib.orc_get_csf(self.nx, self.ny, self.nz, _p(fx), _p(fy), _p(fz), _p(fi), C.c_double(dx),
                             C.c_double(dy), C.c_double(dz), C.c_double(scap), C.c_double(smooth_width))
        return fx, fy, fz

    def csf_faces(self, fx, fy, fz, csf_u=None, csf_v=None, csf_w=None):
        csf_u = self.zeros("uv") if csf_u is None else csf_u
        csf_v = self.zeros("uv") if csf_v is None else csf_v
        csf_w = self.zeros("w") if csf_w is None else csf_w
        self.lib.orc_csf_faces(self.nx, self.ny, self.nz, _p(fx), _p(fy), _p(fz), _p(csf_u), _p(csf_v), _p(csf_w))
        return csf_u, csf_v, csf_w

    def get_viscosity(self, phi, smooth_width, re, mu_minus, mu_plus, viscosity_aug=None):
        va = np.full(self.shape("va"), np.nan, order="F") if viscosity_aug is None else viscosity_aug
        self.lib.orc_viscosity_aug(self.nx, self.ny, self.nz, _p(phi), _p(va), C.c_double(smooth_width),
                                   C.c_double(re), C.c_double(mu_minus), C.c_double(mu_plus))
        return va

    def get_conv_all(self, viscosity_aug, u2, v2, w2, dx, dy, dz):
        ou, ov, ow = self.zeros("uv"), self.zeros("uv"), self.zeros("w")
        self.lib.orc_get_conv_all(self.nx, self.ny, self.nz, _p(ou), _p(ov), _p(ow), _p(viscosity_aug), _p(u2),
                                  _p(v2), _p(w2), C.c_double(dx), C.c_double(dy), C.c_double(dz))
        return ou, ov, ow

    def get_diffusion_all(self, viscosity_aug, u2, v2, w2, dx, dy, dz):
        ou, ov, ow = self.zeros("uv"), self.zeros("uv"), self.zeros("w")
        self.lib.orc_get_diffusion_all(self.nx, self.ny, self.nz, _p(ou), _p(ov), _p(ow), _p(viscosity_aug),
                                       _p(u2), _p(v2), _p(w2), C.c_double(dx), C.c_double(dy), C.c_double(dz))
        return ou, ov, ow

    def _jac(self, comp, x3, x3_old, rhs, va, dx, dy, dz, dt):
        self.lib.orc_do_jacobi(comp, self.nx, self.ny, self.nz, _p(x3), _p(x3_old), _p(rhs), _p(va),
                               C.c_double(dx), C.c_double(dy), C.c_double(dz), C.c_double(dt))
        return x3

    def do_jacobi_u(self, u3, u3_old, rhs, viscosity, dx, dy, dz, dt):
        return self._jac(0, u3, u3_old, rhs, viscosity, dx, dy, dz, dt)

    def do_jacobi_v(self, v3, v3_old, rhs, viscosity, dx, dy, dz, dt):
        return self._jac(1, v3, v3_old, rhs, viscosity, dx, dy, dz, dt)

    def do_jacobi_w(self, w3, w3_old, rhs, viscosity, dx, dy, dz, dt):
        return self._jac(2, w3, w3_old, rhs, viscosity, dx, dy, dz, dt)

    def _sor(self, comp, x3, rhs, va, dx, dy, dz, dt, flg, iteration_time):
        self.lib.orc_do_sor(comp, self.nx, self.ny, self.nz, _p(x3), _p(rhs), _p(va), C.c_double(dx),
                            C.c_double(dy), C.c_double(dz), C.c_double(dt), int(flg), int(iteration_time))
        return x3

    def do_sor_u(self, u3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time):
        return self._sor(0, u3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time)

    def do_sor_v(self, v3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time):
        return self._sor(1, v3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time)

    def do_sor_w(self, w3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time):
        return self._sor(2, w3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time)

    def momentum(self, comp, rhs, viscosity_aug, pres, max_iteration, dx, dy, dz, dt):
        kind = "w" if comp == 2 else "uv"
        x3, xo = self.zeros(kind), self.zeros(kind)
        err = C.c_double(0.0)
        self.lib.orc_momentum(comp, self.nx, self.ny, self.nz, _p(x3), _p(xo), _p(rhs), _p(viscosity_aug),
                              _p(pres), int(max_iteration), C.c_double(dx), C.c_double(dy), C.c_double(dz),
                              C.c_double(dt), C.byref(err))
        return x3, xo, err.value

    def get_difference(self, ua, ub):
        d = (ua[1:self.nx + 1, 1:self.ny + 1, :] - ub[1:self.nx + 1, 1:self.ny + 1, :])
        return float(np.sum(d * d))

    def get_source_pres(self, u3, v3, w3, dx, dy, dz, dt):
        rhs = self.zeros("p")
        self.lib.orc_get_source_pres(self.nx, self.ny, self.nz, _p(rhs), _p(u3), _p(v3), _p(w3),
                                     C.c_double(dx), C.c_double(dy), C.c_double(dz), C.c_double(dt))
        return rhs

    def get_uvw_pres(self, u3, v3, w3, p, dx, dy, dz, dt, u_inlet):
        uin = np.ascontiguousarray(u_inlet, dtype=np.float64)
        self.lib.orc_get_uvw_pres(self.nx, self.ny, self.nz, _p(u3), _p(v3), _p(w3), _p(p), C.c_double(dx),
                                  C.c_double(dy), C.c_double(dz), C.c_double(dt), uin.ctypes.data_as(_DP))
        return u3, v3, w3

    def pressure_solve(self, pres_old, rhs_p, u3, u_inlet, dx, dy, dz, dt, rtol=0.0, maxits=0):
        pres = np.array(pres_old, order="F", copy=True)
        rn = C.c_double(0.0)
        uin = np.ascontiguousarray(u_inlet, dtype=np.float64)
        self.lib.orc_pressure_solve(self.nx, self.ny, self.nz, _p(pres), _p(rhs_p), _p(u3),
                                    uin.ctypes.data_as(_DP), C.c_double(dx), C.c_double(dy), C.c_double(dz),
                                    C.c_double(dt), C.byref(rn))
        return pres, 0, rn.value, 2

    def exchange2d(self, uu):
        self.lib.orc_exchange2d(self.nx, self.ny, 0, uu.shape[2] - 1, _p(uu))
        return uu
