"""Host-side mirror of the reference's hot-path subroutine interface.

Each method of :class:`TplsGpu` has the name and argument meaning of the
reference routine it replaces (advect_phi.f90, two_phase_levelset.f90,
levelset.f90, momentum_allflux.f90, jacobi_iteration_allflux.f90,
sor_iteration_allflux.f90, pressure.f90, and main_ns_hybrid.F90's KSPSolve
call site) and calls the CUDA library through the C ABI of
``include/tpls_gpu.h``.  Arrays are numpy float64 arrays in the reference's
Fortran layout (``order='F'``):

* p-grid ``(nx+2, ny+2, nz+2)`` for index ranges (0:nx+1, 0:ny+1, 0:nz+1)
* u/v    ``(nx+2, ny+2, nz)``   for (0:nx+1, 0:ny+1, 0:nz-1)
* w      ``(nx+2, ny+2, nz+1)`` for (0:nx+1, 0:ny+1, 0:nz)
* viscosity_aug ``(nx+4, ny+4, nz+2)`` for (-1:nx+2, -1:ny+2, 0:nz+1)

``inout`` arguments are updated in place exactly where the reference writes
them.  There is no CPU fallback: if the native library is missing or a call
fails, an exception is raised.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_ROOT = Path(__file__).resolve().parent
LIB_PATH = _ROOT / "_lib" / "libtpls_gb300.so"

TPLS_PREC_FP64 = 0
TPLS_PREC_FP32_MIXED = 1
PART_ADVECT, PART_LEVELSET, PART_MOMENTUM, PART_MULTIGRID, PART_MOM_STENCIL = 1, 2, 4, 8, 16
TPLS_FLAG_NO_TMA = 1  # tpls_params.flags: advection without TMA-staged tiles
TPLS_FLAG_ODD_COLUMNS = 2  # tpls_params.flags: odd half-sweep one block per column, not per segment

# field ids (enum tpls_field)
TIMERS = ["advect", "levelset", "csf", "visc", "mom_rhs", "jacobi", "sor_even", "sor_odd", "pressure", "project",
          "other"]

F = dict(PHI2=0, U2=1, V2=2, W2=3, PRES=4, PRES_OLD=5, CONV0_U=6, CONV1_U=7, CONV0_V=8,
         CONV1_V=9, CONV0_W=10, CONV1_W=11, CSF_U0=12, CSF_U1=13, CSF_V0=14, CSF_V1=15,
         CSF_W0=16, CSF_W1=17, CONV0_PHI=18, CONV1_PHI=19, CONV2_PHI=20, PHI3=21, RHS_P=22,
         U3=23, V3=24, W3=25, CONVPREV_PHI=26)
FIELD_KIND = {name: ("uv" if name in ("U2", "V2", "CONV0_U", "CONV1_U", "CONV0_V", "CONV1_V",
                                      "CSF_U0", "CSF_U1", "CSF_V0", "CSF_V1", "U3", "V3")
                     else "w" if name in ("W2", "CONV0_W", "CONV1_W", "CSF_W0", "CSF_W1", "W3")
                     else "p") for name in F}
STATE_FIELDS = ["PHI2", "U2", "V2", "W2", "PRES", "PRES_OLD", "CONV0_U", "CONV1_U", "CONV0_V",
                "CONV1_V", "CONV0_W", "CONV1_W", "CSF_U0", "CSF_U1", "CSF_V0", "CSF_V1",
                "CSF_W0", "CSF_W1", "CONV0_PHI", "CONV1_PHI"]
# the diffuse-interface method's extra state: ConvPrevPhi and the reference's
# phi3 array (the next step's starting guess)
DIM_STATE_FIELDS = ["CONVPREV_PHI", "PHI3"]
IDM_LSM, IDM_DIM = 0, 1


class TplsParams(C.Structure):
    _fields_ = [("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
                ("re", C.c_double), ("mu_plus", C.c_double), ("mu_minus", C.c_double),
                ("height", C.c_double), ("scap", C.c_double), ("smooth_width", C.c_double),
                ("mom_u", C.c_int), ("mom_v", C.c_int), ("mom_w", C.c_int), ("levelset", C.c_int),
                ("p_rtol", C.c_double), ("p_maxits", C.c_int), ("precision", C.c_int),
                ("fp64_parts", C.c_int), ("mg_fp32", C.c_int), ("idm", C.c_int),
                ("max_iteration_dim", C.c_int), ("flags", C.c_int), ("reserved", C.c_int), ("epn", C.c_double),
                ("pe", C.c_double)]


class TplsStats(C.Structure):
    _fields_ = [("err_phi", C.c_double), ("err_u", C.c_double), ("err_v", C.c_double),
                ("err_w", C.c_double), ("p_rnorm", C.c_double), ("p_bnorm", C.c_double),
                ("p_its", C.c_int), ("p_reason", C.c_int), ("steps_done", C.c_long),
                ("liquid_volume", C.c_double), ("p_worst", C.c_int), ("kernel_timeouts", C.c_int),
                ("reserved_i", C.c_int * 2)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved_i"}


@dataclass
class Params:
    """Physical/solver parameters (the reference's .opt keys)."""
    dx: float
    dy: float
    dz: float
    dt: float
    re: float
    mu_plus: float
    mu_minus: float
    height: float = 0.5
    scap: float = 1.0
    smooth_width: float = 0.0
    mom_u: int = 30
    mom_v: int = 30
    mom_w: int = 30
    levelset: int = 10
    p_rtol: float = 1e-5
    p_maxits: int = 200
    precision: int = TPLS_PREC_FP64
    fp64_parts: int = 0  # FP32-mixed form: PART_* bits kept in FP64
    mg_fp32: int = 0  # FP64 form: FP32 multigrid levels in the CG preconditioner
    idm: int = IDM_LSM  # interface method: level set or diffuse interface (FP64 form)
    max_iteration_dim: int = 18  # tpls_config.opt default
    epn: float = 0.0  # diffuse interface width
    pe: float = 1.0  # Peclet number of the diffuse-interface method
    flags: int = 0  # TPLS_FLAG_* (1: no TMA staging in the FP32 advection)
    extra: dict = field(default_factory=dict)

    def to_c(self) -> TplsParams:
        p = TplsParams()
        for k, _ in TplsParams._fields_:
            if k != "reserved":
                setattr(p, k, getattr(self, k))
        return p


class TplsError(RuntimeError):
    pass


_lib = None

_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)


def load_library(path: Path | None = None) -> C.CDLL:
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise TplsError(f"native library {p} not found: run __graft_entry__.build() first")
    lib = C.CDLL(str(p))
    lib.tpls_status_string.restype = C.c_char_p
    lib.tpls_status_string.argtypes = [C.c_int]
    lib.tpls_gpu_create.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(TplsParams), _DP,
                                    C.POINTER(C.c_void_p)]
    lib.tpls_gpu_destroy.argtypes = [C.c_void_p]
    lib.tpls_set_field.argtypes = [C.c_void_p, C.c_int, _DP]
    lib.tpls_get_field.argtypes = [C.c_void_p, C.c_int, _DP]
    lib.tpls_step.argtypes = [C.c_void_p, C.c_int]
    lib.tpls_step_async.argtypes = [C.c_void_p, C.c_int]
    lib.tpls_graphs_enable.argtypes = [C.c_void_p, C.c_int]
    lib.tpls_autotune.argtypes = [C.c_void_p, C.c_int]
    lib.tpls_get_tiles.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    lib.tpls_get_stats.argtypes = [C.c_void_p, C.POINTER(TplsStats)]
    lib.tpls_sync.argtypes = [C.c_void_p]
    lib.tpls_kernel_launches.argtypes = [C.c_void_p]
    lib.tpls_kernel_launches.restype = C.c_long
    lib.tpls_base_profile.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                      C.c_double, C.c_double, C.c_double, _DP]
    lib.tpls_timing_enable.argtypes = [C.c_void_p, C.c_int]
    lib.tpls_timing_read.argtypes = [C.c_void_p, _DP, C.POINTER(C.c_long), C.c_int]
    lib.tpls_stream.argtypes = [C.c_void_p]
    lib.tpls_stream.restype = C.c_void_p
    lib.tpls_set_steps_done.argtypes = [C.c_void_p, C.c_long]
    lib.tpls_set_fields.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(_DP)]
    lib.tpls_get_fields.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(_DP)]
    lib.tpls_xfer_join.argtypes = [C.c_void_p]
    lib.tpls_selftest_wait_limit.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.tpls_register_host.argtypes = [C.c_void_p, _DP, C.c_longlong]
    lib.tpls_unregister_host.argtypes = [C.c_void_p, _DP]
    lib.tpls_download_host.argtypes = [C.c_void_p, _DP]
    lib.tpls_upload_host.argtypes = [C.c_void_p, _DP]
    lib.tpls_backup_channel.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p]
    lib.tpls_dataload_channel.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p]
    if path is None:
        _lib = lib
    return lib


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    if not (a.dtype == np.float64 and a.flags.f_contiguous):
        raise TypeError("arrays must be float64 and Fortran-contiguous")
    return a.ctypes.data_as(_DP)


def _i(v: int):
    return C.byref(C.c_int(int(v)))


def _d(v: float):
    return C.byref(C.c_double(float(v)))


def shape_of(kind: str, nx: int, ny: int, nz: int) -> tuple:
    return {"p": (nx + 2, ny + 2, nz + 2), "uv": (nx + 2, ny + 2, nz), "w": (nx + 2, ny + 2, nz + 1),
            "va": (nx + 4, ny + 4, nz + 2)}[kind]


def base_profile(nz: int, dz: float, re: float, dpdl: float, mu_minus: float, mu_plus: float,
                 height: float, smooth_width: float) -> np.ndarray:
    """twophase_initialisation_wave.F90:79-122 1-D base state u(z) (host code)."""
    lib = load_library()
    out = np.zeros(nz)
    s = lib.tpls_base_profile(nz, dz, re, dpdl, mu_minus, mu_plus, height, smooth_width,
                              out.ctypes.data_as(_DP))
    if s:
        raise TplsError(lib.tpls_status_string(s).decode())
    return out


class TplsGpu:
    """One channel on one GPU: device-resident state plus the per-routine
    drop-in entries."""

    def __init__(self, nx: int, ny: int, nz: int, params: Params, u_inlet: np.ndarray):
        self.lib = load_library()
        self.nx, self.ny, self.nz = nx, ny, nz
        self.params = params
        self._cp = params.to_c()
        uin = np.ascontiguousarray(u_inlet, dtype=np.float64)
        if uin.shape != (nz,):
            raise ValueError("u_inlet must have nz entries")
        self.u_inlet = uin
        self._registered = {}  # address -> array registered with tpls_register_host
        h = C.c_void_p()
        s = self.lib.tpls_gpu_create(nx, ny, nz, C.byref(self._cp), uin.ctypes.data_as(_DP), C.byref(h))
        self._check(s)
        self.ctx = h

    # -- housekeeping -----------------------------------------------------
    def _check(self, s: int) -> int:
        if s > 0:
            raise TplsError(f"tpls status {s}: {self.lib.tpls_status_string(s).decode()}")
        return s

    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.lib.tpls_gpu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def shape(self, kind: str) -> tuple:
        return shape_of(kind, self.nx, self.ny, self.nz)

    def zeros(self, kind: str) -> np.ndarray:
        return np.zeros(self.shape(kind), order="F")

    def _b(self):  # bounds passed by reference, single-rank values
        nx, ny = self.nx, self.ny
        return dict(sx=_i(1), ex=_i(nx), sy=_i(1), ey=_i(ny))

    # -- device-resident state --------------------------------------------
    def set_field(self, name: str, a: np.ndarray) -> None:
        a = np.asfortranarray(a, dtype=np.float64)
        if a.shape != self.shape(FIELD_KIND[name]):
            raise ValueError(f"{name}: shape {a.shape} != {self.shape(FIELD_KIND[name])}")
        self._check(self.lib.tpls_set_field(self.ctx, F[name], _ptr(a)))

    def get_field(self, name: str) -> np.ndarray:
        out = self.zeros(FIELD_KIND[name])
        self._check(self.lib.tpls_get_field(self.ctx, F[name], _ptr(out)))
        return out

    def get_field_into(self, name: str, out: np.ndarray) -> np.ndarray:
        """Download a field into an existing Fortran-ordered array (e.g. one
        in pinned host memory)."""
        if out.shape != self.shape(FIELD_KIND[name]):
            raise ValueError(f"{name}: shape {out.shape} != {self.shape(FIELD_KIND[name])}")
        self._check(self.lib.tpls_get_field(self.ctx, F[name], _ptr(out)))
        return out

    def set_fields(self, arrays: dict) -> None:
        """Upload several fields in one tpls_set_fields call (enqueued, no
        host wait between fields; later steps run after the uploads).  The
        arrays must stay alive and unchanged until the context is synced."""
        names = list(arrays)
        for k in names:
            a = arrays[k]
            if not (a.dtype == np.float64 and a.flags.f_contiguous) or a.shape != self.shape(FIELD_KIND[k]):
                raise ValueError(f"{k}: needs a Fortran-ordered float64 array of shape {self.shape(FIELD_KIND[k])}")
        ids = (C.c_int * len(names))(*[F[k] for k in names])
        ptrs = (_DP * len(names))(*[_ptr(arrays[k]) for k in names])
        self._check(self.lib.tpls_set_fields(self.ctx, len(names), ids, ptrs))

    def get_fields_into(self, arrays: dict) -> None:
        """Download several fields into existing Fortran-ordered arrays in one
        tpls_get_fields call; the arrays hold the data after sync()."""
        names = list(arrays)
        for k in names:
            a = arrays[k]
            if not (a.dtype == np.float64 and a.flags.f_contiguous) or a.shape != self.shape(FIELD_KIND[k]):
                raise ValueError(f"{k}: needs a Fortran-ordered float64 array of shape {self.shape(FIELD_KIND[k])}")
        ids = (C.c_int * len(names))(*[F[k] for k in names])
        ptrs = (_DP * len(names))(*[_ptr(arrays[k]) for k in names])
        self._check(self.lib.tpls_get_fields(self.ctx, len(names), ids, ptrs))

    def xfer_join(self) -> None:
        """Later work on the context's stream waits for the downloads so far."""
        self._check(self.lib.tpls_xfer_join(self.ctx))

    def set_state(self, state: dict) -> None:
        for k, v in state.items():
            self.set_field(k, v)

    def state_fields(self) -> list:
        return STATE_FIELDS + (DIM_STATE_FIELDS if self.params.idm == IDM_DIM else [])

    def get_state(self) -> dict:
        return {k: self.get_field(k) for k in self.state_fields()}

    def step(self, nsteps: int = 1) -> int:
        """nsteps timesteps on device-resident state; returns the status
        (0, or a negative KSP-style reason of the last pressure solve)."""
        return self._check(self.lib.tpls_step(self.ctx, nsteps))

    def step_async(self, nsteps: int = 1) -> None:
        """Enqueue nsteps graph-launched steps without waiting; the solves'
        outcome is in stats()["p_worst"]."""
        self._check(self.lib.tpls_step_async(self.ctx, nsteps))

    def autotune(self, reps: int = 10) -> dict:
        """Tile shapes of the sweep kernels chosen by timing (tpls_autotune)."""
        self._check(self.lib.tpls_autotune(self.ctx, reps))
        t = (C.c_int * 3)()
        self._check(self.lib.tpls_get_tiles(self.ctx, t))
        return {"jacobi": t[0], "sor_even": t[1], "sor_odd": t[2]}

    def register_host(self, a: np.ndarray) -> None:
        """Keep a host array device-resident behind its address
        (tpls_register_host): routines called with it read and write its
        device mirror, and `a` itself changes only on download_host."""
        self._check(self.lib.tpls_register_host(self.ctx, _ptr(a), a.size))
        self._registered[a.ctypes.data] = a  # the address must stay valid

    def unregister_host(self, a: np.ndarray) -> None:
        self._check(self.lib.tpls_unregister_host(self.ctx, _ptr(a)))
        self._registered.pop(a.ctypes.data, None)

    def download_host(self, a: np.ndarray | None = None) -> None:
        """Host array(s) <- device mirror(s) (all registered when a is None)."""
        self._check(self.lib.tpls_download_host(self.ctx, _ptr(a)))

    def upload_host(self, a: np.ndarray | None = None) -> None:
        """Device mirror(s) <- host array(s) (all registered when a is None)."""
        self._check(self.lib.tpls_upload_host(self.ctx, _ptr(a)))

    def set_steps_done(self, n: int) -> None:
        """Continue an earlier run's step count (tpls_stats.steps_done)."""
        self._check(self.lib.tpls_set_steps_done(self.ctx, int(n)))

    def backup_channel(self, filename, csf_filename=None) -> None:
        """io.F90:647 backup_channel of the device state: the reference's
        text backup, plus (csf_filename) the CSF histories it leaves out."""
        self._check(self.lib.tpls_backup_channel(self.ctx, str(filename).encode(),
                                                 None if csf_filename is None else str(csf_filename).encode()))

    def dataload_channel(self, filename, csf_filename=None) -> None:
        """io.F90:721 dataload_channel into the device state."""
        self._check(self.lib.tpls_dataload_channel(self.ctx, str(filename).encode(),
                                                   None if csf_filename is None else str(csf_filename).encode()))

    def graphs_enable(self, on: bool = True) -> None:
        self._check(self.lib.tpls_graphs_enable(self.ctx, 1 if on else 0))

    def stats(self) -> dict:
        st = TplsStats()
        self._check(self.lib.tpls_get_stats(self.ctx, C.byref(st)))
        return st.as_dict()

    def sync(self) -> None:
        self._check(self.lib.tpls_sync(self.ctx))

    def kernel_launches(self) -> int:
        return int(self.lib.tpls_kernel_launches(self.ctx))

    def stream_ptr(self) -> int:
        """cudaStream_t (as an integer) all kernels of this context run on."""
        return int(self.lib.tpls_stream(self.ctx) or 0)

    def timing_enable(self, on: bool = True) -> None:
        self._check(self.lib.tpls_timing_enable(self.ctx, 1 if on else 0))

    def timing_read(self, reset: bool = False) -> dict:
        """{phase: (device ms, kernel launches)} accumulated since the last
        reset, measured with CUDA events on the context stream."""
        ms = (C.c_double * len(TIMERS))()
        n = (C.c_long * len(TIMERS))()
        self._check(self.lib.tpls_timing_read(self.ctx, ms, n, 1 if reset else 0))
        return {k: (ms[i], n[i]) for i, k in enumerate(TIMERS)}

    # -- per-routine drop-in entries ----------------------------------------
    def do_advect_phi(self, phi2, u2, v2, w2, dx, dy, dz, conv2_phi=None):
        """advect_phi.f90:19 -> conv2_phi; u2, v2, w2 get their halo rows
        exchanged in place, as in the reference."""
        nx, ny, nz = self.nx, self.ny, self.nz
        conv = self.zeros("p") if conv2_phi is None else conv2_phi
        b = self._b()
        nb = (C.c_int * 6)(*([-2] * 6))
        s = self.lib.tpls_do_advect_phi(
            self.ctx, _ptr(phi2), _ptr(u2), _ptr(v2), _ptr(w2), _ptr(conv), b["sx"], b["ex"], b["sy"],
            b["ey"], _i(0), _i(nz + 1), _i(0), _i(0), _i(nz - 1), _i(nz), _i(nx + 1), _i(nz + 1),
            _i(nx), nb, _i(0), _d(dx), _d(dy), _d(dz), *([_i(0)] * 10))
        self._check(s)
        return conv

    def dim(self, phi, phi_old, conv2_phi, conv_prev_phi, phi_new, max_iteration_dim, epn, pe, height, dx,
            dy, dz, dt):
        """cahn_hilliard_solver.f90:41 dim -> (phi_new, conv_prev_phi) (C fields, copies)."""
        nz = self.nz
        phi_new = np.array(phi_new, order="F", copy=True)
        conv_prev_phi = np.array(conv_prev_phi, order="F", copy=True)
        b = self._b()
        nb = (C.c_int * 6)(*([-2] * 6))
        s = self.lib.tpls_dim(self.ctx, _i(self.nx + 1), _i(nz + 1), _d(dx), _d(dy), _d(dz), _d(dt), _d(epn),
                              _d(pe), _ptr(phi), _ptr(phi_old), _ptr(conv2_phi), _ptr(conv_prev_phi),
                              _ptr(phi_new), b["sx"], b["ex"], b["sy"], b["ey"], _i(0), _i(nz + 1), _d(height),
                              _i(0), _i(0), nb, _i(0), _i(max_iteration_dim))
        self._check(s)
        return phi_new, conv_prev_phi

    def do_tpls(self, phi2, conv0_phi, conv1_phi, conv2_phi, max_iteration_levelset, height, dx, dz,
                dt, phi3=None):
        """two_phase_levelset.f90:20 -> (phi3, err2)."""
        nz = self.nz
        phi3 = self.zeros("p") if phi3 is None else phi3
        err2 = C.c_double(0.0)
        b = self._b()
        nb = (C.c_int * 6)(*([-2] * 6))
        s = self.lib.tpls_do_tpls(self.ctx, _ptr(phi2), _ptr(phi3), _ptr(conv0_phi), _ptr(conv1_phi),
                                  _ptr(conv2_phi), b["sx"], b["ex"], b["sy"], b["ey"], _i(0), _i(nz + 1),
                                  _i(nz + 1), _i(self.nx), _i(0), _i(0), _i(max_iteration_levelset), nb,
                                  _i(0), _d(height), C.byref(err2), _d(dx), _d(dz), _d(dt))
        self._check(s)
        return phi3, err2.value

    def get_csf(self, fi, dx, dy, dz, scap, smooth_width, fx=None, fy=None, fz=None):
        """levelset.f90:241 -> (fx_csf, fy_csf, fz_csf)."""
        fx = self.zeros("p") if fx is None else fx
        fy = self.zeros("p") if fy is None else fy
        fz = self.zeros("p") if fz is None else fz
        b = self._b()
        s = self.lib.tpls_get_csf(self.ctx, _ptr(fx), _ptr(fy), _ptr(fz), _ptr(fi), b["sx"], b["ex"], b["sy"],
                                  b["ey"], _i(self.nz + 1), _i(self.nx), _d(dx), _d(dy), _d(dz), _d(scap),
                                  _d(smooth_width))
        self._check(s)
        return fx, fy, fz

    def get_viscosity(self, phi, smooth_width, re, mu_minus, mu_plus, viscosity_aug=None):
        """momentum_allflux.f90:474 plus main_ns_hybrid.F90:646-724 ->
        viscosity_aug (-1:nx+2,-1:ny+2,0:nz+1); x=-1, nx+2 are not written."""
        va = np.full(self.shape("va"), np.nan, order="F") if viscosity_aug is None else viscosity_aug
        b = self._b()
        s = self.lib.tpls_get_viscosity(self.ctx, _ptr(va), _ptr(phi), b["ex"], b["ey"], b["sx"], b["sy"],
                                        _i(self.nz + 1), _d(smooth_width), _d(re), _d(mu_minus), _d(mu_plus))
        self._check(s)
        return va

    def _conv_diff(self, fn, va, u2, v2, w2, dx, dy, dz, out=None):
        ou, ov, ow = (self.zeros("uv"), self.zeros("uv"), self.zeros("w")) if out is None else out
        b = self._b()
        s = fn(self.ctx, _ptr(ou), _ptr(ov), _ptr(ow), _ptr(va), _ptr(u2), _ptr(v2), _ptr(w2), b["sx"],
               b["sy"], b["ex"], b["ey"], _i(self.nz + 1), _i(self.nx), _d(dx), _d(dy), _d(dz))
        self._check(s)
        return ou, ov, ow

    def get_conv_all(self, viscosity_aug, u2, v2, w2, dx, dy, dz, out=None):
        """momentum_allflux.f90:224 -> (conv_u2, conv_v2, conv_w2)."""
        return self._conv_diff(self.lib.tpls_get_conv_all, viscosity_aug, u2, v2, w2, dx, dy, dz, out)

    def get_diffusion_all(self, viscosity_aug, u2, v2, w2, dx, dy, dz, out=None):
        """momentum_allflux.f90:22 -> (diff_u, diff_v, diff_w)."""
        return self._conv_diff(self.lib.tpls_get_diffusion_all, viscosity_aug, u2, v2, w2, dx, dy, dz, out)

    def _jac(self, fn, x3, x3_old, rhs, va, dx, dy, dz, dt):
        b = self._b()
        s = fn(self.ctx, _ptr(x3), _ptr(x3_old), _ptr(rhs), _ptr(va), _d(dx), _d(dy), _d(dz), _d(dt), b["ex"],
               b["ey"], b["sx"], b["sy"], _i(self.nz + 1), _i(self.nx))
        self._check(s)
        return x3

    def do_jacobi_u(self, u3, u3_old, rhs, viscosity, dx, dy, dz, dt):
        """jacobi_iteration_allflux.f90:21 (u3 updated in place)."""
        return self._jac(self.lib.tpls_do_jacobi_u, u3, u3_old, rhs, viscosity, dx, dy, dz, dt)

    def do_jacobi_v(self, v3, v3_old, rhs, viscosity, dx, dy, dz, dt):
        return self._jac(self.lib.tpls_do_jacobi_v, v3, v3_old, rhs, viscosity, dx, dy, dz, dt)

    def do_jacobi_w(self, w3, w3_old, rhs, viscosity, dx, dy, dz, dt):
        return self._jac(self.lib.tpls_do_jacobi_w, w3, w3_old, rhs, viscosity, dx, dy, dz, dt)

    def do_sor_u(self, u3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time):
        """sor_iteration_allflux.f90:19 (u3 updated in place)."""
        b = self._b()
        s = self.lib.tpls_do_sor_u(self.ctx, _ptr(u3), _ptr(rhs), _ptr(viscosity), _d(dx), _d(dy), _d(dz),
                                   _d(dt), b["ex"], b["ey"], b["sx"], b["sy"], _i(self.nz + 1), _i(self.nx),
                                   _i(flg), _i(iteration_time))
        self._check(s)
        return u3

    def _sor_vw(self, fn, x3, rhs, va, dx, dy, dz, dt, flg, iteration_time):
        b = self._b()
        s = fn(self.ctx, _ptr(x3), _ptr(rhs), _ptr(va), _d(dx), _d(dy), _d(dz), _d(dt), b["ex"], b["ey"],
               b["sx"], b["sy"], _i(self.nz + 1), _i(flg), _i(iteration_time))
        self._check(s)
        return x3

    def do_sor_v(self, v3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time):
        return self._sor_vw(self.lib.tpls_do_sor_v, v3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time)

    def do_sor_w(self, w3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time):
        return self._sor_vw(self.lib.tpls_do_sor_w, w3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time)

    def get_difference(self, ua, ub):
        """jacobi_iteration_allflux.f90:285 over i 1..nx, j 1..ny, all planes."""
        out = C.c_double(0.0)
        b = self._b()
        s = self.lib.tpls_get_difference(self.ctx, _ptr(ua), _ptr(ub), b["ex"], b["ey"], _i(ua.shape[2] - 1),
                                         b["sx"], b["sy"], _i(0), C.byref(out))
        self._check(s)
        return out.value

    def get_source_pres(self, u3, v3, w3, dx, dy, dz, dt, rhs=None):
        """pressure.f90:16 -> RHS_p."""
        rhs = self.zeros("p") if rhs is None else rhs
        b = self._b()
        s = self.lib.tpls_get_source_pres(self.ctx, _ptr(rhs), _ptr(u3), _ptr(v3), _ptr(w3), b["ex"], b["ey"],
                                          b["sx"], b["sy"], _i(self.nz + 1), _d(dx), _d(dy), _d(dz), _d(dt))
        self._check(s)
        return rhs

    def get_uvw_pres(self, u3, v3, w3, p, dx, dy, dz, dt, u_inlet):
        """pressure.f90:59 (u3, v3, w3 updated in place on rows 1..ny)."""
        b = self._b()
        uin = np.ascontiguousarray(u_inlet, dtype=np.float64)
        s = self.lib.tpls_get_uvw_pres(self.ctx, _ptr(u3), _ptr(v3), _ptr(w3), _ptr(p), b["ex"], b["ey"],
                                       b["sx"], b["sy"], _i(self.nz + 1), _i(self.nx), _d(dx), _d(dy), _d(dz),
                                       _d(dt), uin.ctypes.data_as(_DP))
        self._check(s)
        return u3, v3, w3

    def pressure_solve(self, pres_old, rhs_p, u3, u_inlet, dx, dy, dz, dt, rtol=0.0, maxits=0, pres=None):
        """`pres=pres_old; KSPSolve; copy_pressure_out_of_petsc`
        (main_ns_hybrid.F90:896-913) -> (pres, its, rnorm, reason)."""
        pres = self.zeros("p") if pres is None else pres
        its, rn, rs = C.c_int(0), C.c_double(0.0), C.c_int(0)
        uin = np.ascontiguousarray(u_inlet, dtype=np.float64)
        s = self.lib.tpls_pressure_solve(self.ctx, _ptr(pres), _ptr(pres_old), _ptr(rhs_p), _ptr(u3),
                                         uin.ctypes.data_as(_DP), _d(dx), _d(dy), _d(dz), _d(dt), _d(rtol),
                                         _i(maxits), C.byref(its), C.byref(rn), C.byref(rs))
        self._check(s)
        return pres, its.value, rn.value, rs.value

    def exchange2d(self, uu):
        """mpi.f90:110 on one rank: periodic copy of the y-ghost rows."""
        b = self._b()
        s = self.lib.tpls_exchange2d(self.ctx, _ptr(uu), b["ex"], b["ey"], _i(uu.shape[2] - 1), b["sx"], b["sy"],
                                     _i(0))
        self._check(s)
        return uu
