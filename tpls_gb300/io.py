"""The reference's file formats, for a drop-in that keeps its inputs and
outputs: 3-D `.dat` arrays (io.F90:47-169 save_data / load_data /
load_data_into_array) and `.opt` option files (options_utils.F90:254-332
load_options), plus the mapping from the option keys to the solver
parameters (option_names.F90, twophase_initialisation_wave.F90:66-75 for
the grid).

.dat layout: a description line, a dimension-header line, one line with
the six bounds `lx ly mx my nx ny`, then one value per line in Fortran
order (i fastest).  .opt layout: `name value` pairs, `#` comments and
blank lines ignored; any other line without a separating space is a format
error.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .api import Params, TPLS_PREC_FP64

OPTION_FILE_NOT_FOUND_ERR = -1  # option_names.F90 error codes
OPTION_FORMAT_ERR = -2


def save_data(filename, description: str, data: np.ndarray, bounds: tuple) -> None:
    """save_data (io.F90:47-73): data has shape (ly-lx+1, my-mx+1, ny-nx+1)."""
    lx, ly, mx, my, nx, ny = bounds
    a = np.asarray(data, dtype=np.float64)
    if a.shape != (ly - lx + 1, my - mx + 1, ny - nx + 1):
        raise ValueError(f"shape {a.shape} does not match bounds {bounds}")
    with open(filename, "w") as f:
        f.write(f" DATA: {description}\n")
        f.write(" DIMENSIONS: Lmin Lmax Mmin Mmax Nmin Nmax\n")
        f.write(f" {lx:11d} {ly:11d} {mx:11d} {my:11d} {nx:11d} {ny:11d}\n")
        for v in a.ravel(order="F"):
            f.write(f"  {v:.17E}\n")


def _read_values(lines, n):
    vals = []
    for line in lines:
        t = line.strip()
        if t:
            vals.append(float(t.replace("D", "E").replace("d", "e")))
        if len(vals) == n:
            break
    return vals


def load_data(filename):
    """load_data (io.F90:82-116): returns (data, bounds, ierr); ierr = 1 when
    the file holds fewer values than its bounds say."""
    with open(filename) as f:
        f.readline()
        f.readline()
        lx, ly, mx, my, nx, ny = (int(t) for t in f.readline().split()[:6])
        shape = (ly - lx + 1, my - mx + 1, ny - nx + 1)
        n = shape[0] * shape[1] * shape[2]
        vals = _read_values(f, n)
    ierr = 0 if len(vals) == n else 1
    data = np.zeros(n)
    data[:len(vals)] = vals
    return data.reshape(shape, order="F"), (lx, ly, mx, my, nx, ny), ierr


def load_data_into_array(filename, bounds: tuple):
    """load_data_into_array (io.F90:127-169): ierr 1 / 2 / 3 when the file's
    l / m / n bounds differ from `bounds` (checked in that order)."""
    lx, ly, mx, my, nx, ny = bounds
    with open(filename) as f:
        f.readline()
        f.readline()
        flx, fly, fmx, fmy, fnx, fny = (int(t) for t in f.readline().split()[:6])
        if (flx, fly) != (lx, ly):
            return None, 1
        if (fmx, fmy) != (mx, my):
            return None, 2
        if (fnx, fny) != (nx, ny):
            return None, 3
        shape = (ly - lx + 1, my - mx + 1, ny - nx + 1)
        vals = _read_values(f, shape[0] * shape[1] * shape[2])
    return np.asarray(vals).reshape(shape, order="F"), 0


def load_options(filename):
    """load_options: returns (dict name -> value string, ierr)."""
    p = Path(filename)
    if not p.exists():
        return {}, OPTION_FILE_NOT_FOUND_ERR
    opts = {}
    for raw in p.read_text().splitlines():
        line = raw.strip()
        if not line or line.startswith("#"):
            continue
        parts = line.split(None, 1)
        if len(parts) < 2:
            return opts, OPTION_FORMAT_ERR
        opts[parts[0]] = parts[1].strip()
    return opts, 0


def params_from_options(opts: dict, precision: int = TPLS_PREC_FP64, p_rtol: float = 1e-5, p_maxits: int = 200):
    """(nx, ny, nz, Params) from the reference's option keys: maxl/maxm/maxn
    are nx+1 / ny+1 / nz+1; the grid is the reference's cubic one,
    dz = 1/(maxn-1), dx = dy = dz; smooth_width = smooth_width_scale * dx."""
    nx, ny, nz = int(opts["maxl"]) - 1, int(opts["maxm"]) - 1, int(opts["maxn"]) - 1
    dz = 1.0 / nz
    dx = dy = dz
    f = lambda k, d=None: float(opts[k]) if k in opts else d
    i = lambda k, d=None: int(opts[k]) if k in opts else d
    params = Params(dx=dx, dy=dy, dz=dz, dt=f("dt"), re=f("re"), mu_plus=f("mu_plus"), mu_minus=f("mu_minus"),
                    height=f("height", 0.5), scap=f("scap", 1.0),
                    smooth_width=f("smooth_width_scale", 1.5) * dx, mom_u=i("mom_u", 30), mom_v=i("mom_v", 30),
                    mom_w=i("mom_w", 30), levelset=i("levelset", 10), p_rtol=p_rtol, p_maxits=p_maxits,
                    precision=precision)
    return nx, ny, nz, params
