"""The reference's file formats, for a drop-in that keeps its inputs and
outputs: 3-D `.dat` arrays (io.F90:47-169 save_data / load_data /
load_data_into_array), the Tecplot-style point files the driver writes
(io.F90:217-246, 503-534, 551-643 channel_output_phi / channel_input_phi /
channel_output_uvw / channel_output2d), `.opt` option files and the
option accessors (options_utils.F90:56-461), plus the mapping from the
option keys to the solver parameters (option_names.F90,
twophase_initialisation_wave.F90:66-75 for the grid).

.dat layout: a description line, a dimension-header line, one line with
the six bounds `lx ly mx my nx ny`, then one value per line in Fortran
order (i fastest).  .opt layout: `name value` pairs split at the first
space, `#` comments and blank lines ignored; a line without a space inside
it is a format error.

Options are an insertion-ordered dict name -> value string, the
reference's two-column array: putting an existing name replaces its value
in place.  Values read back from text follow Fortran list-directed input
(the first blank- or comma-separated item; `d` exponents; logicals by
their first letter after an optional period).  Where the reference's read
would stop the program on an invalid value, the accessors return
OPTION_INVALID_ERR instead.

Numbers in the point files are written with 17 significant digits, which
round-trip exactly; the reference's list-directed output spaces them by
compiler, and its readers (and channel_input_phi here) accept any spacing.
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

from .api import Params, TPLS_PREC_FP64

# options_utils.F90:40-51
OPTION_NOT_FOUND_ERR = 100
OPTION_FORMAT_ERR = 101
OPTION_INVALID_ERR = 102
OPTION_FILE_NOT_FOUND_ERR = 103

_LINE, _NAME, _VALUE, _TYPED = 80, 20, 60, 60  # the reference's character lengths


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


def get_filepath(directory: str, filename: str) -> str:
    """get_filepath (io.F90:25-31): directory/filename, trailing blanks of
    both removed."""
    return f"{directory.rstrip(' ')}/{filename.rstrip(' ')}"


def row_to_grid(lx: int, ly: int, mx: int, my: int, nx: int, ny: int, row: int):
    """row_to_grid (io.F90:801-816): the (l, m, n) index of the 1-based row
    of a .dat file with bounds (lx:ly, mx:my, nx:ny)."""
    nl, nm = ly - lx + 1, my - mx + 1
    return (row - 1) % nl + lx, ((row - 1) // nl) % nm + mx, (row - 1) // (nl * nm) + nx


def save_backup_info(filename, lx: int, ly: int, mx: int, my: int, nx: int, ny: int, dx: int, dy: int,
                     dz: int) -> None:
    """save_backup_info (io.F90:180-200): the bounds and the cell sizes.  The
    reference declares dx, dy, dz integer, so they are written as integers."""
    with open(filename, "w") as f:
        f.write(" DIMENSIONS: Lmin Lmax Mmin Mmax Nmin Nmax\n")
        f.write("".join(f" {int(v):11d}" for v in (lx, ly, mx, my, nx, ny)) + "\n")
        f.write(" DIMENSIONS: Dx,Dy,Dz\n")
        f.write("".join(f" {int(v):11d}" for v in (dx, dy, dz)) + "\n")


def _zone_header(f, variables: str, l: int, m: int | None, n: int) -> None:
    f.write(f" VARIABLES={variables}\n")
    if m is None:
        f.write(f' ZONE T="Floor", I={l - 1:12d}  K={n - 1:12d}  F=POINT\n')
    else:
        f.write(f' ZONE T="Floor", I={l - 1:12d}  J={m - 1:12d}  K={n - 1:12d}  F=POINT\n')


def _row(f, values) -> None:
    f.write("".join(f" {float(v): .17E}" for v in values) + "\n")


def channel_output_phi(phi: np.ndarray, l: int, m: int, n: int, dx: float, dy: float, dz: float,
                       filename) -> None:
    """channel_output_phi (io.F90:217-246): rows `x y z phi(i+1, j, k+1)` for
    k = 0..n-2, j = 0..m-2, i = 1..l-1 (i fastest), x = dx/2 + dx i, likewise
    y, z; phi indexed [0..l, 0..m, 0..n]."""
    with open(filename, "w") as f:
        _zone_header(f, '"X ","Y ","Z ","Phi"', l, m, n)
        for k in range(n - 1):
            z = dz / 2.0 + dz * k
            for j in range(m - 1):
                y = dy / 2.0 + dy * j
                for i in range(1, l):
                    _row(f, (dx / 2.0 + dx * i, y, z, phi[i + 1, j, k + 1]))


def _records(f):
    for line in f:
        yield line.replace(",", " ").split()


def channel_input_phi(filename, l: int, m: int, n: int, phi: np.ndarray | None = None):
    """channel_input_phi (io.F90:503-534): reads what channel_output_phi
    wrote into phi[i+1, j, k+1] (other entries kept; zeros when phi is None)
    and returns (phi, ierr).  Each row is a list-directed read of four items:
    they may span records, and the rest of the record holding the fourth is
    skipped.  ierr = 1 when the file holds fewer than (l-1)(m-1)(n-1) rows
    (where the reference's read stops the program at the end of the file)."""
    out = np.zeros((l + 1, m + 1, n + 1)) if phi is None else phi
    rows = 0
    with open(filename) as f:
        f.readline()
        f.readline()
        rec = _records(f)
        done = False
        for k in range(n - 1):
            for j in range(m - 1):
                for i in range(1, l):
                    items: list = []
                    for r in rec:
                        items += r
                        if len(items) >= 4:
                            break
                    if len(items) < 4:
                        done = True
                        break
                    out[i + 1, j, k + 1] = float(re.sub(r"[dDqQ]", "e", items[3]))
                    rows += 1
                if done:
                    break
            if done:
                break
    return out, (0 if rows == (l - 1) * (m - 1) * (n - 1) else 1)


def channel_output_uvw(u3: np.ndarray, v3: np.ndarray, w3: np.ndarray, p: np.ndarray, l: int, m: int, n: int,
                       dx: float, dy: float, dz: float, filename) -> None:
    """channel_output_uvw (io.F90:551-587): rows `x y z u v w p(i, j, k+1)`
    over the same points as channel_output_phi, with u, v, w the averages of
    the two faces around the cell centre; u3, v3 indexed [0..l, 0..m,
    0..n-2], w3 [0..l, 0..m, 0..n-1], p [0..l, 0..m, 0..n]."""
    with open(filename, "w") as f:
        _zone_header(f, '"X ","Y ","Z ","U","V","W","P"', l, m, n)
        for k in range(n - 1):
            z = dz / 2.0 + dz * k
            for j in range(m - 1):
                y = dy / 2.0 + dy * j
                for i in range(1, l):
                    _row(f, (dx / 2.0 + dx * i, y, z, (u3[i, j, k] + u3[i + 1, j, k]) / 2.0,
                             (v3[i, j, k] + v3[i, j + 1, k]) / 2.0, (w3[i, j, k] + w3[i, j, k + 1]) / 2.0,
                             p[i, j, k + 1]))


def channel_output2d(u3: np.ndarray, v3: np.ndarray, w3: np.ndarray, p: np.ndarray, phi: np.ndarray,
                     visc: np.ndarray, l: int, m: int, n: int, dx: float, dy: float, dz: float, filename) -> None:
    """channel_output2d (io.F90:604-643): the x-z plane j = (m-1)/2, rows
    `x z u v w p(i, j, k+1) phi(i+1, j, k+1) visc(i, j, k+1)`."""
    j = (m - 1) // 2
    with open(filename, "w") as f:
        _zone_header(f, '"X ","Z ","U","V","W","P","fi","Viscosity"', l, None, n)
        for k in range(n - 1):
            z = dz / 2.0 + dz * k
            for i in range(1, l):
                _row(f, (dx / 2.0 + dx * i, z, (u3[i, j, k] + u3[i + 1, j, k]) / 2.0,
                         (v3[i, j, k] + v3[i, j + 1, k]) / 2.0, (w3[i, j, k] + w3[i, j, k + 1]) / 2.0,
                         p[i, j, k + 1], phi[i + 1, j, k + 1], visc[i, j, k + 1]))


def has_option(options: dict, name: str) -> bool:
    """has_option (options_utils.F90:56-70)."""
    return name.rstrip() in options


def get_option(options: dict, name: str):
    """get_option (options_utils.F90:74-91): (value string, 0) or
    (None, OPTION_NOT_FOUND_ERR)."""
    v = options.get(name.rstrip())
    return (v, 0) if v is not None else (None, OPTION_NOT_FOUND_ERR)


get_string_option = get_option  # options_utils.F90:140-148


def _first_item(text: str) -> str:
    """The first item of a list-directed read: leading blanks skipped, ended
    by a blank, a comma or a slash."""
    m = re.match(r"[ \t]*([^ \t,/]*)", text)
    return m.group(1) if m else ""


_INT_RE = re.compile(r"[+-]?\d+$")
_REAL_RE = re.compile(r"[+-]?(\d+\.?\d*|\.\d+)([eEdDqQ][+-]?\d+)?$")


def _typed(options: dict, name: str, parse):
    v, ierr = get_option(options, name)
    if ierr:
        return None, ierr
    try:
        return parse(_first_item(v[:_TYPED])), 0
    except ValueError:
        return None, OPTION_INVALID_ERR


def _parse_int(t: str) -> int:
    if not _INT_RE.match(t):
        raise ValueError(t)
    return int(t)


def _parse_real(t: str) -> float:
    if not _REAL_RE.match(t):
        raise ValueError(t)
    return float(re.sub(r"[dDqQ]", "e", t))


def _parse_logical(t: str) -> bool:
    u = t[1:] if t.startswith(".") else t
    if u[:1] in ("T", "t"):
        return True
    if u[:1] in ("F", "f"):
        return False
    raise ValueError(t)


def get_integer_option(options: dict, name: str):
    """get_integer_option (options_utils.F90:110-121): (int, ierr)."""
    return _typed(options, name, _parse_int)


def get_double_option(options: dict, name: str):
    """get_double_option (options_utils.F90:125-136): (float, ierr)."""
    return _typed(options, name, _parse_real)


def get_logical_option(options: dict, name: str):
    """get_logical_option (options_utils.F90:95-106): (bool, ierr)."""
    return _typed(options, name, _parse_logical)


def get_typed_option(options: dict, name: str, kind=str):
    """get_typed_option (options_utils.F90:17-22), the type chosen by `kind`
    (str, int, float or bool) where Fortran chooses by the argument's type."""
    return {str: get_option, int: get_integer_option, float: get_double_option,
            bool: get_logical_option}[kind](options, name)


def put_option(options: dict, name: str, value: str) -> None:
    """put_option (options_utils.F90:157-174): replace the value of an
    existing name in place, else append the pair."""
    options[name.rstrip()] = str(value).rstrip()


def put_string_option(options: dict, name: str, value: str) -> None:
    """put_string_option (options_utils.F90:220-227)."""
    put_option(options, name, value)


def _fortran_field(text: str, width: int) -> str:
    return text if len(text) <= width else "*" * width


def put_integer_option(options: dict, name: str, value: int) -> None:
    """put_integer_option (options_utils.F90:193-202): the value as I10."""
    put_option(options, name, _fortran_field(f"{int(value):{10}d}", 10))


def put_double_option(options: dict, name: str, value: float) -> None:
    """put_double_option (options_utils.F90:207-216): the value as F20.10."""
    put_option(options, name, _fortran_field(f"{float(value):{20}.10f}", 20))


def put_logical_option(options: dict, name: str, value: bool) -> None:
    """put_logical_option (options_utils.F90:179-188): the value as L1."""
    put_option(options, name, "T" if value else "F")


def put_typed_option(options: dict, name: str, value) -> None:
    """put_typed_option (options_utils.F90:25-30), by the value's type."""
    if isinstance(value, (bool, np.bool_)):
        put_logical_option(options, name, bool(value))
    elif isinstance(value, (int, np.integer)):
        put_integer_option(options, name, int(value))
    elif isinstance(value, (float, np.floating)):
        put_double_option(options, name, float(value))
    else:
        put_string_option(options, name, str(value))


def print_options(options: dict, file=None) -> None:
    """print_options (options_utils.F90:231-240): `name value` lines."""
    out = file if file is not None else sys.stdout
    for k, v in options.items():
        out.write(f"{k} {v.rstrip()}\n")


def load_options(filename):
    """load_options (options_utils.F90:254-332): returns (options, ierr).

    A line is its first 80 characters with leading blanks removed; `#`
    lines and blank lines are skipped; the rest splits at the first space
    into a name (first 20 characters) and a value (the rest with trailing
    blanks removed, first 60 characters; leading blanks kept).  A line with
    no space inside it ends the load with OPTION_FORMAT_ERR, the options
    read so far returned.  A name given twice keeps its first position and
    its last value."""
    p = Path(filename)
    if not p.exists():
        return {}, OPTION_FILE_NOT_FOUND_ERR
    opts: dict = {}
    for raw in p.read_text().splitlines():
        line = raw[:_LINE].lstrip(" ").rstrip(" ")
        if not line or line.startswith("#"):
            continue
        cut = line.find(" ")
        if cut < 0:
            return opts, OPTION_FORMAT_ERR
        put_option(opts, line[:cut][:_NAME], line[cut + 1:].rstrip(" ")[:_VALUE])
    return opts, 0


def append_options(filename, options: dict) -> None:
    """append_options (options_utils.F90:360-374): `name value` lines added
    to an existing file."""
    with open(filename, "a") as f:
        for k, v in options.items():
            f.write(f"{k.rstrip()} {v.rstrip()}\n")


def save_options(filename, options: dict, hdr=()) -> None:
    """save_options (options_utils.F90:338-355): header lines prefixed by
    `# `, then the options."""
    with open(filename, "w") as f:
        for h in hdr:
            f.write(f"# {h.rstrip()}\n")
    append_options(filename, options)


def get_command_line_options(argv) -> dict:
    """get_command_line_options (options_utils.F90:381-413): `-name value`
    and bare `-name` arguments.  Restated as the reference runs it: a flag
    that follows a flag still waiting for its value stores that earlier flag
    with an empty value and is itself dropped (`-a -b 1` gives {-a: 1})."""
    options: dict = {}
    name = ""
    for a in argv:
        arg = str(a)[:_VALUE].rstrip(" ")
        if arg.startswith("-"):
            if name:
                put_option(options, name, "")
            else:
                name = arg
        elif name:
            put_option(options, name, arg)
            name = ""
    if name:
        put_option(options, name, "")
    return options


def missing_option_message(option: str) -> str:
    """missing_option_message (options_utils.F90:418-421)."""
    return f"Error: Missing value: {option}"


def invalid_option_message(option: str, value, expected: str) -> str:
    """invalid_option_message (options_utils.F90:426-461): the value written
    as the type's edit descriptor (A, I6, F20.10, L1)."""
    if isinstance(value, (bool, np.bool_)):
        v = "T" if value else "F"
    elif isinstance(value, (int, np.integer)):
        v = _fortran_field(f"{int(value):6d}", 6)
    elif isinstance(value, (float, np.floating)):
        v = _fortran_field(f"{float(value):20.10f}", 20)
    else:
        v = str(value)
    return f"Error: Invalid value: {option} {v} {expected}"


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
