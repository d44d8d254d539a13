"""Checkpoint / restart of a channel.

* save_checkpoint / load_checkpoint: the full device state (phi, u, v, w,
  p, p_old and the AB3 histories, in the phase-independent order the C ABI
  uses; ConvPrevPhi and phi3 for the diffuse-interface method) with the grid,
  the parameters and the step count, in one .npz file.
* backup_channel / dataload_channel: the reference's own text backup
  (io.F90:647-791, the fieldbackup0.dat / fieldbackup1.dat files
  main_ns_hybrid.F90:2450-2468 alternates between), which the reference can
  read back, plus a companion file with the CSF histories it leaves out.

Restarting from either continues bit-identically."""
from __future__ import annotations

import dataclasses
import json

import numpy as np

from .api import Params, TplsGpu


def save_checkpoint(g: TplsGpu, path) -> None:
    st = g.get_state()
    meta = {k: v for k, v in dataclasses.asdict(g.params).items() if k != "extra"}
    np.savez(path, grid=np.array([g.nx, g.ny, g.nz]), u_inlet=g.u_inlet,
             steps_done=np.array(g.stats()["steps_done"]), params=np.array(json.dumps(meta)),
             **{f"f_{k}": v for k, v in st.items()})


def load_checkpoint(path) -> TplsGpu:
    z = np.load(path, allow_pickle=False)
    nx, ny, nz = (int(v) for v in z["grid"])
    meta = json.loads(str(z["params"]))
    g = TplsGpu(nx, ny, nz, Params(**meta), z["u_inlet"])
    g.set_state({k: np.asfortranarray(z[f"f_{k}"]) for k in g.state_fields()})
    g.set_steps_done(int(z["steps_done"]))
    return g


def csf_companion(path) -> str:
    """Name of the CSF-history file written beside a reference backup:
    fieldbackup0.dat -> fieldbackup0_csf.dat."""
    p = str(path)
    return (p[:-4] if p.endswith(".dat") else p) + "_csf.dat"


def backup_channel(g: TplsGpu, path) -> None:
    """Write the reference's backup file `path` and its CSF companion."""
    g.backup_channel(path, csf_companion(path))


def dataload_channel(g: TplsGpu, path, steps_done: int | None = None) -> None:
    """Load a backup written by backup_channel, or by the reference, into a
    context.  The CSF histories come from the companion file when it exists
    (the reference writes none; they are then left as they are).  The
    reference's files carry no step count, so the caller passes it."""
    import os
    csf = csf_companion(path)
    g.dataload_channel(path, csf if os.path.exists(csf) else None)
    if steps_done is not None:
        g.set_steps_done(steps_done)
