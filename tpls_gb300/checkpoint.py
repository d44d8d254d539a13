"""Checkpoint / restart of a channel: the full device state (phi, u, v, w,
p, p_old and the AB3 histories, in the phase-independent order the C ABI
uses; ConvPrevPhi and phi3 for the diffuse-interface method) with the grid
and parameters, in one .npz file.  Restarting from a checkpoint continues
bit-identically."""
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
    return g
