"""Snapshots and restart: the reference's checkpoint layout
(dedalus/time_stepping/time_step.py:112-151, dedalus/utils/restart.py:33-99)
without h5py and pickle.

A snapshot is a directory ``snap_%05i`` holding
* ``data.cpu0000.npz``: every field component under ``fields/<name>/<comp>``
  in its current space, the space under ``fields/<name>/<comp>@space``, the
  time under ``time`` and the library version under ``@version`` -- the
  HDF5 hierarchy ``/fields/<name>/<comp>`` (attribute ``space``) and
  ``/time`` of the reference's ``data.cpu%04i``;
* ``dedalus_obj_0000.json``: what the reference pickles -- the physics class,
  shape, box and parameters, and the integrator's class, settings and
  counters;
* ``forcing_functions.py``: the forcing sidecar (empty: forcing is not in the
  CUDA path).

``restart(snap_dir)`` returns ``(RHS, data, ti)`` as the reference does.
"""
import json
import os
import time as _time

import numpy as np

from . import _lib

SNAP_DIR = "snap_%05i"
DATA_FILENAME = "data.cpu%04i.npz"
OBJECT_FILENAME = "dedalus_obj_%04i.json"
_TI_STATE = ("CFL", "int_factor", "time", "iteration", "dt_old", "_nsnap", "_tlastsnap", "save_cadence",
             "max_save_period", "stop_iteration", "sim_stop_time", "wall_stop_time", "wall_advance", "use_fused")


def _plain(v):
    """JSON form of a parameter value, or a marker for what JSON cannot hold."""
    if isinstance(v, (np.generic,)):
        v = v.item()
    if v is None or isinstance(v, (bool, int, float, str)):
        return v
    if isinstance(v, (list, tuple)):
        return [_plain(x) for x in v]
    return {"__unsaved__": type(v).__name__}


def save(path, RHS, data, ti, proc=0):
    """Write the snapshot files of (RHS, data, ti) into directory path."""
    os.makedirs(path, exist_ok=True)
    arrays = {"time": np.float64(data.time), "@version": np.array("dedalus_gb300 %d" % _lib.lib().dd_version())}
    for name, field in data:
        for i, c in field:
            key = "fields/%s/%d" % (name, i)
            arrays[key] = c.data.detach().cpu().numpy()
            arrays[key + "@space"] = np.array(c._curr_space)
    np.savez(os.path.join(path, DATA_FILENAME % proc), **arrays)
    obj = {"physics": {"class": type(RHS).__name__, "shape": [int(n) for n in RHS.shape],
                       "length": [float(l) for l in RHS.length],
                       "parameters": {k: _plain(v) for k, v in RHS.parameters.items()},
                       "fields": [[n, type(f).__name__] for n, f in data]},
           "integrator": {"class": type(ti).__name__, **{k: _plain(getattr(ti, k)) for k in _TI_STATE
                                                          if hasattr(ti, k)}}}
    with open(os.path.join(path, OBJECT_FILENAME % proc), "w") as f:
        json.dump(obj, f, indent=1)
    with open(os.path.join(path, "forcing_functions.py"), "w"):
        pass


def load_all_data(data, filename):
    """Load every field component of data from a snapshot data file
    (utils/restart.py:76-99): each component is set in the space it was saved in."""
    z = np.load(filename)
    for name, field in data:
        for i, c in field:
            key = "fields/%s/%d" % (name, i)
            if key not in z.files:
                raise KeyError("Data File field %s component %i is missing or corrupt" % (name, i))
            c[str(z[key + "@space"])] = z[key]
    data.set_time(float(z["time"]))


def restart(snap_dir, proc=0, **physics_kwargs):
    """Rebuild (RHS, data, ti) from a snapshot directory (utils/restart.py:33-74).
    physics_kwargs go to the physics constructor (e.g. closure= for LESHydro,
    whose network is not part of the snapshot)."""
    from . import mods
    with open(os.path.join(snap_dir, OBJECT_FILENAME % proc)) as f:
        obj = json.load(f)
    ph = obj["physics"]
    RHS = getattr(mods, ph["class"])(tuple(ph["shape"]), mods.FourierRepresentation, length=tuple(ph["length"]),
                                     **physics_kwargs)
    for k, v in ph["parameters"].items():
        if not (isinstance(v, dict) and "__unsaved__" in v):
            RHS.parameters[k] = tuple(v) if isinstance(v, list) else v
    z = np.load(os.path.join(snap_dir, DATA_FILENAME % proc))
    data = RHS.create_fields(float(z["time"]))
    load_all_data(data, os.path.join(snap_dir, DATA_FILENAME % proc))
    it = obj["integrator"]
    ti = getattr(mods, it["class"])(RHS, CFL=it.get("CFL", 0.1), int_factor=it.get("int_factor"))
    for k in _TI_STATE:
        if k in it and k not in ("CFL", "int_factor"):
            setattr(ti, k, it[k])
    ti._start_time = _time.time()
    return RHS, data, ti
