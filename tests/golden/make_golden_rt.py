#!/usr/bin/env python3
"""Golden RT-TDHF trajectories from the reference's own ``mmd.realtime.RealTime``.

Runs where the reference tree is present (it reuses make_golden.py's shimmed,
compiled copy of the reference package).  For H2 / STO-3G and water / STO-3G it
runs Magnus2 and Magnus4 with a Gaussian pulse (envelope exp(-(t - 1)^2 / 0.5^2),
field 1e-3, 40 steps of 0.1 atomic time units, z and x directions) and stores the
dipole, energy and pulse-shape records: ``rt_trajectories.npz``.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402

STEPS, DT, FIELD = 40, 0.1, 1e-3


def pulse(t):
    return np.exp(-((t - 1.0) ** 2) / 0.25)


def main():
    MG._prepare_reference()
    from mmd.molecule import Molecule
    from mmd.realtime import RealTime
    out = {}
    for name, geom in (("h2", MG.H2), ("water", MG.WATER)):
        for order, direction in ((2, "z"), (4, "z"), (4, "x")):
            mol = Molecule(geometry=geom, basis="sto-3g")
            rt = RealTime(mol, numsteps=STEPS, stepsize=DT, field=FIELD, pulse=pulse)
            getattr(rt, f"Magnus{order}")(direction=direction)
            key = f"{name}_m{order}{direction}"
            out[key + "_dipole"] = np.array(rt.dipole, dtype=float)
            out[key + "_energy"] = np.array(rt.Energy, dtype=float)
            out[key + "_shape"] = np.array(rt.shape, dtype=float)
            print(key, out[key + "_energy"][[0, -1]], out[key + "_dipole"][[0, -1]])
    np.savez_compressed(os.path.join(HERE, "rt_trajectories.npz"), steps=STEPS, dt=DT, field=FIELD, **out)


if __name__ == "__main__":
    main()
