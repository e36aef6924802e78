#!/usr/bin/env python3
"""Golden RHF nuclear forces from the reference's own ``Molecule.forces`` (its
Cython derivative integrals, cython/grad.pyx, compiled by make_golden.py's recipe).

Conventional RHF at conver 1e-12 (forces are first order in the density error),
then ``mol.forces()``: ``forces.json`` with each case's geometry, basis, energy and
natom x 3 forces.
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402

WATER_BENT = """
0 1
O    0.000000      -0.070000     0.010000
H    0.800000       0.620000     0.030000
H   -0.880000       0.560000    -0.020000
"""
CASES = [("h2", MG.H2, "sto-3g"), ("water", MG.WATER, "sto-3g"), ("water_distorted", WATER_BENT, "sto-3g"),
         ("water_distorted", WATER_BENT, "3-21g"), ("methane", MG.METHANE, "sto-3g"),
         ("formaldehyde", MG.FORMALDEHYDE, "sto-3g"), ("water_distorted", WATER_BENT, "6-31g"),
         ("water_distorted", WATER_BENT, "6-31gs")]


def main():
    MG._prepare_reference()
    from mmd.molecule import Molecule
    out = []
    for name, geom, basis in CASES:
        t0 = time.time()
        mol = Molecule(geometry=geom, basis=basis)
        mol.RHF(doPrint=False, conver=1e-12)
        mol.forces()
        f = mol._forces
        out.append({"name": name, "basis": basis, "geometry": geom, "energy": float(mol.energy.real),
                    "forces": [[float(x) for x in row] for row in f]})
        print(name, basis, f"{time.time() - t0:.1f}s", f.round(8).tolist(), flush=True)
        with open(os.path.join(HERE, "forces.json"), "w") as fh:
            json.dump({"source": "reference Molecule.forces (mmd/forces.py) after RHF(conver=1e-12)", "cases": out},
                      fh, indent=1)


if __name__ == "__main__":
    main()
