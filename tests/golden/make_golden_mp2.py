#!/usr/bin/env python3
"""Golden MP2 energies from the reference's own ``mmd.postscf.PostSCF``.

Runs where the reference tree is present (make_golden.py's shimmed, compiled copy).
The reference module imports ``bitstring`` for its CI methods; MP2 does not use it,
so a stand-in module is registered before the import.  Conventional RHF at
conver 1e-12, then MP2 (spatial and spin-orbital): ``mp2.json``.
"""
from __future__ import annotations

import json
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402

CASES = [("water", MG.WATER, "sto-3g"), ("water", MG.WATER, "6-31g"), ("methane", MG.METHANE, "3-21g"),
         ("h2", MG.H2, "cc-pvdz")]


def main():
    MG._prepare_reference()
    sys.modules.setdefault("bitstring", types.SimpleNamespace(BitArray=None))
    from mmd.molecule import Molecule
    from mmd.postscf import PostSCF
    out = []
    for name, geom, basis in CASES:
        mol = Molecule(geometry=geom, basis=basis)
        mol.RHF(doPrint=False, conver=1e-12)
        PostSCF(mol).MP2()
        spatial = float(mol.emp2.real)
        PostSCF(mol).MP2(spin_orbital=True)
        spin = float(mol.emp2.real)
        out.append({"name": name, "basis": basis, "geometry": geom, "energy": float(mol.energy.real),
                    "emp2_spatial": spatial, "emp2_spin": spin})
        print(name, basis, out[-1]["energy"], spatial, spin)
    with open(os.path.join(HERE, "mp2.json"), "w") as f:
        json.dump({"source": "reference mmd/postscf.py MP2 after RHF(conver=1e-12)", "cases": out}, f, indent=1)


if __name__ == "__main__":
    main()
