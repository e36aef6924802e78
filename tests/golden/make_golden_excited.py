#!/usr/bin/env python3
"""Golden CIS and TDHF excitation energies from the reference's own
``mmd.postscf.PostSCF`` (make_golden.py's shimmed, compiled copy; ``bitstring``, which
only the determinant-based paths use, is replaced by a stand-in module).

Conventional RHF at conver 1e-12, then CIS (water / 3-21G: energies and oscillator
strengths) and TDHF (water / STO-3G, the 'hermitian', 'reduced' and 'full'
algorithms): ``excited.json``.
"""
from __future__ import annotations

import json
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402


def main():
    MG._prepare_reference()
    sys.modules.setdefault("bitstring", types.SimpleNamespace(BitArray=None))
    from mmd.molecule import Molecule
    from mmd.postscf import PostSCF
    out = {"source": "reference mmd/postscf.py CIS/TDHF after RHF(conver=1e-12)"}
    mol = Molecule(geometry=MG.WATER, basis="3-21g")
    mol.RHF(doPrint=False, conver=1e-12)
    PostSCF(mol).CIS()
    out["cis"] = {"geometry": MG.WATER, "basis": "3-21g", "omega": [float(x) for x in mol.cis_omega],
                  "oscil": [float(x) for x in mol.cis_oscil]}
    mol = Molecule(geometry=MG.WATER, basis="sto-3g")
    mol.RHF(doPrint=False, conver=1e-12)
    out["tdhf"] = {"geometry": MG.WATER, "basis": "sto-3g"}
    for alg in ("hermitian", "reduced", "full"):
        PostSCF(mol).TDHF(alg=alg)
        out["tdhf"][alg] = [float(x) for x in mol.tdhf_omega]
    with open(os.path.join(HERE, "excited.json"), "w") as f:
        json.dump(out, f, indent=1)
    print({k: (v["omega"][:4] if k == "cis" else v["hermitian"][:4]) for k, v in out.items() if k != "source"})


if __name__ == "__main__":
    main()
