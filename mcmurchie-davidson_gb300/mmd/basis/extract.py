"""Extract the basis-set data files this package ships (elements H-Ne).

The files are Gaussian94-format exports of the Basis Set Exchange (public data),
read by ``mmd.molecule.Molecule.getBasis`` exactly like the reference's
``mmd/basis/*.gbs``.  This script trims the reference's copies to H-Ne and
derives plain 6-31G (which the reference does not ship) from 6-31G* by dropping
the heavy-atom ``D`` polarisation shell; hydrogen carries no polarisation in
6-31G*, so its entry is unchanged.

Run once where the reference tree is available:
    python mcmurchie-davidson_gb300/mmd/basis/extract.py /root/reference/mmd/basis
"""
import os
import sys

ELEMENTS = {"H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne"}
FILES = ("sto-3g", "sto-6g", "3-21g", "6-31gs", "6-31gss", "6-31ppgss", "dz", "cc-pvdz", "cc-pvtz")


def _blocks(text):
    parts = text.split("****")
    return parts[0], parts[1:-1], parts[-1]


def _symbol(block):
    for line in block.split("\n")[1:]:
        if line.split():
            return line.split()[0]
    return None


def _drop_d(block):
    out, skip = [], 0
    for line in block.split("\n"):
        tok = line.split()
        if skip:
            skip -= 1
            continue
        if tok and tok[0] == "D" and len(tok) >= 2 and tok[1].isdigit():
            skip = int(tok[1])
            continue
        out.append(line)
    return "\n".join(out)


def trim(text, derive_631g=False):
    head, blocks, tail = _blocks(text)
    keep = [b for b in blocks if _symbol(b) in ELEMENTS]
    if derive_631g:
        keep = [_drop_d(b) for b in keep]
        head = head.replace("6-31G*", "6-31G (derived from 6-31G* by dropping D shells)")
    return head + "****" + "****".join(keep) + "****" + tail


def main(src):
    here = os.path.dirname(os.path.abspath(__file__))
    for name in FILES:
        with open(os.path.join(src, name + ".gbs")) as f:
            text = f.read()
        with open(os.path.join(here, name + ".gbs"), "w") as f:
            f.write(trim(text))
    with open(os.path.join(src, "6-31gs.gbs")) as f:
        text = f.read()
    with open(os.path.join(here, "6-31g.gbs"), "w") as f:
        f.write(trim(text, derive_631g=True))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/mmd/basis")
