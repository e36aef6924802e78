"""``Molecule`` -- the reference's user-facing class (mmd/molecule.py), GPU-backed.

Same constructor ``Molecule(geometry, basis='sto-3g')``, same input formats
(geometry string in Angstrom with a ``charge multiplicity`` first line; Gaussian94
basis files), same basis-function order and the same attributes (``bfs``,
``nbasis``, ``nocc``, ``S``, ``T``, ``V``, ``M``, ``Core``, ``X``, ``U``, ``TwoE``,
``screen``, ``nuc_energy`` ...).  Integrals are computed by libmmdg.so on the GPU.
"""
from __future__ import annotations

import itertools
import os
import sys

import numpy as np

from .integrals.shells import shells_from_bfs
from .integrals.twoe import Basis, context_for
from .forces import Forces
from .scf import SCF

ANGSTROM = 0.52917721092  # mmd/molecule.py:224-226


class Atom(object):
    """Class for an atom (mmd/molecule.py:13-22)."""

    def __init__(self, charge, mass, origin=np.zeros(3)):
        self.charge = charge
        self.origin = origin
        self.mass = mass
        self.forces = np.zeros(3)
        self.saved_forces = np.zeros(3)
        self.velocities = np.zeros(3)


SYMBOLS = ["X", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar",
           "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr",
           "Rb", "Sr", "Y", "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In", "Sn", "Sb", "Te", "I", "Xe",
           "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho", "Er", "Tm", "Yb", "Lu",
           "Hf", "Ta", "W", "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po", "At", "Rn"]
# isotope-averaged masses of mmd/molecule.py:205-207 (amu)
MASSES = [0.0, 1.008, 4.003, 6.941, 9.012, 10.812, 12.011, 14.007, 5.999, 18.998, 20.180, 22.990, 24.305, 26.982,
          28.086, 30.974, 32.066, 35.453, 39.948]

SHELLS = {
    "S": [(0, 0, 0)],
    "P": [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
    "D": [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)],
    "F": [(3, 0, 0), (2, 1, 0), (2, 0, 1), (1, 2, 0), (1, 1, 1), (1, 0, 2), (0, 3, 0), (0, 2, 1), (0, 1, 2), (0, 0, 3)],
}

BASIS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis")


def get_basis(filename):
    """Gaussian94 basis parser with the reference's SP splitting (mmd/molecule.py:135-189)."""
    basis = {}
    with open(filename, "r") as basisset:
        data = basisset.read().split("****")
    for i in range(1, len(data)):
        atomData = [x.split() for x in data[i].split("\n")[1:-1]]
        newPrim = True
        for idx, line in enumerate(atomData):
            if not line:
                pass
            elif idx == 0:
                assert len(line) == 2
                atom = SYMBOLS.index(str(line[0]))
                basis[atom] = []
                newPrim = True
            elif idx > 0 and newPrim:
                momentum = line[0]
                numPrims = int(line[1])
                newPrim = False
                count = 0
                prims, prims2 = [], []
            else:
                e = float(line[0].replace("D", "E"))
                if momentum == "SP":
                    prims.append((e, float(line[1].replace("D", "E"))))
                    prims2.append((e, float(line[2].replace("D", "E"))))
                    count += 1
                    if count == numPrims:
                        basis[atom].append(("S", prims))
                        basis[atom].append(("P", prims2))
                        newPrim = True
                else:
                    prims.append((e, float(line[1].replace("D", "E"))))
                    count += 1
                    if count == numPrims:
                        basis[atom].append((momentum, prims))
                        newPrim = True
    return basis


class Molecule(SCF, Forces):
    """Molecule with GPU integrals (mmd/molecule.py:24-315)."""

    @property
    def double_bar(self):
        """Spin-orbital <AB||CD> set up by PostSCF(mol), built on first access."""
        if getattr(self, "_double_bar", None) is None:
            build = getattr(self, "_double_bar_build", None)
            if build is None:
                raise AttributeError("double_bar: run PostSCF(mol) first")
            self._double_bar = build()
        return self._double_bar

    @double_bar.setter
    def double_bar(self, value):
        self._double_bar = value

    @property
    def _forces(self):
        """Forces of every atom, natom x 3 (mmd/molecule.py:47-53)."""
        return np.concatenate([atom.forces for atom in self.atoms]).reshape(-1, 3)

    def __init__(self, geometry, basis="sto-3g"):
        charge, multiplicity, atomlist = self.read_molecule(geometry)
        self.charge = charge
        self.multiplicity = multiplicity
        self.atoms = atomlist
        self.nelec = sum([atom.charge for atom in atomlist]) - charge
        self.nocc = self.nelec // 2
        self.is_built = False
        self.geometry_input = geometry
        basis_file = os.path.join(BASIS_DIR, str(basis).lower() + ".gbs")
        if not os.path.exists(basis_file):
            raise FileNotFoundError(f"basis set '{basis}' not available ({basis_file})")
        self.basis_name = str(basis).lower()
        self.basis_data = self.getBasis(basis_file)
        self.formBasis()

    # ---------------------------------------------------------------- input
    def formBasis(self):
        """Basis functions atom by atom, shell by shell, component by component (molecule.py:57-88)."""
        self.bfs = []
        self.bf_atom = []
        for ia, atom in enumerate(self.atoms):
            if atom.charge not in self.basis_data:
                raise ValueError(f"basis set has no entry for element {SYMBOLS[atom.charge]}")
            for momentum, prims in self.basis_data[atom.charge]:
                exps = [e for e, c in prims]
                coefs = [c for e, c in prims]
                for shell in self.momentum2shell(momentum):
                    self.bfs.append(Basis(np.asarray(atom.origin), np.asarray(shell), len(exps), np.asarray(exps),
                                          np.asarray(coefs)))
                    self.bf_atom.append(ia)
        self.nbasis = len(self.bfs)
        idx = 0
        for atom in self.atoms:
            atom.mask = np.zeros(self.nbasis)
            for momentum, prims in self.basis_data[atom.charge]:
                for shell in self.momentum2shell(momentum):
                    atom.mask[idx] = 1.0
                    idx += 1
        Z = sum([atom.charge for atom in self.atoms])
        self.center_of_charge = np.asarray([sum([atom.charge * atom.origin[k] for atom in self.atoms])
                                            for k in range(3)]) * (1.0 / Z)

    def momentum2shell(self, momentum):
        """Cartesian components of an angular-momentum label, in the reference's
        order (mmd/molecule.py:104-115)."""
        return SHELLS[str(momentum)]

    def sym2num(self, sym):
        """Atomic number of an element symbol (mmd/molecule.py:117-133)."""
        return SYMBOLS.index(str(sym))

    def getBasis(self, filename):
        """Basis-set data of a .gbs file (mmd/molecule.py:135-189)."""
        return get_basis(filename)

    def read_molecule(self, geometry):
        """charge, multiplicity and Angstrom coordinates (molecule.py:191-233)."""
        f = filter(None, geometry.split("\n"))
        atomlist = []
        charge = multiplicity = None
        for line_number, line in enumerate(f):
            if line_number == 0:
                assert len(line.split()) == 2
                charge = int(line.split()[0])
                multiplicity = int(line.split()[1])
            else:
                if len(line.split()) == 0:
                    break
                assert len(line.split()) == 4
                sym = self.sym2num(str(line.split()[0]))
                mass = (MASSES[sym] if sym < len(MASSES) else 0.0) * 1822.8885
                x = float(line.split()[1]) / ANGSTROM
                y = float(line.split()[2]) / ANGSTROM
                z = float(line.split()[3]) / ANGSTROM
                atomlist.append(Atom(charge=sym, mass=mass, origin=np.asarray([x, y, z])))
        return charge, multiplicity, atomlist

    # ---------------------------------------------------------------- integrals
    @property
    def context(self):
        """Device context of this molecule's basis (pairs, Schwarz table).  The lookup
        by basis fingerprint (a pass over every function) runs once per ``bfs`` list;
        later accesses reuse the context while the list is the same object of the same
        length (``formBasis`` makes a new list, hence a new lookup)."""
        bfs = self.bfs
        ref = self.__dict__.get("_context_ref")
        if ref is not None and ref[0] is bfs and ref[1] == len(bfs):
            return ref[2]
        ctx = context_for(bfs)
        self._context_ref = (bfs, len(bfs), ctx)
        return ctx

    def build(self, direct=False):
        """One-electron integrals, then the Schwarz table (direct) or the ERI tensor (molecule.py:90-102)."""
        self.one_electron_integrals()
        # the Schwarz table stays on the device (the SCF's Fock builds screen there);
        # ``screen`` fetches it and builds the reference's dict on first access
        self.__dict__.pop("_screen_dict", None)
        self.__dict__.pop("_screen_array", None)
        if not direct:
            self.two_electron_integrals()
        self.is_built = True

    @property
    def screen(self):
        """The Schwarz dict screen[p(p+1)/2 + q] = (pq|pq) of Molecule.build
        (mmd/molecule.py:95-99), built from the device table on first access."""
        d = self.__dict__.get("_screen_dict")
        if d is None:
            arr = self.__dict__.get("_screen_array")
            if arr is None:
                arr = self.context.screen()
                self._screen_array = arr
            d = {pq: float(v) for pq, v in enumerate(arr)}
            self._screen_dict = d
        return d

    @screen.setter
    def screen(self, value):
        self._screen_dict = value

    def one_electron_integrals(self):
        """S, T, V, dipole integrals on the GPU; Core = T + V; X = S^-1/2, U = S^1/2 (molecule.py:235-286)."""
        ctx = self.context
        torch = ctx.torch
        N = self.nbasis
        dev = f"cuda:{ctx.device}"
        S = torch.empty(N * N, dtype=torch.float64, device=dev)
        T = torch.empty_like(S)
        V = torch.empty_like(S)
        M = torch.empty(3 * N * N, dtype=torch.float64, device=dev)
        nat = len(self.atoms)
        atom_mol = np.zeros(nat, dtype=np.int32)
        xyz = np.ascontiguousarray(np.array([a.origin for a in self.atoms], dtype=np.float64).reshape(-1))
        Zs = np.array([float(a.charge) for a in self.atoms])
        org = np.ascontiguousarray(self.center_of_charge, dtype=np.float64)
        from . import _native
        _native.check(_native.lib().mmdg_one_electron(ctx._h, nat, _native._ptr(atom_mol), _native._ptr(xyz),
                                                       _native._ptr(Zs), _native._ptr(org),
                                                       _native.ctypes.c_void_p(S.data_ptr()),
                                                       _native.ctypes.c_void_p(T.data_ptr()),
                                                       _native.ctypes.c_void_p(V.data_ptr()),
                                                       _native.ctypes.c_void_p(M.data_ptr()), _native.stream_ptr()),
                      "mmdg_one_electron")
        self._dev = {"S": S.view(N, N), "T": T.view(N, N), "V": V.view(N, N), "M": M.view(3, N, N)}
        self.S = self._dev["S"].cpu().numpy()
        self.T = self._dev["T"].cpu().numpy()
        self.V = self._dev["V"].cpu().numpy()
        self.M = self._dev["M"].cpu().numpy()
        self.mu = np.zeros(3, dtype="complex")
        # nuclear repulsion over the atom pairs in itertools.combinations order, summed
        # sequentially (np.add.accumulate) like the reference's loop
        self.nuc_energy = 0.0
        if nat > 1:
            i, j = np.triu_indices(nat, 1)
            R = xyz.reshape(-1, 3)
            d = R[i] - R[j]
            terms = Zs[i] * Zs[j] / np.sqrt(np.einsum("ij,ij->i", d, d))
            self.nuc_energy = float(np.add.accumulate(terms)[-1])
        self.Core = self.T + self.V
        # S^{-1/2} and S^{1/2} by the symmetric eigendecomposition of S on the host cores
        # (LAPACK dsyevd, the SCF's own eigensolver up to ~1000 functions: no dependence
        # on torch's CUDA linear-algebra library); the two products on the GPU
        from .scf import host_eigh
        w, U = host_eigh(self.S)
        Ud = torch.as_tensor(U, device=dev)
        wd = torch.as_tensor(w, device=dev)
        Xd = (Ud * (1.0 / torch.sqrt(wd))) @ Ud.T
        self._dev["X"] = Xd
        self.X = Xd.cpu().numpy()
        self.U = ((Ud * torch.sqrt(wd)) @ Ud.T).cpu().numpy()
        self._dev["Core"] = self._dev["T"] + self._dev["V"]

    def two_electron_integrals(self):
        """Full ERI tensor on the GPU (molecule.py:288-293)."""
        Td = self.context.eri_tensor()
        self._dev["TwoE"] = Td
        self.TwoE = Td.cpu().numpy()

    def save_integrals(self, folder=None):
        """Crawford-format text files (molecule.py:295-315)."""
        if folder is None:
            sys.exit("Please provide a folder to save the integrals.")
        if not self.is_built:
            self.build()
        os.makedirs(folder, exist_ok=True)
        np.savetxt(folder + "/enuc.dat", np.asarray(self.nuc_energy).reshape(1,))
        np.savetxt(folder + "/nbf.dat", np.asarray(self.nbasis, dtype=int).reshape(1,), fmt="%d")
        np.savetxt(folder + "/nelec.dat", np.asarray(self.nelec, dtype=int).reshape(1,), fmt="%d")
        np.savetxt(folder + "/s.dat", self.S)
        np.savetxt(folder + "/t.dat", self.T)
        np.savetxt(folder + "/v.dat", self.V)
        with open(folder + "/eri.dat", "w") as f:
            for i, j, k, l in itertools.product(range(self.nbasis), repeat=4):
                print(i + 1, j + 1, k + 1, l + 1, self.TwoE[i, j, k, l], file=f)
        with open(folder + "/geometry.txt", "w") as f:
            print(self.geometry_input, file=f)
