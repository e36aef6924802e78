"""GB300-native drop-in for the two-electron hot path of McMurchie-Davidson (``mmd``).

Same module layout as the reference package: ``mmd.molecule.Molecule``,
``mmd.scf.SCF``, ``mmd.integrals.twoe`` (``Basis``, ``ERI``, ``doERIs``),
``mmd.integrals.fock`` (``formPT``) and ``mmd.integrals.onee``.  The electron
repulsion integrals, the Fock digestion, the Schwarz table and the one-electron
integrals run in the sm_103a kernels of ``mmd/_lib/libmmdg.so``.
"""
