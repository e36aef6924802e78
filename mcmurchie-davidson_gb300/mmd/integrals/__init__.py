"""Integral modules (GPU): twoe, fock, onee."""
