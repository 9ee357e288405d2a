"""gbpowspec -- GB300-native power-spectrum multipoles (drop-in for jax-powspec's P(k) path).

Reference-compatible entry points (same signatures as dforero0896/jax-powspec):
    gbpowspec.mas.cic_mas_vec, gbpowspec.mas.cic_mas                (src/mas.py)
    gbpowspec.correlations.powspec_vec, ...powspec_vec_fundamental  (src/correlations.py)

Production entry points:
    mesh_deposit       NGP/CIC/TSC/PCS deposit, optional interlacing
    PowerSpectrum      resident deposit -> FFT -> binning pipeline
    power_multipoles   one-shot P_0,2,4(k) of a catalogue

All compute runs in libgbpowspec.so (CUDA, sm_103a); there is no CPU path.
"""
from ._lib import GbpError, DepositStats, load as load_library
from ._native import read_stats
from .mas import cic_mas, cic_mas_vec, mesh_deposit
from .correlations import (powspec_vec, powspec_vec_fundamental, xi_vec, compute_2pt_correlations, bispec, bispectrum,
                           compute_all_correlations, default_kedges)
from .pipeline import PkConfig, PkResult, PowerSpectrum, power_multipoles, algorithmic_bytes
from .grad import power_multipoles_diff

__all__ = [
    "GbpError", "DepositStats", "load_library", "read_stats",
    "cic_mas", "cic_mas_vec", "mesh_deposit",
    "powspec_vec", "powspec_vec_fundamental", "xi_vec", "compute_2pt_correlations", "bispec", "bispectrum", "compute_all_correlations",
    "default_kedges",
    "PkConfig", "PkResult", "PowerSpectrum", "power_multipoles", "algorithmic_bytes", "power_multipoles_diff",
]
