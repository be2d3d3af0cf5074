"""GB300-native DISCO-EB perturbation hot path (import name ``discoeb_gb300``).

Drop-in for ``discoeb.perturbations.evolve_perturbations`` / ``get_power``
(src/discoeb/perturbations.py:926-997, 1101-1123): the k-mode integration
runs in hand-written sm_103a CUDA behind the C ABI of
``include/discoeb_gb300.h``; :mod:`background` / :mod:`recfast` produce the
FP64 input tables on the host.
"""
from .perturbations import (evolve_perturbations, evolve_perturbations_batched, evolve_perturbations_multi,
                            get_power, nvar, solve, DeviceProblem)
from .background import evolve_background, get_neutrino_momentum_bins
from .gradient import PowerSpectrum, THETA, evolve_perturbations_grad, fisher_matrix, loglike_grad
from .tables_gpu import evolve_background_tables, evolve_background_tables_host

__all__ = ["evolve_perturbations", "evolve_perturbations_batched", "evolve_perturbations_multi", "get_power", "nvar",
           "solve", "DeviceProblem", "evolve_background", "get_neutrino_momentum_bins", "evolve_perturbations_grad",
           "fisher_matrix", "PowerSpectrum", "THETA", "evolve_background_tables", "evolve_background_tables_host",
           "loglike_grad"]
