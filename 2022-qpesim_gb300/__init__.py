"""qpesim_gb300: GB300-native (sm_103a) implementation of qpe-sim's hot path.

The controlled, Trotterized time evolution of a fixed-electron-count state
vector and the batched inverse QFT over the ancilla axis, behind the
reference's interfaces (Hamiltonian, StateVector, OffsetComputer,
time_evolve_over_terms). All compute runs in lib/libqpe_gb300.so (C ABI in
include/); there is no CPU fallback.

The directory is named 2022-qpesim_gb300, which is not an importable module
name; __graft_entry__.load_package() registers it as `qpesim_gb300`.
"""
from . import _native
from . import learned_state
from .batching import Batch
from .hamiltonian import Hamiltonian, SpinIndex
from .offset_computer import OffsetComputer
from .readout import (argmax_phase, margin_of_error, phase_to_energy, reference_energy, reference_phase,
                      subbin_phase, success_probability)
from .state_vector import StateVector
from .synthetic import Integrals, hf_block0, synthetic_integrals
from .time_evolution import DeviceState, Program, plan_program, time_evolve_iqpe, time_evolve_over_terms

QpeError = _native.QpeError
TERM_DTYPE = _native.TERM_DTYPE
LIB_PATH = _native.LIB_PATH

__all__ = ["Batch", "Hamiltonian", "SpinIndex", "OffsetComputer", "StateVector", "time_evolve_over_terms",
           "time_evolve_iqpe", "Program",
           "DeviceState", "plan_program", "Integrals", "synthetic_integrals", "hf_block0", "QpeError", "TERM_DTYPE",
           "reference_phase", "reference_energy", "margin_of_error", "phase_to_energy", "argmax_phase",
           "subbin_phase", "success_probability"]
