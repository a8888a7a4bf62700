"""pytreenet_gb300 -- GB300 engine for PyTreeNet's TDVP local-update hot path.

Drop-in surface for the path (names as in PyTreeNet):
TreeTensorNetworkState/TTNS, TreeTensorNetworkOperator/TTNO, Node,
FirstOrderOneSiteTDVP, SecondOrderOneSiteTDVP, FirstOrderTwoSiteTDVP,
SecondOrderTwoSiteTDVP, TDVPConfig, TwoSiteTDVPConfig, SVDParameters, TEBD,
TrotterStep, TrotterSplitting, TimeEvoMode, EvoDirection, TensorProduct; plus
gradients through a hand-written adjoint (OneSiteTDVPAdjoint,
coupling_gradient), the BUG integrators (FixedBUG, rank-adaptive BUG) and
time-dependent TTNOs. Numerics run in libptn_gb300.so
(hand-written CUDA for sm_103a) through a C ABI; see include/ptn_gb300.h.
"""
from .ttn import Node, TreeTensorNetworkState, TreeTensorNetworkOperator, TTNS, TTNO
from .tdvp import (TimeEvoMode, EvoDirection, PathFinderMode, TDVPConfig, TensorProduct,
                   FirstOrderOneSiteTDVP, SecondOrderOneSiteTDVP, leaf_to_root_update_path,
                   TwoSiteTDVPConfig, FirstOrderTwoSiteTDVP, SecondOrderTwoSiteTDVP)
from .truncation import SVDParameters, truncate_singular_values
from .tebd import TEBD, TrotterStep, TrotterSplitting, NumericOperator, SWAPlist, swap_gate
from .operators import nearest_neighbour_ttno, tfim_ttno, heisenberg_ttno
from .hamiltonian import Hamiltonian
from .exact import ExactTimeEvolution, ExactTimeEvolutionConfig
from .application import ApplicationMethod, apply_ttno_to_ttns
from .svd_truncation import SplitMode, TruncationMethod, apply_and_truncate, svd_truncation
from .batch import run_realisations
from .contractions import (SandwichCache, contract_ket_ham_with_envs, contract_any,
                           effective_single_site_evolution, get_effective_single_site_hamiltonian,
                           get_effective_single_site_hamiltonian_nodes, PartialTreeCachDict,
                           contract_bond_tensor, effective_bond_evolution, bond_time_evolution,
                           single_site_time_evolution, get_effective_bond_hamiltonian,
                           get_effective_bond_hamiltonian_nodes, get_effective_bond_hamiltonian_tensor)
from .adjoint import OneSiteTDVPAdjoint, coupling_gradient
from .bug import BUG, BUGConfig, FixedBUG, FixedBUGConfig
from .time_dep import AbstractTimeDepTTNO, TimeDependentTTNO, FactorUpdatable, DiscreetTimeTTNO
from .tdvp import OneSiteTDVP, TwoSiteTDVP, TTNTimeEvolutionConfig
from .results import Results
from .ttno_decomposition import Decomposition
from .application import zipup
from .local_evolution import krylov_exp_action, time_evolve
from .functions import (TDVPUpdatePathFinder, bosonic_operators, canonical_form, completely_contract_tree,
                        contract_two_ttns, expectation_value, hadamard, multi_single_site_expectation_value,
                        pauli_matrices, spin_jumps)

__all__ = [
    "Node", "TreeTensorNetworkState", "TreeTensorNetworkOperator", "TTNS", "TTNO",
    "TimeEvoMode", "EvoDirection", "PathFinderMode", "TDVPConfig", "TensorProduct",
    "FirstOrderOneSiteTDVP", "SecondOrderOneSiteTDVP", "leaf_to_root_update_path",
    "TwoSiteTDVPConfig", "FirstOrderTwoSiteTDVP", "SecondOrderTwoSiteTDVP",
    "SVDParameters", "truncate_singular_values", "TEBD", "TrotterStep", "TrotterSplitting",
    "NumericOperator", "SWAPlist", "swap_gate",
    "nearest_neighbour_ttno", "tfim_ttno", "heisenberg_ttno", "run_realisations", "Hamiltonian",
    "ExactTimeEvolution", "ExactTimeEvolutionConfig", "ApplicationMethod", "apply_ttno_to_ttns",
    "SplitMode", "TruncationMethod", "apply_and_truncate", "svd_truncation",
    "SandwichCache", "contract_ket_ham_with_envs", "contract_any", "effective_single_site_evolution",
    "get_effective_single_site_hamiltonian", "get_effective_single_site_hamiltonian_nodes",
    "OneSiteTDVPAdjoint", "coupling_gradient", "FixedBUG", "FixedBUGConfig", "BUG", "BUGConfig",
    "AbstractTimeDepTTNO", "TimeDependentTTNO", "FactorUpdatable", "DiscreetTimeTTNO",
    "OneSiteTDVP", "TwoSiteTDVP", "TTNTimeEvolutionConfig", "Results", "zipup",
    "krylov_exp_action", "time_evolve", "TDVPUpdatePathFinder", "bosonic_operators", "canonical_form",
    "completely_contract_tree", "contract_two_ttns", "expectation_value", "hadamard",
    "multi_single_site_expectation_value", "pauli_matrices", "spin_jumps",
    "PartialTreeCachDict", "contract_bond_tensor", "effective_bond_evolution", "bond_time_evolution",
    "single_site_time_evolution", "get_effective_bond_hamiltonian", "get_effective_bond_hamiltonian_nodes",
    "get_effective_bond_hamiltonian_tensor", "Decomposition",
]
