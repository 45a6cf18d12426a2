"""GB300 (sm_103a) kernel-polynomial hot path of chenzehan/tight_binding.

The compute lives in libtbk (C ABI in include/tbk.h, CUDA in csrc/); this
package mirrors the reference's model and KPM API on top of it.
"""
from . import capi
from .capi import TbkError, device_count
from .lattice import (Chain, Cubic, FCC, Honeycomb, Kagome, Lieb, PartialLattice, SparseMatrix, Square, TI_sp,
                      UnitCell, commutator, graphene, sawtooth_chain_p, sawtooth_chain_X, stub_1d_p, stub_1d_X)
from .kubo import (bastin_integrate, bastin_zeta, chebyshev_nodes, conductivity_Kubo_Bastin, conductivity_spectrum,
                   generate_V_moments, greenwood_sigma, kubo_last_timing, kubo_mu, kubo_release, mu_from_blocks,
                   conductivity_test_sawtooth)
from .kpm import (Cheb_first_kind_seq_braket, Dirichlet, Fejer, GreenFunction, GreenFunctionImag, Jackson,
                  KpmSolver, Kernel, Lanczos, Lorentz, Wang_and_Zunger, bases_of_uniform_ampl_with_random_phases,
                  density_of_states_function, density_of_states_seq, dos_from_moments, kernel_seq, expn_coef_alpha_seq, trace_braket,
                  trace_braket_complex,
                  spectral_range, cheb_expand, sparse_apply, Cheb_first_kind_seq_view,
                  Cheb_first_kind_seq_on_bases, delta_coefficients, evolution_coefficients,
                  evolution_terms, time_evolve)
from .moments_io import load_moments, output_to_file, save_moments, write_V_moments_text
from .serving import DosServer, request_footprint

__all__ = [n for n in dir() if not n.startswith("_")]
