"""GB300 (sm_103a) two-site DMRG path of chemtensor_mojo.

The compute lives in ``libctdmrg.so`` (hand-written CUDA for sm_103a behind a
plain C ABI, ``include/ctdmrg.h``); this package is the thin host layer that
mirrors the reference's Mojo API (``src/m_tensor``, ``src/state``,
``src/algorithms``) on top of it.  There is no CPU fallback: calls fail when
the library or a CUDA device is missing.
"""
from ._lib import CTDMRGError, load as load_library  # noqa: F401
from .dense_tensor import (DenseTensor, DeviceContext, create_dense_tensor, create_dense_tensor_from_data,  # noqa
                           create_dense_tensor_random, create_dense_tensor_uninitialized, dense_tensor_dot,
                           dense_tensor_qr, dense_tensor_svd_trunc, get_context)
from .mps_state import (MatrixProductOperator, MatrixProductState, MPOSite, MPSSite, create_identity_mpo,  # noqa
                        create_product_mps, create_random_mps_c_compatible, create_single_site_op_mpo,
                        create_two_site_op_mpo, create_uniform_mps, mpo_from_arrays, mps_from_arrays, mps_norm,
                        mps_local_orthonormalize_qr, mps_orthogonalize_qr, mps_right_normalize,
                        mps_to_statevector, random_mps_c_compatible_arrays)
from .hamiltonians import (create_bose_hubbard_mpo, create_fermi_hubbard_mpo, create_heisenberg_mpo,  # noqa
                           create_heisenberg_xxz_mpo, create_ising_1d_mpo, create_spin_half_xxz_mpo,
                           create_transverse_ising_mpo)
from .environments import (apply_mpo, build_right_environments, expectation_value,  # noqa
                           expectation_value_normalized, expectation_value_two_mps, mpo_compose, mps_overlap,
                           mps_vdot_direct, update_left_environment, update_left_environment_two_mps,
                           update_right_environment, variance)
from . import dmrg_utils  # noqa: F401
from .results import (DMRGJsonParams, DMRGReference, dmrg_results_to_json_string, load_dmrg_reference,  # noqa
                      mps_bond_entropies, mps_schmidt_values, print_dmrg_reference_info, save_dmrg_results_to_json)
from .dmrg import (DMRGParams, DMRGStats, DMRGWorkspace, apply_two_site_heff, build_two_site_theta,  # noqa
                   dmrg_local_update_two_site, dmrg_two_site, lanczos_two_site_optimize, split_two_site_theta_svd)

__version__ = "0.1.0"
