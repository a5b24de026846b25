"""GB300-native XRD-tomography forward projector (drop-in for Forward_XRD).

The compute runs in libxrdt.so (CUDA, sm_103a) behind the C ABI declared in
include/xrdt.h; this package is its Python front end.
"""
from .problem import Problem, QUIRK_STALE_VOXEL_A, reference_problem  # noqa: F401
from .api import (Batch, BasisOperator, Context, Forward_XRD, Operator, XrdtError, basis_expand, ct_sinogram, forward,  # noqa: F401
                  forward_rays, forward_tables, lib, mlem_matrix, spectrum_build, debug_decisions,
                  mlem_matrix_noalloc, mlem_checkpoint_write, mlem_checkpoint_read, validate,
                  c_reference_problem, FWD_PLAIN_FP64, FWD_NO_SYNC, TAB_BILINEAR)
