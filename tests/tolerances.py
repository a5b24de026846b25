"""Error measures and tolerances of the parity tests.

FAST_RTOL: the factored FP32 projector against the FP64 oracle.  A count is
compared element by element where it is above FLOOR times the largest count
of its array; below that floor it is compared against FLOOR*max (absolute),
since a count 1e-6 times smaller than its neighbours carries no information
at FP32 accumulation.
PLAIN_RTOL: the FP64 kernel at the reference's launch shape, whose outputs are
rounded to float once.
MLEM_RTOL: an MLEM estimate after up to 50 iterations against the same
iterations in FP64, element by element above MLEM_FLOOR times the largest
entry (below it against that floor).
"""
import numpy as np

FAST_RTOL = 1e-5
PLAIN_RTOL = 1e-6
FLOOR = 1e-6
MLEM_RTOL = 1e-5
MLEM_FLOOR = 1e-4


def max_rel_err(got, ref, floor=FLOOR):
    got = np.asarray(got, np.float64).ravel()
    ref = np.asarray(ref, np.float64).ravel()
    scale = np.abs(ref).max() if ref.size else 0.0
    if scale == 0.0:
        return float(np.abs(got).max()) if got.size else 0.0
    den = np.maximum(np.abs(ref), floor * scale)
    diff = np.abs(got - ref)
    err = np.where(den > 0, diff / np.where(den > 0, den, 1.0), diff)
    return float(err.max())
