"""View-sharded projection and MLEM over several ranks, one GPU per rank.

The forward model's rays are independent, and the rays of one source
position (view) share nothing with those of another but the unknowns.  So
rank r of R takes the views [s0, s1) of view_range(): its problem is the
scanner with those views only (view_shard_problem), its rays are the
full problem's rays of those views (shard_rays), and its projection needs no
exchange at all.  MLEM (main.m:154-176) needs one exchange per iteration:
the back-projection A^T (y / (A x + c)) is a sum over rays, so every rank
back-projects its own rays and the ranks add their [NX*NY*NWT] results with
one all-reduce; the sensitivity A^T 1 is all-reduced once.  Every rank then
applies the same update to its copy of the estimate.  With more ranks than
views some ranks hold no views: they have no operator and add zeros to the
all-reduces, so the collective sequence is the same on every rank.

The reference has no distributed code (one GPU driven by MATLAB); this
split follows from the structure of its ray loop (integrate_diffraction.cu
launches one independent block per ray).
"""
from __future__ import annotations

import numpy as np

from .problem import Problem


def view_range(n_src: int, rank: int, world: int) -> tuple[int, int]:
    """Views [s0, s1) of rank `rank`: contiguous, sizes differing by one at
    most (empty, s0 == s1, for the last ranks when world > n_src)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(n_src, world)
    s0 = rank * base + min(rank, extra)
    return s0, s0 + base + (1 if rank < extra else 0)


def view_shard_problem(p: Problem, s0: int, s1: int) -> Problem:
    """The scanner with views s0 .. s1-1 only.  Source j of the shard sits at
    angle (s0 + j) / SRC * arc + phi0 (integrate_diffraction.cu:93): the same
    positions, written as a problem of s1 - s0 sources over the arc
    arc * (s1 - s0) / SRC from phi0 + s0 / SRC * arc."""
    if not 0 <= s0 < s1 <= p.n_src:
        raise ValueError("bad view range")
    q = p.copy()
    q.n_src = s1 - s0
    q.src_arc = p.src_arc * (s1 - s0) / p.n_src
    q.src_phi0 = p.src_phi0 + p.src_arc * s0 / p.n_src
    return q


def shard_rays(p: Problem, s0: int, s1: int) -> np.ndarray:
    """Indices into the full problem's ray vectors (src + det*SRC +
    nrg*SRC*DET) of the shard's rays, in the shard problem's own ray order."""
    det = p.n_col * p.n_row
    ns = s1 - s0
    src = np.arange(ns)[:, None, None]
    d = np.arange(det)[None, :, None]
    e = np.arange(p.nrg_det)[None, None, :]
    # shard order: j + d*ns + e*ns*det, j fastest
    idx = (s0 + src) + d * p.n_src + e * p.n_src * det
    return np.ascontiguousarray(idx.transpose(2, 1, 0).reshape(-1), np.int64)


class ShardedMLEM:
    """MLEM of main.m:162-176 over ranks that each hold some rays.

    forward(x) -> A_r x (this rank's rays), adjoint(w) -> A_r^T w (all the
    unknowns), all_reduce(t) sums a tensor over the ranks in place (e.g.
    torch.distributed.all_reduce).  x, y and c are torch tensors; the update
    is formed in FP64.  A rank without rays passes forward = adjoint = None
    and empty y and c: it back-projects zeros and still joins every
    all-reduce."""

    def __init__(self, forward, adjoint, all_reduce):
        self.forward = forward
        self.adjoint = adjoint
        self.all_reduce = all_reduce
        self.sens = None

    def _back(self, w, x):
        import torch
        if self.adjoint is None:
            return torch.zeros(x.numel(), dtype=torch.float64, device=x.device)
        return self.adjoint(w).double()

    def sensitivity(self, n_rays_local, like, x):
        if self.sens is None:
            import torch
            ones = torch.ones(n_rays_local, dtype=like.dtype, device=like.device)
            s = self._back(ones, x)
            self.all_reduce(s)
            self.sens = s
        return self.sens

    def run(self, y, c, x, iters: int):
        import torch
        if (self.forward is None) != (self.adjoint is None) or (self.forward is None and y.numel()):
            raise ValueError("a rank without an operator holds no rays: forward, adjoint, y and c all empty")
        s = self.sensitivity(y.numel(), y, x)
        for _ in range(iters):
            if self.forward is None:
                ax = torch.zeros(0, dtype=torch.float64, device=x.device)
            else:
                ax = self.forward(x).double()
            r = (y.double() / (ax + c.double() + 1e-20)).to(y.dtype)
            g = self._back(r, x)
            self.all_reduce(g)
            xn = x.double() * g / (s + 1e-7)
            xn[~torch.isfinite(xn)] = 0.0          # main.m:163
            xn.clamp_(min=0.0)                      # main.m:176
            x.copy_(xn.to(x.dtype))
        return x


def operator_shard(p: Problem, spectrum, seg, a1, a2, rank: int, world: int, ctx=None):
    """This rank's per-voxel operator (views view_range(p.n_src, rank, world))
    and the indices of its rays in the full problem's ray vectors; (None, no
    rays) for a rank without views."""
    from .api import Operator
    s0, s1 = view_range(p.n_src, rank, world)
    if s0 == s1:
        return None, np.empty(0, np.int64)
    op = Operator(view_shard_problem(p, s0, s1), spectrum, seg, a1, a2, ctx=ctx)
    return op, shard_rays(p, s0, s1)
