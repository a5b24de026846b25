"""FP64 restatement of the spectrum-response builder (spectrum_builder.m:64-95).

TEST INFRASTRUCTURE ONLY: the checker of the CUDA builder (xrdt_spectrum_build).
Only the tests and the smoke check use it.

Inputs: a fine source spectrum given by its bin edges e_hd [H+1] (keV) and
photons per keV n_hd [H] (spectrum_builder.m:22-30), and coarse source and
detector bin edges.  The detector response of fine source bin h is a
Gaussian of width sigma(E_h) = sigma0 + sigma1 E_h (spectrum_builder.m:65:
0.5 (1.61 + 0.025 E), i.e. sigma0 = 0.805, sigma1 = 0.0125) over the fine bin
centres E_g (:70, the detector axis is the source axis transposed):

  X[h, g] = n_hd[h] exp(-(E_h - E_g)^2 / (2 sigma_h^2)) / sqrt(2 pi) / sigma_h   (:75)

and the response is the double integral of X over the rectangle of coarse
source bin s and coarse detector bin d, with the overlap lengths of the fine
bins with the coarse ones as weights (:86-91):

  Ndet[s, d] = sum_h sum_g ws[h, s] wd[g, d] X[h, g],
  ws[h, s] = max(0, min(Es2, Eright_h) - max(Es1, Eleft_h))                       (:87)

The reference uses one grid for source and detector; separate grids are the
same formula.  Output layout as the projector reads its spectrum
(Forward_XRD.cu prhs[0]): column-major [NS, ND], element (s, d) at s + d*NS.

Parity unpinned: the reference's builder is MATLAB (gpuArray), absent here,
and ships no outputs.  The restatement is checked against its own literal
loop form (response_loops, the shape of spectrum_builder.m:77-95) and against
photon conservation for source bins away from the ends of the fine grid.
"""
import math

import numpy as np

SIGMA0 = 0.5 * 1.61     # spectrum_builder.m:65
SIGMA1 = 0.5 * 0.025


def _fine(e_hd, n_hd, sigma0, sigma1):
    e = np.asarray(e_hd, np.float64)
    left, right = e[:-1], e[1:]
    ec = 0.5 * (left + right)                                        # :26
    sig = sigma0 + sigma1 * ec                                       # :65
    return left, right, ec, sig, np.asarray(n_hd, np.float64)


def _overlap(left, right, edges):
    """[H, nbins] overlap lengths of the fine bins with the coarse bins (:87-88)."""
    edges = np.asarray(edges, np.float64)
    e1, e2 = edges[:-1][None, :], edges[1:][None, :]
    return np.maximum(0.0, np.minimum(e2, right[:, None]) - np.maximum(e1, left[:, None]))


def response(e_hd, n_hd, src_edges, det_edges, sigma0=SIGMA0, sigma1=SIGMA1):
    """Ndet [NS, ND] in FP64 (matrix form of the double loop)."""
    left, right, ec, sig, n = _fine(e_hd, n_hd, sigma0, sigma1)
    X = n[:, None] * np.exp(-(ec[:, None] - ec[None, :]) ** 2 / (2.0 * sig[:, None] ** 2)) \
        / math.sqrt(2.0 * math.pi) / sig[:, None]                    # :75
    Ws = _overlap(left, right, src_edges)
    Wd = _overlap(left, right, det_edges)
    return Ws.T @ X @ Wd


def response_loops(e_hd, n_hd, src_edges, det_edges, sigma0=SIGMA0, sigma1=SIGMA1):
    """The same, as the reference writes it: one masked double sum per
    (source bin, detector bin) (spectrum_builder.m:77-95).  Small sizes only."""
    left, right, ec, sig, n = _fine(e_hd, n_hd, sigma0, sigma1)
    X = n[:, None] * np.exp(-(ec[:, None] - ec[None, :]) ** 2 / (2.0 * sig[:, None] ** 2)) \
        / math.sqrt(2.0 * math.pi) / sig[:, None]
    src_edges = np.asarray(src_edges, np.float64)
    det_edges = np.asarray(det_edges, np.float64)
    NS, ND = len(src_edges) - 1, len(det_edges) - 1
    out = np.zeros((NS, ND))
    for d in range(ND):
        Ed1, Ed2 = det_edges[d], det_edges[d + 1]
        wt_det = np.maximum(0.0, np.minimum(Ed2, right) - np.maximum(Ed1, left))
        for s in range(NS):
            Es1, Es2 = src_edges[s], src_edges[s + 1]
            wt_src = np.maximum(0.0, np.minimum(Es2, right) - np.maximum(Es1, left))
            out[s, d] = np.sum(wt_src[:, None] * wt_det[None, :] * X)
    return out


def flat(resp):
    """Column-major flat vector of an [NS, ND] response (the spectrum input)."""
    return np.asarray(resp).flatten(order="F")
