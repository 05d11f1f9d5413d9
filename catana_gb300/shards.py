"""Combining the SFB coefficients of a catalog sharded over ranks.

f_lmn is normalised per call by V / W (W = number of points, or sum of weights), so
the coefficients of the union of shards r are  f = sum_r (W_r / W) f_r.  One
all-reduce of the weighted f (and of W) combines them; C_ln follows from the summed
f as sum_{m=-l..l} |f_l|m|n|^2 / (2l+1) (sfb_raw.cpp:91-96).
"""
import torch


def combine_flmn(f, w_local, all_reduce=None):
    """f: real tensor of interleaved (re, im) f_lmn of this rank's shard; w_local:
    the shard's point count or weight sum.  all_reduce(tensor) sums in place across
    ranks (e.g. torch.distributed.all_reduce); None means a single rank.  Returns
    the combined f (in place) and the total weight."""
    wt = torch.tensor([float(w_local)], dtype=torch.float64, device=f.device)
    if all_reduce is not None:
        all_reduce(wt)
    total = float(wt.item())
    f.mul_(float(w_local) / total)
    if all_reduce is not None:
        all_reduce(f)
    return f, total


def cln_from_flmn(f, lmax, nmax):
    """C_ln (lmax x nmax, float64) from interleaved packed f_lmn."""
    fz = torch.view_as_complex(f.view(-1, 2))
    out = torch.empty((lmax, nmax), dtype=torch.float64, device=f.device)
    off = 0
    for l in range(lmax):
        blk = fz[off:off + (l + 1) * nmax].view(l + 1, nmax)
        p = blk.real ** 2 + blk.imag ** 2
        out[l] = (2 * p.sum(0) - p[0]) / (2 * l + 1)
        off += (l + 1) * nmax
    return out
