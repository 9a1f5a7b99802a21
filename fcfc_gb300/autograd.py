"""Differentiable weighted pair counts: a torch.autograd.Function over the
C ABI.  The forward pass is fcfcg_count (weighted), the backward pass
fcfcg_adjoint, which recomputes the pair bins instead of storing them.
Weights are the differentiable inputs; positions are not (binned counts are
piecewise constant in them).

    from fcfc_gb300 import PairCounter
    from fcfc_gb300.autograd import weighted_pair_counts, xi_ls
    pc = PairCounter("survey", BIN_SMU, smin=0, smax=200, ds=5, nmu=100)
    dd = weighted_pair_counts(pc, d_xyz, w_d)            # auto
    dr = weighted_pair_counts(pc, d_xyz, w_d, r_xyz, w_r)
    rr = weighted_pair_counts(pc, r_xyz, w_r)
    xi = xi_ls(dd, dr, rr, w_d.sum(), w_r.sum())
    (g * xi).sum().backward()                             # w_d.grad
"""
from __future__ import annotations

import numpy as np
import torch

from .capi import PREC_FP32_RECHECK

_SLOT_A, _SLOT_B = 6, 7     # slots this module loads catalogues into


def _load(counter, slot, pos, w):
    counter.load(slot, np.asarray(pos, np.float64),
                 w.detach().to("cpu", torch.float64).numpy())


class WeightedPairCounts(torch.autograd.Function):
    """C[k] = sum over counted pairs (i, j) in bin k of w_a[i] w_b[j]
    (undoubled for auto counts, as fcfcg_count returns it), FP64."""

    @staticmethod
    def forward(ctx, w_a, w_b, counter, pos_a, pos_b):
        auto = pos_b is None
        _load(counter, _SLOT_A, pos_a, w_a)
        if not auto:
            _load(counter, _SLOT_B, pos_b, w_b)
        c = counter.count_pairs(_SLOT_A, None if auto else _SLOT_B,
                                weighted=True, precision=PREC_FP32_RECHECK)
        ctx.counter, ctx.pos_a, ctx.pos_b = counter, pos_a, pos_b
        ctx.save_for_backward(w_a, w_a if auto else w_b)
        return torch.from_numpy(c).to(w_a.device)

    @staticmethod
    def backward(ctx, g):
        w_a, w_b = ctx.saved_tensors
        counter, auto = ctx.counter, ctx.pos_b is None
        # other counts may have used the slots since: load these catalogues
        _load(counter, _SLOT_A, ctx.pos_a, w_a)
        if not auto:
            _load(counter, _SLOT_B, ctx.pos_b, w_b)
        dwa, dwb = counter.adjoint(_SLOT_A, None if auto else _SLOT_B,
                                   g.detach().to("cpu", torch.float64).numpy())
        ga = torch.from_numpy(dwa).to(w_a.device, w_a.dtype)
        gb = None
        if not auto and ctx.needs_input_grad[1]:
            gb = torch.from_numpy(dwb).to(w_b.device, w_b.dtype)
        return ga, gb, None, None, None


def weighted_pair_counts(counter, pos_a, w_a, pos_b=None, w_b=None):
    """Weighted pair counts of (pos_a, w_a) with itself, or with
    (pos_b, w_b); differentiable in the weights (FP64 tensors)."""
    if pos_b is not None and w_b is None:
        w_b = torch.ones(len(pos_b), dtype=torch.float64)
    return WeightedPairCounts.apply(w_a, w_b, counter, pos_a, pos_b)


def xi_ls(dd, dr, rr, sw_d, sw_r):
    """Landy-Szalay estimator from undoubled weighted counts, with FCFC's
    normalisations (src/fcfc/2pt/eval_cf.c:117-167): auto counts doubled
    over W (W - 1), cross counts over W_D W_R."""
    DD = 2 * dd / (sw_d * (sw_d - 1))
    DR = dr / (sw_d * sw_r)
    RR = 2 * rr / (sw_r * (sw_r - 1))
    return (DD - 2 * DR + RR) / RR
