"""Free-energy perturbation summary as Qfep computes it.

Restates the exponential-averaging part of Q6 src/qfep.f90:587-644 (Zwanzig
forward and reverse sums between adjacent lambda windows):

    dGf(w) = -RT ln < exp(-(E_{lambda(w+1)} - E_{lambda(w)}) / RT) >_w
    dGr(w) = -RT ln < exp(-(E_{lambda(w-1)} - E_{lambda(w)}) / RT) >_w
    dG(w)  = dG(w-1) + (dGf(w-1) - dGr(w)) / 2

where E_lambda(frame) = sum_s lambda_s * V_s(frame) and V_s is the state's
total Q-atom energy of the frame.
"""
from __future__ import annotations

import numpy as np

BOLTZ = 0.001986   # kcal/(mol K), the value qdyn uses (src/md.f90)


def qfep_dg(v, lambdas, rt):
    """v[w][frame][s]: per-state energies of the frames sampled in window w;
    lambdas[w][s]: the window's state weights.  Returns (dgf, dgr, dg) with
    dgf[w] for w = 0..n-2, dgr[w] for w = 1..n-1 (others 0) and cumulative dG."""
    v = [np.asarray(a, dtype=np.float64) for a in v]
    lam = np.asarray(lambdas, dtype=np.float64)
    n = len(v)
    dgf = np.zeros(n)
    dgr = np.zeros(n)
    for w in range(n - 1):
        e_here = v[w] @ lam[w]
        e_next = v[w] @ lam[w + 1]
        dgf[w] = -rt * np.log(np.mean(np.exp(-(e_next - e_here) / rt)))
    for w in range(n - 1, 0, -1):
        e_here = v[w] @ lam[w]
        e_prev = v[w] @ lam[w - 1]
        dgr[w] = -rt * np.log(np.mean(np.exp(-(e_prev - e_here) / rt)))
    dg = np.zeros(n)
    for w in range(1, n):
        dg[w] = dg[w - 1] + 0.5 * (dgf[w - 1] - dgr[w])
    return dgf, dgr, dg


def window_increments(dg):
    """Per-window-pair contribution dG(w+1) - dG(w)."""
    return np.diff(np.asarray(dg))


def state_energies(EQ):
    """Total Q-atom nonbonded energy per state from qnb_qenergies records
    (qq + qp + qw, el + vdW); bonded Q terms are outside this path."""
    return np.asarray(EQ).sum(axis=-1)
