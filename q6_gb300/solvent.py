"""Intra-molecular solvent pair list for solvents with torsions.

Restates prep_sim_precompute_solvent (Q6 src/simprep.f90:4003-4125), which
qdyn runs when the topology has solvent torsions and whose nonbnd_solv_int
list nonbond_solvent_internal evaluates (qnb_set_solvent_internal takes it):

* interaction(i, j) = ljcod(iac_i, iac_j) for every ordered pair of atoms of
  one molecule, 0 on the diagonal;
* bonded and angle-end pairs are set to 0 both ways;
* for a torsion's end atoms (i, l): if either direction is still non-zero,
  interaction(i, l) = 3 (1-4) and interaction(l, i) = 0;
* every remaining non-zero ordered pair (i outer, j inner) is listed -- so a
  pair that is neither bonded, angled nor a torsion end appears twice, as
  (i, j) and (j, i), exactly as the reference lists it;
* geometric rule: A = a_i a_j, B = b_i b_j with the atoms' factors for that
  LJ code; arithmetic rule: t = (a_i + a_j)^6, A = t^2 b_i b_j,
  B = 2 t b_i b_j; elec = q_i q_j, scaled by el14 for code 3.
"""
from __future__ import annotations

import numpy as np


def solvent_internal_pairs(iac, ljcod, avdw, bvdw, crg, el14_scale, ivdw_rule, bonds=(), angles=(),
                           torsions=()):
    """iac, crg: types and (scaled) charges of the atoms of one solvent
    molecule; ljcod[t1][t2] in 1..2; avdw/bvdw[t][code-1]; bonds (i, j),
    angles (i, j, k) and torsions (i, j, k, l) as 0-based offsets inside the
    molecule.  Returns (pairs (n, 2) int32, A, B, el) in the reference order."""
    n = len(iac)
    inter = np.zeros((n, n), dtype=np.int64)
    for i in range(n):
        for j in range(n):
            inter[i, j] = ljcod[iac[i]][iac[j]]
    for i in range(n):
        inter[i, i] = 0
    for b in bonds:
        inter[b[0], b[1]] = inter[b[1], b[0]] = 0
    for a in angles:
        inter[a[0], a[-1]] = inter[a[-1], a[0]] = 0
    for t in torsions:
        na, nb = t[0], t[-1]
        if inter[na, nb] != 0 or inter[nb, na] != 0:
            inter[na, nb] = 3
            inter[nb, na] = 0
    pairs, A, B, el = [], [], [], []
    for i in range(n):
        for j in range(n):
            code = int(inter[i, j])
            if code == 0:
                continue
            ai, aj = avdw[iac[i]][code - 1], avdw[iac[j]][code - 1]
            bi, bj = bvdw[iac[i]][code - 1], bvdw[iac[j]][code - 1]
            if ivdw_rule == 1:
                a_, b_ = ai * aj, bi * bj
            else:
                t = (ai + aj) ** 2
                t = t * t * t
                tb = bi * bj
                a_, b_ = t * t * tb, 2.0 * t * tb
            e = crg[i] * crg[j]
            if code == 3:
                e *= el14_scale
            pairs.append((i, j))
            A.append(a_)
            B.append(b_)
            el.append(e)
    return np.array(pairs, dtype=np.int32).reshape(-1, 2), np.array(A), np.array(B), np.array(el)
