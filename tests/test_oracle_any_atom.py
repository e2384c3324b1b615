"""The oracle's any-atom charge-group cut-off (topology switch-atom flag 0):
nbpplis2(_lrf), nbpwlis2(_lrf) and nbqplis2 (src/nonbondene.f90:950-1086,
1369-1516, 2137-2242, 2493-2618, 3408-3519).  The reference ships no topology
with the flag off, so these checks pin the oracle against direct numpy
restatements of the group tests and against properties of the two modes."""
import dataclasses

import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.qnb import LIST_PP, LIST_PW, LIST_QP, LIST_QW, LIST_WW
from q6_gb300.system import make_system

CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
# short cut-offs with an LRF radius inside the sphere: some group pairs are
# beyond RcLRF, which exercises the "last atom pair" r2 of the LRF test
CUT_SHORT = dict(Rcq=8.0, RcLRF=11.0, Rcpp=6.0, Rcpw=6.0, Rcww=6.0)


def any_atom(s):
    return dataclasses.replace(s, iuse_switch_atom=0)


@pytest.fixture(scope="module")
def sys_multi():
    return make_system(R=14.0, n_solute=70, group_sizes=(3, 6), ntypes=6, nq=6, nstates=2, seed=606,
                       excl_radius=12.5)


def groups(s):
    return [s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1] for g in range(s.ncgp)]


def pairset(i, j, unordered=False):
    if unordered:
        i, j = np.minimum(i, j), np.maximum(i, j)
    return set(zip(i.tolist(), j.tolist()))


@pytest.mark.parametrize("cut", [CUT, CUT_SHORT])
def test_any_atom_lists_contain_switch_atom_lists(sys_multi, cut):
    """A switch-atom pair within the cut-off is one of the atom pairs, so every
    group pair listed with switch atoms is listed in any-atom mode too."""
    s = sys_multi
    o1, o2 = Oracle(s), Oracle(any_atom(s))
    o1.make_pair_lists(s.x, **cut)
    o2.make_pair_lists(s.x, **cut)
    for kind in (LIST_PP, LIST_PW, LIST_QP):
        a = pairset(*o1.export_pairs(kind), unordered=kind == LIST_PP)
        b = pairset(*o2.export_pairs(kind), unordered=kind == LIST_PP)
        assert a <= b, kind
    assert o2.list_size(LIST_PW) > o1.list_size(LIST_PW)
    for kind in (LIST_WW, LIST_QW):   # water lists do not depend on the flag
        assert pairset(*o1.export_pairs(kind), unordered=kind == LIST_WW) == \
            pairset(*o2.export_pairs(kind), unordered=kind == LIST_WW)


@pytest.mark.parametrize("cut", [CUT, CUT_SHORT])
def test_pw_and_qp_lists_match_direct_restatement(sys_multi, cut):
    s = sys_multi
    o = Oracle(any_atom(s))
    o.make_pair_lists(s.x, **cut)
    iq = np.full(s.natom, -1)
    iq[s.iqseq] = np.arange(s.nqat)
    G = groups(s)
    want_pw, want_qp = set(), set()
    for g in range(s.ncgp_solute):
        if s.excl[s.cgp_iswitch[g]]:
            continue
        atoms = G[g]
        for w in range(s.nwat):
            o_at = s.nat_solute + s.solv_atom * w
            if s.excl[o_at]:
                continue
            r2 = ((s.x[atoms] - s.x[o_at]) ** 2).sum(1)
            if np.any(r2 <= cut["Rcpw"] ** 2):
                for i in atoms:
                    if iq[i] < 0:
                        for a in range(s.solv_atom):
                            want_pw.add((int(i), int(o_at + a)))
        r2c = ((s.x[atoms] - s.xpcent) ** 2).sum(1)
        if np.any(r2c <= cut["Rcq"] ** 2):
            for i in atoms:
                if not np.any(s.qconn[:, i, :] <= 3):
                    for q in range(s.nqat):
                        want_qp.add((q, int(i)))
    assert pairset(*o.export_pairs(LIST_PW)) == want_pw
    assert pairset(*o.export_pairs(LIST_QP)) == want_qp


def test_lrf_far_pairs_match_direct_restatement(sys_multi):
    """phi0 of every LRF record is the sum of q_i / |x_i - centre| over the
    non-Q atoms of its far groups, so it pins the far-pair classification:
    no atom pair inside the cut-off and the last atom pair within RcLRF."""
    s = sys_multi
    cut = CUT_SHORT
    o = Oracle(any_atom(s))
    o.make_pair_lists(s.x, **cut)
    L = o.lrf()
    iq = np.full(s.natom, -1)
    iq[s.iqseq] = np.arange(s.nqat)
    G = groups(s)
    ns = s.ncgp_solute
    dist_atom = [s.cgp_iswitch[g] if g < ns else G[g][0] for g in range(s.ncgp)]
    last_atom = [G[g][-1] if g < ns else G[g][0] for g in range(s.ncgp)]
    rl2 = cut["RcLRF"] ** 2
    phi0 = np.zeros(s.ncgp)
    nfar = 0
    for g2 in range(s.ncgp):
        if s.excl[dist_atom[g2]]:
            continue
        c2 = s.x[G[g2]].mean(0)
        for g1 in range(s.ncgp):
            if g1 == g2 or s.excl[dist_atom[g1]]:
                continue
            sol1, sol2 = g1 < ns, g2 < ns
            if sol1 and sol2:
                d = s.x[G[g1]][:, None, :] - s.x[G[g2]][None, :, :]
                inside = np.any((d ** 2).sum(-1) <= cut["Rcpp"] ** 2)
            elif sol1 or sol2:
                gs, ow = (g1, dist_atom[g2]) if sol1 else (g2, dist_atom[g1])
                inside = np.any(((s.x[G[gs]] - s.x[ow]) ** 2).sum(1) <= cut["Rcpw"] ** 2)
            else:
                inside = ((s.x[dist_atom[g1]] - s.x[dist_atom[g2]]) ** 2).sum() <= cut["Rcww"] ** 2
            r2last = ((s.x[last_atom[g1]] - s.x[last_atom[g2]]) ** 2).sum()
            if inside or r2last > rl2:
                continue
            nfar += 1
            for i in G[g1]:
                if iq[i] < 0:
                    phi0[g2] += s.crg[i] / np.sqrt(((s.x[i] - c2) ** 2).sum())
    assert nfar > 100
    assert np.allclose(L[:, 3], phi0, rtol=1e-9, atol=1e-9)


def test_single_atom_groups_make_both_modes_identical(sys_multi):
    """With one solute atom per group every group test reduces to its switch
    atom, so both modes give the same lists and LRF records."""
    s = sys_multi
    ns = s.nat_solute
    nw = s.ncgp - s.ncgp_solute
    first = np.concatenate([np.arange(ns), ns + s.solv_atom * np.arange(nw)]).astype(np.int32)
    last = np.concatenate([np.arange(ns), ns + s.solv_atom * np.arange(nw) + s.solv_atom - 1]).astype(np.int32)
    split = dataclasses.replace(s, cgp_first=first, cgp_last=last, cgp_iswitch=first.copy(),
                                cgpatom=np.arange(s.natom, dtype=np.int32), ncgp_solute=ns)
    for cut in (CUT, CUT_SHORT):
        o1, o2 = Oracle(split), Oracle(any_atom(split))
        o1.make_pair_lists(s.x, **cut)
        o2.make_pair_lists(s.x, **cut)
        for kind in (LIST_PP, LIST_PW, LIST_QP, LIST_WW, LIST_QW):
            assert pairset(*o1.export_pairs(kind)) == pairset(*o2.export_pairs(kind)), kind
        assert np.array_equal(o1.lrf(), o2.lrf())
