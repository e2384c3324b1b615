"""The box LRF restatement with the topology's switch-atom flag off
(oracle/box.py box_lrf; nbpplis2_box_lrf and nbpwlis2_box_lrf,
src/nonbondene.f90:1220-1367, 2359-2491, with lrf_update 628-725) against a
pair-by-pair loop written the way the reference walks it: for every unit
pair, every atom pair (a water by its first atom) is tested in the minimum
image; the pair is LRF when none lies within Rc and one lies within RcLRF,
and lrf_update shifts the source by its switch atom's lattice vector."""
import dataclasses

import numpy as np

from oracle.box import box_lrf, nint
from q6_gb300.system import make_system

CUT = dict(Rcq=12.0, RcLRF=12.0, Rcpp=6.0, Rcpw=6.0, Rcww=6.0)


def loop_box_lrf_any(s, x, L, cut):
    G, Gs = s.ncgp, s.ncgp_solute
    groups = [np.asarray(s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1], np.int64) for g in range(G)]
    cent = np.array([x[a].mean(0) for a in groups])
    sw = [int(s.cgp_iswitch[g]) if g < Gs else int(groups[g][0]) for g in range(G)]
    isq = np.zeros(s.natom, bool)
    isq[np.asarray(s.iqseq, np.int64)] = True
    rec = np.zeros((G, 43))
    rec[:, :3] = cent
    I = np.eye(3)
    for g2 in range(G):
        for g1 in range(G):
            if g1 == g2:
                continue
            t1 = groups[g1] if g1 < Gs else groups[g1][:1]
            t2 = groups[g2] if g2 < Gs else groups[g2][:1]
            kind = (g1 < Gs) + (g2 < Gs)
            rc2 = (cut["Rcww"], cut["Rcpw"], cut["Rcpp"])[kind] ** 2
            inside = lrf = False
            for i in t1:
                for j in t2:
                    d = x[i] - x[j]
                    t = L * nint(d / L) - d
                    r2 = float(t @ t)
                    inside |= r2 <= rc2
                    lrf |= r2 <= cut["RcLRF"] ** 2
            if inside or not lrf:
                continue
            shift = L * nint((x[sw[g1]] - cent[g2]) / L)
            for i in groups[g1]:
                if isq[i]:
                    continue
                dr = x[i] - cent[g2] - shift
                r2 = float(dr @ dr)
                f0 = s.crg[i] / (r2 * np.sqrt(r2))
                f1 = 3.0 * f0 / r2
                f2 = -f1 / r2
                rec[g2, 3] += f0 * r2
                rec[g2, 4:7] -= dr * f0
                rec[g2, 7:16] += (f1 * np.outer(dr, dr) - f0 * I).reshape(9)
                phi3 = 5.0 * f2 * np.einsum("n,j,c->njc", dr, dr, dr)
                phi3 -= f2 * r2 * (I[:, :, None] * dr[None, None, :] + I[:, None, :] * dr[None, :, None]
                                   + I[None, :, :] * dr[:, None, None])
                rec[g2, 16:43] += phi3.reshape(27)
    return rec


def test_any_atom_box_lrf_matches_the_pair_loop():
    s = dataclasses.replace(make_system(R=8.0, n_solute=24, group_sizes=(3, 5), ntypes=4, nq=3, nstates=2, seed=5),
                            iuse_switch_atom=0)
    L = np.array([19.0] * 3)
    rng = np.random.default_rng(1)
    x = s.x + rng.normal(0.0, 0.05, s.x.shape)
    got = box_lrf(s, x, L, CUT)
    ref = loop_box_lrf_any(s, x, L, CUT)
    scale = np.maximum(np.abs(ref[:, 3:]).max(0), 1e-12)
    assert np.abs(ref[:, 3:]).max() > 0.0
    np.testing.assert_allclose(got[:, :3], ref[:, :3], rtol=0, atol=1e-12)
    assert (np.abs(got[:, 3:] - ref[:, 3:]) / scale).max() < 1e-11
    # the switch-atom selection differs from it on this system
    sw = box_lrf(dataclasses.replace(s, iuse_switch_atom=1), x, L, CUT)
    assert np.abs(sw[:, 3:] - ref[:, 3:]).max() > 1e-6
