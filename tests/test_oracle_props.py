"""Properties of the CPU oracle itself (no GPU): Newton's third law, lambda
linearity of the Q-atom gradient, and gradients against finite differences."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.system import make_system


@pytest.fixture(scope="module")
def small():
    return make_system(R=10.0, n_solute=30, nq=5, nstates=2, seed=11, excl_radius=8.5,
                       soft_pairs=[(0, 4)], el_scale=[((0, 3), (0.5, 0.8))])


def test_newton_third_law_without_lrf(small):
    o = Oracle(small, use_lrf=False)
    d, E, EQ, _ = o.evaluate(small.x, [0.3, 0.7])
    assert np.abs(d.sum(0)).max() < 1e-9 * max(1.0, np.abs(d).max())


def test_q_gradient_is_linear_in_lambda(small):
    o = Oracle(small, use_lrf=False)
    o.set_lambda([0.0, 0.0])
    o.make_pair_lists(small.x)
    d00, _, _ = o.pot_energy_nonbonds(small.x, md=False)
    d00, _ = o.nonbond_qq(small.x, d00)
    grads = []
    for lam in ([1.0, 0.0], [0.0, 1.0], [0.25, 0.75]):
        o.set_lambda(lam)
        d, _, _ = o.pot_energy_nonbonds(small.x, md=False)
        d, _ = o.nonbond_qq(small.x, d)
        grads.append(d - d00)
    mix = 0.25 * grads[0] + 0.75 * grads[1]
    assert np.allclose(grads[2], mix, rtol=1e-9, atol=1e-9)


def test_gradient_matches_finite_differences():
    s = make_system(R=7.0, n_solute=12, nq=3, nstates=2, seed=5)
    o = Oracle(s, use_lrf=False)
    lam = [0.4, 0.6]
    cut = dict(Rcq=99.0, RcLRF=99.0, Rcpp=99.0, Rcpw=99.0, Rcww=99.0)

    def energy(x):
        o.set_lambda(lam)
        d, E, EQ = o.pot_energy_nonbonds(x)
        d, EQ = o.nonbond_qq(x, d, EQ)
        tot = sum(E.values()) + sum(l * EQ[k].sum() for k, l in enumerate(lam))
        return tot, d

    o.make_pair_lists(s.x, **cut)
    e0, d0 = energy(s.x)
    rng = np.random.default_rng(0)
    h = 1e-5
    for i in rng.choice(s.natom, 12, replace=False):
        for c in range(3):
            xp = s.x.copy(); xp[i, c] += h
            xm = s.x.copy(); xm[i, c] -= h
            fd = (energy(xp)[0] - energy(xm)[0]) / (2 * h)
            assert abs(fd - d0[i, c]) <= 1e-4 * max(1.0, abs(fd)), (i, c, fd, d0[i, c])


def test_lrf_energy_approximates_far_field_coulomb():
    """The LRF Taylor energy (lrf_update + lrf_taylor) approximates the exact
    Coulomb energy of the pairs it replaces: non-Q atoms of group pairs beyond
    the cut-off.  An independent numpy sum over those pairs pins the oracle's
    far-pair classification and expansion; the expansion is truncated after
    the third order in |x_i - centre| / r (groups of up to 3 A radius, sources
    beyond 10 A), so the bar is 5 %."""
    s = make_system(R=15.0, n_solute=60, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2, seed=71)
    o = Oracle(s)
    o.make_pair_lists(s.x)
    _, E, _ = o.pot_energy_nonbonds(s.x)
    ns = s.ncgp_solute
    groups = [s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1] for g in range(s.ncgp)]
    dist = np.array([s.cgp_iswitch[g] if g < ns else groups[g][0] for g in range(s.ncgp)])
    gid = np.zeros(s.natom, dtype=int)
    for g, atoms in enumerate(groups):
        gid[atoms] = g
    q = s.crg.copy()
    q[s.iqseq] = 0.0
    d2 = ((s.x[dist][:, None, :] - s.x[dist][None, :, :]) ** 2).sum(-1)
    far_g = (d2 > 100.0) & ~s.excl[dist][:, None].astype(bool) & ~s.excl[dist][None, :].astype(bool)
    e = 0.0
    for i in range(s.natom):
        if q[i] == 0.0 or s.excl[dist[gid[i]]]:
            continue
        far = far_g[gid[i]][gid]
        r = np.sqrt(((s.x - s.x[i]) ** 2).sum(1))
        e += q[i] * np.sum(q[far] / r[far])
    e *= 0.5
    assert abs(E["lrf"] - e) <= 0.05 * abs(e), (E["lrf"], e)
