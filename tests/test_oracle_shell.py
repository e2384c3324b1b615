"""fix_shell (src/potene.f90:386-423) and the shell atoms of make_shell /
make_shell2 (src/topo.f90:1426-1491) in the oracle and q6_gb300.md."""
import dataclasses

import numpy as np

from oracle.oracle import Oracle
from q6_gb300.md import make_shell
from q6_gb300.system import make_system


def test_make_shell_marks_whole_groups_beyond_radius():
    s = make_system(R=14.0, n_solute=60, group_sizes=(3, 5), ntypes=6, nq=4, nstates=2, seed=12)
    sh = make_shell(s, 3.0)
    assert 0 < sh.sum() < s.nat_solute
    for g in range(s.ncgp_solute):
        atoms = s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1]
        sw = s.cgp_iswitch[g]
        beyond = np.sum((s.x[sw] - s.xpcent) ** 2) > 9.0 and s.heavy[sw] and not s.excl[sw]
        assert np.all(sh[atoms] == (1 if beyond else 0)), g
    assert sh[s.nat_solute:].sum() == 0
    # a fraction of rexcl_o, and the any-atom form by group centres
    assert np.array_equal(make_shell(s, 3.0 / s.rexcl_o), sh)
    s0 = dataclasses.replace(s, iuse_switch_atom=0)
    sh0 = make_shell(s0, 3.0)
    for g in range(s.ncgp_solute):
        atoms = s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1]
        sw = s.cgp_iswitch[g]
        beyond = np.sum((s.x[atoms].mean(0) - s.xpcent) ** 2) > 9.0 and s.heavy[sw] and not s.excl[sw]
        assert np.all(sh0[atoms] == (1 if beyond else 0)), g


def test_fix_shell_energy_and_gradient():
    s = make_system(R=12.0, n_solute=40, group_sizes=(3, 5), ntypes=6, nq=4, nstates=2, seed=13,
                    excl_radius=10.0)
    assert np.asarray(s.excl).sum() > 0
    sh = make_shell(s, 5.0)
    rng = np.random.default_rng(1)
    x = s.x + rng.normal(0, 0.1, s.x.shape)
    o = Oracle(s)
    d, E = o.fix_shell(x, s.x, sh, 200.0, 10.0)
    ex = np.asarray(s.excl).astype(bool)
    r2 = ((x - s.x) ** 2).sum(1)
    assert np.isclose(E[0], 0.5 * 200.0 * r2[ex].sum())
    assert np.isclose(E[1], 0.5 * 10.0 * r2[sh.astype(bool)].sum())
    fk = np.where(ex, 200.0, np.where(sh.astype(bool), 10.0, 0.0))
    assert np.allclose(d, (x - s.x) * fk[:, None])
