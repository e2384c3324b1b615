"""The oracle's MD step (newvel_ber, SHAKE, v = (x - xx)/dt, temperature with
Berendsen factors; src/md.f90:1379-1466, 1768-1812, src/bondene.f90:1025-1150)
pinned by properties: constraints hold, total energy is conserved without a
thermostat, the Berendsen factor pulls the free temperature to Temp0, and
the degrees of freedom follow simprep.f90:2439-2448."""
import numpy as np
import pytest

from oracle.oracle import Oracle, OracleMD
from q6_gb300.md import MdSetup, build_constraints, degrees_of_freedom, maxwell_velocities, md_params, temperature_groups
from q6_gb300.system import make_system

CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=99.0, Rcpw=99.0, Rcww=99.0)   # no cut-off, no LRF far field


@pytest.fixture(scope="module")
def small():
    return make_system(R=10.0, n_solute=12, group_sizes=(3, 4), ntypes=4, nq=3, nstates=2, seed=2024)


def run(s, setup, nsteps, T=300.0, seed=1):
    cons = build_constraints(s, setup)
    p = md_params(s, setup, cons)
    o = Oracle(s, use_lrf=False)
    md = OracleMD(o, p, cons, sp=None, lam=[0.7, 0.3])
    x, v = md.prepare(s.x, maxwell_velocities(s, T, seed))
    out = []
    for k in range(nsteps):
        r = md.step(x, v, k, CUT)
        epot = sum(r["E"].values()) + float(np.dot([0.7, 0.3], r["EQ"].sum(1)))
        out.append((epot, r["ekin"], r["temp"], r["tfree"], r["shake_iterations"]))
    return x, v, cons, np.array(out)


def test_constraints_hold_after_steps(small):
    setup = MdSetup(stepsize=1.0, shake_solute=True, shake_heavy=True, cut=CUT)
    x, v, cons, _ = run(small, setup, 8)
    d = np.linalg.norm(x[cons.ij[:, 0]] - x[cons.ij[:, 1]], axis=1)
    # SHAKE marks a constraint done once |d0^2 - d^2| < 1e-4 d0^2 and does not
    # revisit it while later corrections in the same sweep move its atoms (the
    # generated start structure is strained: large first-step displacements)
    rel = np.abs(d * d - cons.dist ** 2) / cons.dist ** 2
    assert rel.max() < 1e-2 and np.median(rel) < 1e-4


def test_total_energy_conserved_without_thermostat(small):
    setup = MdSetup(stepsize=0.25, tau_t=1e12, shake_solute=True, shake_heavy=True, cut=CUT)
    _, _, _, out = run(small, setup, 40)
    etot = out[:, 0] + out[:, 1]
    # leap-frog kinetic energy is half a step off the potential: compare the
    # spread of the total with the spread of the kinetic energy
    assert np.ptp(etot) < 0.1 * np.ptp(out[:, 1]), (np.ptp(etot), np.ptp(out[:, 1]))


def test_berendsen_pulls_temperature_to_target(small):
    setup = MdSetup(stepsize=1.0, tau_t=10.0, temp0=150.0, shake_solute=True, shake_heavy=True, cut=CUT)
    _, _, _, out = run(small, setup, 60, T=450.0)
    t = out[:, 3]
    assert abs(t[-10:].mean() - 150.0) < abs(t[:3].mean() - 150.0) / 2


def test_degrees_of_freedom_rules(small):
    s = small
    setup = MdSetup(shake_solute=False)
    cons = build_constraints(s, setup)
    groups = temperature_groups(s, setup)
    ndegf, ndegfree, tg = degrees_of_freedom(s, cons, groups)
    assert ndegf == 3 * s.natom - 3 * s.nwat
    nexcl = int(np.asarray(s.excl).sum())
    exclw = int(np.asarray(s.excl)[s.nat_solute:].sum())
    assert ndegfree == int(ndegf - 3 * nexcl + exclw)   # 3 constraints x 2 ends x 1/2 per excluded water atom
    assert tg[0] == (3.0 * s.nat_solute, 3.0 * s.nat_solute - 3 * int(np.asarray(s.excl)[:s.nat_solute].sum()))
    assert len(groups) == 2 and groups[1] == (s.nat_solute, s.natom - 1)
    one = temperature_groups(s, MdSetup(separate_scaling=False))
    assert one == [(0, s.natom - 1)]


def test_nose_hoover_removes_heat(small):
    # the generated structure heats up as its strain relaxes; the chain
    # (Temp0 150 K) takes the heat out where the uncoupled run keeps it
    s = small

    def temps(thermostat, tau):
        setup = MdSetup(stepsize=1.0, tau_t=tau, temp0=150.0, shake_solute=True, shake_heavy=True, cut=CUT)
        cons = build_constraints(s, setup)
        o = Oracle(s, use_lrf=False)
        md = OracleMD(o, md_params(s, setup, cons), cons, lam=[0.7, 0.3], thermostat=thermostat, nhchains=4)
        x, v = md.prepare(s.x, maxwell_velocities(s, 450.0, 1))
        return np.array([md.step(x, v, k, CUT)["temp"] for k in range(200)])

    nh = temps("nose-hoover", 10.0)
    nve = temps("berendsen", 1e12)
    assert nh[-30:].mean() < 0.9 * nve[-30:].mean()
    assert nh[-30:].mean() < nh[20:50].mean()


def test_velocity_verlet_half_steps(small):
    # qdyn's velocity Verlet (newvel_*, src/md.f90:1451-1521): two force
    # half-steps of the same gradient around the move, x += (v - F dt/2) dt
    # and v -= F dt; without constraints SHAKE does not overwrite v
    s = small
    setup = MdSetup(stepsize=0.5, tau_t=1e12, shake_solvent=False, shake_solute=False, cut=CUT)
    cons = build_constraints(s, setup)
    o = Oracle(s, use_lrf=False)
    md = OracleMD(o, md_params(s, setup, cons), cons, lam=[0.7, 0.3], integrator="velocity-verlet")
    x, v = md.prepare(s.x, maxwell_velocities(s, 300.0, 1))
    x0, v0 = x.copy(), v.copy()
    o.make_pair_lists(x0, **CUT)
    d, _, EQ = o.pot_energy_nonbonds(x0.copy(), np.zeros_like(x0))
    d, _ = o.nonbond_qq(x0, d, EQ)
    sf = md.sfact.copy()
    md.step(x, v, 0, CUT)
    a = d * md.winv[:, None] * (0.5 * md.dt)
    np.testing.assert_allclose(x, x0 + (v0 - a) * sf[0] * md.dt, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(v, ((v0 - a) * sf[0] - a) * sf[0], rtol=1e-12, atol=1e-12)


def test_langevin_pulls_temperature_to_target(small):
    s = small
    setup = MdSetup(stepsize=1.0, tau_t=10.0, temp0=150.0, shake_solute=True, shake_heavy=True, cut=CUT)
    cons = build_constraints(s, setup)
    o = Oracle(s, use_lrf=False)
    md = OracleMD(o, md_params(s, setup, cons), cons, lam=[0.7, 0.3], thermostat="langevin", seed=7)
    x, v = md.prepare(s.x, maxwell_velocities(s, 450.0, 1))
    t = np.array([md.step(x, v, k, CUT)["temp"] for k in range(200)])
    assert abs(t[-50:].mean() - 150.0) < 0.35 * 150.0
