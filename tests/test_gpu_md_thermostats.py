"""Nose-Hoover and Langevin thermostats and velocity Verlet on the device
(qnb_md_set_thermostat, qnb_md_set_langevin; newvel_lan with the same
SplitMix64 random forces as the oracle;
nh_prop, src/simprep.f90:2509-2550; newvel_nos / newvel_ber with the
velocity-Verlet half steps, src/md.f90:1451-1521, 1768-1812) against the
oracle's MD step in the FP64 form: per-step energies, temperatures and the
final coordinates and velocities of a 12-step run within 1e-9."""
import numpy as np
import pytest

from oracle.oracle import Oracle, OracleMD
from q6_gb300.md import MdSetup, build_constraints, maxwell_velocities, md_params
from q6_gb300.qnb import PREC_FP64, NonbondedEngine, QnbError
from q6_gb300.system import default_solvent_params, make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
SETUP = MdSetup(stepsize=1.0, temp0=300.0, tau_t=20.0, nbcycle=5, shake_solute=True, shake_heavy=True, cut=CUT)


@pytest.fixture(scope="module")
def system():
    return make_system(R=14.0, n_solute=40, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2, seed=5150)


@pytest.mark.parametrize("thermostat,integrator,chains", [("nose-hoover", "leap-frog", 10),
                                                          ("nose-hoover", "velocity-verlet", 3),
                                                          ("berendsen", "velocity-verlet", 10),
                                                          ("langevin", "leap-frog", 0),
                                                          ("langevin", "velocity-verlet", 0)])
def test_fp64_matches_oracle(system, thermostat, integrator, chains):
    s = system
    lam = [0.6, 0.4]
    n = 12
    sp = default_solvent_params(s, itdis=4.0)
    v0 = maxwell_velocities(s, 300.0, 11)
    with NonbondedEngine(s, precision=PREC_FP64, windows=1) as e:
        e.set_solvent_params(sp)
        e.set_lambda(lam)
        e.set_coordinates_dev(s.x[None])
        e.md_init(SETUP)
        if thermostat == "langevin":
            e.md_set_langevin(integrator, seed=7)
        else:
            e.md_set_thermostat(thermostat, integrator, nhchains=chains)
        e.md_set_velocities(v0[None])
        e.md_prepare(stop_cm=True)
        rec, EQ, _ = e.md_run(n)
        xd, vd = e.md_state(0)
    o = Oracle(s)
    o.set_solvent_params(sp)
    cons = build_constraints(s, SETUP)
    md = OracleMD(o, md_params(s, SETUP, cons), cons, sp=sp, lam=lam, thermostat=thermostat,
                  integrator=integrator, nhchains=max(chains, 2), seed=7)
    x, v = md.prepare(s.x, v0)
    for k in range(n):
        r = md.step(x, v, k, CUT)
        for f, key in enumerate(("pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw", "lrf")):
            assert abs(rec[k, 0]["E"][f] - r["E"][key]) <= 1e-9 * max(1.0, abs(r["E"][key])), (k, key)
        for key in ("ekin", "temp", "tfree"):
            assert abs(rec[k, 0][key] - r[key]) <= 1e-9 * abs(r[key]), (k, key)
    assert np.allclose(xd, x, rtol=0, atol=1e-9)
    assert np.allclose(vd, v, rtol=1e-8, atol=1e-10)


def test_rejects_bad_settings(system):
    with NonbondedEngine(system, precision=PREC_FP64, windows=1) as e:
        with pytest.raises(QnbError):
            e.md_set_thermostat("nose-hoover")   # before qnb_md_init
        e.set_coordinates_dev(system.x[None])
        e.md_init(SETUP)
        with pytest.raises(QnbError):
            e.md_set_thermostat("nose-hoover", nhchains=1)
