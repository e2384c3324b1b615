"""CUDA-graph replay of the per-step evaluation and groups of contexts in one
graph launch: results bit-equal to kernel-by-kernel launches (mixed form) and
to separate contexts, across list rebuilds that grow the lists (graph
re-capture) and across watpol's theta_corr update steps (second graph)."""
import numpy as np
import pytest

from q6_gb300.qnb import PREC_FP64, PREC_MIXED, Group, NonbondedEngine
from q6_gb300.system import default_solvent_params, lambdas_for_window, make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


def run_steps(s, graphs, prec=PREC_MIXED, W=3, nsteps=6):
    sp = default_solvent_params(s, itdis=2.0)
    rng = np.random.default_rng(8)
    out = []
    with NonbondedEngine(s, precision=prec, windows=W) as e:
        e.set_graphs(graphs)
        e.set_solvent_params(sp)
        for w in range(W):
            e.set_lambda(lambdas_for_window(w / max(W - 1, 1), s.nstates), window=w)
        x = np.stack([s.x] * W)
        for k in range(nsteps):
            x = x + rng.normal(0.0, 0.01, x.shape)
            if k == 3:   # a larger move: the rebuilt lists may need more room
                x = x * 1.02
            e.set_coordinates_dev(x)
            if k % 3 == 0:
                e.make_pair_lists_dev(**CUT)
            E, EQ, R = e.compute_dev(Tfree=300.0, istep=k, sync=True)
            out.append((E, EQ.copy(), R.copy(), e.gradient_dev()))
        n = e.launches()
    return out, n


def test_graph_replay_bit_equal_to_direct_launches():
    s = make_system(R=14.0, n_solute=50, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2, seed=4242)
    direct, n0 = run_steps(s, graphs=False)
    graph, n1 = run_steps(s, graphs=True)
    assert n0 == n1   # the same kernels run
    for (E0, EQ0, R0, D0), (E1, EQ1, R1, D1) in zip(direct, graph):
        for w in range(len(E0)):
            assert E0[w] == E1[w]
        assert np.array_equal(EQ0, EQ1) and np.array_equal(R0, R1) and np.array_equal(D0, D1)


def test_graph_replay_fp64_matches_direct():
    s = make_system(R=13.0, n_solute=40, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2, seed=4343)
    direct, _ = run_steps(s, graphs=False, prec=PREC_FP64, nsteps=4)
    graph, _ = run_steps(s, graphs=True, prec=PREC_FP64, nsteps=4)
    for (E0, EQ0, R0, D0), (E1, EQ1, R1, D1) in zip(direct, graph):
        for w in range(len(E0)):
            for k in E0[w]:
                assert abs(E0[w][k] - E1[w][k]) <= 1e-9 * max(1.0, abs(E0[w][k]))
        assert np.allclose(EQ0, EQ1, rtol=1e-12, atol=1e-9) and np.allclose(D0, D1, rtol=1e-12, atol=1e-9)


def test_group_of_uneven_systems_equals_separate_contexts():
    systems = [make_system(R=R, n_solute=20, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2, seed=500 + i)
               for i, R in enumerate((12.0, 16.0, 19.5))]
    W = [4, 1, 2]
    res = {}
    for grouped in (False, True):
        engs = []
        for s, nw in zip(systems, W):
            e = NonbondedEngine(s, precision=PREC_MIXED, windows=nw)
            e.set_solvent_params(default_solvent_params(s, itdis=2.0))
            for w in range(nw):
                e.set_lambda(lambdas_for_window(0.25 * w, s.nstates), window=w)
            e.set_coordinates_dev(np.stack([s.x] * nw))
            e.make_pair_lists_dev(**CUT)
            engs.append(e)
        out = []
        grp = Group(engs) if grouped else None
        for k in range(3):   # istep 2 is a theta_corr update step
            if grouped:
                grp.compute(Tfree=300.0, istep=k)
            else:
                for e in engs:
                    e.compute_dev(Tfree=300.0, istep=k, sync=False)
            out.append([(e.energies_dev(), e.gradient_dev()) for e in engs])
        if grp:
            grp.close()
        for e in engs:
            e.close()
        res[grouped] = out
    for step_a, step_b in zip(res[False], res[True]):
        for ((Ea, EQa, Ra), Da), ((Eb, EQb, Rb), Db) in zip(step_a, step_b):
            assert all(a == b for a, b in zip(Ea, Eb))
            assert np.array_equal(EQa, EQb) and np.array_equal(Ra, Rb) and np.array_equal(Da, Db)
