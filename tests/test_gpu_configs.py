"""The benchmark configurations at full size on the GPU.

1  R15 droplet, 20-atom solute, 6 Q atoms, 2 states (FP64, the oracle's size)
2  R25 sphere, 3,000-atom solute, 20 Q atoms, 2 states (the metric's system)
3  51 lambda windows of config 1 in one batched context, and 16 replicas with
   radii drawn from 18-30 A
4  config 1 with a 40-atom solute, 30 Q atoms in 4 states, log-normal Q LJ
5  R40 sphere, 8,000-atom solute, 40 Q atoms in 4 states, 12 A cut-offs, 16
   windows batched

Bars: the FP64 form against the CPU oracle within 1e-6 kcal/mol per energy
term (1e-9 relative for terms above 1,000 kcal/mol: the FP64 form sums with
atomics, so its rounding follows the schedule) and 1e-6 relative per gradient
component; the mixed form within 1e-3 relative; batched windows bit-equal to
single-window contexts; every pair list equal to the oracle's as a set
(configs 1, 2, 4 and 5, both forms)."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.qnb import (LIST_PP, LIST_PP14, LIST_PW, LIST_QP, LIST_QW, LIST_WW, PREC_FP64, PREC_MIXED,
                          NonbondedEngine)
from q6_gb300.system import (config_adjoint, config_large, config_small, config_window, default_solvent_params,
                             lambdas_for_window, make_system)

pytestmark = pytest.mark.gpu

CUT10 = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
CUT12 = dict(Rcq=99.0, RcLRF=99.0, Rcpp=12.0, Rcpw=12.0, Rcww=12.0)


def fp64_bar(e):
    return 1e-6 * max(1.0, abs(e) / 1e3)


def grad_ok(d, d0, rel):
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    return bool(np.all(np.abs(d - d0) <= rel * scale + 1e-9))


UNORDERED = {LIST_PP, LIST_PP14, LIST_WW}


def assert_lists_equal_as_sets(eng, o, natom, label):
    """Every pair list of the engine equals the oracle's as a set, compared
    as sorted int64 keys (config 5 has ~10^7 entries)."""
    for kind in (LIST_PP, LIST_PW, LIST_WW, LIST_QP, LIST_QW, LIST_PP14):
        assert eng.list_size(kind) == o.list_size(kind), (label, kind)
        keys = []
        for i, j in (eng.export_pairs(kind), o.export_pairs(kind)):
            i, j = i.astype(np.int64), j.astype(np.int64)
            if kind in UNORDERED:
                i, j = np.minimum(i, j), np.maximum(i, j)
            keys.append(np.sort(i * natom + j))
        assert np.array_equal(keys[0], keys[1]), (label, kind)
        assert len(np.unique(keys[0])) == len(keys[0]), (label, kind)   # no pair listed twice


def check_vs_oracle(s, cut, lam):
    sp = default_solvent_params(s)
    o = Oracle(s)
    o.set_solvent_params(sp)
    d0, E0, EQ0, R0 = o.evaluate(s.x, lam, cut=cut, solvent=sp)
    o.make_pair_lists(s.x, **cut)
    for prec, tol, gtol in ((PREC_FP64, 1e-6, 1e-6), (PREC_MIXED, 1e-3, 2e-3)):
        with NonbondedEngine(s, precision=prec) as eng:
            eng.set_solvent_params(sp)
            d, E, EQ, R = eng.evaluate(s.x, lam, cut=cut, solvent=sp)
            assert_lists_equal_as_sets(eng, o, s.natom, (s.name, prec))
        for k in E0:
            bar = fp64_bar(E0[k]) if prec == PREC_FP64 else tol * max(1.0, abs(E0[k]))
            assert abs(E[k] - E0[k]) <= bar, (prec, k, E[k], E0[k])
        qbar = tol if prec == PREC_FP64 else tol * np.maximum(1.0, np.abs(EQ0))
        assert np.all(np.abs(EQ - EQ0) <= qbar), (prec, EQ, EQ0)
        assert grad_ok(d, d0, gtol), prec


def test_config1_droplet():
    check_vs_oracle(config_small(), CUT10, [0.5, 0.5])


def test_config2_r25_sphere():
    check_vs_oracle(config_window(), CUT10, [0.5, 0.5])


def test_config4_four_state_evb():
    check_vs_oracle(config_adjoint(), CUT10, [0.4, 0.3, 0.2, 0.1])


@pytest.mark.parametrize("ntypes,pairs", [(100, ((0, 1), (70, 90), (5, 99), (64, 63))),
                                           (140, ((0, 1), (130, 135), (3, 100)))])
def test_many_atom_types(ntypes, pairs):
    """Type-2 LJ pairs among more than 64 atom types: the mixed form's rows
    mark per group which partner types need the general pair path in a
    128-type mask (types 64 and above in its second word); with more than
    128 types every partner takes the general path."""
    s = make_system(R=16.0, n_solute=400, group_sizes=(3, 6), ntypes=ntypes, nq=6, nstates=2,
                    seed=77 + ntypes, type2_pairs=pairs)
    hi = s.iac[: s.nat_solute]
    assert (hi >= 64).any() and any((hi == a).any() and (hi == b).any() for a, b in pairs if a >= 64 or b >= 64)
    check_vs_oracle(s, CUT10, [0.5, 0.5])


def batched_vs_single(s, cut, lams, check_windows, prec=PREC_MIXED):
    W = len(lams)
    sp = default_solvent_params(s)
    rng = np.random.default_rng(17)
    xs = np.stack([s.x + rng.normal(0.0, 0.02, s.x.shape) for _ in range(W)])
    with NonbondedEngine(s, precision=prec, windows=W) as b:
        b.set_solvent_params(sp)
        for w in range(W):
            b.set_lambda(lams[w], window=w)
        b.set_coordinates_dev(xs)
        b.make_pair_lists_dev(**cut)
        E, EQ, R = b.compute_dev(Tfree=300.0, istep=0, sync=True)
        D = b.gradient_dev()
    for w in check_windows:
        with NonbondedEngine(s, precision=prec) as e:
            e.set_solvent_params(sp)
            e.set_lambda(lams[w])
            e.set_coordinates_dev(xs[w][None])
            e.make_pair_lists_dev(**cut)
            E1, EQ1, R1 = e.compute_dev(Tfree=300.0, istep=0, sync=True)
            D1 = e.gradient_dev()
        for k in E1[0]:
            assert E[w][k] == E1[0][k], (w, k)
        assert np.array_equal(EQ[w], EQ1[0]) and np.array_equal(R[w], R1[0]), w
        assert np.array_equal(D[w], D1[0]), w
    return xs, E, EQ, D


def test_config3_51_windows_batched():
    s = config_small()
    lams = [lambdas_for_window(l, s.nstates) for l in np.linspace(0.0, 1.0, 51)]
    batched_vs_single(s, CUT10, lams, check_windows=(0, 25, 50))


def test_config3_uneven_replicas():
    """16 replicas, radii uniform in 18-30 A: each its own context; the mixed
    form within 1e-3 of the FP64 form, and 3 of them (smallest, median,
    largest) FP64 against the oracle."""
    rng = np.random.default_rng(3016)
    radii = np.sort(rng.uniform(18.0, 30.0, 16))
    for r_i, R in enumerate(radii):
        s = make_system(R=float(R), n_solute=20, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2,
                        seed=3100 + r_i)
        sp = default_solvent_params(s)
        out = {}
        for prec in (PREC_FP64, PREC_MIXED):
            with NonbondedEngine(s, precision=prec) as eng:
                eng.set_solvent_params(sp)
                out[prec] = eng.evaluate(s.x, [0.5, 0.5], cut=CUT10, solvent=sp)
        d64, E64, EQ64, _ = out[PREC_FP64]
        dmx, Emx, EQmx, _ = out[PREC_MIXED]
        for k in E64:
            assert abs(Emx[k] - E64[k]) <= 1e-3 * max(1.0, abs(E64[k])), (R, k)
        assert np.allclose(EQmx, EQ64, rtol=1e-3, atol=1e-3), R
        assert grad_ok(dmx, d64, 2e-3), R
        if r_i in (0, 8, 15):
            o = Oracle(s)
            o.set_solvent_params(sp)
            d0, E0, EQ0, _ = o.evaluate(s.x, [0.5, 0.5], cut=CUT10, solvent=sp)
            for k in E0:
                assert abs(E64[k] - E0[k]) <= fp64_bar(E0[k]), (R, k, E64[k], E0[k])
            assert np.all(np.abs(EQ64 - EQ0) <= 1e-6), R
            assert grad_ok(d64, d0, 1e-6), R


@pytest.fixture(scope="module")
def large():
    return config_large()


def test_config5_large_fp64_vs_oracle(large):
    s = large
    lam = [0.25, 0.25, 0.25, 0.25]
    sp = default_solvent_params(s)
    o = Oracle(s)
    o.set_solvent_params(sp)
    d0, E0, EQ0, R0 = o.evaluate(s.x, lam, cut=CUT12, solvent=sp)
    o.make_pair_lists(s.x, **CUT12)
    with NonbondedEngine(s, precision=PREC_FP64) as eng:
        eng.set_solvent_params(sp)
        d, E, EQ, R = eng.evaluate(s.x, lam, cut=CUT12, solvent=sp)
        assert_lists_equal_as_sets(eng, o, s.natom, "config5 fp64")
    with NonbondedEngine(s, precision=PREC_MIXED) as eng:
        eng.make_pair_lists(s.x, **CUT12)
        assert_lists_equal_as_sets(eng, o, s.natom, "config5 mixed")
    for k in E0:
        assert abs(E[k] - E0[k]) <= fp64_bar(E0[k]), (k, E[k], E0[k])
    assert np.all(np.abs(EQ - EQ0) <= 1e-6), (EQ, EQ0)
    assert grad_ok(d, d0, 1e-6)


def test_config5_large_16_windows(large):
    """16 batched windows: window 3 and 12 bit-equal to single contexts, and
    every window's mixed energies within 1e-3 of the FP64 form's."""
    s = large
    lams = [lambdas_for_window(l, s.nstates) for l in np.linspace(0.0, 1.0, 16)]
    xs, E, EQ, D = batched_vs_single(s, CUT12, lams, check_windows=(3, 12))
    sp = default_solvent_params(s)
    with NonbondedEngine(s, precision=PREC_FP64, windows=16) as b:
        b.set_solvent_params(sp)
        for w in range(16):
            b.set_lambda(lams[w], window=w)
        b.set_coordinates_dev(xs)
        b.make_pair_lists_dev(**CUT12)
        E64, EQ64, _ = b.compute_dev(Tfree=300.0, istep=0, sync=True)
        D64 = b.gradient_dev()
    for w in range(16):
        for k in E64[w]:
            assert abs(E[w][k] - E64[w][k]) <= 1e-3 * max(1.0, abs(E64[w][k])), (w, k)
        assert np.allclose(EQ[w], EQ64[w], rtol=1e-3, atol=1e-3), w
        assert grad_ok(D[w], D64[w], 2e-3), w


def test_config3_one_graph_launch_for_windows_and_replicas():
    """Config 3 as one CUDA graph launch per step: the 51-window context of
    the config-1 system plus 16 single-window replicas of uneven radii; every
    context's energies and gradients bit-equal to its own qnb_compute_dev."""
    from q6_gb300.qnb import Group
    base = config_small()
    rng = np.random.default_rng(3016)
    radii = np.sort(rng.uniform(18.0, 30.0, 16))
    systems = [base] + [make_system(R=float(R), n_solute=20, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2,
                                    seed=3100 + i) for i, R in enumerate(radii)]
    nwin = [51] + [1] * 16
    lam51 = [lambdas_for_window(l, 2) for l in np.linspace(0.0, 1.0, 51)]
    res = {}
    for grouped in (False, True):
        engs = []
        for s, W in zip(systems, nwin):
            e = NonbondedEngine(s, precision=PREC_MIXED, windows=W)
            e.set_solvent_params(default_solvent_params(s))
            for w in range(W):
                e.set_lambda(lam51[w] if W == 51 else [0.5, 0.5], window=w)
            e.set_coordinates_dev(np.stack([s.x] * W))
            e.make_pair_lists_dev(**CUT10)
            engs.append(e)
        grp = Group(engs) if grouped else None
        out = []
        for k in range(2):
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
