"""Monitor groups and group contributions on the GPU (k_pair_sets, FP64 in
both forms): nonbond_monitor's per-state Vel / Vlj and calculate_exc's
excluded Q-Q and Q-P energies (src/nonbondene.f90:4517-4680, 6825-6920)
against the oracle restatement on the same coordinates, per window; windows
of one batch bit-equal to single contexts; the values after an MD run
(evaluated inside every qnb_md_run step) against the oracle on the final
coordinates; the group-contribution arrays written to and read back from a
qdyn energy file."""
import numpy as np
import pytest

from oracle.pairsets import group_exclusions, monitor_energies
from q6_gb300.enefile import EnergyFileWriter, read_energy_file
from q6_gb300.md import MdSetup, maxwell_velocities
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine, QnbError
from q6_gb300.system import lambdas_for_window, make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


@pytest.fixture(scope="module")
def case():
    s = make_system(R=13.0, n_solute=36, group_sizes=(3, 5), ntypes=5, nq=6, nstates=2, seed=919,
                    soft_pairs=((0, 3),), el_scale=(((1, 4), (0.5, 0.7)),))
    nonq = np.setdiff1d(np.arange(s.nat_solute), s.iqseq)
    rng = np.random.default_rng(8)
    half = rng.random(len(nonq)) < 0.5
    groups = [list(s.iqseq), list(nonq), list(nonq[half]), list(nonq[~half]),
              list(s.iqseq[:3]), list(s.iqseq[3:]) + list(nonq[:5])]
    pairs = [(0, 1), (2, 3), (4, 5), (3, 0)]
    m1 = np.zeros(s.nat_solute, bool)
    m1[nonq[half]] = True
    m1[s.iqseq[1]] = True
    m2 = np.zeros(s.nat_solute, bool)
    m2[nonq[:7]] = True
    gcs = [(np.nonzero(m1)[0], "full"), (np.nonzero(m2)[0], "all"), (np.nonzero(m2)[0], "electro")]
    return s, groups, pairs, [m1, m2, m2], gcs


def run(s, prec, xs, groups, pairs, gcs):
    W = len(xs)
    with NonbondedEngine(s, precision=prec, windows=W) as e:
        for w in range(W):
            e.set_lambda(lambdas_for_window(w / max(W - 1, 1), 2), window=w)
        e.set_monitor_groups(groups, pairs)
        e.set_group_contributions(gcs)
        e.set_coordinates_dev(np.stack(xs))
        e.make_pair_lists_dev(**CUT)
        _, EQ, _ = e.compute_dev(sync=True)
        mon = e.monitor_energies(lambdas=[lambdas_for_window(w / max(W - 1, 1), 2) for w in range(W)])
        exc = e.group_exclusions()
        arr = [e.group_contribution_EQ(EQ[w], window=w) for w in range(W)]
    return mon, exc, EQ, arr


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_pair_sets_match_oracle(case, prec):
    s, groups, pairs, masks, gcs = case
    rng = np.random.default_rng(5)
    xs = [s.x + rng.normal(0, 0.05, s.x.shape) for _ in range(3)]
    mon, exc, _, _ = run(s, prec, xs, groups, pairs, gcs)
    for w, x in enumerate(xs):
        ref = monitor_energies(s, x, groups, pairs)
        np.testing.assert_allclose(mon["Vel"][w], ref[..., 0], rtol=1e-11, atol=1e-10)
        np.testing.assert_allclose(mon["Vlj"][w], ref[..., 1], rtol=1e-11, atol=1e-10)
        lam = lambdas_for_window(w / 2, 2)
        np.testing.assert_allclose(mon["Vwsum"][w], (ref[..., 0] + ref[..., 1]) @ lam, rtol=1e-11, atol=1e-10)
        np.testing.assert_allclose(exc[w], group_exclusions(s, x, masks), rtol=1e-11, atol=1e-10)
    assert np.abs(mon["Vel"]).min() > 0 and np.abs(exc[:, :, :, 2]).min() > 0


def test_batch_bit_equal_to_single(case):
    s, groups, pairs, _, gcs = case
    rng = np.random.default_rng(6)
    xs = [s.x + rng.normal(0, 0.05, s.x.shape) for _ in range(3)]
    mon, exc, _, _ = run(s, PREC_MIXED, xs, groups, pairs, gcs)
    mon1, exc1, _, _ = run(s, PREC_MIXED, xs[2:], groups, pairs, gcs)
    assert np.array_equal(mon["Vel"][2], mon1["Vel"][0]) and np.array_equal(mon["Vlj"][2], mon1["Vlj"][0])
    assert np.array_equal(exc[2], exc1[0])


def test_energy_file_arrays(case, tmp_path):
    s, groups, pairs, masks, gcs = case
    mon, exc, EQ, arr = run(s, PREC_FP64, [s.x], groups, pairs, gcs)
    EQa, hdr = arr[0]
    assert hdr.arrays == 1 + 1 + 3 + 1 and hdr.gcnum == [-1, 1, 2, 2, 2, 3]
    p = tmp_path / "gc.en"
    lam = lambdas_for_window(0.0, 2)
    with EnergyFileWriter(p, 2, header=hdr) as f:
        f.write_step(lam, EQa)
    ef = read_energy_file(p, 2)
    full = EQ[0]
    # array 2: group 1 'full'; arrays 3-5: group 2 'all' (full, electro, vdw); array 6: group 3 'electro'
    np.testing.assert_allclose(ef.qq[0, :, 0, 0], full[:, 0])
    np.testing.assert_allclose(ef.qq[0, :, 1, 0], full[:, 0] - exc[0, 0, :, 0])
    np.testing.assert_allclose(ef.qp[0, :, 1, 1], full[:, 3] - exc[0, 0, :, 3])
    np.testing.assert_allclose(ef.qp[0, :, 3, 0], full[:, 2] - exc[0, 1, :, 2])
    np.testing.assert_allclose(ef.qp[0, :, 3, 1], full[:, 3])
    np.testing.assert_allclose(ef.qp[0, :, 4, 1], full[:, 3] - exc[0, 1, :, 3])
    np.testing.assert_allclose(ef.qp[0, :, 4, 0], full[:, 2])
    np.testing.assert_allclose(ef.qp[0, :, 5, 0], full[:, 2] - exc[0, 2, :, 2])
    qx = full[:, 0] + full[:, 2] + full[:, 4] - exc[0, 0, :, 0] - exc[0, 0, :, 2] \
        + full[:, 1] + full[:, 3] + full[:, 5] - exc[0, 0, :, 1] - exc[0, 0, :, 3]
    np.testing.assert_allclose(ef.total[0, :, 1], qx)


def test_after_md_run(case):
    s, groups, pairs, masks, gcs = case
    with NonbondedEngine(s, precision=PREC_MIXED, windows=1) as e:
        e.set_lambda([0.5, 0.5])
        e.set_monitor_groups(groups, pairs)
        e.set_group_contributions(gcs)
        e.set_coordinates_dev(s.x[None])
        e.md_init(MdSetup(stepsize=0.5, nbcycle=5, cut=CUT))
        e.md_set_velocities(maxwell_velocities(s, 300.0, 3)[None])
        e.md_prepare(stop_cm=True)
        e.md_run(6)
        mon = e.monitor_energies()
        exc = e.group_exclusions()
        x, _ = e.md_state(0)
    # a step evaluates at its start coordinates: the run's last values belong
    # to the coordinates one step before the final ones; a fresh evaluation
    # at the final coordinates is compared with the oracle
    with NonbondedEngine(s, precision=PREC_MIXED, windows=1) as e2:
        e2.set_lambda([0.5, 0.5])
        e2.set_monitor_groups(groups, pairs)
        e2.set_group_contributions(gcs)
        e2.set_coordinates_dev(x[None])
        e2.make_pair_lists_dev(**CUT)
        e2.compute_dev(sync=True)
        mon2 = e2.monitor_energies()
    ref = monitor_energies(s, x, groups, pairs)
    np.testing.assert_allclose(mon2["Vel"][0], ref[..., 0], rtol=1e-11, atol=1e-10)
    # the run's last evaluation is one step behind and close to it
    np.testing.assert_allclose(mon["Vel"][0], ref[..., 0], rtol=0.05, atol=0.5)
    assert np.isfinite(exc).all()


def test_monitor_rejects_bad_groups(case):
    s, groups, pairs, _, _ = case
    with NonbondedEngine(s, precision=PREC_FP64, windows=1) as e:
        with pytest.raises(QnbError):
            e.set_monitor_groups([[0, 1], [1, 2]], [(0, 1)])
        with pytest.raises(QnbError):
            e.set_monitor_groups([[0, 1], [s.nat_solute]], [(0, 1)])
        with pytest.raises(QnbError):
            e.set_monitor_groups([[0, 1], [2]], [(0, 2)])
        e.set_monitor_groups([], [])
        assert e.monitor_energies()["Vel"].shape == (1, 0, 2)
