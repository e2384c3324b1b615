"""offdiag (src/nonbondene.f90:6238-6260) on the GPU: Hij = A exp(-mu r_kl)
of Q-atom pairs per window, against numpy on the same coordinates, and the
OFFD records written to and read back from a qdyn energy file."""
import numpy as np
import pytest

from q6_gb300.enefile import EnergyFileWriter, read_energy_file
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.system import lambdas_for_window, make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_offdiag(prec, tmp_path):
    s = make_system(R=12.0, n_solute=30, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2, seed=77)
    rows = [(0, 1, 0, 3, 25.0, 0.5), (0, 1, 2, 5, 12.5, 0.8), (1, 0, 1, 4, 3.0, 0.0)]
    W = 3
    rng = np.random.default_rng(4)
    xs = np.stack([s.x + rng.normal(0, 0.05, s.x.shape) for _ in range(W)])
    with NonbondedEngine(s, precision=prec, windows=W) as e:
        for w in range(W):
            e.set_lambda(lambdas_for_window(w / 2, 2), window=w)
        e.set_offdiag(rows)
        e.set_coordinates_dev(xs)
        e.make_pair_lists_dev(**CUT)
        _, EQ, _ = e.compute_dev(sync=True)
        Hij, rkl = e.offdiag()
        recs = e.offd_records(window=1)
    for w in range(W):
        for k, (_, _, qk, ql, A, mu) in enumerate(rows):
            r = np.linalg.norm(xs[w][s.iqseq[qk]] - xs[w][s.iqseq[ql]])
            assert rkl[w, k] == pytest.approx(r, rel=1e-14)
            assert Hij[w, k] == pytest.approx(A * np.exp(-mu * r), rel=1e-13)
    p = tmp_path / "w1.en"
    with EnergyFileWriter(p, 2) as f:
        f.write_step(lambdas_for_window(0.5, 2), EQ[1], offd=recs)
    ef = read_energy_file(p, 2)
    o = ef.offd[0]
    assert o["i"].tolist() == [1, 1, 2] and o["j"].tolist() == [2, 2, 1]
    assert np.array_equal(o["Hij"], Hij[1]) and np.array_equal(o["rkl"], rkl[1])
