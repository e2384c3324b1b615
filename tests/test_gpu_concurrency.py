"""The mixed form's evaluation branches (qnb_set_concurrency): with the water
rows, Q-environment, LRF Taylor, restraint and watpol kernels running beside
the solute rows, every sum is still fixed point, so energies and gradients
equal the single-stream run bit for bit, on the sphere (graph replay and
kernel by kernel, several steps across a watpol update) and in a periodic
box."""
import numpy as np
import pytest

from q6_gb300.qnb import PREC_MIXED, NonbondedEngine
from q6_gb300.system import config_small, default_solvent_params, lambdas_for_window

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


def run(s, branches, graphs, box=None, nsteps=4):
    W = 3
    rng = np.random.default_rng(8)
    xs = np.stack([s.x + rng.normal(0.0, 0.02, s.x.shape) for _ in range(W)])
    out = []
    with NonbondedEngine(s, precision=PREC_MIXED, windows=W, use_lrf=True) as e:
        if box is None:
            e.set_solvent_params(default_solvent_params(s, itdis=2.0))
        else:
            e.set_box(box)
        e.set_concurrency(branches)
        e.set_graphs(graphs)
        for w in range(W):
            e.set_lambda(lambdas_for_window(0.2 + 0.3 * w, s.nstates), window=w)
        e.set_coordinates_dev(xs)
        cut = CUT if box is None else dict(CUT, Rcq=12.0, RcLRF=12.0)
        e.make_pair_lists_dev(**cut)
        for k in range(nsteps):
            E, EQ, R = e.compute_dev(Tfree=300.0, istep=k, sync=True)
            out.append((E, EQ.copy(), R.copy(), e.gradient_dev()))
    return out


@pytest.mark.parametrize("graphs", [True, False])
def test_branches_equal_single_stream_sphere(graphs):
    s = config_small()
    a, b = run(s, True, graphs), run(s, False, graphs)
    for (E1, EQ1, R1, D1), (E0, EQ0, R0, D0) in zip(a, b):
        assert E1 == E0 and np.array_equal(EQ1, EQ0) and np.array_equal(R1, R0) and np.array_equal(D1, D0)
    assert any(r[2][:, 1].any() for r in a)   # watpol contributed


def test_branches_equal_single_stream_box():
    s = config_small()
    a, b = run(s, True, True, box=[40.0] * 3), run(s, False, True, box=[40.0] * 3)
    for (E1, EQ1, R1, D1), (E0, EQ0, R0, D0) in zip(a, b):
        assert E1 == E0 and np.array_equal(EQ1, EQ0) and np.array_equal(D1, D0)
