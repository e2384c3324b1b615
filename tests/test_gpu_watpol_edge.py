"""watpol at a water whose dipole is a few 1e-5 rad off the radial vector:
the mixed form's force stays finite and within the usual bar of the FP64
form.  (An FP32 arc cosine of the rounded cosine gave theta = 0 there, and
the force's 1/sin(theta) turned an O(theta) vector difference into a spike
of ~1e8 kcal/mol/A.)"""
import numpy as np
import pytest

from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.system import default_solvent_params, make_system

pytestmark = pytest.mark.gpu


def rot(axis, ang):
    axis = axis / np.linalg.norm(axis)
    k = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(ang) * k + (1 - np.cos(ang)) * k @ k


@pytest.mark.parametrize("offset", [3e-5, 2e-4, 1e-3])
def test_near_radial_water(offset):
    s = make_system(R=14.0, n_solute=30, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2, seed=9191)
    sp = default_solvent_params(s)
    x = s.x.copy()
    o0 = s.nat_solute
    r = np.linalg.norm(x[o0::3][: s.nwat] - s.xwcent, axis=1)
    w = int(np.argmin(np.abs(r - (s.rwat - 1.0))))   # a water inside the polarisation shells
    o = s.nat_solute + 3 * w
    u = x[o + 1] + x[o + 2] - 2 * x[o]
    q = x[o] - s.xwcent
    axis = np.cross(u, q)
    ang = np.arccos(np.clip(u @ q / np.linalg.norm(u) / np.linalg.norm(q), -1, 1))
    R = rot(axis, ang) if np.linalg.norm(axis) > 0 else np.eye(3)
    perp = np.cross(q, [1.0, 0.0, 0.0])
    R = rot(perp, offset) @ R
    for a in (1, 2):
        x[o + a] = x[o] + R @ (x[o + a] - x[o])
    out = {}
    for prec in (PREC_FP64, PREC_MIXED):
        with NonbondedEngine(s, precision=prec) as e:
            e.set_solvent_params(sp)
            d, E, EQ, R2 = e.evaluate(x, [0.5, 0.5], cut=dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0),
                                       solvent=sp)
        out[prec] = (d, R2)
    d64, d32 = out[PREC_FP64][0], out[PREC_MIXED][0]
    assert np.all(np.isfinite(d32))
    med = float(np.median(np.linalg.norm(d64, axis=1)))   # the suite's gradient bar: 2e-3 of max(|F_i|, median |F|)
    for a in range(3):
        assert np.linalg.norm(d32[o + a] - d64[o + a]) <= 2e-3 * max(med, np.linalg.norm(d64[o + a])), a
    assert abs(out[PREC_MIXED][1][1] - out[PREC_FP64][1][1]) <= 1e-3 * max(1.0, abs(out[PREC_FP64][1][1]))
