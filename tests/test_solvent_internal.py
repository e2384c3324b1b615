"""The solvent-internal pair list (prep_sim_precompute_solvent restated in
q6_gb300.solvent) on a five-atom chain solvent, against the list written out
by hand from src/simprep.f90:4003-4125, and the oracle's
nonbond_solvent_internal against a direct numpy evaluation."""
import numpy as np

from oracle.oracle import Oracle
from q6_gb300.solvent import solvent_internal_pairs
from q6_gb300.system import config_small


def test_chain_solvent_list_matches_hand_derivation():
    iac = [0, 1, 0, 1, 0]
    ljcod = [[1, 2], [2, 1]]
    avdw = [[10.0, 11.0, 12.0], [20.0, 21.0, 22.0]]
    bvdw = [[1.0, 1.1, 1.2], [2.0, 2.1, 2.2]]
    crg = [0.3, -0.2, 0.1, -0.4, 0.2]
    bonds = [(0, 1), (1, 2), (2, 3), (3, 4)]
    angles = [(0, 1, 2), (1, 2, 3), (2, 3, 4)]
    torsions = [(0, 1, 2, 3), (1, 2, 3, 4)]
    pairs, A, B, el = solvent_internal_pairs(iac, ljcod, avdw, bvdw, crg, 0.5, 1, bonds, angles, torsions)
    # left after bonds and angles: (0,3), (0,4), (1,4) and their mirrors;
    # torsion ends (0,3) and (1,4) become 1-4 one way, the mirror is dropped;
    # (0,4) is listed both ways (types 0-0: code ljcod[0][0] = 1)
    assert pairs.tolist() == [[0, 3], [0, 4], [1, 4], [4, 0]]
    want = [(avdw[0][2] * avdw[1][2], bvdw[0][2] * bvdw[1][2], 0.3 * -0.4 * 0.5),
            (avdw[0][0] * avdw[0][0], bvdw[0][0] * bvdw[0][0], 0.3 * 0.2),
            (avdw[1][2] * avdw[0][2], bvdw[1][2] * bvdw[0][2], -0.2 * 0.2 * 0.5),
            (avdw[0][0] * avdw[0][0], bvdw[0][0] * bvdw[0][0], 0.2 * 0.3)]
    assert np.allclose(np.stack([A, B, el], 1), want, rtol=0, atol=1e-15)
    # arithmetic rule for the first pair
    _, A2, B2, _ = solvent_internal_pairs(iac, ljcod, avdw, bvdw, crg, 0.5, 2, bonds, angles, torsions)
    t = (avdw[0][2] + avdw[1][2]) ** 6
    assert np.isclose(A2[0], t * t * bvdw[0][2] * bvdw[1][2]) and np.isclose(B2[0], 2 * t * bvdw[0][2] * bvdw[1][2])


def test_oracle_solvent_internal_matches_numpy():
    s = config_small()
    pairs = np.array([[0, 1], [1, 0], [1, 2]], dtype=np.int32)
    A = np.array([300.0, 0.0, 55.0])
    B = np.array([20.0, 0.0, 3.0])
    el = np.array([0.4, -0.2, 0.15])
    o = Oracle(s, use_lrf=False)
    o.make_pair_lists(s.x)
    d0, E0, _ = o.pot_energy_nonbonds(s.x)
    o.set_solvent_internal(pairs, A, B, el)
    d1, E1, _ = o.pot_energy_nonbonds(s.x)
    eel = evdw = 0.0
    grad = np.zeros_like(s.x)
    for iw in range(s.nwat):
        base = s.nat_solute + 3 * iw
        for (i, j), a, b, q in zip(pairs, A, B, el):
            v = s.x[base + j] - s.x[base + i]
            r2 = 1.0 / (v @ v)
            r = np.sqrt(r2)
            vel, va, vb = q * r, a * r2 ** 6, b * r2 ** 3
            dv = r2 * (-vel) + r2 * (-12 * va + 6 * vb)
            eel += vel
            evdw += va - vb
            grad[base + i] -= v * dv
            grad[base + j] += v * dv
    assert np.isclose(E1["ww_el"] - E0["ww_el"], eel, rtol=1e-12, atol=1e-9)
    assert np.isclose(E1["ww_vdw"] - E0["ww_vdw"], evdw, rtol=1e-12, atol=1e-9)
    assert np.allclose(d1 - d0, grad, rtol=1e-9, atol=1e-9)
