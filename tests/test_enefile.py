"""Energy files in qdyn's put_ene layout and Qfep's summary read from them.

The reference ships no binary energy file, so the layout is pinned to the
write statements (src/simprep.f90:4165-4167, src/nrgy.f90:147-153): record
lengths and field offsets are checked byte by byte, then round trips, a
closed-form dG and agreement with the in-memory Zwanzig sums."""
import struct

import numpy as np
import pytest

from q6_gb300.enefile import (CANARY_DOUBLE, FULL, NOGC, VDW, EnergyFileWriter, EnergyHeader, qfep_files,
                              read_energy_file, state_record)
from q6_gb300.fep import BOLTZ, qfep_dg


def test_default_header_bytes():
    b = EnergyHeader(version="5.10 test").pack()
    n = 3 * 4 + 4 + 4 + 2 * 4 + 4 + 80   # canary arrays totresid types numres resid(2) gcnum version
    assert struct.unpack_from("<i", b, 0)[0] == n and struct.unpack_from("<i", b, 4 + n)[0] == n
    assert struct.unpack_from("<3i", b, 4) == (CANARY_DOUBLE, 1, 2)
    assert struct.unpack_from("<5i", b, 16) == (NOGC, 1, -1, -1, -1)
    assert b[36:36 + 80] == b"5.10 test".ljust(80, b" ")
    assert len(b) == n + 8


def test_state_record_bytes():
    eq = [1.0, 2.0, 3.0, 4.0, 5.0, 6.0]   # qq el/vdw, qp el/vdw, qw el/vdw
    b = state_record(2, 0.25, eq, q_bonded=[0.5, 0.25, 0.125, 0.0625], restraint=[7.0])
    n = 4 + 8 + 8 * (1 + 4 + 2 + 2 + 2 + 2 + 1)
    assert struct.unpack_from("<i", b, 0)[0] == n and len(b) == n + 8
    idx, lam = struct.unpack_from("<id", b, 4)
    assert (idx, lam) == (2, 0.25)
    v = np.frombuffer(b, "<f8", 14, 16)
    qx = (1.0 + 3.0 + 5.0, 2.0 + 4.0 + 6.0)
    assert v[0] == 0.5 + 0.25 + 0.125 + 0.0625 + qx[0] + qx[1] + 7.0   # total, src/potene.f90:229-231
    assert list(v[1:5]) == [0.5, 0.25, 0.125, 0.0625]
    assert tuple(v[5:7]) == qx
    assert list(v[7:13]) == eq and v[13] == 7.0


def write_windows(tmp_path, EQ, lams, header=None):
    """EQ[w][frame][s][arrays*6]"""
    paths = []
    for w in range(len(EQ)):
        p = tmp_path / ("win%02d.en" % w)
        with EnergyFileWriter(p, len(lams[w]), header) as f:
            for fr in EQ[w]:
                f.write_step(lams[w], fr)
        paths.append(p)
    return paths


def test_round_trip_and_offdiagonals(tmp_path):
    rng = np.random.default_rng(5)
    S, npts = 3, 7
    eq = rng.normal(0.0, 50.0, (npts, S, 6))
    lam = [0.2, 0.3, 0.5]
    p = tmp_path / "a.en"
    offd = [(1, 2, -12.5, 2.25), (2, 3, 3.0, 1.5)]
    qb = rng.normal(0.0, 5.0, (S, 4))
    with EnergyFileWriter(p, S) as f:
        for k in range(npts):
            f.write_step(lam, eq[k], q_bonded=qb, restraint=[1.0, 2.0, 3.0], offd=offd)
    ef = read_energy_file(p, S)
    assert ef.total.shape == (npts, S, 1) and np.array_equal(ef.lambdas, lam)
    assert np.array_equal(ef.qq[:, :, 0], eq[:, :, 0:2]) and np.array_equal(ef.qp[:, :, 0], eq[:, :, 2:4])
    assert np.array_equal(ef.qw[:, :, 0], eq[:, :, 4:6])
    assert np.array_equal(ef.q[:, :, 0], np.broadcast_to(qb, (npts, S, 4)))
    assert np.allclose(ef.total[:, :, 0], qb.sum(-1) + eq.sum(-1) + np.array([1.0, 2.0, 3.0]), rtol=0, atol=1e-10)
    assert all(o.shape == (2,) and o["Hij"][0] == -12.5 and o["j"][1] == 3 for o in ef.offd)


def test_truncated_step_is_dropped(tmp_path):
    p = write_windows(tmp_path, [np.ones((3, 2, 6))], [[0.5, 0.5]])[0]
    raw = p.read_bytes()
    rec = 8 + 4 + 8 + 8 * 14
    p.write_bytes(raw[:-(8 + rec)])   # the last step loses its second state and off-diagonal record
    assert read_energy_file(p, 2).total.shape[0] == 2


def test_multi_array_header_round_trip(tmp_path):
    h = EnergyHeader(arrays=3, types=[NOGC, FULL, VDW], numres=[1, 2, 2], resid=[-1, 11, 12, 11, 12],
                     gcnum=[-1, 1, 1], version="gc")
    rng = np.random.default_rng(9)
    eq = rng.normal(0.0, 10.0, (2, 4, 2, 3 * 6))
    paths = write_windows(tmp_path, eq, [[1.0, 0.0], [0.0, 1.0]], header=h)
    ef = read_energy_file(paths[1], 2)
    assert ef.header == h
    assert np.array_equal(ef.qw[:, :, 2], eq[1].reshape(4, 2, 3, 6)[:, :, 2, 4:6])


def test_bad_canary_and_precision(tmp_path):
    p = tmp_path / "x.en"
    p.write_bytes(EnergyHeader(canary=137).pack())
    with pytest.raises(ValueError, match="precision"):
        read_energy_file(p, 2)
    p.write_bytes(EnergyHeader(canary=42).pack())
    with pytest.raises(ValueError, match="canary"):
        read_energy_file(p, 2)


def test_constant_gap_gives_closed_form_dg(tmp_path):
    """Two end-state windows whose state energies differ by a constant c on
    every frame: dGf = c, dGr = -c, dG = c; an alfa shift on state 2 adds to it."""
    c = 1.75
    rng = np.random.default_rng(1)
    base = rng.normal(0.0, 3.0, (2, 6, 1))
    eq = np.zeros((2, 6, 2, 6))
    eq[:, :, 0, 0] = base[:, :, 0]
    eq[:, :, 1, 0] = base[:, :, 0] + c
    paths = write_windows(tmp_path, eq, [[1.0, 0.0], [0.0, 1.0]])
    _, dgf, dgr, dg = qfep_files(paths, 2, rt=BOLTZ * 300.0)
    assert dgf[0] == pytest.approx(c, abs=1e-12) and dgr[1] == pytest.approx(-c, abs=1e-12)
    assert dg[1] == pytest.approx(c, abs=1e-12)
    _, _, _, dg2 = qfep_files(paths, 2, rt=BOLTZ * 300.0, alfa=[9.0, 0.5])
    assert dg2[1] == pytest.approx(c + 0.5, abs=1e-12)


def test_qfep_files_matches_in_memory_sums(tmp_path):
    rng = np.random.default_rng(77)
    W, npts = 6, 20
    lams = [[1.0 - l, l] for l in np.linspace(0.0, 1.0, W)]
    eq = rng.normal(0.0, 0.6, (W, npts, 2, 6))
    paths = write_windows(tmp_path, eq, lams)
    rt = 0.5922
    for nskip in (0, 5):
        lam, dgf, dgr, dg = qfep_files(paths, 2, rt=rt, nskip=nskip)
        v = [eq[w, nskip:].sum(-1) for w in range(W)]
        f0, r0, g0 = qfep_dg(v, lams, rt)
        assert np.allclose(lam, lams)
        assert np.allclose(dgf, f0, rtol=1e-12, atol=1e-12) and np.allclose(dg, g0, rtol=1e-12, atol=1e-12)
    with pytest.raises(ValueError, match="skip"):
        qfep_files(paths, 2, nskip=npts)
    # gas phase: total = bonded + qq + restraint only
    _, _, _, dgg = qfep_files(paths, 2, rt=rt, gas=True)
    _, _, g1 = qfep_dg([eq[w][:, :, 0:2].sum(-1) for w in range(W)], lams, rt)
    assert np.allclose(dgg, g1, rtol=1e-12, atol=1e-12)
