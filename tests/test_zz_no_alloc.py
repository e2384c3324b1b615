"""The allocation-free water-water entry point, qnb_ww_spc_noalloc.

It exists for callers that may not allocate device memory while they run: a
program held to a fixed device-memory budget by its scheduler or by the
application that embeds it, a process whose own pool allocator already holds
the device's free memory, or a timed step loop in which cudaMalloc would
synchronise the device.  Its scratch is a static device array that all calls
share.

Two calls in a row must both reproduce the water-water energies and gradient
of the CPU oracle (nbwwlist + nonbond_ww_spc in FP64) and of the regular entry
point qnb_pot_energy_nonbonds on the same droplet (FP64 form, LRF off, so the
energies and gradient are the ww terms only), within the FP64 tolerance of the
other parity tests: 1e-6 kcal/mol on energies and 1e-6 relative on the
gradient.  Sizes beyond the scratch must come back as QNB_ERR_CAPACITY.  This
file is collected last so a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QNB_ERR_CAPACITY = 3


def _call(lib, x, excl, first, nwat, qO, qH, A, B, rc2, d, e, stream):
    return lib.qnb_ww_spc_noalloc(ctypes.c_void_p(x.data_ptr()),
                                  ctypes.c_void_p(excl.data_ptr()) if excl is not None else None,
                                  first, nwat, qO, qH, A, B, rc2,
                                  ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(e.data_ptr()), stream)


def test_noalloc_ww_matches_oracle_and_pot_energy_nonbonds_on_two_calls():
    torch = pytest.importorskip("torch")
    from q6_gb300 import build as qbuild
    qbuild.build()
    from oracle.oracle import Oracle
    from q6_gb300.qnb import PREC_FP64, NonbondedEngine, load_library
    from q6_gb300.system import make_system

    s = make_system(R=14.0, n_solute=0, nq=0, nstates=1, seed=21, excl_radius=13.0)
    cut = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
    orc = Oracle(s, use_lrf=False)
    orc.set_lambda([1.0])
    orc.make_pair_lists(s.x, **cut)
    d_orc, E_orc, _ = orc.pot_energy_nonbonds(s.x)
    orc.close()
    with NonbondedEngine(s, precision=PREC_FP64, use_lrf=False) as eng:
        eng.set_lambda([1.0])
        eng.make_pair_lists(s.x, **cut)
        d_ref, E_ref, _ = eng.pot_energy_nonbonds(s.x)
    o, h = s.nat_solute, s.nat_solute + 1
    t_o = int(s.iac[o])
    A = float(s.avdw[t_o, 0] * s.avdw[t_o, 0])   # ww_precomp O-O, geometric rule, LJ code 1
    B = float(s.bvdw[t_o, 0] * s.bvdw[t_o, 0])
    lib = load_library()
    dev = torch.device("cuda", 0)
    x = torch.tensor(s.x, dtype=torch.float64, device=dev).contiguous()
    excl = torch.tensor(s.excl, dtype=torch.uint8, device=dev).contiguous()
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    for call in range(2):
        d = torch.zeros_like(x)
        e = torch.zeros(2, dtype=torch.float64, device=dev)
        rc = _call(lib, x, excl, s.nat_solute, s.nwat, float(s.crg[o]), float(s.crg[h]), A, B, 100.0, d, e, stream)
        assert rc == 0, lib.qnb_last_error().decode()
        torch.cuda.synchronize()
        e_h = e.cpu().numpy()
        d_h = d.cpu().numpy()
        for name, E0, d0 in (("oracle", E_orc, d_orc), ("qnb_pot_energy_nonbonds", E_ref, d_ref)):
            assert abs(e_h[0] - E0["ww_el"]) <= 1e-6, (name, call, e_h, E0)
            assert abs(e_h[1] - E0["ww_vdw"]) <= 1e-6, (name, call, e_h, E0)
            scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
            assert np.all(np.abs(d_h - d0) <= 1e-6 * scale + 1e-9), (name, call)


def test_noalloc_ww_rejects_sizes_beyond_the_scratch():
    """More than 65,536 waters is refused before any device work; more than
    1,048,576 water pairs within the cut-off (1,500 waters on a 3.1 A lattice,
    every pair inside a 1,000 A cut-off: 1,124,250 pairs) is refused after the
    selection, whose writes past the array are skipped.  The outputs stay
    untouched and a regular call afterwards still gives the right answer."""
    torch = pytest.importorskip("torch")
    from q6_gb300 import build as qbuild
    qbuild.build()
    from q6_gb300.qnb import load_library
    lib = load_library()
    dev = torch.device("cuda", 0)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    nwat = 1500
    g = np.arange(12) * 3.1
    ox = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)[:nwat]   # 3.1 A lattice
    xs = np.repeat(ox, 3, axis=0)
    xs[1::3] += (1.0, 0.0, 0.0)
    xs[2::3] += (-0.33, 0.94, 0.0)
    x = torch.tensor(xs, dtype=torch.float64, device=dev).contiguous()
    d = torch.zeros_like(x)
    e = torch.zeros(2, dtype=torch.float64, device=dev)
    args = (-0.82, 0.41, 629.4 ** 2, 24.97 ** 2)
    # too many waters: refused on the host, no device access
    rc = _call(lib, x, None, 0, 65537, *args, 100.0, d, e, stream)
    assert rc == QNB_ERR_CAPACITY, rc
    assert "65536" in lib.qnb_last_error().decode()
    # too many pairs within the cut-off
    rc = _call(lib, x, None, 0, nwat, *args, 1.0e6, d, e, stream)
    assert rc == QNB_ERR_CAPACITY, rc
    assert "1048576" in lib.qnb_last_error().decode()
    torch.cuda.synchronize()
    assert float(d.abs().max()) == 0.0 and float(e.abs().max()) == 0.0
    # the next call within limits is unaffected by the refused one
    rc = _call(lib, x, None, 0, nwat, *args, 100.0, d, e, stream)
    assert rc == 0, lib.qnb_last_error().decode()
    torch.cuda.synchronize()
    # closed-form check of the same sum on the CPU (O-O LJ + 9 Coulomb terms per pair)
    q = np.array([-0.82, 0.41, 0.41])
    io = np.arange(nwat) * 3
    dO = xs[io][:, None, :] - xs[io][None, :, :]
    r2 = (dO ** 2).sum(-1)
    iu, ju = np.nonzero(np.triu(r2 <= 100.0, 1))
    el = 0.0
    for a in range(3):
        for b in range(3):
            rv = xs[3 * ju + b] - xs[3 * iu + a]
            el += float((q[a] * q[b] / np.sqrt((rv ** 2).sum(-1))).sum())
    r6 = r2[iu, ju] ** 3
    vdw = float((args[2] / r6 ** 2 - args[3] / r6).sum())
    e_h = e.cpu().numpy()
    assert abs(e_h[0] - el) <= 1e-6 * max(1.0, abs(el)), (e_h, el)
    assert abs(e_h[1] - vdw) <= 1e-6 * max(1.0, abs(vdw)), (e_h, vdw)
