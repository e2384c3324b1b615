"""The allocation-free water-water entry point against the regular one.

qnb_ww_spc_noalloc exists for callers that may not allocate device memory
(a fixed memory budget, work recorded into a CUDA graph, another allocator
owning the device).  Its scratch is a static device array shared by all calls.
Two calls in a row must both reproduce what qnb_pot_energy_nonbonds gives for
the same water droplet (FP64 form, LRF off, so the energy and gradient are
the ww terms only), within the FP64 tolerance of the other parity tests:
1e-6 kcal/mol on energies and 1e-6 relative on the gradient.  This file is
collected last so a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_ww_matches_pot_energy_nonbonds_on_two_calls():
    torch = pytest.importorskip("torch")
    from q6_gb300 import build as qbuild
    qbuild.build()
    from q6_gb300.qnb import PREC_FP64, NonbondedEngine, load_library
    from q6_gb300.system import make_system

    s = make_system(R=14.0, n_solute=0, nq=0, nstates=1, seed=21, excl_radius=13.0)
    with NonbondedEngine(s, precision=PREC_FP64, use_lrf=False) as eng:
        eng.set_lambda([1.0])
        eng.make_pair_lists(s.x, Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
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
    scale = np.maximum(np.abs(d_ref), np.median(np.abs(d_ref)))
    for call in range(2):
        d = torch.zeros_like(x)
        e = torch.zeros(2, dtype=torch.float64, device=dev)
        rc = lib.qnb_ww_spc_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(excl.data_ptr()),
                                    s.nat_solute, s.nwat, float(s.crg[o]), float(s.crg[h]), A, B, 100.0,
                                    ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(e.data_ptr()), stream)
        assert rc == 0, lib.qnb_last_error().decode()
        torch.cuda.synchronize()
        e_h = e.cpu().numpy()
        assert abs(e_h[0] - E_ref["ww_el"]) <= 1e-6, (call, e_h, E_ref)
        assert abs(e_h[1] - E_ref["ww_vdw"]) <= 1e-6, (call, e_h, E_ref)
        d_h = d.cpu().numpy()
        assert np.all(np.abs(d_h - d_ref) <= 1e-6 * scale + 1e-9), call
