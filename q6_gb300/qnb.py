"""Python host mirror of qdyn's nonbonded call sequence over the C ABI.

``NonbondedEngine`` exposes the reference routines this library replaces with
the same names and argument meaning (Q6 src/nonbondene.f90, src/potene.f90):
``make_pair_lists``, ``pot_energy_nonbonds``, ``nonbond_qq``,
``restrain_solvent`` and ``watpol``.  Gradients are ADDED into the array the
caller passes, energies are returned per term and per FEP state.

There is no CPU path: without the CUDA library or a CUDA device the
constructor raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .system import QnbSolventParams, QSystem, TopologyHandle

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqnb.so")

PREC_FP64 = 0
PREC_MIXED = 1
LIST_PP, LIST_PW, LIST_WW, LIST_QP, LIST_QW, LIST_PP14 = range(6)
ROWS_GP, ROWS_GW, ROWS_WW, ROWS_WG = range(4)

E_FIELDS = ("pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw", "lrf")
Q_FIELDS = ("qq_el", "qq_vdw", "qp_el", "qp_vdw", "qw_el", "qw_vdw")

EXPORTED = (
    "qnb_last_error", "qnb_version", "qnb_create", "qnb_destroy", "qnb_set_lambda",
    "qnb_make_pair_lists", "qnb_pot_energy_nonbonds", "qnb_nonbond_qq",
    "qnb_set_solvent_params", "qnb_restrain_solvent", "qnb_watpol", "qnb_get_watpol_state",
    "qnb_list_size", "qnb_export_pairs", "qnb_export_rows", "qnb_get_lrf", "qnb_device_buffers", "qnb_stream",
    "qnb_make_pair_lists_dev", "qnb_compute_dev", "qnb_pot_energy_step", "qnb_step_host", "qnb_take_launch_count",
    "qnb_profile", "qnb_kernel_times", "qnb_create_batch", "qnb_window_count",
    "qnb_set_lambda_window", "qnb_upload_coordinates", "qnb_download_gradient",
    "qnb_ww_spc_noalloc", "qnb_q_adjoint_dev", "qnb_get_energies_dev", "qnb_set_graphs", "qnb_set_concurrency",
    "qnb_group_create", "qnb_group_compute", "qnb_group_destroy", "qnb_profile_collect",
    "qnb_profile_classes", "qnb_set_solvent_internal", "qnb_autotune", "qnb_get_tuning", "qnb_set_tuning",
    "qnb_md_init", "qnb_md_set_velocities", "qnb_md_get_state", "qnb_md_prepare", "qnb_md_run",
    "qnb_set_bonded", "qnb_get_bonded_energies", "qnb_md_minimize", "qnb_set_shell_restraint",
    "qnb_get_restraint_energies", "qnb_set_offdiag", "qnb_get_offdiag", "qnb_set_restraints",
    "qnb_set_monitor_groups", "qnb_get_monitor_energies", "qnb_set_group_exclusions", "qnb_get_group_exclusions",
    "qnb_set_box", "qnb_set_freeze", "qnb_md_set_thermostat", "qnb_md_set_langevin",
    "qnb_set_put_back_in_box", "qnb_put_back_in_box",
)
TUNE_NAMES = ("rows_solute_blocks_per_sm", "rows_water_blocks_per_sm", "qp_blocks_per_sm", "qw_blocks_per_sm",
              "q_chunk_units", "lrf_taylor_blocks_per_sm", "lrf_build_blocks_per_sm", "row_build_blocks_per_sm")
KERNEL_CLASSES = ("ww", "qw", "pw", "pp", "qp", "lrf_taylor", "qq", "restrain", "watpol", "pack",
                  "apply", "build", "lrf_build", "bonded", "md")


class QnbError(RuntimeError):
    pass


class QnbOptions(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("use_lrf", ctypes.c_int32),
                ("device", ctypes.c_int32), ("reserved", ctypes.c_int32)]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libqnb.so (built by ``q6_gb300.build``); raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise QnbError(f"CUDA library {path} not built: run `python -m q6_gb300.build`")
    L = ctypes.CDLL(path)
    P, D, I32, I64 = ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_int64
    L.qnb_last_error.restype = ctypes.c_char_p
    L.qnb_version.restype = I32
    sig = {
        "qnb_create": [P, P, P], "qnb_destroy": [P], "qnb_set_lambda": [P, P],
        "qnb_make_pair_lists": [P, P, D, D, D, D, D, D],
        "qnb_make_pair_lists_dev": [P, D, D, D, D, D, D],
        "qnb_pot_energy_nonbonds": [P, P, P, P, P, I32],
        "qnb_nonbond_qq": [P, P, P, P], "qnb_set_solvent_params": [P, P],
        "qnb_restrain_solvent": [P, P, P, D, P], "qnb_watpol": [P, P, P, I32, I32, P],
        "qnb_get_watpol_state": [P, P, P, P], "qnb_list_size": [P, I32, P],
        "qnb_export_pairs": [P, I32, P, P, I64, P], "qnb_get_lrf": [P, P],
        "qnb_export_rows": [P, I32, I32, P, P, I64, P],
        "qnb_device_buffers": [P, P, P], "qnb_stream": [P, P],
        "qnb_compute_dev": [P, D, I32, I32, P, P, P], "qnb_take_launch_count": [P, P],
        "qnb_pot_energy_step": [P, P, P, D, I32, P, P, P],
        "qnb_step_host": [P, P, P, D, I32, I32, P, P, P],
        "qnb_profile": [P, I32], "qnb_kernel_times": [P, P, P, I32],
        "qnb_create_batch": [P, P, I32, P], "qnb_window_count": [P, P],
        "qnb_set_lambda_window": [P, I32, P], "qnb_upload_coordinates": [P, P],
        "qnb_download_gradient": [P, P, I32],
        "qnb_ww_spc_noalloc": [P, P, I32, I32, D, D, D, D, D, P, P, P],
        "qnb_q_adjoint_dev": [P, P, P, P],
        "qnb_get_energies_dev": [P, P, P, P], "qnb_set_graphs": [P, I32], "qnb_set_concurrency": [P, I32],
        "qnb_group_create": [P, I32, P], "qnb_group_compute": [P, D, I32], "qnb_group_destroy": [P],
        "qnb_profile_collect": [P], "qnb_profile_classes": [P, ctypes.c_uint32],
        "qnb_set_solvent_internal": [P, I32, P, P, P, P],
        "qnb_autotune": [P, I32, P], "qnb_get_tuning": [P, P], "qnb_set_tuning": [P, P],
        "qnb_md_init": [P, P, P, I32, P, P, P], "qnb_md_set_velocities": [P, I32, P],
        "qnb_md_get_state": [P, I32, P, P], "qnb_md_prepare": [P, I32], "qnb_md_run": [P, I32, I32, P, P, P],
        "qnb_set_bonded": [P, P], "qnb_get_bonded_energies": [P, P, P],
        "qnb_md_minimize": [P, I32, D, D, D, P],
        "qnb_set_shell_restraint": [P, P, P, D, D], "qnb_get_restraint_energies": [P, P],
        "qnb_set_offdiag": [P, I32, P, P, P, P], "qnb_get_offdiag": [P, P, P], "qnb_set_restraints": [P, P, P],
        "qnb_set_monitor_groups": [P, I32, P, P, I32, P], "qnb_get_monitor_energies": [P, P],
        "qnb_set_group_exclusions": [P, I32, P], "qnb_get_group_exclusions": [P, P],
        "qnb_set_box": [P, P, I32], "qnb_set_freeze": [P, I32], "qnb_md_set_thermostat": [P, I32, I32, I32, D],
        "qnb_md_set_langevin": [P, I32, D, ctypes.c_uint64],
        "qnb_set_put_back_in_box": [P, I32, P, P, I32, I32, I32, P], "qnb_put_back_in_box": [P, P],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    _lib = L
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class NonbondedEngine:
    """One qdyn system on one GPU (one CUDA stream)."""

    def __init__(self, system: QSystem, precision: int = PREC_FP64, use_lrf: bool = True,
                 device: int = 0, windows: int = 1):
        self.lib = load_library()
        self.s = system
        self.S = system.nstates
        self.nwin = int(windows)
        self.use_lrf = bool(use_lrf)
        self.topo = TopologyHandle(system)
        opt = QnbOptions(precision, int(use_lrf), device, 0)
        h = ctypes.c_void_p()
        self._check(self.lib.qnb_create_batch(self.topo.ptr(), ctypes.byref(opt), self.nwin, ctypes.byref(h)))
        self.h = h
        self.precision = precision

    def _check(self, rc):
        if rc != 0:
            raise QnbError(f"qnb error {rc}: {self.lib.qnb_last_error().decode()}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.qnb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- reference routines ---------------------------------------------
    def set_lambda(self, lam, window=None):
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        if not hasattr(self, "lambdas"):
            self.lambdas = np.zeros((self.nwin, self.S))
        self.lambdas[slice(None) if window is None else int(window)] = lam[: self.S]
        if window is None:
            self._check(self.lib.qnb_set_lambda(self.h, _p(lam)))
        else:
            self._check(self.lib.qnb_set_lambda_window(self.h, int(window), _p(lam)))

    def make_pair_lists(self, x, Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0):
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._check(self.lib.qnb_make_pair_lists(self.h, _p(x), Rcq, Rcq ** 2, RcLRF ** 2,
                                                 Rcpp ** 2, Rcpw ** 2, Rcww ** 2))

    def pot_energy_nonbonds(self, x, d=None, md=True):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if d is None:
            d = np.zeros_like(x)
        E = np.zeros(7)
        EQ = np.zeros((max(self.S, 1), 6))
        self._check(self.lib.qnb_pot_energy_nonbonds(self.h, _p(x), _p(d), _p(E), _p(EQ), int(md)))
        return d, dict(zip(E_FIELDS, E)), EQ[: self.S]

    def nonbond_qq(self, x, d=None, EQ=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if d is None:
            d = np.zeros_like(x)
        EQ = np.zeros((max(self.S, 1), 6)) if EQ is None else np.ascontiguousarray(EQ, dtype=np.float64)
        self._check(self.lib.qnb_nonbond_qq(self.h, _p(x), _p(d), _p(EQ)))
        return d, EQ[: self.S]

    def set_solvent_params(self, p: QnbSolventParams):
        self._check(self.lib.qnb_set_solvent_params(self.h, ctypes.byref(p)))

    def restrain_solvent(self, x, d, Tfree):
        e = np.zeros(1)
        self._check(self.lib.qnb_restrain_solvent(self.h, _p(np.ascontiguousarray(x)), _p(d), Tfree, _p(e)))
        return float(e[0])

    def watpol(self, x, d, istep, md=True):
        e = np.zeros(1)
        self._check(self.lib.qnb_watpol(self.h, _p(np.ascontiguousarray(x)), _p(d), int(istep), int(md), _p(e)))
        return float(e[0])

    def watpol_state(self):
        a, b, c = np.zeros(16), np.zeros(16), np.zeros(16)
        self._check(self.lib.qnb_get_watpol_state(self.h, _p(a), _p(b), _p(c)))
        return a, b, c

    # ---- inspection --------------------------------------------------------
    def list_size(self, kind):
        n = ctypes.c_int64()
        self._check(self.lib.qnb_list_size(self.h, kind, ctypes.byref(n)))
        return int(n.value)

    def export_pairs(self, kind):
        n = self.list_size(kind)
        i = np.zeros(max(n, 1), np.int32)
        j = np.zeros(max(n, 1), np.int32)
        m = ctypes.c_int64()
        self._check(self.lib.qnb_export_pairs(self.h, kind, _p(i), _p(j), n, ctypes.byref(m)))
        return i[:m.value], j[:m.value]

    def export_rows(self, kind, win=0):
        """(row, partner) entries of the mixed form's gather rows of one
        window (ROWS_GP / ROWS_GW / ROWS_WW / ROWS_WG)."""
        m = ctypes.c_int64()
        self.lib.qnb_export_rows(self.h, win, kind, None, None, 0, ctypes.byref(m))
        n = int(m.value)
        r = np.zeros(max(n, 1), np.int32)
        p = np.zeros(max(n, 1), np.int32)
        self._check(self.lib.qnb_export_rows(self.h, win, kind, _p(r), _p(p), n, ctypes.byref(m)))
        return r[:m.value], p[:m.value]

    def lrf(self):
        out = np.zeros((self.s.ncgp, 43))
        self._check(self.lib.qnb_get_lrf(self.h, _p(out)))
        return out

    def launches(self):
        n = ctypes.c_int64()
        self._check(self.lib.qnb_take_launch_count(self.h, ctypes.byref(n)))
        return int(n.value)

    def profile(self, enable=True):
        self._check(self.lib.qnb_profile(self.h, int(enable)))

    def kernel_times(self):
        n = len(KERNEL_CLASSES)
        ms = np.zeros(n)
        cnt = np.zeros(n, np.int64)
        self._check(self.lib.qnb_kernel_times(self.h, _p(ms), _p(cnt), n))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(KERNEL_CLASSES)}

    # ---- device-resident interface ------------------------------------------
    def device_buffers(self):
        x = ctypes.c_void_p()
        d = ctypes.c_void_p()
        self._check(self.lib.qnb_device_buffers(self.h, ctypes.byref(x), ctypes.byref(d)))
        return x.value, d.value

    def stream(self):
        st = ctypes.c_void_p()
        self._check(self.lib.qnb_stream(self.h, ctypes.byref(st)))
        return st.value

    def make_pair_lists_dev(self, Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0):
        self._check(self.lib.qnb_make_pair_lists_dev(self.h, Rcq, Rcq ** 2, RcLRF ** 2, Rcpp ** 2,
                                                     Rcpw ** 2, Rcww ** 2))

    def pot_energy_step(self, x, d=None, Tfree=300.0, istep=0):
        """qnb_pot_energy_step (single-window context): the nonbonded side of
        one pot_energy call through host buffers.  Returns (d, E, EQ, Erst)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        if d is None:
            d = np.zeros_like(x)
        E = np.zeros(7)
        EQ = np.zeros((max(self.S, 1), 6))
        R = np.zeros(2)
        self._check(self.lib.qnb_pot_energy_step(self.h, _p(x), _p(d), Tfree, int(istep), _p(E), _p(EQ), _p(R)))
        return d, dict(zip(E_FIELDS, E)), EQ[: self.S], R

    def compute_dev(self, Tfree=300.0, istep=0, sync=True):
        """All windows; returns per-window energies (lists) when sync, else
        None at once (the evaluation is only enqueued)."""
        if not sync:
            self._check(self.lib.qnb_compute_dev(self.h, Tfree, int(istep), 0, None, None, None))
            return None
        W = self.nwin
        E = np.zeros((W, 7))
        EQ = np.zeros((W, max(self.S, 1), 6))
        R = np.zeros((W, 2))
        self._check(self.lib.qnb_compute_dev(self.h, Tfree, int(istep), 1, _p(E), _p(EQ), _p(R)))
        return [dict(zip(E_FIELDS, e)) for e in E], EQ[:, : self.S], R

    def step_host(self, x_all, out=None, Tfree=300.0, istep=0, rebuild_lists=False):
        """One step of every window through host buffers with one host
        synchronisation (qnb_step_host): coordinates of all windows in (nwin x
        natom x 3; pinned memory for an asynchronous copy), lists rebuilt with
        the last cut-offs when rebuild_lists, the evaluation of compute_dev,
        the gradient of all windows written into `out` (a C-contiguous
        float64 array, e.g. a view of pinned memory; allocated if None).
        Returns (gradient, E [nwin][7] with columns E_FIELDS, EQ
        [nwin][nstates][6], restraints [nwin][2]) as arrays: per-window dicts
        cost more host time than the call itself at 51 windows."""
        W = self.nwin
        xa = np.ascontiguousarray(x_all, dtype=np.float64)
        assert xa.size == W * self.s.natom * 3
        if out is None:
            out = np.zeros((W, self.s.natom, 3))
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == xa.size
        E = np.zeros((W, 7))
        EQ = np.zeros((W, max(self.S, 1), 6))
        R = np.zeros((W, 2))
        self._check(self.lib.qnb_step_host(self.h, _p(xa), _p(out), Tfree, int(istep), int(bool(rebuild_lists)),
                                           _p(E), _p(EQ), _p(R)))
        return out, E, EQ[:, : self.S], R

    def energies_dev(self):
        """Energies of the last evaluation of every window (waits for it):
        per-window dicts, EQ [nwin][nstates][6], restraints [nwin][2]."""
        W = self.nwin
        E = np.zeros((W, 7))
        EQ = np.zeros((W, max(self.S, 1), 6))
        R = np.zeros((W, 2))
        self._check(self.lib.qnb_get_energies_dev(self.h, _p(E), _p(EQ), _p(R)))
        return [dict(zip(E_FIELDS, e)) for e in E], EQ[:, : self.S], R

    def set_solvent_internal(self, pairs, A, B, el):
        """nonbnd_solv_int: (i, j) offsets inside a solvent molecule with their
        vdWA, vdWB, elec; evaluated for every molecule in pot_energy_nonbonds."""
        ij = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        a, b, e = (np.ascontiguousarray(np.asarray(v, dtype=np.float64)) for v in (A, B, el))
        self._check(self.lib.qnb_set_solvent_internal(self.h, len(a), _p(ij), _p(a), _p(b), _p(e)))

    def autotune(self, reps=3):
        """Times the launch-geometry candidates on the current lists; returns
        the chosen values by name (qnb_autotune)."""
        v = np.zeros(len(TUNE_NAMES), dtype=np.int32)
        self._check(self.lib.qnb_autotune(self.h, int(reps), _p(v)))
        return dict(zip(TUNE_NAMES, v.tolist()))

    def tuning(self):
        v = np.zeros(len(TUNE_NAMES), dtype=np.int32)
        self._check(self.lib.qnb_get_tuning(self.h, _p(v)))
        return dict(zip(TUNE_NAMES, v.tolist()))

    def set_tuning(self, values):
        v = np.array([values[n] for n in TUNE_NAMES], dtype=np.int32)
        self._check(self.lib.qnb_set_tuning(self.h, _p(v)))

    # ---- device-resident MD step (qnb_md_*) -----------------------------
    def md_init(self, setup=None, bonded=None):
        """qnb_md_init from an MdSetup (q6_gb300.md): constraints, degrees of
        freedom and temperature groups as qdyn derives them for this system;
        with ``bonded`` (the topology's BondedTerms before the shaken bonds
        are removed) the constraint lengths are its bond library's."""
        from .md import MdSetup, build_constraints, md_params
        setup = setup or MdSetup()
        cons = build_constraints(self.s, setup, bonded)
        self.md_setup, self.md_constraints = setup, cons
        self.md_p = md_params(self.s, setup, cons)
        mass = np.ascontiguousarray(self.s.mass[self.s.iac], dtype=np.float64)
        ij = np.ascontiguousarray(cons.ij, dtype=np.int32)
        dist = np.ascontiguousarray(cons.dist)
        self._check(self.lib.qnb_md_init(self.h, ctypes.byref(self.md_p), _p(mass), len(cons.mol_first) - 1,
                                         _p(cons.mol_first), _p(ij), _p(dist)))

    def md_set_thermostat(self, thermostat="berendsen", integrator="leap-frog", nhchains=10, nhq=0.0):
        """qdyn's thermostat ('berendsen', 'nose-hoover') and integrator
        ('leap-frog', 'velocity-verlet'); nhq <= 0 takes kbT/tau_T^2."""
        t = {"berendsen": 0, "nose-hoover": 1}[thermostat]
        g = {"leap-frog": 0, "velocity-verlet": 1}[integrator]
        self._check(self.lib.qnb_md_set_thermostat(self.h, t, g, int(nhchains), float(nhq)))

    def md_set_langevin(self, integrator="leap-frog", friction=0.0, seed=1):
        """Langevin thermostat (uniform random forces); friction <= 0 takes 1/tau_T."""
        g = {"leap-frog": 0, "velocity-verlet": 1}[integrator]
        self._check(self.lib.qnb_md_set_langevin(self.h, g, float(friction), int(seed)))

    def md_set_velocities(self, v, window=None):
        """v: [natom, 3] for one window (or every window if window is None),
        or [nwin, natom, 3]."""
        v = np.asarray(v, dtype=np.float64)
        wins = range(self.nwin) if window is None else [window]
        for k, w in enumerate(wins):
            vw = np.ascontiguousarray(v[k] if v.ndim == 3 else v)
            self._check(self.lib.qnb_md_set_velocities(self.h, int(w), _p(vw)))

    def md_state(self, window=0):
        x = np.zeros((self.s.natom, 3))
        v = np.zeros((self.s.natom, 3))
        self._check(self.lib.qnb_md_get_state(self.h, int(window), _p(x), _p(v)))
        return x, v

    def md_minimize(self, nsteps, initial_step=1e-4, force_cutoff=1.0, max_move=0.0):
        """Qmin-style steepest descent of every window (max_move > 0 caps
        each step's largest atomic move); returns the largest atomic force
        per window at the last step."""
        maxf = np.zeros(self.nwin)
        self._check(self.lib.qnb_md_minimize(self.h, int(nsteps), float(initial_step), float(force_cutoff),
                                             float(max_move), _p(maxf)))
        return maxf

    def md_prepare(self, stop_cm=True):
        self._check(self.lib.qnb_md_prepare(self.h, int(bool(stop_cm))))

    def md_run(self, nsteps, istep0=0, records=True):
        """nsteps MD steps of every window.  Returns (rec [nsteps][nwin]
        structured as q6_gb300.md.MD_RECORD, EQ [nsteps][nwin][nstates][6],
        Eb [nsteps][nwin][8 + 4*nstates]) or (None, None, None) without
        records."""
        from .md import MD_RECORD
        if not records:
            self._check(self.lib.qnb_md_run(self.h, int(nsteps), int(istep0), None, None, None))
            return None, None, None
        rec = np.zeros((nsteps, self.nwin), MD_RECORD)
        EQ = np.zeros((nsteps, self.nwin, max(self.S, 1), 6))
        Eb = np.zeros((nsteps, self.nwin, 8 + 4 * self.S))
        self._check(self.lib.qnb_md_run(self.h, int(nsteps), int(istep0), _p(rec), _p(EQ), _p(Eb)))
        return rec, EQ[:, :, : self.S], Eb

    # ---- offdiag ------------------------------------------------------------
    def set_offdiag(self, rows):
        """rows: (state_i, state_j, qatom_k, qatom_l, A, mu), 0-based."""
        rows = list(rows)
        st = np.ascontiguousarray([[r[0], r[1]] for r in rows], dtype=np.int32).reshape(-1, 2)
        qa = np.ascontiguousarray([[r[2], r[3]] for r in rows], dtype=np.int32).reshape(-1, 2)
        A = np.ascontiguousarray([r[4] for r in rows], dtype=np.float64)
        mu = np.ascontiguousarray([r[5] for r in rows], dtype=np.float64)
        self.offd_states = st
        self._check(self.lib.qnb_set_offdiag(self.h, len(rows), _p(st), _p(qa), _p(A), _p(mu)))

    def offdiag(self):
        """(Hij, rkl), [nwin][n] each, of the last evaluation."""
        n = len(getattr(self, "offd_states", []))
        Hij = np.zeros((self.nwin, n))
        rkl = np.zeros((self.nwin, n))
        if n:
            self._check(self.lib.qnb_get_offdiag(self.h, _p(Hij), _p(rkl)))
        return Hij, rkl

    def offd_records(self, window=0):
        """put_ene's OFFD records of a window (1-based states), for
        q6_gb300.enefile.EnergyFileWriter.write_step(offd=...)."""
        Hij, rkl = self.offdiag()
        return [(int(i) + 1, int(j) + 1, float(h), float(r))
                for (i, j), h, r in zip(self.offd_states, Hij[window], rkl[window])]

    # ---- periodic box --------------------------------------------------------
    def set_box(self, boxlength, qswitch=None):
        """Periodic boundary conditions (qnb_set_box): boxlength (3 edges, A)
        or None for the sphere; qswitch: 0-based Q switching atom (default
        the first Q atom)."""
        if boxlength is None:
            self._check(self.lib.qnb_set_box(self.h, None, 0))
            self.boxlength = None
            return
        L = np.ascontiguousarray(np.broadcast_to(np.asarray(boxlength, np.float64), (3,)))
        qs = int(self.s.iqseq[0]) if qswitch is None and self.s.nqat else int(qswitch or 0)
        self._check(self.lib.qnb_set_box(self.h, _p(L), qs))
        self.boxlength, self.qswitch = L.copy(), qs

    def set_put_back_in_box(self, molecules=None, put_solute=True, put_solvent=True, boxcentre=None):
        """put_back_in_box for the MD runs of a periodic box (after md_init):
        molecules = lists of atoms, solute molecules first (default: the
        solute's bonded molecules, then each solvent molecule); boxcentre None
        for a floating centre (the mean of the solute atoms)."""
        from .md import solute_molecules
        s = self.s
        if molecules is None:
            molecules = solute_molecules(s) + [list(range(s.nat_solute + s.solv_atom * w,
                                                          s.nat_solute + s.solv_atom * (w + 1)))
                                               for w in range(s.nwat)]
            nslu = len(molecules) - s.nwat
        else:
            nslu = sum(1 for m in molecules if min(m) < s.nat_solute)
        first = np.zeros(len(molecules) + 1, np.int32)
        for q, mol in enumerate(molecules):
            first[q + 1] = first[q] + len(mol)
        atoms = np.ascontiguousarray(np.concatenate([np.asarray(m, np.int32) for m in molecules]), dtype=np.int32)
        bc = None if boxcentre is None else np.ascontiguousarray(boxcentre, dtype=np.float64)
        self.pb_boxcentre = None if bc is None else bc.copy()
        self._check(self.lib.qnb_set_put_back_in_box(self.h, len(molecules), _p(first), _p(atoms), nslu,
                                                     int(put_solute), int(put_solvent),
                                                     None if bc is None else _p(bc)))

    def put_back_in_box(self):
        """Wraps the molecules now; returns the box centres [nwin][3]."""
        c = np.zeros((self.nwin, 3))
        self._check(self.lib.qnb_put_back_in_box(self.h, _p(c)))
        return c

    # ---- monitor groups and group contributions ----------------------------
    def set_monitor_groups(self, groups, pairs):
        """[nonbonded_monitor]: groups = lists of 0-based solute atoms, pairs =
        (group i, group j) to monitor; an empty pairs list removes them."""
        first = np.zeros(len(groups) + 1, np.int32)
        for g, a in enumerate(groups):
            first[g + 1] = first[g] + len(a)
        atoms = np.ascontiguousarray(np.concatenate([np.asarray(a, np.int32) for a in groups])
                                     if groups else np.zeros(0, np.int32), dtype=np.int32)
        pr = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        self.mon_npairs = len(pr)
        self._check(self.lib.qnb_set_monitor_groups(self.h, len(groups), _p(first), _p(atoms), len(pr), _p(pr)))

    def monitor_energies(self, lambdas=None):
        """nonbond_monitor's output of the last evaluation: Vel and Vlj
        [nwin][npairs][nstates]; with lambdas ([nwin][nstates] or [nstates])
        also the lambda-weighted Vwel, Vwlj and Vwsum [nwin][npairs]."""
        n = getattr(self, "mon_npairs", 0)
        out = np.zeros((self.nwin, n, self.S, 2))
        if n:
            self._check(self.lib.qnb_get_monitor_energies(self.h, _p(out)))
        r = {"Vel": out[..., 0], "Vlj": out[..., 1]}
        if lambdas is not None:
            lam = np.broadcast_to(np.asarray(lambdas, np.float64).reshape(-1, self.S), (self.nwin, self.S))
            r["Vwel"] = np.einsum("wps,ws->wp", r["Vel"], lam)
            r["Vwlj"] = np.einsum("wps,ws->wp", r["Vlj"], lam)
            r["Vwsum"] = r["Vwel"] + r["Vwlj"]
        return r

    def set_group_contributions(self, groups):
        """[group_contribution]: groups = (atoms, caltype) with 0-based solute
        atoms and caltype 'full', 'electro', 'vdw' or 'all'; [] removes them.
        The energy-file header for them is group_contribution_header(...)."""
        mask = np.zeros((len(groups), self.s.nat_solute), np.uint8)
        for g, (atoms, caltype) in enumerate(groups):
            if caltype not in ("full", "electro", "vdw", "all"):
                raise ValueError(f"group contribution {g}: unknown calculation type {caltype!r}")
            mask[g, np.asarray(atoms, np.int64)] = 1
        self.gc_groups = [(np.asarray(a), c) for a, c in groups]
        self._check(self.lib.qnb_set_group_exclusions(self.h, len(groups), _p(np.ascontiguousarray(mask))))

    def group_exclusions(self):
        """The excluded interactions of every group, [nwin][ngroups][nstates][4]
        = qq el, qq vdw, qp el, qp vdw, of the last evaluation."""
        n = len(getattr(self, "gc_groups", []))
        out = np.zeros((self.nwin, n, self.S, 4))
        if n:
            self._check(self.lib.qnb_get_group_exclusions(self.h, _p(out)))
        return out

    def group_contribution_EQ(self, EQ, window=0):
        """calculate_exc (src/nonbondene.f90:6825-6920): the per-state Q
        energies of every energy-file array, EQ [nstates][6] of the window
        (array 1) followed by one array per group and calculation type with
        the excluded interactions subtracted; [nstates][arrays*6] for
        q6_gb300.enefile.EnergyFileWriter.write_step."""
        from q6_gb300.enefile import ELECTRO, FULL, VDW, group_contribution_header
        hdr = group_contribution_header([(len(a), c) for a, c in self.gc_groups])
        exc = self.group_exclusions()[window]
        EQ = np.asarray(EQ, np.float64).reshape(self.S, 6)
        arrays = [EQ]
        for a in range(1, hdr.arrays):
            g, t = hdr.gcnum[a] - 1, hdr.types[a]
            e = EQ.copy()
            if t in (FULL, ELECTRO):
                e[:, 0] -= exc[g, :, 0]
                e[:, 2] -= exc[g, :, 2]
            if t in (FULL, VDW):
                e[:, 1] -= exc[g, :, 1]
                e[:, 3] -= exc[g, :, 3]
            arrays.append(e)
        return np.concatenate(arrays, axis=1), hdr

    # ---- fix_shell ---------------------------------------------------------
    def set_freeze(self, freeze=True):
        """excluded_freeze: excluded atoms held at xtop (qnb_set_freeze)."""
        self._check(self.lib.qnb_set_freeze(self.h, int(bool(freeze))))

    def set_shell_restraint(self, xtop, shell, fk_fix=200.0, fk_pshell=10.0):
        """fix_shell restraint to xtop (None removes it); shell: per-atom flags
        (q6_gb300.md.make_shell).  Defaults: qdyn's fk_fix and fk_pshell."""
        if xtop is None:
            self._check(self.lib.qnb_set_shell_restraint(self.h, None, None, 0.0, 0.0))
            return
        xt = np.ascontiguousarray(xtop, dtype=np.float64)
        sh = np.ascontiguousarray(shell, dtype=np.uint8)
        self._check(self.lib.qnb_set_shell_restraint(self.h, _p(xt), _p(sh), float(fk_fix), float(fk_pshell)))

    def restraint_energies(self):
        """[nwin][5 + nstates]: fix, shell, solvent_radial, water_pol, protein,
        then EQ(s)%restraint, of the last evaluation."""
        Er = np.zeros((self.nwin, 5 + self.S))
        self._check(self.lib.qnb_get_restraint_energies(self.h, _p(Er)))
        return Er

    def set_restraints(self, r, xtop=None):
        """qnb_set_restraints from a q6_gb300.restraints.Restraints (None
        removes them); xtop defaults to the topology coordinates."""
        if r is None:
            self._check(self.lib.qnb_set_restraints(self.h, None, None))
            return
        st, keep = r.to_struct()
        xt = np.ascontiguousarray(self.s.x if xtop is None else xtop, dtype=np.float64)
        self._check(self.lib.qnb_set_restraints(self.h, ctypes.byref(st), _p(xt)))

    # ---- bonded terms ------------------------------------------------------
    def set_bonded(self, bt):
        """qnb_set_bonded from a q6_gb300.bonded.BondedTerms."""
        st, keep = bt.to_struct(self.S)
        self._check(self.lib.qnb_set_bonded(self.h, ctypes.byref(st)))
        self.bonded_terms = bt

    def bonded_energies(self):
        """(Eb [nwin][8], EQb [nwin][nstates][4]) of the last evaluation."""
        Eb = np.zeros((self.nwin, 8))
        EQb = np.zeros((self.nwin, max(self.S, 1), 4))
        self._check(self.lib.qnb_get_bonded_energies(self.h, _p(Eb), _p(EQb)))
        return Eb, EQb[:, : self.S]

    def profile_classes(self, names):
        """Profile only the named kernel classes (KERNEL_CLASSES); [] stops."""
        mask = 0
        for n in names:
            mask |= 1 << KERNEL_CLASSES.index(n)
        self._check(self.lib.qnb_profile_classes(self.h, mask))

    def profile_collect(self):
        """Reads the per-class timing events of finished evaluations."""
        self._check(self.lib.qnb_profile_collect(self.h))

    def set_graphs(self, enable: bool):
        """CUDA-graph replay of compute_dev (on by default)."""
        self._check(self.lib.qnb_set_graphs(self.h, int(bool(enable))))

    def set_concurrency(self, enable: bool):
        """The mixed form's parallel evaluation branches (on by default)."""
        self._check(self.lib.qnb_set_concurrency(self.h, int(bool(enable))))

    def q_adjoint_dev(self):
        """dE_s/dqcrg, dE_s/dqA, dE_s/dqB per window: arrays [nwin][nqat][nstates]."""
        n = self.nwin * self.s.nqat * self.S
        dq, dA, dB = np.zeros(n), np.zeros(n), np.zeros(n)
        self._check(self.lib.qnb_q_adjoint_dev(self.h, _p(dq), _p(dA), _p(dB)))
        shp = (self.nwin, self.S, self.s.nqat)
        return tuple(a.reshape(shp).transpose(0, 2, 1).copy() for a in (dq, dA, dB))

    def set_coordinates_dev(self, x_all):
        """Copies coordinates of all windows (nwin x natom x 3) into HBM."""
        xa = np.ascontiguousarray(x_all, dtype=np.float64)
        assert xa.size == self.nwin * self.s.natom * 3
        self._check(self.lib.qnb_upload_coordinates(self.h, _p(xa)))

    def gradient_dev(self, clear=True, out=None):
        """Gradient accumulators of all windows (nwin x natom x 3), into `out`
        (a C-contiguous float64 array, e.g. a view of pinned memory) if given."""
        if out is None:
            out = np.zeros((self.nwin, self.s.natom, 3))
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == self.nwin * self.s.natom * 3
        self._check(self.lib.qnb_download_gradient(self.h, _p(out), int(clear)))
        return out

    def evaluate(self, x, lam, cut=None, solvent=None, Tfree=300.0, istep=0, lists=True):
        """One full nonbonded evaluation in the reference's call order."""
        cut = cut or {}
        self.set_lambda(lam)
        if lists:
            self.make_pair_lists(x, **cut)
        d, E, EQ = self.pot_energy_nonbonds(x)
        d, EQ = self.nonbond_qq(x, d, EQ)
        erst = [0.0, 0.0]
        if solvent is not None:
            erst[0] = self.restrain_solvent(x, d, Tfree)
            if solvent.wpol_restr:
                erst[1] = self.watpol(x, d, istep, True)
        return d, E, EQ, erst


class Group:
    """Several engines (systems of different sizes on one GPU) evaluated as one
    CUDA graph launch per step (qnb_group_*)."""

    def __init__(self, engines):
        self.lib = load_library()
        self.engines = list(engines)
        arr = (ctypes.c_void_p * len(self.engines))(*[e.h.value for e in self.engines])
        h = ctypes.c_void_p()
        rc = self.lib.qnb_group_create(arr, len(self.engines), ctypes.byref(h))
        if rc != 0:
            raise QnbError(f"qnb error {rc}: {self.lib.qnb_last_error().decode()}")
        self.h = h

    def compute(self, Tfree=300.0, istep=0):
        rc = self.lib.qnb_group_compute(self.h, Tfree, int(istep))
        if rc != 0:
            raise QnbError(f"qnb error {rc}: {self.lib.qnb_last_error().decode()}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.qnb_group_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
