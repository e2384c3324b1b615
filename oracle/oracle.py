"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the CPU FP64 oracle.

The oracle (``oracle/qnb_oracle.c``) restates Q6 qdyn's nonbonded path on the
CPU in strict FP64.  It is the checker for the CUDA engine and the CPU
baseline of the benchmark; the product package never imports this module.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
LIB_TIMING = os.path.join(BUILD, "liboracle_timing.so")
SRC = os.path.join(HERE, "qnb_oracle.c")

# the checker: strict IEEE double, no FMA contraction, no fast-math
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
          "-fno-associative-math", "-Wall", "-Wno-unused-function"]
# the timed CPU baseline: the optimisation flags of the reference's own gcc
# build (Q6 src/makefile, COMP=gcc: -Ofast -unroll -finline-limit=10000000);
# no -march=native, so the same flags build on x86 and Arm hosts
CFLAGS_TIMING = ["-Ofast", "-funroll-loops", "-finline-limit=10000000", "-std=c11", "-fPIC", "-shared",
                 "-Wall", "-Wno-unused-function"]


def _build_one(path, flags, force):
    if force or not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(SRC):
        subprocess.check_call(["gcc", *flags, "-o", path, SRC, "-lm"])
    return path


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    _build_one(LIB_TIMING, CFLAGS_TIMING, force)
    return _build_one(LIB, CFLAGS, force)


_libs = {}


def lib(timing: bool = False):
    """The checker library, or with timing=True the -Ofast build that the
    CPU baseline times (never used as a checker)."""
    if timing not in _libs:
        build()
        L = ctypes.CDLL(LIB_TIMING if timing else LIB)
        P = ctypes.c_void_p
        D = ctypes.c_double
        I = ctypes.c_int
        L.orc_create.restype = P
        L.orc_create.argtypes = [P, I]
        L.orc_destroy.argtypes = [P]
        L.orc_set_lambda.argtypes = [P, P]
        L.orc_make_pair_lists.argtypes = [P, P, D, D, D, D, D, D]
        L.orc_pot_energy_nonbonds.argtypes = [P, P, P, P, P, I]
        L.orc_nonbond_qq.argtypes = [P, P, P, P]
        L.orc_set_solvent_params.argtypes = [P, P]
        L.orc_set_solvent_internal.argtypes = [P, ctypes.c_int, P, P, P, P]
        L.orc_restrain_solvent.argtypes = [P, P, P, D, P]
        L.orc_watpol.argtypes = [P, P, P, I, I, P]
        L.orc_get_watpol_state.argtypes = [P, P, P, P]
        L.orc_list_size.restype = ctypes.c_long
        L.orc_list_size.argtypes = [P, I]
        L.orc_export_pairs.restype = ctypes.c_long
        L.orc_export_pairs.argtypes = [P, I, P, P]
        L.orc_get_lrf.argtypes = [P, P]
        L.orc_shake.restype = ctypes.c_long
        L.orc_shake.argtypes = [P, P, I, P, P, P, P, P]
        L.orc_md_newvel.argtypes = [I, P, P, P, P, P, D, I, P, P, P]
        L.orc_md_newvel2.argtypes = [I, P, P, P, P, P, D, D, I, I, P, P, P]
        L.orc_md_newvel_lan.argtypes = [I, P, P, P, P, P, D, D, I, D, D, ctypes.c_uint64, I, I]
        L.orc_md_velocity.argtypes = [I, P, P, P, D]
        L.orc_md_stop_cm.argtypes = [I, P, P]
        L.orc_md_temperature.argtypes = [I, P, P, P, I, P, P, P, P, D, D, D, D, D, D, P, P]
        L.orc_bonded.argtypes = [P, P, P, I, P, P, P]
        L.orc_fix_shell.argtypes = [I, P, P, P, P, P, D, D, P]
        L.orc_p_restrain.argtypes = [P, P, P, P, P, P, P, I, P, P, P]
        L.orc_static_qq_size.restype = ctypes.c_long
        L.orc_static_qq_size.argtypes = [P, I, I]
        _libs[timing] = L
    return _libs[timing]


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """Mirror of the reference call sequence on one system."""

    E_FIELDS = ("pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw", "lrf")
    Q_FIELDS = ("qq_el", "qq_vdw", "qp_el", "qp_vdw", "qw_el", "qw_vdw")

    def __init__(self, system, use_lrf: bool = True, timing_build: bool = False):
        from q6_gb300.system import TopologyHandle
        self.s = system
        self.topo = TopologyHandle(system)
        self.L = lib(timing_build)
        self.h = self.L.orc_create(self.topo.ptr(), int(use_lrf))
        self.S = system.nstates

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_lambda(self, lam):
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        self.L.orc_set_lambda(self.h, _p(lam))

    def make_pair_lists(self, x, Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0):
        x = np.ascontiguousarray(x, dtype=np.float64)
        self.L.orc_make_pair_lists(self.h, _p(x), Rcq, Rcq ** 2, RcLRF ** 2, Rcpp ** 2,
                                  Rcpw ** 2, Rcww ** 2)

    def pot_energy_nonbonds(self, x, d=None, md=True):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if d is None:
            d = np.zeros_like(x)
        E = np.zeros(7)
        EQ = np.zeros((self.S, 6))
        self.L.orc_pot_energy_nonbonds(self.h, _p(x), _p(d), _p(E), _p(EQ), int(md))
        return d, dict(zip(self.E_FIELDS, E)), EQ

    def nonbond_qq(self, x, d=None, EQ=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if d is None:
            d = np.zeros_like(x)
        if EQ is None:
            EQ = np.zeros((self.S, 6))
        self.L.orc_nonbond_qq(self.h, _p(x), _p(d), _p(EQ))
        return d, EQ

    def set_solvent_params(self, p):
        self.L.orc_set_solvent_params(self.h, ctypes.byref(p))

    def set_solvent_internal(self, pairs, A, B, el):
        """nonbnd_solv_int: (i, j) offsets inside a solvent molecule with their
        A, B, elec (applied to every molecule when md)."""
        ij = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        a, b, e = (np.ascontiguousarray(np.asarray(v, dtype=np.float64)) for v in (A, B, el))
        self.L.orc_set_solvent_internal(self.h, len(a), _p(ij), _p(a), _p(b), _p(e))

    def restrain_solvent(self, x, d, Tfree):
        e = np.zeros(1)
        self.L.orc_restrain_solvent(self.h, _p(np.ascontiguousarray(x)), _p(d), Tfree, _p(e))
        return float(e[0])

    def watpol(self, x, d, istep, md=True):
        e = np.zeros(1)
        self.L.orc_watpol(self.h, _p(np.ascontiguousarray(x)), _p(d), int(istep), int(md), _p(e))
        return float(e[0])

    def watpol_state(self):
        a, b, c = np.zeros(16), np.zeros(16), np.zeros(16)
        self.L.orc_get_watpol_state(self.h, _p(a), _p(b), _p(c))
        return a, b, c

    def list_size(self, kind):
        return int(self.L.orc_list_size(self.h, kind))

    def export_pairs(self, kind):
        n = self.list_size(kind)
        i = np.zeros(max(n, 1), np.int32)
        j = np.zeros(max(n, 1), np.int32)
        m = self.L.orc_export_pairs(self.h, kind, _p(i), _p(j))
        return i[:m], j[:m]

    def lrf(self):
        out = np.zeros((self.s.ncgp, 43))
        self.L.orc_get_lrf(self.h, _p(out))
        return out

    def bonded(self, x, bt, lam, d=None):
        """pot_energy_bonds + the Q-atom bonded terms for BondedTerms bt:
        returns (d, Eb[8], EQb[nstates][4])."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        if d is None:
            d = np.zeros_like(x)
        st, keep = bt.to_struct(self.S)
        Eb = np.zeros(8)
        EQb = np.zeros((max(self.S, 1), 4))
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        self.L.orc_bonded(_p(x), _p(d), ctypes.byref(st), self.S, _p(lam), _p(Eb), _p(EQb))
        return d, Eb, EQb[: self.S]

    def fix_shell(self, x, xtop, shell, fk_fix, fk_pshell, d=None):
        """fix_shell: returns (d, [E_fix, E_shell])."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        if d is None:
            d = np.zeros_like(x)
        E = np.zeros(2)
        excl = np.ascontiguousarray(self.s.excl, dtype=np.uint8)
        sh = np.ascontiguousarray(shell, dtype=np.uint8)
        xt = np.ascontiguousarray(xtop, dtype=np.float64)
        self.L.orc_fix_shell(self.s.natom, _p(x), _p(d), _p(xt), _p(excl), _p(sh), float(fk_fix), float(fk_pshell),
                            _p(E))
        return d, E

    def p_restrain(self, x, r, lam, xtop=None, d=None):
        """p_restrain for a q6_gb300.restraints.Restraints: (d, E_protein,
        EQ_restraint[nstates])."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        if d is None:
            d = np.zeros_like(x)
        st, keep = r.to_struct()
        xt = np.ascontiguousarray(self.s.x if xtop is None else xtop, dtype=np.float64)
        heavy = np.ascontiguousarray(self.s.heavy, dtype=np.uint8)
        mass = np.ascontiguousarray(self.s.mass[self.s.iac], dtype=np.float64)
        xw = np.ascontiguousarray(self.s.xwcent, dtype=np.float64)
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        Ep = np.zeros(1)
        EQr = np.zeros(max(self.S, 1))
        self.L.orc_p_restrain(_p(x), _p(d), ctypes.byref(st), _p(xt), _p(heavy), _p(mass), _p(xw), self.S, _p(lam),
                             _p(Ep), _p(EQr))
        return d, float(Ep[0]), EQr[: self.S]

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


def shake(x, molecules, winv):
    """SHAKE of qdyn's initial_constraint (Q6 src/bondene.f90:1025-1048,
    1069-1150): ``molecules`` is a list of [(i, j, b0), ...] per molecule in
    topology bond order; returns the corrected copy of x."""
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    xx = x.copy()
    starts, ci, cj, d2 = [0], [], [], []
    for mol in molecules:
        for i, j, b0 in mol:
            ci.append(i)
            cj.append(j)
            d2.append(b0 * b0)
        starts.append(len(ci))
    starts = np.array(starts, np.int32)
    ci = np.array(ci, np.int32)
    cj = np.array(cj, np.int32)
    d2 = np.array(d2, np.float64)
    winv = np.ascontiguousarray(winv, dtype=np.float64)
    n = lib().orc_shake(_p(x), _p(xx), len(molecules), _p(starts), _p(ci), _p(cj), _p(d2), _p(winv))
    if n < 0:
        raise RuntimeError("shake failure")
    return x


class OracleMD:
    """qdyn's MD step on the CPU (test infrastructure): the oracle's
    nonbonded evaluation plus newvel_ber, SHAKE, v = (x - xx)/dt and
    temperature() with the Berendsen factors, in md_run's order
    (src/md.f90:1687-1812).  ``p`` is a q6_gb300.md.QnbMdParams, ``cons`` the
    matching Constraints, ``sp`` the solvent parameters (or None)."""

    BOLTZ = 0.001986
    MAGIC = 0.020462

    def __init__(self, oracle: Oracle, p, cons, sp=None, lam=None, bonded=None, shell=None,
                 thermostat="berendsen", integrator="leap-frog", nhchains=10, nhq=0.0, friction=0.0, seed=1):
        self.o, self.p, self.cons, self.sp = oracle, p, cons, sp
        self.nh = thermostat == "nose-hoover"
        self.lan = thermostat == "langevin"
        self.seed = int(seed)
        self.vv = integrator == "velocity-verlet"
        self.nhchains = int(nhchains)
        self.bt = bonded
        self.shell = shell   # (xtop, flags, fk_fix, fk_pshell) or None
        self.lam = None if lam is None else np.asarray(lam, dtype=np.float64)
        s = oracle.s
        self.n = s.natom
        self.mass = np.ascontiguousarray(s.mass[s.iac], dtype=np.float64)
        self.winv = 1.0 / self.mass
        self.excl = np.ascontiguousarray(s.excl, dtype=np.uint8)
        self.ntg = p.ntgroups
        self.first = np.array(p.tg_first[:self.ntg], np.int32)
        self.last = np.array(p.tg_last[:self.ntg], np.int32)
        self.tg_ndegf = np.array(p.tg_ndegf[:self.ntg], np.float64)
        self.tg_ndegfree = np.array(p.tg_ndegfree[:self.ntg], np.float64)
        self.dt = self.MAGIC * p.stepsize
        self.tau = self.MAGIC * p.tau_t
        self.sfact = np.zeros(self.ntg)
        self.ci = np.ascontiguousarray(cons.ij[:, 0], dtype=np.int32)
        self.cj = np.ascontiguousarray(cons.ij[:, 1], dtype=np.int32)
        self.d2 = np.ascontiguousarray(cons.dist * cons.dist)
        self.nmol = len(cons.mol_first) - 1
        if lam is not None:
            oracle.set_lambda(lam)
        self.tfree = 0.0
        self.temp = 0.0
        # Nose-Hoover chain, src/simprep.f90:2477-2485 (nhq default kbT/tau_T^2,
        # src/md.f90:282-285)
        self.nhq = nhq if nhq > 0.0 else self.BOLTZ * p.temp0 / (self.tau * self.tau)
        self.qnh = np.full(self.nhchains, self.nhq)
        self.qnh[0] = p.ndegf * self.nhq
        self.vnh = np.zeros(self.nhchains)
        self.xnh = np.zeros(self.nhchains)
        # Langevin, src/md.f90:250-253, 1632-1648 (uniform random forces)
        self.friction = friction if friction > 0.0 else 1.0 / self.tau
        step = 0.5 * self.dt if self.vv else self.dt
        self.gkT = 24.0 * self.friction * self.BOLTZ * p.temp0 / step

    def nh_prop(self):
        """nh_prop, src/simprep.f90:2509-2550: returns the velocity scale."""
        M, q, vn, xn = self.nhchains, self.qnh, self.vnh, self.xnh
        dt2 = 0.5 * self.dt
        dt4 = 0.5 * dt2
        dt8 = 0.5 * dt4
        kbT = self.BOLTZ * self.p.temp0
        G = np.zeros(M)
        G[0] = self.p.ndegf * self.BOLTZ * (self.temp - self.p.temp0) / q[0]
        for i in range(1, M):
            G[i] = (q[i - 1] * vn[i - 1] * vn[i - 1] - kbT) / q[i]
        vn[M - 1] = vn[M - 1] + G[M - 1] * dt4
        xn[M - 1] = xn[M - 1] + vn[M - 1] * dt2
        ex = 1.0
        for i in range(M - 2, -1, -1):
            ex = math.exp(-dt8 * vn[i + 1])
            vn[i] = (vn[i] * ex + G[i] * dt4) * ex
            xn[i] = xn[i] + vn[i] * dt2
        sc = math.exp(-vn[0] * dt2)
        G[0] = self.p.ndegf * self.BOLTZ * (sc * sc * self.temp - self.p.temp0) / q[0]
        vn[0] = (vn[0] * ex + G[0] * dt4) * ex
        for i in range(1, M - 1):
            ex = math.exp(-dt8 * vn[i + 1])
            G[i] = (q[i - 1] * vn[i - 1] * vn[i - 1] - kbT) / q[i]
            vn[i] = (vn[i] * ex + G[i] * dt4) * ex
        G[M - 1] = (q[M - 2] * vn[M - 2] * vn[M - 2] - kbT) / q[M - 1]
        vn[M - 1] = vn[M - 1] + G[M - 1] * dt4
        return sc

    def _shake(self, x, ref):
        n = lib().orc_shake(_p(x), _p(ref), self.nmol, _p(self.cons.mol_first), _p(self.ci), _p(self.cj),
                            _p(self.d2), _p(self.winv))
        if n < 0:
            raise RuntimeError("shake failure")
        return n

    def temperature(self, v):
        out = np.zeros(3 + 3 * self.ntg)
        lib().orc_md_temperature(self.n, _p(v), _p(self.mass), _p(self.excl), self.ntg, _p(self.first),
                                 _p(self.last), _p(self.tg_ndegf), _p(self.tg_ndegfree), self.p.ndegf,
                                 self.p.ndegfree, self.p.temp0, self.dt, self.tau, self.BOLTZ, _p(self.sfact),
                                 _p(out))
        self.tfree = out[2]
        self.temp = out[1]
        return out

    def prepare(self, x, v, stop_cm=True):
        """initial_constraint, stop_cm_translation, temperature()."""
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        v = np.ascontiguousarray(v, dtype=np.float64).copy()
        xx = x.copy()
        self._shake(x, xx)
        xx = x - v * self.dt
        self._shake(xx, x)
        lib().orc_md_velocity(self.n, _p(x), _p(xx), _p(v), self.dt)
        if stop_cm:
            lib().orc_md_stop_cm(self.n, _p(v), _p(self.mass))
        self.temperature(v)
        return x, v

    def minimize(self, x, nsteps, cut, step0=1e-4, fcut=1.0, max_move=0.0):
        """Qmin's steepest descent (src/minim.f90:891-935, 1056-1070) with
        SHAKE against the positions before each move; returns (x, largest
        force of the last step, potential energy per step)."""
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        o = self.o
        oldmax, scale = 0.0, step0
        epot, maxf = [], 0.0
        for k in range(nsteps):
            if k % self.p.nbcycle == 0:
                o.make_pair_lists(x, **cut)
            d = np.zeros_like(x)
            d, E, EQ = o.pot_energy_nonbonds(x, d)
            d, EQ = o.nonbond_qq(x, d, EQ)
            e = sum(E.values()) + float(np.dot(self.lam, EQ.sum(1))) if self.lam is not None else sum(E.values())
            if self.bt is not None:
                d, Eb, EQb = o.bonded(x, self.bt, self.lam, d)
                e += Eb.sum() + float(np.dot(self.lam, EQb.sum(1)))
            if self.sp is not None:
                e += o.restrain_solvent(x, d, 0.0)
                if self.sp.wpol_restr:
                    e += o.watpol(x, d, k, True)
            epot.append(e)
            maxf = float(np.sqrt((d * d).sum(1)).max())
            rv = 1 if maxf > oldmax else 0
            oldmax = maxf
            if maxf < fcut:
                rv = 2
            if rv == 1:
                scale = step0
            elif rv == 0:
                scale = scale * 1.20
            xx = x.copy()
            sc = 0.0 if rv == 2 else scale
            if max_move > 0.0 and sc * maxf > max_move:
                sc = max_move / maxf
            if sc != 0.0:
                x = x - d * sc
            if self.nmol > 0:
                self._shake(x, xx)
        return x, maxf, np.array(epot)

    def step(self, x, v, istep, cut):
        o = self.o
        if istep % self.p.nbcycle == 0:
            o.make_pair_lists(x, **cut)
        d = np.zeros_like(x)
        d, E, EQ = o.pot_energy_nonbonds(x, d)
        d, EQ = o.nonbond_qq(x, d, EQ)
        erst = [0.0, 0.0]
        Eb = EQb = None
        if self.bt is not None:
            d, Eb, EQb = o.bonded(x, self.bt, self.lam, d)
        efs = [0.0, 0.0]
        if self.shell is not None:
            d, efs = o.fix_shell(x, *self.shell, d=d)
        if self.sp is not None:
            erst[0] = o.restrain_solvent(x, d, self.tfree)
            if self.sp.wpol_restr:
                erst[1] = o.watpol(x, d, istep, True)
        xx = np.zeros_like(x)
        if self.nh:
            v *= self.nh_prop()
        sf = np.ones(self.ntg) if self.nh else self.sfact
        step = 0.5 * self.dt if self.vv else self.dt
        if self.lan:
            lib().orc_md_newvel_lan(self.n, _p(x), _p(xx), _p(v), _p(d), _p(self.winv), self.dt, step,
                                    int(self.vv), self.friction, self.gkT, self.seed, 0, int(istep))
        else:
            lib().orc_md_newvel2(self.n, _p(x), _p(xx), _p(v), _p(d), _p(self.winv), self.dt, step, int(self.vv),
                                 self.ntg, _p(self.first), _p(self.last), _p(np.ascontiguousarray(sf)))
        iters = 0
        if self.nmol > 0:
            iters = self._shake(x, xx)
            lib().orc_md_velocity(self.n, _p(x), _p(xx), _p(v), self.dt)
            if self.nh:
                v *= self.nh_prop()
        t = self.temperature(v)
        return dict(E=E, EQ=EQ, erst=erst, Eb=Eb, EQb=EQb, fix_shell=efs, ekin=t[0], temp=t[1], tfree=t[2],
                    shake_iterations=iters)
