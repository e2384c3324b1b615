"""The input file's restraint sections for qnb_set_restraints: p_restrain's
sequence, position, distance, angle and wall restraints (Q6
src/bondene.f90:764-1020; the input sections [sequence_restraints],
[atom_restraints], [distance_restraints], [angle_restraints],
[wall_restraints], read in src/md.f90:1237-1380).  Indices are 0-based;
a state of -1 is the reference's 0 (every state)."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

I32P = ctypes.POINTER(ctypes.c_int32)
F64P = ctypes.POINTER(ctypes.c_double)


class QnbRestraints(ctypes.Structure):
    _fields_ = [
        ("nseq", ctypes.c_int32), ("seq_ij", I32P), ("seq_fk", F64P), ("seq_ih", I32P), ("seq_mode", I32P),
        ("npos", ctypes.c_int32), ("pos_i", I32P), ("pos_state", I32P), ("pos_x", F64P), ("pos_fk", F64P),
        ("ndist", ctypes.c_int32), ("dist_ij", I32P), ("dist_state", I32P), ("dist_d", F64P), ("dist_fk", F64P),
        ("nang", ctypes.c_int32), ("ang_ijk", I32P), ("ang_state", I32P), ("ang_theta", F64P), ("ang_fk", F64P),
        ("nwall", ctypes.c_int32), ("wall_ij", I32P), ("wall_d", F64P), ("wall_fk", F64P),
        ("wall_aMorse", F64P), ("wall_dMorse", F64P), ("wall_ih", I32P),
    ]


@dataclass
class Restraints:
    seq: list = field(default_factory=list)    # (first, last, fk, include_h, mode 0/1/2)
    pos: list = field(default_factory=list)    # (atom, state, (x, y, z), (fkx, fky, fkz))
    dist: list = field(default_factory=list)   # (i, j, d1, d2, fk, state)
    ang: list = field(default_factory=list)    # (i, j, k, theta_deg, fk, state)
    wall: list = field(default_factory=list)   # (first, last, d, fk, aMorse, dMorse, include_h)

    def to_struct(self):
        keep = []

        def i32(v, w):
            a = np.ascontiguousarray(np.asarray(v, dtype=np.int32).reshape(-1, w) if len(v) else
                                     np.zeros((0, w), np.int32))
            keep.append(a)
            return a.ctypes.data_as(I32P)

        def f64(v, w):
            a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1, w) if len(v) else
                                     np.zeros((0, w)))
            keep.append(a)
            return a.ctypes.data_as(F64P)

        r = QnbRestraints()
        r.nseq = len(self.seq)
        r.seq_ij = i32([(a, b) for a, b, *_ in self.seq], 2)
        r.seq_fk = f64([q[2] for q in self.seq], 1)
        r.seq_ih = i32([q[3] for q in self.seq], 1)
        r.seq_mode = i32([q[4] for q in self.seq], 1)
        r.npos = len(self.pos)
        r.pos_i = i32([q[0] for q in self.pos], 1)
        r.pos_state = i32([q[1] for q in self.pos], 1)
        r.pos_x = f64([q[2] for q in self.pos], 3)
        r.pos_fk = f64([q[3] for q in self.pos], 3)
        r.ndist = len(self.dist)
        r.dist_ij = i32([(q[0], q[1]) for q in self.dist], 2)
        r.dist_d = f64([(q[2], q[3]) for q in self.dist], 2)
        r.dist_fk = f64([q[4] for q in self.dist], 1)
        r.dist_state = i32([q[5] for q in self.dist], 1)
        r.nang = len(self.ang)
        r.ang_ijk = i32([(q[0], q[1], q[2]) for q in self.ang], 3)
        r.ang_theta = f64([q[3] for q in self.ang], 1)
        r.ang_fk = f64([q[4] for q in self.ang], 1)
        r.ang_state = i32([q[5] for q in self.ang], 1)
        r.nwall = len(self.wall)
        r.wall_ij = i32([(q[0], q[1]) for q in self.wall], 2)
        r.wall_d = f64([q[2] for q in self.wall], 1)
        r.wall_fk = f64([q[3] for q in self.wall], 1)
        r.wall_aMorse = f64([q[4] for q in self.wall], 1)
        r.wall_dMorse = f64([q[5] for q in self.wall], 1)
        r.wall_ih = i32([q[6] for q in self.wall], 1)
        return r, keep
