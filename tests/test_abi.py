"""CPU checks of the C ABI library: it builds, loads and exports every
function include/qnb.h declares (no GPU calls)."""
import ctypes
import os
import re

from q6_gb300 import build as qbuild
from q6_gb300.qnb import EXPORTED, QnbOptions
from q6_gb300.system import QnbSolventParams, QnbTopology

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "qnb.h")).read()
    return sorted(set(re.findall(r"\b(qnb_[a-z_]+)\s*\(", src)))


def test_header_and_wrapper_agree():
    assert sorted(EXPORTED) == declared()


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(qbuild.build())
    for name in declared():
        assert hasattr(lib, name), name
    lib.qnb_version.restype = ctypes.c_int32
    assert lib.qnb_version() == 0x000300


def test_struct_layouts_match_header():
    # field counts of the ctypes mirrors against the header structs
    src = open(os.path.join(ROOT, "include", "qnb.h")).read()

    def nfields(struct):
        body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (struct, struct), src, re.S).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        n = 0
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            n += decl.count(",") + 1
        return n

    assert nfields("qnb_topology") == len(QnbTopology._fields_)
    assert nfields("qnb_solvent_params") == len(QnbSolventParams._fields_)
    assert nfields("qnb_options") == len(QnbOptions._fields_)


def test_create_fails_loudly_without_gpu_or_bad_args():
    import pytest
    from q6_gb300.qnb import NonbondedEngine, QnbError
    from q6_gb300.system import make_system
    s = make_system(R=8.0, n_solute=6, nq=2, seed=3)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(QnbError):
        NonbondedEngine(s)
