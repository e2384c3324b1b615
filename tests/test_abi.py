"""CPU checks of the C ABI library: it builds, loads and exports every
function include/qnb.h declares (no GPU calls)."""
import ctypes
import os
import re

from q6_gb300 import build as qbuild
from q6_gb300.md import MD_RECORD, QnbMdParams
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
    assert nfields("qnb_md_params") == len(QnbMdParams._fields_)


def test_md_struct_offsets_match_c_compiler(tmp_path):
    """sizeof / offsetof of the MD structs from gcc against the ctypes and
    numpy mirrors."""
    import shutil
    import subprocess
    import pytest
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    from q6_gb300.bonded import QnbBonded
    from q6_gb300.restraints import QnbRestraints
    bnames = [f[0] for f in QnbBonded._fields_]
    rnames = [f[0] for f in QnbRestraints._fields_]
    names = [f[0] for f in QnbMdParams._fields_]
    rec = list(MD_RECORD.names)
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "qnb.h"', "int main(void) {",
           'printf("%zu\\n", sizeof(qnb_md_params));']
    src += ['printf("%%zu\\n", offsetof(qnb_md_params, %s));' % n for n in names]
    src += ['printf("%zu\\n", sizeof(qnb_md_record));', 'printf("%zu\\n", offsetof(qnb_md_record, E));']
    src += ['printf("%%zu\\n", offsetof(qnb_md_record, %s));' % n for n in rec[1:]]
    src += ['printf("%zu\\n", sizeof(qnb_bonded));']
    src += ['printf("%%zu\\n", offsetof(qnb_bonded, %s));' % n for n in bnames]
    src += ['printf("%zu\\n", sizeof(qnb_restraints));']
    src += ['printf("%%zu\\n", offsetof(qnb_restraints, %s));' % n for n in rnames]
    src += ["return 0; }"]
    c = tmp_path / "lay.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "lay"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)])
    out = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    assert out[0] == ctypes.sizeof(QnbMdParams)
    assert out[1:1 + len(names)] == [getattr(QnbMdParams, n).offset for n in names]
    k = 1 + len(names)
    assert out[k] == MD_RECORD.itemsize
    assert out[k + 1:k + 1 + len(rec)] == [MD_RECORD.fields[n][1] for n in rec]
    k += 1 + len(rec)
    assert out[k] == ctypes.sizeof(QnbBonded)
    assert out[k + 1:k + 1 + len(bnames)] == [getattr(QnbBonded, n).offset for n in bnames]
    k += 1 + len(bnames)
    assert out[k] == ctypes.sizeof(QnbRestraints)
    assert out[k + 1:] == [getattr(QnbRestraints, n).offset for n in rnames]


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
