"""The Python binding (tbsla_gb300/capi.py) against the C ABI's header
(include/tbsla_gb300.h), on the CPU: every enum constant the binding names
has the header's value, and the ctypes structures have the header structs'
fields in order, with matching types and sizes."""
import ctypes as C
import os
import re

import pytest

from tbsla_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = open(os.path.join(ROOT, "include", "tbsla_gb300.h")).read()
# comments out, so that field lists and enums parse
CODE = re.sub(r"/\*.*?\*/", " ", HEADER, flags=re.S)


def header_enum(name: str) -> int:
    m = re.search(r"\b" + name + r"\s*=\s*(-?\d+)", CODE)
    assert m, name
    return int(m.group(1))


@pytest.mark.parametrize("py,c", [
    ("F64", "TBSLA_F64"), ("F32", "TBSLA_F32"), ("BF16", "TBSLA_BF16"),
    ("STORE_F64", "TBSLA_STORE_F64"), ("STORE_F32", "TBSLA_STORE_F32"), ("STORE_BF16", "TBSLA_STORE_BF16"),
    ("PR_REFERENCE", "TBSLA_PR_REFERENCE"), ("PR_DANGLING", "TBSLA_PR_DANGLING"), ("PR_TELEPORT", "TBSLA_PR_TELEPORT"),
    ("TUNE_X_L2_KEEP", "TBSLA_TUNE_X_L2_KEEP"), ("TUNE_PR_RELABEL", "TBSLA_TUNE_PR_RELABEL"),
    ("TUNE_X_L2_RANGE", "TBSLA_TUNE_X_L2_RANGE"), ("TUNE_SHORT_ROWS", "TBSLA_TUNE_SHORT_ROWS"),
    ("TUNE_TC_SPLIT", "TBSLA_TUNE_TC_SPLIT"), ("TUNE_SELL_ROWS", "TBSLA_TUNE_SELL_ROWS"),
    ("TUNE_DROP_SLICED_COPY", "TBSLA_TUNE_DROP_SLICED_COPY")])
def test_constants_match_the_header(py, c):
    assert getattr(capi, py) == header_enum(c)


def test_formats_match_the_header():
    for name, v in capi.FMT.items():
        assert v == header_enum("TBSLA_FMT_" + name)


_CTYPES = {"int": C.c_int, "int64_t": C.c_int64, "double": C.c_double, "float": C.c_float}


def header_struct(typedef: str) -> list[tuple[str, str]]:
    m = re.search(r"typedef struct\s*\{([^}]*)\}\s*" + typedef + r"\s*;", CODE, flags=re.S)
    assert m, typedef
    fields = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ty, names = decl.split(None, 1)
        for n in names.split(","):
            fields.append((n.strip(), ty))
    return fields


@pytest.mark.parametrize("py,c", [("MatrixInfo", "tbsla_matrix_info_t"), ("PageRankParams", "tbsla_pagerank_params_t"),
                                  ("PageRankResult", "tbsla_pagerank_result_t"),
                                  ("AutotuneResult", "tbsla_autotune_result_t")])
def test_structures_match_the_header(py, c):
    ours = getattr(capi, py)._fields_
    theirs = header_struct(c)
    assert [n for n, _ in ours] == [n for n, _ in theirs], (py, c)
    for (n, t), (_, ct) in zip(ours, theirs):
        assert t == _CTYPES[ct], (py, n, ct)
