"""The C-ABI library loads and exports every function that include/tropidist_gb300.h declares."""
import os
import re

from helpers import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "tropidist_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"typedef[^;]*;", "", text)            # function-pointer types are not exports
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text)
    return sorted({n for n in names if n not in ("if", "sizeof")})


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_library_reports_version_and_errors(lib):
    assert lib.tg_version() >= 1
    assert lib.tg_dense_set_tuning(99, 99, 99, 99) == -1
    assert b"tuning" in lib.tg_last_error()
