"""The C-ABI library loads without a GPU and exports every entry point that
include/fame.h declares (no compute calls here)."""
import os
import re
import subprocess

import fame

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "fame.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fame_[A-Za-z_0-9]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("fame_plan_create", "fame_apply_A", "fame_apply_B", "fame_apply_Binv", "fame_curl_transform",
              "fame_lanczos", "fame_band_solve"):
        assert s in syms


def test_library_exports_every_declared_symbol(fame_lib):
    nm = subprocess.run(["nm", "-D", "--defined-only", fame.lib_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (fame_[A-Za-z_0-9]+)", nm))
    for s in declared_symbols():
        assert s in exported, s
        assert hasattr(fame_lib, s)
    assert fame_lib.fame_version().decode().startswith("fame-gb300")


def test_python_signatures_cover_header():
    from fame._lib import SIGNATURES

    assert set(declared_symbols()) == set(SIGNATURES)
