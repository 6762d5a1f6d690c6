"""The C ABI: the CUDA library loads and exports every entry point
include/ps3d.h declares (no device calls)."""
import os
import re
import subprocess

from puresoft3d_gb300 import build, pipeline

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in [f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]:
        txt = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(ps3d_\w+)\s*\(", txt, re.M))
    return names


def test_header_declares_entry_points():
    d = declared()
    assert "ps3d_draw" in d and "ps3d_pipeline_create" in d and len(d) >= 30


def test_library_exports_every_declared_symbol():
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (ps3d_\w+)", out))
    missing = declared() - exported
    assert not missing, missing


def test_python_binding_covers_header():
    assert declared() <= set(pipeline.exported_symbols()) | {"ps3d_last_error"}


def test_library_loads():
    lib = pipeline.library()
    assert lib.ps3d_last_error() is not None
