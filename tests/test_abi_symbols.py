"""libflygpu loads and exports every function include/flygpu.h declares (CPU only, no compute)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared() -> list[str]:
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(flygpu_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_header(fly):
    lib = ctypes.CDLL(os.path.join(ROOT, "openfly_gb300", "_build", "libflygpu.so"))
    names = declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(fly):
    assert fly.status_string(fly.SPLINE_OOB) == "spline out of bounds"
    assert fly.status_string(fly.OK) == "ok"
