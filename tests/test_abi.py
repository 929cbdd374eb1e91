"""CPU tests of the C-ABI boundary: the library builds, loads and exports every
function include/elhl_prop.h declares (no compute calls without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    hdrs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]
    names = set()
    for h in hdrs:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_][a-z0-9_ ]*[\s*]+([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M):
            if m.group(1) not in ("if", "for", "while", "return", "sizeof"):
                names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib_path():
    from dynemol_gb300 import build
    return build.build()


def test_header_declares_reference_symbols():
    names = declared_functions()
    for s in ("propagationelhl_gpucaller_", "propagation_gpucaller_", "gpu_init_", "gpu_finalize_", "gpu_pin_",
              "gpu_unpin_"):
        assert s in names


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_library_loads_and_reports_status(lib_path):
    from dynemol_gb300 import api
    L = api.load(lib_path)
    for s in api.EXPORTED_SYMBOLS:
        assert hasattr(L, s)
    assert api.status_string(api.ERR_NO_CONVERGENCE).startswith("no convergence")
    assert L.elhl_last_status() == 0


def test_no_cpu_fallback_when_library_missing(tmp_path):
    from dynemol_gb300 import api
    with pytest.raises(ImportError):
        api._lib = None
        api.load(str(tmp_path / "missing.so"))
    api._lib = None


def test_oracle_not_linked(lib_path):
    """The product library never links or names the oracle."""
    out = subprocess.run(["ldd", lib_path], capture_output=True, text=True).stdout
    assert "orc" not in out
    strings = subprocess.run(["strings", lib_path], capture_output=True, text=True).stdout
    assert "liborc" not in strings and "orc_propagation" not in strings
