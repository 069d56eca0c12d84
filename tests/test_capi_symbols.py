"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares (no compute calls are made)."""
import glob
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(sdpg_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_exports(sdpg):
    lib = sdpg.lib()
    declared = declared_functions()
    assert len(declared) >= 10
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", sdpg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (sdpg_[a-z0-9_]+)", out))
    assert declared <= exported, sorted(declared - exported)
    assert lib.sdpg_version() == 100


def test_command_line_driver_usage(sdpg):
    """The driver is built with the library and answers a call without data (no GPU use)."""
    exe = os.path.join(os.path.dirname(sdpg.LIB_PATH), "sdpa_gmp_gb300")
    assert os.path.exists(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "usage:" in r.stderr and "-ds" in r.stderr and "-is" in r.stderr
