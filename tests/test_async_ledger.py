"""Host-side check of the bookkeeping that lets the tcgen05 kernels give up
promptly after a bounded wait times out (``csrc/dg_ledger.h``): the ledger is
plain C++, compiled here with the host compiler and run on the CPU."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

SRC = Path(__file__).resolve().parent / "native" / "ledger_check.cpp"


def test_async_ledger_bookkeeping(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "ledger_check"
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", str(SRC), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "ledger ok" in res.stdout
