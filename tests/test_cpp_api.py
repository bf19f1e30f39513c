"""The header-only C++ layer (include/rmagine_gb300.hpp): rmagine's simulation known answers and
the CrossStatistics paper example, run as a C++ program that throws on failure."""
import subprocess

import pytest


@pytest.mark.gpu
def test_cpp_api_program(built):
    from rmagine_gb300 import build as b

    exe = b.build_cpp_tests()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "passed" in r.stdout


def test_cpp_api_compiles(built):
    """The header and the test program compile against the C ABI (no GPU needed)."""
    from rmagine_gb300 import build as b

    assert b.build_cpp_tests().exists()
