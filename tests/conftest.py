"""Test configuration.

Markers: ``gpu`` -- needs a GB300 (run with ``-m gpu``); everything else runs
on a CPU-only machine (``-m "not gpu"``).  The oracle (``oracle/``) is the
checker; the product path is ``graphbench_gb300`` (libgbsssp.so).
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the product library and the oracle once per session."""
    import runpy
    runpy.run_path(str(ROOT / "graphbench_gb300" / "build.py"))["build"]()
    import oracle
    oracle.build()
    yield


@pytest.fixture(scope="session")
def gb():
    import graphbench_gb300
    return graphbench_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle


@pytest.fixture(scope="session")
def ref_serial():
    """The reference's own run_sspath_arr (patched D1, D2, D4, P0), built
    from the staged sources; skipped where neither the staged sources nor the
    reference tree exist."""
    import oracle
    from oracle import build_ref
    if not oracle.ref_available("serial"):
        try:
            build_ref.stage()
            build_ref.compile_ref()
        except Exception as e:  # pragma: no cover - depends on the machine
            pytest.skip(f"reference build unavailable: {e}")
    return oracle
