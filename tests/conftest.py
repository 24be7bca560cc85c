import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def ref_cases():
    with open(ROOT / "tests" / "golden" / "reference_cases.json") as f:
        return {c["name"]: c for c in json.load(f)}


@pytest.fixture(scope="session")
def built_lib():
    """Builds libqflex_gb300.so in-tree when it is missing or stale."""
    from qflex_gb300.build import build
    return build()


@pytest.fixture(scope="session")
def gpu_ctx(built_lib):
    from qflex_gb300 import Context
    return Context(0)


def rel_err(got, want):
    """Largest |got - want| over the set, relative to the set's RMS
    magnitude (amplitudes of random circuits are of similar size, and a
    per-element relative error is meaningless for the ones close to 0)."""
    import numpy as np
    g = np.asarray(got, dtype=np.complex128)
    w = np.asarray(want, dtype=np.complex128)
    scale = max(float(np.sqrt(np.mean(np.abs(w) ** 2))), 1e-300)
    return float(np.max(np.abs(g - w))) / scale


def rel_err_per_amplitude(got, want):
    """Largest |got - want| / |want| over the set, amplitude by amplitude."""
    import numpy as np
    g = np.asarray(got, dtype=np.complex128)
    w = np.asarray(want, dtype=np.complex128)
    return float(np.max(np.abs(g - w) / np.abs(w)))
