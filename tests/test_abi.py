"""The C-ABI library: it loads, exports every function include/qflex_gb300.h
declares, and its permutation tiling is exact (checked on the host by
running the kernel's own index schedule)."""
import ctypes
import random
import re

import numpy as np
import pytest

from tests.conftest import ROOT


def declared_functions():
    text = (ROOT / "include" / "qflex_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qflex_gb300_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(str(built_lib))
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    from qflex_gb300._lib import EXPORTS
    assert sorted(EXPORTS) == names


def test_create_without_gpu_reports_error(built_lib):
    """On a machine without a usable GPU, creating a device context fails
    with an error code and a message, never a crash or a CPU fallback."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from qflex_gb300 import Context, QflexGb300Error
    with pytest.raises(QflexGb300Error) as e:
        Context(0)
    assert e.value.code == 2


@pytest.mark.parametrize("seed", range(6))
def test_permute_schedule_exact(built_lib, seed):
    from qflex_gb300._lib import check_permute
    rng = random.Random(seed)
    for _ in range(60):
        r = rng.randint(0, 12)
        dims = [2 ** rng.randint(0, 4) for _ in range(r)]
        while r and np.prod(dims) > 2 ** 20:
            dims[rng.randrange(r)] = 1
        order = list(range(r))
        rng.shuffle(order)
        n = int(np.prod(dims)) if r else 1
        a = (np.arange(n) + 1j * np.arange(n)[::-1]).astype(np.complex64)
        want = a.reshape(dims).transpose(order).reshape(-1) if r else a
        assert np.array_equal(check_permute(a, dims, order), want), (dims, order)


def test_permute_schedule_reference_cases(built_lib):
    """The reorder cases of the reference's tests/src/tensor_test.cpp:271-469
    (10 and 12 binary indices: single right move, single left move,
    left-right, worst case L-R-L)."""
    from qflex_gb300._lib import check_permute
    cases = [
        (10, "jegcfabdih"), (12, "ablde fghijkc".replace(" ", "")), (12, "gacdefbhijkl"),
        (12, "hbcdefgaijkl"), (12, "cdhijkablefg".replace("cdhijkablefg", "cdhijkabefgl")),
        (12, "kcaldgbfeihj"),
    ]
    for n, new in cases:
        names = "abcdefghijkl"[:n]
        assert sorted(new) == sorted(names), new
        order = [names.index(c) for c in new]
        a = np.arange(2 ** n).astype(np.complex64)
        want = a.reshape([2] * n).transpose(order).reshape(-1)
        assert np.array_equal(check_permute(a, [2] * n, order), want)


def test_permute_schedule_large(built_lib):
    from qflex_gb300._lib import check_permute
    rng = random.Random(7)
    order = list(range(24))
    rng.shuffle(order)
    a = np.arange(2 ** 24).astype(np.complex64)
    assert np.array_equal(check_permute(a, [2] * 24, order),
                          a.reshape([2] * 24).transpose(order).reshape(-1))


def _general_cases():
    import json
    return json.loads((ROOT / "tests" / "golden" / "reorder_general.json").read_text())["cases"]


def test_general_permute_matches_reference_reorder(built_lib):
    """Dimensions that are not powers of two take the general kernel; its
    index math (run on the host) reproduces the reference's own reorders
    (oracle/_ref/qflex_ref, tests/golden/reorder_general.json) and
    numpy.transpose, bit for bit."""
    from qflex_gb300._lib import check_permute
    for case in _general_cases():
        dims, order = case["dims"], case["new_order"]
        n = int(np.prod(dims))
        a = (np.arange(n) - 1j * np.arange(n)).astype(np.complex64)
        got = check_permute(a, dims, order)
        assert np.array_equal(got.real.astype(np.int64), np.array(case["reordered"])), (dims, order)
        assert np.array_equal(got, a.reshape(dims).transpose(order).reshape(-1))
    rng = random.Random(5)
    for _ in range(40):
        r = rng.randint(1, 6)
        dims = [rng.randint(1, 9) for _ in range(r)]
        order = list(range(r))
        rng.shuffle(order)
        n = int(np.prod(dims))
        a = (np.arange(n) + 0.5j).astype(np.complex64)
        assert np.array_equal(check_permute(a, dims, order), a.reshape(dims).transpose(order).reshape(-1))


def test_general_permute_rejects_bad_orders(built_lib):
    from qflex_gb300 import QflexGb300Error
    from qflex_gb300._lib import check_permute
    a = np.zeros(6, dtype=np.complex64)
    for dims, order in (([2, 3], [0, 0]), ([2, 3], [0, 2]), ([6, 0], [1, 0])):
        with pytest.raises(QflexGb300Error):
            check_permute(a, dims, order)
