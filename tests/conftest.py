"""Shared test set-up.

Markers: `gpu` tests need a GB300 and libtws.so (built by
`__graft_entry__.build()`); everything else runs on the CPU against the
oracle, the golden fixtures and the library's host-only entry points.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built libtws.so")


def bits(a):
    """View a float array as integers for bit-exact comparison."""
    a = np.ascontiguousarray(a)
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def assert_bitexact(got, want, name="array"):
    if not np.array_equal(bits(got), bits(want)):
        diff = np.abs(got.astype(np.float64) - want.astype(np.float64))
        idx = np.unravel_index(np.argmax(diff), diff.shape)
        raise AssertionError(f"{name}: {int((bits(got) != bits(want)).sum())} elements differ, "
                             f"max abs {diff.max():.3e} at {idx}: got {got[idx]!r} want {want[idx]!r}")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
