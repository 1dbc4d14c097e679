"""The reference-side drop-in sources (baseline/dropin/) and the diff applier of
baseline/build_ref.py, on the CPU.

The GPU test test_reference_dropin.py builds and runs the reference's binding with
these two changes; these checks catch a diff that no longer applies, or a backend
class that misses a member of mpcd::Backend (src/libmpcd/common/backend.hpp:11-31),
before any build.  The checks against the reference's own headers read the staged
copy in baseline/_ref/tree and skip where it is absent.
"""
from __future__ import annotations

import os
import re
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from baseline import build_ref  # noqa: E402

STAGED = os.path.join(ROOT, "baseline", "_ref", "tree", "src", "libmpcd", "common")


def test_unified_diff_applies_and_rejects_mismatches():
    original = "a\nb\nc\nd\n"
    diff = "--- a/f\n+++ b/f\n@@ -2,2 +2,3 @@\n b\n+x\n c\n"
    assert build_ref.apply_unified_diff(original, diff) == "a\nb\nx\nc\nd\n"
    with pytest.raises(RuntimeError, match="does not apply"):
        build_ref.apply_unified_diff("a\nB\nc\nd\n", diff)
    with pytest.raises(RuntimeError, match="malformed"):
        build_ref.apply_unified_diff(original, "no hunks here\n")


def test_dropin_sources_are_present():
    cls, diff = build_ref.dropin_sources()
    assert "class GbBackend final : public Backend" in cls
    assert "USE_GB300" in diff and "gb300::GbBackend" in diff


def _staged(name: str) -> str:
    path = os.path.join(STAGED, name)
    if not os.path.exists(path):
        pytest.skip("no staged copy of the reference's headers")
    with open(path) as f:
        return f.read()


def test_factory_diff_applies_to_the_reference_factory():
    factory = _staged("backend_factory.hpp")
    _, diff = build_ref.dropin_sources()
    patched = build_ref.apply_unified_diff(factory, diff)
    assert patched.count("gb300::GbBackend") == 1
    # the reference's own branches are all still there
    for line in factory.splitlines():
        assert line in patched.splitlines()


def test_backend_class_overrides_every_pure_virtual():
    backend = _staged("backend.hpp")
    pure = re.findall(r"virtual\s+[\w:<>&\s]+?\s(\w+)\s*\([^)]*\)\s*=\s*0", backend)
    assert len(pure) >= 9   # step, stepAndAccumulateSample, getSampleMean, getNParticles, 3 getters/setters, ...
    cls, _ = build_ref.dropin_sources()
    overridden = set(re.findall(r"(\w+)\s*\([^)]*\)\s*(?:const\s*)?override", cls))
    assert set(pure) <= overridden, f"not overridden: {sorted(set(pure) - overridden)}"
