"""Every CUDA source gets the flags it declares: the FP arithmetic of the
kernels is fixed by --fmad=false (no compiler-chosen contractions), so a
declaration the build fails to read changes results silently."""
from __future__ import annotations

import glob
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "derivative-pricing_gb300", "csrc")


def test_declared_nvcc_flags_are_applied():
    import build as B  # derivative-pricing_gb300/build.py
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    assert sources
    for path in sources:
        with open(path) as f:
            text = f.read()
        flags = B.nvcc_flags(path)
        for line in text.splitlines():
            if line.startswith("// nvcc-flags:"):
                for flag in line.split(":", 1)[1].split():
                    assert flag in flags, (path, flag)
        if '#include "device_common.cuh"' in text:  # kernels with the fixed FP arithmetic
            assert "--fmad=false" in flags, path
