"""The integer-path binary64 operations of csrc/fp64_emu.cuh, compiled for
the host, against the host FPU in each rounding mode (round down, round up,
round to nearest). The device twin of this check is
test_gpu_fp64_emu.py; this one needs no GPU."""

from __future__ import annotations

import ctypes as C

import pytest

from cuminlp_gb300._lib import check, lib


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


@pytest.mark.parametrize("family", [0, 1, 2, 3, 4])
def test_integer_path_matches_host_fpu(family):
    out = (C.c_uint64 * 3)()
    check(lib().cmn_fp64_emu_check_host(1 << 18, 31 * family + 5, family, out))
    mismatches, handled, total = out[0], out[1], out[2]
    assert total == 7 * (1 << 18)
    assert mismatches == 0, (family, mismatches)
    assert handled > total // 2  # most pairs exercise the integer path
