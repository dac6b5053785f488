"""The integer-pipe binary64 add / subtract / multiply with directed
rounding (csrc/fp64_emu.cuh) against the device's own FP64 instructions:
bit-identical on every operand pair it takes, over operand families that
cover every class, close and distant exponents, cancellation, the edges of
the normal range and carries out of the significand."""

from __future__ import annotations

import ctypes as C

import pytest

from cuminlp_gb300._lib import check, lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


@pytest.mark.parametrize("family", [0, 1, 2, 3, 4])
def test_integer_pipe_ops_match_fp64_instructions(family):
    out = (C.c_uint64 * 3)()
    for seed in (1, 2):
        check(lib().cmn_fp64_emu_check(1 << 22, seed * 7919 + family, family, out))
        mismatches, handled, total = out[0], out[1], out[2]
        assert total == 7 * (1 << 22)
        assert mismatches == 0, (family, seed, mismatches)
        # the families aimed at normal operands stay mostly on the integer path
        if family in (1, 4):
            assert handled > total // 2
