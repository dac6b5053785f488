"""The C ABI library loads and exports every symbol include/*.h declares;
host-side validation answers without a GPU."""

from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

from cuminlp_gb300 import _abi as A
from cuminlp_gb300 import _lib
from cuminlp_gb300.problem import Problem

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(cmn_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from cuminlp_gb300 import build
    build.build_library()  # incremental: recompiles only stale sources
    return _lib.lib()


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib.SIGNATURES)


def test_version_and_defaults(lib):
    assert b"sm_103a" in lib.cmn_version()
    o = A.SolveOptions()
    lib.cmn_solve_options_default(C.byref(o))
    assert o.iter_limit == 1000000 and o.tolerance == 1e-6 and o.sample_points == 1


def _create(lib, p: Problem):
    desc, keep = p.desc()
    h = C.c_void_p()
    st = lib.cmn_problem_create(C.byref(desc), C.byref(h))
    if st == 0:
        lib.cmn_problem_destroy(h)
    return st, lib.cmn_last_error().decode()


def test_validation_errors_without_gpu(lib):
    # dag_test.cpp:200-310 rejections, reported as status codes
    p = Problem()
    p.var(0.0, 1.0)
    st, msg = _create(lib, p)
    assert st == 2 and "objective" in msg  # INVALID_PROBLEM: objective never set

    p = Problem()
    x = p.int_var(0.5, 3.0)
    p.set_objective(x * x)
    st, msg = _create(lib, p)
    assert st == 2 and "non-integer" in msg

    p = Problem()
    x = p.var(0.0, 1.0)
    p.set_objective(p.fixed(2.0))
    st, msg = _create(lib, p)
    assert st == 1 and "bare Const" in msg  # INVALID_DAG

    p = Problem()
    x = p.var(2.0, 1.0)
    p.set_objective(x * x)
    st, msg = _create(lib, p)
    assert st == 2 and "lower bound exceeds" in msg

    p = Problem()
    b = p.var(0.0, 2.0, A.VAR_BINARY)
    p.set_objective(b * b)
    st, msg = _create(lib, p)
    assert st == 2 and "Binary" in msg

    p = Problem()
    x = p.var(0.0, 1.0)
    p.set_objective(x * x)
    p.add_constraint(x, A.CMP_LE, float("inf"))
    st, msg = _create(lib, p)
    assert st == 2 and "finite" in msg


def test_malformed_node_table_is_rejected(lib):
    p = Problem()
    x = p.var(0.0, 1.0)
    p.set_objective(x + x)
    nodes, lb, ub, kinds, cons = p.arrays()
    nodes[1]["in0"] = 5  # operand after the node itself
    d = A.ProblemDesc()
    d.nodes = nodes.ctypes.data
    d.n_nodes = len(nodes)
    d.var_lb, d.var_ub, d.var_kinds, d.n_vars = lb.ctypes.data, ub.ctypes.data, kinds.ctypes.data, 1
    d.objective_root = 1
    h = C.c_void_p()
    assert lib.cmn_problem_create(C.byref(d), C.byref(h)) == 1
    assert b"topological" in lib.cmn_last_error()


# entry points that start device work from scalar arguments alone
_DEVICE_WORK = {"cmn_measure_fma_peak", "cmn_fp64_emu_check"}


def _is_pointer(t) -> bool:
    return t is C.c_void_p or (isinstance(t, type) and issubclass(t, C._Pointer))


def test_null_handles_are_rejected_without_gpu(lib):
    """Every entry point that takes a handle or an output pointer answers a
    null one with INVALID_CONFIGURATION (the reference's
    InvalidConfiguration) before any device call; counts read 0 and
    destroy is a no-op."""
    seen = 0
    for name, (res, args) in _lib.SIGNATURES.items():
        if name in _DEVICE_WORK or not args:
            continue
        if not _is_pointer(args[0]):
            continue
        call = [None if _is_pointer(a) else 0 for a in args]
        out = getattr(lib, name)(*call)
        if res is None:
            continue
        if res is C.c_int32:
            assert out == 4, (name, out, lib.cmn_last_error())
            assert lib.cmn_last_error(), name
        else:  # counts and stream handles
            assert not out, (name, out)
        seen += 1
    assert seen >= 45, seen
