"""CPU: the build recipes keep the flags bit-exactness depends on.

The kernels reproduce the reference's directed-rounding arithmetic only if
nvcc contracts nothing into FMAs (--fmad=false) and no fast-math flag
relaxes rounding; the oracle needs the same of gcc (-ffp-contract=off,
-frounding-math, no fast math).  The library targets sm_103a alone, with
one -gencode.  The commands are recorded, not run."""

from __future__ import annotations

from cuminlp_gb300 import build as b


def recorded(monkeypatch):
    cmds = []
    monkeypatch.setattr(b, "_run", lambda cmd: cmds.append([str(x) for x in cmd]))
    b.build_library(force=True)
    b.build_oracle(force=True)
    return cmds


def no_fast_math(cmd):
    return not any(("fast-math" in s or "fast_math" in s) and s != "-fno-fast-math" for s in cmd)


def test_library_compiles_for_sm103a_without_contraction(monkeypatch):
    cmds = recorded(monkeypatch)
    compiles = [c for c in cmds if "-c" in c]
    assert sorted(c[c.index("-c") + 1].rsplit("/", 1)[-1] for c in compiles) == sorted(b.SOURCES)
    for c in compiles:
        assert [s for s in c if s.startswith("-gencode")] == ["-gencode=arch=compute_103a,code=sm_103a"]
        assert "--fmad=false" in c and no_fast_math(c)
        assert "-frounding-math" in c
    link = next(c for c in cmds if str(b.LIB) in c)
    assert "-shared" in link and [s for s in link if s.startswith("-gencode")] == [b.ARCH]


def test_oracle_compiles_without_contraction(monkeypatch):
    cmds = recorded(monkeypatch)
    oracle = next(c for c in cmds if str(b.ORACLE_LIB) in c)
    assert "-ffp-contract=off" in oracle and "-frounding-math" in oracle and no_fast_math(oracle)
