"""The reference-side binding (include/cuminlp_gb300/region_backend.hpp)
compiles against the reference's own headers together with the reference's
SearchDriver, so the reference can drive the GB300 roles unchanged.

Runs where CMN_REFERENCE names the reference tree; the GPU host has none.
The linked, running form of the same binding is tests/test_gpu_reference_driver.py."""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF = Path(os.environ.get("CMN_REFERENCE", "")) if os.environ.get("CMN_REFERENCE") else None

TU = r"""
#include "cuminlp/search/driver.hpp"
#include "cuminlp/policy/bisection_budget.hpp"
#include "cuminlp_gb300/region_backend.hpp"

int run(const cuminlp::model::Problem<double>& p)
{
  auto policy = std::make_shared<cuminlp::policy::BisectionBudgetCompositionPolicy<double>>(4);
  auto backend = std::make_shared<cuminlp_gb300::GB300BackendFactory>();
  cuminlp::search::SearchDriver<double> driver(policy, backend, 100);
  auto out = driver.solve(p);
  return out.found_incumbent() ? 0 : 1;
}
"""


@pytest.mark.skipif(REF is None or not (REF / "include" / "cuminlp").is_dir(),
                    reason="CMN_REFERENCE does not name the reference tree")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_binding_compiles_against_reference(tmp_path):
    src = tmp_path / "binding.cpp"
    src.write_text(TU)
    cmd = ["g++", "-std=c++20", "-fsyntax-only", f"-I{ROOT / 'oracle' / 'ref_shim'}", f"-I{REF / 'include'}",
           f"-I{ROOT / 'include'}", str(src)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr[-3000:]
