"""The public header is plain C: a C99 program (gcc -std=c99 -pedantic
-Werror) that includes include/cuminlp_gb300.h, takes the address of every
entry point the header declares, links against libcuminlp_gb300.so and runs
the host-only calls -- the decode, the branching policy and the program
compiler -- without a GPU.  This is the shape of binding a cgo, JNI or
other FFI caller of the library compiles against."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

from cuminlp_gb300 import _abi as A
from cuminlp_gb300.solver import bisection_choose, slot_bounds
from tests.test_abi import declared_symbols

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r"""
#include <stdio.h>
#include <string.h>

#include "cuminlp_gb300.h"

typedef void (*any_entry)(void);
static const any_entry entries[] = {
  @ENTRIES@
};

int main(void)
{
  size_t i;
  int missing = 0;
  double lo = 0.0, hi = 0.0;
  /* x0^2 + x1 over [-1, 2] x [0, 3], no constraints */
  cmn_node nodes[4];
  double lb[2] = {-1.0, 0.0}, ub[2] = {2.0, 3.0};
  int32_t kinds[2] = {CMN_VAR_CONTINUOUS, CMN_VAR_CONTINUOUS};
  cmn_problem_desc desc;
  int64_t length = 0, count = 0;
  cmn_status st;
  double box[4] = {-1.0, 2.0, 0.0, 3.0};
  uint8_t slot_kinds[64];
  uint64_t var_ids[64], widths[64], domains[64];
  int32_t fathom = 0;

  for (i = 0; i < sizeof entries / sizeof entries[0]; ++i)
    if (!entries[i]) ++missing;
  printf("entries %lu missing %d\n", (unsigned long)(sizeof entries / sizeof entries[0]), missing);
  printf("version %s\n", cmn_version());

  cmn_slot_bounds(CMN_SLOT_CONTINUOUS, -1.0, 2.0, 1, 4, &lo, &hi);
  printf("slot %a %a\n", lo, hi);

  memset(nodes, 0, sizeof nodes);
  nodes[0].op = CMN_OP_VAR; nodes[0].in0 = -1; nodes[0].in1 = -1; nodes[0].var_index = 0;
  nodes[1].op = CMN_OP_VAR; nodes[1].in0 = -1; nodes[1].in1 = -1; nodes[1].var_index = 1;
  nodes[2].op = CMN_OP_SQR; nodes[2].n_in = 1; nodes[2].in0 = 0; nodes[2].in1 = -1;
  nodes[3].op = CMN_OP_ADD; nodes[3].n_in = 2; nodes[3].in0 = 2; nodes[3].in1 = 1;
  memset(&desc, 0, sizeof desc);
  desc.nodes = nodes;
  desc.n_nodes = 4;
  desc.var_lb = lb;
  desc.var_ub = ub;
  desc.var_kinds = kinds;
  desc.n_vars = 2;
  desc.objective_root = 3;
  st = cmn_program_compile(&desc, 0, NULL, 0, &length);
  printf("program %d %lld\n", (int)st, (long long)length);
  desc.objective_root = 9; /* no such node */
  st = cmn_program_compile(&desc, 0, NULL, 0, &length);
  printf("rejected %d %d\n", (int)st, cmn_last_error()[0] != '\0');

  st = cmn_bisection_choose(box, kinds, 2, 3, 0, 0, 0, slot_kinds, var_ids, widths, domains, &count, &fathom);
  printf("choose %d %lld", (int)st, (long long)count);
  for (i = 0; i < (size_t)count; ++i) printf(" %u:%llu", (unsigned)var_ids[i], (unsigned long long)widths[i]);
  printf("\n");
  return missing;
}
"""


def test_c99_program_links_and_runs_the_host_calls(tmp_path):
    cc = shutil.which("gcc") or pytest.skip("gcc not found")
    from cuminlp_gb300 import build
    lib = build.build_library()
    cuda_lib = Path(build._nvcc()).resolve().parents[1] / "lib64"
    names = declared_symbols()
    src = tmp_path / "abi_user.c"
    src.write_text(PROGRAM.replace("@ENTRIES@", ",\n  ".join(f"(any_entry)&{n}" for n in names)))
    exe = tmp_path / "abi_user"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{ROOT / 'include'}", str(src),
                    "-o", str(exe), f"-L{lib.parent}", "-lcuminlp_gb300", f"-Wl,-rpath,{lib.parent}",
                    f"-L{cuda_lib}", f"-Wl,-rpath,{cuda_lib}"], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    lines = {ln.split(" ", 1)[0]: ln.split(" ", 1)[1] for ln in out}
    assert lines["entries"] == f"{len(names)} missing 0"
    assert "sm_103a" in lines["version"]
    lo, hi = (float.fromhex(x) for x in lines["slot"].split())
    assert (lo, hi) == slot_bounds(A.SLOT_CONTINUOUS, -1.0, 2.0, 1, 4)
    st, length = (int(x) for x in lines["program"].split())
    assert st == 0 and length > 0
    st, has_msg = (int(x) for x in lines["rejected"].split())
    assert st != 0 and has_msg == 1
    want = bisection_choose([-1.0, 2.0, 0.0, 3.0], [A.VAR_CONTINUOUS] * 2, 3)
    got = lines["choose"].split()
    assert got[0] == "0" and int(got[1]) == want.size()
    assert got[2:] == [f"{v}:{w}" for v, w in zip(want.var_ids, want.widths)]
