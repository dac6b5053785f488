"""Writes one self-contained header from the reference's own headers.

TEST INFRASTRUCTURE ONLY.  The reference tree exists in the build container
but not on the GPU host, and binaries built here (x86-64) do not run there
(aarch64).  So the recipe (oracle/build_ref.sh) runs this script where the
reference is mounted: it follows the reference's quoted includes
(``#include "cuminlp/..."``) from a set of entry headers, writes each file
once, in include order, with ``#line`` markers naming the reference file, and
leaves every angle-bracket include (the standard library, CUDA, and the
``cuinterval`` interval library, which the shim directories provide) in
place.  The output lands in oracle/_ref/ (git-ignored) and travels with the
working tree; the harnesses in oracle/ are compiled against it on whichever
machine runs them.

Usage: python amalgamate.py REF_ROOT OUT_FILE ENTRY [ENTRY ...]
ENTRY is a path relative to REF_ROOT (e.g. include/cuminlp/search/driver.hpp).
"""

from __future__ import annotations

import re
import sys
from pathlib import Path

_INC = re.compile(r'^\s*#\s*include\s*"([^"]+)"')
_ONCE = re.compile(r"^\s*#\s*pragma\s+once\b")


def amalgamate(root: Path, entries: list[str]) -> str:
    include_dir = root / "include"
    seen: set[Path] = set()
    out: list[str] = []

    def resolve(name: str, here: Path) -> Path:
        for cand in (here.parent / name, include_dir / name):
            if cand.is_file():
                return cand.resolve()
        raise FileNotFoundError(f"{name} (included from {here})")

    def emit(path: Path) -> None:
        if path in seen:
            return
        seen.add(path)
        rel = path.relative_to(root.resolve())
        out.append(f'#line 1 "{rel}"')
        for lineno, line in enumerate(path.read_text().splitlines(), start=1):
            if _ONCE.match(line):
                out.append("")
                continue
            m = _INC.match(line)
            if m:
                emit(resolve(m.group(1), path))
                out.append(f'#line {lineno + 1} "{rel}"')
                continue
            out.append(line)

    for e in entries:
        emit((root / e).resolve())
    return "#pragma once\n" + "\n".join(out) + "\n"


def main(argv: list[str]) -> int:
    if len(argv) < 4:
        print(__doc__, file=sys.stderr)
        return 2
    root, out = Path(argv[1]), Path(argv[2])
    text = amalgamate(root, argv[3:])
    out.parent.mkdir(parents=True, exist_ok=True)
    if not out.exists() or out.read_text() != text:
        out.write_text(text)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
