"""Expands a translation unit's reference-local includes into one file.

Build step of the reference benchmark driver for machines that have a C++
compiler but not the reference sources (the aarch64 GPU hosts): run where
the sources are, it writes each translation unit of oracle/_ref/refbench with
every ``#include "..."`` that resolves inside the reference tree replaced by
that file's text (recursively; include guards do their usual work), and
leaves system includes and the project's own stub headers (mpi.h, silo.h)
as includes.  Headers under the directories given with --also (the
project's source-compatible headers, whose own includes name reference
headers) are expanded the same way.  The output goes only to oracle/_ref/src/, which is git-ignored
like the rest of oracle/_ref/: it is a build artefact, compiled there by
``make -C oracle ref-box``.

    python amalgamate.py OUT SRC REF -I DIR [-I DIR ...] [--also DIR ...]
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

INCLUDE = re.compile(r'^\s*#\s*include\s+"([^"]+)"')


def expand(path: Path, ref: list[Path], dirs: list[Path], seen: set, depth: int = 0) -> list[str]:
    """Every reference header has an include guard, so a header already
    expanded in this unit is dropped the second time, as the guard would."""
    if depth > 64:
        raise RuntimeError(f"include nesting too deep at {path}")
    out = []
    for line in path.read_text(errors="replace").splitlines():
        m = INCLUDE.match(line)
        if m:
            name = m.group(1)
            hit = None
            for d in [path.parent, *dirs]:
                cand = (d / name).resolve()
                if cand.is_file():
                    hit = cand
                    break
            if hit is not None and any(r in hit.parents for r in ref):
                if hit not in seen:
                    seen.add(hit)
                    out.extend(expand(hit, ref, dirs, seen, depth + 1))
                continue
        out.append(line)
    return out


def main(argv: list[str]) -> int:
    if len(argv) < 4:
        print(__doc__, file=sys.stderr)
        return 2
    out, src, ref = Path(argv[1]), Path(argv[2]).resolve(), Path(argv[3]).resolve()
    dirs, also, rest = [], [], argv[4:]
    while rest:
        if rest[0] == "-I" and len(rest) > 1:
            dirs.append(Path(rest[1]).resolve())
            rest = rest[2:]
        elif rest[0] == "--also" and len(rest) > 1:
            also.append(Path(rest[1]).resolve())
            rest = rest[2:]
        else:
            print(f"unknown argument {rest[0]}", file=sys.stderr)
            return 2
    out.parent.mkdir(parents=True, exist_ok=True)
    out.write_text("\n".join(expand(src, [ref, *also], dirs, set())) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
