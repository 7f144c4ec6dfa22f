"""Stages the reference checkout's sources into baseline/_ref/lettuce/ (git-ignored, never committed),
so that machines without the checkout can build the reference's own binaries from them:

  baseline/_ref/lettuce/{src,tests,vendor,configs}   copied verbatim from the checkout

The staged copy is the input of three recipes, all of which write only under git-ignored folders:
  oracle/Makefile `ref`        the reference CPU backend (oracle and timed CPU baseline)
  baseline/Makefile            the reference CUDA backend behind a C shim (same-GPU baseline)
  integration/Makefile         the reference's drivers and test binary linked against this engine

  python baseline/stage.py <reference checkout>       (or LETTUCE_REF=<checkout>)
"""
from __future__ import annotations

import filecmp
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
STAGE = os.path.join(HERE, "_ref", "lettuce")
PARTS = ("src", "tests", "vendor", "configs")


def staged_root() -> str | None:
    """The reference checkout to build from: LETTUCE_REF if set, else the staged copy if present."""
    env = os.environ.get("LETTUCE_REF")
    if env:
        return env if os.path.isfile(os.path.join(env, "src", "backend.hpp")) else None
    return STAGE if os.path.isfile(os.path.join(STAGE, "src", "backend.hpp")) else None


def _same_tree(a: str, b: str) -> bool:
    if not os.path.isdir(b):
        return False
    cmp = filecmp.dircmp(a, b)
    if cmp.left_only or cmp.right_only or cmp.diff_files or cmp.funny_files:
        return False
    return all(_same_tree(os.path.join(a, d), os.path.join(b, d)) for d in cmp.common_dirs)


def stage(checkout: str) -> str:
    """Copies the parts of `checkout` into the stage (unchanged files keep their times, so the
    recipes above do not rebuild). Returns the stage path."""
    if not os.path.isfile(os.path.join(checkout, "src", "backend.hpp")):
        raise FileNotFoundError(f"{checkout} is not a lettuce checkout (no src/backend.hpp)")
    os.makedirs(STAGE, exist_ok=True)
    for part in PARTS:
        src = os.path.join(checkout, part)
        dst = os.path.join(STAGE, part)
        if not os.path.isdir(src) or _same_tree(src, dst):
            continue
        if os.path.isdir(dst):
            shutil.rmtree(dst)
        shutil.copytree(src, dst)
    return STAGE


if __name__ == "__main__":
    where = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LETTUCE_REF")
    if not where:
        sys.exit("usage: stage.py <reference checkout>  (or set LETTUCE_REF)")
    print(stage(where))
