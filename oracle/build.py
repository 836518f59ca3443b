"""ORACLE - test infrastructure, not product code.

Builds the checker: the oracle's C restatement (oracle/lib/libumcp_oracle.so)
and, where the reference's source tree is present, the reference-built driver
(oracle/_ref/ref_driver, from oracle/ref/Makefile). This recipe is the one
place that names where the reference's sources lie (UMCP_REFERENCE_SRC, by
default the read-only checkout this project was built beside); on a host
without them only the restatement is built. Outputs are git-ignored.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
ORACLE_LIB = ORACLE_DIR / "lib" / "libumcp_oracle.so"
REF_TREE = Path(os.environ.get("UMCP_REFERENCE_SRC", "/root/reference/src"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def build_oracle(verbose: bool = False) -> Path:
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    src = ORACLE_DIR / "umcp_oracle.c"
    if _stale(ORACLE_LIB, [src, ORACLE_DIR / "umcp_oracle.h"]):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-o", str(ORACLE_LIB), str(src), "-lm"])
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


def build_reference_oracle(verbose: bool = False) -> Path | None:
    """Compiles the reference's own sources where they lie (only where the tree exists)."""
    if not (REF_TREE / "interpLib.C").exists():
        return None
    _run(["make", "-s", "-C", str(ORACLE_DIR / "ref"), f"REF_SRC={REF_TREE}", f"-j{os.cpu_count() or 2}"])
    out = ORACLE_DIR / "_ref" / "ref_driver"
    if verbose:
        print(f"built {out}")
    return out


def build_all(verbose: bool = False) -> None:
    build_oracle(verbose)
    build_reference_oracle(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
