"""Shared fixtures: the gpu marker, the built libraries and the golden cases."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Builds the engine and the oracle if they are missing or stale."""
    from oracle import build as OBLD
    from umcp_gb300 import build as B

    B.build_engine()
    OBLD.build_oracle()
    yield


def golden_cases() -> list[str]:
    # a case is a mesh with its dump; <case>.mass.npz and sub6.npz hold other dumps
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if (GOLDEN / f"{p.stem}.mesh").exists())


def params_from_file(name: str, precision: int = 0):
    import umcp_gb300 as U

    text = (GOLDEN / f"{name}.params").read_text()
    kv = {}
    lipids = []
    for line in text.splitlines():
        parts = line.split()
        if not parts:
            continue
        if parts[0].lower() == "lipid":
            lipids.append(line)
        else:
            kv[parts[0].lower()] = float(parts[1])
    return U.params(kc=kv.get("kc", 14.0), KA=kv.get("ka", 0.215), kg=kv.get("kg", 0.0), k_reg=kv.get("k_reg", 0.0),
                    precision=precision, lipids="\n".join(lipids) + "\n" if lipids else None)


def load_case(name: str, precision: int = 0):
    import umcp_gb300 as U

    prm = params_from_file(name, precision)
    plan = U.Plan(GOLDEN / f"{name}.mesh", prm)
    gold = dict(np.load(GOLDEN / f"{name}.npz"))
    return plan, prm, gold


def rel_inf(a: np.ndarray, b: np.ndarray) -> float:
    """max |a-b| / max |b|: the gradient tolerance measure used throughout."""
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """||a-b||_2 / ||b||_2: the norm-wise gradient measure."""
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
