"""The hd-style driver's keyword checks, which run before any device call:
input it cannot honour stops the run with an error naming it (exit code 2),
instead of being dropped."""
from __future__ import annotations

import subprocess

import pytest

from conftest import GOLDEN
from umcp_gb300 import build as UB


def _run(tmp_path, body):
    inp = tmp_path / "run.inp"
    inp.write_text(f"mesh {GOLDEN / 'ico2_plain.mesh'}\n" + body)
    return subprocess.run([str(UB.HD_EXE), str(inp)], capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize("body,message", [
    ("do_ld yes\nnmin 0\ncollect_hk yes\n", "collect_hk"),
    ("do_ld yes\ns_q yes\nncomplex 3\n", "ncomplex, s_q"),
    ("nsteps 2\n", "set do_ld yes"),
    ("do_bd_membrane yes\nnmin 2\nkv 0.01\nrestrain_volume_inside yes\n", "leaflet-volume restraint"),
])
def test_unsupported_input_is_rejected(tmp_path, body, message):
    res = _run(tmp_path, body)
    assert res.returncode == 2 and message in res.stderr, res.stderr
