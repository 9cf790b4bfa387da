"""CPU: cubble-cli's host behaviour without a GPU — usage text without an
input, and a loud failure (exit status 1, the reference's message) instead of
any CPU fallback when no CUDA device exists (src/simulator.cu:1161-1186)."""
import os
import subprocess

import pytest

from cubble_gb300 import buildlib


def _no_gpu():
    try:
        import torch
        return not torch.cuda.is_available()
    except Exception:
        return True


@pytest.fixture(scope="module")
def cli():
    buildlib.build()
    path = buildlib.build_cli()
    if path is None or not os.path.exists(path):
        pytest.skip("cubble-cli not buildable here")
    return path


def test_usage_without_input(cli):
    p = subprocess.run([cli], capture_output=True, text=True, timeout=60)
    assert p.returncode == 1
    assert "Usage:" in p.stdout and "inputFile" in p.stdout


@pytest.mark.skipif(not _no_gpu(), reason="a CUDA device is present")
def test_no_device_fails_loudly(cli, tmp_path):
    inp = tmp_path / "input.json"
    inp.write_text("{}")
    p = subprocess.run([cli, str(inp)], capture_output=True, text=True, timeout=60,
                       cwd=str(tmp_path))
    assert p.returncode == 1
    assert "No CUDA capable devices found." in p.stdout
    assert not (tmp_path / "results.dat").exists()
