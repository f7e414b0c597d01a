"""The random-row gather probe (csrc/gather_roofline.cu, `bench.py
--gather-roofline`): the ceiling of update_phi's access pattern.

On CPU: the probe (built on demand, outside the library build) rejects bad
arguments before it touches the GPU.  On the GPU: a 1 GiB table gives one line per row size
with a positive rate.
"""
import json
import subprocess

import pytest

from mcmc_for_ammsb_gb300 import build as pkg_build


@pytest.fixture(scope="module")
def probe():
    return pkg_build.build_probe()


def test_probe_rejects_bad_arguments(probe):
    for args in (["0.1"], ["8", "0"], ["8", "9"], ["100"]):
        r = subprocess.run([probe] + args, capture_output=True, text=True)
        assert r.returncode == 2, (args, r.returncode, r.stderr)
        assert "usage" in r.stderr


@pytest.mark.gpu
def test_probe_reports_each_row_size(probe):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    r = subprocess.run([probe, "1", "4"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert [x["row_bytes"] for x in lines] == [1024, 2048, 4096]
    for x in lines:
        assert x["rows"] == 2048 * 4 * 128
        assert 1 <= x["ctas_per_sm"] <= 4
        assert 100.0 < x["GBps"] < 20000.0  # a rate, not a broken timer
