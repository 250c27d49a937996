"""The non-default forms behind the engine's tuning switches give the same
results: the parity tests that exercise each form run again in a child
process with the switch set (the switches are read once per process).

- SPARQ_RADIX_MODE=1: reduce-then-scan radix passes (three launches);
- SPARQ_RADIX_ITEMS=16: 4096-key onesweep tiles;
- SPARQ_RADIX_RANK=1: atomic-OR peer masks in the ranking;
- SPARQ_SMALL_GROUP_MAX=0: small states grouped by the multi-CTA hash path;
- SPARQ_D2H_STREAMS=3 and SPARQ_D2H_BLOCKS=4: copy-engine downloads cut over
  three streams, SM-store downloads by four blocks.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("env, args", [
    ({"SPARQ_RADIX_MODE": "1"}, ["tests/test_radix_sort_gpu.py"]),
    ({"SPARQ_RADIX_ITEMS": "16"}, ["tests/test_radix_sort_gpu.py"]),
    ({"SPARQ_RADIX_RANK": "1"}, ["tests/test_radix_sort_gpu.py"]),
    ({"SPARQ_SMALL_GROUP_MAX": "0"}, ["tests/test_parity_gpu.py", "-k", "hash and (hadamard or condrot)"]),
    ({"SPARQ_D2H_STREAMS": "3", "SPARQ_D2H_BLOCKS": "4"}, ["tests/test_async_download_gpu.py"]),
])
def test_switch_gives_same_results(env, args):
    child_env = dict(os.environ, **env)
    r = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-p", "no:cacheprovider", *args],
                       cwd=ROOT, env=child_env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, f"{env}: {r.stdout[-3000:]}\n{r.stderr[-2000:]}"
