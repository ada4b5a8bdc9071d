"""The committed ncu summaries stay usable: every `python bench.py` command they
quote uses only options bench.py accepts, every traffic line parses, and
bench.py finds the summary of each configuration it reports traffic for."""
from __future__ import annotations

import glob
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROFILES = sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md")))


@pytest.fixture(scope="module")
def bench_options() -> set[str]:
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True,
                         text=True, check=True, cwd=ROOT).stdout
    return set(re.findall(r"--[a-z0-9][a-z0-9-]*", out))


def _bench_commands(text: str) -> list[str]:
    """bench.py invocations, with backslash-continued lines joined."""
    joined = re.sub(r"\\\n\s*", " ", text)
    return [line[line.index("bench.py"):] for line in joined.splitlines() if "python bench.py" in line]


def test_there_are_summaries():
    assert PROFILES


@pytest.mark.parametrize("path", PROFILES, ids=[os.path.basename(p) for p in PROFILES])
def test_summary_commands_use_bench_options(path, bench_options):
    cmds = _bench_commands(open(path).read())
    assert cmds, "a summary gives the command that made it"
    for cmd in cmds:
        for flag in re.findall(r"(?<!\S)--[a-z0-9][a-z0-9-]*", cmd):
            assert flag in bench_options, (os.path.basename(path), flag)


@pytest.mark.parametrize("path", PROFILES, ids=[os.path.basename(p) for p in PROFILES])
def test_traffic_lines_parse(path):
    for line in open(path):
        if line.strip().startswith("traffic_bytes_per_launch:"):
            assert int(float(line.split(":", 1)[1].strip())) > 0


def test_bench_finds_the_summaries_it_reports():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.profiled_traffic("sliced_kernel", "rmat24") > 0
    assert bench.profiled_traffic("mp_spmv_kernel", "rmat24") > 0
    for form in ("fp32", "bf16", "df32"):
        # both layouts: the default shared-pattern tasks and per-lane deltas (--shared-patterns off)
        assert bench.profiled_traffic("sliced_mixed_kernel", f"stencil256_{form}_noshared") > 0
        assert bench.profiled_traffic("sliced_mixed_kernel", f"stencil256_{form}") > 0
