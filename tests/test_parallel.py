"""CPU: the parallel loop of the library's host steps (gpuzip_gb300/csrc/gi_parallel.h), driven
through a small C++ program: every index runs exactly once, the loop takes one thread for each
`per_thread` units of work (of the items, or of a given total), at most GI_HOST_THREADS, and a
small loop stays on the calling thread."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = [  # (n, per_thread, work; -1: the items)
    (0, 1, -1), (1, 1, -1), (7, 1, -1), (1000, 1, -1), (100000, 1000, -1), (100000, 1 << 20, -1),
    (10, 1, 1000000), (10, 1000, 5000), (64, 1, -1), (3, 1, 3), (250000, 65536, -1),
]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("parallel") / "parallel_check")
    subprocess.run([cxx, "-std=c++17", "-O1", "-pthread", "-I", os.path.join(ROOT, "gpuzip_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "parallel_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_every_index_once_and_threads_by_work(driver, threads):
    env = dict(os.environ, GI_HOST_THREADS=str(threads))
    lines = "\n".join(f"{n} {p} {w}" for n, p, w in CASES) + "\n"
    out = subprocess.run([driver], input=lines, capture_output=True, text=True, check=True, env=env).stdout.split("\n")
    for (n, per, work), row in zip(CASES, out):
        ok, used, ht = (int(v) for v in row.split())
        assert ok == 1, (n, per, work)
        assert ht == threads
        units = n if work < 0 else work
        most = max(1, min(threads, units // per, n))
        assert used <= most if n else used == 0, (n, per, work, used, most)
        if units // per <= 1:
            assert used <= 1, (n, per, work, used)  # a small loop: the calling thread alone
