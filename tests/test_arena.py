"""CPU: the request server's input arena (gpuzip_gb300/csrc/gi_arena.h), driven through a small C++
program against a model: ranges never overlap and stay inside the capacity, a request is refused
only when no free range could hold it, freed neighbours merge, and the arena is whole again once
everything is freed."""
import os
import random
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("arena") / "arena_check")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "gpuzip_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "arena_check.cpp"), "-o", exe], check=True)
    return exe


def run(exe, lines):
    out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True).stdout
    return [tuple(int(v) for v in row.split()) for row in out.strip().splitlines()]


def units(n, align):
    return max(1, (n + align - 1) // align) * align


class Model:
    """First fit over a sorted list of free ranges, merged on free."""

    def __init__(self, cap, align):
        self.cap, self.align, self.free, self.live = cap, align, [(0, cap)], {}

    def alloc(self, i, n):
        need = units(n, self.align)
        for k, (o, ln) in enumerate(self.free):
            if ln >= need:
                self.free[k:k + 1] = [(o + need, ln - need)] if ln > need else []
                self.live[i] = (o, need)
                return o
        return -1

    def release(self, i):
        self.free.append(self.live.pop(i))
        self.free.sort()
        merged = []
        for fo, fl in self.free:
            if merged and merged[-1][0] + merged[-1][1] == fo:
                merged[-1] = (merged[-1][0], merged[-1][1] + fl)
            else:
                merged.append((fo, fl))
        self.free = merged


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_alloc_free_against_model(driver, seed):
    rng = random.Random(seed)
    cap, align = 64 << 20, 4096
    m = Model(cap, align)
    lines, expect = [f"c {cap} {align}"], [None]
    live = []
    for nid in range(3000):
        if live and (rng.random() < 0.45 or len(live) > 200):
            i = live.pop(rng.randrange(len(live)))
            m.release(i)
            lines.append(f"f {i}")
            expect.append(None)
        else:
            n = int(2 ** rng.uniform(0, 24))
            off = m.alloc(nid, n)
            lines.append(f"a {nid} {n}")
            expect.append(off)
            if off >= 0:
                live.append(nid)
        expect[-1] = (expect[-1], sum(ln for _, ln in m.live.values()), len(m.free),
                      max([ln for _, ln in m.free], default=0), dict(m.live))
    for i in live:
        m.release(i)
        lines.append(f"f {i}")
        expect.append((None, sum(ln for _, ln in m.live.values()), len(m.free),
                       max([ln for _, ln in m.free], default=0), dict(m.live)))
    rows = run(driver, lines)
    assert len(rows) == len(lines)
    refused = 0
    for line, row, want in zip(lines[1:], rows[1:], expect[1:]):
        off, used_b, peak, nfree, largest = row
        w_off, w_used, w_nfree, w_largest, w_live = want
        if w_off is not None:
            assert off == w_off, line
            if off < 0:
                refused += 1
                assert largest < units(int(line.split()[2]), align)  # refused only when nothing fits
        assert (used_b, nfree, largest) == (w_used, w_nfree, w_largest), line
        assert peak >= used_b
        spans = sorted(w_live.values())
        for (a, la), (b, _) in zip(spans, spans[1:]):
            assert a + la <= b  # live ranges never overlap
        assert all(o % align == 0 and o + ln <= cap for o, ln in spans)
    assert rows[-1][1] == 0 and rows[-1][3] == 1 and rows[-1][4] == cap  # whole again
    assert refused > 0  # the sequence did run the arena full


def test_first_fit_and_merge(driver):
    rows = run(driver, ["c 40960 4096", "a 0 8192", "a 1 8192", "a 2 8192", "f 1", "a 3 16384", "a 4 8192",
                        "a 5 1", "f 0", "a 6 1", "a 7 0", "f 2", "f 3", "f 4", "f 6", "f 7", "a 8 40960"])
    assert [r[0] for r in rows[1:4]] == [0, 8192, 16384]
    assert rows[5][0] == 24576          # 16 KiB does not fit the 8 KiB hole: the tail
    assert rows[6][0] == 8192           # 8 KiB fills the hole (first fit)
    assert rows[7][0] == -1             # full
    assert rows[9][0] == 0 and rows[10][0] == 4096  # 1 byte and 0 bytes take one unit each
    assert rows[15][3] == 1 and rows[15][4] == 40960  # all merged back into one range
    assert rows[16][0] == 0
