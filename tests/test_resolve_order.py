"""CPU: the schedule of the rescue's resolve (gpuzip_gb300/csrc/gi_rescue.cu: k_rs_seq,
k_rs_jump_windows, k_rs_bytes, then k_rs_jump for what stays open), restated at a small scale
on random entries: a final value, or the earlier position copied. Every step replaces an entry by
an entry of its own chain, so each position must end with the value its chain ends in, whatever
the segments, steps and windows. Copies at most a window back are closed without the sweeps; with
longer ones the bytes pass counts entries still open and the sweeps finish them."""
import random

FINAL = 1 << 40  # a final entry: FINAL | value; any smaller entry names the position it copies


def chain_end(e, i):
    while e[i] < FINAL:
        i = e[i]
    return e[i]


def resolve(e, seg, step, win):
    e = list(e)
    n = len(e)
    nseg = (n + seg - 1) // seg
    # the ordered pass: a segment at a time (blocks run at once, but only read their own segment)
    for b in range(nseg):
        S, E = b * seg, min(n, b * seg + seg)
        for ws in range(S, E, step):
            m = min(step, E - ws)
            s = []
            for k in range(m):
                x = e[ws + k]
                if x < FINAL and S <= x < ws:
                    x = e[x]
                s.append(x)
            while True:  # rounds in the step until no entry names a position of the step
                open_ = False
                for k in range(m):
                    x = s[k]
                    if x < FINAL and ws <= x < ws + m:
                        y = s[x - ws]
                        s[k] = y
                        open_ |= y < FINAL and ws <= y < ws + m
                if not open_:
                    break
            e[ws:ws + m] = s
    # pointer jumping over each segment's last window (all segments but the last)
    for _ in range(64):
        left = 0
        for g in range(nseg - 1):
            for i in range((g + 1) * seg - win, (g + 1) * seg):
                if e[i] < FINAL:
                    e[i] = e[e[i]]
                    left += e[i] < FINAL
        if not left:
            break
    # the bytes pass: one hop for an entry still open, counting those it leaves open
    out = [x if x >= FINAL else e[x] for x in e]
    still = sum(1 for x in out if x < FINAL)
    if still:  # (longer copies) sweeps until nothing is open, then the bytes again
        while any(x < FINAL for x in e):
            e = [x if x >= FINAL else e[x] for x in e]
        out = list(e)
    return out, still


def entries(rng, n, far, dist):
    e = []
    for i in range(n):
        if i == 0 or rng.random() < 0.2:
            e.append(FINAL | rng.randrange(256))
        else:
            d = rng.randint(1, min(i, far if rng.random() < 0.01 else dist))
            e.append(i - d)
    return e


def test_chains_end_where_they_did():
    rng = random.Random(11)
    fell_back = 0
    for trial in range(60):
        win = rng.choice([16, 32, 64])
        step = rng.choice([8, 16, 32])
        seg = rng.choice([2, 3, 5]) * max(win, step)
        n = rng.randint(1, 4000)
        long_copies = trial % 3 == 0  # some copies reach further back than a window
        e = entries(rng, n, far=4 * win if long_copies else win, dist=rng.choice([1, 3, win]))
        out, still = resolve(e, seg, step, win)
        assert out == [chain_end(e, i) for i in range(n)], (trial, n, seg, step, win)
        if not long_copies:
            assert still == 0, (trial, still)  # copies within a window: no sweep needed
        fell_back += still > 0
    assert fell_back > 0  # the long copies did take the sweeps
