"""CPU: the inference's host pass over the list of unknown bytes (gpuzip_gb300/csrc/gi_rescue.cu,
Rescue::infer) restated at a small scale: the list cut into chunks taken in any order, each
variable owned by one thread (its number's block of 64, round robin) that takes its entries from
every chunk in list order, must give what one pass over the list in order gives. That pass
finds, per entry, its piece (the last beginning at or before the largest position met so far);
the pieces with a lost byte at an offset that is a multiple of 64; the variables in the order
first met with their counts; and each variable's first 64 places with their pieces."""
import bisect
import random


def one_pass(pos, var, start, plen):
    kp, np_ = 0, len(start)
    lost = set()
    order, count, places = [], {}, {}
    for p, v in zip(pos, var):
        while kp + 1 < np_ and start[kp + 1] <= p:
            kp += 1
        if kp < np_ and start[kp] <= p < start[kp] + plen[kp] and (p - start[kp]) % 64 == 0:
            lost.add(kp)
        if v not in count:
            count[v] = 0
            order.append(v)
            places[v] = []
        count[v] += 1
        if len(places[v]) < 64:
            places[v].append((p, kp))
    return lost, order, count, places


def chunked(pos, var, start, plen, C, rng):
    n, np_ = len(pos), len(start)
    if start != sorted(start):
        C = 1
    P = C
    owner = lambda v: (v >> 6) % P  # noqa: E731
    at = [n * c // C for c in range(C + 1)]
    chunk_max = [max(pos[at[c]:at[c + 1]], default=0) for c in range(C)]
    piece = [0] * n
    buckets = [[[] for _ in range(P)] for _ in range(C)]
    lost = set()
    for c in rng.sample(range(C), C):  # the chunks in any order
        m = max(chunk_max[:c], default=0)
        kp = 0
        if c:
            kp = max(0, bisect.bisect_right(start, m) - 1)
        for i in range(at[c], at[c + 1]):
            m = max(m, pos[i])
            while kp + 1 < np_ and start[kp + 1] <= m:
                kp += 1
            if kp < np_ and start[kp] <= pos[i] < start[kp] + plen[kp] and (pos[i] - start[kp]) % 64 == 0:
                lost.add(kp)
            piece[i] = kp
            buckets[c][owner(var[i])].append(i)
    count, met = {}, []
    for o in rng.sample(range(P), P):  # the owners in any order
        for c in range(C):
            for i in buckets[c][o]:
                v = var[i]
                if v not in count:
                    count[v] = 0
                    met.append((i, v))
                count[v] += 1
    order = [v for _, v in sorted(met)]
    places = {v: [] for v in order}
    for o in rng.sample(range(P), P):
        for c in range(C):
            for i in buckets[c][o]:
                v = var[i]
                if len(places[v]) < 64:
                    places[v].append((pos[i], piece[i]))
    return lost, order, count, places


def test_chunks_and_owners_give_one_pass():
    rng = random.Random(7)
    for trial in range(80):
        np_ = rng.randint(1, 40)
        start = sorted(rng.randrange(0, 5000) for _ in range(np_))
        if trial % 10 == 9:
            rng.shuffle(start)  # (not in output order: one chunk, as in the library)
        plen = [rng.randint(0, 400) for _ in range(np_)]
        n = rng.randint(0, 3000)
        pos = sorted(rng.randrange(0, 6000) for _ in range(n))
        if trial % 4 == 3:  # positions that go back now and then
            for _ in range(n // 20):
                i = rng.randrange(n) if n else 0
                if n:
                    pos[i] = rng.randrange(0, 6000)
        var = [rng.choice([rng.randrange(1, 300), rng.randrange(1, 20)]) for _ in range(n)]
        C = rng.choice([1, 2, 3, 7, 16])
        assert chunked(pos, var, start, plen, C, rng) == one_pass(pos, var, start, plen), trial
