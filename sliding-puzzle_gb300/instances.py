"""Seeded instance generators for the 15- and 24-puzzle.

Random numbers: xoshiro256** seeded through splitmix64, so every workload is
reproducible from (generator, seed).  The goal state is 0 1 2 ... N-1 with the
blank top-left, as in the reference's instance files.

  random_walks       non-backtracking blank walks of a fixed length from the
                     goal, uniform over the legal non-reverse moves
  random_permutations uniformly random solvable states (Fisher-Yates, then a
                     swap of two non-blank tiles when the parity is wrong)
  reference_walks    the reference's generator, seeded: at least 150 random
                     move attempts (off-board attempts count) and until the
                     Manhattan distance reaches `md_min`
                     (src/make_24puzzle_problems.cc:54-77)
"""
import numpy as np

MASK64 = (1 << 64) - 1


def _splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & MASK64
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return x, z ^ (z >> 31)


class Xoshiro256ss:
    def __init__(self, seed):
        x = seed & MASK64
        self.s = []
        for _ in range(4):
            x, v = _splitmix64(x)
            self.s.append(v)

    def next(self):
        s = self.s
        rotl = lambda v, k: ((v << k) | (v >> (64 - k))) & MASK64
        result = (rotl((s[1] * 5) & MASK64, 7) * 9) & MASK64
        t = (s[1] << 17) & MASK64
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = rotl(s[3], 45)
        return result

    def below(self, n):
        """Uniform integer in [0, n) (rejection sampling)."""
        lim = (1 << 64) - ((1 << 64) % n)
        while True:
            v = self.next()
            if v < lim:
                return v % n


def _legal(width, blank):
    r, c = divmod(blank, width)
    out = []
    if r > 0:
        out.append(0)
    if c < width - 1:
        out.append(1)
    if c > 0:
        out.append(2)
    if r < width - 1:
        out.append(3)
    return out


_DELTA = {0: lambda w: -w, 1: lambda w: 1, 2: lambda w: -1, 3: lambda w: w}


def goal(width):
    return np.arange(width * width, dtype=np.uint8)


def manhattan(tiles, width):
    s = 0
    for cell, t in enumerate(int(x) for x in tiles):
        if t:
            s += abs(cell // width - t // width) + abs(cell % width - t % width)
    return s


def is_solvable(tiles, width):
    t = [int(x) for x in tiles]
    inv = sum(1 for i in range(len(t)) for j in range(i + 1, len(t)) if t[i] and t[j] and t[j] < t[i])
    brow = t.index(0) // width
    return (inv % 2 == 0) if width % 2 else ((inv + brow) % 2 == 0)


def random_walks(width, n, moves, seed):
    """n states from non-backtracking walks of `moves` moves (an int, or a
    (lo, hi) inclusive range drawn per instance)."""
    rng = Xoshiro256ss(seed)
    out = np.empty((n, width * width), dtype=np.uint8)
    for i in range(n):
        m = moves if isinstance(moves, int) else moves[0] + rng.below(moves[1] - moves[0] + 1)
        b = list(range(width * width))
        blank, pre = 0, -1
        for _ in range(m):
            opts = [d for d in _legal(width, blank) if pre < 0 or d != 3 - pre]
            d = opts[rng.below(len(opts))]
            src = blank + _DELTA[d](width)
            b[blank], b[src] = b[src], 0
            blank, pre = src, d
        out[i] = b
    return out


def random_permutations(width, n, seed):
    rng = Xoshiro256ss(seed)
    N = width * width
    out = np.empty((n, N), dtype=np.uint8)
    for i in range(n):
        p = list(range(N))
        for j in range(N - 1, 0, -1):
            k = rng.below(j + 1)
            p[j], p[k] = p[k], p[j]
        if not is_solvable(p, width):
            a, b = [c for c in range(N) if p[c]][:2]
            p[a], p[b] = p[b], p[a]
        out[i] = p
    return out


def reference_walks(width, n, seed, md_min=None, min_attempts=150):
    rng = Xoshiro256ss(seed)
    N = width * width
    out = np.empty((n, N), dtype=np.uint8)
    for i in range(n):
        limit = md_min if md_min is not None else 35 + i // 5
        b = list(range(N))
        blank = 0
        it = 0
        while it < min_attempts or manhattan(b, width) < limit:
            d = rng.below(4)
            it += 1
            if d not in _legal(width, blank):
                continue
            src = blank + _DELTA[d](width)
            b[blank], b[src] = b[src], 0
            blank = src
        out[i] = b
    return out


def config_instances(name):
    """The seeded workloads of the benchmark configurations."""
    if name == "15_md_walk60":
        return 4, random_walks(4, 100, 60, seed=0x15A)
    if name == "15_random":
        return 4, random_permutations(4, 100, seed=0x15B)
    if name.startswith("24_walk"):
        m = int(name[len("24_walk"):])
        return 5, random_walks(5, 50, m, seed=0x24000 + m)
    if name == "15_mixed4096":
        a = random_walks(4, 2048, (40, 80), seed=0x15C)
        b = random_permutations(4, 2048, seed=0x15D)
        return 4, np.concatenate([a, b])
    raise KeyError(name)
