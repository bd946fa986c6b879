"""Pure-Python restatements of the reference's algorithms, for small cases.

Test infrastructure: a second, independent restatement of the shaders and JS
orchestration (loops over numpy float32 scalars), used to cross-check the C
oracle on tiny inputs.  Citations are to Twinklebear/webgpu-bcmc.
"""
from __future__ import annotations

import math

import numpy as np

F = np.float32

# compute_vertex_values.comp:48-57
INDEX_TO_VERTEX = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
# compute_block_vertices.comp:10-23
EDGE_VERTICES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (6, 5), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]


def sort_by_key(keys, vals, reverse):
    """radix_sort_by_key.js:161-400 literally: stable 64-chunk sort (UINT_MAX
    padding), pairwise merges with upper/lower bound placement, optional full
    reversal, readback from alignedSize-size."""
    C = 64
    n = len(keys)
    cc = 1
    while cc < math.ceil(n / C):
        cc <<= 1
    A = cc * C
    K = list(keys) + [0xFFFFFFFF] * (A - n)
    V = list(vals) + [0xFFFFFFFF] * (A - n)
    for c in range(cc):
        idx = sorted(range(c * C, (c + 1) * C), key=lambda i: K[i])
        K[c * C:(c + 1) * C] = [K[i] for i in idx]
        V[c * C:(c + 1) * C] = [V[i] for i in idx]
    steps = int(math.log2(cc))
    for s in range(steps):
        groups = cc // (2 << s)
        out = A // groups
        half = out // 2
        OK = [None] * A
        OV = [None] * A
        for g in range(groups):
            o = g * out
            a = K[o:o + half]
            b = K[o + half:o + out]
            for i in range(half):
                pa = i + sum(1 for x in b if x <= a[i])
                OK[o + pa] = a[i]
                OV[o + pa] = V[o + i]
                pb = i + sum(1 for x in a if x < b[i])
                OK[o + pb] = b[i]
                OV[o + pb] = V[o + half + i]
        K, V = OK, OV
    if reverse:
        return V[::-1][A - n:]
    return V[:n]


class LRU:
    """js/lru_cache.js:4-903 (element data omitted)."""

    def __init__(self, initial, total):
        al = lambda v, a: (v + a - 1) // a * a
        self.total = total
        self.aligned_total = al(total, 32)
        self.cache_size = al(initial, 32)
        self.item_slots = [-1] * self.aligned_total
        self.age = [2 + i for i in range(self.cache_size)]
        self.avail = [1] * self.cache_size
        self.item = [-1] * self.cache_size
        self.display = 0

    def update(self, needed):
        for s in range(self.cache_size):
            self.age[s] = (self.age[s] + 1) & 0xFFFFFFFF
        needs = [0] * self.total
        for i in range(self.total):
            slot = self.item_slots[i]
            if slot >= 0:
                if needed[i] == 1:
                    self.age[slot] = 0
                    self.avail[slot] = 0
                else:
                    self.avail[slot] = 1
            else:
                needs[i] = needed[i]
        new = [i for i in range(self.total) if needs[i]]
        if not new:
            return []
        n_av = sum(self.avail)
        if n_av < len(new):
            grown = min(self.cache_size + math.ceil((len(new) - n_av) * 1.5), self.total)
            new_size = (grown + 31) // 32 * 32
            for _ in range(self.cache_size, new_size):
                self.age.append(100000)
                self.avail.append(1)
                self.item.append(-1)
            self.cache_size = new_size
            n_av = sum(self.avail)
        self.display = n_av - len(new)
        ids = [s for s in range(self.cache_size) if self.avail[s]]
        keys = [self.age[s] for s in ids]
        order = sort_by_key(keys, ids, True)
        for i, it in enumerate(new):
            slot = order[i]
            prev = self.item[slot]
            if prev != -1:
                self.item_slots[prev] = -1
            self.age[slot] = 0
            self.item[slot] = it
            self.avail[slot] = 0
            self.item_slots[it] = slot
        return new

    def reset(self):
        for s in range(self.cache_size):
            self.age[s], self.avail[s], self.item[s] = 100000, 1, -1
        for i in range(self.total):
            self.item_slots[i] = -1


def block_dims_with_ghost(active, nb, bp):
    """compute_vertex_values.comp:96-156"""
    def act(x, y, z):
        return active[x + nb[0] * (y + nb[1] * z)] != 0

    d = [5 if bp[i] + 1 < nb[i] else 4 for i in range(3)]
    if d == [5, 5, 5] and not act(bp[0] + 1, bp[1] + 1, bp[2] + 1):
        d = [4, 4, 4]
    if d[0] == 5 and d[1] == 5 and not act(bp[0] + 1, bp[1] + 1, bp[2]):
        d[0] = d[1] = 4
    if d[0] == 5 and d[2] == 5 and not act(bp[0] + 1, bp[1], bp[2] + 1):
        d[0] = d[2] = 4
    if d[1] == 5 and d[2] == 5 and not act(bp[0], bp[1] + 1, bp[2] + 1):
        d[1] = d[2] = 4
    if d[0] == 5 and not act(bp[0] + 1, bp[1], bp[2]):
        d[0] = 4
    if d[1] == 5 and not act(bp[0], bp[1] + 1, bp[2]):
        d[1] = 4
    if d[2] == 5 and not act(bp[0], bp[1], bp[2] + 1):
        d[2] = 4
    return d


def compress_position(p):
    """block_vertex_position.comp:9-17"""
    q = []
    for v in p:
        f = F(F(F(v - F(0.5)) * F(0.25)) * F(1023.0))
        q.append(0 if not f > 0 else int(f))
    return ((q[0] & 0x3FF) << 20) | ((q[1] & 0x3FF) << 10) | (q[2] & 0x3FF)


def block_vertices(decoded, active, nb, block_id, iso, tri):
    """compute_block_vertices.comp:76-174 for one block.  `decoded(b)` returns
    the 64 float32 values of block b.  Returns the list of (pack, block_id)."""
    iso = F(iso)
    bp = (block_id % nb[0], (block_id // nb[0]) % nb[1], block_id // (nb[0] * nb[1]))
    d = block_dims_with_ghost(active, nb, bp)
    vol = {}
    for z in range(d[2]):
        for y in range(d[1]):
            for x in range(d[0]):
                nid = (bp[0] + x // 4) + nb[0] * ((bp[1] + y // 4) + nb[1] * (bp[2] + z // 4))
                vol[(x, y, z)] = F(decoded(nid)[(x % 4) + 4 * ((y % 4) + 4 * (z % 4))])
    out = []
    for cell in range(64):
        vx, vy, vz = cell % 4, (cell // 4) % 4, cell // 16
        if not (vx + 1 < d[0] and vy + 1 < d[1] and vz + 1 < d[2]):
            continue
        vals = [vol[(vx + o[0], vy + o[1], vz + o[2])] for o in INDEX_TO_VERTEX]
        case = sum(1 << i for i in range(8) if vals[i] <= iso)
        row = tri[case]
        t = 0
        while row[t] != -1:
            v0, v1 = EDGE_VERTICES[row[t]]
            fa, fb = vals[v0], vals[v1]
            if abs(F(fa - fb)) < F(0.001):
                tt = F(0.0)
            else:
                tt = F(F(iso - fa) / F(fb - fa))
            p = []
            for k, vp in enumerate((vx, vy, vz)):
                a, b = INDEX_TO_VERTEX[v0][k], INDEX_TO_VERTEX[v1][k]
                lerp = F(F(a) + F(tt * F(b - a)))
                p.append(F(F(lerp + F(vp)) + F(0.5)))
            out.append((compress_position(p), block_id))
            t += 1
    return out
