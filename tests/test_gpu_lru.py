"""LRUCache drop-in on the GPU vs the oracle: new items, slot assignment (with
the reference's tie order among equal ages), ages, availability, growth and
reset, after every update."""
import numpy as np
import pytest

import bcmc
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu


def _compare(c_gpu, c_ref, total):
    g = c_gpu.state()
    r = c_ref.state()
    assert g["cache_size"] == c_ref.cache_size
    assert np.array_equal(g["item_slots"][:total], r["item_slots"][:total])
    assert np.array_equal(g["age"], r["age"])
    assert np.array_equal(g["avail"], r["avail"])
    assert np.array_equal(g["item"], r["item"])


# The age sort's plans are all exercised: one pass on the ranks of the age bins
# (ages below 256 within their class), two passes on 16-bit keys (ages of a
# new cache, 2 + slot, up to 32767; or ages past 255 after 300 updates), four
# passes on 32-bit keys (a new cache of more than 32766 slots).
@pytest.mark.parametrize("total,initial,steps", [(300, 20, 40), (5000, 64, 30), (70000, 3500, 12),
                                                 (262144, 13107, 6), (2000, 300, 300), (80000, 40000, 4)])
def test_lru_sequence_matches_oracle(ctx, oracle, total, initial, steps):
    rs = np.random.default_rng(total)
    g = bcmc.LRUCache(ctx, None, None, initial, 256, total)
    r = oracle.LRUCache(initial, total)
    for step in range(steps):
        if step == steps - 3:
            g.reset()
            r.reset()
        p = rs.uniform(0.01, 0.4)
        # spatially coherent needs: runs of needed items, as active blocks are
        needed = (np.convolve(rs.random(total) < p / 8, np.ones(8), mode="same") > 0).astype(np.uint32)
        if step % 7 == 3:
            needed[:] = 0
        n_gpu, ids = g.update(to_dev(needed))
        ref_ids = r.update(needed)
        assert n_gpu == len(ref_ids), step
        if n_gpu:
            assert np.array_equal(ids.numpy(), ref_ids), step
            assert g.displayNumSlotsAvailable == r.slots_available
        _compare(g, r, total)


def test_lru_ties_after_reset(ctx, oracle):
    """After reset every slot has age 100000: assignment order is then the
    reference's tie order (64-chunks ascending, slots descending inside)."""
    total = 4000
    g = bcmc.LRUCache(ctx, None, None, 1000, 256, total)
    r = oracle.LRUCache(1000, total)
    g.reset()
    r.reset()
    needed = np.zeros(total, np.uint32)
    needed[::3] = 1
    n, ids = g.update(to_dev(needed))
    assert np.array_equal(ids.numpy(), r.update(needed))
    _compare(g, r, total)


def _one_pass_plan(ages):
    """The age sort's one-pass plan applies when every available age lies in
    an age bin (below 256 within its class: an update count, or 100000 plus
    one) and at most 256 bins are in use."""
    ages = ages.astype(np.int64)
    in_bin = (ages < 256) | ((ages >= 100000) & (ages - 100000 < 256))
    if not np.all(in_bin):
        return False
    return len(np.unique(np.where(ages < 256, ages, 256 + ages - 100000))) <= 256


def test_lru_plan_change_from_one_pass_to_keys(ctx, oracle):
    """The cache update expects the sort plan of the update before it: it
    accumulates only the age bins while that plan was the one-pass one, and
    its last CTA builds the keys' digit histograms itself when the plan
    changes.  After a reset (every slot at age 100000), one new item per
    update keeps the one-pass plan until the untouched slots' ages leave the
    bins after 256 updates; the slot state must match the oracle's throughout."""
    total, initial = 2000, 1000
    g = bcmc.LRUCache(ctx, None, None, initial, 256, total)
    r = oracle.LRUCache(initial, total)
    g.reset()
    r.reset()
    prev_one_pass, changes = False, []
    for step in range(270):
        needed = np.zeros(total, np.uint32)
        needed[step] = 1
        st = r.state()
        age, item = st["age"][: r.cache_size], st["item"][: r.cache_size]
        keep = (item >= 0) & (needed[np.maximum(item, 0)] != 0)
        one_pass = _one_pass_plan(np.where(keep, 0, age.astype(np.int64) + 1)[~keep])
        if prev_one_pass and not one_pass:
            changes.append(step)
        prev_one_pass = one_pass
        n_gpu, ids = g.update(to_dev(needed))
        ref_ids = r.update(needed)
        assert n_gpu == len(ref_ids) == 1, step
        assert np.array_equal(ids.numpy(), ref_ids), step
        _compare(g, r, total)
    assert changes == [255]
