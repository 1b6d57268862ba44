"""Host-side logic of the request server: HBM budget accounting and the
visibility-mask LRU cache (no GPU needed)."""
from totri_gb300.serve import Budget, MaskCache


def entry(n):
    return MaskCache.Entry(object(), n, None)


def test_budget_accounting_and_peak():
    b = Budget(1000)
    b.resident = 300
    assert b.fits(700) and not b.fits(701)
    b.take(500)
    assert b.free() == 200 and b.peak == 800
    b.give(500)
    assert b.free() == 700 and b.peak == 800


def test_mask_cache_lru_eviction_respects_pins():
    b = Budget(1000)
    c = MaskCache(b)
    for k in "abc":
        c.put(k, entry(300))
    assert b.resident == 900 and b.free() == 100
    c.get("a")  # a becomes most recently used: order b, c, a
    c.pin("b")
    assert c.make_room(350)  # b pinned: evicts c (LRU among unpinned) -> 400 free
    assert list(c.entries) == ["b", "a"] and b.free() == 400
    assert not c.make_room(800)  # a evicted, b pinned: 700 free < 800
    assert list(c.entries) == ["b"] and b.free() == 700
    c.unpin("b")
    assert c.make_room(1000) and not c.entries and b.free() == 1000


def test_mask_cache_get_miss_and_pin_counts():
    b = Budget(100)
    c = MaskCache(b)
    assert c.get(("m", "g")) is None
    c.put(("m", "g"), entry(10))
    c.pin(("m", "g"))
    c.pin(("m", "g"))
    c.unpin(("m", "g"))
    assert not c.make_room(100)  # still pinned once
    c.unpin(("m", "g"))
    assert c.make_room(100)


def test_new_mask_moves_from_inflight_to_resident():
    """A request that computes a mask counts it in flight at admission; when
    the mask is cached its bytes move to the resident state, so the sum, and
    the peak, never exceed what admission checked."""
    b = Budget(1000)
    c = MaskCache(b)
    b.resident = 400
    need = 600  # outputs 400 + mask 200
    assert b.fits(need)
    b.take(need)
    c.put("m", entry(200))  # cached during the launch
    b.give(200)             # ... and handed over to the resident state
    assert (b.resident, b.inflight, b.peak) == (600, 400, 1000)
    assert b.resident + b.inflight <= b.total
    b.give(need - 200)      # request done: the mask stays cached
    assert (b.resident, b.inflight, b.free()) == (600, 0, 400)
