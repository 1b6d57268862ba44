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


def _bare_server():
    """A Server's request bookkeeping without its CUDA streams: one 16-point
    grid and one 100-bin measurement on it."""
    import torch

    from totri_gb300 import _lib
    from totri_gb300.serve import Server
    from totri_gb300.types import BinDef
    srv = object.__new__(Server)
    srv.lib = _lib.load()
    srv.grids = {"g": torch.zeros(1, 16, 3)}
    srv.meshes = {}
    srv.measurements = {"t": (torch.zeros(1, 100, 16), "g", BinDef(0.01, 0.0, 100))}
    return srv


def test_fit_request_validation():
    import pytest

    from totri_gb300.serve import Request
    from totri_gb300.types import BinDef, VolumeDef
    srv = _bare_server()
    bd = BinDef(0.01, 0.0, 100)
    vd = VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), (1, 8, 8))
    ok = dict(bins=bd, target="t", volume=vd, iterations=3)
    for kind in ("fit_depth_map", "fit_rbf"):
        srv._validate(Request(kind, "g", **ok))
        for bad, err in ((dict(volume=None), ValueError), (dict(iterations=0), ValueError),
                         (dict(bins=None), ValueError), (dict(target="x"), KeyError),
                         (dict(bins=BinDef(0.02, 0.0, 100)), ValueError)):
            with pytest.raises(err):
                srv._validate(Request(kind, "g", **{**ok, **bad}))
    with pytest.raises(ValueError):
        srv._validate(Request("fit_depth_map", "g",
                              **{**ok, "volume": VolumeDef(vd.start, vd.end, (1, 1, 8))}))
    with pytest.raises(ValueError):
        srv._validate(Request("fit_surface", "g", **ok))


def test_fit_request_planning():
    """GPU-time estimates grow with the steps and the grid; the device bytes a
    fit holds cover its scratch, transients and parameters."""
    from totri_gb300.serve import Request
    from totri_gb300.types import BinDef, VolumeDef
    srv = _bare_server()
    bd = BinDef(0.01, 0.0, 100)
    small = VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), (1, 8, 8))
    big = VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), (1, 32, 32))
    r = lambda kind, vd, n: Request(kind, "g", bins=bd, target="t", volume=vd,  # noqa: E731
                                    iterations=n)
    for kind in ("fit_depth_map", "fit_rbf"):
        assert srv.cost_ms(r(kind, small, 10)) == 10 * srv.cost_ms(r(kind, small, 1))
        assert srv.cost_ms(r(kind, big, 1)) > srv.cost_ms(r(kind, small, 1))
        need = srv._need(r(kind, small, 1))
        V, F = (srv._depth_map_size if kind == "fit_depth_map" else srv._rbf_mesh_bound)(
            r(kind, small, 1))
        assert need >= int(srv.lib.totri_mesh_workspace(1, V, F, 16)) + 4 * 4 * 100 * 16
    assert srv._depth_map_size(r("fit_depth_map", small, 1)) == (64, 2 * 7 * 7)
