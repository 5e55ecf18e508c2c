"""Host-side parts of the batched path tracer, no GPU needed: the autotuner's
JSON cache, tuning validation and scratch sizing, and the seeded batch
workload."""
from __future__ import annotations

import json
import math

import numpy as np
import pytest


def _fake_scene(w, h, n_lights=2, accel=0x1000):
    import rtcore
    sc = rtcore.PtScene(accel, 0x2000, 0x3000, 3, 0x4000 if n_lights else 0, n_lights)
    return rtcore.BatchScene(sc, rtcore.Camera((0.0, 0.0, 1.0), 60.0), w, h, 0x5000)


def _scratch_bytes(rtlib, scenes, tuning=None, spp=1, depth=8):
    import ctypes as C
    import rtcore
    arr = (rtcore.BatchScene * len(scenes))(*scenes)
    p = rtcore.BatchParams(spp, depth, 3, 0, 1, 1e-4, 0)
    out = C.c_uint64()
    rc = rtlib.rt_batch_scratch_bytes(arr, len(scenes), C.byref(p), C.byref(tuning) if tuning else None,
                                      C.byref(out))
    return rc, out.value


def test_default_tuning(rtlib):
    import rtcore
    t = rtcore.default_batch_tuning()
    assert t.as_dict() == {"trace_threads": 128, "trace_blocks_per_sm": 8, "stack_ring": 16, "refill": 4,
                           "shade_threads": 256, "wave_paths": 0, "bvh_width": 8}


def test_scratch_sizing_and_validation(rtlib):
    import rtcore
    scenes = [_fake_scene(512, 512), _fake_scene(0, 0, accel=0), _fake_scene(100, 7, n_lights=0)]
    rc, full = _scratch_bytes(rtlib, scenes)
    assert rc == rtcore.RT_OK
    paths = 512 * 512 + 700
    assert paths * 241 <= full < paths * 241 + 64 * 1024  # 241 bytes of queues and path state per path
    t = rtcore.default_batch_tuning()
    t.wave_paths = 4096
    rc, small = _scratch_bytes(rtlib, scenes, t)
    assert rc == rtcore.RT_OK and 4096 * 241 <= small < full
    t.wave_paths = 10 ** 9  # larger than the batch: one wave
    assert _scratch_bytes(rtlib, scenes, t) == (rtcore.RT_OK, full)
    for field, value in (("stack_ring", 12), ("trace_threads", 64), ("refill", 33), ("shade_threads", 1024),
                         ("bvh_width", 3), ("bvh_width", 9)):
        bad = rtcore.default_batch_tuning()
        setattr(bad, field, value)
        assert _scratch_bytes(rtlib, scenes, bad)[0] == rtcore.RT_ERR_INVALID_ARG, field
    # a scene with pixels but no structure, too many lights, too many pixels
    assert _scratch_bytes(rtlib, [_fake_scene(4, 4, accel=0)])[0] == rtcore.RT_ERR_INVALID_ARG
    assert _scratch_bytes(rtlib, [_fake_scene(4, 4, n_lights=(1 << 20) + 1)])[0] == rtcore.RT_ERR_UNSUPPORTED
    assert _scratch_bytes(rtlib, [_fake_scene(65536, 32768)])[0] == rtcore.RT_ERR_UNSUPPORTED
    assert _scratch_bytes(rtlib, [])[0] == rtcore.RT_OK


def test_plan_creation_rejects_bad_arguments_without_a_device(rtlib):
    import ctypes as C
    import rtcore
    arr = (rtcore.BatchScene * 1)(_fake_scene(8, 8))
    p = rtcore.BatchParams(1, 8, 3, 0, 1, 1e-4, 0)
    h = C.c_void_p()
    assert rtlib.rt_batch_plan_create(None, arr, 1, C.byref(p), None, C.c_void_p(256), 1 << 20, 1,
                                      C.byref(h)) == rtcore.RT_ERR_INVALID_ARG
    assert rtlib.rt_batch_launch(None, None, 0) == rtcore.RT_ERR_INVALID_ARG
    assert rtlib.rt_batch_plan_destroy(None) == rtcore.RT_OK


def test_tuning_cache_roundtrip(rtlib, tmp_path):
    import rtcore
    path = tmp_path / "cache.json"
    assert rtcore.tuning_cache_lookup(path, "k") is None
    a = rtcore.default_batch_tuning()
    a.refill, a.stack_ring, a.wave_paths = 8, 32, 123456
    rtcore.tuning_cache_store(path, "sm103-152/n2^6/tris2^25/px2^27/d8", a, 12.3456)
    b = rtcore.default_batch_tuning()
    b.trace_threads, b.trace_blocks_per_sm = 256, 4
    rtcore.tuning_cache_store(path, "other \"quoted\" key", b, 1.5)
    doc = json.loads(path.read_text())
    assert doc["format"] == "rtcore-batch-tuning/1"
    assert set(doc["entries"]) == {"sm103-152/n2^6/tris2^25/px2^27/d8", "other \"quoted\" key"}
    t, ms = rtcore.tuning_cache_lookup(path, "sm103-152/n2^6/tris2^25/px2^27/d8")
    assert t.as_dict() == a.as_dict() and abs(ms - 12.346) < 1e-4
    t, ms = rtcore.tuning_cache_lookup(path, "other \"quoted\" key")
    assert t.as_dict() == b.as_dict() and ms == 1.5
    # updating an entry keeps the other entries and the entry's other fields
    doc = json.loads(path.read_text())
    doc["entries"]["sm103-152/n2^6/tris2^25/px2^27/d8"]["trials"] = [["x", 1.0]]
    path.write_text(json.dumps(doc))
    a.refill = 2
    rtcore.tuning_cache_store(path, "sm103-152/n2^6/tris2^25/px2^27/d8", a, 10.0)
    doc = json.loads(path.read_text())
    e = doc["entries"]["sm103-152/n2^6/tris2^25/px2^27/d8"]
    assert len(doc["entries"]) == 2 and e["refill"] == 2 and e["ms"] == 10 and e["trials"] == [["x", 1]]
    assert not list(tmp_path.glob("*.tmp.*"))


def test_tuning_cache_never_overwrites_foreign_files(rtlib, tmp_path):
    import rtcore
    for text in ("not json", '{"format": "something else", "entries": {}}', "[1, 2]",
                 '{"format": "rtcore-batch-tuning/1", "entries": {"k": {"refill": "x"}}}'):
        path = tmp_path / "f.json"
        path.write_text(text)
        if "entries\": {\"k\"" in text:
            with pytest.raises(rtcore.RtError):
                rtcore.tuning_cache_lookup(path, "k")
            continue
        with pytest.raises(rtcore.RtError):
            rtcore.tuning_cache_lookup(path, "k")
        with pytest.raises(rtcore.RtError):
            rtcore.tuning_cache_store(path, "k", rtcore.default_batch_tuning(), 1.0)
        assert path.read_text() == text


def test_committed_tuning_cache_is_valid(rtlib):
    """The cache shipped with the package parses and holds complete entries."""
    import rtcore
    from rtcore.batch import DEFAULT_CACHE
    if not DEFAULT_CACHE.exists():
        pytest.skip("no tuning cache committed yet")
    doc = json.loads(DEFAULT_CACHE.read_text())
    for key in doc["entries"]:
        t, ms = rtcore.tuning_cache_lookup(DEFAULT_CACHE, key)
        assert t.bvh_width == 8 and ms > 0


def test_batch_workload_is_seeded(rtlib):
    from rtcore.batch import RESOLUTIONS, batch_specs
    a, b = batch_specs(), batch_specs()
    assert a == b and len(a) == 64
    tris = np.array([s.tris for s in a])
    assert tris.min() >= 10_000 and tris.max() <= 5_000_000
    # log-uniform: the median triangle count is near the geometric mean
    assert abs(math.log(np.median(tris)) - 0.5 * (math.log(1e4) + math.log(5e6))) < 1.0
    assert {s.width for s in a} <= set(RESOLUTIONS) and all(s.width == s.height for s in a)
    kinds = [s.kind for s in a]
    assert 16 <= kinds.count("box") <= 48
    assert len({s.camera for s in a}) == 64


def test_lit_soup_and_box_sizes(rtlib):
    import rtcore.scenes as S
    from rtcore.batch import box_shape, lit_soup
    v, i, tm, m = lit_soup(5, 1000)
    assert len(i) == 1004 and (tm[:1000] == 0).all() and list(tm[1000:]) == [1, 1, 2, 2]
    lights = S.emissive_lights(v, i, tm, m)
    assert len(lights) == 2
    for l in lights:
        n = np.cross(l["v1"] - l["v0"], l["v2"] - l["v0"])
        assert n[1] < 0 and abs(n[0]) == 0 and abs(n[2]) == 0  # faces down, toward the soup
    f = v[i[1000]]
    assert np.cross(f[1] - f[0], f[2] - f[0])[1] > 0  # floor faces up
    for n in (10_000, 123_456, 1_000_000, 5_000_000):
        spheres, freq = box_shape(n)
        got = 14 + spheres * 20 * freq * freq
        assert 0.7 * n <= got <= 1.3 * n, (n, got)
