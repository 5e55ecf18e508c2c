"""GPU parity at the full sizes of the box, learned and batched workloads.

The oracle's path tracer is a per-pixel depth-first loop, so it can redo any
subset of a frame: each test traces the whole frame on the GPU through the C
ABI, then has the oracle trace a seeded sample of its pixels on the same
structure with the same random streams, and compares bit for bit.  The
structures themselves are first checked byte-identical with the oracle's
build of the same input.

  * box workload: 2,000,014 triangles (40 icospheres of 50,000), 1920x1080,
    one wave of four samples per pixel, depth 8, Russian roulette from 3;
  * learned workload: the box with 160 icospheres (8,000,014 triangles),
    1920x1080, plain and learned forms (65,536 training paths per sample, Adam
    batches of 4,096); for the learned form the cache query inputs recorded
    at the second vertex (x, -d, n, albedo), the throughput there, the
    training records and targets, and the image after the cache's answers
    are applied;
  * batched workload: five scenes of the 64-scene batch -- soups and boxes of
    26,691 to 3,098,535 triangles at 512^2 to 2048^2 -- in one CUDA-graph
    launch.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import GpuBlas, compare_accels, dev, host

pytestmark = pytest.mark.gpu

W, H = 1920, 1080
N_SAMPLE = 2000


def _pixels(w, h, n, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(w * h, size=min(n, w * h), replace=False)).astype(np.uint32)


def _sum_samples(L):
    """Per-pixel sums of [n, spp, 3] sample radiances in sample order, as the
    accumulation adds them (float32, one rounding per add)."""
    acc = np.zeros((L.shape[0], 3), np.float32)
    for s in range(L.shape[1]):
        acc = acc + L[:, s].astype(np.float32)
    return acc


def _compare(img, px, want, spp, what):
    got = img.reshape(-1, 4)[px]
    assert (got[:, 3] == np.float32(spp)).all(), f"{what}: sample counts"
    bad = np.nonzero((got[:, :3].view(np.uint32) != want.view(np.uint32)).any(1))[0]
    assert len(bad) == 0, (f"{what}: {len(bad)} of {len(px)} sampled pixels differ; first pixel {px[bad[0]]}: "
                           f"gpu {got[bad[0], :3]} oracle {want[bad[0]]}")
    print(f"{what}: {len(px)} sampled pixels bit-exact, {int((want > 0).any(1).sum())} with radiance")


class Box:
    """A box scene on the GPU (built through rt_build_blas) and the oracle's
    build of the same input, checked byte-identical."""

    def __init__(self, ctx, orc, n_spheres):
        import rtcore
        import rtcore.scenes as S
        self.v, self.i, self.tm, self.m = S.box(S.SEED_BASE + 3, n_spheres, 50)
        self.lights = S.emissive_lights(self.v, self.i, self.tm, self.m)
        self.blas = GpuBlas(ctx, [(self.v, self.i, None)])
        self.keep = [dev(self.tm), dev(self.m), dev(self.lights)]
        self.scene = rtcore.PtScene(self.blas.addr, self.keep[0].data_ptr(), self.keep[1].data_ptr(), len(self.m),
                                    self.keep[2].data_ptr(), len(self.lights))
        self.ob, rc = orc.build_blas([(self.v, self.i, None)])
        assert rc == 0
        compare_accels(host(self.blas.accel), self.ob, 48)

    def params(self, spp, offset=0, seed=0x5EED0003):
        import rtcore
        import rtcore.scenes as S
        return rtcore.PtParams(rtcore.Camera(S.BOX_CAMERA[0], S.BOX_CAMERA[1]), W, H, spp, offset, 8, 3, seed,
                               1e-4, 0)

    def oracle_paths(self, orc, px, spp, offset=0, seed=0x5EED0003, train_stride=0):
        import rtcore.scenes as S
        return orc.path_trace_pixels(self.ob, self.tm, self.m, self.lights, S.BOX_CAMERA, W, H, px, spp=spp,
                                     max_depth=8, rr_depth=3, seed=seed, eps=1e-4, sample_offset=offset,
                                     train_stride=train_stride)


def _plain(ctx, orc, box, px, what):
    import torch
    p = box.params(4)
    nb = ctx.pt_scratch_bytes(p)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    accum = torch.zeros(W * H * 4, dtype=torch.float32, device="cuda")
    ctx.path_trace(box.scene, p, accum, scratch, nb)
    ctx.sync()
    img = accum.cpu().numpy()
    rec = box.oracle_paths(orc, px, 4)
    _compare(img, px, _sum_samples(rec["L"]), 4, what)


def test_box_2M_full_frame(ctx, orc):
    """Box workload at full size: byte-identical structure, and 2,000 sampled
    pixels of the 1920x1080 frame (four samples each) bit-exact."""
    box = Box(ctx, orc, 40)
    assert len(box.i) == 2_000_014
    _plain(ctx, orc, box, _pixels(W, H, N_SAMPLE, 3), "box 2M, 1920x1080, 4 spp")


@pytest.fixture(scope="module")
def box8m(ctx, orc):
    box = Box(ctx, orc, 160)
    assert len(box.i) == 8_000_014
    return box


def test_box_8M_plain_full_frame(ctx, orc, box8m):
    _plain(ctx, orc, box8m, _pixels(W, H, N_SAMPLE, 5), "box 8M, 1920x1080, 4 spp")


def test_box_8M_learned_form(ctx, orc, box8m):
    """The learned form at full size: after a first call has trained the
    cache, a second call (one wave of four samples) is checked on 2,000
    sampled pixels against the oracle's learned-form paths -- which paths end
    in a cache query and which train, their recorded inputs, throughputs and
    targets, and the image once the cache's answers are added -- bit for bit
    (the cache's answers themselves come from the GPU)."""
    import torch
    import rtcore
    box = box8m
    npix = W * H
    cache = torch.zeros(ctx.cache_bytes(), dtype=torch.uint8, device="cuda")
    ctx.cache_init(cache, rtcore.cache_config(seed=3))
    cp = rtcore.PtCacheParams(cache.data_ptr(), 65536, 4096)
    p0, p1 = box.params(4, 0), box.params(4, 4)
    nb = ctx.pt_cached_scratch_bytes(p1, cp)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    accum = torch.zeros(npix * 4, dtype=torch.float32, device="cuda")
    ctx.path_trace_cached(box.scene, p0, cp, accum, scratch, nb)
    accum.zero_()
    ctx.path_trace_cached(box.scene, p1, cp, accum, scratch, nb)
    ctx.sync()
    img = accum.cpu().numpy()
    L = ctx.pt_cache_layout(p1, cp, len(box.lights))

    def arr(off, n, dtype, cols=None):
        nbytes = n * np.dtype(dtype).itemsize * (cols or 1)
        a = scratch[off:off + nbytes].cpu().numpy().view(dtype)
        return a.reshape(n, cols) if cols else a

    nq = int(arr(L.query_count, 1, np.uint32)[0])
    nt = int(arr(L.train_count, 1, np.uint32)[0])
    assert 0 < nt <= 4 * ((npix + 30) // 31) and nq > 0
    q_in = arr(L.query_in, nq, np.float32, 12)
    q_t1 = arr(L.query_t1, nq, np.float32, 4)
    q_path = arr(L.query_path, nq, np.uint32)
    q_out = arr(L.query_out, nq, np.float32, 4)
    t_in = arr(L.train_in, nt, np.float32, 12)
    t_t1 = arr(L.train_t1, nt, np.float32, 4)
    t_before = arr(L.train_before, nt, np.float32, 4)
    t_path = arr(L.train_path, nt, np.uint32)
    t_target = arr(L.train_target, nt, np.float32, 4)
    qslot = dict(zip(q_path.tolist(), range(nq)))
    tslot = dict(zip(t_path.tolist(), range(nt)))
    assert len(qslot) == nq and len(tslot) == nt and not (qslot.keys() & tslot.keys())

    stride = npix // 65536
    px = _pixels(W, H, N_SAMPLE, 7)
    rec = box.oracle_paths(orc, px, 4, offset=4, train_stride=stride)
    f32 = np.float32
    radiance = np.zeros((len(px), 4, 3), np.float32)
    kinds = np.zeros(3, int)
    for k, pix in enumerate(px.tolist()):
        for j in range(4):
            r = rec[k, j]
            q = j * npix + pix
            kind = int(r["kind"])
            kinds[kind] += 1
            rec_bits = np.concatenate([r["rec"]["pos"], r["rec"]["dir"], r["rec"]["normal"],
                                       r["rec"]["albedo"]]).astype(np.float32)
            if kind == 1:
                assert q in qslot and q not in tslot, (pix, j, "expected a cache query")
                s = qslot[q]
                assert q_in[s].tobytes() == rec_bits.tobytes(), (pix, j, q_in[s], rec_bits)
                assert q_t1[s, :3].tobytes() == r["t1"].astype(f32).tobytes(), (pix, j)
                c = np.maximum(q_out[s, :3], f32(0))
                radiance[k, j] = r["L"].astype(f32) + r["t1"].astype(f32) * c
            elif kind == 2:
                assert q in tslot and q not in qslot, (pix, j, "expected a training record")
                s = tslot[q]
                assert t_in[s].tobytes() == rec_bits.tobytes(), (pix, j)
                assert t_t1[s, :3].tobytes() == r["t1"].astype(f32).tobytes(), (pix, j)
                assert t_before[s, :3].tobytes() == r["L_before"].astype(f32).tobytes(), (pix, j)
                t = r["t1"].astype(f32)
                with np.errstate(divide="ignore", invalid="ignore"):
                    want_t = np.where(t > 0, (r["L"].astype(f32) - r["L_before"].astype(f32)) / t, f32(0))
                assert t_target[s, :3].tobytes() == want_t.astype(f32).tobytes(), (pix, j)
                radiance[k, j] = r["L"]
            else:
                assert q not in qslot and q not in tslot, (pix, j, "expected neither query nor training record")
                radiance[k, j] = r["L"]
    assert kinds[1] > 0 and kinds[2] > 0, kinds
    print(f"learned form: {nq} queries, {nt} training samples in the wave; sampled paths by kind {kinds.tolist()}")
    _compare(img, px, _sum_samples(radiance), 4, "learned form, box 8M, 1920x1080, 4 spp")


def test_batch_full_size_scenes_in_one_graph(ctx, orc):
    """Five scenes of the 64-scene batched workload at their full sizes --
    including a 3,098,535-triangle box at 2048^2 and a 2,817,949-triangle soup
    at 2048^2 -- traced by one graph launch of rt_batch_launch (two samples,
    depth 8); every structure byte-identical with the oracle's, and 600
    sampled pixels of every image bit-exact with the oracle's paths."""
    import torch
    import rtcore.scenes as S
    from rtcore import batch as B
    specs = B.batch_specs()
    pick = [specs[k] for k in (49, 24, 2, 0, 6)]
    assert pick[0].tris >= 2_000_000 and pick[0].width == 2048
    scenes = B.build_scenes(ctx, pick)
    p = B.batch_params(2, 8)
    table = [sc.batch_scene() for sc in scenes]
    nb = ctx.batch_scratch_bytes(table, p)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    plan = ctx.batch_plan(table, p, scratch, nb, graph=True)
    plan.launch(0)
    ctx.sync()
    plan.close()
    for k, (sp, sc) in enumerate(zip(pick, scenes)):
        v, i, tm, m = B.host_scene(sp)
        ob, rc = orc.build_blas([(v, i, None)])
        assert rc == 0
        compare_accels(host(sc.accel), ob, 48)
        lights = S.emissive_lights(v, i, tm, m)
        px = _pixels(sp.width, sp.height, 600, 100 + k)
        rec = orc.path_trace_pixels(ob, tm, m, lights, sp.camera, sp.width, sp.height, px, spp=2, max_depth=8,
                                    rr_depth=3, seed=B.BATCH_SEED, eps=1e-4)
        _compare(sc.accum.cpu().numpy(), px, _sum_samples(rec["L"]), 2,
                 f"batch scene {sp.kind} {len(i)} tris {sp.width}x{sp.height}")
