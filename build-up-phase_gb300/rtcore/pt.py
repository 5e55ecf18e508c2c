"""Command-line renderer: the box workload (a closed, lit box of 12
triangles with --spheres icospheres of 20 x --freq^2 triangles each) path
traced with rt_path_trace, written as a PPM (8-bit) and/or PFM (lossless
float) image, with its speed reported.

    python -m rtcore.pt [--spheres 40] [--freq 50] [--width 1920] [--height 1080]
                        [--spp 4] [--calls 1] [--depth 8] [--binning]
                        [--ppm out.ppm] [--pfm out.pfm]

One warm-up call, then --calls timed calls of --spp samples each (CUDA events
on the launching stream); the image holds all (calls + 1) x spp samples of
every pixel.  Prints one JSON line with the milliseconds per sample, the
extension and shadow rays per sample and M rays/s.  --binning traces the
bounce rays grouped by direction octant instead of in shading order
(RT_PT_OCTANT_BINNING; the image is the same).  It extends the image dump
of the sample's storage-buffer exercise (vulkan-raytracing-basic/README.md:223)
to the path tracer.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import RT_PT_OCTANT_BINNING, Camera, Context, PtParams, load
from . import scenes as S
from .relmse import GpuBox


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--spheres", type=int, default=40)
    ap.add_argument("--freq", type=int, default=50)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--spp", type=int, default=4)
    ap.add_argument("--calls", type=int, default=1)
    ap.add_argument("--depth", type=int, default=8)
    ap.add_argument("--binning", action="store_true")
    ap.add_argument("--ppm", default=None)
    ap.add_argument("--pfm", default=None)
    a = ap.parse_args(argv)
    import torch
    lib = load()
    ctx = Context(0)
    box = GpuBox(ctx, a.spheres, a.freq)
    w, h = a.width, a.height
    flags = RT_PT_OCTANT_BINNING if a.binning else 0
    cam = Camera(S.BOX_CAMERA[0], S.BOX_CAMERA[1])

    def params(offset):
        return PtParams(cam, w, h, a.spp, offset, a.depth, 3, S.SEED_BASE + 3, 1e-4, flags)

    nb = ctx.pt_scratch_bytes(params(0))
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    accum = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    ctx.path_trace(box.scene, params(0), accum, scratch, nb, st)
    ctx.sync(st)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for c in range(a.calls):
        ctx.path_trace(box.scene, params((c + 1) * a.spp), accum, scratch, nb, st)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / (a.calls * a.spp)
    ext, shadow = ctx.pt_ray_counts(params(0), box.n_lights, scratch, st)
    ctx.sync(st)
    res = {"tris": box.n_tris, "resolution": [w, h], "spp": a.spp, "calls": a.calls, "depth": a.depth,
           "octant_binning": a.binning, "ms_per_spp": round(ms, 3),
           "rays_per_spp": {"extension": ext // a.spp, "shadow": shadow // a.spp},
           "mrays_per_s": round((ext + shadow) / a.spp / (ms * 1e3), 1)}
    print(json.dumps(res))
    if a.ppm or a.pfm:
        img = accum.cpu().numpy().reshape(h, w, 4)
        img = np.ascontiguousarray(img / np.maximum(img[..., 3:4], 1.0), np.float32)
        if a.ppm:
            lib.rt_write_ppm(img.ctypes.data, w, h, a.ppm.encode())
        if a.pfm:
            lib.rt_write_pfm(img.ctypes.data, w, h, a.pfm.encode())
    ctx.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
