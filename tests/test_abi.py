"""The C ABI library loads on a machine without a GPU, exports every symbol
the public headers declare, and its host-only entry points behave."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent.parent


def declared_symbols() -> set[str]:
    names = set()
    for h in sorted((REPO / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(rt_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_headers_declare_the_api():
    names = declared_symbols()
    for must in ("rt_context_create", "rt_build_blas", "rt_build_tlas", "rt_trace_rays", "rt_trace_closest",
                 "rt_trace_any", "rt_get_blas_build_sizes", "rt_write_ppm", "rt_sort_pairs"):
        assert must in names


def test_library_exports_every_declared_symbol(rtlib):
    import rtcore
    out = subprocess.run(["nm", "-D", "--defined-only", str(rtcore.lib_path())], capture_output=True, text=True,
                         check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = declared_symbols() - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    # and the Python mirror binds all of them
    assert declared_symbols() <= set(rtcore.PROTOTYPES)


def test_abi_version(rtlib):
    assert rtlib.rt_abi_version() == 1


def test_host_side_argument_checks(rtlib):
    import rtcore
    # null context / outputs are rejected before any device work
    assert rtlib.rt_get_blas_build_sizes(None, None, 0, 0, None) == rtcore.RT_ERR_INVALID_ARG
    assert rtlib.rt_context_create(0, None) == rtcore.RT_ERR_INVALID_ARG
    assert rtlib.rt_sync(None, None) == rtcore.RT_ERR_INVALID_ARG
    assert rtlib.rt_trace_closest(None, None, 0, None, None, None, 0) == rtcore.RT_ERR_INVALID_ARG
    out = C.c_uint64()
    assert rtlib.rt_get_sort_scratch_bytes(1000, 0, C.byref(out)) == rtcore.RT_ERR_INVALID_ARG
    assert rtlib.rt_get_sort_scratch_bytes(1000, 63, C.byref(out)) == rtcore.RT_OK and out.value > 12000


def test_context_without_gpu(rtlib):
    import rtcore
    import torch
    if torch.cuda.is_available():
        return
    h = C.c_void_p()
    assert rtlib.rt_context_create(0, C.byref(h)) == rtcore.RT_ERR_NO_DEVICE


def test_ppm_and_pfm_writers(rtlib, tmp_path):
    img = np.zeros((2, 3, 4), np.float32)
    img[0, 0] = (1.0, 0.5, 0.0, 0.0)
    img[1, 2] = (2.0, -1.0, 0.2, 0.0)
    p = tmp_path / "a.ppm"
    assert rtlib.rt_write_ppm(img.ctypes.data, 3, 2, str(p).encode()) == 0
    data = p.read_bytes()
    assert data.startswith(b"P6\n3 2\n255\n")
    px = np.frombuffer(data[len(b"P6\n3 2\n255\n"):], np.uint8).reshape(2, 3, 3)
    assert tuple(px[0, 0]) == (255, 128, 0)
    assert tuple(px[1, 2]) == (255, 0, 51)
    q = tmp_path / "a.pfm"
    assert rtlib.rt_write_pfm(img.ctypes.data, 3, 2, str(q).encode()) == 0
    body = q.read_bytes()
    hdr = b"PF\n3 2\n-1.0\n"
    assert body.startswith(hdr)
    f = np.frombuffer(body[len(hdr):], np.float32).reshape(2, 3, 3)
    assert np.array_equal(f[1, 0], img[0, 0, :3])  # bottom row first


def test_python_record_layouts_match_the_headers():
    """The numpy mirrors of rt_ray, rt_hit, rt_hit_ext and rt_instance (the
    bit layout of VkAccelerationStructureInstanceKHR) have the C sizes and
    agree with the oracle's, field for field."""
    import oracle
    import rtcore.scenes as S
    assert S.INSTANCE_DTYPE.itemsize == 64
    assert S.INSTANCE_DTYPE == oracle.INSTANCE_DTYPE
    assert S.RAY_DTYPE.itemsize == 32 and S.HIT_EXT_DTYPE.itemsize == 32
    assert S.INSTANCE_DTYPE.fields["accel_ref"][1] == 56
